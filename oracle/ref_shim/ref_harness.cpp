// C entry points over the reference's own classes, compiled for the CPU with
// the CUDA stand-in in this folder.  Test infrastructure: tests load
// oracle/_ref/libascref.so through ctypes to pin the oracle against the
// reference itself.  Images are float32, row-major; frames are double[12]
// in CoordFrame's storage order (rotation columns, then translation).
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "CoordFrame.hpp"
#include "KeyCurve.hpp"
#include "Quaternion.hpp"
#include "DownhillSimplex.hpp"
#include "PSO.hpp"
#include "Volume.hpp"
#include "VolumeDescription.hpp"
#include "gpu/cuda/BackgroundRenderer.hpp"
#include "gpu/cuda/Compositor_kernels.h"
#include "gpu/cuda/ContrastFilter.hpp"
#include "gpu/cuda/DRRBackground_kernels.h"
#include "gpu/cuda/GaussianFilter.hpp"
#include "gpu/cuda/HDist_kernels.h"
#include "gpu/cuda/Merger_kernels.h"
#include "gpu/cuda/Mult_kernels.h"
#include "gpu/cuda/Ncc_kernels.h"
#include "gpu/cuda/RadRenderer.hpp"
#include "gpu/cuda/RayCaster.hpp"
#include "gpu/cuda/SharpenFilter.hpp"
#include "gpu/cuda/SobelFilter.hpp"

using namespace xromm;
extern int asc_tex_weight_bits;

#define REF_EXPORT extern "C" __attribute__((visibility("default")))

static CoordFrame to_cf(const double f[12]) { return CoordFrame(f, f + 9); }
static void from_cf(const CoordFrame& c, double f[12])
{
  for (int i = 0; i < 9; ++i) f[i] = c.rotation()[i];
  for (int i = 0; i < 3; ++i) f[9 + i] = c.translation()[i];
}

REF_EXPORT void ref_set_tex_weight_bits(int bits) { asc_tex_weight_bits = bits; }

// ---- CoordFrame ----
REF_EXPORT void ref_frame_from_xyzypr(const double v[6], double f[12]) { from_cf(CoordFrame::from_xyzypr(v), f); }
REF_EXPORT void ref_frame_from_axis_angle(const double v[6], double f[12]) { from_cf(CoordFrame::from_xyzAxis_angle(v), f); }
REF_EXPORT void ref_frame_to_xyzypr(const double f[12], double v[6]) { to_cf(f).to_xyzypr(v); }
REF_EXPORT void ref_frame_mul(const double a[12], const double b[12], double o[12]) { from_cf(to_cf(a) * to_cf(b), o); }
REF_EXPORT void ref_frame_inverse(const double a[12], double o[12]) { from_cf(to_cf(a).inverse(), o); }
REF_EXPORT void ref_frame_linear_extrap(const double a[12], const double b[12], double o[12])
{
  from_cf(to_cf(a).linear_extrap(to_cf(b)), o);
}
// A pose as Tracker::optimize writes it to the trial's key curves and reads
// it back (Tracker.cpp:422-438): float x, y, z; the rotation through Quatf.
REF_EXPORT void ref_keycurve_store(const double in[6], double out[6])
{
  const float x = (float)in[0], y = (float)in[1], z = (float)in[2];
  const Quatf q(in[3], in[4], in[5]);
  const Vec3f e = q.toEuler();
  const double o[6] = {x, y, z, e.z, e.y, e.x};
  for (int i = 0; i < 6; ++i) out[i] = o[i];
}

// ---- KeyCurve ----
// A volume's pose curves (x, y, z KeyCurve<float>, rotation KeyCurve<Quatf>)
// driven by a list of operations: kind 0 inserts poses[6 i] at frames[i] into
// the curves of masks[i] (bit 0 x, 1 y, 2 z, 3 rotation) as setPose does,
// kind 1 erases their keys there, kind 2 clears all; then each of n_eval
// frames is read back as getPose does (the rotation's toEuler as z, y, x).
REF_EXPORT void ref_pose_curve_run(int n_ops, const int* kinds, const int* frames, const int* masks,
                                   const double* poses, int n_eval, const int* eval_frames, double* out)
{
  KeyCurve<float> cx(IKeyCurve::X_CURVE), cy(IKeyCurve::Y_CURVE), cz(IKeyCurve::Z_CURVE);
  KeyCurve<Quatf> cq(IKeyCurve::QUAT_CURVE);
  for (int i = 0; i < n_ops; ++i) {
    const int f = frames[i], m = masks[i];
    const double* p = poses + 6 * i;
    if (kinds[i] == 0) {
      if (m & 1) cx.insert(f, p[0]);
      if (m & 2) cy.insert(f, p[1]);
      if (m & 4) cz.insert(f, p[2]);
      if (m & 8) cq.insert(f, Quatf(p[3], p[4], p[5]));
    } else if (kinds[i] == 1) {
      if ((m & 1) && cx.find(f) != cx.end()) cx.erase(cx.find(f));
      if ((m & 2) && cy.find(f) != cy.end()) cy.erase(cy.find(f));
      if ((m & 4) && cz.find(f) != cz.end()) cz.erase(cz.find(f));
      if ((m & 8) && cq.find(f) != cq.end()) cq.erase(cq.find(f));
    } else {
      cx.clear();
      cy.clear();
      cz.clear();
      cq.clear();
    }
  }
  for (int i = 0; i < n_eval; ++i) {
    const unsigned int f = (unsigned int)eval_frames[i];
    const Vec3f e = cq(f).toEuler();
    const double o[6] = {cx(f), cy(f), cz(f), e.z, e.y, e.x};
    for (int j = 0; j < 6; ++j) out[6 * i + j] = o[j];
  }
}

REF_EXPORT void ref_frame_row_matrix(const double a[12], double m[16]) { to_cf(a).to_matrix_row_order(m); }

// ---- VolumeDescription ----
REF_EXPORT void* ref_volume_create(const void* data, int W, int H, int D, int bps, const double scale[3], const int flip[3])
{
  char name[160];
  snprintf(name, sizeof name, "mem:%llx:%d:%d:%d:%d", (unsigned long long)(uintptr_t)data, W, H, D, bps);
  Volume vol{std::string(name)};
  vol.scaleX((float)scale[0]);
  vol.scaleY((float)scale[1]);
  vol.scaleZ((float)scale[2]);
  vol.flipX(flip[0] != 0);
  vol.flipY(flip[1] != 0);
  vol.flipZ(flip[2] != 0);
  return new gpu::VolumeDescription(vol);
}
REF_EXPORT void ref_volume_info(void* h, int dims[3], float inv_scale[3], float inv_trans[3], double trans_center[3],
                                float minmax[2], void* cropped_out)
{
  auto* vd = (gpu::VolumeDescription*)h;
  const cudaArray* a = (const cudaArray*)vd->image();
  dims[0] = (int)a->w; dims[1] = (int)a->h; dims[2] = (int)a->d;
  for (int i = 0; i < 3; ++i) {
    inv_scale[i] = vd->invScale()[i];
    inv_trans[i] = vd->invTrans()[i];
    trans_center[i] = vd->transCenter()[i];
  }
  minmax[0] = vd->minValue();
  minmax[1] = vd->maxValue();
  if (cropped_out) memcpy(cropped_out, a->data.data(), a->data.size());
}
REF_EXPORT void ref_volume_destroy(void* h) { delete (gpu::VolumeDescription*)h; }

// ---- RayCaster (RayCaster.cpp:88-143) ----
REF_EXPORT void ref_raycast(void* h, const double imv[16], const float vp[4], float step, float intensity, float cutoff,
                            float* out, int w, int hgt)
{
  gpu::RayCaster rc;
  rc.setVolume(*(gpu::VolumeDescription*)h);
  rc.setInvModelView(imv);
  rc.setViewport(vp[0], vp[1], vp[2], vp[3]);
  rc.setSampleDistance(step);
  rc.setRayIntensity(intensity);
  rc.setCutoff(cutoff);
  rc.render(out, (size_t)w, (size_t)hgt);
}

// ---- RadRenderer / BackgroundRenderer ----
REF_EXPORT void ref_rad_render(const void* img, int W, int H, int bps, const float ip[4], const float vp[4], float* out,
                               int w, int h)
{
  gpu::RadRenderer r;
  r.set_rad(img, (size_t)W, (size_t)H, (size_t)bps);
  r.set_image_plane(ip[0], ip[1], ip[2], ip[3]);
  r.set_viewport(vp[0], vp[1], vp[2], vp[3]);
  r.render(out, (size_t)w, (size_t)h);
}
REF_EXPORT void ref_background_render(const float* img, int W, int H, const float ip[4], const float vp[4],
                                      float threshold, float* out, int w, int h)
{
  gpu::BackgroundRenderer r;
  r.set_back(img, (size_t)W, (size_t)H);
  r.set_image_plane(ip[0], ip[1], ip[2], ip[3]);
  r.set_viewport(vp[0], vp[1], vp[2], vp[3]);
  r.render(out, (size_t)w, (size_t)h, threshold);
}

// ---- elementwise ----
REF_EXPORT void ref_drr_background(float* src, float* dst, int w, int h) { gpu::drr_background(src, dst, w, h); }
REF_EXPORT void ref_multiply(float* a, float* b, float* d, int w, int h) { gpu::multiply(a, b, d, w, h); }
REF_EXPORT void ref_merge(float* a, float* b, float* d, int w, int h) { gpu::merge(a, b, d, w, h); }
REF_EXPORT void ref_composite(float* a, float* b, float* c, float* e, float* d, int w, int h)
{
  gpu::composite(a, b, c, e, d, w, h);
}
REF_EXPORT void ref_fill(float* p, unsigned n, float v) { gpu::fill(p, n, v); }

// ---- filters ----
REF_EXPORT void ref_sobel(const float* in, float* out, int w, int h, float scale, float blend)
{
  gpu::SobelFilter f;
  f.setScale(scale);
  f.setBlend(blend);
  f.apply(in, out, w, h);
}
REF_EXPORT void ref_contrast(const float* in, float* out, int w, int h, float alpha, float beta)
{
  gpu::ContrastFilter f;
  f.set_alpha(alpha);
  f.set_beta(beta);
  f.apply(in, out, w, h);
}
REF_EXPORT void ref_gaussian(const float* in, float* out, int w, int h, float radius)
{
  gpu::GaussianFilter f;
  f.set_radius(radius);
  f.apply(in, out, w, h);
}
REF_EXPORT void ref_sharpen(const float* in, float* out, int w, int h, float radius, float contrast, float threshold)
{
  gpu::SharpenFilter f;
  f.set_radius(radius);
  f.set_contrast(contrast);
  f.set_threshold(threshold);
  f.apply(in, out, w, h);
}

// ---- cost reductions ----
REF_EXPORT float ref_ncc(float* f, float* g, float* m, unsigned n)
{
  // the reference's kernels write up to the next multiple of 256 (Ncc_kernels.cu:208-211)
  gpu::ncc_init((n + 255) / 256 * 256);
  float r = gpu::ncc(f, g, m, n);  // ncc_init re-allocates on the next size change
  return r;
}
REF_EXPORT float ref_hdist(float* f, float* g, float* m, unsigned n)
{
  gpu::hdist_init((n + 255) / 256 * 256);
  float r = gpu::hdist(f, g, m, n);
  return r;
}

// ---- optimizers (PSO.cpp, DownhillSimplex.cpp) with a caller-supplied cost ----
typedef double (*ref_cost_fn)(const double* x, void* ctx);
static ref_cost_fn g_cost = nullptr;
static void* g_ctx = nullptr;
double PSO_FUNC(double* P) { return g_cost(P, g_ctx); }
double FUNC(double* P) { return g_cost(P + 1, g_ctx); }

// Runs pso() after srand(seed); writes gBest position (6 floats) and NCC.
REF_EXPORT void ref_pso(ref_cost_fn cost, void* ctx, float lo, float hi, unsigned epochs, unsigned stall, unsigned seed,
                        float pos[6], float* ncc)
{
  g_cost = cost;
  g_ctx = ctx;
  srand(seed);
  Particle p = pso(lo, hi, epochs, stall);
  for (int i = 0; i < 6; ++i) pos[i] = p.Position[i];
  *ncc = p.NCC;
}

// AMOEBA on NDIM+1 vertices given row-major in p (NDIM <= 20); updated in place.
REF_EXPORT int ref_amoeba(ref_cost_fn cost, void* ctx, double* p, double* y, int ndim, double ftol)
{
  g_cost = cost;
  g_ctx = ctx;
  MAT P;
  double Y[MP];
  for (int i = 0; i <= ndim; ++i) {
    for (int j = 0; j < ndim; ++j) P[i + 1][j + 1] = p[i * ndim + j];
    Y[i + 1] = y[i];
  }
  int iter = 0;
  AMOEBA(P, Y, ndim, ftol, &iter);
  for (int i = 0; i <= ndim; ++i) {
    for (int j = 0; j < ndim; ++j) p[i * ndim + j] = P[i + 1][j + 1];
    y[i] = Y[i + 1];
  }
  return iter;
}

// glibc rand() stream used by the reference's PSO (for the host PSO mirror).
REF_EXPORT void ref_srand(unsigned s) { srand(s); }
REF_EXPORT int ref_rand() { return rand(); }
