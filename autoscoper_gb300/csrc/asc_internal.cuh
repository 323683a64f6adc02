// Internal declarations shared by the CUDA translation units of
// libautoscoper_gb300.so: status handling, the device volume layout, the
// FP32 ray march, FP64 rigid-frame algebra (host and device), and the
// reduction helpers.
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include "../../include/autoscoper_gb300.h"

#define ASC_API extern "C" __attribute__((visibility("default")))

namespace asc {

void set_cuda_error(cudaError_t e);
int cuda_status(cudaError_t e);
inline cudaStream_t S(void* s) { return (cudaStream_t)s; }

#define ASC_CUDA(call)                            \
  do {                                            \
    cudaError_t e_ = (call);                      \
    if (e_ != cudaSuccess) return cuda_status(e_); \
  } while (0)

#define ASC_LAUNCH_CHECK() ASC_CUDA(cudaGetLastError())

// --------------------------------------------------------------------------
// Device volume.  Voxels are stored "x-paired": word (x, y, z) holds voxel
// x in its low half and voxel min(x+1, nx-1) in its high half, so that one
// 32-bit load fetches both x taps of a trilinear sample.  The halves are u16
// integers (ASC_STORE_U16), IEEE half (ASC_STORE_F16) or bfloat16
// (ASC_STORE_BF16), all holding the stored integer value; `norm` (1/65535
// or 1/255) turns a raw value into the normalized float that
// cudaReadModeNormalizedFloat would return.
// --------------------------------------------------------------------------
struct DevVolume {
  const uint32_t* pairs;  // nz * ny * nx words
  int nx, ny, nz;
  int storage;
  float norm;
};

struct asc_volume_host {
  DevVolume dev;
  uint32_t* pairs;
  uint8_t* occ;     // occupancy grid of the plain ray caster ...
  float occ_cutoff; // ... for this raw cutoff (NaN = not built)
  float inv_scale[3], inv_trans[3];
  double trans_center[3];
  float min_value, max_value;
  int dims[3];
  int bps;
};

template <int STORE>
__device__ __forceinline__ void unpack(uint32_t w, float& lo, float& hi)
{
  if (STORE == ASC_STORE_BF16) {
    lo = __uint_as_float(w << 16);
    hi = __uint_as_float(w & 0xffff0000u);
  } else if (STORE == ASC_STORE_F16) {
    __half2_raw r;
    r.x = (unsigned short)(w & 0xffffu);
    r.y = (unsigned short)(w >> 16);
    float2 f = __half22float2(*reinterpret_cast<__half2*>(&r));
    lo = f.x;
    hi = f.y;
  } else {
    // u16 -> float without a conversion unit: 2^23 + v is exact in FP32.
    lo = __uint_as_float(0x4b000000u | (w & 0xffffu)) - 8388608.0f;
    hi = __uint_as_float(0x4b000000u | (w >> 16)) - 8388608.0f;
  }
}

// Index and weight of the lower tap of a linear filter at voxel coordinate
// X (texel centres at integers): k = nearest integer to X - 0.5, a = X - k in
// [0, 1].  Where X is an integer the tie may give k = floor(X) - 1 with
// a = 1, which selects the same value.
__device__ __forceinline__ void tap(float X, int& k, float& a)
{
  const float M = 12582912.0f;  // 1.5 * 2^23
  float t = __fadd_rn(__fadd_rn(X, -0.5f), M);
  k = __float_as_int(t) - 0x4b400000;
  a = __fadd_rn(X, -__fadd_rn(t, -M));
}

// Occupancy of 8x8x8-voxel cells for one cutoff: cell (cx, cy, cz) is 0 when
// every voxel of [8c-1, 8c+9) on each axis (the taps of any sample whose
// lower tap lies in the cell) is <= cutoff.  A trilinear sample is a convex
// combination of its taps, so such a sample is <= cutoff and adds exactly
// nothing to the DRR (RayCaster_kernels.cu:189); the march skips it.
constexpr int OCC = 8;

// ---- double-float arithmetic: a value is the unevaluated sum h + l of two
// FP32 numbers (Dekker/Knuth error-free transformations with FMA), about 48
// significant bits.  Used once per ray so that sample positions match FP64.
struct df {
  float h, l;
};

__device__ __forceinline__ df df_two_sum(float a, float b)
{
  const float s = __fadd_rn(a, b);
  const float bb = __fadd_rn(s, -a);
  return {s, __fadd_rn(__fadd_rn(a, -__fadd_rn(s, -bb)), __fadd_rn(b, -bb))};
}

__device__ __forceinline__ df df_fast(float a, float b)  // requires |a| >= |b|
{
  const float s = __fadd_rn(a, b);
  return {s, __fadd_rn(b, -__fadd_rn(s, a))};
}

__device__ __forceinline__ df df_add(df a, df b)
{
  df s = df_two_sum(a.h, b.h);
  const df t = df_two_sum(a.l, b.l);
  s.l = __fadd_rn(s.l, t.h);
  s = df_fast(s.h, s.l);
  s.l = __fadd_rn(s.l, t.l);
  return df_fast(s.h, s.l);
}

__device__ __forceinline__ df df_neg(df a) { return {-a.h, -a.l}; }

__device__ __forceinline__ df df_mulf(df a, float b)
{
  const float p = __fmul_rn(a.h, b);
  float e = fmaf(a.h, b, -p);
  e = fmaf(a.l, b, e);
  return df_fast(p, e);
}

__device__ __forceinline__ df df_mul(df a, df b)
{
  const float p = __fmul_rn(a.h, b.h);
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  return df_fast(p, e);
}

__device__ __forceinline__ df df_div(df a, df b)
{
  const float q1 = __fdiv_rn(a.h, b.h);
  df r = df_add(a, df_neg(df_mulf(b, q1)));
  const float q2 = __fdiv_rn(r.h, b.h);
  r = df_add(r, df_neg(df_mulf(b, q2)));
  const float q3 = __fdiv_rn(r.h, b.h);
  return df_add(df_fast(q1, q2), df{q3, 0.f});
}

__device__ __forceinline__ df df_sqrt(df a)
{
  const float s = __fsqrt_rn(a.h);
  if (!(s > 0.f)) return {s, 0.f};
  const df e = df_add(a, df_neg(df_mul(df{s, 0.f}, df{s, 0.f})));
  return df_fast(s, __fdiv_rn(e.h, 2.0f * s));
}

__device__ __forceinline__ bool df_lt(df a, df b) { return a.h < b.h || (a.h == b.h && a.l < b.l); }

// Per-ray set-up of cuda_volume_render_kernel (RayCaster_kernels.cu:144-186)
// for pixel (x, y) of a w x h image over `vp`, with camera->volume matrix m
// (3x4 row-major, normalisation folded), in double-float: the reference's
// FP32 set-up misplaces the far intersection by ~1e-7 of its length, which
// shifts every sample of the ray; here positions agree with FP64 to ~1e-6
// voxel.  Sample k (k = 0 .. K-1) sits at t = far - k, texel coordinates
// (X - k dX, Y - k dY, Z - k dZ) with texel centres at integers.
struct RaySetup {
  int K;
  df X, Y, Z, dX, dY, dZ;
};

__device__ __forceinline__ bool ray_setup(const float* m, const float* vp, int x, int y, int w, int h, float step,
                                          int nx, int ny, int nz, RaySetup& r)
{
  const df u = df_add(df{vp[0], 0.f}, df_mulf(df_div(df{(float)x, 0.f}, df{(float)w, 0.f}), vp[2]));
  const df v = df_add(df{vp[1], 0.f}, df_mulf(df_div(df{(float)y, 0.f}, df{(float)h, 0.f}), vp[3]));
  const df len = df_sqrt(df_add(df_add(df_mul(u, u), df_mul(v, v)), df{4.0f, 0.f}));
  const df sc = df_div(df{step, 0.f}, len);
  const df l0 = df_mul(u, sc), l1 = df_mul(v, sc), l2 = df_mulf(sc, -2.0f);
  df d[3];
  for (int i = 0; i < 3; ++i)
    d[i] = df_add(df_add(df_mulf(l0, m[4 * i]), df_mulf(l1, m[4 * i + 1])), df_mulf(l2, m[4 * i + 2]));
  const float o[3] = {m[3], m[7], m[11]};
  const float lo[3] = {0.0f, 0.0f, -1.0f}, hi[3] = {1.0f, 1.0f, 0.0f};
  df tn = {-3.0e38f, 0.f}, tf = {3.0e38f, 0.f};
  for (int i = 0; i < 3; ++i) {
    if (d[i].h == 0.f) {  // parallel to the slab
      if (!(o[i] > lo[i] && o[i] < hi[i])) return false;
      continue;
    }
    df a = df_div(df_two_sum(lo[i], -o[i]), d[i]);
    df b = df_div(df_two_sum(hi[i], -o[i]), d[i]);
    if (df_lt(b, a)) {
      const df c = a;
      a = b;
      b = c;
    }
    if (df_lt(tn, a)) tn = a;
    if (df_lt(b, tf)) tf = b;
  }
  if (!df_lt(tn, tf)) return false;  // also a miss for NaN
  if (tn.h < 0.f) tn = df{0.f, 0.f};
  // samples t = far - k > near: K = #{k >= 0 : k < far - near}
  const df D = df_add(tf, df_neg(tn));
  // t -= 1 stops making progress at 2^24; the reference would spin forever on
  // such a degenerate ray, here it counts as a miss.
  if (!(D.h < 8388608.0f)) return false;
  if (D.h < 0.f || (D.h == 0.f && D.l <= 0.f)) {
    r.K = 0;
  } else {
    const float c = ceilf(D.h);
    r.K = (int)c + ((c == D.h && D.l > 0.f) ? 1 : 0);
  }
  // texture coordinates (p.x, 1 - p.y, -p.z) at t = far, minus the half texel
  const df p0 = df_add(df{o[0], 0.f}, df_mul(tf, d[0]));
  const df p1 = df_add(df{o[1], 0.f}, df_mul(tf, d[1]));
  const df p2 = df_add(df{o[2], 0.f}, df_mul(tf, d[2]));
  r.X = df_add(df_mulf(p0, (float)nx), df{-0.5f, 0.f});
  r.Y = df_add(df_mulf(df_add(df{1.0f, 0.f}, df_neg(p1)), (float)ny), df{-0.5f, 0.f});
  r.Z = df_add(df_mulf(df_neg(p2), (float)nz), df{-0.5f, 0.f});
  r.dX = df_mulf(d[0], (float)nx);   // X decreases by dX per sample (t decreases)
  r.dY = df_mulf(d[1], -(float)ny);
  r.dZ = df_mulf(d[2], -(float)nz);
  return true;
}

// Integer base and FP32 fraction of coordinate C - k dC (re-based every
// RB samples so that the fraction stays small and exact to ~1e-6 voxel).
constexpr float REBASE = 32.0f;
__device__ __forceinline__ void coord_base(df C, df dC, float k, int& base_i, float& base_f, float& frac)
{
  const df c = df_add(C, df_neg(df_mulf(dC, k)));
  const float fl = floorf(c.h);
  base_f = fl;
  base_i = (int)fminf(fmaxf(fl, -1.0e6f), 1.0e6f);
  frac = __fadd_rn(__fadd_rn(c.h, -fl), c.l);
}

// One ray of cuda_volume_render_kernel (RayCaster_kernels.cu:187-195): the K
// samples from t = far towards near.  Returns the compensated (Kahan) sum of
// raw samples above cutoff_raw (the caller scales by step * norm /
// intensity).  With `occ`, runs of samples inside empty cells are stepped
// over without being read: the same samples contribute, in the same order.
template <int STORE>
__device__ __forceinline__ float march(const DevVolume& V, const uint8_t* __restrict__ occ, const RaySetup& r,
                                       float cutoff_raw)
{
  const uint32_t* __restrict__ P = V.pairs;
  const int nx = V.nx, ny = V.ny, nz = V.nz;
  const int sxy = nx * ny;
  const int bx = (nx + OCC - 1) / OCC, by = (ny + OCC - 1) / OCC, bz = (nz + OCC - 1) / OCC;
  const float dXh = r.dX.h, dXl = r.dX.l, dYh = r.dY.h, dYl = r.dY.l, dZh = r.dZ.h, dZl = r.dZ.l;
  float acc = 0.f, comp = 0.f;
  int bix = 0, biy = 0, biz = 0;
  float bfx = 0.f, bfy = 0.f, bfz = 0.f, fx = 0.f, fy = 0.f, fz = 0.f;
  float j = REBASE;  // samples since the last base
  for (int k = 0; k < r.K;) {
    if (j >= REBASE) {
      const float kf = (float)k;
      coord_base(r.X, r.dX, kf, bix, bfx, fx);
      coord_base(r.Y, r.dY, kf, biy, bfy, fy);
      coord_base(r.Z, r.dZ, kf, biz, bfz, fz);
      j = 0.f;
    }
    const float FX = fmaf(-j, dXh, fmaf(-j, dXl, fx));
    const float FY = fmaf(-j, dYh, fmaf(-j, dYl, fy));
    const float FZ = fmaf(-j, dZh, fmaf(-j, dZl, fz));
    if (occ) {
      // the lower tap is floor(X) (or floor(X) - 1 at an integer X, see tap)
      // and its cell floor(X / OCC); X here is approximate (~1e-5 voxel)
      const float X = bfx + FX, Y = bfy + FY, Z = bfz + FZ;
      const int cx = min(max(__float2int_rd(X * (1.0f / OCC)), 0), bx - 1);
      const int cy = min(max(__float2int_rd(Y * (1.0f / OCC)), 0), by - 1);
      const int cz = min(max(__float2int_rd(Z * (1.0f / OCC)), 0), bz - 1);
      if (!__ldg(occ + (cz * by + cy) * bx + cx)) {
        // whole samples during which the lower tap stays at least 1e-3 voxel
        // inside the cell (well above the error of X); a coordinate moves by
        // -d per sample
        const float G = 1.0e-3f;
        float s = 3.0e38f;
        if (dXh > 0.f) s = fminf(s, (X - (float)(OCC * cx) - G) / dXh);
        if (dXh < 0.f) s = fminf(s, ((float)(OCC * cx + OCC) - X - G) / -dXh);
        if (dYh > 0.f) s = fminf(s, (Y - (float)(OCC * cy) - G) / dYh);
        if (dYh < 0.f) s = fminf(s, ((float)(OCC * cy + OCC) - Y - G) / -dYh);
        if (dZh > 0.f) s = fminf(s, (Z - (float)(OCC * cz) - G) / dZh);
        if (dZh < 0.f) s = fminf(s, ((float)(OCC * cz + OCC) - Z - G) / -dZh);
        const float m = fminf(fmaxf(floorf(s), 0.f), 1.0e6f) + 1.0f;
        k += (int)m;
        j += m;
        continue;
      }
    }
    int ix, iy, iz;
    float ax, ay, az;
    tap(FX, ix, ax);
    tap(FY, iy, ay);
    tap(FZ, iz, az);
    ix += bix;
    iy += biy;
    iz += biz;
    // clamp-to-edge; below the first texel both taps are texel 0
    if (ix < 0) { ix = 0; ax = 0.f; }
    ix = min(ix, nx - 1);
    int y0 = max(iy, 0), y1 = min(iy + 1, ny - 1);
    y0 = min(y0, ny - 1);
    y1 = max(y1, 0);
    int z0 = max(iz, 0), z1 = min(iz + 1, nz - 1);
    z0 = min(z0, nz - 1);
    z1 = max(z1, 0);
    const int r00 = z0 * sxy + y0 * nx + ix;
    const int r10 = z0 * sxy + y1 * nx + ix;
    const int r01 = z1 * sxy + y0 * nx + ix;
    const int r11 = z1 * sxy + y1 * nx + ix;
    uint32_t w00 = __ldg(P + r00), w10 = __ldg(P + r10), w01 = __ldg(P + r01), w11 = __ldg(P + r11);
    float a0, a1, b0, b1, c0, c1, d0, d1;
    unpack<STORE>(w00, a0, a1);
    unpack<STORE>(w10, b0, b1);
    unpack<STORE>(w01, c0, c1);
    unpack<STORE>(w11, d0, d1);
    float e00 = fmaf(ax, a1 - a0, a0);
    float e10 = fmaf(ax, b1 - b0, b0);
    float e01 = fmaf(ax, c1 - c0, c0);
    float e11 = fmaf(ax, d1 - d0, d0);
    float f0 = fmaf(ay, e10 - e00, e00);
    float f1 = fmaf(ay, e11 - e01, e01);
    float s = fmaf(az, f1 - f0, f0);
    if (s > cutoff_raw) {  // a sample at or below the cutoff leaves the sum untouched
      const float y = s - comp;
      const float tt = acc + y;
      comp = (tt - acc) - y;
      acc = tt;
    }
    ++k;
    j += 1.0f;
  }
  return acc;
}

// Builds the occupancy grid of a device volume for one raw cutoff.
void build_occupancy(const DevVolume& V, float cutoff_raw, uint8_t* occ, cudaStream_t s);
inline size_t occupancy_cells(const DevVolume& V)
{
  return (size_t)((V.nx + OCC - 1) / OCC) * ((V.ny + OCC - 1) / OCC) * ((V.nz + OCC - 1) / OCC);
}

// Global switches (asc_set_option).
extern int g_empty_skip;

// Bilinear read of an 8/16-bit (normalized) or float image with normalized
// coordinates and clamp-to-edge, as tex2D<float> with the reference's
// texture object (cutil_create_tex_obj.h:6-28).
__device__ __forceinline__ float image_texel(const void* img, int bps, int i)
{
  if (bps == 16) return __ldg((const unsigned short*)img + i) * (1.0f / 65535.0f);
  if (bps == 8) return __ldg((const unsigned char*)img + i) * (1.0f / 255.0f);
  return __ldg((const float*)img + i);
}

__device__ __forceinline__ float bilinear(const void* img, int bps, int W, int H, float s, float t)
{
  float X = s * W - 0.5f, Y = t * H - 0.5f;
  float fx = floorf(X), fy = floorf(Y);
  float ax = X - fx, ay = Y - fy;
  fx = fminf(fmaxf(fx, -1.0f), (float)W);
  fy = fminf(fmaxf(fy, -1.0f), (float)H);
  int x0 = (int)fx, y0 = (int)fy;
  int xa = min(max(x0, 0), W - 1), xb = min(max(x0 + 1, 0), W - 1);
  int ya = min(max(y0, 0), H - 1), yb = min(max(y0 + 1, 0), H - 1);
  float v00 = image_texel(img, bps, ya * W + xa), v01 = image_texel(img, bps, ya * W + xb);
  float v10 = image_texel(img, bps, yb * W + xa), v11 = image_texel(img, bps, yb * W + xb);
  float r0 = fmaf(ax, v01 - v00, v00), r1 = fmaf(ax, v11 - v10, v10);
  return fmaf(ay, r1 - r0, r0);
}

// Film-plane pixel of RadRenderer/BackgroundRenderer (RadRenderer_kernels.cu:103-107).
__device__ __forceinline__ bool image_coords(const float* ip, const float* vp, int x, int y, int w, int h, float& s,
                                             float& t)
{
  float u = vp[0] + vp[2] * (x / (float)w);
  float v = vp[1] + vp[3] * (y / (float)h);
  s = (u - ip[0]) / ip[2] + 0.5f;
  t = 0.5f - (v - ip[1]) / ip[3];
  return !(s < 0.0f || t < 0.0f || s > 1.0f || t > 1.0f);
}

// Whether element i of n reaches the reference's multi-level sum()
// (Ncc_kernels.cu:151-187): levels of T = min(n_l, 256) threads fold shared
// memory with s = T/2, T/4, ..., never reading slots at or above 2s.
__host__ __device__ __forceinline__ bool tree_keep(unsigned i, unsigned n)
{
  unsigned idx = i;
  while (n > 1) {
    unsigned T = n < 256u ? n : 256u;
    if (T & (T - 1)) {
      unsigned t = idx % T;
      for (unsigned s = T >> 1; s > 0; s >>= 1) {
        if (t >= 2 * s) return false;
        if (t >= s) t -= s;
      }
    }
    idx /= T;
    n = (n + T - 1) / T;
  }
  return true;
}

// Moments of one block or tile for the NCC (combined in FP64 with Chan et
// al.'s pairwise update): sums over all covered pixels, and count, means and
// co-moments over the covered pixels whose mask > 0.5.
struct Moments {
  double sm, sf, sg;   // sum of mask, f, g over covered pixels
  double n;            // covered pixels with mask > 0.5
  double mf, mg;       // their means
  double cff, cgg, cfg;  // their centred co-moments
};

__host__ __device__ inline void moments_merge(Moments& a, const Moments& b)
{
  a.sm += b.sm;
  a.sf += b.sf;
  a.sg += b.sg;
  double n = a.n + b.n;
  if (b.n == 0) return;
  if (a.n == 0) {
    a.n = b.n; a.mf = b.mf; a.mg = b.mg; a.cff = b.cff; a.cgg = b.cgg; a.cfg = b.cfg;
    return;
  }
  double df = b.mf - a.mf, dg = b.mg - a.mg, k = a.n * b.n / n;
  a.cff += b.cff + df * df * k;
  a.cgg += b.cgg + dg * dg * k;
  a.cfg += b.cfg + df * dg * k;
  a.mf += df * b.n / n;
  a.mg += dg * b.n / n;
  a.n = n;
}

// gpu::ncc's result from the merged moments (Ncc_kernels.cu:116-134):
// means over all covered pixels (sum f / sum mask), centred products over
// mask > 0.5, den < 1e-5 -> 1e5.
__host__ __device__ inline double moments_ncc(const Moments& m)
{
  double mF = m.sf / m.sm, mG = m.sg / m.sm;
  double ef = m.mf - mF, eg = m.mg - mG;
  double num = m.cfg + m.n * ef * eg;
  double d1 = m.cff + m.n * ef * ef;
  double d2 = m.cgg + m.n * eg * eg;
  if (m.n == 0) num = d1 = d2 = 0.0;
  double den = sqrt(d1 * d2);
  if (!(den >= 1e-5)) return den != den ? den : 1e5;
  return num / den;
}

// ---- FP64 rigid frames (CoordFrame.cpp), host and device ----
__host__ __device__ inline void frame_identity(double* f)
{
  for (int i = 0; i < 12; ++i) f[i] = 0.0;
  f[0] = f[4] = f[8] = 1.0;
}

__host__ __device__ inline void frame_rotate(double* f, const double* caxis, double angle)
{
  const double PI = 3.14159265358979323846;
  double a0 = caxis[0], a1 = caxis[1], a2 = caxis[2];
  double c = cos(PI * angle / 180.0), s = sin(PI * angle / 180.0);
  double mag = sqrt(a0 * a0 + a1 * a1 + a2 * a2);
  if (mag == 0) return;
  a0 /= mag; a1 /= mag; a2 /= mag;
  double oc = 1.0 - c;
  double R[9] = {oc * a0 * a0 + c,      oc * a0 * a1 + s * a2, oc * a0 * a2 - s * a1,
                 oc * a0 * a1 - s * a2, oc * a1 * a1 + c,      oc * a1 * a2 + s * a0,
                 oc * a0 * a2 + s * a1, oc * a1 * a2 - s * a0, oc * a2 * a2 + c};
  double t[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) t[3 * i + j] = f[3 * i] * R[j] + f[3 * i + 1] * R[3 + j] + f[3 * i + 2] * R[6 + j];
  for (int i = 0; i < 9; ++i) f[i] = t[i];
}

__host__ __device__ inline void frame_from_xyzypr(const double* v, double* f)
{
  frame_identity(f);
  double ax[3];
  ax[0] = f[6]; ax[1] = f[7]; ax[2] = f[8];
  frame_rotate(f, ax, v[3]);
  ax[0] = f[3]; ax[1] = f[4]; ax[2] = f[5];
  frame_rotate(f, ax, v[4]);
  ax[0] = f[0]; ax[1] = f[1]; ax[2] = f[2];
  frame_rotate(f, ax, v[5]);
  f[9] += v[0]; f[10] += v[1]; f[11] += v[2];
}

__host__ __device__ inline void frame_from_axis_angle(const double* v, double* f)
{
  frame_identity(f);
  double ang = sqrt(v[3] * v[3] + v[4] * v[4] + v[5] * v[5]);
  if (ang != 0) frame_rotate(f, v + 3, ang);
  f[9] += v[0]; f[10] += v[1]; f[11] += v[2];
}

__host__ __device__ inline void frame_to_xyzypr(const double* f, double* v)
{
  const double PI = 3.14159265358979323846;
  v[0] = f[9]; v[1] = f[10]; v[2] = f[11];
  v[3] = 180.0 * atan2(f[1], f[0]) / PI;
  v[4] = 180.0 * atan2(-f[2], sqrt(f[5] * f[5] + f[8] * f[8])) / PI;
  v[5] = 180.0 * atan2(f[5], f[8]) / PI;
}

__host__ __device__ inline void frame_mul(const double* a, const double* b, double* out)
{
  double r[12];
  for (int c = 0; c < 3; ++c)
    for (int i = 0; i < 3; ++i) r[3 * c + i] = a[i] * b[3 * c] + a[3 + i] * b[3 * c + 1] + a[6 + i] * b[3 * c + 2];
  for (int i = 0; i < 3; ++i) r[9 + i] = a[i] * b[9] + a[3 + i] * b[10] + a[6 + i] * b[11] + a[9 + i];
  for (int i = 0; i < 12; ++i) out[i] = r[i];
}

__host__ __device__ inline void frame_inverse(const double* a, double* out)
{
  double r[12] = {a[0], a[3], a[6], a[1], a[4], a[7], a[2], a[5], a[8], 0, 0, 0};
  r[9] = -(r[0] * a[9] + r[3] * a[10] + r[6] * a[11]);
  r[10] = -(r[1] * a[9] + r[4] * a[10] + r[7] * a[11]);
  r[11] = -(r[2] * a[9] + r[5] * a[10] + r[8] * a[11]);
  for (int i = 0; i < 12; ++i) out[i] = r[i];
}

__host__ __device__ inline void frame_point(const double* f, const double* p, double* q)
{
  double r0 = f[0] * p[0] + f[3] * p[1] + f[6] * p[2] + f[9];
  double r1 = f[1] * p[0] + f[4] * p[1] + f[7] * p[2] + f[10];
  double r2 = f[2] * p[0] + f[5] * p[1] + f[8] * p[2] + f[11];
  q[0] = r0; q[1] = r1; q[2] = r2;
}

// RayCaster::setInvModelView (RayCaster.cpp:88-114) applied to the inverse of
// `modelview`: the 3x4 camera->volume matrix with the volume normalisation
// folded in, rounded to float as the reference stores it.
__host__ __device__ inline void fold_matrix(const double* imv16, const float* inv_scale, const float* inv_trans,
                                            float* m12)
{
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 4; ++c)
      m12[4 * r + c] = (float)(imv16[4 * r + c] * (double)inv_scale[r] + imv16[12 + c] * (double)inv_trans[r]);
}

__host__ __device__ inline void frame_row_matrix(const double* f, double* m)
{
  m[0] = f[0]; m[1] = f[3]; m[2] = f[6]; m[3] = f[9];
  m[4] = f[1]; m[5] = f[4]; m[6] = f[7]; m[7] = f[10];
  m[8] = f[2]; m[9] = f[5]; m[10] = f[8]; m[11] = f[11];
  m[12] = 0; m[13] = 0; m[14] = 0; m[15] = 1;
}

// Tracker::calculate_viewport (Tracker.cpp:923-1032).
__host__ __device__ inline bool calculate_viewport(const double* mv, const double* cam, const double* ip,
                                                   const float* inv_scale, const float* inv_trans, double* vp)
{
  double mm[4] = {1.0, 1.0, -1.0, -1.0};
  const double corners[24] = {0, 0, -1, 0, 0, 0, 0, 1, -1, 0, 1, 0, 1, 0, -1, 1, 0, 0, 1, 1, -1, 1, 1, 0};
  for (int j = 0; j < 8; ++j) {
    double p[3], q[3];
    for (int k = 0; k < 3; ++k) p[k] = (corners[3 * j + k] - (double)inv_trans[k]) / (double)inv_scale[k];
    frame_point(mv, p, q);
    double fx = -2 * q[0] / q[2], fy = -2 * q[1] / q[2];
    if (mm[0] > fx) mm[0] = fx;
    if (mm[1] > fy) mm[1] = fy;
    if (mm[2] < fx) mm[2] = fx;
    if (mm[3] < fy) mm[3] = fy;
  }
  double ci[12], a[3], b[3];
  frame_inverse(cam, ci);
  frame_point(ci, ip + 3, a);
  frame_point(ci, ip + 9, b);
  double rf[4] = {-2 * a[0] / a[2], -2 * a[1] / a[2], -2 * b[0] / b[2], -2 * b[1] / b[2]};
  if (mm[0] > rf[2] && mm[2] > rf[2]) return false;
  if (mm[1] > rf[3] && mm[3] > rf[3]) return false;
  if (mm[0] < rf[0] && mm[2] < rf[0]) return false;
  if (mm[1] < rf[1] && mm[3] < rf[1]) return false;
  if (mm[0] == 1.0 && mm[1] == 1.0 && mm[2] == -1.0 && mm[3] == -1.0) return false;
  if (mm[0] < rf[0]) mm[0] = rf[0];
  if (mm[1] < rf[1]) mm[1] = rf[1];
  if (mm[2] > rf[2]) mm[2] = rf[2];
  if (mm[3] > rf[3]) mm[3] = rf[3];
  vp[0] = mm[0];
  vp[1] = mm[1];
  vp[2] = mm[2] - mm[0];
  vp[3] = mm[3] - mm[1];
  return true;
}

// Gaussian weights of GaussianFilter::set_radius / SharpenFilter::makeFilter:
// K = 2 floor(3r) + 1 taps per axis; the 2-D kernel 2.71828^(-(i^2+j^2)/(2r))
// normalised to 1 is the outer product of the returned 1-D weights g (sum 1).
// Returns K (1 = identity).
int gauss_1d(float radius, float* g, int cap);

// Filter dispatch used by the plain operators and the engine set-up.
int launch_filter(const asc_filter_desc& f, const float* in, float* out, int w, int h, cudaStream_t s);

// One plain ray-cast launch with an already folded float matrix.
int raycast_launch(const DevVolume& V, const uint8_t* occ, const float* m12, const float* vp, float step,
                   float intensity, float cutoff, float* out, int w, int h, cudaStream_t s);

}  // namespace asc
