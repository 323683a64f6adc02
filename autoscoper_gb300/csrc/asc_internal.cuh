// Internal declarations shared by the CUDA translation units of
// libautoscoper_gb300.so: status handling, the device volume layout, the
// FP32 ray march, FP64 rigid-frame algebra (host and device), and the
// reduction helpers.
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include <mutex>

#include "../../include/autoscoper_gb300.h"

#define ASC_API extern "C" __attribute__((visibility("default")))

namespace asc {

void set_cuda_error(cudaError_t e);
void set_error_message(const char* msg);
int cuda_status(cudaError_t e);
inline cudaStream_t S(void* s) { return (cudaStream_t)s; }

#define ASC_CUDA(call)                            \
  do {                                            \
    cudaError_t e_ = (call);                      \
    if (e_ != cudaSuccess) return cuda_status(e_); \
  } while (0)

#define ASC_LAUNCH_CHECK() ASC_CUDA(cudaGetLastError())

// Stream capture on one thread must not overlap a call on another thread that
// waits for the whole device (cudaDeviceSynchronize, cudaFree, pinned host
// allocation, synchronous copies): that wait would include the capturing
// stream, which fails the call and invalidates the capture.  Captures and
// every library call that allocates, frees or synchronizes the device hold
// this process-wide lock.
std::recursive_mutex& device_gate();
using Gate = std::lock_guard<std::recursive_mutex>;

}  // namespace asc

#include "asc_march.cuh"

namespace asc {

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

// Builds the occupancy grid of a device volume for one raw cutoff.
void build_occupancy(const DevVolume& V, float cutoff_raw, uint8_t* occ, cudaStream_t s);
inline size_t occupancy_cells(const DevVolume& V)
{
  return (size_t)occ_dim(V.nx) * occ_dim(V.ny) * occ_dim(V.nz);
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

// One axis of the film-plane mapping of RadRenderer / BackgroundRenderer
// (RadRenderer_kernels.cu:103-112, BackgroundRenderer_kernels.cu:103-116) and
// of tex2D's linear filter set-up, in FP64: pixel x of a crop n pixels wide
// over the viewport span [v0, v0 + vw) lands at the normalized coordinate
// s = (u - i0) / iw + 0.5 (columns) or s = 0.5 - (u - i0) / iw (rows, `rows`)
// of an image N texels wide; false when s leaves [0, 1] (the pixel is 0).
// Otherwise k receives the lower texel of the bilinear pair (floor(s N - 0.5),
// held to [-1, N] before the edge clamp) and a the weight of the upper one.
// In FP32 the coordinate s N - 0.5 of a 1024-texel image carries errors of
// ~1e-4 texel, which on a noisy radiograph moves the sample by ~5e-6; the
// FP64 mapping leaves only the FP32 interpolation's rounding.  Every pixel
// of a column (row) shares its column's (row's) mapping, so a tile computes
// it once per column and once per row.
__host__ __device__ __forceinline__ bool image_axis(double v0, double vw, int x, int n, double i0, double iw, int N,
                                                    bool rows, int& k, float& a)
{
  const double u = v0 + vw * ((double)x / (double)n);
  const double q = (u - i0) / iw;
  const double s = rows ? 0.5 - q : q + 0.5;
  if (s < 0.0 || s > 1.0) return false;
  const double X = s * N - 0.5;
  double fl = floor(X);
  a = (float)(X - fl);
  fl = fmin(fmax(fl, -1.0), (double)N);
  k = (int)fl;
  return true;
}

// Bilinear read of an 8/16-bit (normalized) or float image at the pair
// (x0, x0 + 1) x (y0, y0 + 1) with weights (ax, ay), clamp-to-edge, as
// tex2D<float> with the reference's texture object (cutil_create_tex_obj.h:6-28).
__device__ __forceinline__ float bilinear_at(const void* img, int bps, int W, int H, int x0, float ax, int y0,
                                             float ay)
{
  int xa = min(max(x0, 0), W - 1), xb = min(max(x0 + 1, 0), W - 1);
  int ya = min(max(y0, 0), H - 1), yb = min(max(y0 + 1, 0), H - 1);
  float v00 = image_texel(img, bps, ya * W + xa), v01 = image_texel(img, bps, ya * W + xb);
  float v10 = image_texel(img, bps, yb * W + xa), v11 = image_texel(img, bps, yb * W + xb);
  float r0 = fmaf(ax, v01 - v00, v00), r1 = fmaf(ax, v11 - v10, v10);
  return fmaf(ay, r1 - r0, r0);
}

// Whether the reference's multi-level sum() of n elements drops any: only a
// level whose thread count is not a power of two does (tree_keep).
__host__ __device__ __forceinline__ bool tree_needed(unsigned n)
{
  while (n > 1) {
    unsigned T = n < 256u ? n : 256u;
    if (T & (T - 1)) return true;
    n = (n + T - 1) / T;
  }
  return false;
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

// ---- compensated FP32 sums ----
// A double-float accumulator, value = h + l: each addition is Knuth's
// TwoSum (the rounding error of h + x, exact in FP32, is carried in l) and
// each product is split exactly into its rounded value and the FMA residual
// x y - RN(x y).  The sums of a tile's pixels then carry ~2^-44 relative
// error instead of FP32's accumulated ~2^-20.  The _rn intrinsics keep the
// compiler from contracting or reordering the error terms.
struct DFs {
  float h, l;
};

__device__ __forceinline__ void dfs_add(DFs& a, float x)
{
  const float s = __fadd_rn(a.h, x);
  const float bp = __fsub_rn(s, a.h);
  const float e = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bp)), __fsub_rn(x, bp));
  a.h = s;
  a.l = __fadd_rn(a.l, e);
}

__device__ __forceinline__ void dfs_add_prod(DFs& a, float x, float y)
{
  const float p = __fmul_rn(x, y);
  dfs_add(a, p);
  a.l = __fadd_rn(a.l, __fmaf_rn(x, y, -p));
}

__device__ __forceinline__ void dfs_merge(DFs& a, const DFs& b)
{
  dfs_add(a, b.h);
  a.l = __fadd_rn(a.l, b.l);
}

// Block-wide sums of N compensated accumulators: a TwoSum butterfly within
// each warp, then the warps' pairs added in FP64 by N threads.  red: 2 N
// floats per warp of the block; out (shared): the N sums, visible to every
// thread on return.
template <int N>
__device__ __forceinline__ void block_sum_dfs(DFs (&v)[N], float* red, double* out)
{
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < N; ++k)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      DFs b = {__shfl_xor_sync(0xffffffffu, v[k].h, o), __shfl_xor_sync(0xffffffffu, v[k].l, o)};
      dfs_merge(v[k], b);
    }
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < N; ++k) {
      red[(warp * N + k) * 2] = v[k].h;
      red[(warp * N + k) * 2 + 1] = v[k].l;
    }
  __syncthreads();
  if (threadIdx.x < N) {
    double t = 0.0;
    for (int j = 0; j < nw; ++j) t += (double)red[(j * N + threadIdx.x) * 2] + (double)red[(j * N + threadIdx.x) * 2 + 1];
    out[threadIdx.x] = t;
  }
  __syncthreads();
}

// Block-wide FP32 sums of N values (a shuffle butterfly per warp, the warps'
// sums added in FP64 by N threads); out (shared) is visible to every thread
// on return.  red: N floats per warp.
template <int N>
__device__ __forceinline__ void block_sum_f(float (&v)[N], float* red, double* out)
{
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < N; ++k)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < N; ++k) red[warp * N + k] = v[k];
  __syncthreads();
  if (threadIdx.x < N) {
    double t = 0.0;
    for (int j = 0; j < nw; ++j) t += (double)red[j * N + threadIdx.x];
    out[threadIdx.x] = t;
  }
  __syncthreads();
}

// One tile's Moments from its compensated sums: s = (sum mask, sum f, sum g
// over covered pixels; count, sum f, sum g over mask > 0.5) and the
// co-moments c = (ff, gg, fg) taken about the FP32 centres (cf, cg).  The
// exact tile means replace the centres, with the co-moments moved to them
// (C - n (mean - centre)(mean' - centre')), so the FP64 merge sees exact
// centred moments whatever the centres' rounding.
__device__ __forceinline__ Moments tile_moments(const double* s, const double* c, float cf, float cg)
{
  Moments p = {s[0], s[1], s[2], s[3], 0.0, 0.0, 0.0, 0.0, 0.0};
  if (s[3] > 0) {
    const double n = s[3], mf = s[4] / n, mg = s[5] / n, df = mf - (double)cf, dg = mg - (double)cg;
    p.mf = mf;
    p.mg = mg;
    // sums of squares about the mean: rounding must not leave them below 0
    // (a tile of equal values gives C = n (mean - centre)^2 up to rounding)
    const double ff = c[0] - n * df * df, gg = c[1] - n * dg * dg;
    p.cff = ff < 0.0 ? 0.0 : ff;
    p.cgg = gg < 0.0 ? 0.0 : gg;
    p.cfg = c[2] - n * df * dg;
  }
  return p;
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
  if (d1 < 0.0) d1 = 0.0;  // sums of squares (a NaN stays NaN)
  if (d2 < 0.0) d2 = 0.0;
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

// CoordFrame::linear_extrap (CoordFrame.cpp:419-476): from a at frame f - 2d
// and b at f - d, the pose at f: b's translation step doubled, and a rotated
// by twice the angle (about the axis) of the rotation from a to b.
inline void frame_linear_extrap(const double* a, const double* b, double* out)
{
  const double PI = 3.14159265358979323846, t = 2.0;
  const double trans[3] = {t * (b[9] - a[9]), t * (b[10] - a[10]), t * (b[11] - a[11])};
  double A[9];  // a's rotation applied to b's, as the reference's element order
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) A[3 * r + c] = b[c] * a[r] + b[3 + c] * a[3 + r] + b[6 + c] * a[6 + r];
  const double ang = acos((A[0] + A[4] + A[8] - 1.0) / 2.0);
  double axis[3] = {1.0, 0.0, 0.0};  // angle 0: any axis
  if (ang > 0.0 && ang < PI) {
    axis[0] = A[5] - A[7];
    axis[1] = A[6] - A[2];
    axis[2] = A[1] - A[3];
  }
  for (int i = 0; i < 12; ++i) out[i] = a[i];
  frame_rotate(out, axis, t * 180.0 * ang / PI);
  out[9] += trans[0];
  out[10] += trans[1];
  out[11] += trans[2];
}

// A float quaternion (Quat<float>: w, x, y, z).
struct QuatF {
  float w, x, y, z;
};

// Quat<float>(yaw, pitch, roll) (Quaternion.hpp:80-94), degrees, float math.
inline QuatF quat_from_ypr(float yaw, float pitch, float roll)
{
  const float pi = (float)3.14159265358979323846;
  const float cr = cosf(roll * pi / 360.0f), sr = sinf(roll * pi / 360.0f);
  const float cp = cosf(pitch * pi / 360.0f), sp = sinf(pitch * pi / 360.0f);
  const float cy = cosf(yaw * pi / 360.0f), sy = sinf(yaw * pi / 360.0f);
  return {cr * cp * cy + sr * sp * sy, sr * cp * cy - cr * sp * sy, cr * sp * cy + sr * cp * sy,
          cr * cp * sy - sr * sp * cy};
}

// Quat<float>::toEuler (Quaternion.hpp:220-243) read as (yaw, pitch, roll) =
// (e.z, e.y, e.x), degrees.
inline void quat_to_ypr(const QuatF& q, double* ypr)
{
  const float pi = (float)3.14159265358979323846;
  const float w = q.w, x = q.x, y = q.y, z = q.z;
  const float rx = atan2f(2.0f * (w * x + y * z), 1.0f - 2.0f * (x * x + y * y));
  const float ry = 2.0f * atan2f(sqrtf(1.0f + 2.0f * (w * y - x * z)), sqrtf(1.0f - 2.0f * (w * y - x * z))) - pi / 2.0f;
  const float rz = atan2f(2.0f * (w * z + x * y), 1.0f - 2.0f * (y * y + z * z));
  ypr[0] = rz * (180.0f / pi);
  ypr[1] = ry * (180.0f / pi);
  ypr[2] = rx * (180.0f / pi);
}

// The pose a trial's key curves hold after Tracker::optimize stores v and
// reads it back (Tracker.cpp:422-438): x, y, z as float; the rotation as a
// float quaternion from (yaw, pitch, roll) (Quaternion.hpp:80-94) read back
// as Euler angles (Quaternion.hpp:220-243), in float math as there.
inline void keycurve_store(const double* v, double* out)
{
  const QuatF q = quat_from_ypr((float)v[3], (float)v[4], (float)v[5]);
  double o[6] = {(float)v[0], (float)v[1], (float)v[2], 0, 0, 0};
  quat_to_ypr(q, o + 3);
  for (int i = 0; i < 6; ++i) out[i] = o[i];
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
