// Plain per-operator kernels of the registration cost path and their C ABI:
// one launch per reference operator call, the drop-in form of
// libautoscoper/src/gpu/cuda/*.  The batched engine (asc_engine.cu) reuses
// the same device functions.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "asc_internal.cuh"

namespace asc {

static thread_local std::string g_last_error;

void set_cuda_error(cudaError_t e) { g_last_error = cudaGetErrorString(e); }
void set_error_message(const char* msg) { g_last_error = msg; }

int cuda_status(cudaError_t e)
{
  set_cuda_error(e);
  (void)cudaGetLastError();  // clear a non-sticky error so the context stays usable
  return e == cudaErrorMemoryAllocation ? ASC_ERR_NOMEM : ASC_ERR_CUDA;
}

int gauss_1d(float radius, float* g, int cap)
{
  if (radius < 0) radius = 0;
  int R = (int)(3 * radius);  // float -> int truncation as GaussianFilter.cpp:79
  int K = 2 * R + 1;
  if (K == 1) return 1;
  if (K > cap) return -1;
  double e[128], sum = 0;
  for (int i = 0; i < K; ++i) {
    e[i] = pow(2.71828, -pow((double)(i - R), 2) / (2 * radius));
    sum += e[i];
  }
  for (int i = 0; i < K; ++i) g[i] = (float)(e[i] / sum);
  return K;
}

// ---------------------------------------------------------------- kernels

// cuda_volume_render_kernel (RayCaster_kernels.cu:144-195) for one image.
// 16x16 pixel blocks; each warp covers an 8x4 sub-tile so that its rays
// sample neighbouring voxels.
struct RayArgs {
  float m[12];
  float vp[4];
  float step, scale;
  Cutoff cut;
  float sx[2], sy[2];  // vp[2] / w and vp[3] / h as double-floats
};

template <int STORE>
__global__ void __launch_bounds__(256) k_raycast(DevVolume V, const uint8_t* __restrict__ occ, RayArgs a,
                                                 float* __restrict__ out, int w, int h)
{
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int x = blockIdx.x * 16 + (warp & 1) * 8 + (lane & 7);
  const int y = blockIdx.y * 16 + (warp >> 1) * 4 + (lane >> 3);
  if (x >= w || y >= h) return;
  RaySetup r;
  float d = 0.f;
  if (ray_setup(a.m, a.vp, x, y, df{a.sx[0], a.sx[1]}, df{a.sy[0], a.sy[1]}, a.step, V.nx, V.ny, V.nz, r))
    d = march<STORE>(V, occ, r, a.cut) * a.scale;
  out[(size_t)y * w + x] = fminf(fmaxf(d, 0.f), 1.f);
}

// image_render_kernel (RadRenderer_kernels.cu:85-116) and
// background_render_kernel (BackgroundRenderer_kernels.cu:88-120).
struct ImgArgs {
  float ip[4], vp[4];
  float threshold;
  int mode;  // 0 radiograph, 1 background mask
};

__global__ void __launch_bounds__(256) k_image_render(const void* __restrict__ img, int bps, int W, int H, ImgArgs a,
                                                      float* __restrict__ out, int w, int h)
{
  // the film-plane mapping of the block's 32 columns and 8 rows, in FP64
  // (image_axis), shared by its pixels
  __shared__ int s_k[40];
  __shared__ float s_a[40];
  const int t = threadIdx.y * 32 + threadIdx.x;
  if (t < 40) {
    const bool row = t >= 32;
    const int j = row ? blockIdx.y * 8 + (t - 32) : blockIdx.x * 32 + t;
    int k = 0;
    float wgt = 0.f;
    const bool ok = row ? j < h && image_axis(a.vp[1], a.vp[3], j, h, a.ip[1], a.ip[3], H, true, k, wgt)
                        : j < w && image_axis(a.vp[0], a.vp[2], j, w, a.ip[0], a.ip[2], W, false, k, wgt);
    s_k[t] = ok ? k : INT_MIN;
    s_a[t] = wgt;
  }
  __syncthreads();
  int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
  if (x >= w || y >= h) return;
  const int kx = s_k[threadIdx.x], ky = s_k[32 + threadIdx.y];
  float r = 0.f;
  if (kx != INT_MIN && ky != INT_MIN) {
    float v = bilinear_at(img, bps, W, H, kx, s_a[threadIdx.x], ky, s_a[32 + threadIdx.y]);
    r = a.mode == 0 ? 1.0f - v : (a.threshold <= v ? 1.0f : 0.0f);
  }
  out[(size_t)y * w + x] = r;
}

// Elementwise operators (DRRBackground / Mult / Merger / Compositor kernels).
__global__ void k_elementwise(int op, const float* __restrict__ a, const float* __restrict__ b,
                              const float* __restrict__ c, float* __restrict__ d, size_t n, float val)
{
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    switch (op) {
      case 0: d[i] = a[i] != 0.0f ? 1.0f : 0.0f; break;
      case 1: d[i] = a[i] * b[i]; break;
      case 2: d[i] = (float)fmin((double)(a[i] + b[i]), 1.0); break;
      case 3: {
        float multi = c[i] < 0.5f ? 0.0f : 1.0f;
        float s1 = a[i], s2 = b[i];
        d[3 * i + 0] = s1;
        d[3 * i + 1] = multi * (s1 / 2.0f + s2 / 2.0f);
        d[3 * i + 2] = s2;
        break;
      }
      default: d[i] = val; break;
    }
  }
}

// ---- 2-D stencil filters, 32x32 output tiles staged in shared memory ----
// Out-of-image positions of the staged tile hold 0, so a tap that falls
// outside the image contributes nothing: the "skip" rule of the reference's
// Gaussian/Sharpen (GaussianFilter_kernels.cu:66-89) and, because the
// weights are an outer product, the 2-D sum splits exactly into a
// horizontal and a vertical pass.
constexpr int FT = 32;  // output tile edge

struct StencilArgs {
  int kind;    // 0 contrast, 1 sobel, 3 gaussian, 4 sharpen
  int K;       // taps per axis (gaussian / sharpen) or window (contrast)
  float p0, p1, p2;
  float g[64];
};

__global__ void __launch_bounds__(256) k_stencil(const float* __restrict__ in, float* __restrict__ out, int w, int h,
                                                 StencilArgs a)
{
  extern __shared__ float sm[];
  const int R = a.kind == 1 ? 1 : (a.kind == 0 ? (a.K / 2 > (a.K - 1) / 2 ? a.K / 2 : (a.K - 1) / 2) : a.K / 2);
  const int E = FT + 2 * R;  // staged edge
  float* tile = sm;           // E x E
  float* hp = sm + E * E;     // E rows x FT (horizontal pass)
  const int x0 = blockIdx.x * FT - R, y0 = blockIdx.y * FT - R;
  for (int i = threadIdx.x; i < E * E; i += blockDim.x) {
    int ty = i / E, tx = i % E, gx = x0 + tx, gy = y0 + ty;
    tile[i] = (gx >= 0 && gx < w && gy >= 0 && gy < h) ? __ldg(in + (size_t)gy * w + gx) : 0.0f;
  }
  __syncthreads();
  if (a.kind == 3 || a.kind == 4) {
    for (int i = threadIdx.x; i < E * FT; i += blockDim.x) {
      int ty = i / FT, tx = i % FT;
      float s = 0.f;
      for (int k = 0; k < a.K; ++k) s = fmaf(a.g[k], tile[ty * E + tx + k], s);
      hp[i] = s;
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < FT * FT; i += blockDim.x) {
    int ty = i / FT, tx = i % FT;
    int gx = blockIdx.x * FT + tx, gy = blockIdx.y * FT + ty;
    if (gx >= w || gy >= h) continue;
    float f = tile[(ty + R) * E + tx + R], r;
    if (a.kind == 3 || a.kind == 4) {
      float blur = 0.f;
      for (int k = 0; k < a.K; ++k) blur = fmaf(a.g[k], hp[(ty + k) * FT + tx], blur);
      if (a.kind == 3) {
        r = fminf(fmaxf(blur, 0.f), 1.f);
      } else {
        r = fabsf(f - blur) > a.p2 ? fminf(fmaxf(f + a.p1 * (f - blur), 0.f), 1.f) : f;
      }
    } else if (a.kind == 1) {
      // Sobel with clamp-to-edge neighbours (SobelFilter_kernels.cu:69-96)
      int xm = gx > 0 ? -1 : 0, xp = gx < w - 1 ? 1 : 0, ym = gy > 0 ? -1 : 0, yp = gy < h - 1 ? 1 : 0;
      const float* c = tile + (ty + R) * E + tx + R;
      float p00 = c[ym * E + xm], p01 = c[ym * E], p02 = c[ym * E + xp];
      float p10 = c[xm], p12 = c[xp];
      float p20 = c[yp * E + xm], p21 = c[yp * E], p22 = c[yp * E + xp];
      float horz = p02 + 2 * p12 + p22 - p00 - 2 * p10 - p20;
      float vert = p00 + 2 * p01 + p02 - p20 - 2 * p21 - p22;
      float grad = sqrtf(horz * horz + vert * vert);
      float s = a.p1 < 0.5f ? a.p0 * grad + 2.0f * a.p1 * f : 2.0f * (1.0f - a.p1) * a.p0 * grad + f;
      r = fminf(fmaxf(s, 0.f), 1.f);
    } else {
      // Contrast: box mean over the in-image part of the window
      // (ContrastFilter_kernels.cu:64-80), then axy^(a-b) * f^b.
      int size = a.K;
      int i0 = max(gy - size / 2, 0), i1 = min(gy + (size + 1) / 2, h);
      int j0 = max(gx - size / 2, 0), j1 = min(gx + (size + 1) / 2, w);
      float n = 0.f, s = 0.f;
      for (int yy = i0; yy < i1; ++yy)
        for (int xx = j0; xx < j1; ++xx) {
          n += 1.0f;
          s += tile[(yy - y0) * E + (xx - x0)];
        }
      float axy = s / n;
      r = axy > 0.01f ? powf(axy, a.p0 - a.p1) * powf(f, a.p1) : 0.0f;
    }
    out[(size_t)gy * w + gx] = r;
  }
}

// ---- cost reductions ----
constexpr int RB = 256;          // threads per reduction block
constexpr int RE = 16;           // elements per thread
constexpr int RCHUNK = RB * RE;  // elements per block

template <class T>
__device__ __forceinline__ T warp_sum(T v)
{
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum of up to 6 floats (pairwise: shuffle tree, then warps).
template <int N>
__device__ __forceinline__ void block_sum(float (&v)[N], float* red)
{
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < N; ++k) v[k] = warp_sum(v[k]);
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < N; ++k) red[warp * N + k] = v[k];
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < N; ++k) {
      float x = lane < nw ? red[lane * N + k] : 0.f;
      v[k] = warp_sum(x);
    }
    if (lane == 0)
#pragma unroll
      for (int k = 0; k < N; ++k) red[k] = v[k];
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < N; ++k) v[k] = red[k];
  __syncthreads();
}

struct ReduceScratch {
  Moments* part;        // one per block
  double* means;        // hdist: (mF, mG)
  unsigned* ticket;     // last-block election
};

// Merges `nb` partials in FP64 with one block; returns the result in m (thread 0).
__device__ void merge_partials(const Moments* part, int nb, Moments& m)
{
  __shared__ Moments sh[RB];
  Moments a = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int i = threadIdx.x; i < nb; i += blockDim.x) moments_merge(a, part[i]);
  sh[threadIdx.x] = a;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) moments_merge(sh[threadIdx.x], sh[threadIdx.x + s]);
    __syncthreads();
  }
  m = sh[0];
}

// NCC (Ncc_kernels.cu:116-213) in one launch: each block computes the
// moments of its 4096 elements in two passes over registers, the last block
// to finish merges all partials in FP64 and writes the correlation.
__global__ void __launch_bounds__(RB) k_ncc(const float* __restrict__ f, const float* __restrict__ g,
                                            const float* __restrict__ mask, unsigned n, int tree, ReduceScratch sc,
                                            double* __restrict__ result)
{
  __shared__ float red[(RB / 32) * 6 * 2];
  __shared__ double ds[6], dc[3];
  __shared__ bool last;
  float fv[RE], gv[RE], mv[RE];
  unsigned flags = 0;  // bit k: covered; bit 16+k: covered and mask > 0.5
  const size_t base = (size_t)blockIdx.x * RCHUNK + threadIdx.x;
  DFs s[6] = {};  // sm, sf, sg (covered), n, sf, sg (masked)
#pragma unroll
  for (int k = 0; k < RE; ++k) {
    size_t i = base + (size_t)k * RB;
    fv[k] = gv[k] = mv[k] = 0.f;
    if (i < n && (!tree || tree_keep((unsigned)i, n))) {
      fv[k] = __ldg(f + i);
      gv[k] = __ldg(g + i);
      mv[k] = __ldg(mask + i);
      flags |= 1u << k;
      dfs_add(s[0], mv[k]);
      dfs_add(s[1], fv[k]);
      dfs_add(s[2], gv[k]);
      if (mv[k] > 0.5f) {
        flags |= 1u << (16 + k);
        dfs_add(s[3], 1.f);
        dfs_add(s[4], fv[k]);
        dfs_add(s[5], gv[k]);
      }
    }
  }
  block_sum_dfs<6>(s, red, ds);
  const double cnt = ds[3];
  const float mf = cnt > 0 ? (float)(ds[4] / cnt) : 0.f, mg = cnt > 0 ? (float)(ds[5] / cnt) : 0.f;
  DFs c[3] = {};
#pragma unroll
  for (int k = 0; k < RE; ++k)
    if (flags & (1u << (16 + k))) {
      float a = fv[k] - mf, b = gv[k] - mg;
      dfs_add_prod(c[0], a, a);
      dfs_add_prod(c[1], b, b);
      dfs_add_prod(c[2], a, b);
    }
  block_sum_dfs<3>(c, red, dc);
  if (threadIdx.x == 0) {
    Moments p = tile_moments(ds, dc, mf, mg);
    sc.part[blockIdx.x] = p;
    __threadfence();
    last = atomicAdd(sc.ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  Moments m;
  merge_partials(sc.part, gridDim.x, m);
  if (threadIdx.x == 0) {
    *result = moments_ncc(m);
    *sc.ticket = 0;
  }
}

// SAD ("hdist", HDist_kernels.cu:111-203): pass 1 computes the masked means
// (as k_ncc's covered sums), pass 2 sums |(f-mF)-(g-mG)| over mask > 0.5.
__global__ void __launch_bounds__(RB) k_hdist_means(const float* __restrict__ f, const float* __restrict__ g,
                                                    const float* __restrict__ mask, unsigned n, int tree,
                                                    ReduceScratch sc)
{
  __shared__ float red[(RB / 32) * 3];
  __shared__ bool last;
  float s[3] = {0, 0, 0};
  const size_t base = (size_t)blockIdx.x * RCHUNK + threadIdx.x;
  for (int k = 0; k < RE; ++k) {
    size_t i = base + (size_t)k * RB;
    if (i < n && (!tree || tree_keep((unsigned)i, n))) {
      s[0] += __ldg(mask + i);
      s[1] += __ldg(f + i);
      s[2] += __ldg(g + i);
    }
  }
  block_sum<3>(s, red);
  if (threadIdx.x == 0) {
    Moments p = {s[0], s[1], s[2], 0, 0, 0, 0, 0, 0};
    sc.part[blockIdx.x] = p;
    __threadfence();
    last = atomicAdd(sc.ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  Moments m;
  merge_partials(sc.part, gridDim.x, m);
  if (threadIdx.x == 0) {
    sc.means[0] = m.sf / m.sm;
    sc.means[1] = m.sg / m.sm;
    *sc.ticket = 0;
  }
}

__global__ void __launch_bounds__(RB) k_hdist_sad(const float* __restrict__ f, const float* __restrict__ g,
                                                  const float* __restrict__ mask, unsigned n, int tree,
                                                  ReduceScratch sc, double* __restrict__ result)
{
  __shared__ float red[RB / 32];
  __shared__ bool last;
  const float mF = (float)sc.means[0], mG = (float)sc.means[1];
  float s[1] = {0};
  const size_t base = (size_t)blockIdx.x * RCHUNK + threadIdx.x;
  for (int k = 0; k < RE; ++k) {
    size_t i = base + (size_t)k * RB;
    if (i < n && (!tree || tree_keep((unsigned)i, n)) && __ldg(mask + i) > 0.5f)
      s[0] += fabsf((__ldg(f + i) - mF) - (__ldg(g + i) - mG));
  }
  block_sum<1>(s, red);
  if (threadIdx.x == 0) {
    Moments p = {s[0], 0, 0, 0, 0, 0, 0, 0, 0};
    sc.part[blockIdx.x] = p;
    __threadfence();
    last = atomicAdd(sc.ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  Moments m;
  merge_partials(sc.part, gridDim.x, m);
  if (threadIdx.x == 0) {
    *result = m.sm;
    *sc.ticket = 0;
  }
}

// Occupancy bytes and boxes of OCC^3-voxel cells (occ_cell in asc_march.cuh),
// margin cells included: one thread per cell scans the cell and its apron
// (voxels outside the volume are 0).
template <int STORE>
__global__ void k_occupancy(DevVolume V, float cutoff_raw, uint8_t* __restrict__ occ)
{
  const int px = occ_dim(V.nx), py = occ_dim(V.ny), pz = occ_dim(V.nz);
  const int n = px * py * pz;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const int cx = c % px - OCC_PAD, cy = (c / px) % py - OCC_PAD, cz = c / (px * py) - OCC_PAD;
  int box[4];
  occ[c] = occ_cell(cx, cy, cz, V.nx, V.ny, V.nz, cutoff_raw,
                    [&](int x, int y, int z) {
                      return voxel_value<STORE>(V, (size_t)(z + PAD) * V.pxy + (size_t)(y + PAD) * V.px + (x + PAD));
                    },
                    box);
  reinterpret_cast<int4*>(occ + occ_box_offset((size_t)n))[c] = make_int4(box[0], box[1], box[2], box[3]);
}

int g_empty_skip = 1;

void build_occupancy(const DevVolume& V, float cutoff_raw, uint8_t* occ, cudaStream_t s)
{
  int n = (int)occupancy_cells(V);
  if (V.storage == ASC_STORE_F32)
    k_occupancy<ASC_STORE_F32><<<(n + 127) / 128, 128, 0, s>>>(V, cutoff_raw, occ);
  else if (V.storage == ASC_STORE_BF16)
    k_occupancy<ASC_STORE_BF16><<<(n + 127) / 128, 128, 0, s>>>(V, cutoff_raw, occ);
  else if (V.storage == ASC_STORE_F16)
    k_occupancy<ASC_STORE_F16><<<(n + 127) / 128, 128, 0, s>>>(V, cutoff_raw, occ);
  else
    k_occupancy<ASC_STORE_U16><<<(n + 127) / 128, 128, 0, s>>>(V, cutoff_raw, occ);
}

// ---------------------------------------------------------------- host side

int launch_filter(const asc_filter_desc& f, const float* in, float* out, int w, int h, cudaStream_t s)
{
  if (w <= 0 || h <= 0) return ASC_OK;
  StencilArgs a;
  memset(&a, 0, sizeof a);
  a.kind = f.kind;
  a.p0 = f.p0;
  a.p1 = f.p1;
  a.p2 = f.p2;
  int R;
  if (f.kind == 1) {
    a.K = 3;
    R = 1;
  } else if (f.kind == 0) {
    a.K = (int)f.p2;
    if (a.K < 1) return ASC_ERR_ARG;
    R = std::max(a.K / 2, (a.K - 1) / 2);
    if (R > 16) return ASC_ERR_RANGE;
  } else if (f.kind == 3 || f.kind == 4) {
    a.K = gauss_1d(f.p0, a.g, 64);
    if (a.K < 0) return ASC_ERR_RANGE;
    if (a.K == 1) {
      ASC_CUDA(cudaMemcpyAsync(out, in, (size_t)w * h * sizeof(float), cudaMemcpyDeviceToDevice, s));
      return ASC_OK;
    }
    if (f.kind == 4) a.p1 = f.p1 < 1 ? 1 : f.p1;  // SharpenFilter::set_contrast
    R = a.K / 2;
  } else {
    return ASC_ERR_ARG;
  }
  int E = FT + 2 * R;
  size_t smem = (size_t)(E * E + E * FT) * sizeof(float);
  static std::once_flag once;
  std::call_once(once, [] { cudaFuncSetAttribute(k_stencil, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024); });
  dim3 grid((w + FT - 1) / FT, (h + FT - 1) / FT);
  k_stencil<<<grid, 256, smem, s>>>(in, out, w, h, a);
  ASC_LAUNCH_CHECK();
  return ASC_OK;
}

// Per-process reduction scratch sized by asc_ncc_init (the reference keeps
// module globals too, Ncc_kernels.cu:50-57).  It lives on the device that was
// current when it was sized; every read or change of it holds g_red_mu.
static std::mutex g_red_mu;
static Moments* g_part = nullptr;
static double* g_means = nullptr;
static unsigned* g_ticket = nullptr;
static unsigned g_max_n = 0;
static int g_red_dev = -1;

std::recursive_mutex& device_gate()
{
  static std::recursive_mutex m;
  return m;
}

static int ncc_init_locked(unsigned max_n);

// The scratch for n elements on the current device, copied out under the
// lock: a thread that grows it frees the old buffers only after taking the
// lock (and cudaFree waits for the kernels still using them).  Scratch sized
// on another device is ASC_ERR_STATE: like the reference's module globals it
// serves one device per process.
static int ensure_scratch(unsigned n, ReduceScratch* out)
{
  std::lock_guard<std::mutex> l(g_red_mu);
  int dev = 0;
  ASC_CUDA(cudaGetDevice(&dev));
  if (g_part && dev != g_red_dev) {
    set_error_message("asc_ncc/asc_hdist: the reduction scratch belongs to another device (asc_ncc_init there)");
    return ASC_ERR_STATE;
  }
  if (!(n <= g_max_n && g_part)) {
    int rc = ncc_init_locked(n);
    if (rc) return rc;
  }
  *out = ReduceScratch{g_part, g_means, g_ticket};
  return ASC_OK;
}

}  // namespace asc

using namespace asc;

// ---------------------------------------------------------------- C ABI

ASC_API const char* asc_version(void) { return "autoscoper_gb300 0.1 (sm_103a)"; }

ASC_API const char* asc_status_string(int st)
{
  switch (st) {
    case ASC_OK: return "ok";
    case ASC_ERR_ARG: return "bad argument";
    case ASC_ERR_CUDA: return "CUDA error";
    case ASC_ERR_EMPTY: return "empty volume";
    case ASC_ERR_RANGE: return "size out of range";
    case ASC_ERR_NOMEM: return "out of device memory";
    case ASC_ERR_TIMEOUT: return "device wait timed out";
    case ASC_ERR_STATE: return "call out of order";
  }
  return "unknown status";
}

ASC_API const char* asc_last_error(void) { return g_last_error.c_str(); }

ASC_API int asc_set_option(int option, int value)
{
  if (option == ASC_OPT_EMPTY_SKIP) {
    g_empty_skip = value != 0;
    return ASC_OK;
  }
  return ASC_ERR_ARG;
}

ASC_API int asc_malloc(void** p, size_t bytes)
{
  if (!p) return ASC_ERR_ARG;
  Gate g(device_gate());
  ASC_CUDA(cudaMalloc(p, bytes ? bytes : 1));
  return ASC_OK;
}
ASC_API int asc_free(void* p)
{
  Gate g(device_gate());
  ASC_CUDA(cudaFree(p));
  return ASC_OK;
}
ASC_API int asc_memcpy_h2d(void* d, const void* s, size_t n, void* st)
{
  ASC_CUDA(cudaMemcpyAsync(d, s, n, cudaMemcpyHostToDevice, S(st)));
  return ASC_OK;
}
ASC_API int asc_memcpy_d2h(void* d, const void* s, size_t n, void* st)
{
  ASC_CUDA(cudaMemcpyAsync(d, s, n, cudaMemcpyDeviceToHost, S(st)));
  ASC_CUDA(cudaStreamSynchronize(S(st)));
  return ASC_OK;
}
ASC_API int asc_memcpy_d2d(void* d, const void* s, size_t n, void* st)
{
  ASC_CUDA(cudaMemcpyAsync(d, s, n, cudaMemcpyDeviceToDevice, S(st)));
  return ASC_OK;
}
ASC_API int asc_memset(void* d, int v, size_t n, void* st)
{
  ASC_CUDA(cudaMemsetAsync(d, v, n, S(st)));
  return ASC_OK;
}
ASC_API int asc_stream_sync(void* st)
{
  ASC_CUDA(cudaStreamSynchronize(S(st)));
  return ASC_OK;
}
ASC_API int asc_device_sync(void)
{
  Gate g(device_gate());
  ASC_CUDA(cudaDeviceSynchronize());
  return ASC_OK;
}
ASC_API int asc_set_device(int d)
{
  ASC_CUDA(cudaSetDevice(d));
  return ASC_OK;
}
ASC_API int asc_stream_create(void** s)
{
  if (!s) return ASC_ERR_ARG;
  ASC_CUDA(cudaStreamCreateWithFlags((cudaStream_t*)s, cudaStreamNonBlocking));
  return ASC_OK;
}
ASC_API int asc_stream_destroy(void* s)
{
  ASC_CUDA(cudaStreamDestroy(S(s)));
  return ASC_OK;
}
ASC_API int asc_event_create(void** e)
{
  if (!e) return ASC_ERR_ARG;
  ASC_CUDA(cudaEventCreate((cudaEvent_t*)e));
  return ASC_OK;
}
ASC_API int asc_event_record(void* e, void* s)
{
  ASC_CUDA(cudaEventRecord((cudaEvent_t)e, S(s)));
  return ASC_OK;
}
ASC_API int asc_event_elapsed(void* a, void* b, float* ms)
{
  if (!ms) return ASC_ERR_ARG;
  ASC_CUDA(cudaEventSynchronize((cudaEvent_t)b));
  ASC_CUDA(cudaEventElapsedTime(ms, (cudaEvent_t)a, (cudaEvent_t)b));
  return ASC_OK;
}
ASC_API int asc_event_destroy(void* e)
{
  ASC_CUDA(cudaEventDestroy((cudaEvent_t)e));
  return ASC_OK;
}
ASC_API int asc_host_alloc(void** p, size_t n)
{
  if (!p) return ASC_ERR_ARG;
  Gate g(device_gate());
  ASC_CUDA(cudaMallocHost(p, n ? n : 1));
  return ASC_OK;
}
ASC_API int asc_host_free(void* p)
{
  Gate g(device_gate());
  ASC_CUDA(cudaFreeHost(p));
  return ASC_OK;
}
ASC_API int asc_mem_info(size_t* free_bytes, size_t* total_bytes)
{
  if (!free_bytes || !total_bytes) return ASC_ERR_ARG;
  ASC_CUDA(cudaMemGetInfo(free_bytes, total_bytes));
  return ASC_OK;
}

// ---- volumes (VolumeDescription.cpp:152-305) ----
template <class T>
static void describe(const T* data, int W, int H, int D, const int* flip, std::vector<T>& crop, int mn[3], int mx[3],
                     T& vmin, T& vmax)
{
  std::vector<T> fl((size_t)W * H * D);
  for (int k = 0; k < D; ++k)
    for (int i = 0; i < H; ++i)
      for (int j = 0; j < W; ++j) {
        int x = flip[0] ? W - 1 - j : j, y = flip[1] ? H - 1 - i : i, z = flip[2] ? D - 1 - k : k;
        fl[(size_t)z * W * H + (size_t)y * W + x] = data[(size_t)k * W * H + (size_t)i * W + j];
      }
  mn[0] = W; mn[1] = H; mn[2] = D;
  mx[0] = mx[1] = mx[2] = 0;
  size_t p = 0;
  for (int k = 0; k < D; ++k) {
    bool col = false;
    for (int i = 0; i < H; ++i) {
      bool row = false;
      for (int j = 0; j < W; ++j, ++p)
        if (fl[p] != T(0)) {
          mn[0] = std::min(mn[0], j);
          mx[0] = std::max(mx[0], j);
          row = true;
        }
      if (row) {
        mn[1] = std::min(mn[1], i);
        mx[1] = std::max(mx[1], i);
        col = true;
      }
    }
    if (col) {
      mn[2] = std::min(mn[2], k);
      mx[2] = std::max(mx[2], k);
    }
  }
  if (mn[0] > mx[0] || mn[1] > mx[1] || mn[2] > mx[2]) return;
  vmin = std::numeric_limits<T>::max();
  vmax = std::numeric_limits<T>::min();
  crop.clear();
  crop.reserve((size_t)(mx[0] - mn[0] + 1) * (mx[1] - mn[1] + 1) * (mx[2] - mn[2] + 1));
  for (int k = mn[2]; k <= mx[2]; ++k)
    for (int i = mn[1]; i <= mx[1]; ++i)
      for (int j = mn[0]; j <= mx[0]; ++j) {
        T v = fl[(size_t)k * W * H + (size_t)i * W + j];
        vmin = std::min(vmin, v);
        vmax = std::max(vmax, v);
        crop.push_back(v);
      }
}

// A voxel as stored: a 16-bit half (u16, IEEE half, bfloat16) or FP32 bits.
static uint32_t to_store(unsigned v, int storage)
{
  if (storage == ASC_STORE_F16) return __half_as_ushort(__float2half_rn((float)v));
  if (storage == ASC_STORE_BF16) return __bfloat16_as_ushort(__float2bfloat16_rn((float)v));
  if (storage == ASC_STORE_F32) {
    const float f = (float)v;
    uint32_t b;
    memcpy(&b, &f, 4);
    return b;
  }
  return (uint16_t)v;
}

ASC_API int asc_volume_create(const void* data, int W, int H, int D, int bps, const double scale[3],
                              const int flip[3], int storage, asc_volume* out)
{
  if (!data || !out || !scale || W <= 0 || H <= 0 || D <= 0) return ASC_ERR_ARG;
  if (bps != 8 && bps != 16) return ASC_ERR_ARG;
  if (storage < ASC_STORE_U16 || storage > ASC_STORE_F32) return ASC_ERR_ARG;
  static const int noflip[3] = {0, 0, 0};
  if (!flip) flip = noflip;
  int mn[3], mx[3];
  std::vector<unsigned> vals;
  unsigned vmin = 0, vmax = 0;
  if (bps == 8) {
    std::vector<uint8_t> crop;
    uint8_t a = 0, b = 0;
    describe((const uint8_t*)data, W, H, D, flip, crop, mn, mx, a, b);
    vals.assign(crop.begin(), crop.end());
    vmin = a; vmax = b;
  } else {
    std::vector<uint16_t> crop;
    uint16_t a = 0, b = 0;
    describe((const uint16_t*)data, W, H, D, flip, crop, mn, mx, a, b);
    vals.assign(crop.begin(), crop.end());
    vmin = a; vmax = b;
  }
  if (mn[0] > mx[0] || mn[1] > mx[1] || mn[2] > mx[2]) return ASC_ERR_EMPTY;
  // the march indexes the padded grid in 32-bit arithmetic
  if ((double)(mx[0] - mn[0] + 1 + 2 * PAD) * (mx[1] - mn[1] + 1 + 2 * PAD) * (mx[2] - mn[2] + 1 + 2 * PAD) >=
      2147483648.0)
    return ASC_ERR_RANGE;
  auto* v = new asc_volume_host();
  v->occ = nullptr;
  v->occ_cutoff = NAN;
  int dims[3] = {mx[0] - mn[0] + 1, mx[1] - mn[1] + 1, mx[2] - mn[2] + 1};
  float norm = bps == 8 ? 255.0f : 65535.0f;
  v->min_value = vmin / norm;
  v->max_value = vmax / norm;
  float sc[3] = {(float)scale[0], (float)scale[1], (float)scale[2]};
  v->trans_center[0] = -sc[0] * 0.5 * (mn[0] + mx[0]);
  v->trans_center[1] = -sc[1] * 0.5 * (mn[1] + mx[1]);
  v->trans_center[2] = sc[2] * 0.5 * (mn[2] + mx[2]);
  for (int a = 0; a < 3; ++a) {
    v->inv_scale[a] = 1.0f / (float)(sc[a] * dims[a]);
    v->dims[a] = dims[a];
  }
  v->inv_trans[0] = -mn[0] / (float)dims[0];
  v->inv_trans[1] = -((H - mx[1] - 1) / (float)dims[1]);
  v->inv_trans[2] = mn[2] / (float)dims[2];
  v->bps = bps;
  // x-paired words on the padded grid (see DevVolume)
  const size_t nwords = padded_words(dims[0], dims[1], dims[2], storage);
  std::vector<uint32_t> pairs(nwords);
  const int dx = dims[0], dxy = dims[0] * dims[1];
  pack_pairs(dims[0], dims[1], dims[2], storage,
             [&](int x, int y, int z) { return to_store(vals[(size_t)z * dxy + (size_t)y * dx + x], storage); },
             pairs.data());
  Gate g(device_gate());
  cudaError_t e = cudaMalloc(&v->pairs, nwords * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMemcpy(v->pairs, pairs.data(), nwords * sizeof(uint32_t), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    if (v->pairs) cudaFree(v->pairs);
    delete v;
    return cuda_status(e);
  }
  const int px = dims[0] + 2 * PAD, pxy = px * (dims[1] + 2 * PAD);
  // the stored values' largest neighbour step (the march's cutoff band)
  const float gmax = volume_gmax(dims[0], dims[1], dims[2], [&](int x, int y, int z) {
    const uint32_t w = to_store(vals[(size_t)z * dxy + (size_t)y * dx + x], storage);
    if (storage == ASC_STORE_F16) return __half2float(__ushort_as_half((unsigned short)w));
    if (storage == ASC_STORE_BF16) return __bfloat162float(__ushort_as_bfloat16((unsigned short)w));
    if (storage == ASC_STORE_F32) {
      float f;
      memcpy(&f, &w, 4);
      return f;
    }
    return (float)w;
  });
  v->dev = DevVolume{v->pairs, dims[0], dims[1], dims[2], px, pxy, storage, 1.0f / norm, gmax};
  *out = (asc_volume)v;
  return ASC_OK;
}

ASC_API int asc_volume_info(asc_volume vol, float inv_scale[3], float inv_trans[3], double trans_center[3],
                            float* min_value, float* max_value, int dims[3])
{
  auto* v = (asc_volume_host*)vol;
  if (!v) return ASC_ERR_ARG;
  for (int a = 0; a < 3; ++a) {
    if (inv_scale) inv_scale[a] = v->inv_scale[a];
    if (inv_trans) inv_trans[a] = v->inv_trans[a];
    if (trans_center) trans_center[a] = v->trans_center[a];
    if (dims) dims[a] = v->dims[a];
  }
  if (min_value) *min_value = v->min_value;
  if (max_value) *max_value = v->max_value;
  return ASC_OK;
}

ASC_API int asc_volume_destroy(asc_volume vol)
{
  auto* v = (asc_volume_host*)vol;
  if (!v) return ASC_ERR_ARG;
  Gate g(device_gate());
  cudaFree(v->pairs);
  if (v->occ) cudaFree(v->occ);
  delete v;
  return ASC_OK;
}

namespace asc {
int raycast_launch(const DevVolume& V, const uint8_t* occ, const float* m12, const float* vp, float step,
                   float intensity, float cutoff, float* out, int w, int h, cudaStream_t s)
{
  RayArgs a;
  memcpy(a.m, m12, sizeof a.m);
  memcpy(a.vp, vp, sizeof a.vp);
  a.step = step;
  // density = step * sum(norm * raw) / intensity; cutoff compares normalized samples
  a.scale = step * V.norm / intensity;
  a.cut = make_cutoff(cutoff, V.norm, V.gmax);
  df_split((double)vp[2] / (double)w, a.sx[0], a.sx[1]);
  df_split((double)vp[3] / (double)h, a.sy[0], a.sy[1]);
  dim3 grid((w + 15) / 16, (h + 15) / 16);
  if (V.storage == ASC_STORE_F32)
    k_raycast<ASC_STORE_F32><<<grid, 256, 0, s>>>(V, occ, a, out, w, h);
  else if (V.storage == ASC_STORE_BF16)
    k_raycast<ASC_STORE_BF16><<<grid, 256, 0, s>>>(V, occ, a, out, w, h);
  else if (V.storage == ASC_STORE_F16)
    k_raycast<ASC_STORE_F16><<<grid, 256, 0, s>>>(V, occ, a, out, w, h);
  else
    k_raycast<ASC_STORE_U16><<<grid, 256, 0, s>>>(V, occ, a, out, w, h);
  ASC_LAUNCH_CHECK();
  return ASC_OK;
}
}  // namespace asc

ASC_API int asc_raycast(asc_volume vol, const double imv[16], const float vp[4], float step, float intensity,
                        float cutoff, int visible, float* out, int w, int h, void* stream)
{
  auto* v = (asc_volume_host*)vol;
  if (!v) return ASC_ERR_STATE;  // RayCaster::render without a volume
  if (!imv || !vp || !out || w < 0 || h < 0) return ASC_ERR_ARG;
  if (w == 0 || h == 0) return ASC_OK;
  if (!visible) {
    ASC_CUDA(cudaMemsetAsync(out, 0, (size_t)w * h * sizeof(float), S(stream)));
    return ASC_OK;
  }
  float m[12];
  fold_matrix(imv, v->inv_scale, v->inv_trans, m);
  const uint8_t* occ = nullptr;
  if (g_empty_skip) {
    const float cut = occupancy_threshold(make_cutoff(cutoff, v->dev.norm, v->dev.gmax));
    if (!v->occ) {
      Gate g(device_gate());
      ASC_CUDA(cudaMalloc(&v->occ, occ_grid_bytes(occupancy_cells(v->dev))));
    }
    if (!(v->occ_cutoff == cut)) {
      build_occupancy(v->dev, cut, v->occ, S(stream));
      ASC_LAUNCH_CHECK();
      v->occ_cutoff = cut;
    }
    occ = v->occ;
  }
  return raycast_launch(v->dev, occ, m, vp, step, intensity, cutoff, out, w, h, S(stream));
}

// ---- images ----
struct asc_image_s {
  void* data;
  int w, h, bps;
};

ASC_API int asc_image_create(const void* data, int w, int h, int bps, asc_image* out)
{
  if (!data || !out || w <= 0 || h <= 0 || (bps != 8 && bps != 16 && bps != 32)) return ASC_ERR_ARG;
  auto* im = new asc_image_s{nullptr, w, h, bps};
  size_t bytes = (size_t)w * h * (bps / 8);
  Gate g(device_gate());
  cudaError_t e = cudaMalloc(&im->data, bytes);
  if (e == cudaSuccess) e = cudaMemcpy(im->data, data, bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    if (im->data) cudaFree(im->data);
    delete im;
    return cuda_status(e);
  }
  *out = im;
  return ASC_OK;
}

ASC_API int asc_image_update(asc_image im, const void* data, void* st)
{
  if (!im || !data) return ASC_ERR_ARG;
  ASC_CUDA(cudaMemcpyAsync(im->data, data, (size_t)im->w * im->h * (im->bps / 8), cudaMemcpyHostToDevice, S(st)));
  return ASC_OK;
}

ASC_API int asc_image_destroy(asc_image im)
{
  if (!im) return ASC_ERR_ARG;
  Gate g(device_gate());
  cudaFree(im->data);
  delete im;
  return ASC_OK;
}

// Video::create_background_image (Video.cpp:147-218): per pixel, the largest
// normalized value over the frames (8, 16 or 32 bits per sample).
__global__ void k_background_max(const void* __restrict__ img, int bps, size_t n, float* __restrict__ out)
{
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    float v;
    if (bps == 8)
      v = (float)__ldg((const unsigned char*)img + i) / 255.0f;
    else if (bps == 16)
      v = (float)__ldg((const unsigned short*)img + i) / 65535.0f;
    else
      v = (float)__ldg((const unsigned*)img + i) / 4294967295.0f;
    if (v > out[i]) out[i] = v;
  }
}

ASC_API int asc_background_from_frames(const asc_image* frames, int n, float* out, void* st)
{
  if (!frames || !out || n < 2) return ASC_ERR_ARG;  // the reference wants two images at least
  const int w = frames[0]->w, h = frames[0]->h;
  for (int i = 0; i < n; ++i)
    if (!frames[i] || frames[i]->w != w || frames[i]->h != h || frames[i]->bps == 32) return ASC_ERR_ARG;
  const size_t px = (size_t)w * h;
  ASC_CUDA(cudaMemsetAsync(out, 0, px * sizeof(float), S(st)));
  const int blocks = (int)std::min<size_t>((px + 255) / 256, 4096);
  for (int i = 0; i < n; ++i) k_background_max<<<blocks, 256, 0, S(st)>>>(frames[i]->data, frames[i]->bps, px, out);
  ASC_LAUNCH_CHECK();
  return ASC_OK;
}

namespace asc {
const void* image_data(asc_image im, int* w, int* h, int* bps)
{
  *w = im->w;
  *h = im->h;
  *bps = im->bps;
  return im->data;
}
}  // namespace asc

static int image_render(asc_image im, const float ip[4], const float vp[4], int mode, float thr, float* out, int w,
                        int h, void* stream)
{
  if (!im || !ip || !vp || !out || w < 0 || h < 0) return ASC_ERR_ARG;
  if (w == 0 || h == 0) return ASC_OK;
  ImgArgs a;
  memcpy(a.ip, ip, sizeof a.ip);
  memcpy(a.vp, vp, sizeof a.vp);
  a.threshold = thr;
  a.mode = mode;
  dim3 b(32, 8), g((w + 31) / 32, (h + 7) / 8);
  k_image_render<<<g, b, 0, S(stream)>>>(im->data, im->bps, im->w, im->h, a, out, w, h);
  ASC_LAUNCH_CHECK();
  return ASC_OK;
}

ASC_API int asc_rad_render(asc_image im, const float ip[4], const float vp[4], float* out, int w, int h, void* st)
{
  return image_render(im, ip, vp, 0, 0.f, out, w, h, st);
}

ASC_API int asc_background_render(asc_image im, const float ip[4], const float vp[4], float thr, float* out, int w,
                                  int h, void* st)
{
  return image_render(im, ip, vp, 1, thr, out, w, h, st);
}

// ---- elementwise ----
static int elementwise(int op, const float* a, const float* b, const float* c, float* d, size_t n, float val,
                       void* st)
{
  if (!d || (op <= 3 && !a) || ((op == 1 || op == 2 || op == 3) && !b) || (op == 3 && !c)) return ASC_ERR_ARG;
  if (n == 0) return ASC_OK;
  int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 16);
  k_elementwise<<<blocks, 256, 0, S(st)>>>(op, a, b, c, d, n, val);
  ASC_LAUNCH_CHECK();
  return ASC_OK;
}

ASC_API int asc_drr_background(const float* s, float* d, int w, int h, void* st)
{
  if (w < 0 || h < 0) return ASC_ERR_ARG;
  return elementwise(0, s, nullptr, nullptr, d, (size_t)w * h, 0.f, st);
}
ASC_API int asc_multiply(const float* a, const float* b, float* d, int w, int h, void* st)
{
  if (w < 0 || h < 0) return ASC_ERR_ARG;
  return elementwise(1, a, b, nullptr, d, (size_t)w * h, 0.f, st);
}
ASC_API int asc_merge(const float* a, const float* b, float* d, int w, int h, void* st)
{
  if (w < 0 || h < 0) return ASC_ERR_ARG;
  return elementwise(2, a, b, nullptr, d, (size_t)w * h, 0.f, st);
}
ASC_API int asc_composite(const float* a, const float* b, const float* c, const float*, float* d, int w, int h,
                          void* st)
{
  if (w < 0 || h < 0) return ASC_ERR_ARG;
  return elementwise(3, a, b, c, d, (size_t)w * h, 0.f, st);
}
ASC_API int asc_fill(float* d, size_t n, float v, void* st) { return elementwise(4, nullptr, nullptr, nullptr, d, n, v, st); }

// ---- filters ----
static int filter(int kind, const float* in, float* out, int w, int h, float p0, float p1, float p2, void* st)
{
  if (!in || !out || w < 0 || h < 0 || in == out) return ASC_ERR_ARG;
  asc_filter_desc f = {kind, 1, p0, p1, p2};
  return launch_filter(f, in, out, w, h, S(st));
}
ASC_API int asc_sobel(const float* in, float* out, int w, int h, float scale, float blend, void* st)
{
  return filter(1, in, out, w, h, scale, blend, 0.f, st);
}
ASC_API int asc_contrast(const float* in, float* out, int w, int h, float alpha, float beta, int size, void* st)
{
  return filter(0, in, out, w, h, alpha, beta, (float)size, st);
}
ASC_API int asc_gaussian(const float* in, float* out, int w, int h, float radius, void* st)
{
  return filter(3, in, out, w, h, radius, 0.f, 0.f, st);
}
ASC_API int asc_sharpen(const float* in, float* out, int w, int h, float radius, float contrast, float threshold,
                        void* st)
{
  return filter(4, in, out, w, h, radius, contrast, threshold, st);
}

// ---- reductions ----
ASC_API int asc_ncc_init(unsigned max_n)
{
  std::lock_guard<std::mutex> l(g_red_mu);
  return ncc_init_locked(max_n);
}

int asc::ncc_init_locked(unsigned max_n)
{
  Gate g(device_gate());
  if (g_part) cudaFree(g_part);
  if (g_means) cudaFree(g_means);
  if (g_ticket) cudaFree(g_ticket);
  g_part = nullptr;
  g_means = nullptr;
  g_ticket = nullptr;
  g_max_n = 0;
  if (max_n == 0) return ASC_OK;
  size_t nb = (max_n + RCHUNK - 1) / RCHUNK;
  ASC_CUDA(cudaMalloc(&g_part, nb * sizeof(Moments)));
  ASC_CUDA(cudaMalloc(&g_means, 2 * sizeof(double)));
  ASC_CUDA(cudaMalloc(&g_ticket, sizeof(unsigned)));
  ASC_CUDA(cudaMemset(g_ticket, 0, sizeof(unsigned)));
  g_max_n = max_n;
  ASC_CUDA(cudaGetDevice(&g_red_dev));
  return ASC_OK;
}

ASC_API int asc_ncc(const float* f, const float* g, const float* m, unsigned n, int coverage, double* res, void* st)
{
  if (!f || !g || !m || !res || n == 0 || (coverage != ASC_SUM_TREE && coverage != ASC_SUM_FULL)) return ASC_ERR_ARG;
  ReduceScratch sc;
  int rc = ensure_scratch(n, &sc);
  if (rc) return rc;
  int tree = coverage == ASC_SUM_TREE && tree_needed(n);
  k_ncc<<<(n + RCHUNK - 1) / RCHUNK, RB, 0, S(st)>>>(f, g, m, n, tree, sc, res);
  ASC_LAUNCH_CHECK();
  return ASC_OK;
}

ASC_API int asc_hdist(const float* f, const float* g, const float* m, unsigned n, int coverage, double* res,
                      void* st)
{
  if (!f || !g || !m || !res || n == 0 || (coverage != ASC_SUM_TREE && coverage != ASC_SUM_FULL)) return ASC_ERR_ARG;
  ReduceScratch sc;
  int rc = ensure_scratch(n, &sc);
  if (rc) return rc;
  int tree = coverage == ASC_SUM_TREE && tree_needed(n);
  unsigned nb = (n + RCHUNK - 1) / RCHUNK;
  k_hdist_means<<<nb, RB, 0, S(st)>>>(f, g, m, n, tree, sc);
  k_hdist_sad<<<nb, RB, 0, S(st)>>>(f, g, m, n, tree, sc, res);
  ASC_LAUNCH_CHECK();
  return ASC_OK;
}

static int host_result(int rc, double* dev, double* out, void* st)
{
  if (rc == ASC_OK) {
    cudaError_t e = cudaMemcpyAsync(out, dev, sizeof(double), cudaMemcpyDeviceToHost, S(st));
    if (e == cudaSuccess) e = cudaStreamSynchronize(S(st));
    if (e != cudaSuccess) rc = cuda_status(e);
  }
  Gate g(device_gate());
  cudaFree(dev);
  return rc;
}

ASC_API int asc_ncc_host(const float* f, const float* g, const float* m, unsigned n, int coverage, double* out,
                         void* st)
{
  if (!out) return ASC_ERR_ARG;
  double* dev = nullptr;
  {
    Gate g(device_gate());
    ASC_CUDA(cudaMalloc(&dev, sizeof(double)));
  }
  return host_result(asc_ncc(f, g, m, n, coverage, dev, st), dev, out, st);
}

ASC_API int asc_hdist_host(const float* f, const float* g, const float* m, unsigned n, int coverage, double* out,
                           void* st)
{
  if (!out) return ASC_ERR_ARG;
  double* dev = nullptr;
  {
    Gate g(device_gate());
    ASC_CUDA(cudaMalloc(&dev, sizeof(double)));
  }
  return host_result(asc_hdist(f, g, m, n, coverage, dev, st), dev, out, st);
}
