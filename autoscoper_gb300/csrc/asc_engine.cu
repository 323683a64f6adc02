// Batched registration engine: Tracker::minimizationFunc (Tracker.cpp:775-827)
// for many (bone, manipulator) candidates per pass, with the scene resident
// on the device.
//
// One evaluation is six launches on one stream (seven with cf_model 1):
//   k_setup_iv    a thread per (item, view): FP64 pose composition, view
//                            matrix, viewport (Tracker.cpp:603-634) and crop;
//   k_setup       1 block:  the tile layout of every crop, with prefix sums;
//   k_tile_map    grid-stride: each ray and view tile's (item, view);
//   k_ray         persistent: 16x16-ray tiles pulled from an atomic queue,
//                            DRRs written to a packed buffer; rays with a
//                            sample within rounding of the cutoff are listed;
//   k_ray_fix     a warp per listed tile: its marked rays marched again
//                            with exact cutoff decisions;
//   k_view        persistent: 48x48 output tiles pulled from a queue; each
//                            stages DRR and radiograph regions with the chain's
//                            halo in shared memory, runs both filter chains,
//                            the masks and the NCC moments; the last tile of a
//                            view merges its tiles in FP64, the last view of an
//                            item sums the view costs.
// The PSO driver adds an update kernel before and a best-update kernel after,
// and captures one iteration as a CUDA graph.
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "asc_internal.cuh"

namespace asc {
const void* image_data(asc_image im, int* w, int* h, int* bps);
}

using namespace asc;

namespace {

constexpr int MAX_VIEWS = 16;  // views of an engine (a serving engine holds several jobs' views)
constexpr int MAX_SLOTS = 4;   // views one bone is scored in (the public bone desc's per-view settings)
constexpr int MAX_BONES = 64;
constexpr int MAX_FILTERS = 8;
#ifndef ASC_VT
#define ASC_VT 48
#endif
#ifndef ASC_VIEW_MINBLOCKS
#define ASC_VIEW_MINBLOCKS 3
#endif
constexpr int VT = ASC_VT;   // k_view output tile edge
constexpr int VNT = 256;     // k_view threads per block
constexpr int RTX = 16, RTY = 16;  // k_ray work item: one block, 16 x 16 rays
constexpr int NRAY = RTX * RTY;    // k_ray threads per block, one ray each
constexpr int NBW = 8;             // march segments per ray per k_ray pass

struct FilterDev {
  int kind, K, R;
  float p0, p1, p2;
  float g[32];
};

struct ViewDev {
  double cam[12], cam_inv[12], ip[12], cvp[4];
  float ipf[4];
  int rw, rh;  // render size of this view's trial (Trial::render_width/height)
  int E;       // k_view region edge: VT + 2 x the larger chain halo
  const void* rad;
  int rad_w, rad_h, rad_bps;
  const float* bg;
  int bg_w, bg_h;
  float bg_thr;
  int n_drr, n_rad, h_drr, h_rad;
  FilterDev fdrr[MAX_FILTERS], frad[MAX_FILTERS];
};

struct BoneDev {
  DevVolume vol;
  float inv_scale[3], inv_trans[3];
  double pivot[12], pivot_inv[12], base[6];
  // per slot: the bone is scored in views view_of[0 .. n_slots), with that
  // view's RayCaster settings and its empty-cell grid
  float step[MAX_SLOTS], scale[MAX_SLOTS];
  Cutoff cut[MAX_SLOTS];
  const uint8_t* occ[MAX_SLOTS];
  int view_of[MAX_SLOTS];
  int n_slots;
  int visible;                    // RayCaster::setVisible: a hidden volume renders zeros
};

struct SceneDev {
  int n_views, n_bones, rw, rh, coverage, E;  // rw, rh, E: the largest of the views'
  int slots;     // (item, slot) entries per item: the most views a bone is scored in
  int cf_model;  // 0: 1 - NCC per view; 1: SAD ("hdist") per view
  ViewDev views[MAX_VIEWS];
  BoneDev bones[MAX_BONES];
};

struct IV {
  float m[12];
  float vp[4];
  float sx[2], sy[2];  // vp[2] / w and vp[3] / h as double-floats
  int w, h, ok, bone;
  int view, slot;  // the engine view and the bone's slot of this (item, view)
  int rtx, rty, ftx, fty;
  int err;        // the crop exceeded the render size (the reference throws)
  float band[3];  // the bone's cutoff here: raw - t0, hi0 + t0, t1 (k_ray's band)
  long long pix;  // offset of this crop in the DRR buffer
};

struct Counters {
  int n_items, n_iv;
  int rtiles, ftiles;
  int rnext, fnext;
  int error;
  int nfix;   // rays whose march met the cutoff's band (k_ray_fix marches them again)
  int nfixt;  // ray tiles holding such rays
  int pad;
  unsigned long long samples, pixels;
  unsigned long long marched, slots;  // marched samples, 32 x warp-max span
};

struct Bufs {
  IV* iv;
  int* roff;       // n_iv + 1 prefix of ray tiles
  int* foff;       // n_iv + 1 prefix of view tiles
  float* drr;
  Moments* part;   // per view tile
  float2* fg;      // cf_model 1: masked DRR and radiograph per crop pixel
  double2* hmean;  // cf_model 1: per-iv means of f and g
  float* tsad;     // cf_model 1: per view tile SAD
  double* vcost;   // per iv
  unsigned* ivt;   // per-iv tile tickets
  unsigned* itt;   // per-item view tickets
  int* fixt;       // ray tiles holding rays to march again exactly (k_ray_fix)
  int* rtile_iv;   // per ray tile: its (item, view) (k_tile_map)
  int* ftile_iv;   // per view tile: its (item, view)
  Counters* C;
};

__device__ __forceinline__ int find_iv(const int* off, int n, int tile)
{
  int lo = 0, hi = n;  // off[lo] <= tile < off[hi]
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (__ldg(off + mid) <= tile) lo = mid; else hi = mid;
  }
  return lo;
}

__device__ void finish_item(const SceneDev* sc, const Bufs& b, int item, double* cost)
{
  double tot = 0;
  for (int j = 0; j < sc->slots; ++j) tot += b.vcost[item * sc->slots + j];
  cost[item] = tot < 0 ? 9999.0 : tot;  // Tracker.cpp:823-825
}

// ---------------------------------------------------------------- k_setup
// One (item, view) of trackFrame's set-up: the pose (minimizationFunc), the
// folded matrix, the viewport and crop size, its ray and view tile counts.
__device__ void setup_iv(const SceneDev* __restrict__ sc, int k, const int* __restrict__ bone_in,
                         const double* __restrict__ manip, const Bufs& b)
{
  const int ns = sc->slots;
  const int item = k / ns, j = k % ns;
  IV r;
  memset(&r, 0, sizeof r);
  int bi = bone_in[item];
  if (bi < 0 || bi >= sc->n_bones) bi = 0;
  r.bone = bi;
  r.slot = j;
  const BoneDev& B = sc->bones[bi];
  if (j >= B.n_slots) {  // a slot this bone has no view in: adds nothing to the cost
    r.view = -1;
    b.iv[k] = r;
    b.vcost[k] = 0.0;
    b.ivt[k] = 0;
    return;
  }
  const int v = B.view_of[j];
  r.view = v;
  const ViewDev& V = sc->views[v];
  // minimizationFunc: pose . V^-1 . manip . V, then the xyzypr round trip
  double base[12], man[12], t1[12], t2[12], xyz[6];
  frame_from_xyzypr(B.base, base);
  frame_from_axis_angle(manip + 6 * item, man);
  frame_mul(base, B.pivot_inv, t1);
  frame_mul(t1, man, t2);
  frame_mul(t2, B.pivot, t1);
  frame_to_xyzypr(t1, xyz);
  frame_from_xyzypr(xyz, t1);
  // trackFrame (1a)-(1c)
  double mv[12], imv[12], imv16[16], vp[4];
  frame_mul(V.cam_inv, t1, mv);
  frame_inverse(mv, imv);
  frame_row_matrix(imv, imv16);
  fold_matrix(imv16, B.inv_scale, B.inv_trans, r.m);
  const Cutoff& cut = B.cut[j];
  r.band[0] = cut.raw - cut.t0;
  r.band[1] = cut.hi0 + cut.t0;
  r.band[2] = cut.t1;
  double vc = 0.0;
  if (!calculate_viewport(mv, V.cam, V.ip, B.inv_scale, B.inv_trans, vp)) {
    vc = 9999.0;  // Tracker.cpp:614-617
  } else {
    double fw = vp[2] * V.rw / V.cvp[2], fh = vp[3] * V.rh / V.cvp[3];
    unsigned w = fw > 0 ? (unsigned)fw : 0u, h = fh > 0 ? (unsigned)fh : 0u;
    if (w > (unsigned)V.rw || h > (unsigned)V.rh) {
      r.err = 1;  // the reference throws (Tracker.cpp:625-629)
      w = 0;
      h = 0;
    }
    r.w = (int)w;
    r.h = (int)h;
    for (int j = 0; j < 4; ++j) r.vp[j] = (float)vp[j];
    if (w > 0 && h > 0) {
      df_split((double)r.vp[2] / (double)w, r.sx[0], r.sx[1]);
      df_split((double)r.vp[3] / (double)h, r.sy[0], r.sy[1]);
    }
    if (w == 0 || h == 0 || !B.visible) {
      // an empty crop, or the all-zero DRR of a hidden volume (RayCaster.cpp:131-134),
      // whose mask is empty: the degenerate NCC (1e5), or the SAD of no pixels
      vc = sc->cf_model ? 0.0 : 1.0 - 1e5;
    } else {
      r.ok = 1;
      r.rtx = (r.w + RTX - 1) / RTX;
      r.rty = (r.h + RTY - 1) / RTY;
      r.ftx = (r.w + VT - 1) / VT;
      r.fty = (r.h + VT - 1) / VT;
    }
  }
  b.iv[k] = r;
  b.vcost[k] = vc;
  b.ivt[k] = 0;
}

// Every (item, view) at once: the FP64 set-up of each runs on its own thread
// across the GPU.
__global__ void __launch_bounds__(128) k_setup_iv(const SceneDev* __restrict__ sc, int n_items,
                                                  const int* __restrict__ bone_in, const double* __restrict__ manip,
                                                  Bufs b)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n_items * sc->slots) setup_iv(sc, k, bone_in, manip, b);
}

// The layout of a batch after k_setup_iv: prefix sums of the tile counts and
// crop sizes (ray tiles, view tiles, DRR offsets), the batch counters, and
// the items' view tickets (views finished in set-up count as arrived).
__global__ void __launch_bounds__(1024) k_setup(const SceneDev* __restrict__ sc, int n_items, Bufs b,
                                                 double* __restrict__ cost)
{
  __shared__ int s_err;
  const int nv = sc->slots, n_iv = n_items * nv;
  const int per = (n_iv + blockDim.x - 1) / blockDim.x;
  const int i0 = threadIdx.x * per, i1 = min(i0 + per, n_iv);
  if (threadIdx.x == 0) s_err = 0;
  __syncthreads();
  int rsum = 0, fsum = 0;
  long long psum = 0;
  for (int k = i0; k < i1; ++k) {
    const IV& r = b.iv[k];
    if (r.err) s_err = ASC_ERR_RANGE;
    psum += (long long)r.w * r.h;
    rsum += r.rtx * r.rty;
    fsum += r.ftx * r.fty;
  }
  // block-wide exclusive scan of (rsum, fsum, psum)
  __shared__ long long sp[1024];
  __shared__ int sr[1024], sf[1024];
  sr[threadIdx.x] = rsum;
  sf[threadIdx.x] = fsum;
  sp[threadIdx.x] = psum;
  __syncthreads();
  for (int o = 1; o < blockDim.x; o <<= 1) {
    int a = threadIdx.x >= o ? sr[threadIdx.x - o] : 0;
    int c = threadIdx.x >= o ? sf[threadIdx.x - o] : 0;
    long long p = threadIdx.x >= o ? sp[threadIdx.x - o] : 0;
    __syncthreads();
    sr[threadIdx.x] += a;
    sf[threadIdx.x] += c;
    sp[threadIdx.x] += p;
    __syncthreads();
  }
  int rbase = sr[threadIdx.x] - rsum, fbase = sf[threadIdx.x] - fsum;
  long long pbase = sp[threadIdx.x] - psum;
  for (int k = i0; k < i1; ++k) {
    IV& r = b.iv[k];
    r.pix = pbase;
    b.roff[k] = rbase;
    b.foff[k] = fbase;
    pbase += (long long)r.w * r.h;
    rbase += r.rtx * r.rty;
    fbase += r.ftx * r.fty;
  }
  if (threadIdx.x == blockDim.x - 1) {
    b.roff[n_iv] = rbase;
    b.foff[n_iv] = fbase;
    b.C->n_items = n_items;
    b.C->n_iv = n_iv;
    b.C->rtiles = rbase;
    b.C->ftiles = fbase;
    b.C->rnext = 0;
    b.C->fnext = 0;
    b.C->error = s_err;
    b.C->nfix = 0;
    b.C->nfixt = 0;
    b.C->samples = 0;
    b.C->marched = 0;
    b.C->slots = 0;
    b.C->pixels = (unsigned long long)(sp[threadIdx.x]);
  }
  __syncthreads();
  // item tickets: views finished here count as arrived
  for (int item = threadIdx.x; item < n_items; item += blockDim.x) {
    unsigned pre = 0;
    for (int v = 0; v < nv; ++v) pre += b.iv[item * nv + v].ok ? 0u : 1u;
    b.itt[item] = pre;
    if (pre == (unsigned)nv) finish_item(sc, b, item, cost);
  }
}

// Every ray tile's and view tile's (item, view), so that the persistent
// kernels look a grabbed tile up with one load instead of a binary search
// over the prefix sums (ten dependent loads while the block waits).
// (Dealing most ray tiles to the blocks in turn, with a queue for the rest,
// measured 9 % slower: a block then owns fixed columns of every crop, and the
// central ones cost more.)
__global__ void __launch_bounds__(256) k_tile_map(Bufs b)
{
  const int rt = b.C->rtiles, ft = b.C->ftiles, n = b.C->n_iv;
  const int stride = gridDim.x * blockDim.x;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < rt; t += stride) b.rtile_iv[t] = find_iv(b.roff, n, t);
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ft; t += stride) b.ftile_iv[t] = find_iv(b.foff, n, t);
}

// ---------------------------------------------------------------- k_ray
#ifndef ASC_RAY_MINBLOCKS
#define ASC_RAY_MINBLOCKS 4  // 4 x 256 threads resident per SM (<= 64 registers)
#endif

// Rays of one 16 x 16 tile of one (item, view) crop per block.  Each ray's
// march is cut into segments: the REBASE-sample march blocks that hold
// occupied samples, each trimmed to its occupied extent (walk_segments).
// The block's segments are sorted by length (counting sort, longest first)
// and marched 32 at a time by whichever warp is free, so the lanes of a warp
// march segments of nearly equal length whatever the rays' lengths; each ray
// then adds its blocks' sums in order (add_block), as march() does for a
// single ray.  A ray with more than NBW segments takes further passes.
template <int STORE>
__device__ __forceinline__ void march_segments(const DevVolume& V, const float4 (*rec)[NRAY], const unsigned* ord,
                                               float* part, int nseg, int* grab, const float4* band,
                                               const Cutoff& cut, unsigned long long& marched,
                                               unsigned long long& slots)
{
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  for (;;) {
    int g = 0;
    if (lane == 0) g = atomicAdd(grab, 32);
    g = __shfl_sync(FULL, g, 0);
    if (g >= nseg) return;
    int len = 0;
    if (g + lane < nseg) {
      const unsigned d = ord[g + lane];
      const int slot = d & 2047u, js = (d >> 11) & 63u, je = (d >> 17) & 63u;
      const int ray = slot / NBW;
      RaySetup r;
      const float4 q0 = rec[0][ray], q1 = rec[1][ray], q2 = rec[2][ray];
      r.X = df{q0.x, q0.y};
      r.Y = df{q0.z, q0.w};
      r.Z = df{q1.x, q1.y};
      r.dX = df{q1.z, q1.w};
      r.dY = df{q2.x, q2.y};
      r.dZ = df{q2.z, q2.w};
      const int kb = __float_as_int(part[slot]);  // the block start, until the sum replaces it
      // this ray's band: the tile's raw - t0, hi0 + t0 and t1 (cutoff_bounds)
      const float4 c = *band;
      const float S = fabsf(q1.z) + fabsf(q2.x) + fabsf(q2.z);
      part[slot] = march_block<STORE, false>(V, r, kb, js, je, fmaf(-c.z, S, c.x), fmaf(c.z, S, c.y), cut);
      len = je - js + 1;
    }
    const unsigned tot = __reduce_add_sync(FULL, (unsigned)len), mx = __reduce_max_sync(FULL, (unsigned)len);
    marched += tot;
    slots += 32ull * mx;
  }
}

// shape: log2 of the width of the ray block each warp takes in a 16 x 16
// tile (2: 4 x 8, 3: 8 x 4, 4: 16 x 2), the autotuner's choice.  A ray any
// of whose samples fell in the cutoff's band (march_block) leaves the mark
// -1 in its DRR pixel, and its tile goes on the fix list for k_ray_fix.
__global__ void __launch_bounds__(NRAY, ASC_RAY_MINBLOCKS) k_ray(const SceneDev* __restrict__ sc, Bufs b, int skip,
                                                                 int shape)
{
  static_assert(REBASE == 64 && NRAY * NBW <= 2048, "segment fields: 11-bit slot, 6-bit offsets");
  __shared__ float4 s_rec[3][NRAY];      // per ray: X, Y, Z, dX, dY, dZ as double-floats
  __shared__ float s_trim[3][NRAY];      // per ray: RayTrim's 1 / (8 dC) per axis (its C is in s_rec)
  __shared__ float s_part[NRAY * NBW];   // per segment slot: the block start (int bits), then its sum
  __shared__ unsigned s_seg[NRAY * NBW]; // per segment slot: slot | js << 11 | je << 17
  __shared__ unsigned s_ord[NRAY * NBW]; // the segments, longest first
  __shared__ int s_cnt[REBASE];          // segments per length - 1, then placement cursors
  __shared__ int s_tile, s_nseg, s_grab, s_k;
  __shared__ float4 s_band;              // the tile's cutoff: raw - t0, hi0 + t0, t1
  __shared__ int s_fix;                  // 1 + the last tile, when one of its rays was marked
  const unsigned FULL = 0xffffffffu;
  const int tid = threadIdx.x, lane = tid & 31;
  unsigned long long marched = 0, slots = 0, sampled = 0;
  if (tid == 0) s_fix = 0;
  for (;;) {
    if (tid == 0) {
      const int tl = atomicAdd(&b.C->rnext, 1);
      s_tile = tl;
      int kk = 0;
      if (tl < b.C->rtiles) {
        kk = b.rtile_iv[tl];
        const float* bd = b.iv[kk].band;
        s_band = make_float4(bd[0], bd[1], bd[2], 0.f);
      }
      s_k = kk;
    }
    __syncthreads();
    // the last tile's mark (set after its last barrier, visible past this one)
    if (tid == 0 && s_fix) {
      b.fixt[atomicAdd(&b.C->nfixt, 1)] = s_fix - 1;
      s_fix = 0;
    }
    const int tile = s_tile;
    if (tile >= b.C->rtiles) break;
    const int k = s_k;
    const IV& r = b.iv[k];
    const int t = tile - b.roff[k];
    // each warp takes a (1 << shape) x (32 >> shape) block of the 16 x 16
    // tile (coherent walks)
    const int wsh = shape, wpr = 4 - shape;  // log2 of the block width, of the blocks per tile row
    const int wrp = tid >> 5;
    const int x = (t % r.rtx) * RTX + ((wrp & ((1 << wpr) - 1)) << wsh) + (lane & ((1 << wsh) - 1)),
              y = (t / r.rtx) * RTY + ((wrp >> wpr) << (5 - wsh)) + (lane >> wsh);
    const bool valid = x < r.w && y < r.h;
    const BoneDev& B = sc->bones[r.bone];
    const int j = r.slot;
    const Cutoff& cut = B.cut[j];
    const uint8_t* occ = skip ? B.occ[j] : nullptr;
    RaySetup rs{};
    const bool hit = valid && ray_setup(r.m, r.vp, x, y, df{r.sx[0], r.sx[1]}, df{r.sy[0], r.sy[1]}, B.step[j],
                                        B.vol.nx, B.vol.ny, B.vol.nz, rs);
    // trilinear samples of the reference's march (the work figure of the
    // roofline), counted per warp and added to the global count once at the end
    sampled += __reduce_add_sync(FULL, hit ? (unsigned)rs.K : 0u);
    bool done = true;
    CellWalk cw = cell_walk(B.vol, rs, 0);
    if (hit && rs.K > 0) {
      s_rec[0][tid] = make_float4(rs.X.h, rs.X.l, rs.Y.h, rs.Y.l);
      s_rec[1][tid] = make_float4(rs.Z.h, rs.Z.l, rs.dX.h, rs.dX.l);
      s_rec[2][tid] = make_float4(rs.dY.h, rs.dY.l, rs.dZ.h, rs.dZ.l);
      // ray_trim's 1 / (8 dC) from the walk's crossing intervals (dt = 8 / |dC|)
      const bool big = B.vol.nx > OCC_TRIM_MAX || B.vol.ny > OCC_TRIM_MAX || B.vol.nz > OCC_TRIM_MAX;
      const float nan = __int_as_float(0x7fffffff);
      s_trim[0][tid] = big || cw.ix == 0 ? nan : (cw.ix < 0 ? cw.dtx : -cw.dtx) * (1.0f / 64.0f);
      s_trim[1][tid] = big || cw.iy == 0 ? nan : (cw.iy < 0 ? cw.dty : -cw.dty) * (1.0f / 64.0f);
      s_trim[2][tid] = big || cw.iz == 0 ? nan : (cw.iz < 0 ? cw.dtz : -cw.dtz) * (1.0f / 64.0f);
      done = false;
    }
    WalkState ws{0, rs.K - 1, 0, -1, 0};
    df total{0.f, 0.f};  // NaN once a segment met the cutoff's band
    for (;;) {
      if (tid < REBASE) s_cnt[tid] = 0;
      if (tid == 0) s_grab = 0;
      __syncthreads();
      // ---- walk: up to NBW segments of this ray
      int n = 0;
      const auto trim = [&](int i, float& ia, float& c) {
        ia = s_trim[i][tid];
        c = i == 0 ? s_rec[0][tid].x : (i == 1 ? s_rec[0][tid].z : s_rec[1][tid].x);  // X.h, Y.h, Z.h
      };
      if (!done)
        done = walk_segments(cw, occ, trim, ws, [&](int kb, int js, int je) {
          if (n == NBW) return false;
          const int slot = tid * NBW + n++;
          s_seg[slot] = (unsigned)slot | (unsigned)js << 11 | (unsigned)je << 17;
          s_part[slot] = __int_as_float(kb);
          atomicAdd(&s_cnt[je - js], 1);
          return true;
        });
      __syncthreads();
      // ---- counting sort by length, longest first
      if (tid < 32) {
        const int c0 = s_cnt[REBASE - 1 - 2 * lane], c1 = s_cnt[REBASE - 2 - 2 * lane];
        int incl = c0 + c1;
        for (int o = 1; o < 32; o <<= 1) {
          const int u = __shfl_up_sync(FULL, incl, o);
          if (lane >= o) incl += u;
        }
        const int excl = incl - c0 - c1;
        s_cnt[REBASE - 1 - 2 * lane] = excl;
        s_cnt[REBASE - 2 - 2 * lane] = excl + c0;
        if (lane == 31) s_nseg = incl;
      }
      __syncthreads();
      for (int i = 0; i < n; ++i) {
        const unsigned d = s_seg[tid * NBW + i];
        const int len1 = (int)((d >> 17) & 63u) - (int)((d >> 11) & 63u);
        s_ord[atomicAdd(&s_cnt[len1], 1)] = d;
      }
      __syncthreads();
      const int nseg = s_nseg;
      // ---- march the segments, 32 at a time per warp
      if (B.vol.storage == ASC_STORE_F32)
        march_segments<ASC_STORE_F32>(B.vol, s_rec, s_ord, s_part, nseg, &s_grab, &s_band, cut, marched,
                                      slots);
      else if (B.vol.storage == ASC_STORE_BF16)
        march_segments<ASC_STORE_BF16>(B.vol, s_rec, s_ord, s_part, nseg, &s_grab, &s_band, cut, marched,
                                      slots);
      else if (B.vol.storage == ASC_STORE_F16)
        march_segments<ASC_STORE_F16>(B.vol, s_rec, s_ord, s_part, nseg, &s_grab, &s_band, cut, marched,
                                      slots);
      else
        march_segments<ASC_STORE_U16>(B.vol, s_rec, s_ord, s_part, nseg, &s_grab, &s_band, cut, marched,
                                      slots);
      __syncthreads();
      // ---- this ray's segments, in order
      for (int i = 0; i < n; ++i) {
        const float p = s_part[tid * NBW + i];
        if (block_flagged(p))
          total.h = __int_as_float(0x7fffffff);  // NaN stays NaN through add_block
        else
          add_block(total, p);
      }
      if (!__syncthreads_or(!done)) break;
    }
    if (valid) {
      const bool flagged = total.h != total.h;
      b.drr[r.pix + (long long)y * r.w + x] =
          flagged ? -1.0f : fminf(fmaxf((total.h + total.l) * B.scale[j], 0.f), 1.f);
      if (flagged) s_fix = tile + 1;
    }
  }
  if (lane == 0 && sampled) atomicAdd(&b.C->samples, sampled);
  if (lane == 0 && slots) {
    atomicAdd(&b.C->marched, marched);
    atomicAdd(&b.C->slots, slots);
  }
}

// The marked rays of the tiles on the fix list, marched again with every
// cutoff decision the exact one (march_pass with EXACT); each overwrites its
// mark.  A warp per listed tile: its marked rays, found by ballots over the
// tile's 256 pixels, are dealt to the lanes, so a tile's rays march side by
// side.  The ray set-up is k_ray's, so the samples are the same.
constexpr int FIX_THREADS = 128;
__global__ void __launch_bounds__(FIX_THREADS) k_ray_fix(const SceneDev* __restrict__ sc, Bufs b, int skip)
{
  __shared__ unsigned char s_pix[FIX_THREADS / 32][NRAY];  // per warp: the tile's marked rays
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int nt = b.C->nfixt;
  const int nw = gridDim.x * (FIX_THREADS / 32);
  for (int w = blockIdx.x * (FIX_THREADS / 32) + wib; w < nt; w += nw) {
    const int tile = b.fixt[w];
    const int k = b.rtile_iv[tile];
    const IV& r = b.iv[k];
    const int t = tile - b.roff[k];
    const int x0 = (t % r.rtx) * RTX, y0 = (t / r.rtx) * RTY;
    int cnt = 0;
    for (int c = 0; c < NRAY / 32; ++c) {
      const int p = c * 32 + lane, x = x0 + p % RTX, y = y0 + p / RTX;
      const bool marked = x < r.w && y < r.h && b.drr[r.pix + (long long)y * r.w + x] < 0.f;
      const unsigned m = __ballot_sync(0xffffffffu, marked);
      if (marked) s_pix[wib][cnt + __popc(m & ((1u << lane) - 1u))] = (unsigned char)p;
      cnt += __popc(m);
    }
    __syncwarp();
    if (lane == 0) atomicAdd(&b.C->nfix, cnt);
    const BoneDev& B = sc->bones[r.bone];
    const int j = r.slot;
    const uint8_t* occ = skip ? B.occ[j] : nullptr;
    for (int i = lane; i < cnt; i += 32) {
      const int p = s_pix[wib][i], x = x0 + p % RTX, y = y0 + p / RTX;
      RaySetup rs;
      float d = 0.f;
      if (ray_setup(r.m, r.vp, x, y, df{r.sx[0], r.sx[1]}, df{r.sy[0], r.sy[1]}, B.step[j], B.vol.nx, B.vol.ny,
                    B.vol.nz, rs) &&
          rs.K > 0) {
        if (B.vol.storage == ASC_STORE_F32)
          d = march_pass<ASC_STORE_F32, true>(B.vol, occ, rs, B.cut[j], nullptr);
        else if (B.vol.storage == ASC_STORE_BF16)
          d = march_pass<ASC_STORE_BF16, true>(B.vol, occ, rs, B.cut[j], nullptr);
        else if (B.vol.storage == ASC_STORE_F16)
          d = march_pass<ASC_STORE_F16, true>(B.vol, occ, rs, B.cut[j], nullptr);
        else
          d = march_pass<ASC_STORE_U16, true>(B.vol, occ, rs, B.cut[j], nullptr);
      }
      b.drr[r.pix + (long long)y * r.w + x] = fminf(fmaxf(d * B.scale[j], 0.f), 1.f);
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------- k_view
// Region coordinates: buffer index (ry, rx) <-> image (y0 + ry, x0 + rx) with
// x0 = tile x - E_h, where E_h = (E - VT) / 2 is the largest chain halo.
// `in` is set when the whole E x E region lies inside the image: the stages
// then skip every bounds test.
struct Region {
  int x0, y0, E, w, h;
  bool in;
};

__device__ __forceinline__ bool inside(const Region& g, int ry, int rx)
{
  int x = g.x0 + rx, y = g.y0 + ry;
  return x >= 0 && x < g.w && y >= 0 && y < g.h;
}

// Calls f(ry, rx) for every position of the band [y0, y1) x [x0, x1), the
// positions dealt to the block's threads in row-major order (consecutive
// threads take consecutive columns, wrapping to the next row), so no lane
// idles on bands narrower or wider than a warp.
template <class F>
__device__ __forceinline__ void for_band(int y0, int y1, int x0, int x1, F&& f)
{
  const int bw = x1 - x0, n = bw * (y1 - y0);
  if (bw <= 0 || n <= 0) return;
  const int dq = VNT / bw, dr = VNT - dq * bw;
  int ry = (int)threadIdx.x / bw;
  int rx = (int)threadIdx.x - ry * bw;
  ry += y0;
  for (int i = threadIdx.x; i < n; i += VNT) {
    f(ry, x0 + rx);
    rx += dr;
    ry += dq;
    if (rx >= bw) {
      rx -= bw;
      ++ry;
    }
  }
}

// axy^e1 * v^e2 of ContrastFilter_kernels.cu (two powf there) as one exp2 of
// the summed logarithms; axy > 0.01 here.  v^0 is 1 for every v, as powf's.
__device__ __forceinline__ float contrast_pow(float axy, float v, float e1, float e2)
{
  float l = e1 * log2f(axy);
  if (e2 != 0.f) l = fmaf(e2, log2f(v), l);
  return exp2f(l);
}

// Calls f(ry, rx, nr) for column units: column rx of the band [y0, y1) x
// [x0, x1), rows ry .. ry + nr - 1 (nr <= VR), consecutive threads taking
// consecutive columns.  A unit reads a few rows past the band; those reads
// stay inside the block's shared memory (VR rows of slack follow the
// buffers) and their results are discarded.
constexpr int VR = 4;

// k_view's dynamic shared memory, in 4-byte words: three E x E stage
// buffers, the VT x VT tile, VR + 2 rows of slack for the column units'
// reads past a band, then the region's per-column and per-row radiograph
// mapping (texel index and weight each).
__host__ __device__ constexpr size_t view_tail_floats(int E)
{
  return (size_t)3 * E * E + (size_t)VT * VT + (size_t)(VR + 2) * E;
}
__host__ __device__ constexpr size_t view_smem_floats(int E) { return view_tail_floats(E) + (size_t)4 * E; }
constexpr int kNoTexel = -0x7fffffff;  // a column or row that maps outside the radiograph
template <class F>
__device__ __forceinline__ void for_units(int y0, int y1, int x0, int x1, F&& f)
{
  const int bw = x1 - x0, gh = (y1 - y0 + VR - 1) / VR, n = bw * gh;
  if (bw <= 0 || gh <= 0) return;
  const int dq = VNT / bw, dr = VNT - dq * bw;
  int q = (int)threadIdx.x / bw;
  int c = (int)threadIdx.x - q * bw;
  for (int i = threadIdx.x; i < n; i += VNT) {
    const int ry = y0 + q * VR;
    f(ry, x0 + c, min(VR, y1 - ry));
    c += dr;
    q += dq;
    if (c >= bw) {
      c -= bw;
      ++q;
    }
  }
}

__device__ __forceinline__ float clamp01(float v) { return fminf(fmaxf(v, 0.f), 1.f); }

// Gaussian (kind 3) or Sharpen (kind 4) with a K-tap kernel: the 1-D weights
// in registers, a horizontal pass into `tmp`, then a vertical pass in column
// units that reuse each loaded value for up to VR outputs.  Positions outside
// the image hold 0 in every stage buffer, which is the reference's skipping
// of out-of-image taps.
template <bool IN, int K>
__device__ void blur_stage(const FilterDev& f, const float* in, float* out, float* tmp, const Region& g, int lo, int hi)
{
  constexpr int R = K / 2;
  const int E = g.E;
  float w[K];
#pragma unroll
  for (int k = 0; k < K; ++k) w[k] = f.g[k];
  for_band(lo - R, hi + R, lo, hi, [&](int ry, int rx) {
    const float* p = in + ry * E + rx - R;
    float sum = 0.f;
#pragma unroll
    for (int k = 0; k < K; ++k) sum = fmaf(w[k], p[k], sum);
    tmp[ry * E + rx] = sum;
  });
  __syncthreads();
  const bool gauss = f.kind == 3;
  const float p1 = f.p1, p2 = f.p2;
  for_units(lo, hi, lo, hi, [&](int ry, int rx, int nr) {
    float col[K + VR - 1];
    const float* p = tmp + (ry - R) * E + rx;
#pragma unroll
    for (int t = 0; t < K + VR - 1; ++t) col[t] = p[t * E];
#pragma unroll
    for (int t = 0; t < VR; ++t) {
      if (t < nr) {
        float r = 0.f;
        if (IN || inside(g, ry + t, rx)) {
          float blur = 0.f;
#pragma unroll
          for (int k = 0; k < K; ++k) blur = fmaf(w[k], col[t + k], blur);
          if (gauss) {
            r = clamp01(blur);
          } else {
            const float v = in[(ry + t) * E + rx];
            r = fabsf(v - blur) > p2 ? clamp01(v + p1 * (v - blur)) : v;
          }
        }
        out[(ry + t) * E + rx] = r;
      }
    }
  });
}

// Any kernel size: per-element passes with the weights in shared memory.
template <bool IN>
__device__ void blur_stage_any(const FilterDev& f, const float* in, float* out, float* tmp, float* wsh,
                               const Region& g, int lo, int hi)
{
  const int E = g.E, K = f.K, R = f.R;
  const float p1 = f.p1, p2 = f.p2;
  if (threadIdx.x < K) wsh[threadIdx.x] = f.g[threadIdx.x];
  __syncthreads();
  for_band(lo - R, hi + R, lo, hi, [&](int ry, int rx) {
    const float* p = in + ry * E + rx - R;
    float sum = 0.f;
    for (int k = 0; k < K; ++k) sum = fmaf(wsh[k], p[k], sum);
    tmp[ry * E + rx] = sum;
  });
  __syncthreads();
  for_band(lo, hi, lo, hi, [&](int ry, int rx) {
    float r = 0.f;
    if (IN || inside(g, ry, rx)) {
      const float* p = tmp + (ry - R) * E + rx;
      float blur = 0.f;
      for (int k = 0; k < K; ++k) blur = fmaf(wsh[k], p[k * E], blur);
      if (f.kind == 3) {
        r = clamp01(blur);
      } else {
        const float v = in[ry * E + rx];
        r = fabsf(v - blur) > p2 ? clamp01(v + p1 * (v - blur)) : v;
      }
    }
    out[ry * E + rx] = r;
  });
}

// SobelFilter_kernels.cu:63-113 at one pixel from its 3 x 3 neighbourhood.
__device__ __forceinline__ float sobel_px(float p00, float p01, float p02, float p10, float p11, float p12, float p20,
                                          float p21, float p22, float scale, float blend)
{
  const float horz = p02 + 2 * p12 + p22 - p00 - 2 * p10 - p20;
  const float vert = p00 + 2 * p01 + p02 - p20 - 2 * p21 - p22;
  const float grad = sqrtf(horz * horz + vert * vert);
  const float s = blend < 0.5f ? scale * grad + 2.0f * blend * p11 : 2.0f * (1.0f - blend) * scale * grad + p11;
  return clamp01(s);
}

// Applies one filter from `in` to `out` over the square band
// [lo, hi) x [lo, hi) of region coordinates; positions outside the image get
// 0.  `tmp` holds the horizontal pass of a Gaussian/Sharpen blur, `wsh` the
// 1-D weights of a blur of uncommon size.  IN: the region lies inside the
// image.
template <bool IN>
__device__ void apply_stage(const FilterDev& f, const float* in, float* out, float* tmp, float* wsh, const Region& g,
                            int lo, int hi)
{
  const int E = g.E;
  const int kind = f.kind, K = f.K;
  const float p0 = f.p0, p1 = f.p1;
  if (kind == 3 || kind == 4) {
    switch (K) {
      case 3: blur_stage<IN, 3>(f, in, out, tmp, g, lo, hi); break;
      case 5: blur_stage<IN, 5>(f, in, out, tmp, g, lo, hi); break;
      case 7: blur_stage<IN, 7>(f, in, out, tmp, g, lo, hi); break;
      case 9: blur_stage<IN, 9>(f, in, out, tmp, g, lo, hi); break;
      case 11: blur_stage<IN, 11>(f, in, out, tmp, g, lo, hi); break;
      case 13: blur_stage<IN, 13>(f, in, out, tmp, g, lo, hi); break;
      default: blur_stage_any<IN>(f, in, out, tmp, wsh, g, lo, hi);
    }
  } else if (kind == 1) {
    for_units(lo, hi, lo, hi, [&](int ry, int rx, int nr) {
      float L[VR + 2], C[VR + 2], Rt[VR + 2];
      const float* p = in + (ry - 1) * E + rx;
#pragma unroll
      for (int t = 0; t < VR + 2; ++t) {
        L[t] = p[t * E - 1];
        C[t] = p[t * E];
        Rt[t] = p[t * E + 1];
      }
#pragma unroll
      for (int t = 0; t < VR; ++t) {
        if (t < nr) {
          float r = 0.f;
          const int y = g.y0 + ry + t, x = g.x0 + rx;
          if (IN || (x >= 0 && x < g.w && y >= 0 && y < g.h)) {
            if (IN || (x > 0 && x < g.w - 1 && y > 0 && y < g.h - 1)) {
              r = sobel_px(L[t], C[t], Rt[t], L[t + 1], C[t + 1], Rt[t + 1], L[t + 2], C[t + 2], Rt[t + 2], p0, p1);
            } else {  // image border: neighbours outside the image repeat the edge
              const int xm = x > 0 ? -1 : 0, xp = x < g.w - 1 ? 1 : 0, ym = y > 0 ? -E : 0, yp = y < g.h - 1 ? E : 0;
              const float* c = in + (ry + t) * E + rx;
              r = sobel_px(c[ym + xm], c[ym], c[ym + xp], c[xm], c[0], c[xp], c[yp + xm], c[yp], c[yp + xp], p0, p1);
            }
          }
          out[(ry + t) * E + rx] = r;
        }
      }
    });
  } else if (kind == 0 && K == 3) {
    // ContrastFilter_kernels.cu:62-96 with a 3 x 3 box: the mean over the
    // window's in-image pixels (out-of-image positions hold 0, so the sum
    // runs over the whole window and only the count depends on the border)
    const float e1 = p0 - p1, e2 = p1;
    for_units(lo, hi, lo, hi, [&](int ry, int rx, int nr) {
      float rs[VR + 2];
      const float* p = in + (ry - 1) * E + rx - 1;
#pragma unroll
      for (int t = 0; t < VR + 2; ++t) rs[t] = p[t * E] + p[t * E + 1] + p[t * E + 2];
#pragma unroll
      for (int t = 0; t < VR; ++t) {
        if (t < nr) {
          float r = 0.f;
          const int y = g.y0 + ry + t, x = g.x0 + rx;
          if (IN || (x >= 0 && x < g.w && y >= 0 && y < g.h)) {
            float cnt = 9.0f;
            if (!IN) cnt = (float)((min(y + 2, g.h) - max(y - 1, 0)) * (min(x + 2, g.w) - max(x - 1, 0)));
            const float axy = (rs[t] + rs[t + 1] + rs[t + 2]) / cnt, v = in[(ry + t) * E + rx];
            r = axy > 0.01f ? contrast_pow(axy, v, e1, e2) : 0.0f;
          }
          out[(ry + t) * E + rx] = r;
        }
      }
    });
  } else if (kind == 0) {
    const int size = K, h0 = size / 2, h1 = (size + 1) / 2;
    const float e1 = p0 - p1, e2 = p1;
    for_band(lo, hi, lo, hi, [&](int ry, int rx) {
      float r = 0.f;
      if (IN || inside(g, ry, rx)) {
        const int x = g.x0 + rx, y = g.y0 + ry;
        const int i0 = max(y - h0, 0), i1 = min(y + h1, g.h);
        const int j0 = max(x - h0, 0), j1 = min(x + h1, g.w);
        float cnt = 0.f, sum = 0.f;
        for (int yy = i0; yy < i1; ++yy)
          for (int xx = j0; xx < j1; ++xx) {
            cnt += 1.0f;
            sum += in[(yy - g.y0) * E + (xx - g.x0)];
          }
        const float axy = sum / cnt, v = in[ry * E + rx];
        r = axy > 0.01f ? contrast_pow(axy, v, e1, e2) : 0.0f;
      }
      out[ry * E + rx] = r;
    });
  }
  __syncthreads();
}

// Runs a filter chain on buf[0] (valid on [eh - H, eh + VT + H)); returns the
// buffer index holding the result on the tile band [eh, eh + VT).
__device__ int run_chain(const FilterDev* fl, int nf, int H, float* bufs[3], float* wsh, const Region& g, int eh)
{
  int cur = 0, halo = H;
  for (int s = 0; s < nf; ++s) {
    const FilterDev& f = fl[s];
    int nh = halo - f.R;
    int nxt = cur == 0 ? 1 : 0;
    if (g.in)
      apply_stage<true>(f, bufs[cur], bufs[nxt], bufs[2], wsh, g, eh - nh, eh + VT + nh);
    else
      apply_stage<false>(f, bufs[cur], bufs[nxt], bufs[2], wsh, g, eh - nh, eh + VT + nh);
    cur = nxt;
    halo = nh;
  }
  return cur;
}

__global__ void __launch_bounds__(VNT, ASC_VIEW_MINBLOCKS)
    k_view(const SceneDev* __restrict__ sc, Bufs b, double* __restrict__ cost, double* __restrict__ view_cost_out)
{
  extern __shared__ float smem[];
  __shared__ int s_tile, s_k;
  __shared__ bool s_last;
  __shared__ float red[8 * 6 * 2];
  __shared__ double ds[6], dc[3];
  __shared__ float wsh[32];
  Moments* msh = (Moments*)smem;          // reused by the merge
  const int ns = sc->slots;
  for (;;) {
    if (threadIdx.x == 0) {
      const int tl = atomicAdd(&b.C->fnext, 1);
      s_tile = tl;
      s_k = tl < b.C->ftiles ? b.ftile_iv[tl] : 0;
    }
    __syncthreads();
    const int tile = s_tile, k = s_k;
    __syncthreads();
    if (tile >= b.C->ftiles) return;
    const IV& r = b.iv[k];
    const int t = tile - b.foff[k];
    const int tx0 = (t % r.ftx) * VT, ty0 = (t / r.ftx) * VT;
    const ViewDev& V = sc->views[r.view];
    // this view's region edge E (its chain's halo) lays out the shared memory
    const int E = V.E, eh = (E - VT) / 2;
    float* bufs[3] = {smem, smem + E * E, smem + 2 * E * E};
    float* fdrr = smem + 3 * E * E;  // VT x VT final DRR, then f = DRR * mask
    // per region column / row: the radiograph texel pair and weight of the
    // film-plane mapping (image_axis; kNoTexel where the pixel maps outside)
    int* tcx = (int*)(smem + view_tail_floats(E));
    float* tax = (float*)(tcx + E);
    int* tcy = (int*)(tax + E);
    float* tay = (float*)(tcy + E);
    const int rx0 = tx0 - eh, ry0 = ty0 - eh;
    const Region g{rx0, ry0, E, r.w, r.h, rx0 >= 0 && ry0 >= 0 && rx0 + E <= r.w && ry0 + E <= r.h};
    const float* drr = b.drr + r.pix;
    // ---- DRR region; a region of zeros filters to zeros (every filter maps
    // 0 to 0), so its tile masks out entirely and adds nothing to the moments
    bool live;
    {
      // the region's words copied asynchronously (all in flight at once;
      // zero-filled outside the image), then tested for a nonzero DRR
      const int lo = eh - V.h_drr, hi = eh + VT + V.h_drr;
      for_band(lo, hi, lo, hi, [&](int ry, int rx) {
        const bool in = g.in || inside(g, ry, rx);
        const float* src = in ? drr + (long long)(g.y0 + ry) * r.w + g.x0 + rx : drr;
        const unsigned dst = (unsigned)__cvta_generic_to_shared(bufs[0] + ry * E + rx);
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(dst), "l"(src), "r"(in ? 4 : 0)
                     : "memory");
      });
      asm volatile("cp.async.commit_group;\n" ::: "memory");
      asm volatile("cp.async.wait_group 0;\n" ::: "memory");
      __syncthreads();
      bool nz = false;
      for_band(lo, hi, lo, hi, [&](int ry, int rx) { nz |= bufs[0][ry * E + rx] != 0.f; });
      live = __syncthreads_or(nz);
    }
    float mf = 0.f, mg = 0.f;
    if (live) {
      // the film-plane mapping of the region's columns and rows, in FP64
      // (visible to the radiograph band after the chain's barriers)
      for (int i = threadIdx.x; i < 2 * E; i += VNT) {
        const bool row = i >= E;
        const int j = row ? i - E : i;
        int k;
        float a = 0.f;
        const bool ok = row ? image_axis(r.vp[1], r.vp[3], g.y0 + j, r.h, V.ipf[1], V.ipf[3], V.rad_h, true, k, a)
                            : image_axis(r.vp[0], r.vp[2], g.x0 + j, r.w, V.ipf[0], V.ipf[2], V.rad_w, false, k, a);
        (row ? tcy : tcx)[j] = ok ? k : kNoTexel;
        (row ? tay : tax)[j] = a;
      }
      // ---- DRR chain
      {
        int res = run_chain(V.fdrr, V.n_drr, V.h_drr, bufs, wsh, g, eh);
        for (int i = threadIdx.x; i < VT * VT; i += VNT) fdrr[i] = bufs[res][(eh + i / VT) * E + eh + i % VT];
        __syncthreads();
      }
      // ---- radiograph crop and its chain
      int rres;
      {
        const int lo = eh - V.h_rad, hi = eh + VT + V.h_rad;
        for_band(lo, hi, lo, hi, [&](int ry, int rx) {
          float val = 0.f;
          const int kx = tcx[rx], ky = tcy[ry];
          if ((g.in || inside(g, ry, rx)) && kx != kNoTexel && ky != kNoTexel)
            val = 1.0f - bilinear_at(V.rad, V.rad_bps, V.rad_w, V.rad_h, kx, tax[rx], ky, tay[ry]);
          bufs[0][ry * E + rx] = val;
        });
        __syncthreads();
        rres = run_chain(V.frad, V.n_rad, V.h_rad, bufs, wsh, g, eh);
      }
      // ---- masks and moments (Tracker.cpp:744-770), two passes over the
      // tile: f = DRR * mask over fdrr, g = rad * mask over the chain result,
      // the m > 0.5 flags in the free blur buffer
      const unsigned n = (unsigned)r.w * (unsigned)r.h;
      const bool tree = sc->coverage == ASC_SUM_TREE && tree_needed(n);  // else every pixel counts
      const bool sad = sc->cf_model != 0;
      float* gres = bufs[rres];
      float* flag = bufs[2];
      // per tile: the pixels with mask 1 and their sums of f and g.  The
      // mask is 0 or 1 and f, g are 0 where it is 0, so these are also the
      // covered pixels' sums of mask, f and g.  Plain FP32 suffices for them:
      // an error in a tile's mean moves the centred moments only at second
      // order; the products are the sums that need compensating.
      float s[3] = {0.f, 0.f, 0.f};
      for (int i = threadIdx.x; i < VT * VT; i += VNT) {
        const int ly = i / VT, lx = i % VT, x = tx0 + lx, y = ty0 + ly;
        const int gi = (eh + ly) * E + eh + lx;
        float f = 0.f, gm = 0.f, fl = 0.f;
        if (x < r.w && y < r.h && (!tree || tree_keep((unsigned)(y * r.w + x), n))) {
          float d = fdrr[i], gg = gres[gi];
          float bg = 1.0f;
          if (V.bg && V.bg_thr >= 0.f) {
            int kx, ky;
            float ax, ay;
            bg = image_axis(r.vp[0], r.vp[2], x, r.w, V.ipf[0], V.ipf[2], V.bg_w, false, kx, ax) &&
                     image_axis(r.vp[1], r.vp[3], y, r.h, V.ipf[1], V.ipf[3], V.bg_h, true, ky, ay)
                   ? (V.bg_thr <= bilinear_at(V.bg, 32, V.bg_w, V.bg_h, kx, ax, ky, ay) ? 1.0f : 0.0f)
                   : 0.0f;
          }
          float m = bg * (d != 0.0f ? 1.0f : 0.0f);
          f = d * m;
          gm = gg * m;
          if (m > 0.5f) {
            fl = 1.f;
            s[0] += 1.f;
            s[1] += f;
            s[2] += gm;
          }
        }
        fdrr[i] = f;
        gres[gi] = gm;
        flag[i] = fl;
        // SAD needs the view's global means first: keep f and g for k_sad
        if (sad && x < r.w && y < r.h) b.fg[r.pix + (long long)y * r.w + x] = make_float2(f, gm);
      }
      block_sum_f<3>(s, red, ds + 3);
      if (threadIdx.x < 3) ds[threadIdx.x] = ds[3 + threadIdx.x];  // read by thread 0 after the next barrier
      const double cnt = ds[3];
      mf = cnt > 0 ? (float)(ds[4] / cnt) : 0.f;
      mg = cnt > 0 ? (float)(ds[5] / cnt) : 0.f;
      DFs c[3] = {};  // compensated co-moments about (mf, mg)
      for (int i = threadIdx.x; i < VT * VT && !sad; i += VNT)
        if (flag[i] != 0.f) {
          const int ly = i / VT, lx = i % VT;
          float a = fdrr[i] - mf, bb = gres[(eh + ly) * E + eh + lx] - mg;
          dfs_add_prod(c[0], a, a);
          dfs_add_prod(c[1], bb, bb);
          dfs_add_prod(c[2], a, bb);
        }
      block_sum_dfs<3>(c, red, dc);
    } else if (threadIdx.x == 0) {  // a tile of zeros adds nothing
      for (int j = 0; j < 6; ++j) ds[j] = 0.0;
      for (int j = 0; j < 3; ++j) dc[j] = 0.0;
    }
    if (threadIdx.x == 0) {
      Moments p = tile_moments(ds, dc, mf, mg);
      b.part[tile] = p;
      __threadfence();
      s_last = atomicAdd(&b.ivt[k], 1u) == (unsigned)(r.ftx * r.fty) - 1;
    }
    __syncthreads();
    if (!s_last) continue;
    __threadfence();
    // ---- last tile of this view: merge its tiles in FP64
    const int nt = r.ftx * r.fty, base = b.foff[k];
    Moments a = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = threadIdx.x; i < nt; i += blockDim.x) moments_merge(a, b.part[base + i]);
    msh[threadIdx.x] = a;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
      if (threadIdx.x < st) moments_merge(msh[threadIdx.x], msh[threadIdx.x + st]);
      __syncthreads();
    }
    if (threadIdx.x == 0 && sc->cf_model) {
      // HDist_kernels.cu:111-115: the means over the mask sum; k_sad takes
      // the view from here and reuses its tile tickets
      const Moments& m = msh[0];
      b.hmean[k] = make_double2(m.sf / m.sm, m.sg / m.sm);
      b.ivt[k] = 0;
    } else if (threadIdx.x == 0) {
      double vc = 1.0 - moments_ncc(msh[0]);
      b.vcost[k] = vc;
      __threadfence();
      const int item = k / ns;
      if (atomicAdd(&b.itt[item], 1u) == (unsigned)ns - 1) {
        __threadfence();
        finish_item(sc, b, item, cost);
        if (view_cost_out)
          for (int j = 0; j < ns; ++j) view_cost_out[item * ns + j] = b.vcost[item * ns + j];
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------- k_sad
// cf_model 1 (HDist_kernels.cu:111-203): per view, sum over mask > 0.5 of
// |(f - mean f) - (g - mean g)| with the means k_view left in hmean.  The
// mask is 0 or 1 and a DRR pixel under it is non-zero, so f != 0 marks the
// pixels under the mask; tiles k_view found without such pixels are skipped.
// Tile partials in FP32, the view's sum in FP64 by the view's last tile.
__global__ void __launch_bounds__(256) k_sad(const SceneDev* __restrict__ sc, Bufs b, double* __restrict__ cost,
                                             double* __restrict__ view_cost_out)
{
  __shared__ float red[8];
  __shared__ double dred[8];
  __shared__ bool s_last;
  const int nv = sc->slots, ftiles = b.C->ftiles;
  for (int tile = blockIdx.x; tile < ftiles; tile += gridDim.x) {
    const int k = b.ftile_iv[tile];
    const IV& r = b.iv[k];
    const int t = tile - b.foff[k];
    const int tx0 = (t % r.ftx) * VT, ty0 = (t / r.ftx) * VT;
    float a = 0.f;
    if (b.part[tile].n > 0) {
      const double2 mu = b.hmean[k];
      const float mf = (float)mu.x, mg = (float)mu.y;
      for (int i = threadIdx.x; i < VT * VT; i += blockDim.x) {
        const int x = tx0 + i % VT, y = ty0 + i / VT;
        if (x < r.w && y < r.h) {
          const float2 v = b.fg[r.pix + (long long)y * r.w + x];
          if (v.x != 0.f) a += fabsf((v.x - mf) - (v.y - mg));
        }
      }
    }
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
      float tot = 0.f;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
      b.tsad[tile] = tot;
      __threadfence();
      s_last = atomicAdd(&b.ivt[k], 1u) == (unsigned)(r.ftx * r.fty) - 1;
    }
    __syncthreads();
    if (s_last) {
      __threadfence();
      const int nt = r.ftx * r.fty, base = b.foff[k];
      double d = 0.0;
      for (int i = threadIdx.x; i < nt; i += blockDim.x) d += (double)__ldcg(b.tsad + base + i);
      for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
      if ((threadIdx.x & 31) == 0) dred[threadIdx.x >> 5] = d;
      __syncthreads();
      if (threadIdx.x == 0) {
        double vc = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) vc += dred[w];
        b.vcost[k] = vc;
        __threadfence();
        const int item = k / nv;
        if (atomicAdd(&b.itt[item], 1u) == (unsigned)nv - 1) {
          __threadfence();
          finish_item(sc, b, item, cost);
          if (view_cost_out)
            for (int j = 0; j < nv; ++j) view_cost_out[item * nv + j] = b.vcost[item * nv + j];
        }
      }
    }
    __syncthreads();
  }
}

// Copies view costs of items finished entirely in k_setup.
__global__ void k_copy_vcost(const double* vc, double* out, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = vc[i];
}

// ---------------------------------------------------------------- PSO
struct Swarm {
  double* x;    // [bone][particle][6]
  double* v;
  double* pbx;
  double* pbc;
  double* gx;   // [bone][6]
  double* gc;   // [bone]
  int* iter;
  int* frozen;  // [bone] the swarm stalled: its particles stay put
  int* bone;    // item -> bone
  double* manip;  // item -> x
};

__device__ __forceinline__ double urand(unsigned long long seed, unsigned long long ctr)
{
  unsigned long long z = seed + 0x9e3779b97f4a7c15ull * (ctr + 1);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  z ^= z >> 31;
  return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

__global__ void k_pso_init(Swarm s, int nb, int np, double lo, double hi, unsigned long long seed)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb * np) return;
  int p = i % np;
  for (int d = 0; d < 6; ++d) {
    double x = p == 0 ? 0.0 : lo + urand(seed, (unsigned long long)i * 6 + d) * (hi - lo);
    s.x[6 * i + d] = x;
    s.v[6 * i + d] = 0.0;
    s.pbx[6 * i + d] = x;
  }
  s.pbc[i] = 1e300;
  if (p == 0) {
    int b = i / np;
    for (int d = 0; d < 6; ++d) s.gx[6 * b + d] = 0.0;
    s.gc[b] = 1e300;
    s.frozen[b] = 0;
  }
  if (i == 0) *s.iter = 0;
}

// Synchronous velocity/position update (the rule of PSO.cpp:83-109 with
// runtime w, c1, c2) for every particle of every swarm.
__global__ void k_pso_update(Swarm s, int nb, int np, double w, double c1, double c2, unsigned long long seed)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nb * np) return;
  int b = i / np;
  s.bone[i] = b;
  if (s.frozen[b]) {  // re-scored where it is: the same cost, no best changes
    for (int d = 0; d < 6; ++d) s.manip[6 * i + d] = s.x[6 * i + d];
    return;
  }
  unsigned long long it = (unsigned long long)*s.iter + 1;
  for (int d = 0; d < 6; ++d) {
    unsigned long long c = ((it * (unsigned long long)(nb * np) + i) * 6 + d) * 2;
    double rp = urand(seed, c), rg = urand(seed, c + 1);
    double x = s.x[6 * i + d];
    double vv = w * s.v[6 * i + d] + c1 * rp * (s.pbx[6 * i + d] - x) + c2 * rg * (s.gx[6 * b + d] - x);
    s.v[6 * i + d] = vv;
    s.x[6 * i + d] = x + vv;
    s.manip[6 * i + d] = x + vv;
  }
}

// pBest / gBest update after an iteration's costs (one block per swarm).
__global__ void k_pso_best(Swarm s, int nb, int np, const double* cost)
{
  int b = blockIdx.x;
  __shared__ double bc[256];
  __shared__ int bi[256];
  double best = 1e300;
  int arg = -1;
  for (int p = threadIdx.x; p < np; p += blockDim.x) {
    int i = b * np + p;
    double c = cost[i];
    if (c < s.pbc[i]) {
      s.pbc[i] = c;
      for (int d = 0; d < 6; ++d) s.pbx[6 * i + d] = s.x[6 * i + d];
    }
    if (c < best || (c == best && arg >= 0 && p < arg)) {
      best = c;
      arg = p;
    }
  }
  bc[threadIdx.x] = best;
  bi[threadIdx.x] = arg;
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) {
      double o = bc[threadIdx.x + st];
      int oi = bi[threadIdx.x + st];
      if (o < bc[threadIdx.x] || (o == bc[threadIdx.x] && oi >= 0 && (bi[threadIdx.x] < 0 || oi < bi[threadIdx.x]))) {
        bc[threadIdx.x] = o;
        bi[threadIdx.x] = oi;
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    if (bi[0] >= 0 && bc[0] < s.gc[b]) {
      s.gc[b] = bc[0];
      for (int d = 0; d < 6; ++d) s.gx[6 * b + d] = s.x[6 * (b * np + bi[0]) + d];
    }
    if (b == 0) *s.iter += 1;
  }
}

}  // namespace

// ---------------------------------------------------------------- host side

struct asc_engine_s {
  SceneDev host;
  SceneDev* dev = nullptr;
  int max_items = 0, n_views = 0, n_bones = 0;
  Bufs b{};
  size_t smem = 0;
  int sms = 152;
  int view_blocks = 1;  // resident k_view blocks per SM (the occupancy limit)
  // launch shapes (asc_engine_set_launch): the defaults, or the tuning
  // table's entry for this engine's workload class
  asc_launch_config launch{ASC_RAY_MINBLOCKS, 0, 3};
  // k_view blocks per SM: the configured count, at most the occupancy limit
  int view_grid() const
  {
    const int want = launch.view_blocks_per_sm;
    return want > 0 ? std::min(want, view_blocks) : view_blocks;
  }
  bool prof = false;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  // device PSO: swarm state, the captured iteration and a private stream
  double* sw_buf = nullptr;
  int* sw_iter = nullptr;
  int* sw_frozen = nullptr;
  cudaGraphExec_t pso_exec = nullptr;
  double pso_key[5] = {0, 0, 0, 0, 0};
  cudaStream_t own_stream = nullptr;
  int* d_bone = nullptr;
  double* d_manip = nullptr;
  double* d_cost = nullptr;
  double* d_vcost = nullptr;
  // plain per-pose path: the reference's Tracker buffers (Tracker.cpp:292-298)
  std::vector<asc_view_desc> vdesc;
  std::vector<asc_bone_desc> bdesc;
  float *p_drr = nullptr, *p_rad = nullptr, *p_mask = nullptr, *p_bg = nullptr, *p_tmp = nullptr, *p_bgr = nullptr;
  double* p_res = nullptr;
  std::vector<void*> allocs;
  // empty-cell grids of bones replaced by asc_engine_set_bone, per (bone,
  // slot), with their capacity in bytes
  uint8_t* occ_own[MAX_BONES][MAX_SLOTS] = {};
  size_t occ_cap[MAX_BONES][MAX_SLOTS] = {};
  ~asc_engine_s()
  {
    for (void* p : allocs) cudaFree(p);
    for (auto& row : occ_own)
      for (uint8_t* p : row)
        if (p) cudaFree(p);
    for (cudaEvent_t x : ev)
      if (x) cudaEventDestroy(x);
    if (pso_exec) cudaGraphExecDestroy(pso_exec);
    if (own_stream) cudaStreamDestroy(own_stream);
  }
  template <class T>
  cudaError_t alloc(T*& p, size_t n)
  {
    cudaError_t e = cudaMalloc((void**)&p, std::max<size_t>(n, 1) * sizeof(T));
    if (e == cudaSuccess) allocs.push_back((void*)p);
    return e;
  }
};

static int prep_filters(const asc_filter_desc* in, int n, FilterDev* out, int* halo)
{
  if (n < 0 || n > MAX_FILTERS) return ASC_ERR_RANGE;
  int H = 0, m = 0;
  for (int i = 0; i < n; ++i) {
    const asc_filter_desc& f = in[i];
    if (!f.enabled) continue;  // View::filter copies through a disabled filter
    FilterDev d;
    memset(&d, 0, sizeof d);
    d.kind = f.kind;
    d.p0 = f.p0;
    d.p1 = f.p1;
    d.p2 = f.p2;
    if (f.kind == 1) {
      d.K = 3;
      d.R = 1;
    } else if (f.kind == 0) {
      d.K = (int)f.p2;
      if (d.K < 1) return ASC_ERR_ARG;
      d.R = std::max(d.K / 2, (d.K - 1) / 2);
    } else if (f.kind == 3 || f.kind == 4) {
      d.K = gauss_1d(f.p0, d.g, 32);
      if (d.K < 0) return ASC_ERR_RANGE;
      if (d.K == 1) continue;  // identity
      if (f.kind == 4) d.p1 = f.p1 < 1 ? 1 : f.p1;
      d.R = d.K / 2;
    } else {
      return ASC_ERR_ARG;
    }
    out[m++] = d;
    H += d.R;
  }
  *halo = H;
  return m;
}

static int fill_view(ViewDev& d, const asc_view_desc& v)
{
  memcpy(d.cam, v.frame, sizeof d.cam);
  frame_inverse(v.frame, d.cam_inv);
  memcpy(d.ip, v.image_plane, sizeof d.ip);
  memcpy(d.cvp, v.viewport, sizeof d.cvp);
  for (int j = 0; j < 4; ++j) d.ipf[j] = (float)v.viewport[j];
  if (!v.radiograph) return ASC_ERR_ARG;
  int bps;
  d.rad = image_data(v.radiograph, &d.rad_w, &d.rad_h, &bps);
  d.rad_bps = bps;
  if (bps == 32) return ASC_ERR_ARG;
  d.bg = nullptr;
  d.bg_thr = v.bg_threshold;
  if (v.background) {
    d.bg = (const float*)image_data(v.background, &d.bg_w, &d.bg_h, &bps);
    if (bps != 32) return ASC_ERR_ARG;
  }
  int n = prep_filters(v.drr_filters, v.n_drr_filters, d.fdrr, &d.h_drr);
  if (n < 0) return n;
  d.n_drr = n;
  n = prep_filters(v.rad_filters, v.n_rad_filters, d.frad, &d.h_rad);
  if (n < 0) return n;
  d.n_rad = n;
  d.E = VT + 2 * std::max(d.h_drr, d.h_rad);
  // three E x E stage buffers, the tile and the mapping tables must fit one
  // block's shared memory (227 KB less the static arrays)
  if (view_smem_floats(d.E) * sizeof(float) > 224 * 1024) return ASC_ERR_RANGE;
  return ASC_OK;
}

static void set_base(BoneDev& B, const double* xyzypr) { memcpy(B.base, xyzypr, sizeof B.base); }

namespace {
void apply_tuning(asc_engine_s* e);  // the tuning table's launch shapes, below

// k_view's dynamic shared-memory limit is an attribute of the function, one
// per device for the whole process: it only ever grows here, so an engine
// with a narrower filter chain never lowers it below what an earlier engine
// launches with.
std::mutex g_view_smem_mu;
size_t g_view_smem[64] = {};

cudaError_t ensure_view_smem(size_t bytes)
{
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err) return err;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> l(g_view_smem_mu);
  if (bytes <= g_view_smem[dev]) return cudaSuccess;
  err = cudaFuncSetAttribute(k_view, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (!err) g_view_smem[dev] = bytes;
  return err;
}
}

ASC_API int asc_engine_create(int n_views, const asc_view_desc* views, int n_bones, const asc_bone_desc* bones,
                              int rw, int rh, int max_items, int coverage, int cf_model, asc_engine* out)
{
  if (!views || !bones || !out || n_views < 1 || n_views > MAX_VIEWS || n_bones < 1 || n_bones > MAX_BONES ||
      rw < 1 || rh < 1 || max_items < 1 || (coverage != ASC_SUM_TREE && coverage != ASC_SUM_FULL))
    return ASC_ERR_ARG;
  if (cf_model != 0 && cf_model != 1) return ASC_ERR_ARG;
  Gate g(device_gate());
  // set-up work runs on a private stream, so that creating an engine does not
  // wait for other engines' work
  cudaStream_t cs = nullptr;
  if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking)) return ASC_ERR_CUDA;
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() { cudaStreamDestroy(s); }
  } cs_guard{cs};
  auto* e = new asc_engine_s();
  SceneDev& S = e->host;
  memset(&S, 0, sizeof S);
  S.n_views = n_views;
  S.n_bones = n_bones;
  S.rw = rw;
  S.rh = rh;
  S.coverage = coverage;
  S.cf_model = cf_model;
  S.slots = std::min(n_views, MAX_SLOTS);
  S.E = 0;
  for (int v = 0; v < n_views; ++v) {
    int rc = fill_view(S.views[v], views[v]);
    if (rc) {
      delete e;
      return rc;
    }
    S.views[v].rw = rw;
    S.views[v].rh = rh;
    S.E = std::max(S.E, S.views[v].E);
  }
  for (int i = 0; i < n_bones; ++i) {
    auto* vh = (asc_volume_host*)bones[i].volume;
    if (!vh) {
      delete e;
      return ASC_ERR_ARG;
    }
    BoneDev& B = S.bones[i];
    B.vol = vh->dev;
    memcpy(B.inv_scale, vh->inv_scale, sizeof B.inv_scale);
    memcpy(B.inv_trans, vh->inv_trans, sizeof B.inv_trans);
    memcpy(B.pivot, bones[i].pivot, sizeof B.pivot);
    frame_inverse(B.pivot, B.pivot_inv);
    set_base(B, bones[i].base_pose);
    B.visible = 1;
    B.n_slots = S.slots;  // bone i is scored in views 0 .. slots - 1
    for (int j = 0; j < S.slots; ++j) {
      B.view_of[j] = j;
      B.step[j] = bones[i].step[j];
      B.scale[j] = bones[i].step[j] * vh->dev.norm / bones[i].intensity[j];
      B.cut[j] = make_cutoff(bones[i].cutoff[j], vh->dev.norm, vh->dev.gmax);
      uint8_t* occ = nullptr;
      if (e->alloc(occ, occ_grid_bytes(occupancy_cells(vh->dev)))) {
        delete e;
        return ASC_ERR_NOMEM;
      }
      build_occupancy(vh->dev, occupancy_threshold(B.cut[j]), occ, cs);
      B.occ[j] = occ;
    }
  }
  e->max_items = max_items;
  e->n_views = n_views;
  e->n_bones = n_bones;
  size_t n_iv = (size_t)max_items * S.slots;
  size_t tiles = (size_t)((rw + VT - 1) / VT) * ((rh + VT - 1) / VT);
  cudaError_t err = e->alloc(e->dev, 1);
  if (!err) err = e->alloc(e->b.iv, n_iv);
  if (!err) err = e->alloc(e->b.roff, n_iv + 1);
  if (!err) err = e->alloc(e->b.foff, n_iv + 1);
  if (!err) err = e->alloc(e->b.drr, n_iv * (size_t)rw * rh);
  if (!err) err = e->alloc(e->b.part, n_iv * tiles);
  if (!err) err = e->alloc(e->b.ftile_iv, n_iv * tiles);
  if (!err && cf_model) err = e->alloc(e->b.fg, n_iv * (size_t)rw * rh);
  if (!err && cf_model) err = e->alloc(e->b.hmean, n_iv);
  if (!err && cf_model) err = e->alloc(e->b.tsad, n_iv * tiles);
  if (!err) err = e->alloc(e->b.vcost, n_iv);
  if (!err) err = e->alloc(e->b.ivt, n_iv);
  if (!err) err = e->alloc(e->b.itt, (size_t)max_items);
  // at most every ray tile of a full batch
  if (!err) err = e->alloc(e->b.fixt, n_iv * (size_t)((rw + RTX - 1) / RTX) * ((rh + RTY - 1) / RTY));
  if (!err) err = e->alloc(e->b.rtile_iv, n_iv * (size_t)((rw + RTX - 1) / RTX) * ((rh + RTY - 1) / RTY));
  if (!err) err = e->alloc(e->b.C, 1);
  if (!err) err = e->alloc(e->d_bone, (size_t)max_items);
  if (!err) err = e->alloc(e->d_manip, (size_t)max_items * 6);
  if (!err) err = e->alloc(e->d_cost, (size_t)max_items);
  if (!err) err = e->alloc(e->d_vcost, n_iv);
  const size_t npix = (size_t)rw * rh;
  if (!err) err = e->alloc(e->p_drr, npix);
  if (!err) err = e->alloc(e->p_rad, npix);
  if (!err) err = e->alloc(e->p_mask, npix);
  if (!err) err = e->alloc(e->p_bg, npix);
  if (!err) err = e->alloc(e->p_tmp, npix);
  if (!err) err = e->alloc(e->p_bgr, npix);
  if (!err) err = e->alloc(e->p_res, 1);
  if (!err) err = cudaMemcpyAsync(e->dev, &S, sizeof S, cudaMemcpyHostToDevice, cs);
  if (!err) err = cudaMemsetAsync(e->b.C, 0, sizeof(Counters), cs);
  if (err) {
    delete e;
    return cuda_status(err);
  }
  e->vdesc.assign(views, views + n_views);
  e->bdesc.assign(bones, bones + n_bones);
  if (asc_fill(e->p_bg, npix, 1.0f, cs) || cudaStreamSynchronize(cs)) {
    delete e;
    return ASC_ERR_CUDA;
  }
  // three stage buffers, the final DRR tile and VR + 2 rows of slack for the
  // column units' reads past a band
  e->smem = view_smem_floats(S.E) * sizeof(float);
  e->smem = std::max(e->smem, (size_t)256 * sizeof(Moments));
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&e->sms, cudaDevAttrMultiProcessorCount, dev);
  err = ensure_view_smem(e->smem);
  if (!err) err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&e->view_blocks, k_view, VNT, e->smem);
  if (err) {
    delete e;
    return cuda_status(err);
  }
  e->view_blocks = std::max(e->view_blocks, 1);
  apply_tuning(e);
  *out = e;
  return ASC_OK;
}

ASC_API int asc_engine_destroy(asc_engine e)
{
  if (!e) return ASC_ERR_ARG;
  Gate g(device_gate());
  cudaDeviceSynchronize();
  delete e;
  return ASC_OK;
}

ASC_API int asc_engine_set_base_pose(asc_engine e, int bone, const double xyzypr[6])
{
  if (!e || !xyzypr || bone < 0 || bone >= e->n_bones) return ASC_ERR_ARG;
  set_base(e->host.bones[bone], xyzypr);
  Gate g(device_gate());
  ASC_CUDA(cudaMemcpy(&e->dev->bones[bone].base, xyzypr, 6 * sizeof(double), cudaMemcpyHostToDevice));
  return ASC_OK;
}

ASC_API int asc_engine_set_visible(asc_engine e, int bone, int visible)
{
  if (!e || bone < 0 || bone >= e->n_bones) return ASC_ERR_ARG;
  e->host.bones[bone].visible = visible ? 1 : 0;
  Gate g(device_gate());
  ASC_CUDA(cudaMemcpy(&e->dev->bones[bone].visible, &e->host.bones[bone].visible, sizeof(int),
                      cudaMemcpyHostToDevice));
  return ASC_OK;
}

ASC_API int asc_engine_set_radiograph(asc_engine e, int view, asc_image rad)
{
  if (!e || !rad || view < 0 || view >= e->n_views) return ASC_ERR_ARG;
  ViewDev& d = e->host.views[view];
  int bps;
  const void* data = image_data(rad, &d.rad_w, &d.rad_h, &bps);
  if (bps == 32) return ASC_ERR_ARG;
  d.rad = data;
  d.rad_bps = bps;
  e->vdesc[view].radiograph = rad;  // the plain path and the image exports read it there
  Gate g(device_gate());
  ASC_CUDA(cudaMemcpy(&e->dev->views[view], &d, sizeof d, cudaMemcpyHostToDevice));
  return ASC_OK;
}

ASC_API int asc_engine_set_view(asc_engine e, int view, const asc_view_desc* desc, int rw, int rh)
{
  if (!e || !desc || view < 0 || view >= e->n_views || rw < 1 || rh < 1 || rw > e->host.rw || rh > e->host.rh)
    return ASC_ERR_ARG;
  ViewDev d;
  memset(&d, 0, sizeof d);
  int rc = fill_view(d, *desc);
  if (rc) return rc;
  d.rw = rw;
  d.rh = rh;
  Gate g(device_gate());
  const size_t need = view_smem_floats(d.E) * sizeof(float);
  if (need > e->smem) {  // a wider filter chain than the engine's views had so far
    int blocks = 0;
    ASC_CUDA(ensure_view_smem(need));
    ASC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_view, VNT, need));
    e->smem = need;
    e->view_blocks = std::max(blocks, 1);
    e->host.E = std::max(e->host.E, d.E);
    if (e->pso_exec) {  // its k_view node holds the old launch shape
      cudaGraphExecDestroy(e->pso_exec);
      e->pso_exec = nullptr;
    }
  }
  e->host.views[view] = d;
  e->vdesc[view] = *desc;
  ASC_CUDA(cudaMemcpy(&e->dev->views[view], &d, sizeof d, cudaMemcpyHostToDevice));
  return ASC_OK;
}

ASC_API int asc_engine_set_bone(asc_engine e, int bone, const asc_bone_desc* desc, int n_views, const int* views)
{
  if (!e || !desc || !desc->volume || bone < 0 || bone >= e->n_bones || n_views < 1 || n_views > e->host.slots ||
      !views)
    return ASC_ERR_ARG;
  for (int j = 0; j < n_views; ++j)
    if (views[j] < 0 || views[j] >= e->n_views) return ASC_ERR_ARG;
  auto* vh = (asc_volume_host*)desc->volume;
  BoneDev B = e->host.bones[bone];
  B.vol = vh->dev;
  memcpy(B.inv_scale, vh->inv_scale, sizeof B.inv_scale);
  memcpy(B.inv_trans, vh->inv_trans, sizeof B.inv_trans);
  memcpy(B.pivot, desc->pivot, sizeof B.pivot);
  frame_inverse(B.pivot, B.pivot_inv);
  set_base(B, desc->base_pose);
  B.visible = 1;
  B.n_slots = n_views;
  Gate g(device_gate());
  const size_t grid = occ_grid_bytes(occupancy_cells(vh->dev));
  for (int j = 0; j < n_views; ++j) {
    B.view_of[j] = views[j];
    B.step[j] = desc->step[j];
    B.scale[j] = desc->step[j] * vh->dev.norm / desc->intensity[j];
    B.cut[j] = make_cutoff(desc->cutoff[j], vh->dev.norm, vh->dev.gmax);
    uint8_t*& occ = e->occ_own[bone][j];
    if (e->occ_cap[bone][j] < grid) {
      if (occ) cudaFree(occ);
      occ = nullptr;
      e->occ_cap[bone][j] = 0;
      ASC_CUDA(cudaMalloc(&occ, grid));
      e->occ_cap[bone][j] = grid;
    }
    build_occupancy(vh->dev, occupancy_threshold(B.cut[j]), occ, nullptr);
    B.occ[j] = occ;
  }
  ASC_CUDA(cudaStreamSynchronize(nullptr));
  e->host.bones[bone] = B;
  e->bdesc[bone] = *desc;
  ASC_CUDA(cudaMemcpy(&e->dev->bones[bone], &B, sizeof B, cudaMemcpyHostToDevice));
  return ASC_OK;
}

// ---- the tuning table: launch shapes per workload class, written by the
// project's autotuner (autoscoper_gb300/tune.py) and read at engine creation.
// A class is (ceil log2 of the render pixels, ceil log2 of the largest
// volume's voxels, views); a line of the table holds
//   rpx vox views ray_blocks_per_sm view_blocks_per_sm ray_shape
// ('#' starts a comment).  An engine takes the entry of its render size and
// view count with the nearest volume class; without one it keeps the defaults.
namespace {
struct TuneEntry {
  int rpx, vox, views;
  asc_launch_config cfg;
};
std::mutex g_tune_mu;
std::vector<TuneEntry> g_tune;

int ceil_log2(double x)
{
  int k = 0;
  while ((double)(1ull << k) < x && k < 62) ++k;
  return k;
}

void workload_class(const asc_engine_s* e, int out[3])
{
  double vox = 0;
  for (int b = 0; b < e->n_bones; ++b) {
    const DevVolume& V = e->host.bones[b].vol;
    vox = std::max(vox, (double)V.nx * V.ny * V.nz);
  }
  out[0] = ceil_log2((double)e->host.rw * e->host.rh);
  out[1] = ceil_log2(vox);
  out[2] = e->n_views;
}

void apply_tuning(asc_engine_s* e)
{
  int c[3];
  workload_class(e, c);
  std::lock_guard<std::mutex> l(g_tune_mu);
  const TuneEntry* best = nullptr;
  for (const TuneEntry& t : g_tune)
    if (t.rpx == c[0] && t.views == c[2] && (!best || std::abs(t.vox - c[1]) < std::abs(best->vox - c[1])))
      best = &t;
  if (best) e->launch = best->cfg;
}
}  // namespace

ASC_API int asc_tuning_load(const char* path)
{
  if (!path) return ASC_ERR_ARG;
  FILE* f = fopen(path, "r");
  if (!f) return ASC_ERR_ARG;
  std::vector<TuneEntry> t;
  char line[512];
  int rc = ASC_OK;
  while (fgets(line, sizeof line, f)) {
    char* hash = strchr(line, '#');
    if (hash) *hash = 0;
    TuneEntry x;
    int n = sscanf(line, "%d %d %d %d %d %d", &x.rpx, &x.vox, &x.views, &x.cfg.ray_blocks_per_sm,
                   &x.cfg.view_blocks_per_sm, &x.cfg.ray_shape);
    if (n <= 0) continue;  // blank or comment
    if (n != 6 || x.cfg.ray_blocks_per_sm < 1 || x.cfg.ray_blocks_per_sm > ASC_RAY_MINBLOCKS ||
        x.cfg.view_blocks_per_sm < 0 || x.cfg.ray_shape < 2 || x.cfg.ray_shape > 4) {
      rc = ASC_ERR_ARG;
      break;
    }
    t.push_back(x);
  }
  fclose(f);
  if (rc) {
    set_error_message("asc_tuning_load: a line is not 'rpx vox views ray_blocks view_blocks ray_shape'");
    return rc;
  }
  std::lock_guard<std::mutex> l(g_tune_mu);
  g_tune = t;
  return ASC_OK;
}

ASC_API int asc_engine_workload_class(asc_engine e, int out[3])
{
  if (!e || !out) return ASC_ERR_ARG;
  workload_class(e, out);
  return ASC_OK;
}

ASC_API int asc_engine_set_launch(asc_engine e, const asc_launch_config* cfg)
{
  if (!e || !cfg || cfg->ray_blocks_per_sm < 1 || cfg->ray_blocks_per_sm > ASC_RAY_MINBLOCKS ||
      cfg->view_blocks_per_sm < 0 || cfg->ray_shape < 2 || cfg->ray_shape > 4)
    return ASC_ERR_ARG;
  Gate g(device_gate());
  e->launch = *cfg;
  if (e->pso_exec) {  // the captured iteration holds the old launch shapes
    cudaGraphExecDestroy(e->pso_exec);
    e->pso_exec = nullptr;
  }
  return ASC_OK;
}

ASC_API int asc_engine_get_launch(asc_engine e, asc_launch_config* cfg, int* view_blocks_max)
{
  if (!e || !cfg) return ASC_ERR_ARG;
  *cfg = e->launch;
  if (view_blocks_max) *view_blocks_max = e->view_blocks;
  return ASC_OK;
}

static int engine_launch(asc_engine e, int n, const int* bone, const double* manip, double* cost, double* vcost,
                         cudaStream_t s, bool capturing = false)
{
  const bool prof = e->prof && !capturing;
  if (prof) ASC_CUDA(cudaEventRecord(e->ev[0], s));
  k_setup_iv<<<(n * e->host.slots + 127) / 128, 128, 0, s>>>(e->dev, n, bone, manip, e->b);
  k_setup<<<1, 1024, 0, s>>>(e->dev, n, e->b, cost);
  k_tile_map<<<e->sms * 2, 256, 0, s>>>(e->b);
  if (prof) ASC_CUDA(cudaEventRecord(e->ev[1], s));
  k_ray<<<e->sms * e->launch.ray_blocks_per_sm, NRAY, 0, s>>>(e->dev, e->b, g_empty_skip, e->launch.ray_shape);
  k_ray_fix<<<e->sms * 4, FIX_THREADS, 0, s>>>(e->dev, e->b, g_empty_skip);
  if (prof) ASC_CUDA(cudaEventRecord(e->ev[2], s));
  k_view<<<e->sms * e->view_grid(), VNT, e->smem, s>>>(e->dev, e->b, cost, vcost);
  if (e->host.cf_model) k_sad<<<e->sms * 8, 256, 0, s>>>(e->dev, e->b, cost, vcost);
  if (prof) ASC_CUDA(cudaEventRecord(e->ev[3], s));
  if (vcost) k_copy_vcost<<<8, 256, 0, s>>>(e->b.vcost, vcost, n * e->host.slots);
  ASC_LAUNCH_CHECK();
  return ASC_OK;
}

ASC_API int asc_engine_profile(asc_engine e, int enable)
{
  if (!e) return ASC_ERR_ARG;
  if (enable && !e->ev[0])
    for (int i = 0; i < 4; ++i) ASC_CUDA(cudaEventCreate(&e->ev[i]));
  e->prof = enable != 0;
  return ASC_OK;
}

ASC_API int asc_engine_stats(asc_engine e, float ms[3], unsigned long long* samples, unsigned long long* pixels)
{
  if (!e) return ASC_ERR_ARG;
  if (ms) {
    if (!e->ev[0]) return ASC_ERR_STATE;
    ASC_CUDA(cudaEventSynchronize(e->ev[3]));
    for (int i = 0; i < 3; ++i) ASC_CUDA(cudaEventElapsedTime(&ms[i], e->ev[i], e->ev[i + 1]));
  }
  Counters C;
  ASC_CUDA(cudaMemcpy(&C, e->b.C, sizeof C, cudaMemcpyDeviceToHost));
  if (samples) *samples = C.samples;
  if (pixels) *pixels = C.pixels;
  return ASC_OK;
}

ASC_API int asc_engine_exact_rays(asc_engine e, int* n)
{
  if (!e || !n) return ASC_ERR_ARG;
  Counters C;
  ASC_CUDA(cudaMemcpy(&C, e->b.C, sizeof C, cudaMemcpyDeviceToHost));
  *n = C.nfix;
  return ASC_OK;
}

ASC_API int asc_engine_counters(asc_engine e, unsigned long long out[4])
{
  if (!e || !out) return ASC_ERR_ARG;
  Counters C;
  ASC_CUDA(cudaMemcpy(&C, e->b.C, sizeof C, cudaMemcpyDeviceToHost));
  out[0] = C.samples;
  out[1] = C.pixels;
  out[2] = C.marched;
  out[3] = C.slots;
  return ASC_OK;
}

ASC_API int asc_engine_eval(asc_engine e, int n, const int* bone, const double* manip, double* cost, double* vcost,
                            void* stream)
{
  if (!e || !bone || !manip || !cost || n < 1 || n > e->max_items) return ASC_ERR_ARG;
  return engine_launch(e, n, bone, manip, cost, vcost, S(stream));
}

ASC_API int asc_engine_eval_host(asc_engine e, int n, const int* bone, const double* manip, double* cost,
                                 double* vcost, void* stream)
{
  if (!e || !bone || !manip || !cost || n < 1 || n > e->max_items) return ASC_ERR_ARG;
  cudaStream_t s = S(stream);
  ASC_CUDA(cudaMemcpyAsync(e->d_bone, bone, n * sizeof(int), cudaMemcpyHostToDevice, s));
  ASC_CUDA(cudaMemcpyAsync(e->d_manip, manip, n * 6 * sizeof(double), cudaMemcpyHostToDevice, s));
  int rc = engine_launch(e, n, e->d_bone, e->d_manip, e->d_cost, vcost ? e->d_vcost : nullptr, s);
  if (rc) return rc;
  ASC_CUDA(cudaMemcpyAsync(cost, e->d_cost, n * sizeof(double), cudaMemcpyDeviceToHost, s));
  if (vcost)
    ASC_CUDA(cudaMemcpyAsync(vcost, e->d_vcost, (size_t)n * e->host.slots * sizeof(double), cudaMemcpyDeviceToHost, s));
  Counters C;
  ASC_CUDA(cudaMemcpyAsync(&C, e->b.C, sizeof C, cudaMemcpyDeviceToHost, s));
  ASC_CUDA(cudaStreamSynchronize(s));
  return C.error ? C.error : ASC_OK;
}

ASC_API int asc_engine_debug(asc_engine e, const float** drr, const int** layout)
{
  if (!e) return ASC_ERR_ARG;
  if (drr) *drr = e->b.drr;
  if (layout) *layout = (const int*)e->b.iv;
  return ASC_OK;
}

ASC_API int asc_engine_pso_stall(asc_engine e, int np, int n_iter, int max_stall, double w, double c1, double c2,
                                 double lo, double hi, uint64_t seed, double* best_manip, double* best_cost,
                                 long long* evals, int* iterations, void* stream)
{
  if (!e || np < 1 || n_iter < 1 || max_stall < 0 || !best_manip || !best_cost) return ASC_ERR_ARG;
  const int nb = e->n_bones, n = nb * np;
  if (n > e->max_items) return ASC_ERR_RANGE;
  cudaStream_t s = S(stream);
  if (!s) {  // one private non-blocking stream per engine
    if (!e->own_stream) ASC_CUDA(cudaStreamCreateWithFlags(&e->own_stream, cudaStreamNonBlocking));
    s = e->own_stream;
  }
  // swarm state: allocated once per engine, sized for max_items particles
  if (!e->sw_buf) {
    Gate g(device_gate());
    const size_t cap = (size_t)e->max_items, nbm = (size_t)e->n_bones;
    cudaError_t err = e->alloc(e->sw_buf, cap * 6 * 3 + cap + nbm * 6 + nbm);
    if (!err) err = e->alloc(e->sw_iter, 1);
    if (!err) err = e->alloc(e->sw_frozen, nbm);
    if (err) return cuda_status(err);
  }
  Swarm sw;
  sw.x = e->sw_buf;
  sw.v = sw.x + (size_t)n * 6;
  sw.pbx = sw.v + (size_t)n * 6;
  sw.pbc = sw.pbx + (size_t)n * 6;
  sw.gx = sw.pbc + n;
  sw.gc = sw.gx + nb * 6;
  sw.iter = e->sw_iter;
  sw.frozen = e->sw_frozen;
  sw.bone = e->d_bone;
  sw.manip = e->d_manip;
  const int tb = 128, gb = (n + tb - 1) / tb;
  k_pso_init<<<gb, tb, 0, s>>>(sw, nb, np, lo, hi, seed);
  cudaError_t err = cudaGetLastError();
  // one iteration = update -> setup -> ray -> view -> best, captured once per
  // (particles, w, c1, c2, seed) and replayed n_iter times
  const double key[5] = {(double)np, w, c1, c2, (double)seed};
  if (!err && (!e->pso_exec || memcmp(key, e->pso_key, sizeof key) != 0)) {
    if (e->pso_exec) {
      cudaGraphExecDestroy(e->pso_exec);
      e->pso_exec = nullptr;
    }
    cudaGraph_t graph = nullptr;
    Gate g(device_gate());
    err = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (!err) {
      k_pso_update<<<gb, tb, 0, s>>>(sw, nb, np, w, c1, c2, seed);
      engine_launch(e, n, e->d_bone, e->d_manip, e->d_cost, nullptr, s, true);
      k_pso_best<<<nb, 256, 0, s>>>(sw, nb, np, e->d_cost);
      err = cudaStreamEndCapture(s, &graph);
    }
    if (!err) err = cudaGraphInstantiate(&e->pso_exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (!err) memcpy(e->pso_key, key, sizeof key);
  }
  long long scored = 0;
  int it = 0;
  if (max_stall == 0) {
    for (; !err && it < n_iter; ++it) err = cudaGraphLaunch(e->pso_exec, s);
    scored = (long long)n * it;
  } else {
    // the stall rule of PSO.cpp:271-285 per swarm, read back after every
    // iteration: |gBest change| < 1e-4 counts a stall, > 1e-3 resets the
    // count, max_stall stalls in a row stop that swarm (it is frozen, and
    // the iterations end when every swarm is)
    std::vector<double> gc(nb), prev(nb, 1e300);
    std::vector<int> stall(nb, 0), frozen(nb, 0);
    int live = nb;
    for (; !err && it < n_iter && live > 0; ++it) {
      err = cudaGraphLaunch(e->pso_exec, s);
      scored += (long long)np * live;
      if (!err) err = cudaMemcpyAsync(gc.data(), sw.gc, nb * sizeof(double), cudaMemcpyDeviceToHost, s);
      if (!err) err = cudaStreamSynchronize(s);
      for (int b = 0; !err && b < nb; ++b) {
        if (frozen[b]) continue;
        const double d = std::fabs(gc[b] - prev[b]);
        if (d < 1e-4)
          ++stall[b];
        else if (d > 1e-3)
          stall[b] = 0;
        prev[b] = gc[b];
        if (stall[b] == max_stall) {
          frozen[b] = 1;
          --live;
          err = cudaMemcpyAsync(sw.frozen + b, &frozen[b], sizeof(int), cudaMemcpyHostToDevice, s);
        }
      }
    }
  }
  if (!err) err = cudaMemcpyAsync(best_manip, sw.gx, nb * 6 * sizeof(double), cudaMemcpyDeviceToHost, s);
  if (!err) err = cudaMemcpyAsync(best_cost, sw.gc, nb * sizeof(double), cudaMemcpyDeviceToHost, s);
  if (!err) err = cudaStreamSynchronize(s);
  if (evals) *evals = scored;
  if (iterations) *iterations = it;
  return err ? cuda_status(err) : ASC_OK;
}

ASC_API int asc_engine_pso(asc_engine e, int np, int n_iter, double w, double c1, double c2, double lo, double hi,
                           uint64_t seed, double* best_manip, double* best_cost, long long* evals, void* stream)
{
  return asc_engine_pso_stall(e, np, n_iter, 0, w, c1, c2, lo, hi, seed, best_manip, best_cost, evals, nullptr,
                              stream);
}

// ---------------------------------------------------------------- plain path
// Tracker::trackFrame (Tracker.cpp:583-773) one pose at a time over the plain
// per-operator kernels: the same launch sequence as the reference (ray cast,
// DRR filters, radiograph crop, radiograph filters, masks, three multiplies,
// NCC) with the NCC read back to the host after every view.  This is the
// drop-in form the batched engine is measured against.
static int chain_plain(const asc_filter_desc* fl, int nf, float*& cur, float*& other, int w, int h, cudaStream_t s)
{
  for (int i = 0; i < nf; ++i) {
    if (fl[i].enabled) {
      int rc = launch_filter(fl[i], cur, other, w, h, s);
      if (rc) return rc;
      std::swap(cur, other);
    }
  }
  return ASC_OK;
}

// One view of one bone at `xyzypr` over `vp`: the folded camera->volume
// matrix (Tracker.cpp:603-612 with RayCaster::setInvModelView).
static void view_matrix(const ViewDev& V, const BoneDev& B, const double* xyzypr, float m[12])
{
  double f[12], mv[12], imv[12], imv16[16];
  frame_from_xyzypr(xyzypr, f);
  frame_mul(V.cam_inv, f, mv);
  frame_inverse(mv, imv);
  frame_row_matrix(imv, imv16);
  fold_matrix(imv16, B.inv_scale, B.inv_trans, m);
}

// Whether every bone is scored in every view, slot j being view j (the
// layout asc_engine_create makes for up to MAX_SLOTS views).  The plain
// per-pose path and the image exports read the bones' per-view settings by
// view and need it; engines whose bones asc_engine_set_bone moved to other
// views serve batched evaluations only.
static bool identity_slots(const asc_engine_s* e)
{
  if (e->host.slots != e->n_views) return false;
  for (int b = 0; b < e->n_bones; ++b) {
    const BoneDev& B = e->host.bones[b];
    if (B.n_slots != e->n_views) return false;
    for (int j = 0; j < B.n_slots; ++j)
      if (B.view_of[j] != j) return false;
  }
  return true;
}

// RayCaster::render (RayCaster.cpp:123-143) of one bone into `out`: zeros
// for a hidden volume.
static int render_bone(const BoneDev& B, const asc_bone_desc& BD, int v, const float* m, const float* vpf,
                       float* out, int w, int h, cudaStream_t s)
{
  if (!B.visible) {
    ASC_CUDA(cudaMemsetAsync(out, 0, (size_t)w * h * sizeof(float), s));
    return ASC_OK;
  }
  return raycast_launch(B.vol, g_empty_skip ? B.occ[v] : nullptr, m, vpf, BD.step[v], BD.intensity[v], BD.cutoff[v],
                        out, w, h, s);
}

ASC_API int asc_engine_eval_plain(asc_engine e, int n, const int* bone, const double* manip, double* cost,
                                  double* view_cost, void* stream)
{
  if (!e || !bone || !manip || !cost || n < 1) return ASC_ERR_ARG;
  if (!identity_slots(e)) return ASC_ERR_STATE;
  cudaStream_t s = S(stream);
  const SceneDev& S_ = e->host;
  const int nv = e->n_views;
  for (int it = 0; it < n; ++it) {
    int bi = bone[it];
    if (bi < 0 || bi >= e->n_bones) return ASC_ERR_ARG;
    const BoneDev& B = S_.bones[bi];
    const asc_bone_desc& BD = e->bdesc[bi];
    double base[12], man[12], t1[12], t2[12], xyz[6];
    frame_from_xyzypr(B.base, base);
    frame_from_axis_angle(manip + 6 * it, man);
    frame_mul(base, B.pivot_inv, t1);
    frame_mul(t1, man, t2);
    frame_mul(t2, B.pivot, t1);
    frame_to_xyzypr(t1, xyz);
    frame_from_xyzypr(xyz, t1);
    double total = 0.0;
    for (int v = 0; v < nv; ++v) {
      const ViewDev& V = S_.views[v];
      const asc_view_desc& VD = e->vdesc[v];
      double mv[12], imv[12], imv16[16], vp[4];
      float m[12];
      frame_mul(V.cam_inv, t1, mv);
      frame_inverse(mv, imv);
      frame_row_matrix(imv, imv16);
      fold_matrix(imv16, B.inv_scale, B.inv_trans, m);
      double vc;
      if (!calculate_viewport(mv, V.cam, V.ip, B.inv_scale, B.inv_trans, vp)) {
        vc = 9999.0;
      } else {
        double fw = vp[2] * S_.rw / V.cvp[2], fh = vp[3] * S_.rh / V.cvp[3];
        unsigned w = fw > 0 ? (unsigned)fw : 0u, h = fh > 0 ? (unsigned)fh : 0u;
        if (w > (unsigned)S_.rw || h > (unsigned)S_.rh) return ASC_ERR_RANGE;
        if (w == 0 || h == 0) {
          vc = S_.cf_model ? 0.0 : 1.0 - 1e5;
        } else {
          float vpf[4] = {(float)vp[0], (float)vp[1], (float)vp[2], (float)vp[3]};
          int rc = render_bone(B, BD, v, m, vpf, e->p_drr, w, h, s);
          float *d = e->p_drr, *o = e->p_tmp;
          if (!rc) rc = chain_plain(VD.drr_filters, VD.n_drr_filters, d, o, w, h, s);
          // the DRR chain ping-pongs p_drr/p_tmp and leaves one of them free (o);
          // the radiograph chain ping-pongs p_rad/o; p_mask stays free
          if (!rc) rc = asc_rad_render(VD.radiograph, V.ipf, vpf, e->p_rad, w, h, s);
          float *r = e->p_rad, *ro = o;
          if (!rc) rc = chain_plain(VD.rad_filters, VD.n_rad_filters, r, ro, w, h, s);
          float* mask = e->p_mask;
          float* bgm = e->p_bg;  // all ones: the mask of a disabled background
          if (!rc && VD.background && VD.bg_threshold >= 0) {
            bgm = e->p_bgr;
            rc = asc_background_render(VD.background, V.ipf, vpf, VD.bg_threshold, bgm, w, h, s);
          }
          if (!rc) rc = asc_drr_background(d, mask, w, h, s);
          if (!rc) rc = asc_multiply(bgm, mask, mask, w, h, s);
          if (!rc) rc = asc_multiply(r, mask, r, w, h, s);
          if (!rc) rc = asc_multiply(d, mask, d, w, h, s);
          double res = 0;
          if (!rc)
            rc = S_.cf_model ? asc_hdist(d, r, mask, w * h, S_.coverage, e->p_res, s)
                             : asc_ncc(d, r, mask, w * h, S_.coverage, e->p_res, s);
          if (!rc) {
            cudaError_t err = cudaMemcpyAsync(&res, e->p_res, sizeof(double), cudaMemcpyDeviceToHost, s);
            if (!err) err = cudaStreamSynchronize(s);
            if (err) rc = cuda_status(err);
          }
          if (rc) return rc;
          vc = S_.cf_model ? res : 1.0 - res;  // Tracker.cpp:762-770
        }
      }
      if (view_cost) view_cost[it * nv + v] = vc;
      total += vc;
    }
    cost[it] = total < 0 ? 9999.0 : total;
  }
  return ASC_OK;
}

// ---------------------------------------------------------------- Tracker::optimize
namespace {

struct EvalCtx {
  asc_engine e;
  cudaStream_t s;
  long long evals;
};

// Batch cost for asc_amoeba_batch: candidate i belongs to simplex (bone) who[i].
int engine_batch_cost(int n, const int* who, const double* x, double* y, void* ctx)
{
  EvalCtx* c = (EvalCtx*)ctx;
  const int cap = c->e->max_items;
  for (int i0 = 0; i0 < n; i0 += cap) {
    const int m = std::min(cap, n - i0);
    int rc = asc_engine_eval_host(c->e, m, who + i0, x + 6 * (size_t)i0, y + i0, nullptr, c->s);
    if (rc) return rc;
  }
  c->evals += n;
  return ASC_OK;
}

// The pose base * V^-1 * manip * V as xyzypr (Tracker.cpp:479-483, :558-562).
void compose_pose(const BoneDev& B, const double* base6, const double* manip, double* out)
{
  double base[12], man[12], t1[12], t2[12];
  frame_from_xyzypr(base6, base);
  frame_from_axis_angle(manip, man);
  frame_mul(base, B.pivot_inv, t1);
  frame_mul(t1, man, t2);
  frame_mul(t2, B.pivot, t1);
  frame_to_xyzypr(t1, out);
}

}  // namespace

ASC_API int asc_engine_optimize_frame_ex(asc_engine e, const asc_opt_params* p, double* pose_out, double* raw_out,
                                         double* cost_out, long long* evals_out, void* stream)
{
  if (!e || !p || !pose_out) return ASC_ERR_ARG;
  const int nb = e->n_bones;
  if (nb * 7 > e->max_items) return ASC_ERR_RANGE;
  cudaStream_t s = S(stream);
  if (!s) {  // the engine's private stream, so that engines on other threads overlap
    if (!e->own_stream) ASC_CUDA(cudaStreamCreateWithFlags(&e->own_stream, cudaStreamNonBlocking));
    s = e->own_stream;
  }
  EvalCtx ctx{e, s, 0};
  std::vector<int> bones(nb);
  for (int b = 0; b < nb; ++b) bones[b] = b;
  // the frame's pose as read from the key curves (the engine's base poses)
  std::vector<double> xyzypr(6 * nb);
  for (int b = 0; b < nb; ++b)
    for (int j = 0; j < 6; ++j) xyzypr[6 * b + j] = e->host.bones[b].base[j];
  // init_ncc = minimizationFunc(0) (Tracker.cpp:441-443)
  std::vector<double> zero(6 * nb, 0.0), init(nb), fin(nb);
  int rc = engine_batch_cost(nb, bones.data(), zero.data(), init.data(), &ctx);
  if (rc) return rc;
  if (p->method == 0) {
    // PSO, then move the pose to the swarm's best: the key curves take the
    // stored (rounded) pose, which the simplex evaluates around, while the
    // final composition starts from the unrounded one (Tracker.cpp:445-491)
    std::vector<double> best(6 * nb), bc(nb);
    long long ev = 0;
    rc = asc_engine_pso_stall(e, p->n_particles, p->n_iter, p->max_stall, p->w, p->c1, p->c2, p->lo, p->hi, p->seed,
                              best.data(), bc.data(), &ev, nullptr, (void*)s);
    if (rc) return rc;
    ctx.evals += ev;
    for (int b = 0; b < nb; ++b) {
      double np[6], st[6];
      compose_pose(e->host.bones[b], xyzypr.data() + 6 * b, best.data() + 6 * b, np);
      keycurve_store(np, st);
      for (int j = 0; j < 6; ++j) xyzypr[6 * b + j] = np[j];
      rc = asc_engine_set_base_pose(e, b, st);
      if (rc) return rc;
    }
  }
  // Downhill Simplex from the offsets (Tracker.cpp:493-515), all bones at once
  const int mp = 7;
  std::vector<double> P((size_t)nb * mp * 6, 0.0), Y((size_t)nb * mp);
  std::vector<int> who((size_t)nb * mp);
  for (int b = 0; b < nb; ++b)
    for (int i = 0; i < mp; ++i) {
      who[b * mp + i] = b;
      if (i > 0) P[((size_t)b * mp + i) * 6 + (i - 1)] = p->offsets[i - 1];
    }
  rc = engine_batch_cost(nb * mp, who.data(), P.data(), Y.data(), &ctx);
  if (rc) return rc;
  std::vector<int> iters(nb);
  rc = asc_amoeba_batch(engine_batch_cost, &ctx, nb, P.data(), Y.data(), 6, p->ftol, iters.data());
  if (rc) return rc;
  // final_ncc = minimizationFunc(P[1]); keep the start of the simplex if not better (Tracker.cpp:517-525)
  std::vector<double> vert0(6 * nb);
  for (int b = 0; b < nb; ++b)
    for (int j = 0; j < 6; ++j) vert0[6 * b + j] = P[(size_t)b * mp * 6 + j];
  rc = engine_batch_cost(nb, bones.data(), vert0.data(), fin.data(), &ctx);
  if (rc) return rc;
  for (int b = 0; b < nb; ++b) {
    const bool take = p->method != 0 || fin[b] < init[b];
    double manip[6] = {0, 0, 0, 0, 0, 0};
    if (take)
      for (int j = 0; j < 6; ++j) manip[j] = vert0[6 * b + j];
    double np[6], st[6];
    compose_pose(e->host.bones[b], xyzypr.data() + 6 * b, manip, np);
    keycurve_store(np, st);
    rc = asc_engine_set_base_pose(e, b, st);
    if (rc) return rc;
    for (int j = 0; j < 6; ++j) pose_out[6 * b + j] = st[j];
    if (raw_out)
      for (int j = 0; j < 6; ++j) raw_out[6 * b + j] = np[j];
    if (cost_out) cost_out[b] = take ? fin[b] : init[b];
  }
  if (evals_out) *evals_out = ctx.evals;
  return ASC_OK;
}

ASC_API int asc_engine_optimize_frame(asc_engine e, const asc_opt_params* p, double* pose_out, double* cost_out,
                                      long long* evals_out, void* stream)
{
  return asc_engine_optimize_frame_ex(e, p, pose_out, nullptr, cost_out, evals_out, stream);
}

ASC_API int asc_keycurve_store(const double pose[6], double out[6])
{
  if (!pose || !out) return ASC_ERR_ARG;
  keycurve_store(pose, out);
  return ASC_OK;
}

ASC_API int asc_engine_track(asc_engine e, int n_frames, const asc_image* rads, const asc_track_params* tp,
                             double* poses, double* costs, long long* evals_out, void* stream)
{
  if (!e || n_frames < 1 || !rads || !tp || !poses || tp->repeats < 1 || (tp->dframe != 1 && tp->dframe != -1) ||
      tp->guess < 0 || tp->guess > 2)
    return ASC_ERR_ARG;
  const int nb = e->n_bones, nv = e->n_views, d = tp->dframe;
  long long evals = 0;
  for (int i = 0; i < n_frames; ++i) {
    const int f = d > 0 ? i : n_frames - 1 - i;
    double* pf = poses + (size_t)f * nb * 6;
    for (int v = 0; v < nv; ++v) {
      int rc = asc_engine_set_radiograph(e, v, rads[(size_t)f * nv + v]);
      if (rc) return rc;
    }
    // initial guess (Tracker.cpp:388-426); i frames are already tracked in
    // this direction.  Without a guess the frame starts from its key curve
    // value: its own key, or for an unkeyed frame the last tracked frame's
    // pose (a key curve holds its last key beyond it)
    for (int b = 0; b < nb; ++b) {
      const double* prev = poses + ((size_t)(f - d) * nb + b) * 6;
      double g[6];
      if (tp->guess == 2 && i > 1) {
        double a[12], c[12], x[12];
        frame_from_xyzypr(poses + ((size_t)(f - 2 * d) * nb + b) * 6, a);
        frame_from_xyzypr(prev, c);
        frame_linear_extrap(a, c, x);
        frame_to_xyzypr(x, g);
        keycurve_store(g, pf + 6 * b);
      } else if (tp->guess == 1 && i > 0) {
        keycurve_store(prev, pf + 6 * b);
      } else if (i > 0 && !(tp->keyed && tp->keyed[f])) {
        for (int j = 0; j < 6; ++j) pf[6 * b + j] = prev[j];
      }
    }
    for (int r = 0; r < tp->repeats; ++r) {
      for (int b = 0; b < nb; ++b) {
        int rc = asc_engine_set_base_pose(e, b, pf + 6 * b);
        if (rc) return rc;
      }
      long long ev = 0;
      int rc = asc_engine_optimize_frame(e, &tp->opt, pf, costs ? costs + (size_t)f * nb : nullptr, &ev, stream);
      if (rc) return rc;
      evals += ev;
    }
  }
  if (evals_out) *evals_out = evals;
  return ASC_OK;
}

ASC_API int asc_engine_optimize_curves(asc_engine e, const asc_pose_curve* curves, int frame, int n_frames,
                                       const asc_track_params* tp, double* costs, long long* evals_out, void* stream)
{
  if (!e || !curves || !tp || tp->repeats < 0 || tp->guess < 0 || frame < 0 || frame >= n_frames)
    return ASC_ERR_ARG;
  const int nb = e->n_bones, d = tp->dframe;
  for (int b = 0; b < nb; ++b)
    if (!curves[b]) return ASC_ERR_ARG;
  // initial guess (Tracker.cpp:386-426), written into the curves at `frame`
  const int behind = d > 0 ? frame : n_frames - frame - 1;
  for (int b = 0; b < nb; ++b) {
    double p1[6], p2[6], g[6];
    if (tp->guess == 2 && behind > 1) {
      double a[12], c[12], x[12];
      asc_pose_curve_eval(curves[b], frame - 2 * d, p1);
      asc_pose_curve_eval(curves[b], frame - d, p2);
      frame_from_xyzypr(p1, a);
      frame_from_xyzypr(p2, c);
      frame_linear_extrap(a, c, x);
      frame_to_xyzypr(x, g);
      asc_pose_curve_insert(curves[b], frame, g, ASC_CURVE_ALL);
    } else if (tp->guess == 1 && behind > 0) {
      asc_pose_curve_eval(curves[b], frame - d, g);
      asc_pose_curve_insert(curves[b], frame, g, ASC_CURVE_ALL);
    }
  }
  // repeats (Tracker.cpp:428-572): from the curves' pose at the frame, the
  // optimized pose inserted back
  long long evals = 0;
  std::vector<double> stored(6 * nb), raw(6 * nb);
  for (int r = 0; r < tp->repeats; ++r) {
    for (int b = 0; b < nb; ++b) {
      double base[6];
      asc_pose_curve_eval(curves[b], frame, base);
      int rc = asc_engine_set_base_pose(e, b, base);
      if (rc) return rc;
    }
    long long ev = 0;
    int rc = asc_engine_optimize_frame_ex(e, &tp->opt, stored.data(), raw.data(), costs, &ev, stream);
    if (rc) return rc;
    evals += ev;
    for (int b = 0; b < nb; ++b) asc_pose_curve_insert(curves[b], frame, raw.data() + 6 * b, ASC_CURVE_ALL);
  }
  if (evals_out) *evals_out = evals;
  return ASC_OK;
}

// ---------------------------------------------------------------- images
ASC_API int asc_engine_render_drr(asc_engine e, int view, const double* poses, const double* viewport, float* out,
                                  void* stream)
{
  if (!e || !poses || !out || view < 0 || view >= e->n_views) return ASC_ERR_ARG;
  if (!identity_slots(e)) return ASC_ERR_STATE;
  cudaStream_t s = S(stream);
  const ViewDev& V = e->host.views[view];
  const asc_view_desc& VD = e->vdesc[view];
  const double full[4] = {-V.cvp[2] / 2, -V.cvp[3] / 2, V.cvp[2], V.cvp[3]};
  const double* vp = viewport ? viewport : full;
  // the render size of the viewport (Tracker.cpp:617-621), at most the buffer
  const double fw = vp[2] * e->host.rw / V.cvp[2], fh = vp[3] * e->host.rh / V.cvp[3];
  const int w = fw > 0 ? std::min((int)fw, e->host.rw) : 0, h = fh > 0 ? std::min((int)fh, e->host.rh) : 0;
  if (w == 0 || h == 0) return ASC_OK;
  const float vpf[4] = {(float)vp[0], (float)vp[1], (float)vp[2], (float)vp[3]};
  // View::renderDrr (View.cpp:201-231): each bone's DRR merged (sum clamped
  // to 1) into a zeroed buffer, then the view's DRR filters
  ASC_CUDA(cudaMemsetAsync(e->p_mask, 0, (size_t)w * h * sizeof(float), s));
  for (int b = 0; b < e->n_bones; ++b) {
    const BoneDev& B = e->host.bones[b];
    const asc_bone_desc& BD = e->bdesc[b];
    float m[12];
    view_matrix(V, B, poses + 6 * b, m);
    if (!B.visible) continue;  // its zeros leave the merge unchanged
    int rc = raycast_launch(B.vol, g_empty_skip ? B.occ[view] : nullptr, m, vpf, BD.step[view], BD.intensity[view],
                            BD.cutoff[view], e->p_drr, w, h, s);
    if (!rc) rc = asc_merge(e->p_mask, e->p_drr, e->p_mask, w, h, s);
    if (rc) return rc;
  }
  float *d = e->p_mask, *o = e->p_tmp;
  int rc = chain_plain(VD.drr_filters, VD.n_drr_filters, d, o, w, h, s);
  if (!rc) ASC_CUDA(cudaMemcpyAsync(out, d, (size_t)w * h * sizeof(float), cudaMemcpyDeviceToDevice, s));
  return rc;
}

ASC_API int asc_engine_image_data(asc_engine e, int view, int bone, const double pose[6], float* rad, float* drr,
                                  float* mask, int* width, int* height, void* stream)
{
  if (!e || !pose || !rad || !drr || !mask || view < 0 || view >= e->n_views || bone < 0 || bone >= e->n_bones)
    return ASC_ERR_ARG;
  if (!identity_slots(e)) return ASC_ERR_STATE;
  cudaStream_t s = S(stream);
  const ViewDev& V = e->host.views[view];
  const asc_view_desc& VD = e->vdesc[view];
  const BoneDev& B = e->host.bones[bone];
  const asc_bone_desc& BD = e->bdesc[bone];
  // Tracker::getImageData (Tracker.cpp:865-925): the whole image, viewport
  // (-w/2, -h/2, w, h) of the camera's, at the render size
  const double vp[4] = {-V.cvp[2] / 2, -V.cvp[3] / 2, V.cvp[2], V.cvp[3]};
  const int w = e->host.rw, h = e->host.rh;
  const float vpf[4] = {(float)vp[0], (float)vp[1], (float)vp[2], (float)vp[3]};
  float m[12];
  view_matrix(V, B, pose, m);
  int rc = render_bone(B, BD, view, m, vpf, e->p_drr, w, h, s);
  float *d = e->p_drr, *o = e->p_tmp;
  if (!rc) rc = chain_plain(VD.drr_filters, VD.n_drr_filters, d, o, w, h, s);
  if (!rc) rc = asc_rad_render(VD.radiograph, V.ipf, vpf, e->p_rad, w, h, s);
  float *r = e->p_rad, *ro = o;
  if (!rc) rc = chain_plain(VD.rad_filters, VD.n_rad_filters, r, ro, w, h, s);
  float* bgm = e->p_bg;
  if (!rc && VD.background && VD.bg_threshold >= 0) {
    bgm = e->p_bgr;
    rc = asc_background_render(VD.background, V.ipf, vpf, VD.bg_threshold, bgm, w, h, s);
  }
  if (!rc) rc = asc_drr_background(d, mask, w, h, s);
  if (!rc) rc = asc_multiply(bgm, mask, mask, w, h, s);
  if (!rc) rc = asc_multiply(r, mask, rad, w, h, s);
  if (!rc) rc = asc_multiply(d, mask, drr, w, h, s);
  if (rc) return rc;
  if (width) *width = w;
  if (height) *height = h;
  return ASC_OK;
}
