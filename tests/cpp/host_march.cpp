// The DRR ray march of the CUDA kernels (asc_march.cuh) compiled as host
// C++: lets CPU tests check the kernel's own ray set-up, sample positions,
// empty-cell skipping and accumulation against the FP64 oracle.
#include <vector>

#include "host_march_shim.h"
#include "../../include/autoscoper_gb300.h"
#include "../../autoscoper_gb300/csrc/asc_march.cuh"

using namespace asc;

static uint16_t to_bf16(unsigned v)
{
  uint32_t b;
  float f = (float)v;
  std::memcpy(&b, &f, 4);
  b += 0x7fffu + ((b >> 16) & 1u);  // round to nearest even
  return (uint16_t)(b >> 16);
}

extern "C" int hm_raycast(const uint16_t* vol, int nx, int ny, int nz, int storage, int skip, const float* m,
                          const float* vp, float step, float intensity, float cutoff, float* out, int w, int h,
                          int* nsamples)
{
  if (storage != ASC_STORE_U16 && storage != ASC_STORE_BF16 && storage != ASC_STORE_F32) return -1;
  std::vector<uint32_t> pairs(padded_words(nx, ny, nz, storage));
  pack_pairs(nx, ny, nz, storage, [&](int x, int y, int z) {
    unsigned v = vol[((size_t)z * ny + y) * nx + x];
    if (storage == ASC_STORE_F32) {
      const float f = (float)v;
      uint32_t b;
      std::memcpy(&b, &f, 4);
      return b;
    }
    return (uint32_t)(storage == ASC_STORE_BF16 ? to_bf16(v) : v);
  }, pairs.data());
  const int px = nx + 2 * PAD, pxy = px * (ny + 2 * PAD);
  DevVolume V{pairs.data(), nx, ny, nz, px, pxy, storage, 1.0f / 65535.0f, 0.f};
  V.gmax = volume_gmax(nx, ny, nz, [&](int x, int y, int z) {
    const size_t i = (size_t)(z + PAD) * pxy + (size_t)(y + PAD) * px + (x + PAD);
    return storage == ASC_STORE_BF16  ? voxel_value<ASC_STORE_BF16>(V, i)
           : storage == ASC_STORE_F32 ? voxel_value<ASC_STORE_F32>(V, i)
                                      : voxel_value<ASC_STORE_U16>(V, i);
  });
  const Cutoff cut = make_cutoff(cutoff, V.norm, V.gmax);
  // occupancy as k_occupancy builds it
  const int bx = occ_dim(nx), by = occ_dim(ny), bz = occ_dim(nz);
  const size_t ncell = (size_t)bx * by * bz;
  std::vector<uint8_t> occ(occ_grid_bytes(ncell) + 16);
  uint8_t* o8 = occ.data() + ((16 - ((uintptr_t)occ.data() & 15)) & 15);  // 16-byte aligned, as cudaMalloc's
  for (int cz = -OCC_PAD; cz < bz - OCC_PAD; ++cz)
    for (int cy = -OCC_PAD; cy < by - OCC_PAD; ++cy)
      for (int cx = -OCC_PAD; cx < bx - OCC_PAD; ++cx) {
        const size_t c = ((size_t)(cz + OCC_PAD) * by + (cy + OCC_PAD)) * bx + (cx + OCC_PAD);
        int box[4];
        o8[c] = occ_cell(cx, cy, cz, nx, ny, nz, occupancy_threshold(cut), [&](int x, int y, int z) {
          const size_t i = (size_t)(z + PAD) * pxy + (size_t)(y + PAD) * px + (x + PAD);
          return storage == ASC_STORE_BF16  ? voxel_value<ASC_STORE_BF16>(V, i)
                 : storage == ASC_STORE_F32 ? voxel_value<ASC_STORE_F32>(V, i)
                                            : voxel_value<ASC_STORE_U16>(V, i);
        }, box);
        std::memcpy(o8 + occ_box_offset(ncell) + 16 * c, box, 16);
      }
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      RaySetup r;
      float d = 0.f;
      int n = 0;
      df sx, sy;
      df_split((double)vp[2] / (double)w, sx.h, sx.l);
      df_split((double)vp[3] / (double)h, sy.h, sy.l);
      if (ray_setup(m, vp, x, y, sx, sy, step, nx, ny, nz, r)) {
        const uint8_t* o = skip ? o8 : nullptr;
        const float acc = storage == ASC_STORE_BF16  ? march<ASC_STORE_BF16>(V, o, r, cut)
                          : storage == ASC_STORE_F32 ? march<ASC_STORE_F32>(V, o, r, cut)
                                                     : march<ASC_STORE_U16>(V, o, r, cut);
        d = acc * (step * V.norm / intensity);
        n = r.K;
      }
      out[y * w + x] = std::min(std::max(d, 0.f), 1.f);
      nsamples[y * w + x] = n;
    }
  return 0;
}

// Occupancy bytes of a u16 volume's padded grid at a cutoff (normalized as
// hm_raycast's): counts[b] = cells with byte b (0 empty, 1 trimmed to the
// box, 2 box covering the cell).
extern "C" void hm_occupancy(const uint16_t* vol, int nx, int ny, int nz, float cutoff, long long* counts)
{
  const float g = volume_gmax(nx, ny, nz, [&](int x, int y, int z) { return (float)vol[((size_t)z * ny + y) * nx + x]; });
  // the grids' threshold, as the library builds them
  const float cut = occupancy_threshold(make_cutoff(cutoff, 1.0f / 65535.0f, g));
  const int bx = occ_dim(nx), by = occ_dim(ny), bz = occ_dim(nz);
  counts[0] = counts[1] = counts[2] = 0;
  for (int cz = -OCC_PAD; cz < bz - OCC_PAD; ++cz)
    for (int cy = -OCC_PAD; cy < by - OCC_PAD; ++cy)
      for (int cx = -OCC_PAD; cx < bx - OCC_PAD; ++cx) {
        int box[4];
        const uint8_t b = occ_cell(cx, cy, cz, nx, ny, nz, cut, [&](int x, int y, int z) {
          return (float)vol[((size_t)z * ny + y) * nx + x];
        }, box);
        ++counts[b];
      }
}

// Soundness of the cutoff band (Cutoff): every sample of every ray of the
// image, its FP32 value as the march computes it (a one-sample march block
// whose band (lo = +inf, hi = -inf) counts every value and marks none, so
// the block returns the value itself) and the exact decision
// (sample_above).  counts[0] = samples, [1] = samples
// whose FP32 decision (v > raw) differs from the exact one, [2] = such
// samples outside the ray's band, [3] = samples in the band.
extern "C" void hm_band(const uint16_t* vol, int nx, int ny, int nz, const float* m, const float* vp, float step,
                        float cutoff, int w, int h, long long* counts)
{
  std::vector<uint32_t> pairs(padded_words(nx, ny, nz, ASC_STORE_U16));
  pack_pairs(nx, ny, nz, ASC_STORE_U16, [&](int x, int y, int z) { return (uint32_t)vol[((size_t)z * ny + y) * nx + x]; },
             pairs.data());
  const int px = nx + 2 * PAD, pxy = px * (ny + 2 * PAD);
  DevVolume V{pairs.data(), nx, ny, nz, px, pxy, ASC_STORE_U16, 1.0f / 65535.0f, 0.f};
  V.gmax = volume_gmax(nx, ny, nz, [&](int x, int y, int z) { return (float)vol[((size_t)z * ny + y) * nx + x]; });
  const Cutoff cut = make_cutoff(cutoff, V.norm, V.gmax);
  counts[0] = counts[1] = counts[2] = counts[3] = 0;
  df sx, sy;
  df_split((double)vp[2] / (double)w, sx.h, sx.l);
  df_split((double)vp[3] / (double)h, sy.h, sy.l);
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      RaySetup r;
      if (!ray_setup(m, vp, x, y, sx, sy, step, nx, ny, nz, r)) continue;
      float lo, hi;
      cutoff_bounds(cut, r.dX.h, r.dY.h, r.dZ.h, lo, hi);
      for (int k = 0; k < r.K; ++k) {
        const int kb = k - k % REBASE, j = k % REBASE;
        const float v = march_block<ASC_STORE_U16, false>(V, r, kb, j, j, INFINITY, -INFINITY, cut);
        const bool fp32 = v > cut.raw, exact = sample_above<ASC_STORE_U16>(V, r, k, cut);
        const bool in_band = v > lo && v < hi;
        ++counts[0];
        counts[1] += fp32 != exact;
        counts[2] += fp32 != exact && !in_band;
        counts[3] += in_band;
      }
    }
}
