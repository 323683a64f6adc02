// Ray march of the DRR ray caster: device volume layout, double-float ray
// set-up and the FP32 march.  Self-contained so that it also compiles as
// host C++ (tests/cpp/host_march.cpp provides the few intrinsics).
#pragma once

namespace asc {

// --------------------------------------------------------------------------
// Device volume.  Voxels are stored "x-paired": a word for voxel x holds
// voxel x in its low half and voxel x+1 in its high half, so that one 32-bit
// word carries both x taps of a trilinear sample.  The grid is padded by PAD
// voxels on every side with copies of the edge voxels, which is
// clamp-to-edge addressing (cutil_create_tex_obj.h:18-23) built into the
// layout: the taps of any sample inside the volume box need no per-sample
// clamping.  The halves are u16 integers (ASC_STORE_U16), IEEE half
// (ASC_STORE_F16) or bfloat16 (ASC_STORE_BF16), all holding the stored
// integer value; `norm` (1/65535 or 1/255) turns a raw value into the
// normalized float that cudaReadModeNormalizedFloat would return.
// --------------------------------------------------------------------------
constexpr int PAD = 2;
// Each voxel holds two words, the x-pairs of rows y and y+1 ("quads"), so
// that one 8-byte load fetches four taps of a sample and a sample takes two
// loads (ASC_QUADS=0 builds the one-word pair layout, four loads a sample).
#ifndef ASC_QUADS
#define ASC_QUADS 1
#endif
constexpr int QROWS = ASC_QUADS ? 2 : 1;  // x-pairs (rows y, y+1) per voxel

// 32-bit words per voxel: an x-pair is one word of two 16-bit halves, or two
// FP32 words (ASC_STORE_F32).
__host__ __device__ inline int voxel_words(int storage) { return (storage == ASC_STORE_F32 ? 2 : 1) * QROWS; }

struct DevVolume {
  const uint32_t* pairs;  // (nz + 2 PAD) slices of (ny + 2 PAD) rows of (nx + 2 PAD) voxels
  int nx, ny, nz;         // voxels of the volume itself
  int px, pxy;            // padded row and slice pitch in voxels
  int storage;
  float norm;
  float gmax;  // largest step between neighbouring stored voxels along an axis (raw units)
};

inline size_t padded_words(int nx, int ny, int nz, int storage)
{
  return (size_t)voxel_words(storage) * (nx + 2 * PAD) * (ny + 2 * PAD) * (nz + 2 * PAD);
}

// Fills the padded layout from stored values v(x, y, z) of an nx x ny x nz
// volume (host side): 16-bit halves, or FP32 bits for ASC_STORE_F32.
template <class F>
inline void pack_pairs(int nx, int ny, int nz, int storage, F v, uint32_t* out)
{
  const int px = nx + 2 * PAD, py = ny + 2 * PAD, pz = nz + 2 * PAD, wpv = voxel_words(storage);
  auto cl = [](int i, int n) { return i < 0 ? 0 : (i > n - 1 ? n - 1 : i); };
  for (int zp = 0; zp < pz; ++zp)
    for (int yp = 0; yp < py; ++yp)
      for (int xp = 0; xp < px; ++xp) {
        const int z = cl(zp - PAD, nz), x0 = cl(xp - PAD, nx), x1 = cl(xp - PAD + 1, nx);
        uint32_t* o = out + (((size_t)zp * py + yp) * px + xp) * wpv;
        for (int r = 0; r < QROWS; ++r) {
          const int y = cl(yp - PAD + r, ny);
          if (storage == ASC_STORE_F32) {
            o[2 * r] = v(x0, y, z);
            o[2 * r + 1] = v(x1, y, z);
          } else {
            o[r] = v(x0, y, z) | (v(x1, y, z) << 16);
          }
        }
      }
}

// The largest step between neighbouring voxels along an axis, max |v(p + e_i)
// - v(p)|, of stored values v(x, y, z) (host side).  Bounds the slope of the
// trilinear interpolant along every axis, so it turns a sample's position
// error into a value error (Cutoff).  The clamp-to-edge apron adds no steps.
template <class F>
inline float volume_gmax(int nx, int ny, int nz, F v)
{
  float g = 0.f;
  for (int z = 0; z < nz; ++z)
    for (int y = 0; y < ny; ++y)
      for (int x = 0; x < nx; ++x) {
        const float a = v(x, y, z);
        if (x + 1 < nx) g = std::max(g, std::fabs(v(x + 1, y, z) - a));
        if (y + 1 < ny) g = std::max(g, std::fabs(v(x, y + 1, z) - a));
        if (z + 1 < nz) g = std::max(g, std::fabs(v(x, y, z + 1) - a));
      }
  return g;
}

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

// Linear interpolation between the two halves of a paired word with weight
// a on the high half.  For u16 halves the values stay biased by 2^23: the
// biased values, their difference and the removal of the bias are exact in
// FP32, so this equals fmaf(a, hi - lo, lo) of the unbiased values.
template <int STORE>
__device__ __forceinline__ float lerp_pair(uint32_t w, float a)
{
  if (STORE == ASC_STORE_U16) {
    // 2^23 + v: the half's two bytes under the exponent byte 0x4b
    const float lo = __uint_as_float(__byte_perm(w, 0x4b000000u, 0x7610)),
                hi = __uint_as_float(__byte_perm(w, 0x4b000000u, 0x7632));
    return fmaf(a, hi - lo, lo - 8388608.0f);
  } else {
    float lo, hi;
    unpack<STORE>(w, lo, hi);
    return fmaf(a, hi - lo, lo);
  }
}

// Raw value of padded voxel i (the low half of its first x-pair).
template <int STORE>
__device__ __forceinline__ float voxel_value(const DevVolume& V, size_t i)
{
  const uint32_t w = V.pairs[(size_t)voxel_words(STORE) * i];
  if constexpr (STORE == ASC_STORE_F32) {
    return __uint_as_float(w);
  } else {
    float lo, hi;
    unpack<STORE>(w, lo, hi);
    return lo;
  }
}

// The eight taps of a sample whose lower taps are voxel i, as its four
// x-pairs (rows y, y+1 of slices z, z+1) in the storage's own form, and their
// linear interpolation along x with weight a.
template <int STORE>
struct Taps {
  uint32_t w[4];
};
template <>
struct Taps<ASC_STORE_F32> {
  float2 p[4];
};

template <int STORE>
__device__ __forceinline__ Taps<STORE> fetch_taps(const uint32_t* __restrict__ P, unsigned i, unsigned px,
                                                  unsigned pxy)
{
  Taps<STORE> t;
  if constexpr (STORE == ASC_STORE_F32) {
#if ASC_QUADS
    const float4* Q = reinterpret_cast<const float4*>(P);
    const float4 a = __ldg(Q + i), c = __ldg(Q + i + pxy);
    t.p[0] = make_float2(a.x, a.y);
    t.p[1] = make_float2(a.z, a.w);
    t.p[2] = make_float2(c.x, c.y);
    t.p[3] = make_float2(c.z, c.w);
#else
    const float2* Q = reinterpret_cast<const float2*>(P);
    t.p[0] = __ldg(Q + i);
    t.p[1] = __ldg(Q + i + px);
    t.p[2] = __ldg(Q + i + pxy);
    t.p[3] = __ldg(Q + i + pxy + px);
#endif
  } else {
#if ASC_QUADS
    const uint2* Q = reinterpret_cast<const uint2*>(P);
    const uint2 a = __ldg(Q + i), c = __ldg(Q + i + pxy);
    t.w[0] = a.x;
    t.w[1] = a.y;
    t.w[2] = c.x;
    t.w[3] = c.y;
#else
    t.w[0] = __ldg(P + i);
    t.w[1] = __ldg(P + i + px);
    t.w[2] = __ldg(P + i + pxy);
    t.w[3] = __ldg(P + i + pxy + px);
#endif
  }
  return t;
}

template <int STORE>
__device__ __forceinline__ float lerp_tap(const Taps<STORE>& t, int k, float a)
{
  if constexpr (STORE == ASC_STORE_F32)
    return fmaf(a, t.p[k].y - t.p[k].x, t.p[k].x);
  else
    return lerp_pair<STORE>(t.w[k], a);
}

// ---- two samples at once.  The packed FP32 operations of sm_100 and later
// (fma.rn.f32x2, add.f32x2) apply one IEEE operation to each half, so every
// value below equals, bit for bit, the scalar expression cited beside it.
__device__ __forceinline__ float2 bcast2(float a) { return make_float2(a, a); }
// a - b with one rounding
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, bcast2(-1.0f), a); }

// lerp_tap of tap word k of samples A (x) and B (y), weights a
template <int STORE>
__device__ __forceinline__ float2 lerp_tap2(const Taps<STORE>& A, const Taps<STORE>& B, int k, float2 a)
{
  float2 lo, hi;
  if constexpr (STORE == ASC_STORE_F32) {
    lo = make_float2(A.p[k].x, B.p[k].x);
    hi = make_float2(A.p[k].y, B.p[k].y);
  } else if constexpr (STORE == ASC_STORE_U16) {
    // lerp_pair: fmaf(a, hi - lo, lo - 2^23) of the biased halves
    lo = make_float2(__uint_as_float(__byte_perm(A.w[k], 0x4b000000u, 0x7610)),
                     __uint_as_float(__byte_perm(B.w[k], 0x4b000000u, 0x7610)));
    hi = make_float2(__uint_as_float(__byte_perm(A.w[k], 0x4b000000u, 0x7632)),
                     __uint_as_float(__byte_perm(B.w[k], 0x4b000000u, 0x7632)));
    return __ffma2_rn(a, sub2(hi, lo), __fadd2_rn(lo, bcast2(-8388608.0f)));
  } else {
    unpack<STORE>(A.w[k], lo.x, hi.x);
    unpack<STORE>(B.w[k], lo.y, hi.y);
  }
  return __ffma2_rn(a, sub2(hi, lo), lo);  // fmaf(a, hi - lo, lo)
}

// The trilinear values of samples A and B (march_block's accumulate)
template <int STORE>
__device__ __forceinline__ float2 trilinear2(const Taps<STORE>& A, const Taps<STORE>& B, float2 wx, float2 wy,
                                             float2 wz)
{
  const float2 e00 = lerp_tap2<STORE>(A, B, 0, wx), e10 = lerp_tap2<STORE>(A, B, 1, wx);
  const float2 e01 = lerp_tap2<STORE>(A, B, 2, wx), e11 = lerp_tap2<STORE>(A, B, 3, wx);
  const float2 f0 = __ffma2_rn(wy, sub2(e10, e00), e00);  // fmaf(wy, e10 - e00, e00)
  const float2 f1 = __ffma2_rn(wy, sub2(e11, e01), e01);
  return __ffma2_rn(wz, sub2(f1, f0), f0);                // fmaf(wz, f1 - f0, f0)
}

// Occupancy of OCC^3-voxel cells for one cutoff (OCC = 8): cell (cx, cy, cz)
// is empty (byte 0) when every voxel of [8c-1, 8c+10) on each axis is <=
// cutoff.  That range holds the taps of nonzero weight of every sample at a
// texel coordinate in (8c-1, 8c+9), i.e. within one voxel of the cell's own
// [8c, 8c+8), so a walk may place a sample in a cell with an error of up to a
// voxel.  A trilinear sample is a convex combination of its taps (each FP32
// lerp stays between its ends), so a sample placed in an empty cell is <=
// cutoff and adds exactly nothing to the DRR (RayCaster_kernels.cu:189); the
// march skips it.
//
// An occupied cell also keeps the box of its voxels above the cutoff: a
// sample can touch such a voxel v only at texel coordinates in [v-1, v+1)
// per axis, and an eighth of a voxel of margin covers the walk's placement
// error (FP32 positions, ~1e-4 voxel).  The walk marches only the cell's
// samples that lie in the box, so a cell occupied by a few voxels costs a few
// samples.  Bounds are int16 eighths of a voxel, so trimming applies to
// volumes of at most OCC_TRIM_MAX voxels per axis.
constexpr int OCC = 8;
constexpr int OCC_LO = 1, OCC_HI = 2;  // apron voxels below and above a cell
// The grid holds OCC_PAD cells of margin on every side (cells -2 .. b + 1 of
// an axis of b cells), so that a walk, whose cells stay within one of the
// box's, indexes it without clamping.
constexpr int OCC_PAD = 2;
constexpr int OCC_TRIM_MAX = 4094;
__host__ __device__ __forceinline__ int occ_dim(int n) { return (n + OCC - 1) / OCC + 2 * OCC_PAD; }

// The grid of n cells: n occupancy bytes, then at the next 16-byte boundary
// n boxes, each an int4 of (lo | hi << 16) per axis x, y, z (int16 texel
// coordinates in eighths of a voxel) and a spare word.
__host__ __device__ __forceinline__ size_t occ_box_offset(size_t n) { return (n + 15) & ~(size_t)15; }
__host__ __device__ __forceinline__ size_t occ_grid_bytes(size_t n) { return occ_box_offset(n) + 16 * n; }

// Occupancy byte and box of cell (cx, cy, cz) (margin cells included) of an
// nx x ny x nz volume; val(x, y, z) is the voxel's raw value.
template <class Val>
__host__ __device__ inline uint8_t occ_cell(int cx, int cy, int cz, int nx, int ny, int nz, float cutoff, Val&& val,
                                            int* box)
{
  int lo[3] = {0x7fff, 0x7fff, 0x7fff}, hi[3] = {-0x7fff, -0x7fff, -0x7fff};
  bool any = false;
  const int a = -OCC_LO, e = OCC + OCC_HI;
  for (int z = max(cz * OCC + a, 0); z < min(cz * OCC + e, nz); ++z)
    for (int y = max(cy * OCC + a, 0); y < min(cy * OCC + e, ny); ++y)
      for (int x = max(cx * OCC + a, 0); x < min(cx * OCC + e, nx); ++x)
        if (val(x, y, z) > cutoff) {
          any = true;
          lo[0] = min(lo[0], 8 * (x - 1) - 1);
          hi[0] = max(hi[0], 8 * (x + 1) + 1);
          lo[1] = min(lo[1], 8 * (y - 1) - 1);
          hi[1] = max(hi[1], 8 * (y + 1) + 1);
          lo[2] = min(lo[2], 8 * (z - 1) - 1);
          hi[2] = max(hi[2], 8 * (z + 1) + 1);
        }
  for (int i = 0; i < 3; ++i) box[i] = (lo[i] & 0xffff) | (int)((unsigned)hi[i] << 16);
  box[3] = 0;
  // byte 2: the box covers the cell with a voxel to spare on every side, so
  // trimming keeps every sample the walk places in the cell
  const int c[3] = {cx, cy, cz};
  bool covers = true;
  for (int i = 0; i < 3; ++i) covers = covers && lo[i] <= 8 * (OCC * c[i] - 1) && hi[i] >= 8 * (OCC * c[i] + OCC + 1);
  return any ? (covers ? 2 : 1) : 0;
}


// ---- double-float arithmetic: a value is the unevaluated sum h + l of two
// FP32 numbers (Dekker/Knuth error-free transformations with FMA), 44 to 48
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
  return {s, __fadd_rn(b, -__fadd_rn(s, -a))};
}

// Sum with an exact sum of the high parts and the low parts added in FP32
// (Dekker's addition): relative error ~2^-44 of the larger operand.  Every
// use here needs absolute accuracy in coordinates and ray parameters whose
// magnitudes are at most ~1e4 (voxels, samples): ~1e-9 at worst, far below
// the FP32 rounding of the sample positions the march then uses.
__device__ __forceinline__ df df_add(df a, df b)
{
  df s = df_two_sum(a.h, b.h);
  s.l = __fadd_rn(s.l, __fadd_rn(a.l, b.l));
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

// 1/a and 1/sqrt(a) in double-float: one Newton step from the FP32 value
// (relative error of the FP32 start squared, ~1e-13).
__device__ __forceinline__ df df_rcp(df a)
{
  const float r = __frcp_rn(a.h);
  const df e = df_add(df{1.0f, 0.f}, df_neg(df_mulf(a, r)));  // 1 - a r
  return df_fast(r, __fmul_rn(r, e.h));
}

__device__ __forceinline__ df df_rsqrt(df a)
{
  const float r = rsqrtf(a.h);
  const df r2 = df_mul(df{r, 0.f}, df{r, 0.f});
  const df e = df_add(df{1.0f, 0.f}, df_neg(df_mul(a, r2)));  // 1 - a r^2
  return df_fast(r, __fmul_rn(0.5f * r, e.h));
}

// A float value as a double-float from a double (host or device).
__device__ __host__ __forceinline__ void df_split(double d, float& h, float& l)
{
  h = (float)d;
  l = (float)(d - (double)h);
}

// The cutoff test of the march (RayCaster_kernels.cu:189: density += s >
// cutoff ? step * s : 0), on raw voxel values.  The reference compares
// raw / vmax with c (vmax 65535 or 255); the exact threshold is c x vmax,
// kept as the double-float (th, tl); the FP32 march compares with raw = c /
// norm.
//
// An FP32 sample v differs from the exact trilinear value at its exact
// position by at most
//   u (3 |v| + 11 G)                   the seven lerps' roundings (the taps
//                                      lie within 3 G of v)
//   + G u (9 + 130 (|dX| + |dY| + |dZ|))  the position per axis: the
//                                      fraction's rounding, the FMA of the
//                                      sample offset (values below 1 + 64 |d|)
//                                      and the offset times the dropped low
//                                      part of d; the interpolant's slope
//                                      along an axis is at most G
// with u = 2^-24, G = DevVolume::gmax and d the per-sample step of each axis
// in voxels; raw differs from c x vmax by at most 2 u |raw|.  So a sample
// with |v - raw| >= t0 + t1 (|dX| + |dY| + |dZ|), t0 = u (8 |raw| + 24 G) +
// 1e-6 and t1 = 140 u G, lies on the same side of the threshold in FP32 as
// exactly (3 u |raw| of t0 cover the roundings of the band's ends).  The
// march decides such samples in FP32 and flags the rest (the band); a
// flagged march is redone with the samples in the band decided from their
// double-float position and a double-float trilinear value against (th, tl)
// (sample_above).
//
// When |raw| <= 2 t0 the band is dropped (t0 = t1 = 0, the samples above
// raw, i.e. at or above the next float hi0, counted): a sample decided the
// other way then adds or leaves out at most |raw| + t0, a few times the FP32
// error every counted sample carries, and a cutoff of 0 keeps its empty
// cells (a band reaching below 0 would leave none).
//
// The occupancy grids are built at raw - t0 (<= c x vmax): a cell whose
// voxels all lie at or below it holds only samples that the exact test
// leaves out.
struct Cutoff {
  float raw;      // c / norm, the FP32 threshold
  float hi0;      // raw, or with the band dropped the next float above it
  float t0, t1;   // the band's half-width: t0 + t1 (|dX| + |dY| + |dZ|)
  float th, tl;   // c x vmax as a double-float
};

__host__ __device__ inline Cutoff make_cutoff(float c, float norm, float gmax)
{
  Cutoff k;
  k.raw = c / norm;
  const float u = 5.9604645e-8f;  // 2^-24
  k.t0 = u * (8.0f * fabsf(k.raw) + 24.0f * gmax) + 1e-6f;
  k.t1 = 140.0f * u * gmax;
  k.hi0 = k.raw;
  if (!(fabsf(k.raw) > 2.0f * k.t0)) {
    k.t0 = k.t1 = 0.f;
    k.hi0 = nextafterf(k.raw, INFINITY);
  }
  const double vmax = (double)(int)(1.0f / norm + 0.5f);
  df_split((double)c * vmax, k.th, k.tl);
  return k;
}

// The occupancy grids' threshold (Cutoff).
__host__ __device__ inline float occupancy_threshold(const Cutoff& k) { return k.raw - k.t0; }

// The band of a ray with per-sample steps dX, dY, dZ: samples in (lo, hi)
// are decided exactly, samples at or above hi count.
__host__ __device__ inline void cutoff_bounds(const Cutoff& k, float dX, float dY, float dZ, float& lo, float& hi)
{
  const float tol = fmaf(k.t1, fabsf(dX) + fabsf(dY) + fabsf(dZ), k.t0);
  lo = k.raw - tol;
  hi = k.hi0 + tol;
}

// Per-ray set-up of cuda_volume_render_kernel (RayCaster_kernels.cu:144-186)
// for pixel (x, y) of an image over viewport `vp`, with camera->volume matrix
// m (3x4 row-major, normalisation folded), in double-float: the reference's
// FP32 set-up misplaces the far intersection by ~1e-7 of its length, which
// shifts every sample of the ray; here positions agree with FP64 to ~1e-6
// voxel.  (sxh, sxl) and (syh, syl) are vp[2] / w and vp[3] / h as
// double-floats, so that u = vp[0] + x vp[2] / w.  Sample k (k = 0 .. K-1)
// sits at t = far - k, texel coordinates (X - k dX, Y - k dY, Z - k dZ) with
// texel centres at integers.
struct RaySetup {
  int K;
  df X, Y, Z, dX, dY, dZ;
};

__device__ __forceinline__ bool ray_setup(const float* m, const float* vp, int x, int y, df sx, df sy, float step,
                                          int nx, int ny, int nz, RaySetup& r)
{
  const df u = df_add(df{vp[0], 0.f}, df_mulf(sx, (float)x));
  const df v = df_add(df{vp[1], 0.f}, df_mulf(sy, (float)y));
  const df sc = df_mulf(df_rsqrt(df_add(df_add(df_mul(u, u), df_mul(v, v)), df{4.0f, 0.f})), step);
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
    const df rd = df_rcp(d[i]);
    df a = df_mul(df_two_sum(lo[i], -o[i]), rd);
    df b = df_mul(df_two_sum(hi[i], -o[i]), rd);
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

// The march re-bases its FP32 coordinates every REBASE samples (march_block).
#ifndef ASC_REBASE
#define ASC_REBASE 64
#endif
constexpr int REBASE = ASC_REBASE;

// A ray's walk through the occupancy grid (a 3-D DDA over cells, in units of
// samples): the sample index of each axis' next cell-plane crossing, the
// samples between crossings and the cell step per crossing.  FP32 throughout:
// a sample's cell comes out within ~1e-3 voxel of the exact one, far inside
// the one-voxel apron of the occupancy grid.
struct CellWalk {
  float tx, ty, tz;     // next crossing per axis (sample index; +inf if none)
  float dtx, dty, dtz;  // samples between crossings
  int cell;             // the current cell's index in the padded grid
  int ix, iy, iz;       // index change per crossing of each axis
  unsigned last;        // the grid's last index (a bound no walk reaches)
  int steps;            // crossings a ray can make through the grid
};

__device__ __forceinline__ void walk_axis(float C, float dC, float kf, float& t, float& dt, int& c, int& st)
{
  // coordinate at sample k: C - k dC
  const float X = fmaf(-kf, dC, C);
  c = __float2int_rd(X * (1.0f / OCC));
  if (dC > 0.f) {  // decreasing: next plane at OCC * c
    st = -1;
    const float ri = __frcp_rn(dC);
    dt = OCC * ri;
    t = fmaf(X - (float)(OCC * c), ri, kf);
  } else if (dC < 0.f) {  // increasing: next plane at OCC * (c + 1)
    st = 1;
    const float ri = __frcp_rn(dC);
    dt = -OCC * ri;
    t = fmaf(X - (float)(OCC * (c + 1)), ri, kf);
  } else {
    st = 0;
    dt = 3.0e38f;
    t = 3.0e38f;
  }
}

__device__ __forceinline__ CellWalk cell_walk(const DevVolume& V, const RaySetup& r, int k)
{
  CellWalk w;
  const float kf = (float)k;
  int cx, cy, cz, sx, sy, sz;
  walk_axis(r.X.h, r.dX.h, kf, w.tx, w.dtx, cx, sx);
  walk_axis(r.Y.h, r.dY.h, kf, w.ty, w.dty, cy, sy);
  walk_axis(r.Z.h, r.dZ.h, kf, w.tz, w.dtz, cz, sz);
  const int px = occ_dim(V.nx), py = occ_dim(V.ny), pz = occ_dim(V.nz);
  w.cell = ((cz + OCC_PAD) * py + (cy + OCC_PAD)) * px + (cx + OCC_PAD);
  w.ix = sx;
  w.iy = sy * px;
  w.iz = sz * px * py;
  w.last = (unsigned)(px * py * pz - 1);
  w.steps = 2 * (px + py + pz);
  return w;
}

// The walk's view of one ray for trimming a cell to its box: per axis
// ia = 1 / (8 dC) (box bounds are eighths of a voxel) and the start C
// (sample k sits at C - k dC); ia is NaN for an axis the ray runs parallel
// to and for every axis of a volume too large for the boxes (no bound).
struct RayTrim {
  float ia[3], c[3];
};

__device__ __forceinline__ RayTrim ray_trim(const DevVolume& V, const RaySetup& r)
{
  RayTrim t;
  const float C[3] = {r.X.h, r.Y.h, r.Z.h}, d[3] = {r.dX.h, r.dY.h, r.dZ.h};
  const bool big = V.nx > OCC_TRIM_MAX || V.ny > OCC_TRIM_MAX || V.nz > OCC_TRIM_MAX;
  for (int i = 0; i < 3; ++i) {
    t.ia[i] = big || d[i] == 0.f ? __int_as_float(0x7fffffff) : 0.125f * __frcp_rn(d[i]);
    t.c[i] = C[i];
  }
  return t;
}

// Walk state of one ray between calls of walk_segments: the next sample to
// place, and the open march block (index pb, occupied extent [pf, pl]; pf < 0
// when none is open).
struct WalkState {
  int k, kend;
  int pb, pf, pl;
};

// Walks samples s.k .. s.kend and hands each march block that holds occupied
// samples to emit(kb, js, je) -- block start kb (a multiple of REBASE) and the
// occupied extent [kb + js, kb + je] -- in increasing k.  emit returns false
// when it can take no more; the walk then stops, and a later call resumes
// where it stopped.  Returns true when the ray is done.  Without `occ` every
// sample counts as occupied.  The steps are bounded by the cells the ray
// crosses; past that bound the rest of the ray counts as occupied.
template <class Emit, class Trim>
__device__ __forceinline__ bool walk_segments(CellWalk& w, const uint8_t* __restrict__ occ, Trim&& trim, WalkState& s,
                                              Emit&& emit)
{
  const int4* __restrict__ boxes = occ ? (const int4*)(occ + occ_box_offset((size_t)w.last + 1)) : nullptr;
  int steps = w.steps;
  // tp: the cell's entry crossing; its first sample is floor(tp) + 1
  const float kendf = (float)s.kend;
  float tp = (float)s.k - 0.5f;
  while (tp < kendf) {
    bool full = true;
    unsigned cb = 0;  // the cell's occupancy byte; 1: trim to the box
    float tn = 3.0e38f;
    if (occ && steps > 0) {
      tn = fminf(w.tx, fminf(w.ty, w.tz));
      cb = __ldg(occ + min((unsigned)w.cell, w.last));
      full = cb != 0;
      --steps;
    }
    if (full) {
      // add the cell's samples [a, ke] that lie in its box to the open block(s)
      int ke = tn < kendf ? (int)floorf(tn) : s.kend;
      int a = (int)floorf(tp) + 1;
      if (cb == 1) {
        const int4 bx = __ldg(boxes + min((unsigned)w.cell, w.last));
        float klo = -1.0e9f, khi = 1.0e9f;
        const int pk[3] = {bx.x, bx.y, bx.z};
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const float lo = (float)((pk[i] << 16) >> 16), hi = (float)(pk[i] >> 16);
          float ia, c;
          trim(i, ia, c);  // the ray's RayTrim entries of axis i
          const float ca = 8.0f * c * ia;  // C / dC
          const float k1 = fmaf(-hi, ia, ca), k2 = fmaf(-lo, ia, ca);
          klo = fmaxf(klo, fminf(k1, k2));  // a NaN bound (parallel axis) leaves klo and khi
          khi = fminf(khi, fmaxf(k1, k2));
        }
        a = max(a, (int)ceilf(klo));
        ke = min(ke, (int)floorf(khi));
      }
      for (; a <= ke;) {
        const int bb = (int)((unsigned)a / REBASE), hi = min(ke, bb * REBASE + REBASE - 1);
        if (s.pf >= 0 && s.pb != bb) {
          if (!emit(s.pb * REBASE, s.pf - s.pb * REBASE, s.pl - s.pb * REBASE)) {
            s.k = a;  // resume here; the walk state still describes this cell
            return false;
          }
          s.pf = -1;
        }
        if (s.pf < 0) {
          s.pb = bb;
          s.pf = a;
        }
        s.pl = hi;
        a = hi + 1;
      }
    }
    tp = tn;
    if (tn == w.tx) {
      w.cell += w.ix;
      w.tx += w.dtx;
    } else if (tn == w.ty) {
      w.cell += w.iy;
      w.ty += w.dty;
    } else {
      w.cell += w.iz;
      w.tz += w.dtz;
    }
  }
  s.k = s.kend + 1;
  if (s.pf >= 0) {
    if (!emit(s.pb * REBASE, s.pf - s.pb * REBASE, s.pl - s.pb * REBASE)) return false;
    s.pf = -1;
  }
  return true;
}

// Integer base and FP32 fraction of coordinate C - k dC.  The march re-bases
// at every multiple of REBASE samples, so that the fraction stays small
// (|fraction| < 1 + REBASE |d|, exact to a few 1e-6 voxel) and a sample's
// coordinates depend on its index k alone.
__device__ __forceinline__ void coord_base(df C, df dC, float k, int& base_i, float& frac)
{
  const df c = df_add(C, df_neg(df_mulf(dC, k)));
  const float fl = floorf(c.h);
  base_i = (int)fminf(fmaxf(fl, -1.0e6f), 1.0e6f);
  frac = __fadd_rn(__fadd_rn(c.h, -fl), c.l);
}

// Whether sample k of a ray lies above the cutoff, computed exactly enough
// to agree with FP64: the position and the trilinear value in double-float,
// against the threshold (th, tl) (Cutoff).  Decides the samples in the band.
template <int STORE>
__device__ __forceinline__ bool sample_above(const DevVolume& V, const RaySetup& r, int k, const Cutoff& cut)
{
  const float kf = (float)k;
  const df C[3] = {df_add(r.X, df_neg(df_mulf(r.dX, kf))), df_add(r.Y, df_neg(df_mulf(r.dY, kf))),
                   df_add(r.Z, df_neg(df_mulf(r.dZ, kf)))};
  int b[3];
  df f[3];
  for (int i = 0; i < 3; ++i) {
    float fl = floorf(C[i].h);
    if (fl == C[i].h && C[i].l < 0.f) fl -= 1.0f;  // h + l lies just below the integer h
    fl = fminf(fmaxf(fl, -1.0f), 1.0e6f);
    b[i] = (int)fl;
    f[i] = df_two_sum(__fadd_rn(C[i].h, -fl), C[i].l);  // C - floor(C): h - floor(h) is exact
  }
  const unsigned px = (unsigned)V.px, pxy = (unsigned)V.pxy;
  const unsigned imax = ASC_QUADS ? (unsigned)(V.nz + 2 * PAD - 1) * pxy - 1u
                                  : (unsigned)(V.nz + 2 * PAD - 1) * pxy - px - 1u;
  const unsigned i = min((unsigned)(b[2] + PAD) * pxy + (unsigned)(b[1] + PAD) * px + (unsigned)(b[0] + PAD), imax);
  const Taps<STORE> t = fetch_taps<STORE>(V.pairs, i, px, pxy);
  df e[4];
  for (int q = 0; q < 4; ++q) {
    float lo, hi;
    if constexpr (STORE == ASC_STORE_F32) {
      lo = t.p[q].x;
      hi = t.p[q].y;
    } else {
      unpack<STORE>(t.w[q], lo, hi);
    }
    e[q] = df_add(df{lo, 0.f}, df_mulf(f[0], __fadd_rn(hi, -lo)));  // raw values: hi - lo is exact
  }
  const df f0 = df_add(e[0], df_mul(f[1], df_add(e[1], df_neg(e[0]))));
  const df f1 = df_add(e[2], df_mul(f[1], df_add(e[3], df_neg(e[2]))));
  const df v = df_add(f0, df_mul(f[2], df_add(f1, df_neg(f0))));
  return df_lt(df{cut.th, cut.tl}, v);
}

// Samples kb + js .. kb + je of one march block (kb a multiple of REBASE) of
// cuda_volume_render_kernel's loop (RayCaster_kernels.cu:187-195; t = far -
// k).  Returns the block's FP32 sum of raw samples above the cutoff (at most
// REBASE of them, so its relative error stays below ~4e-6 and typically near
// 1e-7; the blocks are combined in double-float); a sample at or below the
// cutoff leaves it untouched, so trimming samples that add nothing changes no
// bit.
//
// lo, hi: the cutoff's band for this ray (cutoff_bounds): samples at or
// above hi count, samples in (lo, hi) need the exact test.  EXACT false: a
// sample in the band marks the block, whose sum then comes back negated with
// its sign bit set (-0 for an empty sum; a sum of samples above a cutoff >= 0
// is never negative otherwise, see block_flagged), and the ray must be
// marched again with EXACT true, which decides those samples with
// sample_above.  cut is read only with EXACT.
template <int STORE, bool EXACT>
__device__ __forceinline__ float march_block(const DevVolume& V, const RaySetup& r, int kb, int js, int je,
                                              float lo, float hi, const Cutoff& cut)
{
  const uint32_t* __restrict__ P = V.pairs;
  const unsigned px = (unsigned)V.px, pxy = (unsigned)V.pxy;
  const float dXh = r.dX.h, dYh = r.dY.h, dZh = r.dZ.h;
  int bix, biy, biz;
  float fx, fy, fz;
  const float kbf = (float)kb;
  coord_base(r.X, r.dX, kbf, bix, fx);
  coord_base(r.Y, r.dY, kbf, biy, fy);
  coord_base(r.Z, r.dZ, kbf, biz, fz);
  // Lower tap and weight per axis at fraction X (|X| < 2^22): t = M + X
  // rounded down is M + floor(X), so floor(X) = bits(t) - bits(M) and the
  // weight X - floor(X) in [0, 1) is exact.  The word of the lower taps has
  // padded index (base + PAD + floor) per axis, i.e. bits(tz) pxy + bits(ty)
  // px + bits(tx) + i_base in unsigned (mod 2^32) arithmetic, i_base folding
  // the bases, the padding and bits(M).  Inside the box the taps stay in the
  // padded grid; the one clamp keeps degenerate input in bounds.
  const float M = 12582912.0f;  // 1.5 * 2^23
  const unsigned BM = 0x4b400000u;
  const unsigned i_base = ((unsigned)(biz + PAD) - BM) * pxy + ((unsigned)(biy + PAD) - BM) * px +
                          ((unsigned)(bix + PAD) - BM);
  const unsigned imax = ASC_QUADS ? (unsigned)(V.nz + 2 * PAD - 1) * pxy - 1u
                                  : (unsigned)(V.nz + 2 * PAD - 1) * pxy - px - 1u;
  float acc = 0.f;
  // the largest sample not counted (below hi): above lo once a sample fell
  // in the band (one max, predicated on the test that decides the add)
  float nearf = -3.0e38f;
  // the cutoff test of sample ks with value v: adds v when above
  auto take = [&](float v, int ks) {
    if constexpr (EXACT) {
      if (v >= hi) {
        acc += v;
      } else if (v > lo) {
        if (sample_above<STORE>(V, r, ks, cut)) acc += v;
      }
    } else {
      if (v >= hi)
        acc += v;
      else
        nearf = fmaxf(nearf, v);
    }
  };
  float j = (float)js;
  // the taps' voxel index and weights of sample j (j * the low part of d
  // stays below 1e-6 voxel for j < REBASE)
  auto locate = [&](float jj, float& ax, float& ay, float& az) {
    const float X = fmaf(-jj, dXh, fx), Y = fmaf(-jj, dYh, fy), Z = fmaf(-jj, dZh, fz);
    const float tx = __fadd_rd(X, M), ty = __fadd_rd(Y, M), tz = __fadd_rd(Z, M);
    ax = __fadd_rn(X, -__fadd_rn(tx, -M));
    ay = __fadd_rn(Y, -__fadd_rn(ty, -M));
    az = __fadd_rn(Z, -__fadd_rn(tz, -M));
    return min(__float_as_uint(tz) * pxy + __float_as_uint(ty) * px + __float_as_uint(tx) + i_base, imax);
  };
  // Samples two at a time (jj and jj + 1) in packed pairs, both samples'
  // loads issued together; the samples add in order.  The positions are
  // scalar FMAs (the same values as locate's): packed ones would hold six
  // more registers, which the march, at 64 per thread, spills.
  auto locate2 = [&](float jj, float2& wx, float2& wy, float2& wz, unsigned& ia, unsigned& ib) {
    const float j1 = jj + 1.0f;
    const float2 X = make_float2(fmaf(-jj, dXh, fx), fmaf(-j1, dXh, fx));
    const float2 Y = make_float2(fmaf(-jj, dYh, fy), fmaf(-j1, dYh, fy));
    const float2 Z = make_float2(fmaf(-jj, dZh, fz), fmaf(-j1, dZh, fz));
    const float2 tx = __fadd2_rd(X, bcast2(M)), ty = __fadd2_rd(Y, bcast2(M)), tz = __fadd2_rd(Z, bcast2(M));
    wx = sub2(X, __fadd2_rn(tx, bcast2(-M)));
    wy = sub2(Y, __fadd2_rn(ty, bcast2(-M)));
    wz = sub2(Z, __fadd2_rn(tz, bcast2(-M)));
    ia = min(__float_as_uint(tz.x) * pxy + __float_as_uint(ty.x) * px + __float_as_uint(tx.x) + i_base, imax);
    ib = min(__float_as_uint(tz.y) * pxy + __float_as_uint(ty.y) * px + __float_as_uint(tx.y) + i_base, imax);
  };
  int k = js;
  for (; k < je; k += 2) {
    float2 wx, wy, wz;
    unsigned ia, ib;
    locate2(j, wx, wy, wz, ia, ib);
    const Taps<STORE> A = fetch_taps<STORE>(P, ia, px, pxy), B = fetch_taps<STORE>(P, ib, px, pxy);
    const float2 v = trilinear2<STORE>(A, B, wx, wy, wz);
    take(v.x, kb + k);
    take(v.y, kb + k + 1);
    j += 2.0f;
  }
  if (k == je) {
    float ax, ay, az;
    const Taps<STORE> t = fetch_taps<STORE>(P, locate(j, ax, ay, az), px, pxy);
    const float e00 = lerp_tap<STORE>(t, 0, ax);
    const float e10 = lerp_tap<STORE>(t, 1, ax);
    const float e01 = lerp_tap<STORE>(t, 2, ax);
    const float e11 = lerp_tap<STORE>(t, 3, ax);
    const float f0 = fmaf(ay, e10 - e00, e00);
    const float f1 = fmaf(ay, e11 - e01, e01);
    const float v = fmaf(az, f1 - f0, f0);
    take(v, kb + k);
  }
  if constexpr (EXACT) return acc;
  return nearf > lo ? -acc - 0.0f : acc;
}

// Whether a march block's sum carries the band's mark (march_block).
__device__ __forceinline__ bool block_flagged(float p) { return (__float_as_uint(p) >> 31) != 0u; }

// Adds a block's sum to the ray's double-float total; blocks that added
// nothing leave it untouched.
__device__ __forceinline__ void add_block(df& total, float p)
{
  if (p != 0.f) total = df_add(total, df{p, 0.f});
}

// One march pass over a whole ray: the march blocks that hold occupied
// samples, in order, each trimmed to its occupied extent, their sums combined
// in double-float.  EXACT false: *flagged is set when a sample fell in the
// cutoff's band (the pass's total then leaves the band's samples out).
template <int STORE, bool EXACT>
__device__ __forceinline__ float march_pass(const DevVolume& V, const uint8_t* __restrict__ occ, const RaySetup& r,
                                            const Cutoff& cut, bool* flagged)
{
  CellWalk w = cell_walk(V, r, 0);
  WalkState s{0, r.K - 1, 0, -1, 0};
  const RayTrim t = ray_trim(V, r);
  df total{0.f, 0.f};
  bool fl = false;
  float lo, hi;
  cutoff_bounds(cut, r.dX.h, r.dY.h, r.dZ.h, lo, hi);
  walk_segments(w, occ, [&](int i, float& ia, float& c) {
    ia = t.ia[i];
    c = t.c[i];
  }, s, [&](int kb, int js, int je) {
    const float p = march_block<STORE, EXACT>(V, r, kb, js, je, lo, hi, cut);
    if (!EXACT && block_flagged(p))
      fl = true;
    else
      add_block(total, p);
    return true;
  });
  if (flagged) *flagged = fl;
  return total.h + total.l;
}

// One whole ray, with every cutoff decision the exact one: the FP32 pass,
// and the exact pass when a sample fell in the band.  The result depends
// only on the samples above the cutoff, so it is the same with and without
// `occ`, and the same as the batched engine's.
template <int STORE>
__device__ __forceinline__ float march(const DevVolume& V, const uint8_t* __restrict__ occ, const RaySetup& r,
                                       const Cutoff& cut)
{
  if (r.K <= 0) return 0.f;
  bool flagged = false;
  const float d = march_pass<STORE, false>(V, occ, r, cut, &flagged);
  return flagged ? march_pass<STORE, true>(V, occ, r, cut, nullptr) : d;
}

}  // namespace asc
