// Ray march of the DRR ray caster: device volume layout, double-float ray
// set-up and the FP32 march.  Self-contained so that it also compiles as
// host C++ (tests/cpp/host_march.cpp provides the few intrinsics).
#pragma once

namespace asc {

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
  return {s, __fadd_rn(b, -__fadd_rn(s, -a))};
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

// Integer base and FP32 fraction of coordinate C - k dC.  The march re-bases
// at every multiple of REBASE samples, so that the fraction stays small
// (|fraction| < 1 + REBASE |d|, exact to a few 1e-6 voxel) and a sample's
// coordinates depend on its index k alone, whatever was skipped before it.
#ifndef ASC_REBASE
#define ASC_REBASE 64
#endif
constexpr int REBASE = ASC_REBASE;
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
  const float dXh = r.dX.h, dYh = r.dY.h, dZh = r.dZ.h;
  // per-sample change of the coordinates, and its reciprocal for the
  // cell-exit distances (only the sign and a 1e-3 voxel margin matter there)
  const float iX = dXh != 0.f ? 1.0f / dXh : 0.f, iY = dYh != 0.f ? 1.0f / dYh : 0.f;
  const float iZ = dZh != 0.f ? 1.0f / dZh : 0.f;
  float acc = 0.f, comp = 0.f;
  int bix = 0, biy = 0, biz = 0;
  float bfx = 0.f, bfy = 0.f, bfz = 0.f, fx = 0.f, fy = 0.f, fz = 0.f;
  int kb = -REBASE;  // index of the current base, a multiple of REBASE
  float j = 0.f;     // k - kb
  int kj = 0;        // the k that j belongs to
  int inside = 0;    // samples from k on known to lie in an occupied cell
  for (int k = 0; k < r.K;) {
    if (k - kb >= REBASE) {
      kb = k & ~(REBASE - 1);
      const float kf = (float)kb;
      coord_base(r.X, r.dX, kf, bix, bfx, fx);
      coord_base(r.Y, r.dY, kf, biy, bfy, fy);
      coord_base(r.Z, r.dZ, kf, biz, bfz, fz);
      kj = k - 1;  // force j below
    }
    if (kj != k) {  // after a base change or a skip
      j = (float)(k - kb);
      kj = k;
    }
    // j * (low part of d) stays below 1e-6 voxel for j < REBASE
    const float FX = fmaf(-j, dXh, fx), FY = fmaf(-j, dYh, fy), FZ = fmaf(-j, dZh, fz);
    if (occ && inside <= 0) {
      // the lower tap is floor(X) (or floor(X) - 1 at an integer X, see tap)
      // and its cell floor(X / OCC); X here is approximate (~1e-5 voxel)
      const float X = bfx + FX, Y = bfy + FY, Z = bfz + FZ;
      const int cx = min(max(__float2int_rd(X * (1.0f / OCC)), 0), bx - 1);
      const int cy = min(max(__float2int_rd(Y * (1.0f / OCC)), 0), by - 1);
      const int cz = min(max(__float2int_rd(Z * (1.0f / OCC)), 0), bz - 1);
      // whole samples after this one during which the lower tap stays at
      // least 1e-3 voxel inside the cell (well above the error of X); a
      // coordinate moves by -d per sample
      const float G = 1.0e-3f;
      float s = 3.0e38f;
      if (dXh > 0.f) s = fminf(s, (X - (float)(OCC * cx) - G) * iX);
      if (dXh < 0.f) s = fminf(s, (X - (float)(OCC * cx + OCC) + G) * iX);
      if (dYh > 0.f) s = fminf(s, (Y - (float)(OCC * cy) - G) * iY);
      if (dYh < 0.f) s = fminf(s, (Y - (float)(OCC * cy + OCC) + G) * iY);
      if (dZh > 0.f) s = fminf(s, (Z - (float)(OCC * cz) - G) * iZ);
      if (dZh < 0.f) s = fminf(s, (Z - (float)(OCC * cz + OCC) + G) * iZ);
      const int m = (int)fminf(fmaxf(floorf(s), 0.f), 1.0e6f) + 1;  // this sample and the next m - 1
      if (!__ldg(occ + (cz * by + cy) * bx + cx)) {
        k += m;  // all of them add nothing
        continue;
      }
      inside = m;
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
    ++kj;
    --inside;
    j += 1.0f;
  }
  return acc;
}

}  // namespace asc
