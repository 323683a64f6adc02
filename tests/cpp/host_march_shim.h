// Host stand-ins for the handful of CUDA intrinsics that the ray march
// (autoscoper_gb300/csrc/asc_march.cuh) uses, so that the same source
// compiles as host C++ for CPU tests.  Build with -ffp-contract=off.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#define __device__
#define __host__
#define __forceinline__ inline
#define __noinline__
using std::max;
using std::min;
inline float __fadd_rn(float a, float b) { volatile float r = a + b; return r; }
inline float __fmul_rn(float a, float b) { volatile float r = a * b; return r; }
// a + b rounded towards -inf (the sum of two floats is exact in double here)
inline float __fadd_rd(float a, float b)
{
  const double s = (double)a + (double)b;
  float f = (float)s;
  if ((double)f > s) f = std::nextafter(f, -INFINITY);
  return f;
}
inline float __fdiv_rn(float a, float b) { volatile float r = a / b; return r; }
inline float __fsqrt_rn(float a) { return std::sqrt(a); }
inline float __frcp_rn(float a) { volatile float r = 1.0f / a; return r; }
inline float rsqrtf(float a) { volatile float r = 1.0f / std::sqrt(a); return r; }
inline int __float_as_int(float f) { int i; std::memcpy(&i, &f, 4); return i; }
inline unsigned __float_as_uint(float f) { unsigned i; std::memcpy(&i, &f, 4); return i; }
// bytes of (y:x) picked by the selector's nibbles, lowest result byte first
inline unsigned __byte_perm(unsigned x, unsigned y, unsigned s)
{
  const unsigned long long v = ((unsigned long long)y << 32) | x;
  unsigned r = 0;
  for (int i = 0; i < 4; ++i) r |= (unsigned)((v >> (8 * ((s >> (4 * i)) & 7u))) & 0xffu) << (8 * i);
  return r;
}
inline float __uint_as_float(unsigned u) { float f; std::memcpy(&f, &u, 4); return f; }
inline float __int_as_float(int u) { float f; std::memcpy(&f, &u, 4); return f; }
inline int __float2int_rd(float f) { return (int)std::floor(f); }
template <class T> inline T __ldg(const T* p) { return *p; }
struct float2 { float x, y; };
// the packed FP32 pairs of sm_100: one IEEE operation per half
inline float2 __ffma2_rn(float2 a, float2 b, float2 c) { return {std::fma(a.x, b.x, c.x), std::fma(a.y, b.y, c.y)}; }
inline float2 __fadd2_rn(float2 a, float2 b) { return {__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y)}; }
inline float2 __fadd2_rd(float2 a, float2 b) { return {__fadd_rd(a.x, b.x), __fadd_rd(a.y, b.y)}; }
struct uint2 { unsigned x, y; };
struct float4 { float x, y, z, w; };
struct int4 { int x, y, z, w; };
inline float2 make_float2(float x, float y) { return {x, y}; }
struct __half2_raw { unsigned short x, y; };
struct __half2 { unsigned short x, y; };
// IEEE binary16 -> binary32
inline float host_half_to_float(unsigned short h)
{
  unsigned s = (h >> 15) & 1u, e = (h >> 10) & 31u, m = h & 1023u;
  float v;
  if (e == 0) v = (float)m * (1.0f / 16777216.0f);
  else if (e == 31) v = m ? NAN : INFINITY;
  else v = __uint_as_float(((e + 112u) << 23) | (m << 13));
  return s ? -v : v;
}
inline float2 __half22float2(__half2 h) { return {host_half_to_float(h.x), host_half_to_float(h.y)}; }
