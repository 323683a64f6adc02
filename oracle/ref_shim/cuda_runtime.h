// Host-only stand-in for the CUDA runtime, used to compile the reference's
// own kernel and operator sources (libautoscoper/src/gpu/cuda/*) as plain C++
// so they run on the CPU as a parity pin for the oracle.  Test
// infrastructure: never part of the product.
//
// "Device" memory is host memory; cudaArray is a host buffer; texture
// objects are emulated in software (normalized coordinates, linear or point
// filtering, clamp-to-edge).  Kernels launch through asc_launcher(), which
// runs every thread of every block in turn; kernels that synchronise their
// block (__syncthreads) run through asc_launcher_coop(), one std::thread per
// CUDA thread and a std::barrier per block.
#pragma once
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stddef.h>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <condition_variable>
#include <mutex>
#include <thread>
#include <vector>

using std::abs;

#define __global__
#define __device__
#define __host__
#define __constant__
#define __shared__
#define __forceinline__ inline
#ifndef __inline__
#define __inline__ inline
#endif
// cutil_math.h takes the device-side branch (math builtins below) when this is set.
#ifndef __CUDACC__
#define __CUDACC__ 1
#endif

typedef unsigned int uint;
struct float2 { float x, y; };
struct float3 { float x, y, z; };
struct float4 { float x, y, z, w; };
struct int2 { int x, y; };
struct int3 { int x, y, z; };
struct int4 { int x, y, z, w; };
struct uint2 { unsigned x, y; };
struct uint3 { unsigned x, y, z; };
struct uint4 { unsigned x, y, z, w; };
struct dim3 {
  unsigned x, y, z;
  dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};
inline float2 make_float2(float x, float y) { return {x, y}; }
inline float3 make_float3(float x, float y, float z) { return {x, y, z}; }
inline float4 make_float4(float x, float y, float z, float w) { return {x, y, z, w}; }
inline int2 make_int2(int x, int y) { return {x, y}; }
inline int3 make_int3(int x, int y, int z) { return {x, y, z}; }
inline int4 make_int4(int x, int y, int z, int w) { return {x, y, z, w}; }
inline uint2 make_uint2(unsigned x, unsigned y) { return {x, y}; }
inline uint3 make_uint3(unsigned x, unsigned y, unsigned z) { return {x, y, z}; }
inline uint4 make_uint4(unsigned x, unsigned y, unsigned z, unsigned w) { return {x, y, z, w}; }

inline int max(int a, int b) { return a > b ? a : b; }
inline int min(int a, int b) { return a < b ? a : b; }
inline unsigned max(unsigned a, unsigned b) { return a > b ? a : b; }
inline unsigned min(unsigned a, unsigned b) { return a < b ? a : b; }
inline float max(float a, float b) { return fmaxf(a, b); }
inline float min(float a, float b) { return fminf(a, b); }
inline double max(double a, double b) { return fmax(a, b); }
inline double min(double a, double b) { return fmin(a, b); }
inline float rsqrtf(float x) { return 1.0f / sqrtf(x); }

extern thread_local uint3 threadIdx;
extern thread_local uint3 blockIdx;
extern thread_local dim3 blockDim;
extern thread_local dim3 gridDim;
void __syncthreads();

// ---- errors, memory ----
typedef int cudaError_t;
enum { cudaSuccess = 0 };
enum cudaMemcpyKind { cudaMemcpyHostToHost = 0, cudaMemcpyHostToDevice = 1, cudaMemcpyDeviceToHost = 2,
                      cudaMemcpyDeviceToDevice = 3, cudaMemcpyDefault = 4 };
inline cudaError_t cudaMalloc(void** p, size_t n) { *p = calloc(n ? n : 1, 1); return cudaSuccess; }
template <class T> inline cudaError_t cudaMalloc(T** p, size_t n) { return cudaMalloc((void**)p, n); }
inline cudaError_t cudaFree(void* p) { free(p); return cudaSuccess; }
inline cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind) { memmove(d, s, n); return cudaSuccess; }
inline cudaError_t cudaMemset(void* d, int v, size_t n) { memset(d, v, n); return cudaSuccess; }
template <class T>
inline cudaError_t cudaMemcpyToSymbol(T& sym, const void* src, size_t n, size_t off = 0,
                                      cudaMemcpyKind = cudaMemcpyHostToDevice)
{
  memcpy((char*)&sym + off, src, n);
  return cudaSuccess;
}
inline cudaError_t cudaGetLastError() { return cudaSuccess; }
inline cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
inline const char* cudaGetErrorString(cudaError_t) { return "no error"; }

// ---- arrays and textures ----
enum cudaChannelFormatKind { cudaChannelFormatKindSigned = 0, cudaChannelFormatKindUnsigned = 1,
                             cudaChannelFormatKindFloat = 2 };
struct cudaChannelFormatDesc { int x, y, z, w; cudaChannelFormatKind f; };
template <class T> cudaChannelFormatDesc cudaCreateChannelDesc();
template <> inline cudaChannelFormatDesc cudaCreateChannelDesc<unsigned char>() { return {8, 0, 0, 0, cudaChannelFormatKindUnsigned}; }
template <> inline cudaChannelFormatDesc cudaCreateChannelDesc<unsigned short>() { return {16, 0, 0, 0, cudaChannelFormatKindUnsigned}; }
template <> inline cudaChannelFormatDesc cudaCreateChannelDesc<unsigned int>() { return {32, 0, 0, 0, cudaChannelFormatKindUnsigned}; }
template <> inline cudaChannelFormatDesc cudaCreateChannelDesc<float>() { return {32, 0, 0, 0, cudaChannelFormatKindFloat}; }

struct cudaArray {
  cudaChannelFormatDesc desc;
  size_t w, h, d;
  std::vector<unsigned char> data;
};
typedef cudaArray* cudaArray_t;
struct cudaExtent { size_t width, height, depth; };
inline cudaExtent make_cudaExtent(size_t w, size_t h, size_t d) { return {w, h, d}; }
struct cudaPitchedPtr { void* ptr; size_t pitch, xsize, ysize; };
inline cudaPitchedPtr make_cudaPitchedPtr(void* p, size_t pitch, size_t xs, size_t ys) { return {p, pitch, xs, ys}; }
struct cudaPos { size_t x, y, z; };
struct cudaMemcpy3DParms {
  cudaArray_t srcArray; cudaPos srcPos; cudaPitchedPtr srcPtr;
  cudaArray_t dstArray; cudaPos dstPos; cudaPitchedPtr dstPtr;
  cudaExtent extent; cudaMemcpyKind kind;
};
inline cudaError_t cudaMalloc3DArray(cudaArray_t* a, const cudaChannelFormatDesc* desc, cudaExtent e, unsigned = 0)
{
  *a = new cudaArray{*desc, e.width, e.height ? e.height : 1, e.depth ? e.depth : 1, {}};
  (*a)->data.resize((*a)->w * (*a)->h * (*a)->d * (desc->x / 8));
  return cudaSuccess;
}
inline cudaError_t cudaMallocArray(cudaArray_t* a, const cudaChannelFormatDesc* desc, size_t w, size_t h = 0, unsigned = 0)
{
  return cudaMalloc3DArray(a, desc, make_cudaExtent(w, h, 1));
}
inline cudaError_t cudaFreeArray(cudaArray_t a) { delete a; return cudaSuccess; }
inline cudaError_t cudaMemcpyToArray(cudaArray_t a, size_t, size_t, const void* src, size_t n, cudaMemcpyKind)
{
  memcpy(a->data.data(), src, n);
  return cudaSuccess;
}
inline cudaError_t cudaMemcpy3D(const cudaMemcpy3DParms* p)
{
  size_t es = p->dstArray->desc.x / 8, row = p->extent.width * es;
  for (size_t z = 0; z < p->extent.depth; ++z)
    for (size_t y = 0; y < p->extent.height; ++y)
      memcpy(p->dstArray->data.data() + (z * p->dstArray->h + y) * p->dstArray->w * es,
             (const char*)p->srcPtr.ptr + (z * p->srcPtr.ysize + y) * p->srcPtr.pitch, row);
  return cudaSuccess;
}

enum cudaResourceType { cudaResourceTypeArray = 0 };
struct cudaResourceDesc {
  cudaResourceType resType;
  union { struct { cudaArray_t array; } array; } res;
};
enum cudaTextureAddressMode { cudaAddressModeWrap = 0, cudaAddressModeClamp = 1, cudaAddressModeMirror = 2,
                              cudaAddressModeBorder = 3 };
enum cudaTextureFilterMode { cudaFilterModePoint = 0, cudaFilterModeLinear = 1 };
enum cudaTextureReadMode { cudaReadModeElementType = 0, cudaReadModeNormalizedFloat = 1 };
struct cudaTextureDesc {
  cudaTextureAddressMode addressMode[3];
  cudaTextureFilterMode filterMode;
  cudaTextureReadMode readMode;
  int sRGB;
  float borderColor[4];
  int normalizedCoords;
  unsigned maxAnisotropy;
  int mipmapFilterMode;
  float mipmapLevelBias, minMipmapLevelClamp, maxMipmapLevelClamp;
  int disableTrilinearOptimization;
};
typedef unsigned long long cudaTextureObject_t;
struct cudaResourceViewDesc;
cudaError_t cudaCreateTextureObject(cudaTextureObject_t*, const cudaResourceDesc*, const cudaTextureDesc*,
                                    const cudaResourceViewDesc*);
cudaError_t cudaDestroyTextureObject(cudaTextureObject_t);
float asc_tex_fetch(cudaTextureObject_t, float x, float y, float z, int dims);
template <class T> inline T tex2D(cudaTextureObject_t t, float x, float y) { return asc_tex_fetch(t, x, y, 0.f, 2); }
template <class T> inline T tex3D(cudaTextureObject_t t, float x, float y, float z) { return asc_tex_fetch(t, x, y, z, 3); }

// ---- kernel launches (the build rewrites k<<<cfg>>>(args) into these) ----
struct asc_cfg {
  dim3 g, b;
  asc_cfg(dim3 g_, dim3 b_, size_t = 0) : g(g_), b(b_) {}
};
template <class F> struct asc_serial_launch {
  asc_cfg c; F f;
  template <class... A> void operator()(A... a) const
  {
    gridDim = c.g; blockDim = c.b;
    for (unsigned bz = 0; bz < c.g.z; ++bz) for (unsigned by = 0; by < c.g.y; ++by) for (unsigned bx = 0; bx < c.g.x; ++bx)
      for (unsigned tz = 0; tz < c.b.z; ++tz) for (unsigned ty = 0; ty < c.b.y; ++ty) for (unsigned tx = 0; tx < c.b.x; ++tx) {
        blockIdx = {bx, by, bz}; threadIdx = {tx, ty, tz};
        f(a...);
      }
  }
};
template <class F> asc_serial_launch<F> asc_launcher(asc_cfg c, F f) { return {c, f}; }

// Reusable barrier for the threads of one emulated block (C++17 has no std::barrier).
struct asc_barrier {
  std::mutex m; std::condition_variable cv; unsigned n, count, gen = 0;
  explicit asc_barrier(unsigned k) : n(k), count(k) {}
  void arrive_and_wait()
  {
    std::unique_lock<std::mutex> l(m);
    unsigned g = gen;
    if (--count == 0) { gen++; count = n; cv.notify_all(); return; }
    cv.wait(l, [&] { return g != gen; });
  }
  void arrive_and_drop()
  {
    std::unique_lock<std::mutex> l(m);
    --n;
    if (--count == 0) { gen++; count = n; cv.notify_all(); }
  }
};
void asc_set_block_barrier(asc_barrier* b);
template <class F> struct asc_coop_launch {
  asc_cfg c; F f;
  // One std::thread per CUDA thread of a block, reused across blocks; the
  // blocks run one after another, separated by a barrier.
  template <class... A> void operator()(A... a) const
  {
    unsigned nt = c.b.x * c.b.y * c.b.z;
    asc_barrier bar(nt);
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; ++t)
      th.emplace_back([&, t] {
        gridDim = c.g; blockDim = c.b;
        threadIdx = {t % c.b.x, (t / c.b.x) % c.b.y, t / (c.b.x * c.b.y)};
        asc_set_block_barrier(&bar);
        for (unsigned bz = 0; bz < c.g.z; ++bz) for (unsigned by = 0; by < c.g.y; ++by)
          for (unsigned bx = 0; bx < c.g.x; ++bx) {
            blockIdx = {bx, by, bz};
            f(a...);
            bar.arrive_and_wait();
          }
      });
    for (auto& x : th) x.join();
  }
};
template <class F> asc_coop_launch<F> asc_launcher_coop(asc_cfg c, F f) { return {c, f}; }
