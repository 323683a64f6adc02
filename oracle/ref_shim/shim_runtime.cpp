// Host implementation of the CUDA stand-in (see cuda_runtime.h): thread
// indices, block barriers and software texture fetches.  Test infrastructure.
#include "cuda_runtime.h"

thread_local uint3 threadIdx;
thread_local uint3 blockIdx;
thread_local dim3 blockDim;
thread_local dim3 gridDim;
static thread_local asc_barrier* g_bar = nullptr;
void asc_set_block_barrier(asc_barrier* b) { g_bar = b; }
void __syncthreads() { g_bar->arrive_and_wait(); }

// Dynamic shared memory of the reduction kernels (blocks run one at a time).
float sdata[1 << 16];

// Weight precision of the emulated texture unit: 0 = exact FP32 weights,
// 8 = weights rounded to 8 fractional bits (the fixed-point format that the
// CUDA programming guide documents for hardware linear filtering).
int asc_tex_weight_bits = 0;

struct TexObj { cudaArray* a; cudaTextureDesc d; };

cudaError_t cudaCreateTextureObject(cudaTextureObject_t* t, const cudaResourceDesc* r, const cudaTextureDesc* d,
                                    const cudaResourceViewDesc*)
{
  *t = (cudaTextureObject_t) new TexObj{r->res.array.array, *d};
  return cudaSuccess;
}
cudaError_t cudaDestroyTextureObject(cudaTextureObject_t t)
{
  delete (TexObj*)t;
  return cudaSuccess;
}

static float texel(const TexObj* o, long i)
{
  const cudaArray* a = o->a;
  bool norm = o->d.readMode == cudaReadModeNormalizedFloat;
  if (a->desc.f == cudaChannelFormatKindFloat) return ((const float*)a->data.data())[i];
  if (a->desc.x == 8) { unsigned v = a->data[i]; return norm ? v / 255.0f : (float)v; }
  if (a->desc.x == 16) { unsigned v = ((const unsigned short*)a->data.data())[i]; return norm ? v / 65535.0f : (float)v; }
  unsigned v = ((const unsigned*)a->data.data())[i];
  return (float)v;
}

static float qweight(float a)
{
  if (!asc_tex_weight_bits) return a;
  float s = (float)(1 << asc_tex_weight_bits);
  return rintf(a * s) / s;
}

static void setup(float u, long n, bool normalized, long* i0, long* i1, float* a, bool linear)
{
  float x = normalized ? u * (float)n : u;
  if (!linear) {
    long i = (long)floorf(x);
    if (i < 0) i = 0;
    if (i > n - 1) i = n - 1;
    *i0 = *i1 = i;
    *a = 0.f;
    return;
  }
  x -= 0.5f;
  float fl = floorf(x);
  *a = qweight(x - fl);
  if (fl < -1.f) fl = -1.f;
  if (fl > (float)n) fl = (float)n;
  long i = (long)fl;
  *i0 = i < 0 ? 0 : (i > n - 1 ? n - 1 : i);
  *i1 = i + 1 < 0 ? 0 : (i + 1 > n - 1 ? n - 1 : i + 1);
}

float asc_tex_fetch(cudaTextureObject_t t, float x, float y, float z, int dims)
{
  const TexObj* o = (const TexObj*)t;
  const cudaArray* a = o->a;
  bool lin = o->d.filterMode == cudaFilterModeLinear, nc = o->d.normalizedCoords != 0;
  long x0, x1, y0, y1, z0 = 0, z1 = 0;
  float ax, ay, az = 0.f;
  setup(x, (long)a->w, nc, &x0, &x1, &ax, lin);
  setup(y, (long)a->h, nc, &y0, &y1, &ay, lin);
  if (dims == 3) setup(z, (long)a->d, nc, &z0, &z1, &az, lin);
  long sx = (long)a->w, sxy = (long)(a->w * a->h);
#define T(i, j, k) texel(o, (k) * sxy + (j) * sx + (i))
  float c00 = (1 - ax) * T(x0, y0, z0) + ax * T(x1, y0, z0);
  float c10 = (1 - ax) * T(x0, y1, z0) + ax * T(x1, y1, z0);
  float c0 = (1 - ay) * c00 + ay * c10;
  if (dims == 2) return c0;
  float c01 = (1 - ax) * T(x0, y0, z1) + ax * T(x1, y0, z1);
  float c11 = (1 - ax) * T(x0, y1, z1) + ax * T(x1, y1, z1);
#undef T
  float c1 = (1 - ay) * c01 + ay * c11;
  return (1 - az) * c0 + az * c1;
}
