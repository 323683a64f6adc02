// NCC without any device allocation.
//
// Some callers cannot allocate device memory when they need a score: a host
// application that owns a fixed device-memory budget (its own pool, or a
// serving loop that admits work by the bytes it reserved) and must not see a
// plugin grow it, and latency-critical loops where cudaMalloc's implicit
// device-wide synchronisation is not acceptable.  asc_ncc_noalloc serves
// them: it runs the same one-launch NCC kernel as asc_ncc, with the kernel's
// per-block partials and its completion counter in a fixed array compiled
// into this library instead of memory from asc_ncc_init.
//
// The array below is a file-scope device variable: every GPU that loads the
// library holds it (ASC_NOALLOC_BYTES) until the process exits, and all calls
// on a device share it.
#include <mutex>

#include "asc_internal.cuh"

namespace asc {

struct ReduceScratch {
  Moments* part;
  double* means;
  unsigned* ticket;
};
__global__ void __launch_bounds__(256) k_ncc(const float* __restrict__ f, const float* __restrict__ g,
                                             const float* __restrict__ mask, unsigned n, int tree, ReduceScratch sc,
                                             double* __restrict__ result);

}  // namespace asc

using namespace asc;

namespace {

constexpr unsigned kChunk = 256 * 16;                      // elements per block of k_ncc
constexpr unsigned kMaxBlocks = ASC_NOALLOC_MAX_N / kChunk;  // 4096 blocks
constexpr size_t kPartBytes = kMaxBlocks * sizeof(Moments);

// [partials: kMaxBlocks Moments][means: 2 doubles][ticket: 1 unsigned]
static __device__ __align__(256) unsigned char g_noalloc[kPartBytes + 2 * sizeof(double) + 256];

struct Slot {
  void* base = nullptr;
  unsigned long long ctx = 0;  // unique id of the context the address belongs to
  bool ready = false;
};
std::mutex g_mu;
Slot g_slots[64];  // one per device ordinal

// cuCtxGetId of the driver, reached through the runtime (no link against
// libcuda): the id of the current context, unique for the life of the
// process, so a context created anew on a device (after a cudaDeviceReset by
// the host) never matches an address looked up in the one before it.
typedef int (*CtxGetIdFn)(void* ctx, unsigned long long* id);
CtxGetIdFn ctx_get_id()
{
  static CtxGetIdFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return (CtxGetIdFn)p;
  }();
  return fn;
}

bool current_ctx_id(unsigned long long* id)
{
  CtxGetIdFn fn = ctx_get_id();
  return fn && fn(nullptr, id) == 0;
}

// Device address of g_noalloc in the current device's current context.  The
// first call in a context looks it up (cudaGetSymbolAddress with that device
// current); later calls in the same context reuse it.  Where the driver
// cannot name the context, every call looks the address up.
int noalloc_base(void** out)
{
  int dev = 0;
  ASC_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return ASC_ERR_RANGE;
  unsigned long long ctx = 0;
  bool known = current_ctx_id(&ctx);
  std::lock_guard<std::mutex> lock(g_mu);
  Slot& s = g_slots[dev];
  if (!s.ready || !known || s.ctx != ctx) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc);
    if (e != cudaSuccess) {
      s.ready = false;
      return cuda_status(e);
    }
    if (!known) known = current_ctx_id(&ctx);  // the lookup made the runtime's context current
    s.base = p;
    s.ctx = ctx;
    s.ready = known;
  }
  *out = s.base;
  return ASC_OK;
}

}  // namespace

ASC_API int asc_ncc_noalloc(const float* f, const float* g, const float* m, unsigned n, int coverage, double* res,
                            void* stream)
{
  if (!f || !g || !m || !res || n == 0 || (coverage != ASC_SUM_TREE && coverage != ASC_SUM_FULL)) return ASC_ERR_ARG;
  if (n > ASC_NOALLOC_MAX_N) {
    set_error_message("asc_ncc_noalloc: n exceeds the fixed maximum of ASC_NOALLOC_MAX_N elements");
    return ASC_ERR_RANGE;
  }
  void* base = nullptr;
  int rc = noalloc_base(&base);
  if (rc) return rc;
  unsigned char* b = (unsigned char*)base;
  ReduceScratch sc{(Moments*)b, (double*)(b + kPartBytes), (unsigned*)(b + kPartBytes + 2 * sizeof(double))};
  // the completion counter must start at zero; the partials are written before they are read
  ASC_CUDA(cudaMemsetAsync(sc.ticket, 0, sizeof(unsigned), S(stream)));
  const unsigned blocks = (n + kChunk - 1) / kChunk;
  const int tree = coverage == ASC_SUM_TREE && tree_needed(n);
  k_ncc<<<blocks, 256, 0, S(stream)>>>(f, g, m, n, tree, sc, res);
  ASC_LAUNCH_CHECK();
  return ASC_OK;
}
