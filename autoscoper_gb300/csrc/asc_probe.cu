// Read-bandwidth probe: the denominators of the roofline fractions the
// benchmark reports.  The ray cast gathers its taps from L1/L2 (every volume
// of the path is far smaller than the 129 MB L2), so its memory roofline is
// the L2 read bandwidth, which the measured HBM copy figure does not
// give.  This kernel streams a device buffer with 16-byte loads that bypass
// L1 (ld.global.cg), `passes` times over, one grid of resident blocks per SM
// slot; with the buffer well inside L2 after a first pass it measures L2 read
// bandwidth, with a buffer far larger than L2 it measures HBM.  No
// counterpart in the reference.
#include <algorithm>

#include "asc_internal.cuh"

using namespace asc;

namespace {

__global__ void __launch_bounds__(512) k_probe_read(const uint4* __restrict__ buf, size_t n16, int passes,
                                                    unsigned* __restrict__ sink)
{
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  unsigned acc = 0;
  for (int p = 0; p < passes; ++p) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += stride) {
      uint4 v;
      asm volatile("ld.global.cg.v4.u32 {%0, %1, %2, %3}, [%4];"
                   : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                   : "l"(buf + i));
      acc ^= v.x ^ v.y ^ v.z ^ v.w;
    }
  }
  if (acc == 0x9e3779b9u) sink[0] = acc;  // keeps the loads; the buffer is zero, so never taken
}

}  // namespace

ASC_API int asc_probe_read_bandwidth(size_t bytes, int passes, double* gbs, float* ms_out)
{
  if (!gbs || bytes < 16 || passes < 1) return ASC_ERR_ARG;
  const size_t n16 = bytes / 16;
  int dev = 0, sms = 0, per_sm = 0;
  ASC_CUDA(cudaGetDevice(&dev));
  ASC_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  ASC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_probe_read, 512, 0));
  const int grid = sms * std::max(per_sm, 1);
  uint4* buf = nullptr;
  unsigned* sink = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaStream_t s = nullptr;
  int rc = ASC_OK;
  float ms = 0.f;
  {
    Gate g(device_gate());
    cudaError_t e = cudaMalloc(&buf, n16 * 16);
    if (e == cudaSuccess) e = cudaMalloc(&sink, sizeof(unsigned));
    if (e != cudaSuccess) {
      cudaFree(buf);
      return cuda_status(e);
    }
  }
  cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMemsetAsync(buf, 0, n16 * 16, s);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e == cudaSuccess) {
    k_probe_read<<<grid, 512, 0, s>>>(buf, n16, 1, sink);  // warm-up: fills L2 when the buffer fits
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaEventRecord(e0, s);
  if (e == cudaSuccess) {
    k_probe_read<<<grid, 512, 0, s>>>(buf, n16, passes, sink);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaEventRecord(e1, s);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  if (e != cudaSuccess) rc = cuda_status(e);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (s) cudaStreamDestroy(s);
  {
    Gate g(device_gate());
    cudaFree(buf);
    cudaFree(sink);
  }
  if (rc) return rc;
  *gbs = (double)n16 * 16.0 * passes / (ms * 1e-3) / 1e9;
  if (ms_out) *ms_out = ms;
  return ASC_OK;
}
