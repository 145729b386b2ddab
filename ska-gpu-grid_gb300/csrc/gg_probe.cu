// Measurement helper for the roofline of the gridding kernels (built as
// libgg_probe.so, used by the benchmark; not part of the gridder's ABI).
//
// gg_probe_red_rate measures the rate of FP32 global reductions
// (red.global.add.f32, scalar or .v2) that the L2 sustains: the ceiling of a
// scatter gridder, which issues one reduction per grid tap.  Patterns:
//   0  coalesced: consecutive lanes on consecutive cells
//   1  scattered: every reduction on a hashed cell
// over an array of `cells` cells (a power of two): L2-resident or
// HBM-sized, or a few cells for the contended case.  Each thread issues a
// fixed number of reductions; nothing waits on anything.
#include <cuda_runtime.h>
#include <stdint.h>

namespace {

template <bool V2, int PATTERN>
__global__ void __launch_bounds__(256) red_probe_kernel(float *a, uint64_t mask, int iters) {
  const uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  const uint64_t nt = (uint64_t)gridDim.x * blockDim.x;
  for (int i = 0; i < iters; ++i) {
    uint64_t c;
    if (PATTERN == 0) {
      c = (t + (uint64_t)i * nt) & mask;
    } else {
      c = ((t * (uint64_t)iters + (uint64_t)i) * 0x9E3779B97F4A7C15ull) >> 17;
      c &= mask;
    }
    if (V2) {
      float *p = a + 2 * c;
      asm volatile("red.global.add.v2.f32 [%0], {%1, %2};" ::"l"(p), "f"(1.0f), "f"(1.0f)
                   : "memory");
    } else {
      asm volatile("red.global.add.f32 [%0], %1;" ::"l"(a + c), "f"(1.0f) : "memory");
    }
  }
}

template <bool V2, int PATTERN>
cudaError_t run(float *a, uint64_t mask, int blocks, int iters, cudaStream_t s) {
  red_probe_kernel<V2, PATTERN><<<blocks, 256, 0, s>>>(a, mask, iters);
  return cudaGetLastError();
}

}  // namespace

// ops_per_s: reductions (instructions) per second; 0 on success
extern "C" int gg_probe_red_rate(int device, int64_t cells, int v2, int pattern,
                                 double *ops_per_s) {
  if (!ops_per_s || cells < 1 || (cells & (cells - 1)) || pattern < 0 || pattern > 1) return 1;
  if (cudaSetDevice(device) != cudaSuccess) return 2;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const int blocks = sms * 8, iters = 256;
  float *a = nullptr;
  const size_t bytes = (size_t)cells * (v2 ? 8 : 4);
  if (cudaMalloc(&a, bytes) != cudaSuccess) return 3;
  cudaStream_t s;
  cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaMemsetAsync(a, 0, bytes, s);
  const uint64_t mask = (uint64_t)cells - 1;
  auto launch = [&]() {
    if (v2) return pattern ? run<true, 1>(a, mask, blocks, iters, s) : run<true, 0>(a, mask, blocks, iters, s);
    return pattern ? run<false, 1>(a, mask, blocks, iters, s) : run<false, 0>(a, mask, blocks, iters, s);
  };
  int st = 0;
  if (launch() != cudaSuccess) st = 4;
  const int reps = 5;
  cudaEventRecord(e0, s);
  for (int r = 0; r < reps && !st; ++r)
    if (launch() != cudaSuccess) st = 4;
  cudaEventRecord(e1, s);
  if (cudaEventSynchronize(e1) != cudaSuccess) st = 5;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  *ops_per_s = st ? 0.0 : (double)reps * blocks * 256.0 * iters / (ms * 1e-3);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(s);
  cudaFree(a);
  return st;
}
