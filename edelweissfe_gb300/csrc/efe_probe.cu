// efe_probe.cu -- arithmetic-pipe probe for the roofline of the element pass.
//
// The element pass of the plastic Hexa8 workload is bound by FP64 issue, not by HBM: its roofline
// needs the FP64 (and, for the float-float forms, FP32) FMA throughput of the GPU it runs on.  This
// kernel measures it: every thread runs CHAINS independent FMA chains x <- x * a + b for `iterations`
// steps, so the pipe is issue-bound (enough independent work per warp to cover the FMA latency, many
// warps per SM).  FLOPs = 2 * CHAINS * iterations * threads; the caller times the launch.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/efe_gb300.h"

namespace efe {

constexpr int PROBE_CHAINS = 8;

template <typename T>
__global__ void __launch_bounds__(256) fma_probe_kernel(int64_t iterations, T a, T b, T* sink) {
  T x[PROBE_CHAINS];
#pragma unroll
  for (int k = 0; k < PROBE_CHAINS; ++k) x[k] = T(threadIdx.x % 7 + k) * T(0.125);
  for (int64_t i = 0; i < iterations; ++i) {
#pragma unroll
    for (int k = 0; k < PROBE_CHAINS; ++k) x[k] = fma(x[k], a, b);
  }
  T s = T(0);
#pragma unroll
  for (int k = 0; k < PROBE_CHAINS; ++k) s += x[k];
  // x converges to b / (1 - a) = 1 per chain: the sum is never negative, the store never happens,
  // but the compiler cannot drop the chains
  if (s < T(0)) sink[0] = s;
}

cudaError_t fma_probe(int fp64, int blocks, int64_t iterations, void* sink, cudaStream_t st) {
  if (fp64)
    fma_probe_kernel<double><<<blocks, 256, 0, st>>>(iterations, 0.999999, 1e-6, static_cast<double*>(sink));
  else
    fma_probe_kernel<float><<<blocks, 256, 0, st>>>(iterations, 0.9999f, 1e-4f, static_cast<float*>(sink));
  return cudaGetLastError();
}

int64_t fma_probe_flops(int blocks, int64_t iterations) {
  return (int64_t)2 * PROBE_CHAINS * iterations * blocks * 256;
}

}  // namespace efe
