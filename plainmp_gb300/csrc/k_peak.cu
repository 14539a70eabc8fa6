// FMA throughput microbenchmark: the measured FP32 / FP64 peak that the benchmark's rooflines of the
// arithmetic-bound kernels (the IK descent, the trajectory costs) divide by, in place of a nominal
// figure.  Each thread runs 8 independent FMA chains (enough independent work per warp to keep the
// pipe busy), with start values that depend on the thread so nothing folds at compile time, and
// writes one sum so nothing is dead.  Work per launch: 2 flops x 8 chains x iters per thread.
#include "pm_launch.h"

namespace {

template <class T>
__global__ void k_fma_peak(int iters, T* __restrict__ out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const T a = (T)1.0000001, b = (T)0.9999999;
  T x[8];
#pragma unroll
  for (int k = 0; k < 8; k++) x[k] = (T)(t & 255) * (T)1e-3 + (T)k;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = fma(x[k], a, b);
  }
  T s = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += x[k];
  out[t] = s;
}

}  // namespace

namespace pmg {

cudaError_t launch_fma_peak(int fp64, int iters, void* out, int blocks, int threads, cudaStream_t s) {
  if (fp64)
    k_fma_peak<double><<<blocks, threads, 0, s>>>(iters, static_cast<double*>(out));
  else
    k_fma_peak<float><<<blocks, threads, 0, s>>>(iters, static_cast<float*>(out));
  return cudaGetLastError();
}

}  // namespace pmg
