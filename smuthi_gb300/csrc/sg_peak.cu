// FMA-throughput probe used to state FP64 / FP32 pipe rooflines next to measured kernels.
// Each thread runs 8 independent FMA chains; the grid fills every SM several times.
#include <cuda_runtime.h>

#include "sg_internal.h"

namespace sg {

template <typename T>
__global__ void fma_probe_kernel(T *out, int iters, T a, T b) {
  T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b);
    x1 = fma(x1, a, b);
    x2 = fma(x2, a, b);
    x3 = fma(x3, a, b);
    x4 = fma(x4, a, b);
    x5 = fma(x5, a, b);
    x6 = fma(x6, a, b);
    x7 = fma(x7, a, b);
  }
  const T s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (s == T(-12345)) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the chains live
}

// returns TFLOP/s (2 flops per FMA)
double fma_peak(int fp64, cudaStream_t st) {
  int dev = 0, sms = 0;
  SG_CUDA(cudaGetDevice(&dev));
  SG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int threads = 256, blocks = sms * 8;
  const int iters = fp64 ? 512 : 16384;
  DevBuf<double> out;
  out.reserve((size_t)threads * blocks);
  cudaEvent_t e0, e1;
  SG_CUDA(cudaEventCreate(&e0));
  SG_CUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    SG_CUDA(cudaEventRecord(e0, st));
    if (fp64)
      fma_probe_kernel<double><<<blocks, threads, 0, st>>>(out.ptr, iters, 0.999999, 1e-7);
    else
      fma_probe_kernel<float><<<blocks, threads, 0, st>>>((float *)out.ptr, iters, 0.999999f, 1e-7f);
    SG_CUDA(cudaGetLastError());
    SG_CUDA(cudaEventRecord(e1, st));
    SG_CUDA(cudaEventSynchronize(e1));
    float ms = 0;
    SG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if (rep > 0 && ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const double flops = 2.0 * 8.0 * iters * (double)threads * blocks;
  return flops / (best * 1e-3) / 1e12;
}

}  // namespace sg
