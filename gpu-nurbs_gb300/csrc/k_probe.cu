// Peak-throughput probe: independent FMA chains in FP64 or FP32, timed with CUDA events.
// The benchmark uses it as the measured denominator of its FP64/FP32 roofline fractions.
#include <cuda_runtime.h>

#include "gpu_nurbs.h"

namespace {

template <typename T>
__global__ void k_fma_chains(T* out, int iters, T a, T b) {
  T x0 = (T)threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
      x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

}  // namespace

extern "C" int nurbs_probe_fp_peak(int bits, double* tflops, void* stream) {
  if (!tflops || (bits != 32 && bits != 64)) return NURBS_E_INVALID;
  cudaStream_t st = (cudaStream_t)stream;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 8, threads = 256;
  const int iters = bits == 64 ? 100 : 2000;
  void* out = nullptr;
  if (cudaMallocAsync(&out, (size_t)blocks * threads * 8, st) != cudaSuccess) return NURBS_E_NOMEM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float ms = 0;
  for (int rep = 0; rep < 2; ++rep) {  // first launch warms up
    cudaEventRecord(e0, st);
    if (bits == 64) k_fma_chains<double><<<blocks, threads, 0, st>>>((double*)out, iters, 0.999999, 1e-7);
    else k_fma_chains<float><<<blocks, threads, 0, st>>>((float*)out, iters, 0.999999f, 1e-7f);
    cudaEventRecord(e1, st);
  }
  cudaError_t e = cudaEventSynchronize(e1);
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(out, st);
  if (e != cudaSuccess || ms <= 0) return NURBS_E_CUDA;
  double flops = 2.0 * blocks * threads * (double)iters * 16 * 8;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return NURBS_OK;
}
