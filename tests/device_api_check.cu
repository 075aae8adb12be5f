// Test helper: evaluates S, Su, Sv, Suu, Suv, Svv through the header-only device API
// (include/gpu_nurbs_device.cuh) on the host and in a CUDA kernel, the way the reference's
// EvaluateRandom (src/NURBS/Evaluate.cu:1023-1038) walks a point: findSpan, local parameters,
// MatrixNPosition, MatrixSurfacePoint, then each derivative.  Built by the tests with nvcc
// --fmad=false into a temporary directory; output is SoA, 18 planes of n doubles.
#include <cuda_runtime.h>

#include "../include/gpu_nurbs_device.cuh"

namespace {
struct Surf {
  int p, q, nu, nv;
  const double *ku, *kv, *M;
};

__host__ __device__ void eval_one(const Surf& s, double uu, double vv, long long k, long long n, double* out) {
  using namespace nurbs_device;
  int m = findSpan(s.p, s.nu, s.ku, uu);
  int l = findSpan(s.q, s.nv, s.kv, vv);
  double u = (uu - s.ku[m]) / (s.ku[m + 1] - s.ku[m]);
  double v = (vv - s.kv[l]) / (s.kv[l + 1] - s.kv[l]);
  double spanU = (s.ku[s.p + s.nu] - s.ku[0]) / (s.ku[m + 1] - s.ku[m]);
  double spanV = (s.kv[s.q + s.nv] - s.kv[0]) / (s.kv[l + 1] - s.kv[l]);
  const double* mid = s.M + MatrixNPosition(m, l, s.p, s.q, s.nu, s.nv, 0);
  d4 R = MatrixSurfacePoint(mid, s.p, s.q, u, v);
  d3 blk[6] = {homogenousToCartesian(R),
               MatrixSurfaceDerivativeU(mid, s.p, s.q, u, v, R, spanU),
               MatrixSurfaceDerivativeV(mid, s.p, s.q, u, v, R, spanV),
               MatrixSurfaceDerivativeUU(mid, s.p, s.q, u, v, R, spanU, spanV),
               MatrixSurfaceDerivativeUV(mid, s.p, s.q, u, v, R, spanU, spanV),
               MatrixSurfaceDerivativeVV(mid, s.p, s.q, u, v, R, spanU, spanV)};
  for (int b = 0; b < 6; ++b) {
    out[(3 * b + 0) * n + k] = blk[b].x;
    out[(3 * b + 1) * n + k] = blk[b].y;
    out[(3 * b + 2) * n + k] = blk[b].z;
  }
}

__global__ void k_eval(Surf s, const double* uv, long long n, double* out) {
  long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (k < n) eval_one(s, uv[2 * k], uv[2 * k + 1], k, n, out);
}
}  // namespace

extern "C" int dapi_eval_host(int p, int q, int nu, int nv, const double* ku, const double* kv, const double* M,
                              const double* uv, long long n, double* out) {
  if (p < 1 || q < 1 || p > gnurbs::kMaxDegree || q > gnurbs::kMaxDegree) return -1;
  Surf s{p, q, nu, nv, ku, kv, M};
  for (long long k = 0; k < n; ++k) eval_one(s, uv[2 * k], uv[2 * k + 1], k, n, out);
  return 0;
}

// Copies the inputs to the device, runs one thread per point, copies the 18 planes back.
extern "C" int dapi_eval_device(int p, int q, int nu, int nv, const double* ku, const double* kv, const double* M,
                                long long m_len, const double* uv, long long n, double* out) {
  if (p < 1 || q < 1 || p > gnurbs::kMaxDegree || q > gnurbs::kMaxDegree || n <= 0) return -1;
  size_t bku = sizeof(double) * (nu + p + 1), bkv = sizeof(double) * (nv + q + 1);
  size_t bM = sizeof(double) * m_len, buv = sizeof(double) * 2 * n, bout = sizeof(double) * 18 * n;
  double *dku = nullptr, *dkv = nullptr, *dM = nullptr, *duv = nullptr, *dout = nullptr;
  cudaError_t e = cudaSuccess;
  if (!e) e = cudaMalloc(&dku, bku);
  if (!e) e = cudaMalloc(&dkv, bkv);
  if (!e) e = cudaMalloc(&dM, bM);
  if (!e) e = cudaMalloc(&duv, buv);
  if (!e) e = cudaMalloc(&dout, bout);
  if (!e) e = cudaMemcpy(dku, ku, bku, cudaMemcpyHostToDevice);
  if (!e) e = cudaMemcpy(dkv, kv, bkv, cudaMemcpyHostToDevice);
  if (!e) e = cudaMemcpy(dM, M, bM, cudaMemcpyHostToDevice);
  if (!e) e = cudaMemcpy(duv, uv, buv, cudaMemcpyHostToDevice);
  if (!e) {
    k_eval<<<(unsigned)((n + 127) / 128), 128>>>(Surf{p, q, nu, nv, dku, dkv, dM}, duv, n, dout);
    e = cudaGetLastError();
  }
  if (!e) e = cudaMemcpy(out, dout, bout, cudaMemcpyDeviceToHost);
  cudaFree(dku);
  cudaFree(dkv);
  cudaFree(dM);
  cudaFree(duv);
  cudaFree(dout);
  return (int)e;
}
