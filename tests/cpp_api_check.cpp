// Test helper: drives the C++ classes of gpu_nurbs.hpp end to end on one small bicubic patch.
// Evaluates points on the surface (Surface::eval), recovers their parameters through a Pool
// (direct call, autotuned call, graph replay) and through a Server (submit / wait), and prints
// "ok <max parameter error>" on success.  Built and run by tests/test_cpp_api.py.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "gpu_nurbs.hpp"

static const char* kPatch =
    "NU 3 3\nCP 4 4\n"
    "KNu 0 0 0 0 1 1 1 1\nKNv 0 0 0 0 1 1 1 1\n"
    "DP 0 0 0 1\nDP 0 0.33 0.1 1\nDP 0 0.66 -0.1 1\nDP 0 1 0 1\n"
    "DP 0.33 0 0.1 1\nDP 0.33 0.33 0.3 1.5\nDP 0.33 0.66 0.2 1\nDP 0.33 1 0 1\n"
    "DP 0.66 0 -0.1 1\nDP 0.66 0.33 0.2 1\nDP 0.66 0.66 0.3 0.7\nDP 0.66 1 0.1 1\n"
    "DP 1 0 0 1\nDP 1 0.33 0.1 1\nDP 1 0.66 0 1\nDP 1 1 0.2 1\n";

#define CK(x)                                                           \
  do {                                                                  \
    cudaError_t e_ = (x);                                               \
    if (e_ != cudaSuccess) {                                            \
      std::printf("cuda error %s at %d\n", cudaGetErrorString(e_), __LINE__); \
      return 2;                                                         \
    }                                                                   \
  } while (0)

int main() {
  try {
    const int n = 64;
    nurbs::SurfaceDesc desc = nurbs::NuFile::parse(kPatch);
    nurbs::Surface surf(desc);

    std::vector<double> uv(2 * n);
    for (int k = 0; k < n; ++k) {
      uv[2 * k] = 0.1 + 0.8 * ((k * 37) % n) / double(n);
      uv[2 * k + 1] = 0.1 + 0.8 * ((k * 11) % n) / double(n);
    }
    double *d_uv, *d_S, *d_P, *d_out_uv, *d_res;
    int* d_st;
    CK(cudaMalloc(&d_uv, sizeof(double) * 2 * n));
    CK(cudaMalloc(&d_S, sizeof(double) * 3 * n));
    CK(cudaMalloc(&d_P, sizeof(double) * 3 * n));
    CK(cudaMalloc(&d_out_uv, sizeof(double) * 2 * n));
    CK(cudaMalloc(&d_res, sizeof(double) * n));
    CK(cudaMalloc(&d_st, sizeof(int) * n));
    CK(cudaMemcpy(d_uv, uv.data(), sizeof(double) * 2 * n, cudaMemcpyHostToDevice));
    surf.eval(d_uv, n, NURBS_S, d_S);
    std::vector<double> S(3 * n), P(3 * n);
    CK(cudaMemcpy(S.data(), d_S, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost));
    for (int k = 0; k < n; ++k)  // SoA planes -> interleaved query points
      for (int c = 0; c < 3; ++c) P[3 * k + c] = S[c * n + k];
    CK(cudaMemcpy(d_P, P.data(), sizeof(double) * 3 * n, cudaMemcpyHostToDevice));

    double worst = 0;
    auto check_uv = [&](const std::vector<double>& got) {
      for (int k = 0; k < 2 * n; ++k) worst = std::fmax(worst, std::fabs(got[k] - uv[k]));
    };
    std::vector<double> got(2 * n);

    // the surface calls beyond the inversion: projection, quadtree inversion, p-curve (points on
    // the surface: each returns the generating parameters)
    int* d_fl;
    CK(cudaMalloc(&d_fl, sizeof(int) * n));
    surf.project(d_P, n, d_out_uv, d_st, d_res);
    CK(cudaMemcpy(got.data(), d_out_uv, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost));
    check_uv(got);
    surf.invert_quadtree(d_P, n, 1e-4, d_out_uv, d_st, d_res);
    CK(cudaMemcpy(got.data(), d_out_uv, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost));
    check_uv(got);
    surf.pcurve(d_P, n, d_out_uv, d_st, d_res, d_fl);
    CK(cudaMemcpy(got.data(), d_out_uv, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost));
    check_uv(got);
    CK(cudaFree(d_fl));

    nurbs::Pool pool(int64_t(64) << 20, 16);
    std::vector<int> ids = pool.add({desc, desc});
    nurbs::Batch batch{{ids[0], ids[1]}, {0, n / 2, n}};
    pool.invert(batch, d_P, d_out_uv, d_st, d_res, NURBS_PREC_MIXED);
    CK(cudaMemcpy(got.data(), d_out_uv, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost));
    check_uv(got);

    std::pair<int, int> cfg = pool.autotune(batch, d_P, d_out_uv, d_st, d_res, NURBS_PREC_FP64);
    if (pool.info().tile_queries != cfg.first) throw std::runtime_error("autotune did not keep its choice");
    {
      nurbs::Graph g = pool.graph(batch, d_P, d_out_uv, d_st, d_res, NURBS_PREC_MIXED);
      CK(cudaMemset(d_out_uv, 0, sizeof(double) * 2 * n));
      g.launch();
      CK(cudaDeviceSynchronize());
      CK(cudaMemcpy(got.data(), d_out_uv, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost));
      check_uv(got);
    }

    {
      nurbs_server_config sc{2, 4096, 64, NURBS_PREC_MIXED};
      nurbs::Server server(pool, sc);
      std::vector<double> suv(2 * n), sres(n);
      std::vector<int> sst(n);
      uint64_t t = server.submit_invert(ids[1], P.data(), n, suv.data(), sst.data(), sres.data());
      if (server.wait(t) != NURBS_OK) throw std::runtime_error("server request failed");
      int new_id = -1;
      uint64_t tu = server.submit_upload(desc, &new_id);
      if (server.wait(tu) != NURBS_OK || new_id < 0) throw std::runtime_error("server upload failed");
      server.drain();
      check_uv(suv);
      if (server.stats().completed < 2) throw std::runtime_error("server stats");
    }
    for (void* p : {(void*)d_uv, (void*)d_S, (void*)d_P, (void*)d_out_uv, (void*)d_res, (void*)d_st}) cudaFree(p);
    if (!(worst <= 1e-9)) {
      std::printf("parameter error %.3e\n", worst);
      return 1;
    }
    std::printf("ok %.3e\n", worst);
    return 0;
  } catch (const nurbs::Error& e) {
    std::printf("nurbs::Error %d: %s\n", e.code(), e.what());
    return 1;
  } catch (const std::exception& e) {
    std::printf("error: %s\n", e.what());
    return 1;
  }
}
