// gpu_nurbs.hpp — C++ classes over the C-ABI of gpu_nurbs.h (header-only, RAII).
//
// The reference (Qiang-Zou/GPU-NURBS) has no classes: its host code is main() with raw
// cudaMalloc'd buffers (src/main.cu:128-724).  These wrappers give C++ callers the same calls —
// readNu, GetMatrixN, MatrixSurfacePoint/Derivative*, the tree build and NewInverse — as
// methods, with ownership and errors handled:
//   nurbs::NuFile   readNu (src/main.cu:45-113) / writer
//   nurbs::Surface  a device-resident surface in matrix form with its subdivision tree:
//                   matrix_n() = GetMatrixN layout, eval() = batched S..Svv,
//                   candidates() = the NewInverse scan, invert() = NewInverse + GaussNewton
//   nurbs::Pool     many surfaces under a device budget, batched invert/eval, autotune, graphs
//   nurbs::Server   the continuous-batching request loop over a pool (submit / wait / drain)
//   nurbs::Error    thrown for any non-zero status (message from nurbs_last_error)
#pragma once
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "gpu_nurbs.h"

namespace nurbs {

class Error : public std::runtime_error {
 public:
  Error(int code, const std::string& what)
      : std::runtime_error(what + ": " + nurbs_status_string(code) + " (" + nurbs_last_error() + ")"), code_(code) {}
  int code() const { return code_; }

 private:
  int code_;
};

inline void check(int rc, const char* what) {
  if (rc != NURBS_OK) throw Error(rc, what);
}

// Host-side description of a surface (what readNu fills in).
struct SurfaceDesc {
  int degree_u = 0, degree_v = 0, cp_u = 0, cp_v = 0;
  std::vector<double> knots_u, knots_v, cps /* xyz interleaved */, weights;
};

class NuFile {
 public:
  static SurfaceDesc read(const std::string& path) {
    nurbs_nu_desc d{};
    check(nurbs_nu_read(path.c_str(), &d), "nurbs_nu_read");
    SurfaceDesc s = from(d);
    nurbs_nu_free(&d);
    return s;
  }
  static SurfaceDesc parse(const std::string& text) {
    nurbs_nu_desc d{};
    check(nurbs_nu_parse(text.data(), (int64_t)text.size(), &d), "nurbs_nu_parse");
    SurfaceDesc s = from(d);
    nurbs_nu_free(&d);
    return s;
  }
  static void write(const std::string& path, const SurfaceDesc& s) {
    nurbs_nu_desc d{s.degree_u, s.degree_v, s.cp_u, s.cp_v, const_cast<double*>(s.knots_u.data()),
                    const_cast<double*>(s.knots_v.data()), const_cast<double*>(s.cps.data()),
                    const_cast<double*>(s.weights.data())};
    check(nurbs_nu_write(path.c_str(), &d), "nurbs_nu_write");
  }

 private:
  static SurfaceDesc from(const nurbs_nu_desc& d) {
    SurfaceDesc s;
    s.degree_u = d.degree_u;
    s.degree_v = d.degree_v;
    s.cp_u = d.cp_u;
    s.cp_v = d.cp_v;
    s.knots_u.assign(d.knots_u, d.knots_u + d.degree_u + d.cp_u + 1);
    s.knots_v.assign(d.knots_v, d.knots_v + d.degree_v + d.cp_v + 1);
    s.cps.assign(d.cps, d.cps + 3 * (size_t)d.cp_u * d.cp_v);
    s.weights.assign(d.weights, d.weights + (size_t)d.cp_u * d.cp_v);
    return s;
  }
};

// A surface resident on the GPU.  Device buffers passed to the methods are caller-owned.
class Surface {
 public:
  explicit Surface(const SurfaceDesc& s, void* stream = nullptr) {
    check(nurbs_surface_create(s.degree_u, s.degree_v, s.cp_u, s.cp_v, s.knots_u.data(), s.knots_v.data(),
                               s.cps.data(), s.weights.data(), NURBS_PTR_HOST, stream, &h_),
          "nurbs_surface_create");
  }
  Surface(const Surface&) = delete;
  Surface& operator=(const Surface&) = delete;
  Surface(Surface&& o) noexcept : h_(std::exchange(o.h_, nullptr)) {}
  Surface& operator=(Surface&& o) noexcept {
    if (this != &o) {
      reset();
      h_ = std::exchange(o.h_, nullptr);
    }
    return *this;
  }
  ~Surface() { reset(); }

  nurbs_surface_t handle() const { return h_; }
  nurbs_surface_info_t info() const {
    nurbs_surface_info_t i{};
    check(nurbs_surface_info(h_, &i), "nurbs_surface_info");
    return i;
  }
  // GetMatrixN layout into a caller device buffer of nurbs_matrix_n_size() doubles
  void matrix_n(double* matrix_n_dev, void* stream = nullptr) const {
    check(nurbs_get_matrix_n(h_, matrix_n_dev, stream), "nurbs_get_matrix_n");
  }
  // S / Su / Sv / Suu / Suv / Svv / Suuu..Svvv (mask bits) at n device (u,v) pairs, SoA output;
  // precision NURBS_PREC_EXACT: the reference's expressions term by term (mask <= 63)
  void eval(const double* uv_dev, int64_t n, unsigned mask, double* out_dev, void* stream = nullptr,
            int precision = NURBS_PREC_FP64) const {
    check(nurbs_eval(h_, uv_dev, n, mask, out_dev, precision, stream), "nurbs_eval");
  }
  // N = Su x Sv and its derivatives (NURBS_N..NURBS_NVV bits), SoA output
  void eval_normal(const double* uv_dev, int64_t n, unsigned mask, double* out_dev, void* stream = nullptr) const {
    check(nurbs_eval_normal(h_, uv_dev, n, mask, out_dev, stream), "nurbs_eval_normal");
  }
  void eval_f32(const float* uv_dev, int64_t n, unsigned mask, float* out_dev, void* stream = nullptr) const {
    check(nurbs_eval_f32(h_, uv_dev, n, mask, out_dev, stream), "nurbs_eval_f32");
  }
  void candidates(const double* P_dev, int64_t n, int* list_dev, int* counts_dev, void* stream = nullptr) const {
    check(nurbs_candidates(h_, P_dev, n, list_dev, counts_dev, stream), "nurbs_candidates");
  }
  void invert(const double* P_dev, int64_t n, double* uv_dev, int* status_dev, double* residual_dev,
              int precision = NURBS_PREC_MIXED, void* stream = nullptr) const {
    check(nurbs_invert(h_, P_dev, n, uv_dev, status_dev, residual_dev, precision, stream), "nurbs_invert");
  }
  void invert_host(const double* P, int64_t n, double* uv, int* status, double* residual,
                   int precision = NURBS_PREC_MIXED, void* stream = nullptr) const {
    check(nurbs_invert_host(h_, P, n, uv, status, residual, precision, stream), "nurbs_invert_host");
  }
  // closest points over the closed domain (nurbs_project)
  void project(const double* P_dev, int64_t n, double* uv_dev, int* status_dev, double* residual_dev,
               int precision = NURBS_PREC_MIXED, void* stream = nullptr) const {
    check(nurbs_project(h_, P_dev, n, uv_dev, status_dev, residual_dev, precision, stream), "nurbs_project");
  }
  // the tree-free adaptive quadtree inversion (nurbs_invert_quadtree)
  void invert_quadtree(const double* P_dev, int64_t n, double max_edge, double* uv_dev, int* status_dev,
                       double* residual_dev, int precision = NURBS_PREC_MIXED, void* stream = nullptr) const {
    check(nurbs_invert_quadtree(h_, P_dev, n, max_edge, uv_dev, status_dev, residual_dev, precision, stream),
          "nurbs_invert_quadtree");
  }
  // p-curve of ordered curve samples (nurbs_pcurve)
  void pcurve(const double* C_dev, int64_t n, double* uv_dev, int* status_dev, double* residual_dev, int* flags_dev,
              int precision = NURBS_PREC_MIXED, void* stream = nullptr) const {
    check(nurbs_pcurve(h_, C_dev, n, uv_dev, status_dev, residual_dev, flags_dev, precision, stream), "nurbs_pcurve");
  }

 private:
  void reset() {
    if (h_) nurbs_surface_destroy(h_);
    h_ = nullptr;
  }
  nurbs_surface_t h_ = nullptr;
};

inline nurbs_surface_desc view(const SurfaceDesc& s) {
  return {s.degree_u, s.degree_v, s.cp_u, s.cp_v, s.knots_u.data(), s.knots_v.data(), s.cps.data(), s.weights.data()};
}

// One batch layout: surface ids[k] owns queries [offsets[k], offsets[k+1]).
struct Batch {
  std::vector<int> ids;
  std::vector<int64_t> offsets;
  int size() const { return (int)ids.size(); }
};

// A captured batched inversion (nurbs_pool_graph_create); replays on new query values.
class Graph {
 public:
  explicit Graph(nurbs_graph_t g) : g_(g) {}
  Graph(const Graph&) = delete;
  Graph& operator=(const Graph&) = delete;
  Graph(Graph&& o) noexcept : g_(std::exchange(o.g_, nullptr)) {}
  ~Graph() {
    if (g_) nurbs_graph_destroy(g_);
  }
  void launch(void* stream = nullptr) const { check(nurbs_graph_launch(g_, stream), "nurbs_graph_launch"); }

 private:
  nurbs_graph_t g_ = nullptr;
};

// Many surfaces under one device-memory budget, inverted and evaluated in one launch.
class Pool {
 public:
  explicit Pool(int64_t budget_bytes, int max_surfaces = 65536) {
    check(nurbs_pool_create(budget_bytes, max_surfaces, &h_), "nurbs_pool_create");
  }
  Pool(const Pool&) = delete;
  Pool& operator=(const Pool&) = delete;
  ~Pool() {
    if (h_) nurbs_pool_destroy(h_);
  }
  nurbs_pool_t handle() const { return h_; }

  std::vector<int> add(const std::vector<SurfaceDesc>& surfaces, void* stream = nullptr) {
    std::vector<nurbs_surface_desc> d;
    for (const SurfaceDesc& s : surfaces) d.push_back(view(s));
    std::vector<int> ids(d.size());
    check(nurbs_pool_add(h_, (int)d.size(), d.data(), stream, ids.data()), "nurbs_pool_add");
    return ids;
  }
  void remove(int id, void* stream = nullptr) { check(nurbs_pool_remove(h_, id, stream), "nurbs_pool_remove"); }
  nurbs_pool_info_t info() const {
    nurbs_pool_info_t i{};
    check(nurbs_pool_info(h_, &i), "nurbs_pool_info");
    return i;
  }
  void set_config(int tile_queries, int ctas_per_sm) {
    check(nurbs_pool_set_config(h_, tile_queries, ctas_per_sm), "nurbs_pool_set_config");
  }
  void invert(const Batch& b, const double* P_dev, double* uv_dev, int* status_dev, double* residual_dev,
              int precision = NURBS_PREC_MIXED, void* stream = nullptr) const {
    check(nurbs_pool_invert(h_, b.size(), b.ids.data(), b.offsets.data(), P_dev, uv_dev, status_dev, residual_dev,
                            precision, stream),
          "nurbs_pool_invert");
  }
  void eval(const Batch& b, const double* uv_dev, unsigned mask, double* out_dev, void* stream = nullptr) const {
    check(nurbs_pool_eval(h_, b.size(), b.ids.data(), b.offsets.data(), uv_dev, b.offsets.back(), mask, out_dev,
                          stream),
          "nurbs_pool_eval");
  }
  // Times the launch configurations on the batch and keeps the fastest; returns {tile, ctas}.
  std::pair<int, int> autotune(const Batch& b, const double* P_dev, double* uv_dev, int* status_dev,
                               double* residual_dev, int precision = NURBS_PREC_MIXED, int64_t max_queries = 0,
                               const char* cache_path = nullptr, void* stream = nullptr) {
    int tile = 0, ctas = 0;
    float ms = 0;
    check(nurbs_pool_autotune(h_, b.size(), b.ids.data(), b.offsets.data(), P_dev, uv_dev, status_dev, residual_dev,
                              precision, max_queries, cache_path, stream, &tile, &ctas, &ms),
          "nurbs_pool_autotune");
    return {tile, ctas};
  }
  Graph graph(const Batch& b, const double* P_dev, double* uv_dev, int* status_dev, double* residual_dev,
              int precision = NURBS_PREC_MIXED) const {
    nurbs_graph_t g = nullptr;
    check(nurbs_pool_graph_create(h_, b.size(), b.ids.data(), b.offsets.data(), P_dev, uv_dev, status_dev,
                                  residual_dev, precision, &g),
          "nurbs_pool_graph_create");
    return Graph(g);
  }

 private:
  nurbs_pool_t h_ = nullptr;
};

// The continuous-batching request loop over a pool (the pool must outlive it).
class Server {
 public:
  Server(Pool& pool, const nurbs_server_config& cfg) { check(nurbs_server_create(pool.handle(), &cfg, &h_), "nurbs_server_create"); }
  Server(const Server&) = delete;
  Server& operator=(const Server&) = delete;
  ~Server() {
    if (h_) nurbs_server_destroy(h_);
  }
  nurbs_server_t handle() const { return h_; }
  // Host buffers stay owned by the caller and must live until the request completes.
  uint64_t submit_invert(int surf_id, const double* P, int64_t n, double* uv, int* status, double* residual,
                         double* latency_us = nullptr) {
    uint64_t t = 0;
    check(nurbs_server_submit_invert(h_, surf_id, P, n, uv, status, residual, latency_us, &t),
          "nurbs_server_submit_invert");
    return t;
  }
  uint64_t submit_upload(const SurfaceDesc& s, int* surf_id_out, double* latency_us = nullptr) {
    nurbs_surface_desc d = view(s);
    uint64_t t = 0;
    check(nurbs_server_submit_upload(h_, &d, surf_id_out, latency_us, &t), "nurbs_server_submit_upload");
    return t;
  }
  // The request's own status (NURBS_OK or its error); throws on a timeout or a bad ticket.
  int wait(uint64_t ticket, int timeout_ms = 10000) {
    int result = 0;
    check(nurbs_server_wait(h_, ticket, timeout_ms, &result), "nurbs_server_wait");
    return result;
  }
  void drain(int timeout_ms = 60000) { check(nurbs_server_drain(h_, timeout_ms), "nurbs_server_drain"); }
  void pause(bool paused) { check(nurbs_server_pause(h_, paused ? 1 : 0), "nurbs_server_pause"); }
  nurbs_server_stats_t stats() const {
    nurbs_server_stats_t s{};
    check(nurbs_server_stats(h_, &s), "nurbs_server_stats");
    return s;
  }

 private:
  nurbs_server_t h_ = nullptr;
};

}  // namespace nurbs
