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
  // S / Su / Sv / Suu / Suv / Svv (mask bits) at n device (u,v) pairs, SoA output
  void eval(const double* uv_dev, int64_t n, unsigned mask, double* out_dev, void* stream = nullptr) const {
    check(nurbs_eval(h_, uv_dev, n, mask, out_dev, NURBS_PREC_FP64, stream), "nurbs_eval");
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

 private:
  void reset() {
    if (h_) nurbs_surface_destroy(h_);
    h_ = nullptr;
  }
  nurbs_surface_t h_ = nullptr;
};

}  // namespace nurbs
