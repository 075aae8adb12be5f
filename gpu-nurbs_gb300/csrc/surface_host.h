// Host-side preparation of one surface for the device: validation, breakpoint tables and the
// layout of its device block.  Shared by the single-surface handle (api.cpp) and the pool
// (pool.cpp).
#pragma once
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "gpu_nurbs.h"
#include "nurbs_internal.h"

namespace gnurbs {

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Distinct breakpoints of the domain [k[p], k[n]] and the knot index of each non-empty span.
// Spans are the m in [p, cp-1] with k[m] < k[m+1]: exactly those findSpan can return for a
// parameter in the domain (src/NURBS/Evaluate.cu:504-533).
inline void breakpoints(const double* k, int p, int cp, std::vector<double>& b, std::vector<int>& idx) {
  b.clear();
  idx.clear();
  for (int m = p; m < cp; ++m) {
    if (k[m] < k[m + 1]) {
      if (b.empty()) b.push_back(k[m]);
      idx.push_back(m);
      b.push_back(k[m + 1]);
    }
  }
}

// Everything the device block of one surface is built from.  Its block has two parts: the
// input part (uploaded: tables, knots, control net, zeroed tree) and the computed part (span
// matrices and basis matrices, written by the conversion kernels).
struct SurfaceHost {
  int p = 0, q = 0, nu = 0, nv = 0;
  std::vector<double> ku, kv, bu, bv, idu, idv, cps, w;
  std::vector<float> bu32, bv32, idu32, idv32;
  std::vector<int> iu, iv;
  // offsets inside the input part
  size_t o_bu, o_bv, o_idu, o_idv, o_bu32, o_bv32, o_idu32, o_idv32, o_iu, o_iv, o_ku, o_kv, o_cps, o_w, o_tree,
      o_div, o_built, in_bytes;
  // offsets inside the computed part
  size_t o_m64, o_m32, o_bas_u, o_bas_v, o_cd32, o_cd64, o_nbox, o_cone, o_lat, o_qtb, out_bytes;
};

// Validates and prepares a surface given by host arrays.  Returns NURBS_OK or an error code,
// with a message in err.
inline int prepare_surface(int p, int q, int nu, int nv, const double* ku, const double* kv, const double* cps,
                           const double* w, SurfaceHost& S, std::string& err) {
  auto bad = [&](int code, const std::string& m) {
    err = m;
    return code;
  };
  if (!ku || !kv || !cps || !w) return bad(NURBS_E_INVALID, "NULL surface array");
  if (p < 1 || q < 1 || p > NURBS_MAX_DEGREE || q > NURBS_MAX_DEGREE)
    return bad(NURBS_E_INVALID, "degrees outside 1..7");
  if (nu < p + 1 || nv < q + 1) return bad(NURBS_E_INVALID, "control net too small for the degree");
  if ((int64_t)nu * nv > (int64_t)1 << 28) return bad(NURBS_E_UNSUPPORTED, "control net too large");
  auto check_knots = [&](const double* k, int deg, int cp, const char* name) {
    for (int i = 0; i < deg + cp + 1; ++i)
      if (!std::isfinite(k[i])) return bad(NURBS_E_INVALID, std::string(name) + " has a non-finite knot");
    for (int i = 0; i + 1 < deg + cp + 1; ++i)
      if (k[i] > k[i + 1]) return bad(NURBS_E_INVALID, std::string(name) + " is not non-decreasing");
    if (!(k[deg] < k[cp])) return bad(NURBS_E_INVALID, std::string(name) + ": empty parameter domain");
    return (int)NURBS_OK;
  };
  int rc = check_knots(ku, p, nu, "knots_u");
  if (rc) return rc;
  if ((rc = check_knots(kv, q, nv, "knots_v"))) return rc;
  const size_t ncp = (size_t)nu * nv;
  for (size_t i = 0; i < ncp; ++i) {
    if (!(w[i] > 0) || !std::isfinite(w[i])) return bad(NURBS_E_INVALID, "a weight is not a finite positive number");
    for (int c = 0; c < 3; ++c)
      if (!std::isfinite(cps[3 * i + c])) return bad(NURBS_E_INVALID, "a control point is not finite");
  }
  S.p = p; S.q = q; S.nu = nu; S.nv = nv;
  S.ku.assign(ku, ku + p + nu + 1);
  S.kv.assign(kv, kv + q + nv + 1);
  S.cps.assign(cps, cps + 3 * ncp);
  S.w.assign(w, w + ncp);
  breakpoints(S.ku.data(), p, nu, S.bu, S.iu);
  breakpoints(S.kv.data(), q, nv, S.bv, S.iv);
  const int nsu = (int)S.iu.size(), nsv = (int)S.iv.size();
  S.idu.resize(nsu);
  S.idv.resize(nsv);
  S.idu32.resize(nsu);
  S.idv32.resize(nsv);
  S.bu32.assign(S.bu.begin(), S.bu.end());
  S.bv32.assign(S.bv.begin(), S.bv.end());
  for (int i = 0; i < nsu; ++i) S.idu[i] = 1.0 / (S.bu[i + 1] - S.bu[i]), S.idu32[i] = (float)S.idu[i];
  for (int i = 0; i < nsv; ++i) S.idv[i] = 1.0 / (S.bv[i + 1] - S.bv[i]), S.idv32[i] = (float)S.idv[i];
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off = align256(off + bytes);
    return o;
  };
  S.o_bu = take((nsu + 1) * 8); S.o_bv = take((nsv + 1) * 8);
  S.o_idu = take(nsu * 8); S.o_idv = take(nsv * 8);
  S.o_bu32 = take((nsu + 1) * 4); S.o_bv32 = take((nsv + 1) * 4);
  S.o_idu32 = take(nsu * 4); S.o_idv32 = take(nsv * 4);
  S.o_iu = take(nsu * 4); S.o_iv = take(nsv * 4);
  S.o_ku = take(S.ku.size() * 8); S.o_kv = take(S.kv.size() * 8);
  S.o_cps = take(ncp * 3 * 8); S.o_w = take(ncp * 8);
  S.o_tree = take(kTreeNodes * sizeof(TreeNodeDev));
  S.o_div = take(kTreeNodes); S.o_built = take(kTreeNodes);
  S.in_bytes = off;
  off = 0;
  const size_t k12 = (size_t)(p + 1) * (q + 1), nspan = (size_t)nsu * nsv;
  S.o_m64 = take(nspan * k12 * 4 * 8);
  S.o_m32 = take(nspan * (size_t)span_coefs32(p, q) * 4 * 4);
  S.o_bas_u = take((size_t)nsu * (p + 1) * (p + 1) * 8);
  S.o_bas_v = take((size_t)nsv * (q + 1) * (q + 1) * 8);
  S.o_cd32 = take(kTreeNodes * 9 * 4);
  S.o_cd64 = take(kTreeNodes * 9 * 8);
  S.o_nbox = take(kTreeNodes * 6 * 8);
  S.o_cone = take(kTreeNodes * kConeStride * 4);
  S.o_lat = take(kTreeNodes * kPts * kPts * 3 * 4);
  S.o_qtb = take(21 * 6 * 8);
  S.out_bytes = off;
  return NURBS_OK;
}

// Writes the input part of the block into host memory `img` (in_bytes, zero-initialised by the
// caller) and fills the device view for blocks at device addresses in_dev / out_dev.
inline void fill_surface(const SurfaceHost& S, char* img, char* in_dev, char* out_dev, SurfDev& d) {
  auto put = [&](size_t o, const void* src, size_t bytes) {
    if (bytes) std::memcpy(img + o, src, bytes);
  };
  const int nsu = (int)S.iu.size(), nsv = (int)S.iv.size();
  put(S.o_bu, S.bu.data(), S.bu.size() * 8);
  put(S.o_bv, S.bv.data(), S.bv.size() * 8);
  put(S.o_idu, S.idu.data(), nsu * 8);
  put(S.o_idv, S.idv.data(), nsv * 8);
  put(S.o_bu32, S.bu32.data(), S.bu32.size() * 4);
  put(S.o_bv32, S.bv32.data(), S.bv32.size() * 4);
  put(S.o_idu32, S.idu32.data(), nsu * 4);
  put(S.o_idv32, S.idv32.data(), nsv * 4);
  put(S.o_iu, S.iu.data(), nsu * 4);
  put(S.o_iv, S.iv.data(), nsv * 4);
  put(S.o_ku, S.ku.data(), S.ku.size() * 8);
  put(S.o_kv, S.kv.data(), S.kv.size() * 8);
  put(S.o_cps, S.cps.data(), S.cps.size() * 8);
  put(S.o_w, S.w.data(), S.w.size() * 8);
  d = SurfDev{};
  d.p = S.p; d.q = S.q; d.nu = S.nu; d.nv = S.nv; d.ns_u = nsu; d.ns_v = nsv;
  d.range_u = S.ku[S.p + S.nu] - S.ku[0];  // kernel.cu:167
  d.range_v = S.kv[S.q + S.nv] - S.kv[0];
  d.range_u32 = (float)d.range_u;
  d.range_v32 = (float)d.range_v;
  d.dom_u0 = S.ku[S.p]; d.dom_u1 = S.ku[S.nu]; d.dom_v0 = S.kv[S.q]; d.dom_v1 = S.kv[S.nv];
  for (int c = 0; c < 3; ++c) {
    double lo = S.cps[c], hi = S.cps[c];
    for (size_t k = 3 + c; k < S.cps.size(); k += 3) {
      lo = std::min(lo, S.cps[k]);
      hi = std::max(hi, S.cps[k]);
    }
    d.org[c] = 0.5 * (lo + hi);
    d.org32[c] = (float)d.org[c];
  }
  d.bu = (const double*)(in_dev + S.o_bu); d.bv = (const double*)(in_dev + S.o_bv);
  d.inv_du = (const double*)(in_dev + S.o_idu); d.inv_dv = (const double*)(in_dev + S.o_idv);
  d.bu32 = (const float*)(in_dev + S.o_bu32); d.bv32 = (const float*)(in_dev + S.o_bv32);
  d.inv_du32 = (const float*)(in_dev + S.o_idu32); d.inv_dv32 = (const float*)(in_dev + S.o_idv32);
  d.knot_u = (const int*)(in_dev + S.o_iu); d.knot_v = (const int*)(in_dev + S.o_iv);
  d.knots_u = (const double*)(in_dev + S.o_ku); d.knots_v = (const double*)(in_dev + S.o_kv);
  d.cps = (const double*)(in_dev + S.o_cps); d.weights = (const double*)(in_dev + S.o_w);
  d.tree = (TreeNodeDev*)(in_dev + S.o_tree);
  d.divided = (unsigned char*)(in_dev + S.o_div);
  d.built = (unsigned char*)(in_dev + S.o_built);
  d.m64 = (const double*)(out_dev + S.o_m64); d.m32 = (const float*)(out_dev + S.o_m32);
  d.basis_u = (double*)(out_dev + S.o_bas_u);
  d.basis_v = (double*)(out_dev + S.o_bas_v);
  d.cd32 = (float*)(out_dev + S.o_cd32);
  d.cd64 = (double*)(out_dev + S.o_cd64);
  d.nbox = (double*)(out_dev + S.o_nbox);
  d.cone = (float*)(out_dev + S.o_cone);
  d.lattice = (float*)(out_dev + S.o_lat);
  d.qtbox = (double*)(out_dev + S.o_qtb);
}

}  // namespace gnurbs
