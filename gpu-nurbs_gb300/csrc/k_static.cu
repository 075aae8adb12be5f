// GetMatrixN into a caller buffer without any device allocation.
//
// nurbs_get_matrix_n_raw needs scratch memory for the per-span basis-to-power matrices and
// the span index tables, which it takes from a stream-ordered pool.  Some callers cannot allocate
// device memory at the point where they convert a surface: code that runs under a device
// allocator it does not own (a host application whose caching allocator claims all free
// memory, or a memory-budget admitter that forbids allocations outside its pool), and
// real-time or serving loops that must not touch the allocator between requests because an
// allocation can block on device-wide synchronisation.  nurbs_get_matrix_n_noalloc serves
// them: its scratch lives in the file-scope array below, of fixed size, that every GPU which
// loads this library holds until the process exits.
//
// The scratch is shared by all calls: overlapping calls on the GPU (on different streams or
// host threads) race on it and must be serialised by the caller.  Each call rewrites all of
// the scratch it reads (the span tables and their counts are cleared and rebuilt first).
//
// The device address of the array is looked up once per device, on the first call made with
// that device current, and cached.  cudaDeviceReset destroys the context that holds the array;
// the cached address then names freed memory, so the entry point must not be used again in a
// process that has reset the device.
#include <cuda_runtime.h>

#include <mutex>

#include "gpu_nurbs.h"
#include "nurbs_internal.h"

namespace gnurbs {

namespace {

constexpr size_t kStaticScratchBytes = 1u << 20;  // NURBS_NOALLOC_SCRATCH_BYTES
static_assert(kStaticScratchBytes == NURBS_NOALLOC_SCRATCH_BYTES, "scratch size");

// One array per device that loads the library.  In host code `g_scratch` names a host-side
// stand-in, not device memory: only the address from cudaGetSymbolAddress may be passed to a
// kernel.
__device__ __align__(256) unsigned char g_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char* g_scratch_ptr[kMaxDevices] = {};

// Scratch layout: [0, 16) counts {ns_u, ns_v, bad_u, bad_v}; [256, ...) knot indices of u then
// v spans (ints), then the u and v basis matrices (doubles, 256-byte aligned).
struct Counts {
  int ns_u, ns_v, bad_u, bad_v;
};

// Span tables on the device: the knot index m of every non-empty span m in [p, cp-1]
// (the spans findSpan can return, src/NURBS/Evaluate.cu:504-533) and a flag for knots that
// are not finite or not non-decreasing or leave an empty domain.
__global__ void k_span_tables(const double* __restrict__ ku, int p, int nu, const double* __restrict__ kv, int q,
                              int nv, int cap_u, int cap_v, Counts* counts, int* idx_u, int* idx_v) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (int d = 0; d < 2; ++d) {
    const double* k = d == 0 ? ku : kv;
    const int deg = d == 0 ? p : q, cp = d == 0 ? nu : nv, cap = d == 0 ? cap_u : cap_v;
    int* idx = d == 0 ? idx_u : idx_v;
    int n = 0, bad = 0;
    for (int i = 0; i < deg + cp + 1; ++i) {
      if (!isfinite(k[i])) bad = 1;
      if (i > 0 && k[i - 1] > k[i]) bad = 1;
    }
    if (!(k[deg] < k[cp])) bad = 1;
    for (int m = deg; m < cp && !bad; ++m)
      if (k[m] < k[m + 1]) {
        if (n < cap) idx[n] = m;
        ++n;
      }
    if (n > cap) bad = 2;
    if (d == 0) {
      counts->ns_u = n;
      counts->bad_u = bad;
    } else {
      counts->ns_v = n;
      counts->bad_v = bad;
    }
  }
}

size_t up256(size_t x) { return (x + 255) & ~size_t(255); }

// Address of this device's scratch array, looked up once per device with it current.
int scratch_for_current_device(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return fail(NURBS_E_UNSUPPORTED, "device ordinal %d above %d", dev, kMaxDevices - 1);
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_ptr[dev]) {
    void* ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress of the static scratch");
    if (ptr == nullptr) return fail(NURBS_E_CUDA, "cudaGetSymbolAddress returned NULL for the static scratch");
    g_scratch_ptr[dev] = static_cast<unsigned char*>(ptr);
  }
  *out = g_scratch_ptr[dev];
  return NURBS_OK;
}

}  // namespace
}  // namespace gnurbs

using namespace gnurbs;

extern "C" int nurbs_get_matrix_n_noalloc(double* matrix_n_dev, int p, int q, int nu, int nv,
                                          const double* knots_u_dev, const double* knots_v_dev,
                                          const double* control_points_dev, const double* weights_dev,
                                          void* stream) {
  if (!matrix_n_dev || !knots_u_dev || !knots_v_dev || !control_points_dev || !weights_dev)
    return fail(NURBS_E_INVALID, "NULL argument");
  if (p < 1 || q < 1 || p > NURBS_MAX_DEGREE || q > NURBS_MAX_DEGREE)
    return fail(NURBS_E_INVALID, "degrees (%d,%d) outside 1..%d", p, q, NURBS_MAX_DEGREE);
  if (nu < p + 1 || nv < q + 1)
    return fail(NURBS_E_INVALID, "control net %dx%d too small for degree (%d,%d)", nu, nv, p, q);
  const int k1 = p + 1, k2 = q + 1;
  // worst case: every knot interval in the domain is a span
  const size_t max_su = (size_t)(nu - p), max_sv = (size_t)(nv - q);
  const size_t o_idx_u = 256, o_idx_v = o_idx_u + up256(max_su * 4);
  const size_t o_bas_u = o_idx_v + up256(max_sv * 4);
  const size_t o_bas_v = o_bas_u + up256(max_su * k1 * k1 * 8);
  const size_t need = o_bas_v + up256(max_sv * k2 * k2 * 8);
  if (need > kStaticScratchBytes)
    return fail(NURBS_E_UNSUPPORTED, "surface needs %zu bytes of scratch in the worst case, above the static %zu",
                need, kStaticScratchBytes);
  unsigned char* scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc != NURBS_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  Counts* counts = reinterpret_cast<Counts*>(scratch);
  int* idx_u = reinterpret_cast<int*>(scratch + o_idx_u);
  int* idx_v = reinterpret_cast<int*>(scratch + o_idx_v);
  double* bas_u = reinterpret_cast<double*>(scratch + o_bas_u);
  double* bas_v = reinterpret_cast<double*>(scratch + o_bas_v);
  // clear the counts left by the previous call, then rebuild the span tables
  cudaError_t e = cudaMemsetAsync(counts, 0, sizeof(Counts), st);
  if (e != cudaSuccess) return cuda_fail(e, "clearing the static scratch");
  k_span_tables<<<1, 32, 0, st>>>(knots_u_dev, p, nu, knots_v_dev, q, nv, (int)max_su, (int)max_sv, counts, idx_u,
                                  idx_v);
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "span-table launch");
  Counts h{};
  if ((e = cudaMemcpyAsync(&h, counts, sizeof(Counts), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
    return cuda_fail(e, "span-count copy");
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_fail(e, "span-count wait");
  if (h.bad_u || h.bad_v)
    return fail(NURBS_E_INVALID, "%s knot vector is not finite and non-decreasing or has an empty domain",
                h.bad_u ? "u" : "v");
  SurfDev d{};
  d.p = p;
  d.q = q;
  d.nu = nu;
  d.nv = nv;
  d.ns_u = h.ns_u;
  d.ns_v = h.ns_v;
  d.knot_u = idx_u;
  d.knot_v = idx_v;
  d.cps = control_points_dev;
  d.weights = weights_dev;
  e = launch_basis(knots_u_dev, p, idx_u, h.ns_u, bas_u, st);
  if (e == cudaSuccess) e = launch_basis(knots_v_dev, q, idx_v, h.ns_v, bas_v, st);
  if (e == cudaSuccess) e = launch_span_matrices(d, bas_u, bas_v, matrix_n_dev, nullptr, st);
  return e == cudaSuccess ? NURBS_OK : cuda_fail(e, "matrix-form conversion");
}
