// Surface pool: many surfaces resident in one device arena under a memory budget, converted in
// batches, and inverted together by one persistent launch (k_pool.cu).
//
//  * Arena: one cudaMalloc of the budget at creation; surfaces and per-stream workspaces are
//    carved from it first-fit, so admission is a budget check (NURBS_E_BUDGET when nothing fits).
//  * Batched upload: the input parts of all surfaces of a batch are staged contiguously and sent
//    with one copy; conversion runs one launch per stage for the whole batch (basis columns,
//    span matrices, tree level 0, tree level 1).
//  * Batched inversion: the batch (CSR: surface k owns queries [offsets[k], offsets[k+1]) ) is cut
//    into tiles of at most tile_queries queries of one surface, ordered most expensive first
//    (degree, then count) so the persistent CTAs finish together.
//  * Autotuner: times tile size x CTAs per SM on the batch (or a prefix of it) and keeps the
//    fastest; results can be cached in a text file keyed by GPU, precision and batch signature.
//  * CUDA graph: a batch layout is captured once (counter reset + persistent kernel) and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <new>
#include <set>
#include <sstream>
#include <string>
#include <vector>

#include "gpu_nurbs.h"
#include "nurbs_internal.h"
#include "surface_host.h"

using namespace gnurbs;

namespace {

thread_local std::string g_pool_error;

int pfail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_pool_error = buf;
  return code;
}

// First-fit allocator over [0, size) in 256-byte units.
class Arena {
 public:
  void init(size_t size) {
    free_.clear();
    free_[0] = size;
    used_ = 0;
  }
  bool alloc(size_t bytes, size_t& off) {
    bytes = align256(bytes ? bytes : 256);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= bytes) {
        off = it->first;
        size_t rest = it->second - bytes;
        free_.erase(it);
        if (rest) free_[off + bytes] = rest;
        used_ += bytes;
        return true;
      }
    }
    return false;
  }
  void release(size_t off, size_t bytes) {
    bytes = align256(bytes ? bytes : 256);
    used_ -= bytes;
    auto it = free_.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
  size_t used() const { return used_; }

 private:
  std::map<size_t, size_t> free_;
  size_t used_ = 0;
};

struct PoolSurface {
  bool live = false;
  bool reserved = false;  // being converted by a pool_add in progress
  size_t in_off = 0, in_bytes = 0, out_off = 0, out_bytes = 0;
  int p = 0, q = 0;
  int64_t spans = 0;
};

struct Workspace {
  size_t off = 0, cap_tiles = 0;  // device: counter (256 B) + tiles
  InvTile* host = nullptr;        // pinned staging of the tile list
  size_t host_cap = 0;
  cudaEvent_t ev = nullptr;       // completion of the last upload from `host`
};

}  // namespace

struct nurbs_pool_s {
  std::mutex mu;
  char* base = nullptr;
  size_t budget = 0;
  Arena arena;
  int max_surfaces = 0;
  std::vector<PoolSurface> surf;
  SurfDev* d_table = nullptr;  // device table of max_surfaces records (outside the arena)
  int tile_queries = 128;
  int ctas_per_sm = 6;  // the CTA-tile kernel is budgeted for 6 (mixed)
  int sms = 152;
  std::map<cudaStream_t, Workspace> ws;
  std::set<struct nurbs_graph_s*> graphs;  // live graphs, detached if the pool goes first
};

struct nurbs_graph_s {
  nurbs_pool_t pool = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  size_t off = 0, bytes = 0;  // counter + tiles in the arena
};

namespace {

// Tile list of a CSR batch: per surface, ranges of at most tile_q queries; most expensive
// (higher degree, then larger) tiles first.
int make_tiles(nurbs_pool_t P, int nbatch, const int* ids, const int64_t* offsets, int tile_q,
               std::vector<InvTile>& tiles) {
  tiles.clear();
  for (int k = 0; k < nbatch; ++k) {
    int id = ids[k];
    if (id < 0 || id >= (int)P->surf.size() || !P->surf[id].live) return pfail(NURBS_E_INVALID, "surface id %d not in the pool", id);
    int64_t b = offsets[k], e = offsets[k + 1];
    if (e < b) return pfail(NURBS_E_INVALID, "offsets are not non-decreasing at %d", k);
    for (int64_t q = b; q < e; q += tile_q) {
      InvTile t;
      t.surf = id;
      t.begin = q;
      t.count = (int)std::min<int64_t>(tile_q, e - q);
      tiles.push_back(t);
    }
  }
  std::stable_sort(tiles.begin(), tiles.end(), [&](const InvTile& a, const InvTile& b) {
    const PoolSurface &A = P->surf[a.surf], &B = P->surf[b.surf];
    int ca = (A.p + 1) * (A.q + 1), cb = (B.p + 1) * (B.q + 1);
    if (ca != cb) return ca > cb;
    return a.count > b.count;
  });
  return NURBS_OK;
}

int workspace_for(nurbs_pool_t P, cudaStream_t st, size_t ntiles, Workspace*& out) {
  Workspace& w = P->ws[st];
  if (!w.ev) {
    if (cudaEventCreateWithFlags(&w.ev, cudaEventDisableTiming) != cudaSuccess)
      return pfail(NURBS_E_CUDA, "event creation failed");
  }
  if (w.cap_tiles < ntiles) {
    if (w.cap_tiles) {
      cudaStreamSynchronize(st);  // the previous list may still be read
      P->arena.release(w.off, 256 + w.cap_tiles * sizeof(InvTile));
      w.cap_tiles = 0;
    }
    size_t cap = std::max<size_t>(ntiles, 1024);
    if (!P->arena.alloc(256 + cap * sizeof(InvTile), w.off))
      return pfail(NURBS_E_BUDGET, "no room in the pool budget for a %zu-tile workspace", cap);
    w.cap_tiles = cap;
  }
  if (w.host_cap < ntiles) {
    cudaEventSynchronize(w.ev);
    if (w.host) cudaFreeHost(w.host);
    w.host = nullptr;
    size_t cap = std::max<size_t>(ntiles, 1024);
    if (cudaMallocHost((void**)&w.host, cap * sizeof(InvTile)) != cudaSuccess)
      return pfail(NURBS_E_NOMEM, "pinned allocation failed");
    w.host_cap = cap;
  }
  out = &w;
  return NURBS_OK;
}

int run_tiles(nurbs_pool_t P, const std::vector<InvTile>& tiles, const double* Pd, double* uv, int* st_out,
              double* res, int precision, cudaStream_t st, int ctas_per_sm, int tile_q) {
  if (tiles.empty()) return NURBS_OK;
  Workspace* w = nullptr;
  int rc = workspace_for(P, st, tiles.size(), w);
  if (rc) return rc;
  cudaEventSynchronize(w->ev);  // the pinned staging buffer is free again
  std::memcpy(w->host, tiles.data(), tiles.size() * sizeof(InvTile));
  char* dev = P->base + w->off;
  cudaError_t e = cudaMemcpyAsync(dev + 256, w->host, tiles.size() * sizeof(InvTile), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaEventRecord(w->ev, st);
  if (e == cudaSuccess)
    e = launch_invert_pool(P->d_table, (const InvTile*)(dev + 256), (int)tiles.size(), (int*)dev, Pd, uv, st_out, res,
                           precision, P->sms * ctas_per_sm, tile_q, st);
  if (e != cudaSuccess) return pfail(NURBS_E_CUDA, "pool inversion: %s", cudaGetErrorString(e));
  return NURBS_OK;
}

int check_batch_args(nurbs_pool_t P, int nbatch, const int* ids, const int64_t* offsets, const double* Pd, double* uv,
                     int* st, double* res, int precision) {
  if (!P) return pfail(NURBS_E_INVALID, "NULL pool");
  if (nbatch < 0 || (nbatch > 0 && (!ids || !offsets))) return pfail(NURBS_E_INVALID, "bad batch description");
  if (precision != NURBS_PREC_FP64 && precision != NURBS_PREC_MIXED) return pfail(NURBS_E_INVALID, "bad precision");
  if (nbatch > 0 && offsets[nbatch] > offsets[0] && (!Pd || !uv || !st || !res)) return pfail(NURBS_E_INVALID, "NULL buffer");
  return NURBS_OK;
}

std::string batch_key(nurbs_pool_t P, int nbatch, const int* ids, const int64_t* offsets, int precision) {
  cudaDeviceProp prop;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaGetDeviceProperties(&prop, dev);
  uint64_t h = 1469598103934665603ull;
  auto mix = [&](uint64_t v) {
    h ^= v;
    h *= 1099511628211ull;
  };
  int64_t total = 0;
  int64_t hist[8][8] = {};
  for (int k = 0; k < nbatch; ++k) {
    const PoolSurface& S = P->surf[ids[k]];
    int64_t c = offsets[k + 1] - offsets[k];
    total += c;
    hist[S.p][S.q] += c;
  }
  for (int a = 0; a < 8; ++a)
    for (int b = 0; b < 8; ++b) mix((uint64_t)hist[a][b]);
  std::ostringstream o;
  std::string name = prop.name;
  for (char& ch : name)
    if (ch == ' ') ch = '_';
  o << name << "/sm" << prop.multiProcessorCount << "/prec" << precision << "/n" << nbatch << "/q" << total << "/h"
    << std::hex << h;
  return o.str();
}

}  // namespace

// ---- internal entry points for the server (pool_internal.h)
namespace gnurbs {
bool pool_is_live(nurbs_pool_t P, int id) {
  std::lock_guard<std::mutex> lock(P->mu);
  return id >= 0 && id < (int)P->surf.size() && P->surf[id].live;
}
int pool_release_surface(nurbs_pool_t P, int id) {  // caller guarantees no queued work uses it
  std::lock_guard<std::mutex> lock(P->mu);
  if (id < 0 || id >= (int)P->surf.size() || !P->surf[id].live) return NURBS_E_INVALID;
  PoolSurface& s = P->surf[id];
  P->arena.release(s.in_off, s.in_bytes);
  P->arena.release(s.out_off, s.out_bytes);
  s = PoolSurface{};
  return NURBS_OK;
}
char* pool_arena_alloc(nurbs_pool_t P, size_t bytes, size_t* off) {
  std::lock_guard<std::mutex> lock(P->mu);
  if (!P->arena.alloc(bytes, *off)) return nullptr;
  return P->base + *off;
}
void pool_arena_release(nurbs_pool_t P, size_t off, size_t bytes) {
  std::lock_guard<std::mutex> lock(P->mu);
  P->arena.release(off, bytes);
}
}  // namespace gnurbs

extern "C" {

const char* nurbs_pool_last_error(void) { return g_pool_error.c_str(); }

int nurbs_pool_create(int64_t budget_bytes, int max_surfaces, nurbs_pool_t* out) {
  if (!out || budget_bytes <= 0 || max_surfaces <= 0) return pfail(NURBS_E_INVALID, "bad pool arguments");
  *out = nullptr;
  nurbs_pool_s* P = new (std::nothrow) nurbs_pool_s();
  if (!P) return pfail(NURBS_E_NOMEM, "host allocation failed");
  P->budget = align256((size_t)budget_bytes);
  if (cudaMalloc((void**)&P->base, P->budget) != cudaSuccess) {
    cudaGetLastError();
    delete P;
    return pfail(NURBS_E_NOMEM, "device allocation of the %lld-byte pool budget failed", (long long)budget_bytes);
  }
  if (cudaMalloc((void**)&P->d_table, sizeof(SurfDev) * (size_t)max_surfaces) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(P->base);
    delete P;
    return pfail(NURBS_E_NOMEM, "device allocation of the surface table failed");
  }
  P->arena.init(P->budget);
  P->max_surfaces = max_surfaces;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&P->sms, cudaDevAttrMultiProcessorCount, dev);
  *out = P;
  return NURBS_OK;
}

int nurbs_pool_destroy(nurbs_pool_t P) {
  if (!P) return NURBS_OK;
  cudaDeviceSynchronize();
  // graphs still alive lose their device resources now; nurbs_graph_destroy frees the rest
  for (nurbs_graph_s* G : P->graphs) {
    if (G->exec) cudaGraphExecDestroy(G->exec);
    if (G->graph) cudaGraphDestroy(G->graph);
    G->exec = nullptr;
    G->graph = nullptr;
    G->pool = nullptr;
  }
  for (auto& kv : P->ws) {
    if (kv.second.host) cudaFreeHost(kv.second.host);
    if (kv.second.ev) cudaEventDestroy(kv.second.ev);
  }
  cudaFree(P->d_table);
  cudaFree(P->base);
  delete P;
  return NURBS_OK;
}

int nurbs_pool_add(nurbs_pool_t P, int count, const nurbs_surface_desc* descs, void* stream, int* ids_out) {
  if (!P || count < 0 || (count > 0 && (!descs || !ids_out))) return pfail(NURBS_E_INVALID, "bad arguments");
  if (count == 0) return NURBS_OK;
  cudaStream_t st = (cudaStream_t)stream;
  // 1. host preparation (no lock)
  std::vector<SurfaceHost> S(count);
  std::string err;
  size_t in_total = 0;
  for (int k = 0; k < count; ++k) {
    const nurbs_surface_desc& d = descs[k];
    int rc = prepare_surface(d.degree_u, d.degree_v, d.cp_u, d.cp_v, d.knots_u, d.knots_v, d.cps, d.weights, S[k], err);
    if (rc) return pfail(rc, "surface %d: %s", k, err.c_str());
    in_total += S[k].in_bytes;
  }
  std::vector<BasisJob> bjobs;
  std::vector<SpanJob> sjobs;
  const size_t jb = align256(2 * (size_t)count * sizeof(BasisJob)), js = align256((size_t)count * sizeof(SpanJob));
  const size_t ji = align256((size_t)count * sizeof(int)), scratch_bytes = jb + js + ji;
  // 2. admission (locked): ids and arena blocks are reserved; the conversion runs unlocked so
  //    inversions of live surfaces proceed meanwhile
  std::vector<int> ids;
  size_t in_off = 0, scratch_off = 0;
  std::vector<size_t> out_off(count);
  {
    std::lock_guard<std::mutex> lock(P->mu);
    for (int id = 0; id < (int)P->surf.size() && (int)ids.size() < count; ++id)
      if (!P->surf[id].live && !P->surf[id].reserved) ids.push_back(id);
    int append = count - (int)ids.size();
    if ((int)P->surf.size() + append > P->max_surfaces)
      return pfail(NURBS_E_BUDGET, "the pool holds its maximum of %d surfaces", P->max_surfaces);
    if (!P->arena.alloc(in_total, in_off)) return pfail(NURBS_E_BUDGET, "no room in the pool budget for the batch");
    for (int k = 0; k < count; ++k) {
      if (!P->arena.alloc(S[k].out_bytes, out_off[k])) {
        for (int j = 0; j < k; ++j) P->arena.release(out_off[j], S[j].out_bytes);
        P->arena.release(in_off, in_total);
        return pfail(NURBS_E_BUDGET, "no room in the pool budget for surface %d of the batch", k);
      }
    }
    if (!P->arena.alloc(scratch_bytes, scratch_off)) {
      for (int j = 0; j < count; ++j) P->arena.release(out_off[j], S[j].out_bytes);
      P->arena.release(in_off, in_total);
      return pfail(NURBS_E_BUDGET, "no room in the pool budget for the conversion scratch");
    }
    for (int k = 0; k < append; ++k) {
      P->surf.emplace_back();
      ids.push_back((int)P->surf.size() - 1);
    }
    for (int id : ids) P->surf[id].reserved = true;
  }
  // 3. images, one copy, one launch per conversion stage (unlocked)
  std::vector<char> img(in_total, 0);
  std::vector<SurfDev> recs(count);
  int64_t bitems = 0, sitems = 0;
  size_t o = 0;
  for (int k = 0; k < count; ++k) {
    fill_surface(S[k], img.data() + o, P->base + in_off + o, P->base + out_off[k], recs[k]);
    const SurfDev& d = recs[k];
    bjobs.push_back(BasisJob{d.knots_u, d.knot_u, d.basis_u, d.p, d.ns_u, bitems});
    bitems += (int64_t)d.ns_u * (d.p + 1);
    bjobs.push_back(BasisJob{d.knots_v, d.knot_v, d.basis_v, d.q, d.ns_v, bitems});
    bitems += (int64_t)d.ns_v * (d.q + 1);
    sjobs.push_back(SpanJob{ids[k], sitems});
    sitems += (int64_t)d.ns_u * d.ns_v * 4;
    o += S[k].in_bytes;
  }
  std::vector<char> scr(scratch_bytes, 0);
  std::memcpy(scr.data(), bjobs.data(), bjobs.size() * sizeof(BasisJob));
  std::memcpy(scr.data() + jb, sjobs.data(), sjobs.size() * sizeof(SpanJob));
  std::memcpy(scr.data() + jb + js, ids.data(), ids.size() * sizeof(int));
  char* sdev = P->base + scratch_off;
  cudaError_t e = cudaMemcpyAsync(P->base + in_off, img.data(), in_total, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(sdev, scr.data(), scratch_bytes, cudaMemcpyHostToDevice, st);
  for (int k = 0; k < count && e == cudaSuccess; ++k)
    e = cudaMemcpyAsync(P->d_table + ids[k], &recs[k], sizeof(SurfDev), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = launch_basis_batched((const BasisJob*)sdev, (int)bjobs.size(), bitems, st);
  if (e == cudaSuccess)
    e = launch_span_matrices_batched(P->d_table, (const SpanJob*)(sdev + jb), (int)sjobs.size(), sitems, st);
  if (e == cudaSuccess) e = launch_tree_batched(P->d_table, (const int*)(sdev + jb + js), count, st);
  if (e == cudaSuccess) e = launch_centre_ders_batched(P->d_table, (const int*)(sdev + jb + js), count, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // host images must outlive the copies
  // 4. publication (locked)
  std::lock_guard<std::mutex> lock(P->mu);
  P->arena.release(scratch_off, scratch_bytes);
  if (e != cudaSuccess) {
    for (int j = 0; j < count; ++j) P->arena.release(out_off[j], S[j].out_bytes);
    P->arena.release(in_off, in_total);
    for (int id : ids) P->surf[id].reserved = false;
    return pfail(NURBS_E_CUDA, "pool conversion: %s", cudaGetErrorString(e));
  }
  o = 0;
  for (int k = 0; k < count; ++k) {
    PoolSurface& ps = P->surf[ids[k]];
    ps.live = true;
    ps.reserved = false;
    // the batch's input region is released piecewise: each surface owns its slice
    ps.in_off = in_off + o;
    ps.in_bytes = S[k].in_bytes;
    ps.out_off = out_off[k];
    ps.out_bytes = S[k].out_bytes;
    ps.p = S[k].p;
    ps.q = S[k].q;
    ps.spans = (int64_t)recs[k].ns_u * recs[k].ns_v;
    ids_out[k] = ids[k];
    o += S[k].in_bytes;
  }
  return NURBS_OK;
}

int nurbs_pool_remove(nurbs_pool_t P, int id, void* stream) {
  if (!P) return pfail(NURBS_E_INVALID, "NULL pool");
  std::lock_guard<std::mutex> lock(P->mu);
  if (id < 0 || id >= (int)P->surf.size() || !P->surf[id].live) return pfail(NURBS_E_INVALID, "surface id %d not in the pool", id);
  // work already queued on the stream may still read the surface
  cudaStreamSynchronize((cudaStream_t)stream);
  PoolSurface& s = P->surf[id];
  P->arena.release(s.in_off, s.in_bytes);
  P->arena.release(s.out_off, s.out_bytes);
  s = PoolSurface{};
  return NURBS_OK;
}

int nurbs_pool_info(nurbs_pool_t P, nurbs_pool_info_t* info) {
  if (!P || !info) return pfail(NURBS_E_INVALID, "NULL argument");
  std::lock_guard<std::mutex> lock(P->mu);
  info->budget_bytes = (int64_t)P->budget;
  info->used_bytes = (int64_t)P->arena.used();
  int live = 0;
  for (auto& s : P->surf) live += s.live;
  info->surfaces = live;
  info->max_surfaces = P->max_surfaces;
  info->tile_queries = P->tile_queries;
  info->ctas_per_sm = P->ctas_per_sm;
  return NURBS_OK;
}

int nurbs_pool_surface_bytes(int p, int q, int nu, int nv, const double* ku, const double* kv, int64_t* bytes) {
  if (!bytes || !ku || !kv) return pfail(NURBS_E_INVALID, "NULL argument");
  std::vector<double> cps((size_t)nu * nv * 3, 0.0), w((size_t)nu * nv, 1.0);
  SurfaceHost S;
  std::string err;
  int rc = prepare_surface(p, q, nu, nv, ku, kv, cps.data(), w.data(), S, err);
  if (rc) return pfail(rc, "%s", err.c_str());
  *bytes = (int64_t)(align256(S.in_bytes) + align256(S.out_bytes));
  return NURBS_OK;
}

int nurbs_pool_set_config(nurbs_pool_t P, int tile_queries, int ctas_per_sm) {
  if (!P || tile_queries < 1 || (tile_queries > 32 && tile_queries % 32) || ctas_per_sm < 1 || ctas_per_sm > 16)
    return pfail(NURBS_E_INVALID, "tile_queries must be 1..32 (warp chunks) or a multiple of 32 (CTA tiles), "
                                  "ctas_per_sm in 1..16");
  std::lock_guard<std::mutex> lock(P->mu);
  P->tile_queries = tile_queries;
  P->ctas_per_sm = ctas_per_sm;
  return NURBS_OK;
}

int nurbs_pool_invert(nurbs_pool_t P, int nbatch, const int* ids, const int64_t* offsets, const double* Pd, double* uv,
                      int* st_out, double* res, int precision, void* stream) {
  int rc = check_batch_args(P, nbatch, ids, offsets, Pd, uv, st_out, res, precision);
  if (rc) return rc;
  std::lock_guard<std::mutex> lock(P->mu);
  std::vector<InvTile> tiles;
  if ((rc = make_tiles(P, nbatch, ids, offsets, P->tile_queries, tiles))) return rc;
  return run_tiles(P, tiles, Pd, uv, st_out, res, precision, (cudaStream_t)stream, P->ctas_per_sm, P->tile_queries);
}

int nurbs_pool_eval(nurbs_pool_t P, int nbatch, const int* ids, const int64_t* offsets, const double* uv, int64_t n,
                    unsigned mask, double* out, void* stream) {
  if (!P || nbatch < 0 || (nbatch > 0 && (!ids || !offsets))) return pfail(NURBS_E_INVALID, "bad batch description");
  if (mask == 0 || mask > 63u) return pfail(NURBS_E_INVALID, "mask outside 1..63");
  if (n > 0 && (!uv || !out)) return pfail(NURBS_E_INVALID, "NULL buffer");
  if (nbatch > 0 && offsets[nbatch] > n) return pfail(NURBS_E_INVALID, "offsets exceed n");
  std::lock_guard<std::mutex> lock(P->mu);
  std::vector<InvTile> tiles;
  int rc = make_tiles(P, nbatch, ids, offsets, 1024, tiles);  // evaluation tiles: one CTA each
  if (rc) return rc;
  if (tiles.empty()) return NURBS_OK;
  cudaStream_t st = (cudaStream_t)stream;
  Workspace* w = nullptr;
  if ((rc = workspace_for(P, st, tiles.size(), w))) return rc;
  cudaEventSynchronize(w->ev);
  std::memcpy(w->host, tiles.data(), tiles.size() * sizeof(InvTile));
  char* dev = P->base + w->off;
  cudaError_t e = cudaMemcpyAsync(dev + 256, w->host, tiles.size() * sizeof(InvTile), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaEventRecord(w->ev, st);
  if (e == cudaSuccess) e = launch_eval_pool(P->d_table, (const InvTile*)(dev + 256), (int)tiles.size(), uv, n, mask, out, st);
  if (e != cudaSuccess) return pfail(NURBS_E_CUDA, "pool evaluation: %s", cudaGetErrorString(e));
  return NURBS_OK;
}

int nurbs_pool_autotune(nurbs_pool_t P, int nbatch, const int* ids, const int64_t* offsets, const double* Pd,
                        double* uv, int* st_out, double* res, int precision, int64_t max_queries, const char* cache_path,
                        void* stream, int* best_tile, int* best_ctas, float* best_ms) {
  int rc = check_batch_args(P, nbatch, ids, offsets, Pd, uv, st_out, res, precision);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  // a prefix of the batch of at most max_queries queries
  int nb = nbatch;
  if (max_queries > 0) {
    nb = 0;
    while (nb < nbatch && offsets[nb + 1] - offsets[0] <= max_queries) ++nb;
    if (nb == 0) nb = 1;
  }
  std::string key;
  {
    std::lock_guard<std::mutex> lock(P->mu);
    key = batch_key(P, nb, ids, offsets, precision);
  }
  if (cache_path) {
    std::ifstream f(cache_path);
    std::string k;
    int t, c;
    float ms;
    while (f >> k >> t >> c >> ms)
      if (k == key) {
        nurbs_pool_set_config(P, t, c);
        if (best_tile) *best_tile = t;
        if (best_ctas) *best_ctas = c;
        if (best_ms) *best_ms = ms;
        return NURBS_OK;
      }
  }
  // above 32: CTA tiles (throughput); 32 and below: warp chunks (latency, small batches)
  const int tile_opts[] = {128, 256, 32, 16};
  const int cta_opts[] = {4, 5, 6};
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  int bt = P->tile_queries, bc = P->ctas_per_sm;
  for (int t : tile_opts)
    for (int c : cta_opts) {
      std::vector<InvTile> tiles;
      {
        std::lock_guard<std::mutex> lock(P->mu);
        if ((rc = make_tiles(P, nb, ids, offsets, t, tiles))) break;
      }
      float ms = 0, sum = 0;
      for (int rep = 0; rep < 3 && rc == NURBS_OK; ++rep) {  // first run warms up
        cudaEventRecord(e0, st);
        {
          std::lock_guard<std::mutex> lock(P->mu);
          rc = run_tiles(P, tiles, Pd, uv, st_out, res, precision, st, c, t);
        }
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep) sum += ms;
      }
      if (rc) break;
      if (sum / 2 < best) {
        best = sum / 2;
        bt = t;
        bc = c;
      }
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  nurbs_pool_set_config(P, bt, bc);
  if (best_tile) *best_tile = bt;
  if (best_ctas) *best_ctas = bc;
  if (best_ms) *best_ms = best;
  if (cache_path) {
    std::ofstream f(cache_path, std::ios::app);
    if (f) f << key << " " << bt << " " << bc << " " << best << "\n";
  }
  return NURBS_OK;
}

int nurbs_pool_graph_create(nurbs_pool_t P, int nbatch, const int* ids, const int64_t* offsets, const double* Pd,
                            double* uv, int* st_out, double* res, int precision, nurbs_graph_t* out) {
  if (!out) return pfail(NURBS_E_INVALID, "out is NULL");
  *out = nullptr;
  int rc = check_batch_args(P, nbatch, ids, offsets, Pd, uv, st_out, res, precision);
  if (rc) return rc;
  std::lock_guard<std::mutex> lock(P->mu);
  std::vector<InvTile> tiles;
  if ((rc = make_tiles(P, nbatch, ids, offsets, P->tile_queries, tiles))) return rc;
  nurbs_graph_s* G = new (std::nothrow) nurbs_graph_s();
  if (!G) return pfail(NURBS_E_NOMEM, "host allocation failed");
  G->pool = P;
  G->bytes = 256 + std::max<size_t>(tiles.size(), 1) * sizeof(InvTile);
  if (!P->arena.alloc(G->bytes, G->off)) {
    delete G;
    return pfail(NURBS_E_BUDGET, "no room in the pool budget for the graph's tile list");
  }
  char* dev = P->base + G->off;
  cudaStream_t cs;
  cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  if (e == cudaSuccess && !tiles.empty())
    e = cudaMemcpyAsync(dev + 256, tiles.data(), tiles.size() * sizeof(InvTile), cudaMemcpyHostToDevice, cs);
  if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
  if (e == cudaSuccess) e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    cudaError_t le = launch_invert_pool(P->d_table, (const InvTile*)(dev + 256), (int)tiles.size(), (int*)dev, Pd, uv,
                                        st_out, res, precision, P->sms * P->ctas_per_sm, P->tile_queries, cs);
    e = cudaStreamEndCapture(cs, &G->graph);
    if (le != cudaSuccess) e = le;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&G->exec, G->graph, 0);
  cudaStreamDestroy(cs);
  if (e != cudaSuccess) {
    if (G->graph) cudaGraphDestroy(G->graph);
    P->arena.release(G->off, G->bytes);
    delete G;
    return pfail(NURBS_E_CUDA, "graph capture: %s", cudaGetErrorString(e));
  }
  P->graphs.insert(G);
  *out = G;
  return NURBS_OK;
}

int nurbs_graph_launch(nurbs_graph_t G, void* stream) {
  if (!G) return pfail(NURBS_E_INVALID, "NULL graph");
  if (!G->pool) return pfail(NURBS_E_STATE, "the graph's pool was destroyed");
  cudaError_t e = cudaGraphLaunch(G->exec, (cudaStream_t)stream);
  if (e != cudaSuccess) return pfail(NURBS_E_CUDA, "graph launch: %s", cudaGetErrorString(e));
  return NURBS_OK;
}

int nurbs_graph_destroy(nurbs_graph_t G) {
  if (!G) return NURBS_OK;
  if (G->pool) {
    cudaDeviceSynchronize();
    if (G->exec) cudaGraphExecDestroy(G->exec);
    if (G->graph) cudaGraphDestroy(G->graph);
    std::lock_guard<std::mutex> lock(G->pool->mu);
    G->pool->arena.release(G->off, G->bytes);
    G->pool->graphs.erase(G);
  }
  delete G;
  return NURBS_OK;
}

}  // extern "C"
