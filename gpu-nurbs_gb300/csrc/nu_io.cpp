// .nu text format reader/writer (replaces readNu, src/main.cu:45-113).
//
// Grammar, as the reference scans it: lines whose first token is a tag; other lines
// (e.g. "** comment") are skipped.  In order:
//   NU <degree_u> <degree_v>
//   CP <cp_u> <cp_v>
//   KNu <degree_u+cp_u+1 knots>        (extra values on the line are ignored)
//   KNv <degree_v+cp_v+1 knots>
//   DP <x> <y> <z> <w>                 cp_u*cp_v lines, row-major i*cp_v + j
// Each tag is searched forward from the previous one.  Where the reference would loop
// forever on a missing tag (getline at EOF leaves the tag unchanged) or read garbage from a
// short line, this reader returns NURBS_E_PARSE.
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "gpu_nurbs.h"

namespace {

struct Lines {
  const char* p;
  const char* end;
  bool next(std::string& line) {
    if (p >= end) return false;
    const char* e = (const char*)memchr(p, '\n', (size_t)(end - p));
    if (!e) e = end;
    line.assign(p, (size_t)(e - p));
    p = e < end ? e + 1 : end;
    return true;
  }
};

void split(const std::string& s, std::vector<std::string>& tok) {
  tok.clear();
  size_t i = 0, n = s.size();
  while (i < n) {
    while (i < n && (s[i] == ' ' || s[i] == '\t' || s[i] == '\r')) ++i;
    size_t j = i;
    while (j < n && !(s[j] == ' ' || s[j] == '\t' || s[j] == '\r')) ++j;
    if (j > i) tok.emplace_back(s.substr(i, j - i));
    i = j;
  }
}

bool to_double(const std::string& t, double& v) {
  char* e = nullptr;
  errno = 0;
  v = strtod(t.c_str(), &e);
  return e && *e == '\0' && errno != ERANGE;
}
bool to_int(const std::string& t, int& v) {
  char* e = nullptr;
  long x = strtol(t.c_str(), &e, 10);
  if (!e || *e != '\0' || x < -1000000000L || x > 1000000000L) return false;
  v = (int)x;
  return true;
}

// Finds the next line tagged `tag`; returns its remaining tokens.
bool seek(Lines& L, const char* tag, std::vector<std::string>& rest) {
  std::string line;
  std::vector<std::string> tok;
  while (L.next(line)) {
    split(line, tok);
    if (!tok.empty() && tok[0] == tag) {
      rest.assign(tok.begin() + 1, tok.end());
      return true;
    }
  }
  return false;
}

thread_local char g_err[256];

}  // namespace

extern "C" {

void nurbs_nu_free(nurbs_nu_desc* d) {
  if (!d) return;
  free(d->knots_u);
  free(d->knots_v);
  free(d->cps);
  free(d->weights);
  memset(d, 0, sizeof(*d));
}

int nurbs_nu_parse(const char* text, int64_t len, nurbs_nu_desc* out) {
  if (!text || !out || len < 0) return NURBS_E_INVALID;
  memset(out, 0, sizeof(*out));
  Lines L{text, text + len};
  std::vector<std::string> r;
  int p, q, nu, nv;
  if (!seek(L, "NU", r) || r.size() < 2 || !to_int(r[0], p) || !to_int(r[1], q)) return NURBS_E_PARSE;
  if (!seek(L, "CP", r) || r.size() < 2 || !to_int(r[0], nu) || !to_int(r[1], nv)) return NURBS_E_PARSE;
  if (p < 1 || q < 1 || p > NURBS_MAX_DEGREE || q > NURBS_MAX_DEGREE || nu < p + 1 || nv < q + 1 ||
      (int64_t)nu * nv > (int64_t)1 << 28)
    return NURBS_E_PARSE;
  out->degree_u = p;
  out->degree_v = q;
  out->cp_u = nu;
  out->cp_v = nv;
  out->knots_u = (double*)malloc(sizeof(double) * (p + nu + 1));
  out->knots_v = (double*)malloc(sizeof(double) * (q + nv + 1));
  out->cps = (double*)malloc(sizeof(double) * 3 * (size_t)nu * nv);
  out->weights = (double*)malloc(sizeof(double) * (size_t)nu * nv);
  if (!out->knots_u || !out->knots_v || !out->cps || !out->weights) {
    nurbs_nu_free(out);
    return NURBS_E_NOMEM;
  }
  auto read_knots = [&](const char* tag, double* k, int n) {
    if (!seek(L, tag, r) || (int)r.size() < n) return false;
    for (int i = 0; i < n; ++i)
      if (!to_double(r[i], k[i])) return false;
    return true;
  };
  if (!read_knots("KNu", out->knots_u, p + nu + 1) || !read_knots("KNv", out->knots_v, q + nv + 1)) {
    nurbs_nu_free(out);
    return NURBS_E_PARSE;
  }
  for (int64_t k = 0; k < (int64_t)nu * nv; ++k) {
    double x, y, z, w;
    if (!seek(L, "DP", r) || r.size() < 4 || !to_double(r[0], x) || !to_double(r[1], y) || !to_double(r[2], z) ||
        !to_double(r[3], w)) {
      nurbs_nu_free(out);
      return NURBS_E_PARSE;
    }
    out->cps[3 * k] = x;
    out->cps[3 * k + 1] = y;
    out->cps[3 * k + 2] = z;
    out->weights[k] = w;
  }
  return NURBS_OK;
}

int nurbs_nu_read(const char* path, nurbs_nu_desc* out) {
  if (!path || !out) return NURBS_E_INVALID;
  FILE* f = fopen(path, "rb");
  if (!f) {
    snprintf(g_err, sizeof(g_err), "cannot open %s", path);
    return NURBS_E_IO;
  }
  std::string text;
  char buf[65536];
  size_t got;
  while ((got = fread(buf, 1, sizeof(buf), f)) > 0) text.append(buf, got);
  fclose(f);
  return nurbs_nu_parse(text.data(), (int64_t)text.size(), out);
}

int nurbs_nu_write(const char* path, const nurbs_nu_desc* d) {
  if (!path || !d || !d->knots_u || !d->knots_v || !d->cps || !d->weights) return NURBS_E_INVALID;
  FILE* f = fopen(path, "wb");
  if (!f) return NURBS_E_IO;
  const int p = d->degree_u, q = d->degree_v, nu = d->cp_u, nv = d->cp_v;
  fprintf(f, "** NURBS degree [2]\nNU %d %d\nCP %d %d\n\n** NURBS Knots\nKNu", p, q, nu, nv);
  for (int i = 0; i < p + nu + 1; ++i) fprintf(f, " %.17g", d->knots_u[i]);
  fprintf(f, "\nKNv");
  for (int i = 0; i < q + nv + 1; ++i) fprintf(f, " %.17g", d->knots_v[i]);
  fprintf(f, "\n\n** control points and weights [4]\n");
  for (int64_t k = 0; k < (int64_t)nu * nv; ++k)
    fprintf(f, "DP %.17g %.17g %.17g %.17g\n", d->cps[3 * k], d->cps[3 * k + 1], d->cps[3 * k + 2], d->weights[k]);
  int bad = ferror(f);
  if (fclose(f) != 0 || bad) return NURBS_E_IO;
  return NURBS_OK;
}

}  // extern "C"
