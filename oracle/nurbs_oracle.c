/*
 * CPU ORACLE — test infrastructure only (see nurbs_oracle.h).
 *
 * Plain-C restatement of the reference FP64 path.  Arithmetic follows the reference's
 * expression order term by term (and is compiled without FMA contraction) so that the
 * values match the reference's own functions bit for bit where the reference is
 * deterministic.  Two documented substitutions:
 *   - pow(h,2) is h*h (IEEE-exact rounding of the square) and pow(h,3) is orc_cube(h),
 *     the once-rounded cube; both equal a correctly rounded pow.
 *   - the tree's block max/min reductions are done sequentially; max/min are exact, so
 *     only the sign of a zero could differ from the reference's shared-memory tree.
 */
#include "nurbs_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---------------------------------------------------------------- small helpers */

double orc_cube(double x) {
    /* x^2 = a + b exactly (Dekker/Ogita-Rump-Oishi TwoProduct via fma). */
    double a = x * x;
    double b = fma(x, x, -a);
    /* a*x = c + d exactly; b*x is ~2^-53 of the result, so its own rounding is ~2^-106. */
    double c = a * x;
    double d = fma(a, x, -c);
    double e = b * x;
    return c + (d + e);
}

static double sq(double x) { return x * x; }

int64_t orc_matrix_n_position(int i, int j, int degree_u, int degree_v, int cp_u, int cp_v, int c) {
    /* MatrixNPosition, src/NURBS/Evaluate.cu:110-112 */
    (void)cp_u;
    int64_t k12 = (int64_t)(degree_u + 1) * (degree_v + 1);
    return (((int64_t)i * (degree_v + cp_v) + j) * 4 + c) * k12;
}

int64_t orc_matrix_n_size(const orc_surface* s) {
    /* cudaMalloc size of MatrixN, src/main.cu:182 */
    return (int64_t)(s->degree_u + s->cp_u) * (s->degree_v + s->cp_v) * 4 *
           (s->degree_u + 1) * (s->degree_v + 1);
}

int orc_find_span(int degree, int cp, const double* knots, double u) {
    /* findSpan, src/NURBS/Evaluate.cu:504-533 */
    int n = cp - 1;
    if (u >= knots[n + 1]) return n;
    if (u <= knots[degree]) return degree;
    int low = degree, high = n + 1;
    int mid = (int)((low + high) / 2.0);
    while (u < knots[mid] || u >= knots[mid + 1]) {
        if (u < knots[mid]) high = mid; else low = mid;
        mid = (int)((low + high) / 2.0);
    }
    return mid;
}

/* ------------------------------------------------- stage a: span matrices (GetMatrixN) */

/* Nabla(knot, d, i, k) = knot[i+d-1+k] - knot[i+d-1]   (Evaluate.cu:105-108) */
static double nabla(const double* knot, int d, int i, int k) {
    int index = i + d - 1;
    return knot[index + k] - knot[index];
}

/* Basis-to-power matrix of one span: N[r][c] = Nrc(knot, d, r+1, c+1, I, I, d) with
 * I = span - (d-1) (Evaluate.cu:16-20).  Nrc (Evaluate.cu:90-103) is a pure function of
 * (m, r, c, j); it is tabulated bottom-up over m so each state is computed once, with the
 * reference's expression for every state, which gives the same values as the recursion. */
static void span_basis_matrix(const double* knot, int d, int span, double* N /* (d+1)^2 */) {
    const int I = span - (d - 1);
    const int R0 = 1 - d, RN = 2 * d + 1;     /* r in [1-d, d+1] */
    const int J0 = I - d, JN = d + 1;         /* j in [I-d, I]   */
    double prev[(2 * ORC_MAX_DEGREE + 1) * (ORC_MAX_DEGREE + 1)];
    double cur[(2 * ORC_MAX_DEGREE + 1) * (ORC_MAX_DEGREE + 1)];
    for (int c = 1; c <= d + 1; ++c) {
        /* m = 0 (Evaluate.cu:91-95) */
        for (int ri = 0; ri < RN; ++ri)
            for (int ji = 0; ji < JN; ++ji) {
                int r = R0 + ri, j = J0 + ji;
                prev[ri * JN + ji] = (((I + c - 1) == (j + d)) && (r == 1)) ? 1.0 : 0.0;
            }
        for (int m = 1; m <= d; ++m) {
            /* states reachable at depth m: j in [I-(d-m), I], r in [1-(d-m), d+1] */
            for (int ri = 0; ri < RN; ++ri)
                for (int ji = 0; ji < JN; ++ji) cur[ri * JN + ji] = 0.0;
            for (int r = 1 - (d - m); r <= d + 1; ++r) {
                int ri = r - R0;
                for (int j = I - (d - m); j <= I; ++j) {
                    int ji = j - J0;
                    /* ri-1 >= 0 and ji-1 >= 0 hold on the reachable set */
                    double n1 = prev[(ri - 1) * JN + ji];       /* Nrc(m-1, r-1, c, j)   */
                    double n2 = prev[ri * JN + ji];             /* Nrc(m-1, r,   c, j)   */
                    double n3 = prev[ri * JN + (ji - 1)];       /* Nrc(m-1, r,   c, j-1) */
                    double n4 = prev[(ri - 1) * JN + (ji - 1)]; /* Nrc(m-1, r-1, c, j-1) */
                    double A = nabla(knot, d, I, 1);
                    double B = nabla(knot, d, j, d - m + 1);
                    double C = nabla(knot, d, j, I - j);
                    cur[ri * JN + ji] = A / B * n1 + C / B * n2 + (1 - C / B) * n3 + (-A / B) * n4;
                }
            }
            memcpy(prev, cur, sizeof(double) * RN * JN);
        }
        for (int r = 1; r <= d + 1; ++r) N[(r - 1) * (d + 1) + (c - 1)] = prev[(r - R0) * JN + (I - J0)];
    }
}

/* matrix_mult (src/util/Matrix.cu:43-52): c[i][j] = sum over l ascending, from 0. */
static void mat_mult(const double* a, const double* b, double* c, int m, int n, int k) {
    for (int i = 0; i < m; i++)
        for (int j = 0; j < k; j++) {
            double acc = 0;
            for (int l = 0; l < n; l++) acc += a[i * n + l] * b[l * k + j];
            c[i * k + j] = acc;
        }
}

int orc_matrix_n(const orc_surface* s, double* matrix_n) {
    const int p = s->degree_u, q = s->degree_v, k1 = p + 1, k2 = q + 1;
    const int nu = s->cp_u, nv = s->cp_v;
    if (p < 1 || q < 1 || p > ORC_MAX_DEGREE || q > ORC_MAX_DEGREE || nu < p + 1 || nv < q + 1) return -1;
    double* Nu = (double*)malloc(sizeof(double) * k1 * k1 * (nu));
    double* Nv = (double*)malloc(sizeof(double) * k2 * k2 * (nv));
    /* Nu depends on i only and Nv on j only: compute each once (the reference recomputes
     * them per (i,j) thread, with identical results). */
    for (int i = p; i < nu; ++i)
        if (s->knots_u[i] != s->knots_u[i + 1]) span_basis_matrix(s->knots_u, p, i, Nu + (size_t)i * k1 * k1);
    for (int j = q; j < nv; ++j)
        if (s->knots_v[j] != s->knots_v[j + 1]) span_basis_matrix(s->knots_v, q, j, Nv + (size_t)j * k2 * k2);
    int written = 0;
    double mid[4][(ORC_MAX_DEGREE + 1) * (ORC_MAX_DEGREE + 1)];
    double tmp[(ORC_MAX_DEGREE + 1) * (ORC_MAX_DEGREE + 1)];
    double nvt[(ORC_MAX_DEGREE + 1) * (ORC_MAX_DEGREE + 1)];
    for (int i = p; i < nu; ++i) {
        if (s->knots_u[i] == s->knots_u[i + 1]) continue;   /* Evaluate.cu:10-11 */
        for (int j = q; j < nv; ++j) {
            if (s->knots_v[j] == s->knots_v[j + 1]) continue;
            const double* nvm = Nv + (size_t)j * k2 * k2;
            for (int m = 0; m < k2; ++m)          /* NvT[n][m] = Nv[m][n]  (Evaluate.cu:24-28) */
                for (int n = 0; n < k2; ++n) nvt[n * k2 + m] = nvm[m * k2 + n];
            for (int a = 0; a <= p; ++a)          /* Middle_c = P_c * w  (Evaluate.cu:35-43) */
                for (int b = 0; b <= q; ++b) {
                    size_t idx = (size_t)(a + i - p) * nv + (b + j - q);
                    double w = s->weights[idx];
                    mid[0][a * k2 + b] = s->cps[3 * idx + 0] * w;
                    mid[1][a * k2 + b] = s->cps[3 * idx + 1] * w;
                    mid[2][a * k2 + b] = s->cps[3 * idx + 2] * w;
                    mid[3][a * k2 + b] = w;
                }
            for (int c = 0; c < 4; ++c) {         /* temp = Middle*NvT ; out = Nu*temp  (:58-66) */
                mat_mult(mid[c], nvt, tmp, k1, k2, k2);
                mat_mult(Nu + (size_t)i * k1 * k1, tmp,
                         matrix_n + orc_matrix_n_position(i, j, p, q, nu, nv, c), k1, k1, k2);
            }
            ++written;
        }
    }
    free(Nu);
    free(Nv);
    return written;
}

/* ------------------------------------------------------------- stage b: evaluation */

typedef struct { double x, y, z, w; } d4;
typedef struct { double x, y, z; } d3;

static void power_vec(double t, int k, double* out) {      /* [1, t, t^2, ...] running product */
    double now = 1;
    for (int i = 0; i < k; i++) { out[i] = now; now *= t; }
}
static void dpower_vec(double t, int k, double* out) {     /* Evaluate.cu:540-545 */
    double now = 1;
    out[0] = 0;
    for (int i = 0; i < k - 1; i++) { out[i + 1] = (i + 1) * now; now *= t; }
}
static void ddpower_vec(double t, int k, double* out) {    /* Evaluate.cu:680-685 */
    double now = 1;
    out[0] = 0;
    if (k > 1) out[1] = 0;
    for (int i = 0; i < k - 2; i++) { out[i + 2] = (i + 2) * (i + 1) * now; now *= t; }
}

/* temp_c = M_c * vec (k1 rows), then r.c = uvec . temp_c  (matrix_mult order) */
static void mv4(const double* middle, int k1, int k2, const double* vec, double tmp[4][8]) {
    for (int c = 0; c < 4; ++c) mat_mult(middle + c * k1 * k2, vec, tmp[c], k1, k2, 1);
}
static d4 dot4(const double* uvec, int k1, double tmp[4][8]) {
    d4 r;
    mat_mult(uvec, tmp[0], &r.x, 1, k1, 1);
    mat_mult(uvec, tmp[1], &r.y, 1, k1, 1);
    mat_mult(uvec, tmp[2], &r.z, 1, k1, 1);
    mat_mult(uvec, tmp[3], &r.w, 1, k1, 1);
    return r;
}

void orc_point_r(const double* middle, int p, int q, double u, double v, double R[4]) {
    /* MatrixSurfacePoint, Evaluate.cu:159-227 */
    int k1 = p + 1, k2 = q + 1;
    double U[8], V[8], tmp[4][8];
    power_vec(u, k1, U);
    power_vec(v, k2, V);
    mv4(middle, k1, k2, V, tmp);
    d4 r = dot4(U, k1, tmp);
    R[0] = r.x; R[1] = r.y; R[2] = r.z; R[3] = r.w;
}

static d4 R_of(const double* middle, int p, int q, double u, double v) {
    double R[4];
    orc_point_r(middle, p, q, u, v, R);
    d4 r = {R[0], R[1], R[2], R[3]};
    return r;
}

/* old MatrixSurfaceDerivativeU, Evaluate.cu:535-598 */
static d3 der_u(const double* middle, int p, int q, double u, double v, d4 R, double spanU) {
    int k1 = p + 1, k2 = q + 1;
    double dU[8], V[8], tmp[4][8];
    dpower_vec(u, k1, dU);
    power_vec(v, k2, V);
    mv4(middle, k1, k2, V, tmp);
    d4 RdU = dot4(dU, k1, tmp);
    double h = R.w, hdU = RdU.w;
    double s = -hdU / sq(h);
    d3 o;
    o.x = (R.x * s + RdU.x / h) * spanU;
    o.y = (R.y * s + RdU.y / h) * spanU;
    o.z = (R.z * s + RdU.z / h) * spanU;
    return o;
}

/* old MatrixSurfaceDerivativeV, Evaluate.cu:600-665 */
static d3 der_v(const double* middle, int p, int q, double u, double v, d4 R, double spanV) {
    int k1 = p + 1, k2 = q + 1;
    double U[8], dV[8], tmp[4][8];
    power_vec(u, k1, U);
    dpower_vec(v, k2, dV);
    mv4(middle, k1, k2, dV, tmp);
    d4 RdV = dot4(U, k1, tmp);
    double h = R.w, hdV = RdV.w;
    double s = -hdV / sq(h);
    d3 o;
    o.x = (R.x * s + RdV.x / h) * spanV;
    o.y = (R.y * s + RdV.y / h) * spanV;
    o.z = (R.z * s + RdV.z / h) * spanV;
    return o;
}

/* old MatrixSurfaceDerivativeUU, Evaluate.cu:667-741 */
static d3 der_uu(const double* middle, int p, int q, double u, double v, d4 R, double spanU) {
    int k1 = p + 1, k2 = q + 1;
    double dU[8], ddU[8], V[8], tmp[4][8];
    dpower_vec(u, k1, dU);
    ddpower_vec(u, k1, ddU);
    power_vec(v, k2, V);
    mv4(middle, k1, k2, V, tmp);
    d4 RdU = dot4(dU, k1, tmp);
    d4 RdUU = dot4(ddU, k1, tmp);
    double h = R.w, hdU = RdU.w, hdUU = RdUU.w;
    double s1 = (2 * sq(hdU) / orc_cube(h)) - (hdUU / sq(h));
    double s2 = -hdU / sq(h);
    d3 o;
    o.x = ((R.x * s1 + (2 * RdU.x) * s2) + RdUU.x / h) * spanU * spanU;
    o.y = ((R.y * s1 + (2 * RdU.y) * s2) + RdUU.y / h) * spanU * spanU;
    o.z = ((R.z * s1 + (2 * RdU.z) * s2) + RdUU.z / h) * spanU * spanU;
    return o;
}

/* old MatrixSurfaceDerivativeUV, Evaluate.cu:743-847 */
static d3 der_uv(const double* middle, int p, int q, double u, double v, d4 R, double spanU, double spanV) {
    int k1 = p + 1, k2 = q + 1;
    double U[8], dU[8], V[8], dV[8], tmp[4][8];
    power_vec(u, k1, U);
    dpower_vec(u, k1, dU);
    power_vec(v, k2, V);
    dpower_vec(v, k2, dV);
    mv4(middle, k1, k2, V, tmp);
    d4 RdU = dot4(dU, k1, tmp);
    mv4(middle, k1, k2, dV, tmp);
    d4 RdV = dot4(U, k1, tmp);
    d4 RdUV = dot4(dU, k1, tmp);
    double h = R.w, hdU = RdU.w, hdV = RdV.w, hdUV = RdUV.w;
    double h2 = sq(h), h3 = orc_cube(h);
    d3 o;
    o.x = ((((RdUV.x * h - hdV * RdU.x) - RdV.x * hdU) - R.x * hdUV) / h2 + ((2 * R.x) * hdU * hdV) / h3) * spanU * spanV;
    o.y = ((((RdUV.y * h - hdV * RdU.y) - RdV.y * hdU) - R.y * hdUV) / h2 + ((2 * R.y) * hdU * hdV) / h3) * spanU * spanV;
    o.z = ((((RdUV.z * h - hdV * RdU.z) - RdV.z * hdU) - R.z * hdUV) / h2 + ((2 * R.z) * hdU * hdV) / h3) * spanU * spanV;
    return o;
}

/* old MatrixSurfaceDerivativeVV, Evaluate.cu:849-930 (contracts U first: temp = U^T M) */
static d3 der_vv(const double* middle, int p, int q, double u, double v, d4 R, double spanV) {
    int k1 = p + 1, k2 = q + 1;
    double U[8], dV[8], ddV[8], tmp[4][8];
    power_vec(u, k1, U);
    dpower_vec(v, k2, dV);
    ddpower_vec(v, k2, ddV);
    for (int c = 0; c < 4; ++c) mat_mult(U, middle + c * k1 * k2, tmp[c], 1, k1, k2);
    d4 RdV, RdVV;
    mat_mult(tmp[0], dV, &RdV.x, 1, k2, 1);
    mat_mult(tmp[1], dV, &RdV.y, 1, k2, 1);
    mat_mult(tmp[2], dV, &RdV.z, 1, k2, 1);
    mat_mult(tmp[3], dV, &RdV.w, 1, k2, 1);
    mat_mult(tmp[0], ddV, &RdVV.x, 1, k2, 1);
    mat_mult(tmp[1], ddV, &RdVV.y, 1, k2, 1);
    mat_mult(tmp[2], ddV, &RdVV.z, 1, k2, 1);
    mat_mult(tmp[3], ddV, &RdVV.w, 1, k2, 1);
    double h = R.w, hdV = RdV.w, hdVV = RdVV.w;
    double s1 = (2 * sq(hdV) / orc_cube(h)) - (hdVV / sq(h));
    double s2 = -hdV / sq(h);
    d3 o;
    o.x = ((R.x * s1 + (2 * RdV.x) * s2) + RdVV.x / h) * spanV * spanV;
    o.y = ((R.y * s1 + (2 * RdV.y) * s2) + RdVV.y / h) * spanV * spanV;
    o.z = ((R.z * s1 + (2 * RdV.z) * s2) + RdVV.z / h) * spanV * spanV;
    return o;
}

typedef struct {
    const double* middle;
    double u, v;           /* local parameters in [0,1] of the span */
    double spanU, spanV;   /* derivative scale (kernel.cu:167-168) */
} span_loc;

/* findSpan + local parameter + MatrixNPosition as in EvaluateRandom (Evaluate.cu:1029-1034)
 * and GaussNewton (kernel.cu:161-169). */
static span_loc locate(const orc_surface* s, const double* M, double uu, double vv) {
    const int p = s->degree_u, q = s->degree_v;
    const double* ku = s->knots_u;
    const double* kv = s->knots_v;
    int m = orc_find_span(p, s->cp_u, ku, uu);
    int n = orc_find_span(q, s->cp_v, kv, vv);
    span_loc L;
    L.u = (uu - ku[m]) / (ku[m + 1] - ku[m]);
    L.v = (vv - kv[n]) / (kv[n + 1] - kv[n]);
    L.spanU = (ku[p + s->cp_u] - ku[0]) / (ku[m + 1] - ku[m]);
    L.spanV = (kv[q + s->cp_v] - kv[0]) / (kv[n + 1] - kv[n]);
    L.middle = M + orc_matrix_n_position(m, n, p, q, s->cp_u, s->cp_v, 0);
    return L;
}

static d3 cart(d4 R) {     /* homogenousToCartesian, src/util/ExtraMath.cu:3-5 */
    d3 o = {R.x / R.w, R.y / R.w, R.z / R.w};
    return o;
}

static d3 d3at(const double* a, int b) { d3 o = {a[3 * b], a[3 * b + 1], a[3 * b + 2]}; return o; }
static d3 d3add(d3 a, d3 b) { d3 o = {a.x + b.x, a.y + b.y, a.z + b.z}; return o; }
static d3 d3scale(double s, d3 a) { d3 o = {s * a.x, s * a.y, s * a.z}; return o; }

void orc_eval(const orc_surface* s, const double* M, const double* uv, int64_t n, unsigned mask,
              double* out, int threads) {
    const int p = s->degree_u, q = s->degree_v;
    int nblk = 0;
    for (int b = 0; b < 6; ++b) nblk += (mask >> b) & 1u;
    (void)nblk;
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(threads)
#endif
    for (int64_t k = 0; k < n; ++k) {
        span_loc L = locate(s, M, uv[2 * k], uv[2 * k + 1]);
        d4 R = R_of(L.middle, p, q, L.u, L.v);
        d3 blk[10];
        if (mask & 0x3C0u) {
            double d[30];
            orc_ders3(s, M, uv[2 * k], uv[2 * k + 1], d);
            for (int b3 = 6; b3 < 10; ++b3) blk[b3] = d3at(d, b3);
        }
        if (mask & ORC_S) blk[0] = cart(R);
        if (mask & ORC_SU) blk[1] = der_u(L.middle, p, q, L.u, L.v, R, L.spanU);
        if (mask & ORC_SV) blk[2] = der_v(L.middle, p, q, L.u, L.v, R, L.spanV);
        if (mask & ORC_SUU) blk[3] = der_uu(L.middle, p, q, L.u, L.v, R, L.spanU);
        if (mask & ORC_SUV) blk[4] = der_uv(L.middle, p, q, L.u, L.v, R, L.spanU, L.spanV);
        if (mask & ORC_SVV) blk[5] = der_vv(L.middle, p, q, L.u, L.v, R, L.spanV);
        int o = 0;
        for (int b = 0; b < 10; ++b) {
            if (!((mask >> b) & 1u)) continue;
            out[(3 * o + 0) * n + k] = blk[b].x;
            out[(3 * o + 1) * n + k] = blk[b].y;
            out[(3 * o + 2) * n + k] = blk[b].z;
            ++o;
        }
    }
}


/* ------------------------------------------- third order and normals (new-style quotient rule)
 *
 * The reference's projection code (src/kernel/kernel.cu:1386-1560, src/NURBS/Evaluate.cu:
 * 288-502, 932-1020) forms every derivative from the homogeneous R-derivatives: power vectors
 * and their derivatives (GetVector, kernel.cu:1386-1450: d^k vectors as (i+k)...(i+1) * U[i]),
 * R^(a,b) = U^(a) . (M_c . V^(b)) scaled by spanU^a spanV^b (MatrixSurfaceRd*), then
 * S = R.xyz / h and the quotient rule applied to derivatives already computed.  Its mixed third
 * derivatives (Evaluate.cu:963-1020) add 2 h_uv S_u and h_uuv S where the rule subtracts them (the
 * same defect as its new S_uv, D1); here the rule's signs:
 *   S_uv  = (R_uv  - h_v S_u  - h_u S_v  - h_uv S) / h
 *   S_uuv = (R_uuv - h_v S_uu - 2 h_u S_uv - 2 h_uv S_u - h_uu S_v - h_uuv S) / h
 *   S_uvv = (R_uvv - h_u S_vv - 2 h_v S_uv - 2 h_uv S_v - h_vv S_u - h_uvv S) / h
 * Normal N = S_u x S_v (getNormals, kernel.cu:1043-1058) and SurfaceNormalDerivative{UU,UV,VV}
 * (Evaluate.cu:1125-1135); first derivatives N_u = S_uu x S_v + S_u x S_uv, N_v likewise. */

static void vectors_k(double t, int k, double* V0, double* V1, double* V2, double* V3) {
    double now = 1;
    for (int i = 0; i < k; i++) { V0[i] = now; now *= t; }
    V1[0] = 0;
    for (int i = 0; i < k - 1; i++) V1[i + 1] = (i + 1) * V0[i];
    V2[0] = 0;
    if (k > 1) V2[1] = 0;
    for (int i = 0; i < k - 2; i++) V2[i + 2] = (i + 2) * (i + 1) * V0[i];
    V3[0] = 0;
    if (k > 1) V3[1] = 0;
    if (k > 2) V3[2] = 0;
    for (int i = 0; i < k - 3; i++) V3[i + 3] = (i + 3) * (i + 2) * (i + 1) * V0[i];
}

static d4 rd(const double* middle, int k1, int k2, const double* vu, const double* vv) {
    double tmp[4][8];
    mv4(middle, k1, k2, vv, tmp);
    return dot4(vu, k1, tmp);
}
/* the same contracting u first (MatrixSurfaceRdVV, Evaluate.cu:384-405) */
static d4 rd_ufirst(const double* middle, int k1, int k2, const double* vu, const double* vv) {
    double tmp[4][8];
    d4 r;
    for (int c = 0; c < 4; ++c) mat_mult(vu, middle + c * k1 * k2, tmp[c], 1, k1, k2);
    mat_mult(tmp[0], vv, &r.x, 1, k2, 1);
    mat_mult(tmp[1], vv, &r.y, 1, k2, 1);
    mat_mult(tmp[2], vv, &r.z, 1, k2, 1);
    mat_mult(tmp[3], vv, &r.w, 1, k2, 1);
    return r;
}
static d4 d4s(d4 a, double s) { d4 o = {a.x * s, a.y * s, a.z * s, a.w * s}; return o; }
static d3 cross3(d3 a, d3 b) {   /* cross_product, src/util/Matrix.cu:62-64 */
    d3 o = {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
    return o;
}

/* S and its derivatives to third order at (uu, vv): out[0..9] = S, Su, Sv, Suu, Suv, Svv, Suuu,
 * Suuv, Suvv, Svvv. */
void orc_ders3(const orc_surface* s, const double* M, double uu, double vv, double out[30]) {
    const int p = s->degree_u, q = s->degree_v, k1 = p + 1, k2 = q + 1;
    span_loc L = locate(s, M, uu, vv);
    double U[4][8], V[4][8];
    vectors_k(L.u, k1, U[0], U[1], U[2], U[3]);
    vectors_k(L.v, k2, V[0], V[1], V[2], V[3]);
    const double su = L.spanU, sv = L.spanV;
    d4 R = rd(L.middle, k1, k2, U[0], V[0]);
    d4 Ru = d4s(rd(L.middle, k1, k2, U[1], V[0]), su);
    d4 Rv = d4s(rd(L.middle, k1, k2, U[0], V[1]), sv);
    d4 Ruu = d4s(d4s(rd(L.middle, k1, k2, U[2], V[0]), su), su);
    d4 Ruv = d4s(d4s(rd(L.middle, k1, k2, U[1], V[1]), su), sv);
    d4 Rvv = d4s(d4s(rd_ufirst(L.middle, k1, k2, U[0], V[2]), sv), sv);
    d4 Ruuu = d4s(d4s(d4s(rd(L.middle, k1, k2, U[3], V[0]), su), su), su);
    d4 Ruuv = d4s(d4s(d4s(rd(L.middle, k1, k2, U[2], V[1]), su), su), sv);
    d4 Ruvv = d4s(d4s(d4s(rd(L.middle, k1, k2, U[1], V[2]), su), sv), sv);
    d4 Rvvv = d4s(d4s(d4s(rd(L.middle, k1, k2, U[0], V[3]), sv), sv), sv);
    const double h = R.w, hu = Ru.w, hv = Rv.w, huu = Ruu.w, huv = Ruv.w, hvv = Rvv.w;
    d3 S = cart(R), Su, Sv, Suu, Suv, Svv, Suuu, Suuv, Suvv, Svvv;
#define ORC_Q(o, expr) do { double* oo = &(o).x; for (int c = 0; c < 3; ++c) oo[c] = (expr); } while (0)
#define CMP(a) (((const double*)&(a))[c])
    ORC_Q(Su, (CMP(Ru) - hu * CMP(S)) / h);
    ORC_Q(Sv, (CMP(Rv) - hv * CMP(S)) / h);
    ORC_Q(Suu, ((CMP(Ruu) - 2 * hu * CMP(Su)) - huu * CMP(S)) / h);
    ORC_Q(Suv, (((CMP(Ruv) - hv * CMP(Su)) - hu * CMP(Sv)) - huv * CMP(S)) / h);
    ORC_Q(Svv, ((CMP(Rvv) - 2 * hv * CMP(Sv)) - hvv * CMP(S)) / h);
    ORC_Q(Suuu, (((CMP(Ruuu) - 3 * hu * CMP(Suu)) - 3 * huu * CMP(Su)) - Ruuu.w * CMP(S)) / h);
    ORC_Q(Suuv, (((((CMP(Ruuv) - hv * CMP(Suu)) - 2 * hu * CMP(Suv)) - 2 * huv * CMP(Su)) - huu * CMP(Sv)) -
                 Ruuv.w * CMP(S)) / h);
    ORC_Q(Suvv, (((((CMP(Ruvv) - hu * CMP(Svv)) - 2 * hv * CMP(Suv)) - 2 * huv * CMP(Sv)) - hvv * CMP(Su)) -
                 Ruvv.w * CMP(S)) / h);
    ORC_Q(Svvv, (((CMP(Rvvv) - 3 * hv * CMP(Svv)) - 3 * hvv * CMP(Sv)) - Rvvv.w * CMP(S)) / h);
#undef CMP
#undef ORC_Q
    const d3 all[10] = {S, Su, Sv, Suu, Suv, Svv, Suuu, Suuv, Suvv, Svvv};
    for (int b = 0; b < 10; ++b) {
        out[3 * b] = all[b].x;
        out[3 * b + 1] = all[b].y;
        out[3 * b + 2] = all[b].z;
    }
}


/* N, N_u, N_v, N_uu, N_uv, N_vv from the third-order derivatives d[30] (see above). */
static void normals_of(const double d[30], double out[18]) {
    const d3 Su = d3at(d, 1), Sv = d3at(d, 2), Suu = d3at(d, 3), Suv = d3at(d, 4), Svv = d3at(d, 5);
    const d3 Suuu = d3at(d, 6), Suuv = d3at(d, 7), Suvv = d3at(d, 8), Svvv = d3at(d, 9);
    const d3 N[6] = {
        cross3(Su, Sv),
        d3add(cross3(Suu, Sv), cross3(Su, Suv)),
        d3add(cross3(Suv, Sv), cross3(Su, Svv)),
        d3add(d3add(cross3(Suuu, Sv), d3scale(2, cross3(Suu, Suv))), cross3(Su, Suuv)),
        d3add(d3add(d3add(cross3(Suuv, Sv), cross3(Suu, Svv)), cross3(Suv, Suv)), cross3(Su, Suvv)),
        d3add(d3add(cross3(Suvv, Sv), d3scale(2, cross3(Suv, Svv))), cross3(Su, Svvv))};
    for (int b = 0; b < 6; ++b) {
        out[3 * b] = N[b].x;
        out[3 * b + 1] = N[b].y;
        out[3 * b + 2] = N[b].z;
    }
}

void orc_normals(const orc_surface* s, const double* M, double uu, double vv, double out[18]) {
    double d[30];
    orc_ders3(s, M, uu, vv, d);
    normals_of(d, out);
}

void orc_eval_normal(const orc_surface* s, const double* M, const double* uv, int64_t n, unsigned mask,
                     double* out, int threads) {
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(threads)
#endif
    for (int64_t k = 0; k < n; ++k) {
        double N[18];
        orc_normals(s, M, uv[2 * k], uv[2 * k + 1], N);
        int o = 0;
        for (int b = 0; b < 6; ++b) {
            if (!((mask >> b) & 1u)) continue;
            for (int c = 0; c < 3; ++c) out[(3 * o + c) * n + k] = N[3 * b + c];
            ++o;
        }
    }
}

/* ---------------------------------------------------------------- stage c: the tree */

#define GAP 8               /* GapPerEdge, src/kernel/kernel.cuh:17 */
#define PTS (GAP + 1)       /* PointsPerEdge */

static double max_abs3(d3 d) {   /* GetSecondDerivatives, kernel.cu:399 */
    return fmax(fabs(d.x), fmax(fabs(d.y), fabs(d.z)));
}

static int need_divide(const orc_tree_node* n) {   /* NeedDivide, kernel.cu:859-878 */
    double dx = n->rt[0] - n->lb[0], dy = n->rt[1] - n->lb[1], dz = n->rt[2] - n->lb[2], t;
    if (dx > dy) { t = dx; dx = dy; dy = t; }
    if (dx > dz) { t = dx; dx = dz; dz = t; }
    if ((dx < 0.5 * dy) && (dx < 0.5 * dz)) return 0;
    return 1;
}

/* One node of level grid g at block (bx,by): GetPoints (kernel.cu:404-431),
 * GetSecondDerivatives (:375-402), the three block maxima (:707-733) and
 * TightBoundingBox (:544-621). */
static void build_node(const orc_surface* s, const double* M, unsigned g, unsigned bx, unsigned by,
                       orc_tree_node* node, const orc_tree_node* parent) {
    const int p = s->degree_u, q = s->degree_v;
    double base_unit = 1.0 / g;
    double unit = base_unit / GAP;
    double base_u = base_unit * bx, base_v = base_unit * by;
    double M1 = 0, M2 = 0, M3 = 0;
    d3 mx = {0, 0, 0}, mn = {0, 0, 0};
    for (int tx = 0; tx < PTS; ++tx)
        for (int ty = 0; ty < PTS; ++ty) {
            double p1 = base_u + tx * unit, p2 = base_v + ty * unit;
            span_loc L = locate(s, M, p1, p2);
            d4 R = R_of(L.middle, p, q, L.u, L.v);
            double a = max_abs3(der_uu(L.middle, p, q, L.u, L.v, R, L.spanU));
            double b = max_abs3(der_uv(L.middle, p, q, L.u, L.v, R, L.spanU, L.spanV));
            double c = max_abs3(der_vv(L.middle, p, q, L.u, L.v, R, L.spanV));
            d3 S = cart(R);
            if (tx == 0 && ty == 0) {
                M1 = a; M2 = b; M3 = c; mx = S; mn = S;
            } else {
                /* lhs < rhs ? rhs : lhs  (kernel.cu:725, 562-564) */
                M1 = M1 < a ? a : M1;
                M2 = M2 < b ? b : M2;
                M3 = M3 < c ? c : M3;
                mx.x = mx.x < S.x ? S.x : mx.x;
                mx.y = mx.y < S.y ? S.y : mx.y;
                mx.z = mx.z < S.z ? S.z : mx.z;
                mn.x = mn.x > S.x ? S.x : mn.x;
                mn.y = mn.y > S.y ? S.y : mn.y;
                mn.z = mn.z > S.z ? S.z : mn.z;
            }
        }
    /* K = (M1 + 2 M2 + M3) * sqrt(3) / (8 * GAP*g * GAP*g)   (kernel.cu:574, 601) */
    unsigned den = 8u * GAP * g * GAP * g;
    double K = (M1 + 2 * M2 + M3) * sqrt(3.0) / den;
    node->rt[0] = mx.x + K; node->rt[1] = mx.y + K; node->rt[2] = mx.z + K;
    node->lb[0] = mn.x - K; node->lb[1] = mn.y - K; node->lb[2] = mn.z - K;
    double uunit = 1.0 / g;
    node->uv_lb[0] = bx * uunit; node->uv_lb[1] = by * uunit;
    node->uv_rt[0] = (bx + 1) * uunit; node->uv_rt[1] = (by + 1) * uunit;
    if (parent) {   /* min/max(TreeNode) clip, kernel.cu:609-611, 885-901 */
        for (int c = 0; c < 3; ++c) {
            node->rt[c] = fmin(node->rt[c], parent->rt[c]);
            node->lb[c] = fmax(node->lb[c], parent->lb[c]);
        }
    }
}

void orc_build_tree(const orc_surface* s, const double* M, orc_tree_node* tree, unsigned char* divided,
                    unsigned char* built) {
    memset(tree, 0, sizeof(orc_tree_node) * ORC_TREE_NODES);
    memset(divided, 0, ORC_TREE_NODES);
    memset(built, 0, ORC_TREE_NODES);
    /* level 0: the root; its parent index (0-1)/64 truncates to 0 itself, so the clip is a
     * no-op (kernel.cu:606-611) */
    build_node(s, M, 1, 0, 0, &tree[0], NULL);
    built[0] = 1;
    divided[0] = (unsigned char)need_divide(&tree[0]);
    if (!divided[0]) return;
    /* level 1: 8x8 children, tree index 1 + bx*8 + by (kernel.cu:545-548) */
    for (unsigned bx = 0; bx < GAP; ++bx)
        for (unsigned by = 0; by < GAP; ++by) {
            int t = 1 + (int)(bx * GAP + by);
            build_node(s, M, GAP, bx, by, &tree[t], &tree[0]);
            built[t] = 1;
            divided[t] = (unsigned char)need_divide(&tree[t]);
        }
}

int orc_candidates(const orc_tree_node* tree, const unsigned char* built, const double P[3], int* list) {
    int n = 0;
    for (int i = 0; i < ORC_TREE_NODES; ++i) {
        if (!built[i]) continue;
        const orc_tree_node* T = &tree[i];
        if ((P[0] >= T->lb[0]) && (P[1] >= T->lb[1]) && (P[2] >= T->lb[2]) && (P[0] <= T->rt[0]) &&
            (P[1] <= T->rt[1]) && (P[2] <= T->rt[2]))
            list[n++] = i;
    }
    return n;
}

/* --------------------------------------------------------- stage d: Gauss-Newton */

/* One reference GN update (kernel.cu:161-243).  Returns S at C in *Sout; writes step. */
static void gn_step(const orc_surface* s, const double* M, const double C[2], const double P[3], d3* Sout,
                    double step[2]) {
    const int p = s->degree_u, q = s->degree_v;
    span_loc L = locate(s, M, C[0], C[1]);
    d4 R = R_of(L.middle, p, q, L.u, L.v);
    d3 S = cart(R);
    *Sout = S;
    d3 du = der_u(L.middle, p, q, L.u, L.v, R, L.spanU);
    d3 dv = der_v(L.middle, p, q, L.u, L.v, R, L.spanV);
    double J[6] = {du.x, dv.x, du.y, dv.y, du.z, dv.z};
    double JT[6];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 2; j++) JT[j * 3 + i] = J[i * 2 + j];
    double t[4];
    mat_mult(JT, J, t, 2, 3, 2);
    double det = t[0] * t[3] - t[1] * t[2];
    double inv[4] = {t[3] / det, -t[1] / det, -t[2] / det, t[0] / det};
    double IJ[6];
    mat_mult(inv, JT, IJ, 2, 2, 3);
    double dif[3] = {S.x - P[0], S.y - P[1], S.z - P[2]};
    mat_mult(IJ, dif, step, 2, 3, 1);
}

static double dist3(d3 S, const double P[3]) {   /* norm(S-P), src/util/Matrix.cu:39-41 */
    double x = S.x - P[0], y = S.y - P[1], z = S.z - P[2];
    return sqrt(x * x + y * y + z * z);
}

static d3 surface_point(const orc_surface* s, const double* M, const double C[2]) {
    span_loc L = locate(s, M, C[0], C[1]);
    return cart(R_of(L.middle, s->degree_u, s->degree_v, L.u, L.v));
}

int orc_gauss_newton_shipped(const orc_surface* s, const double* M, const double seed[2], const double P[3],
                             double max_edge, double uv[2]) {
    double C[2] = {seed[0], seed[1]};
    for (int i = 0; i < 10; i++) {
        d3 S;
        double step[2];
        gn_step(s, M, C, P, &S, step);
        if (dist3(S, P) < max_edge) {   /* kernel.cu:178 — tested before the step */
            uv[0] = C[0];
            uv[1] = C[1];
            return 1;
        }
        C[0] = C[0] - step[0];
        C[1] = C[1] - step[1];
    }
    return 0;
}


/* ---------------------------------------------- normal cones and projection (nurbs_project)
 *
 * The reference's projection (Project, src/kernel/kernel.cu:471-485; NormalBoundingBoxCheck
 * :487-513; NormalBoundingBox :623-704; NormalBoxToNormalTreeNode :1613-1636; GetAngle
 * :1638-1641; driven by src/main.cu:329-396) is unfinished: NormalNeedDivide returns true, the
 * query point is a constant, N_M3 is taken from N_uv, the corner test ignores contain_zero and
 * looks along one side of the normal only, and the first Gauss-Newton success is printed.  The
 * oracle's definition of nurbs_project, with a decision on each of those:
 *  - normal box of a built node: the unnormalised normal N = Su x Sv at the node's 9x9 lattice
 *    (the box tree's samples), its component range widened by K = (M1 + 2 M2 + M3) sqrt(3) /
 *    (8 (8g)^2) with M1, M2, M3 the largest components of N_uu, N_uv, N_vv over the samples (the
 *    box tree's bound applied to N), intersected with the parent's normal box;
 *  - cone: every direction when the box contains 0, is empty, or has a corner 90 degrees or more
 *    from its centre; otherwise the axis is the box centre and the half-angle the largest angle
 *    to a corner (as NormalBoxToNormalTreeNode), widened by 2 atan(2^-11) for the FP32 test;
 *  - bound box of a node: its box intersected with the box of the control points whose basis
 *    functions are not zero on its parameter rectangle (which holds the surface there by the
 *    convex hull property; the reference's boxes, sampled and widened by K, are too wide on wavy
 *    surfaces to bound a distance, the control net too wide on smooth ones);
 *  - candidates of a query P: the nodes whose bound box is within the distance bound (its distance from P at most UB, the least
 *    distance from P to the surface points of the nodes' 3x3 sub-lattices (1, 4, 7)^2) and whose bound box's
 *    bounding ball (centre c, radius r) is seen from P inside the double cone (the normal may point towards P or away from it):
 *    cos(a) sqrt(|d|^2 - r^2) <= |d.axis| + sin(a) r, d = P - c.  Every direction from P to a
 *    point of the ball lies within asin(r/|d|) of d, so this accepts every node for which some
 *    S - P in its box can be parallel to a normal in its cone, and every node the reference's
 *    corner test accepts unless its box is farther than the bound.  The test runs in FP32 relative to the control net's centre (boxes rounded
 *    outward), in this order and with these roundings in the CUDA kernel too, so both select the
 *    same nodes;
 *  - seeds: per candidate, the point of its 9x9 lattice closest to P (one seed at the centre
 *    of a node spanning many waves of the surface often converges to a farther minimum);
 *  - trajectories minimise |S - P|^2 over the closed domain, so that minima on its boundary,
 *    where S - P is not normal to the surface, are found too: projected Newton steps (the
 *    Hessian J^T J + r.d2S where it is positive definite, J^T J elsewhere; a coordinate at a
 *    bound whose descent direction points out of the domain is held there and the other takes
 *    the 1-D step, Newton where its curvature is positive; the new point is clamped to the
 *    domain), each halved until the distance does not grow (at most 30 times; steps below 1e-6
 *    are taken whole, their decrease being below the rounding of the distance); converged at a move <= 1e-12 after a Newton step or <= 1e-14
 *    (1e-12, not the inversion's 1e-10: far points have flat minima, where Newton converges
 *    slowly and a stop at 1e-10 leaves the parameters ~1e-9 apart),
 *    or at a corner where the distance grows into the domain; at most max_iter iterations;
 *  - the answer is the closest result; AMBIGUOUS as in the inversion. */

static void surface_origin(const orc_surface* s, double org[3]);

/* x rounded to float towards -inf (down != 0) or +inf: the box stays outside the FP64 box. */
static float f_round_out(double x, int down) {
    float f = (float)x;
    if (down && (double)f > x) f = nextafterf(f, -INFINITY);
    if (!down && (double)f < x) f = nextafterf(f, INFINITY);
    return f;
}

/* Box of the control points whose basis functions are not zero on the node's parameter
 * rectangle: the surface over that rectangle lies in their convex hull (positive weights).  Not
 * a box of the reference; a rigorous bound for the distance test.  hb = lb xyz, rt xyz. */
static void hull_box(const orc_surface* s, const orc_tree_node* T, double hb[6]) {
    const int p = s->degree_u, q = s->degree_v;
    int i0 = orc_find_span(p, s->cp_u, s->knots_u, T->uv_lb[0]);
    int i1 = orc_find_span(p, s->cp_u, s->knots_u, T->uv_rt[0]);
    int j0 = orc_find_span(q, s->cp_v, s->knots_v, T->uv_lb[1]);
    int j1 = orc_find_span(q, s->cp_v, s->knots_v, T->uv_rt[1]);
    if (i1 > i0 && s->knots_u[i1] >= T->uv_rt[0]) --i1;   /* the span starting at the right end */
    if (j1 > j0 && s->knots_v[j1] >= T->uv_rt[1]) --j1;
    for (int c = 0; c < 3; ++c) { hb[c] = INFINITY; hb[3 + c] = -INFINITY; }
    for (int i = i0 - p; i <= i1; ++i)
        for (int j = j0 - q; j <= j1; ++j) {
            const double* x = s->cps + 3 * ((int64_t)i * s->cp_v + j);
            for (int c = 0; c < 3; ++c) {
                hb[c] = hb[c] > x[c] ? x[c] : hb[c];
                hb[3 + c] = hb[3 + c] < x[c] ? x[c] : hb[3 + c];
            }
        }
}

static void cone_record(const double hb[6], const double nb[6], const double org[3], float* rec) {
    double ctr[3], h[3];
    for (int c = 0; c < 3; ++c) {
        ctr[c] = (hb[c] + hb[3 + c]) / 2;
        h[c] = (hb[3 + c] - hb[c]) / 2;
    }
    const double r = sqrt(h[0] * h[0] + h[1] * h[1] + h[2] * h[2]);
    const double cm = fmax(fabs(ctr[0] - org[0]), fmax(fabs(ctr[1] - org[1]), fabs(ctr[2] - org[2])));
    for (int c = 0; c < 3; ++c) rec[c] = (float)(ctr[c] - org[c]);
    rec[3] = (float)(r * (1 + 0x1p-20) + cm * 0x1p-20);   /* covers the FP32 rounding of the centre */
    int all = nb[0] > nb[3] || nb[1] > nb[4] || nb[2] > nb[5];
    all = all || (nb[0] <= 0 && nb[3] >= 0 && nb[1] <= 0 && nb[4] >= 0 && nb[2] <= 0 && nb[5] >= 0);
    double cosA = 0, sinA = 1, ax[3] = {0, 0, 1};
    if (!all) {
        const double m[3] = {(nb[0] + nb[3]) / 2, (nb[1] + nb[4]) / 2, (nb[2] + nb[5]) / 2};
        const double mm = sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
        double cmin = 1;
        for (int i = 0; i < 2; ++i)
            for (int j = 0; j < 2; ++j)
                for (int k = 0; k < 2; ++k) {
                    const double c[3] = {nb[3 * i], nb[3 * j + 1], nb[3 * k + 2]};
                    const double cc = (m[0] * c[0] + m[1] * c[1] + m[2] * c[2]) /
                                      (mm * sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]));
                    cmin = cmin < cc ? cmin : cc;
                }
        if (cmin > 0) {
            const double sn = sqrt(fmax(0.0, 1 - cmin * cmin));
            const double t = 0x1p-11, cd = (1 - t * t) / (1 + t * t), sd = (2 * t) / (1 + t * t);
            const double ca = cmin * cd - sn * sd, sa = sn * cd + cmin * sd;
            if (ca > 0) {
                cosA = ca;
                sinA = sa;
                ax[0] = m[0] / mm;
                ax[1] = m[1] / mm;
                ax[2] = m[2] / mm;
            }
        }
    }
    for (int c = 0; c < 3; ++c) rec[4 + c] = (float)ax[c];
    rec[7] = (float)cosA;
    rec[8] = (float)sinA;
    for (int c = 0; c < 3; ++c) {
        rec[9 + c] = f_round_out(hb[c] - org[c], 1);
        rec[12 + c] = f_round_out(hb[3 + c] - org[c], 0);
    }
    for (int c = 15; c < ORC_CONE_STRIDE; ++c) rec[c] = 0;
}

static void cone_node(const orc_surface* s, const double* M, unsigned g, unsigned bx, unsigned by,
                      const orc_tree_node* T, const double* parent_nb, const double org[3], double* nb, float* rec,
                      float* upts) {
    double base_unit = 1.0 / g;
    double unit = base_unit / GAP;
    double base_u = base_unit * bx, base_v = base_unit * by;
    double M1 = 0, M2 = 0, M3 = 0, mx[3] = {0, 0, 0}, mn[3] = {0, 0, 0};
    for (int tx = 0; tx < PTS; ++tx)
        for (int ty = 0; ty < PTS; ++ty) {
            double p1 = base_u + tx * unit, p2 = base_v + ty * unit;
            double d[30], N[18];
            orc_ders3(s, M, p1, p2, d);
            normals_of(d, N);
            const double a = max_abs3(d3at(N, 3)), b = max_abs3(d3at(N, 4)), c = max_abs3(d3at(N, 5));
            {   /* the lattice's surface points: distance bounds and projection seeds */
                float* o = upts + 3 * (PTS * tx + ty);
                for (int c = 0; c < 3; ++c) o[c] = (float)(d[c] - org[c]);
            }
            if (tx == 0 && ty == 0) {
                M1 = a; M2 = b; M3 = c;
                for (int k = 0; k < 3; ++k) mx[k] = mn[k] = N[k];
            } else {
                M1 = M1 < a ? a : M1;
                M2 = M2 < b ? b : M2;
                M3 = M3 < c ? c : M3;
                for (int k = 0; k < 3; ++k) {
                    mx[k] = mx[k] < N[k] ? N[k] : mx[k];
                    mn[k] = mn[k] > N[k] ? N[k] : mn[k];
                }
            }
        }
    unsigned den = 8u * GAP * g * GAP * g;
    double K = (M1 + 2 * M2 + M3) * sqrt(3.0) / den;
    for (int k = 0; k < 3; ++k) {
        nb[k] = mn[k] - K;
        nb[3 + k] = mx[k] + K;
        if (parent_nb) {
            nb[k] = fmax(nb[k], parent_nb[k]);
            nb[3 + k] = fmin(nb[3 + k], parent_nb[3 + k]);
        }
    }
    double hb[6];
    hull_box(s, T, hb);
    /* the node's own box where it is narrower (smooth surfaces) */
    double xb[6];
    int empty = 0;
    for (int c = 0; c < 3; ++c) {
        xb[c] = hb[c] > T->lb[c] ? hb[c] : T->lb[c];
        xb[3 + c] = hb[3 + c] < T->rt[c] ? hb[3 + c] : T->rt[c];
        empty = empty || xb[c] > xb[3 + c];
    }
    cone_record(empty ? hb : xb, nb, org, rec);
}

void orc_build_cones(const orc_surface* s, const double* M, const orc_tree_node* tree, const unsigned char* built,
                     double* nbox, float* cone, float* upts) {
    double org[3];
    surface_origin(s, org);
    memset(nbox, 0, sizeof(double) * 6 * ORC_TREE_NODES);
    memset(cone, 0, sizeof(float) * ORC_CONE_STRIDE * ORC_TREE_NODES);
    memset(upts, 0, sizeof(float) * ORC_UPTS * 3 * ORC_TREE_NODES);
    if (!built[0]) return;
    cone_node(s, M, 1, 0, 0, &tree[0], NULL, org, nbox, cone, upts);
    if (!built[1]) return;
    for (unsigned bx = 0; bx < GAP; ++bx)
        for (unsigned by = 0; by < GAP; ++by) {
            int t = 1 + (int)(bx * GAP + by);
            cone_node(s, M, GAP, bx, by, &tree[t], nbox, org, nbox + 6 * t, cone + ORC_CONE_STRIDE * t,
                      upts + ORC_UPTS * 3 * t);
        }
}

static float fdot3(const float a[3], const float b[3]) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }

/* Projection candidates of P (ascending nodes) and edge seeds (node * 4 + edge, ascending; edge
 * 0: u = u0, 1: u = u1, 2: v = v0, 3: v = v1).  Returns the candidate count. */
int orc_project_cull(const orc_tree_node* tree, const unsigned char* built, const float* cone, const float* upts,
                     const double* P, const double org[3], int* list) {
    (void)tree;
    const int nb = built[1] ? ORC_TREE_NODES : (built[0] ? 1 : 0);
    const float Pf[3] = {(float)(P[0] - org[0]), (float)(P[1] - org[1]), (float)(P[2] - org[2])};
    float ub2 = INFINITY;
    for (int k = 0; k < nb; ++k)
        for (int a = 1; a < PTS; a += 3)   /* the 3x3 sub-lattice (1, 4, 7)^2 of each node */
            for (int b = 1; b < PTS; b += 3) {
                const float* x = upts + 3 * (ORC_UPTS * k + PTS * a + b);
                const float d[3] = {x[0] - Pf[0], x[1] - Pf[1], x[2] - Pf[2]};
                const float dd = fdot3(d, d);
                ub2 = ub2 < dd ? ub2 : dd;
            }
    ub2 = ub2 * (1.0f + 0x1p-10f);
    int n = 0;
    for (int k = 0; k < nb; ++k) {
        const float* rc = cone + ORC_CONE_STRIDE * k;
        float g[3];
        for (int c = 0; c < 3; ++c) {
            const float lo = rc[9 + c] - Pf[c], hi = Pf[c] - rc[12 + c];
            g[c] = lo > hi ? lo : hi;
            g[c] = g[c] > 0.0f ? g[c] : 0.0f;
        }
        const int nearb = fdot3(g, g) <= ub2;
        const float d[3] = {Pf[0] - rc[0], Pf[1] - rc[1], Pf[2] - rc[2]};
        const float dd = fdot3(d, d), r = rc[3];
        float e = dd - r * r;
        e = e > 0.0f ? e : 0.0f;
        const int seen = rc[7] * sqrtf(e) <= fabsf(fdot3(d, rc + 4)) + rc[8] * r;
        if (nearb && seen) {
            /* seed: the node's lattice point closest to P (first of equals) */
            float best = INFINITY;
            int bi = 0;
            for (int j = 0; j < ORC_UPTS; ++j) {
                const float* x = upts + 3 * (ORC_UPTS * k + j);
                const float e3[3] = {x[0] - Pf[0], x[1] - Pf[1], x[2] - Pf[2]};
                const float ee = fdot3(e3, e3);
                if (ee < best) { best = ee; bi = j; }
            }
            list[n++] = 128 * k + bi;
        }
    }
    return n;
}

/* Seed of projection candidate c = 128 * node + j: the node's lattice point j = 9 tx + ty (the
 * same arithmetic as the samples). */
static void projection_seed(int c, double C[2]) {
    const int k = c >> 7, j = c & 127;
    const unsigned g = k == 0 ? 1u : GAP, bx = k == 0 ? 0u : (unsigned)(k - 1) / GAP, by = k == 0 ? 0u : (unsigned)(k - 1) % GAP;
    const double base_unit = 1.0 / g, unit = base_unit / GAP;
    const int tx = j / PTS, ty = j % PTS;
    C[0] = base_unit * bx + tx * unit;
    C[1] = base_unit * by + ty * unit;
}

/* ------------------------------------------- inversion: the oracle's definition of the answer
 *
 * The reference stops Gauss-Newton when |S - P| < max_edge (kernel.cu:178), which cannot reach
 * 1e-9 parameter error for points off the surface, and returns the first success (kernel.cu:
 * 458-461).  The oracle's answer is defined instead as follows (a decision on those defects):
 *   - every candidate node seeds one trajectory at its uv-centre (kernel.cu:154), in ascending
 *     node order;
 *   - a trajectory takes the reference's Gauss-Newton update (gn_step, kernel.cu:161-243) while
 *     its last step was at least ORC_NEWTON_SWITCH in max-norm, and Newton steps once a step has
 *     fallen below it: H = J^T J + sum_k r_k d2S_k (old second derivatives, Evaluate.cu:667-930)
 *     when H is positive definite, the reference's GN update otherwise.  Both have the fixed
 *     point J^T r = 0; GN converges only linearly, at rate ~|r| kappa, which is not small at
 *     offsets of 1e-2, so a pure-GN definition leaves many queries unconverged;
 *   - it has converged when a Newton-phase step is <= 1e-10 (the error is then ~1e-20) or any
 *     step is <= 1e-14, and is dropped when it has not converged after max_iter iterations, when
 *     its system is singular or when it converges outside the knot domain;
 *   - the answer is the converged result of least distance (ties: lowest node); it is
 *     AMBIGUOUS when another result more than 1e-7 away is within 1e-6 relative of it. */

#define ORC_NEWTON_SWITCH 1e-2

/* Newton step at C: returns 0 when H is not positive definite (the caller then takes the GN
 * update).  r = S - P; H = [Su.Su + r.Suu, Su.Sv + r.Suv; Sv.Sv + r.Svv]; g = [Su.r, Sv.r]. */
static int newton_step(const orc_surface* s, const double* M, const double C[2], const double P[3], double step[2]) {
    const int p = s->degree_u, q = s->degree_v;
    span_loc L = locate(s, M, C[0], C[1]);
    d4 R = R_of(L.middle, p, q, L.u, L.v);
    d3 S = cart(R);
    d3 Su = der_u(L.middle, p, q, L.u, L.v, R, L.spanU);
    d3 Sv = der_v(L.middle, p, q, L.u, L.v, R, L.spanV);
    d3 Suu = der_uu(L.middle, p, q, L.u, L.v, R, L.spanU);
    d3 Suv = der_uv(L.middle, p, q, L.u, L.v, R, L.spanU, L.spanV);
    d3 Svv = der_vv(L.middle, p, q, L.u, L.v, R, L.spanV);
    d3 r = {S.x - P[0], S.y - P[1], S.z - P[2]};
    double h00 = (Su.x * Su.x + Su.y * Su.y + Su.z * Su.z) + (r.x * Suu.x + r.y * Suu.y + r.z * Suu.z);
    double h01 = (Su.x * Sv.x + Su.y * Sv.y + Su.z * Sv.z) + (r.x * Suv.x + r.y * Suv.y + r.z * Suv.z);
    double h11 = (Sv.x * Sv.x + Sv.y * Sv.y + Sv.z * Sv.z) + (r.x * Svv.x + r.y * Svv.y + r.z * Svv.z);
    double det = h00 * h11 - h01 * h01;
    if (!(h00 > 0 && det > 0)) return 0;
    double g0 = Su.x * r.x + Su.y * r.y + Su.z * r.z;
    double g1 = Sv.x * r.x + Sv.y * r.y + Sv.z * r.z;
    step[0] = (h11 * g0 - h01 * g1) / det;
    step[1] = (h00 * g1 - h01 * g0) / det;
    return 1;
}

/* One trajectory from C (updated in place).  newton: start in the Newton phase (used to polish
 * a given point).  Returns 1 when it converged; *iters counts the iterations. */
static int run_trajectory(const orc_surface* s, const double* M, const double P[3], double C[2], int max_iter,
                          int newton, int* iters) {
    for (int it = 0; it < max_iter; ++it) {
        double step[2];
        if (!(newton && newton_step(s, M, C, P, step))) {
            d3 S;
            gn_step(s, M, C, P, &S, step);   /* the reference's update, kernel.cu:161-243 */
        }
        if (!(isfinite(step[0]) && isfinite(step[1]))) { *iters = it + 1; return 0; }
        C[0] = C[0] - step[0];
        C[1] = C[1] - step[1];
        double m = fmax(fabs(step[0]), fabs(step[1]));
        if ((newton && m <= 1e-10) || m <= 1e-14) { *iters = it + 1; return 1; }
        newton = m < ORC_NEWTON_SWITCH;
    }
    *iters = max_iter;
    return 0;
}

/* One projection trajectory from C (the definition above): projected Newton with a line search,
 * C stays in the domain.  Returns 1 when it converged; *iters counts the iterations. */
static void ders2_at(const orc_surface* s, const double* M, const double C[2], d3* S, d3* Su, d3* Sv, d3* Suu,
                     d3* Suv, d3* Svv) {
    const int p = s->degree_u, q = s->degree_v;
    span_loc L = locate(s, M, C[0], C[1]);
    d4 R = R_of(L.middle, p, q, L.u, L.v);
    *S = cart(R);
    *Su = der_u(L.middle, p, q, L.u, L.v, R, L.spanU);
    *Sv = der_v(L.middle, p, q, L.u, L.v, R, L.spanV);
    *Suu = der_uu(L.middle, p, q, L.u, L.v, R, L.spanU);
    *Suv = der_uv(L.middle, p, q, L.u, L.v, R, L.spanU, L.spanV);
    *Svv = der_vv(L.middle, p, q, L.u, L.v, R, L.spanV);
}

static double dot3d(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static double clampd(double x, double lo, double hi) { return x < lo ? lo : (x > hi ? hi : x); }

static int project_trajectory(const orc_surface* s, const double* M, const double P[3], double C[2],
                              const double dom[4], int max_iter, int* iters) {
    d3 S, Su, Sv, Suu, Suv, Svv;
    C[0] = clampd(C[0], dom[0], dom[1]);
    C[1] = clampd(C[1], dom[2], dom[3]);
    ders2_at(s, M, C, &S, &Su, &Sv, &Suu, &Suv, &Svv);
    for (int it = 0; it < max_iter; ++it) {
        const d3 r = {S.x - P[0], S.y - P[1], S.z - P[2]};
        const double f = dot3d(r, r);
        const double g0 = dot3d(Su, r), g1 = dot3d(Sv, r);
        const double a00 = dot3d(Su, Su), a01 = dot3d(Su, Sv), a11 = dot3d(Sv, Sv);
        const double n00 = a00 + dot3d(r, Suu), n01 = a01 + dot3d(r, Suv), n11 = a11 + dot3d(r, Svv);
        /* a coordinate at a bound whose descent direction -g points out of the domain stays */
        const int fu = !((C[0] <= dom[0] && g0 > 0) || (C[0] >= dom[1] && g0 < 0));
        const int fv = !((C[1] <= dom[2] && g1 > 0) || (C[1] >= dom[3] && g1 < 0));
        double d0 = 0, d1 = 0;
        int newton;
        if (fu && fv) {
            newton = n00 > 0 && n00 * n11 - n01 * n01 > 0;
            const double h00 = newton ? n00 : a00, h01 = newton ? n01 : a01, h11 = newton ? n11 : a11;
            const double det = h00 * h11 - h01 * h01;
            if (!(det > 0)) { *iters = it + 1; return 0; }
            d0 = (h11 * g0 - h01 * g1) / det;
            d1 = (h00 * g1 - h01 * g0) / det;
        } else if (fu) {   /* the 1-D Newton step along u where its curvature is positive */
            newton = n00 > 0;
            const double h = newton ? n00 : a00;
            if (!(h > 0)) { *iters = it + 1; return 0; }
            d0 = g0 / h;
        } else if (fv) {
            newton = n11 > 0;
            const double h = newton ? n11 : a11;
            if (!(h > 0)) { *iters = it + 1; return 0; }
            d1 = g1 / h;
        } else {
            *iters = it + 1;   /* a corner where the distance grows into the domain */
            return 1;
        }
        if (!(isfinite(d0) && isfinite(d1))) { *iters = it + 1; return 0; }
        /* line search: halve the step until the distance does not grow (at most 30 times); a step
         * below 1e-6 is taken whole (the decrease it makes is below the rounding of the distance,
         * so comparing distances would stop it at random near the minimum) */
        const int search = fmax(fabs(d0), fabs(d1)) > 1e-6;
        double alpha = 1, Cn[2];
        d3 Sn, Snu, Snv, Snuu, Snuv, Snvv;
        for (int ls = 0;; ++ls) {
            Cn[0] = clampd(C[0] - alpha * d0, dom[0], dom[1]);
            Cn[1] = clampd(C[1] - alpha * d1, dom[2], dom[3]);
            ders2_at(s, M, Cn, &Sn, &Snu, &Snv, &Snuu, &Snuv, &Snvv);
            const d3 rn = {Sn.x - P[0], Sn.y - P[1], Sn.z - P[2]};
            if (!search || dot3d(rn, rn) <= f || ls == 30) break;
            alpha *= 0.5;
        }
        const double moved = fmax(fabs(Cn[0] - C[0]), fabs(Cn[1] - C[1]));
        C[0] = Cn[0];
        C[1] = Cn[1];
        S = Sn; Su = Snu; Sv = Snv; Suu = Snuu; Suv = Snuv; Svv = Snvv;
        if (moved <= 1e-14 || (newton && moved <= 1e-12)) { *iters = it + 1; return 1; }
    }
    *iters = max_iter;
    return 0;
}


/* cone == NULL: the inversion; else the projection (candidates, seeds and trajectories above). */
static void invert_one(const orc_surface* s, const double* M, const orc_tree_node* tree, const unsigned char* built,
                       const float* cone, const double org[3], const double* Pk, int max_iter, const double dom[4],
                       double* uv, int* status, double* residual, int* iters) {
    int list[ORC_TREE_NODES];
    int nc = cone ? orc_project_cull(tree, built, cone, cone + ORC_CONE_STRIDE * ORC_TREE_NODES, Pk, org, list)
                  : orc_candidates(tree, built, Pk, list);
    double best_uv[2] = {NAN, NAN}, best_r = INFINITY;
    double sol_uv[ORC_TREE_NODES][2], sol_r[ORC_TREE_NODES];
    int nsol = 0, total = 0;
    for (int c = 0; c < nc; ++c) {
        double C[2];
        if (cone) {
            projection_seed(list[c], C);
        } else {
            /* seed = uv-centre of the node (kernel.cu:154) */
            const orc_tree_node* T = &tree[list[c]];
            C[0] = (T->uv_lb[0] + T->uv_rt[0]) / 2;
            C[1] = (T->uv_lb[1] + T->uv_rt[1]) / 2;
        }
        int its = 0;
        int converged = cone ? project_trajectory(s, M, Pk, C, dom, max_iter, &its)
                             : run_trajectory(s, M, Pk, C, max_iter, 0, &its);
        total += its;
        if (!converged) continue;
        if (!(C[0] >= dom[0] && C[0] <= dom[1] && C[1] >= dom[2] && C[1] <= dom[3])) continue;
        double r = dist3(surface_point(s, M, C), Pk);
        if (!isfinite(r)) continue;
        sol_uv[nsol][0] = C[0];
        sol_uv[nsol][1] = C[1];
        sol_r[nsol] = r;
        ++nsol;
        if (r < best_r) { best_r = r; best_uv[0] = C[0]; best_uv[1] = C[1]; }
    }
    int st;
    if (nc == 0) st = ORC_NO_CANDIDATE;
    else if (nsol == 0) st = ORC_NOT_CONVERGED;
    else {
        st = ORC_FOUND_UNIQUE;
        for (int t = 0; t < nsol; ++t) {
            int same = fabs(sol_uv[t][0] - best_uv[0]) <= 1e-7 && fabs(sol_uv[t][1] - best_uv[1]) <= 1e-7;
            if (!same && sol_r[t] <= best_r * (1 + 1e-6) + 1e-12) st = ORC_FOUND_AMBIGUOUS;
        }
    }
    uv[0] = best_uv[0];
    uv[1] = best_uv[1];
    *status = st;
    *residual = nsol ? best_r : NAN;
    if (iters) *iters = total;
}

static void domain_of(const orc_surface* s, double dom[4]) {
    dom[0] = s->knots_u[s->degree_u];
    dom[1] = s->knots_u[s->cp_u];
    dom[2] = s->knots_v[s->degree_v];
    dom[3] = s->knots_v[s->cp_v];
}

static void invert_all(const orc_surface* s, const double* M, const orc_tree_node* tree, const unsigned char* built,
                       const float* cone, const double* P, int64_t n, int max_iter, double* uv, int* status,
                       double* residual, int* iters, int threads) {
    double dom[4], org[3];
    domain_of(s, dom);
    surface_origin(s, org);
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads)
#endif
    for (int64_t k = 0; k < n; ++k)
        invert_one(s, M, tree, built, cone, org, P + 3 * k, max_iter, dom, uv + 2 * k, status + k, residual + k,
                   iters ? iters + k : NULL);
}

void orc_invert(const orc_surface* s, const double* M, const orc_tree_node* tree, const unsigned char* built,
                const double* P, int64_t n, int max_iter, double* uv, int* status, double* residual, int* iters,
                int threads) {
    invert_all(s, M, tree, built, NULL, P, n, max_iter, uv, status, residual, iters, threads);
}

void orc_project(const orc_surface* s, const double* M, const orc_tree_node* tree, const unsigned char* built,
                 const float* cone, const double* P, int64_t n, int max_iter, double* uv, int* status,
                 double* residual, int* iters, int threads) {
    invert_all(s, M, tree, built, cone, P, n, max_iter, uv, status, residual, iters, threads);
}

/* ------------------------------------------------------ stability of the answer at FP32 resolution */

/* Centre of the control net's bounding box: FP32 arithmetic of the surface is done relative to
 * it, and perturbations at FP32 resolution are relative to it. */
static void surface_origin(const orc_surface* s, double org[3]) {
    for (int c = 0; c < 3; ++c) {
        double lo = s->cps[c], hi = lo;
        for (int i = 1; i < s->cp_u * s->cp_v; ++i) {
            lo = fmin(lo, s->cps[3 * i + c]);
            hi = fmax(hi, s->cps[3 * i + c]);
        }
        org[c] = 0.5 * (lo + hi);
    }
}

/* Sign (+1/-1) of perturbation k of coordinate i: a fixed hash (splitmix64), so the perturbed
 * points are the same on every machine. */
static double perturb_sign(int k, int64_t i) {
    uint64_t z = (uint64_t)(k + 1) * 0x9E3779B97F4A7C15ull + (uint64_t)i * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (z & 1) ? 1.0 : -1.0;
}

/* Perturbation k of coordinate c of point i: (x - org) scaled by (1 +- eps_k), eps_k = eps for
 * even k and 4 eps for odd k (the FP32 evaluation of S errs by a few units of rounding). */
static double perturbed(const double org[3], const double* P, int k, int64_t i, int c, double eps) {
    const double e = (k & 1) ? 4 * eps : eps;
    return org[c] + (P[c] - org[c]) * (1.0 + e * perturb_sign(k, 3 * i + c));
}

static void perturbed_all(const orc_surface* s, const double* M, const orc_tree_node* tree,
                          const unsigned char* built, const float* cone, const double* P, int64_t n, int max_iter,
                          int K, double eps, double* uv, int* found, double* residual, int threads) {
    double dom[4], org[3];
    domain_of(s, dom);
    surface_origin(s, org);
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads) collapse(2)
#endif
    for (int k = 0; k < K; ++k)
        for (int64_t i = 0; i < n; ++i) {
            const double* Pk = P + 3 * i;
            double Pp[3];
            for (int c = 0; c < 3; ++c) Pp[c] = perturbed(org, Pk, k, i, c, eps);
            double C[2];
            int st, its;
            double r;
            invert_one(s, M, tree, built, cone, org, Pp, max_iter, dom, C, &st, &r, NULL);
            const int64_t o = (int64_t)k * n + i;
            int ok = 0;
            if (st == ORC_FOUND_UNIQUE || st == ORC_FOUND_AMBIGUOUS) {
                /* the minimum of the true point next to the perturbed answer */
                if (cone)
                    ok = project_trajectory(s, M, Pk, C, dom, max_iter, &its);
                else
                    ok = run_trajectory(s, M, Pk, C, max_iter, 1, &its) && C[0] >= dom[0] && C[0] <= dom[1] &&
                         C[1] >= dom[2] && C[1] <= dom[3];
            }
            uv[2 * o] = ok ? C[0] : NAN;
            uv[2 * o + 1] = ok ? C[1] : NAN;
            found[o] = ok;
            residual[o] = ok ? dist3(surface_point(s, M, C), Pk) : NAN;
        }
}

void orc_invert_perturbed(const orc_surface* s, const double* M, const orc_tree_node* tree,
                          const unsigned char* built, const double* P, int64_t n, int max_iter, int K, double eps,
                          double* uv, int* found, double* residual, int threads) {
    perturbed_all(s, M, tree, built, NULL, P, n, max_iter, K, eps, uv, found, residual, threads);
}

void orc_project_perturbed(const orc_surface* s, const double* M, const orc_tree_node* tree,
                           const unsigned char* built, const float* cone, const double* P, int64_t n, int max_iter,
                           int K, double eps, double* uv, int* found, double* residual, int threads) {
    perturbed_all(s, M, tree, built, cone, P, n, max_iter, K, eps, uv, found, residual, threads);
}

/* The same trajectories as invert_one computed in FP32 arithmetic (span matrices, local
 * parameters, evaluation and the 2x2 solves rounded to float), each stopped at the FP32
 * resolution of the parameters; every distinct FP32 minimum within 5 % of the closest then takes
 * FP64 Newton steps to the true point's minimum, and the closest of those is the answer.  The FP32
 * arithmetic works relative to the centre of the control net's bounding box (the span matrices
 * of the translated surface, the point minus that centre), so its resolution follows the
 * surface's extent rather than its distance from the origin.  A query whose FP64 answer this does
 * not reproduce has an answer that FP32 arithmetic cannot determine: some trajectory that reaches
 * it is chaotic at FP32 resolution. */

typedef struct { float x, y, z; } f3;
typedef struct { f3 S, Su, Sv, Suu, Suv, Svv; } f3ders;

static float f3dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

static f3ders eval32(const orc_surface* s, const double* M, const double org[3], float uu, float vv) {
    const int p = s->degree_u, q = s->degree_v, k1 = p + 1, k2 = q + 1;
    const double* ku = s->knots_u;
    const double* kv = s->knots_v;
    int m = orc_find_span(p, s->cp_u, ku, (double)uu);
    int n = orc_find_span(q, s->cp_v, kv, (double)vv);
    float iu = (float)(1.0 / (ku[m + 1] - ku[m])), iv = (float)(1.0 / (kv[n + 1] - kv[n]));
    float u = (uu - (float)ku[m]) * iu, v = (vv - (float)kv[n]) * iv;
    float su = (float)(ku[p + s->cp_u] - ku[0]) * iu, sv = (float)(kv[q + s->cp_v] - kv[0]) * iv;
    const double* mid = M + orc_matrix_n_position(m, n, p, q, s->cp_u, s->cp_v, 0);
    float U[8], dU[8], ddU[8], V[8], dV[8], ddV[8];
    for (int a = 0; a < k1; ++a) {
        U[a] = a == 0 ? 1.0f : U[a - 1] * u;
        dU[a] = a == 0 ? 0.0f : (float)a * U[a - 1];
        ddU[a] = a < 2 ? 0.0f : (float)(a * (a - 1)) * U[a - 2];
    }
    for (int b = 0; b < k2; ++b) {
        V[b] = b == 0 ? 1.0f : V[b - 1] * v;
        dV[b] = b == 0 ? 0.0f : (float)b * V[b - 1];
        ddV[b] = b < 2 ? 0.0f : (float)(b * (b - 1)) * V[b - 2];
    }
    float R[4] = {0}, Ru[4] = {0}, Rv[4] = {0}, Ruu[4] = {0}, Ruv[4] = {0}, Rvv[4] = {0};
    for (int c = 0; c < 4; ++c)
        for (int a = 0; a < k1; ++a) {
            float t = 0, td = 0, tdd = 0;
            for (int b = 0; b < k2; ++b) {
                /* coefficient of the surface translated by -org: xw - org_x w, ... */
                double mm = mid[c * k1 * k2 + a * k2 + b];
                float coef = (float)(c < 3 ? mm - org[c] * mid[3 * k1 * k2 + a * k2 + b] : mm);
                t += coef * V[b];
                td += coef * dV[b];
                tdd += coef * ddV[b];
            }
            R[c] += U[a] * t;
            Ru[c] += dU[a] * t;
            Rv[c] += U[a] * td;
            Ruu[c] += ddU[a] * t;
            Ruv[c] += dU[a] * td;
            Rvv[c] += U[a] * tdd;
        }
    float w = R[3], wu = Ru[3] * su, wv = Rv[3] * sv, wuu = Ruu[3] * su * su, wuv = Ruv[3] * su * sv,
          wvv = Rvv[3] * sv * sv;
    float S[3], Su[3], Sv[3], Suu[3], Suv[3], Svv[3];
    for (int c = 0; c < 3; ++c) {
        S[c] = R[c] / w;
        Su[c] = (Ru[c] * su - S[c] * wu) / w;
        Sv[c] = (Rv[c] * sv - S[c] * wv) / w;
        Suu[c] = (Ruu[c] * su * su - 2 * Su[c] * wu - S[c] * wuu) / w;
        Suv[c] = (Ruv[c] * su * sv - Su[c] * wv - Sv[c] * wu - S[c] * wuv) / w;
        Svv[c] = (Rvv[c] * sv * sv - 2 * Sv[c] * wv - S[c] * wvv) / w;
    }
    f3ders d = {{S[0], S[1], S[2]}, {Su[0], Su[1], Su[2]}, {Sv[0], Sv[1], Sv[2]},
                {Suu[0], Suu[1], Suu[2]}, {Suv[0], Suv[1], Suv[2]}, {Svv[0], Svv[1], Svv[2]}};
    return d;
}

/* One FP32 trajectory (the FP64 schedule's rules, stopped at FP32 resolution; steps that do not
 * shrink end it only where the Newton Hessian is positive definite).  Returns 1 when it
 * converged; dist2 = |S - P|^2 at its last evaluation. */
static int trajectory32(const orc_surface* s, const double* M, const double org[3], const float P[3], float C[2],
                        const double dom[4], int max_iter, float* dist2) {
    const float eu = (float)(dom[1] - dom[0]), ev = (float)(dom[3] - dom[2]);
    const float far[4] = {(float)dom[0] - 2 * eu, (float)dom[1] + 2 * eu, (float)dom[2] - 2 * ev,
                          (float)dom[3] + 2 * ev};
    int newton = 0;
    float prev = INFINITY;
    for (int it = 0; it < max_iter; ++it) {
        f3ders d = eval32(s, M, org, C[0], C[1]);
        f3 r = {d.S.x - P[0], d.S.y - P[1], d.S.z - P[2]};
        float h00 = f3dot(d.Su, d.Su), h01 = f3dot(d.Su, d.Sv), h11 = f3dot(d.Sv, d.Sv);
        float g0 = f3dot(d.Su, r), g1 = f3dot(d.Sv, r);
        int pd = 0;
        if (newton) {
            float n00 = h00 + f3dot(r, d.Suu), n01 = h01 + f3dot(r, d.Suv), n11 = h11 + f3dot(r, d.Svv);
            if (n00 > 0 && n00 * n11 - n01 * n01 > 0) { h00 = n00; h01 = n01; h11 = n11; pd = 1; }
        }
        float det = h00 * h11 - h01 * h01;
        if (!(det > 0)) return 0;
        float du = (h11 * g0 - h01 * g1) / det, dv = (h00 * g1 - h01 * g0) / det;
        if (!(isfinite(du) && isfinite(dv))) return 0;
        C[0] -= du;
        C[1] -= dv;
        float step = fmaxf(fabsf(du), fabsf(dv));
        *dist2 = f3dot(r, r);
        float smag = fmaxf(fmaxf(fabsf(d.S.x), fabsf(d.S.y)), fmaxf(fabsf(d.S.z), 1.0f));
        f3 dS = {d.Su.x * du + d.Sv.x * dv, d.Su.y * du + d.Sv.y * dv, d.Su.z * du + d.Sv.z * dv};
        float fl = 8.0f * 5.96e-8f * smag;
        if (step <= 3e-7f || f3dot(dS, dS) <= fl * fl) return 1;
        if (pd && step < 1e-4f && step > 0.5f * prev) return 1;
        prev = step;
        newton = step < (float)ORC_NEWTON_SWITCH;
        if (!(C[0] >= far[0] && C[0] <= far[1] && C[1] >= far[2] && C[1] <= far[3])) return 0;
    }
    return 0;
}

static void explore_all(const orc_surface* s, const double* M, const orc_tree_node* tree,
                        const unsigned char* built, const double* P, int64_t n, int max_iter, int pk, double eps,
                        double* uv, int* found, double* residual, int threads) {
    double dom[4], org[3];
    domain_of(s, dom);
    surface_origin(s, org);
    const double cell_u = 1e-4 * (dom[1] - dom[0]), cell_v = 1e-4 * (dom[3] - dom[2]);
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads)
#endif
    for (int64_t k = 0; k < n; ++k) {
        const double* Pk = P + 3 * k;
        float Pf[3];
        for (int c = 0; c < 3; ++c) Pf[c] = (float)((pk < 0 ? Pk[c] : perturbed(org, Pk, pk, k, c, eps)) - org[c]);
        int list[ORC_TREE_NODES];
        int nc = orc_candidates(tree, built, Pk, list);
        float mu[ORC_TREE_NODES], mv[ORC_TREE_NODES], md[ORC_TREE_NODES];
        long mcu[ORC_TREE_NODES], mcv[ORC_TREE_NODES];
        int nm = 0;
        for (int c = 0; c < nc; ++c) {
            const orc_tree_node* T = &tree[list[c]];
            float C[2] = {(float)((T->uv_lb[0] + T->uv_rt[0]) / 2), (float)((T->uv_lb[1] + T->uv_rt[1]) / 2)};
            float d2 = 0;
            if (!trajectory32(s, M, org, Pf, C, dom, max_iter, &d2)) continue;
            if (!(C[0] >= (float)dom[0] - 1e-4f && C[0] <= (float)dom[1] + 1e-4f && C[1] >= (float)dom[2] - 1e-4f &&
                  C[1] <= (float)dom[3] + 1e-4f))
                continue;
            long cu = (long)floor((C[0] - dom[0]) / cell_u), cv = (long)floor((C[1] - dom[2]) / cell_v);
            int f = -1;
            for (int t = 0; t < nm; ++t)
                if (mcu[t] == cu && mcv[t] == cv) f = t;
            if (f < 0) { f = nm++; mcu[f] = cu; mcv[f] = cv; md[f] = INFINITY; }
            if (d2 < md[f]) { md[f] = d2; mu[f] = C[0]; mv[f] = C[1]; }
        }
        float dbest = INFINITY;
        for (int t = 0; t < nm; ++t) dbest = fminf(dbest, md[t]);
        double bu = NAN, bv = NAN, br = INFINITY;
        for (int t = 0; t < nm; ++t) {
            if (!(sqrtf(md[t]) <= sqrtf(dbest) * 1.05f + 1e-5f)) continue;
            double C[2] = {mu[t], mv[t]};
            int its;
            if (!run_trajectory(s, M, Pk, C, max_iter, 1, &its)) continue;
            if (!(C[0] >= dom[0] && C[0] <= dom[1] && C[1] >= dom[2] && C[1] <= dom[3])) continue;
            double r = dist3(surface_point(s, M, C), Pk);
            if (r < br) { br = r; bu = C[0]; bv = C[1]; }
        }
        found[k] = isfinite(br);
        uv[2 * k] = bu;
        uv[2 * k + 1] = bv;
        residual[k] = isfinite(br) ? br : NAN;
    }
}

void orc_invert_fp32_explore(const orc_surface* s, const double* M, const orc_tree_node* tree,
                             const unsigned char* built, const double* P, int64_t n, int max_iter, int pk,
                             double eps, double* uv, int* found, double* residual, int threads) {
    explore_all(s, M, tree, built, P, n, max_iter, pk, eps, uv, found, residual, threads);
}

/* ------------------------------------------------------------------------------ p-curves
 * The oracle of nurbs_pcurve: orc_invert of every sample, then FP64 Newton steps (the
 * trajectory's Newton phase) from the two neighbours' answers, kept when strictly closer than
 * the own answer or when there is none; flags from the final answers (jump: parameter step above
 * 4 |chord| / sigma_min(J) at the sample's answer; ambiguous; not found). */
void orc_pcurve(const orc_surface* s, const double* M, const orc_tree_node* tree, const unsigned char* built,
                const double* C, int64_t n, int max_iter, double* uv, int* status, double* residual, int* flags,
                int threads) {
    double dom[4];
    domain_of(s, dom);
    double* uv0 = (double*)malloc(sizeof(double) * 2 * (size_t)(n > 0 ? n : 1));
    int* st0 = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    double* r0 = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    orc_invert(s, M, tree, built, C, n, max_iter, uv0, st0, r0, NULL, threads);
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads)
#endif
    for (int64_t i = 0; i < n; ++i) {
        const double* Pk = C + 3 * i;
        double bu = uv0[2 * i], bv = uv0[2 * i + 1], br = r0[i];
        int bs = st0[i];
        const double scale = fmax(1.0, fmax(fabs(Pk[0]), fmax(fabs(Pk[1]), fabs(Pk[2]))));
        for (int side = 0; side < 2; ++side) {
            const int64_t j = side == 0 ? i - 1 : i + 1;
            if (j < 0 || j >= n || st0[j] > ORC_FOUND_AMBIGUOUS) continue;
            double Cc[2] = {uv0[2 * j], uv0[2 * j + 1]};
            int its;
            if (!run_trajectory(s, M, Pk, Cc, max_iter, 1, &its)) continue;
            if (!(Cc[0] >= dom[0] && Cc[0] <= dom[1] && Cc[1] >= dom[2] && Cc[1] <= dom[3])) continue;
            double r = dist3(surface_point(s, M, Cc), Pk);
            if (!isfinite(r)) continue;
            int found = bs <= ORC_FOUND_AMBIGUOUS;
            if (!found || (r < br - (1e-12 * br + 1e-14 * scale) && (fabs(Cc[0] - bu) > 1e-7 || fabs(Cc[1] - bv) > 1e-7))) {
                bu = Cc[0]; bv = Cc[1]; br = r; bs = ORC_FOUND_UNIQUE;
            }
        }
        uv[2 * i] = bu;
        uv[2 * i + 1] = bv;
        residual[i] = br;
        status[i] = bs;
    }
    for (int64_t i = 0; i < n; ++i) {
        int f = 0;
        if (status[i] > ORC_FOUND_AMBIGUOUS) f |= 4;
        if (status[i] == ORC_FOUND_AMBIGUOUS) f |= 2;
        if (i > 0 && status[i] <= ORC_FOUND_AMBIGUOUS && status[i - 1] <= ORC_FOUND_AMBIGUOUS) {
            span_loc L = locate(s, M, uv[2 * i], uv[2 * i + 1]);
            d4 R = R_of(L.middle, s->degree_u, s->degree_v, L.u, L.v);
            d3 Su = der_u(L.middle, s->degree_u, s->degree_v, L.u, L.v, R, L.spanU);
            d3 Sv = der_v(L.middle, s->degree_u, s->degree_v, L.u, L.v, R, L.spanV);
            double a = Su.x * Su.x + Su.y * Su.y + Su.z * Su.z, b = Su.x * Sv.x + Su.y * Sv.y + Su.z * Sv.z,
                   c = Sv.x * Sv.x + Sv.y * Sv.y + Sv.z * Sv.z;
            double m = 0.5 * (a + c), h = 0.5 * (a - c);
            double lmin = m - sqrt(h * h + b * b);
            double dx = C[3 * i] - C[3 * i - 3], dy = C[3 * i + 1] - C[3 * i - 2], dz = C[3 * i + 2] - C[3 * i - 1];
            double chord = sqrt(dx * dx + dy * dy + dz * dz);
            double du = uv[2 * i] - uv[2 * i - 2], dv = uv[2 * i + 1] - uv[2 * i - 1];
            double step = sqrt(du * du + dv * dv);
            if (!(lmin > 0) || step * sqrt(lmin) > 4.0 * chord + 1e-12) f |= 1;
        }
        flags[i] = f;
    }
    free(uv0);
    free(st0);
    free(r0);
}

/* --------------------------------------------------- adaptive quadtree inversion (v1 seeding)
 * The reference's first inversion (Inverse, src/kernel/kernel.cu:4-104; BoundingBoxCheck
 * :106-149; getSplitType :251-298; Node, NODE_MAX_SIZE 64, src/kernel/kernel.cuh:13, 30-33)
 * needs no tree: per query, a breadth-first quadtree over the parameter domain.  The oracle's
 * definition, with a decision on each defect:
 *  - the root is the knot domain (the reference starts from [0,1]^2);
 *  - a node passes when P lies in the box of the control points of its span range, widened by
 *    max_edge (BoundingBoxCheck: rows findSpan(lb.u) - p .. findSpan(rt.u), the same in v);
 *  - every passing node seeds one trajectory at its centre (the inversion's trajectory: GN
 *    update, Newton below a 1e-2 step, converged at 1e-10 / 1e-14, 40 iterations); it succeeds
 *    when it converged inside the domain with |S - P| < max_edge (the reference's success test);
 *  - the first layer with a success ends the query: its closest success is the answer (the
 *    reference returns the first success in node order), AMBIGUOUS as in the inversion;
 *  - otherwise every passing node is split by getSplitType (4 samples on its diagonal, the
 *    u- and v-lengths sum |S_u| and |S_v| times a quarter of the side; the reference takes the
 *    v-derivative with MatrixSurfaceDerivativeU) and its children, in the reference's order,
 *    form the next layer; nodes that do not pass are not split (the hull is a bound, so their
 *    subtrees cannot hold an answer; the reference splits every node and overflows its 64-node
 *    layer at depth 4); NOT_SPLIT nodes end there;
 *  - a layer of more than 64 nodes, or 60 layers, ends the query unanswered (NOT_CONVERGED); an
 *    empty layer ends it with NO_CANDIDATE when no node ever passed, else NOT_CONVERGED. */

#define ORC_QT_MAX 64
#define ORC_QT_LAYERS 60

typedef struct { double lb[2], rt[2]; } qt_node;

static int qt_hull_check(const orc_surface* s, const qt_node* nd, const double* P, double max_edge) {
    const int p = s->degree_u, q = s->degree_v;
    const int i0 = orc_find_span(p, s->cp_u, s->knots_u, nd->lb[0]) - p;
    const int j0 = orc_find_span(q, s->cp_v, s->knots_v, nd->lb[1]) - q;
    const int i1 = orc_find_span(p, s->cp_u, s->knots_u, nd->rt[0]);
    const int j1 = orc_find_span(q, s->cp_v, s->knots_v, nd->rt[1]);
    double mn[3], mx[3];
    for (int c = 0; c < 3; ++c) mn[c] = mx[c] = s->cps[3 * ((int64_t)i0 * s->cp_v + j0) + c];
    for (int i = i0; i <= i1; ++i)
        for (int j = j0; j <= j1; ++j) {
            const double* x = s->cps + 3 * ((int64_t)i * s->cp_v + j);
            for (int c = 0; c < 3; ++c) {
                if (mn[c] > x[c]) mn[c] = x[c];
                if (mx[c] < x[c]) mx[c] = x[c];
            }
        }
    return P[0] >= mn[0] - max_edge && P[0] <= mx[0] + max_edge && P[1] >= mn[1] - max_edge &&
           P[1] <= mx[1] + max_edge && P[2] >= mn[2] - max_edge && P[2] <= mx[2] + max_edge;
}

/* 0 NOT_SPLIT, 1 SPLIT_V, 2 SPLIT_U, 3 SPLIT_UV (getSplitType); as_reference: the v-length from
 * MatrixSurfaceDerivativeU with spanV, as the reference computes it (for pinning only). */
static int qt_split_type_x(const orc_surface* s, const double* M, const qt_node* nd, double max_edge,
                           int as_reference) {
    const int p = s->degree_u, q = s->degree_v;
    const double iu = (nd->rt[0] - nd->lb[0]) / 4, iv = (nd->rt[1] - nd->lb[1]) / 4;
    double ul = 0, vl = 0;
    for (int i = 0; i < 4; ++i) {
        span_loc L = locate(s, M, nd->lb[0] + i * iu, nd->lb[1] + i * iv);
        d4 R = R_of(L.middle, p, q, L.u, L.v);
        d3 a = der_u(L.middle, p, q, L.u, L.v, R, L.spanU);
        d3 b = as_reference ? der_u(L.middle, p, q, L.u, L.v, R, L.spanV) : der_v(L.middle, p, q, L.u, L.v, R, L.spanV);
        ul += sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
        vl += sqrt(b.x * b.x + b.y * b.y + b.z * b.z);
    }
    ul *= (nd->rt[0] - nd->lb[0]) * 0.25;
    vl *= (nd->rt[1] - nd->lb[1]) * 0.25;
    if (ul < max_edge && vl < max_edge) return 0;
    if (nd->rt[0] - nd->lb[0] > 0.25 || nd->rt[1] - nd->lb[1] > 0.25) return 3;
    if (ul < max_edge) return 1;
    if (vl < max_edge) return 2;
    return 3;
}

static int qt_split_type(const orc_surface* s, const double* M, const qt_node* nd, double max_edge) {
    return qt_split_type_x(s, M, nd, max_edge, 0);
}

int orc_qt_hull_check(const orc_surface* s, const double node4[4], const double P[3], double max_edge) {
    qt_node nd = {{node4[0], node4[1]}, {node4[2], node4[3]}};
    return qt_hull_check(s, &nd, P, max_edge);
}

int orc_qt_split_type(const orc_surface* s, const double* M, const double node4[4], double max_edge, int as_reference) {
    qt_node nd = {{node4[0], node4[1]}, {node4[2], node4[3]}};
    return qt_split_type_x(s, M, &nd, max_edge, as_reference);
}

/* children of nd by split type t, appended to out (the reference's order) */
static int qt_children(const qt_node* nd, int t, qt_node* out) {
    const double lx = nd->lb[0], ly = nd->lb[1], rx = nd->rt[0], ry = nd->rt[1];
    const double mx = (lx + rx) / 2, my = (ly + ry) / 2;
    if (t == 3) {
        qt_node c[4] = {{{lx, ly}, {mx, my}}, {{lx, my}, {mx, ry}}, {{mx, my}, {rx, ry}}, {{mx, ly}, {rx, my}}};
        memcpy(out, c, sizeof c);
        return 4;
    }
    if (t == 2) {
        qt_node c[2] = {{{lx, ly}, {mx, ry}}, {{mx, ly}, {rx, ry}}};
        memcpy(out, c, sizeof c);
        return 2;
    }
    if (t == 1) {
        qt_node c[2] = {{{lx, ly}, {rx, my}}, {{lx, my}, {rx, ry}}};
        memcpy(out, c, sizeof c);
        return 2;
    }
    return 0;
}

void orc_invert_quadtree(const orc_surface* s, const double* M, const double* P, int64_t n, double max_edge,
                         int max_iter, double* uv, int* status, double* residual, int* layers, int threads) {
    double dom[4];
    domain_of(s, dom);
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 16) num_threads(threads)
#endif
    for (int64_t k = 0; k < n; ++k) {
        const double* Pk = P + 3 * k;
        qt_node cur[ORC_QT_MAX], nxt[ORC_QT_MAX + 4];
        int size = 1, passed_any = 0, st = ORC_NOT_CONVERGED, layer = 0;
        double bu = NAN, bv = NAN, br = NAN;
        cur[0].lb[0] = dom[0]; cur[0].lb[1] = dom[2]; cur[0].rt[0] = dom[1]; cur[0].rt[1] = dom[3];
        for (; layer < ORC_QT_LAYERS && size > 0; ++layer) {
            unsigned char pass[ORC_QT_MAX];
            double su[ORC_QT_MAX][2], sr[ORC_QT_MAX];
            int ns = 0;
            for (int i = 0; i < size; ++i) {
                pass[i] = (unsigned char)qt_hull_check(s, &cur[i], Pk, max_edge);
                if (!pass[i]) continue;
                passed_any = 1;
                double C[2] = {(cur[i].lb[0] + cur[i].rt[0]) / 2, (cur[i].lb[1] + cur[i].rt[1]) / 2};
                int its;
                if (!run_trajectory(s, M, Pk, C, max_iter, 0, &its)) continue;
                if (!(C[0] >= dom[0] && C[0] <= dom[1] && C[1] >= dom[2] && C[1] <= dom[3])) continue;
                const double r = dist3(surface_point(s, M, C), Pk);
                if (!(r < max_edge)) continue;
                su[ns][0] = C[0];
                su[ns][1] = C[1];
                sr[ns] = r;
                ++ns;
            }
            if (ns > 0) {
                int b = 0;
                for (int t = 1; t < ns; ++t)
                    if (sr[t] < sr[b]) b = t;
                st = ORC_FOUND_UNIQUE;
                for (int t = 0; t < ns; ++t) {
                    const int same = fabs(su[t][0] - su[b][0]) <= 1e-7 && fabs(su[t][1] - su[b][1]) <= 1e-7;
                    if (!same && sr[t] <= sr[b] * (1 + 1e-6) + 1e-12) st = ORC_FOUND_AMBIGUOUS;
                }
                bu = su[b][0];
                bv = su[b][1];
                br = sr[b];
                break;
            }
            int nn = 0, overflow = 0;
            for (int i = 0; i < size && !overflow; ++i) {
                if (!pass[i]) continue;
                nn += qt_children(&cur[i], qt_split_type(s, M, &cur[i], max_edge), nxt + nn);
                overflow = nn > ORC_QT_MAX;
            }
            if (overflow) { ++layer; break; }
            if (nn == 0) {
                st = passed_any ? ORC_NOT_CONVERGED : ORC_NO_CANDIDATE;
                ++layer;
                break;
            }
            memcpy(cur, nxt, sizeof(qt_node) * nn);
            size = nn;
        }
        uv[2 * k] = bu;
        uv[2 * k + 1] = bv;
        status[k] = st;
        residual[k] = br;
        if (layers) layers[k] = layer;
    }
}
