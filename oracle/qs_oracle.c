/*
 * qs_oracle.c -- CPU restatement of QuSpin.jl's spin-1/2 symmetry-reduced basis
 * construction and matrix-free operator action.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library links, loads or calls
 * this file; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * use it, and only as the checker.
 *
 * Two independent restatements live here:
 *
 *  (1) The reference algorithm itself, operation for operation in IEEE double
 *      arithmetic (compile with -ffp-contract=off): Gosper enumeration of the
 *      parent sector, the explicit sparse projector P built by cyclic orbit walks
 *      and eigenspace intersections, argmax representatives, 1/|amp|^2
 *      normalisations, and the QuantumLinearOperator matvec done as
 *      lift (P x) -> scatter on the parent with per-state lookups -> project (P').
 *        src/basis.jl:229-250       _fixed_weight_states (Gosper)
 *        src/basis.jl:622-777       SpinBasis1D constructor (generator order)
 *        src/symmetry_basis.jl:38-55    _signed_permutation
 *        src/symmetry_basis.jl:57-108   _cyclic_projector
 *        src/symmetry_basis.jl:110-213  _intersect_eigenspace (permutation-like branch)
 *        src/symmetry_basis.jl:215-232  _representative_states
 *        src/discrete_basis.jl:2386-2422 representative / normalization / get_amp
 *        src/operators.jl:343-379   _apply_local
 *        src/operators.jl:2372-2429 diagonal extraction + projection
 *        src/operators.jl:2554-2636 _apply_spin_term! / _apply_spin_terms!
 *        src/operators.jl:3097-3179 _add_qlo_diagonal! / mul!
 *      Julia's scalar semantics that decide representatives bit for bit are
 *      restated from their published algorithms: complex division is the robust
 *      Baudin & Smith (2012) algorithm, abs(::Complex) is the correctly rounded
 *      hypot of Borges (2019) with FMA, and norm() of a short vector is the
 *      unscaled sum of abs2 followed by sqrt.  Sparse products follow the
 *      Gustavson column accumulation order of SparseArrays' spmatmul.
 *
 *  (2) A representative-space restatement (orbit minimum + character, group
 *      enumerated by closure of the generators) that scales to sectors whose
 *      parent sector is too large for (1).  It is threaded with OpenMP and is
 *      the CPU baseline where the reference algorithm is infeasible.
 */
#define _GNU_SOURCE
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORA_EXPORT __attribute__((visibility("default")))

typedef struct { double re, im; } cx;

static inline cx mkc(double r, double i) { cx z; z.re = r; z.im = i; return z; }
static inline cx cmul(cx z, cx w) {
    return mkc(z.re * w.re - z.im * w.im, z.re * w.im + z.im * w.re);
}
static inline cx cadd(cx a, cx b) { return mkc(a.re + b.re, a.im + b.im); }
static inline cx cconj(cx z) { return mkc(z.re, -z.im); }
static inline cx cdivr(cx z, double x) { return mkc(z.re / x, z.im / x); }
static inline double cabs2(cx z) { return z.re * z.re + z.im * z.im; }

/* Robust complex division, Baudin & Smith, "A Robust Complex Division in
 * Scilab" (2012); the form Julia uses for ComplexF64 '/'. */
static double rcdiv2(double a, double b, double c, double d, double r, double t) {
    if (r != 0) {
        double br = b * r;
        return (br != 0) ? (a + br) * t : a * t + (b * t) * r;
    }
    return (a + d * (b / c)) * t;
}
static void rcdiv1(double a, double b, double c, double d, double *p, double *q) {
    double r = d / c;
    double t = 1.0 / (c + d * r);
    *p = rcdiv2(a, b, c, d, r, t);
    *q = rcdiv2(b, -a, c, d, r, t);
}
static cx jl_cdiv(cx z, cx w) {
    double a = z.re, b = z.im, c = w.re, d = w.im;
    double absa = fabs(a), absb = fabs(b);
    double ab = absa >= absb ? absa : absb;
    double absc = fabs(c), absd = fabs(d);
    double cd = absc >= absd ? absc : absd;
    const double halfov = 0.5 * DBL_MAX;
    const double twoune = DBL_MIN * 2.0 / DBL_EPSILON;
    const double bs = 2.0 / (DBL_EPSILON * DBL_EPSILON);
    double s = 1.0, p, q;
    if (ab >= halfov) { a = 0.5 * a; b = 0.5 * b; s = 2.0; }
    if (cd >= halfov) { c = 0.5 * c; d = 0.5 * d; s = s * 0.5; }
    if (ab <= twoune) { a = a * bs; b = b * bs; s = s / bs; }
    if (cd <= twoune) { c = c * bs; d = d * bs; s = s * bs; }
    if (absd <= absc) {
        rcdiv1(a, b, c, d, &p, &q);
    } else {
        rcdiv1(b, a, d, c, &p, &q);
        q = -q;
    }
    return mkc(p * s, q * s);
}

/* Correctly rounded hypot (Borges, "An Improved Algorithm for hypot(a,b)",
 * ACM TOMS 2019), FMA-corrected form. */
static double jl_hypot(double x, double y) {
    if (isinf(x) || isinf(y)) return INFINITY;
    double ax = fabs(x), ay = fabs(y);
    if (ay > ax) { double t = ax; ax = ay; ay = t; }
    if (ay <= ax * sqrt(DBL_EPSILON / 2)) return ax;
    double scale = DBL_EPSILON * sqrt(DBL_MIN);
    if (ax > sqrt(DBL_MAX / 2)) {
        ax = ax * scale; ay = ay * scale; scale = 1.0 / scale;
    } else if (ay < sqrt(DBL_MIN)) {
        ax = ax / scale; ay = ay / scale;
    } else {
        scale = 1.0;
    }
    double h = sqrt(fma(ax, ax, ay * ay));
    double hsq = h * h;
    double axsq = ax * ax;
    h -= ((fma(-ay, ay, hsq - axsq) + fma(h, h, -hsq)) - fma(ax, ax, -axsq)) / (2 * h);
    return h * scale;
}
static inline double jl_cabs(cx z) { return jl_hypot(z.re, z.im); }

/* 2-norm of a short vector as LinearAlgebra.generic_norm2 computes it (no
 * scaling in the normal range).  Vectors of length >= 32 go to BLAS nrm2 in
 * the reference; this restatement uses the same formula for them, which is
 * exact for equal-magnitude real entries and otherwise unpinned. */
static double jl_norm2(const cx *v, int64_t n) {
    if (n == 0) return 0.0;
    double maxabs = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        double a = jl_cabs(v[i]);
        if (a > maxabs) maxabs = a;
    }
    if (maxabs == 0.0 || isinf(maxabs)) return maxabs;
    if (isfinite((double)n * maxabs * maxabs) && maxabs * maxabs != 0.0) {
        double sum = cabs2(v[0]);
        for (int64_t i = 1; i < n; ++i) sum += cabs2(v[i]);
        return sqrt(sum);
    }
    double sum = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        double q = jl_cabs(v[i]) / maxabs;
        sum = (i == 0) ? q * q : sum + q * q;
    }
    return maxabs * sqrt(sum);
}

static int jl_isapprox(cx a, cx b, double atol, double rtol) {
    double d = jl_cabs(mkc(a.re - b.re, a.im - b.im));
    double na = jl_cabs(a), nb = jl_cabs(b);
    double m = na > nb ? na : nb;
    double tol = atol > rtol * m ? atol : rtol * m;
    return d <= tol;
}

/* ------------------------------------------------------------------ sparse */
typedef struct {
    int64_t m, n;      /* rows, columns */
    int64_t *colptr;   /* n + 1 */
    int64_t *rowval;
    cx *nzval;
} csc_t;

static void csc_free(csc_t *a) {
    free(a->colptr); free(a->rowval); free(a->nzval);
    memset(a, 0, sizeof(*a));
}

typedef struct { int64_t row, col, ord; cx v; } trip_t;
static int trip_cmp(const void *x, const void *y) {
    const trip_t *a = (const trip_t *)x, *b = (const trip_t *)y;
    if (a->col != b->col) return a->col < b->col ? -1 : 1;
    if (a->row != b->row) return a->row < b->row ? -1 : 1;
    return a->ord < b->ord ? -1 : (a->ord > b->ord);
}
/* sparse(rows, cols, vals, m, n): duplicates summed in input order. */
static int csc_from_triplets(csc_t *out, int64_t m, int64_t n, int64_t nt,
                             const int64_t *rows, const int64_t *cols, const cx *vals) {
    trip_t *t = (trip_t *)malloc(sizeof(trip_t) * (nt ? nt : 1));
    if (!t) return -1;
    for (int64_t i = 0; i < nt; ++i) { t[i].row = rows[i]; t[i].col = cols[i]; t[i].v = vals[i]; t[i].ord = i; }
    qsort(t, nt, sizeof(trip_t), trip_cmp);
    out->m = m; out->n = n;
    out->colptr = (int64_t *)calloc(n + 1, sizeof(int64_t));
    out->rowval = (int64_t *)malloc(sizeof(int64_t) * (nt ? nt : 1));
    out->nzval = (cx *)malloc(sizeof(cx) * (nt ? nt : 1));
    int64_t k = 0;
    for (int64_t i = 0; i < nt; ++i) {
        if (k > 0 && t[i].col == t[i - 1].col && t[i].row == out->rowval[k - 1]) {
            out->nzval[k - 1] = cadd(out->nzval[k - 1], t[i].v);
            continue;
        }
        out->rowval[k] = t[i].row; out->nzval[k] = t[i].v; k++;
        out->colptr[t[i].col + 1]++;
    }
    for (int64_t j = 0; j < n; ++j) out->colptr[j + 1] += out->colptr[j];
    free(t);
    return 0;
}
/* copy(adjoint(A)) */
static void csc_adjoint(csc_t *out, const csc_t *a) {
    int64_t nnz = a->colptr[a->n];
    out->m = a->n; out->n = a->m;
    out->colptr = (int64_t *)calloc(out->n + 1, sizeof(int64_t));
    out->rowval = (int64_t *)malloc(sizeof(int64_t) * (nnz ? nnz : 1));
    out->nzval = (cx *)malloc(sizeof(cx) * (nnz ? nnz : 1));
    for (int64_t p = 0; p < nnz; ++p) out->colptr[a->rowval[p] + 1]++;
    for (int64_t j = 0; j < out->n; ++j) out->colptr[j + 1] += out->colptr[j];
    int64_t *next = (int64_t *)malloc(sizeof(int64_t) * (out->n + 1));
    memcpy(next, out->colptr, sizeof(int64_t) * (out->n + 1));
    for (int64_t j = 0; j < a->n; ++j)
        for (int64_t p = a->colptr[j]; p < a->colptr[j + 1]; ++p) {
            int64_t q = next[a->rowval[p]]++;
            out->rowval[q] = j;
            out->nzval[q] = cconj(a->nzval[p]);
        }
    free(next);
}
static int cmp_i64(const void *x, const void *y) {
    int64_t a = *(const int64_t *)x, b = *(const int64_t *)y;
    return a < b ? -1 : (a > b);
}
/* spmatmul(A, B): for each column of B, walk its nonzeros in stored order and
 * accumulate A[:,k]*B[k,j] into the output column (first product assigned, later
 * ones added), rows sorted afterwards. */
static int csc_matmul(csc_t *out, const csc_t *A, const csc_t *B) {
    int64_t m = A->m, n = B->n;
    cx *acc = (cx *)malloc(sizeof(cx) * (m ? m : 1));
    char *seen = (char *)calloc(m ? m : 1, 1);
    int64_t *rows = (int64_t *)malloc(sizeof(int64_t) * (m ? m : 1));
    int64_t cap = 16, nnz = 0;
    out->m = m; out->n = n;
    out->colptr = (int64_t *)calloc(n + 1, sizeof(int64_t));
    out->rowval = (int64_t *)malloc(sizeof(int64_t) * cap);
    out->nzval = (cx *)malloc(sizeof(cx) * cap);
    for (int64_t j = 0; j < n; ++j) {
        int64_t cnt = 0;
        for (int64_t pb = B->colptr[j]; pb < B->colptr[j + 1]; ++pb) {
            int64_t k = B->rowval[pb];
            cx nzb = B->nzval[pb];
            for (int64_t pa = A->colptr[k]; pa < A->colptr[k + 1]; ++pa) {
                cx prod = cmul(A->nzval[pa], nzb);
                int64_t i = A->rowval[pa];
                if (seen[i]) acc[i] = cadd(acc[i], prod);
                else { seen[i] = 1; acc[i] = prod; rows[cnt++] = i; }
            }
        }
        qsort(rows, cnt, sizeof(int64_t), cmp_i64);
        if (nnz + cnt > cap) {
            while (nnz + cnt > cap) cap *= 2;
            out->rowval = (int64_t *)realloc(out->rowval, sizeof(int64_t) * cap);
            out->nzval = (cx *)realloc(out->nzval, sizeof(cx) * cap);
        }
        for (int64_t q = 0; q < cnt; ++q) {
            out->rowval[nnz] = rows[q]; out->nzval[nnz] = acc[rows[q]]; nnz++;
            seen[rows[q]] = 0;
        }
        out->colptr[j + 1] = nnz;
    }
    free(acc); free(seen); free(rows);
    return 0;
}
/* droptol!(A, tol): keep entries with abs(x) > tol. */
static void csc_droptol(csc_t *a, double tol) {
    int64_t k = 0, start = 0;
    for (int64_t j = 0; j < a->n; ++j) {
        int64_t end = a->colptr[j + 1];
        for (int64_t p = start; p < end; ++p)
            if (jl_cabs(a->nzval[p]) > tol) { a->rowval[k] = a->rowval[p]; a->nzval[k] = a->nzval[p]; k++; }
        start = end;
        a->colptr[j + 1] = k;
    }
}

/* ------------------------------------------------------------- bit helpers */
static inline uint64_t lmask(int L) { return L >= 64 ? ~0ULL : ((1ULL << L) - 1ULL); }
static inline uint64_t rotl_L(uint64_t s, int L, int k) {
    k %= L; if (k < 0) k += L;
    if (k == 0) return s;
    return ((s << k) | (s >> (L - k))) & lmask(L);
}
static inline uint64_t brev_L(uint64_t s, int L) {
    uint64_t r = 0;
    for (int b = 0; b < L; ++b) if (s >> b & 1ULL) r |= 1ULL << (L - 1 - b);
    return r;
}

/* Symmetry generators in the order the reference applies them
 * (basis.jl:691-735): translation first, then p, z, pz, zA, zB. */
enum { G_T = 0, G_P, G_Z, G_PZ, G_ZA, G_ZB, G_GEN };
/* G_GEN: a general site map (_general_spin_transform, src/basis.jl:325-337):
 * source site b goes to perm[b], its spin flipped where flips has bit b. */
typedef struct { int kind; int L, a; uint64_t full, odd, even; int perm[64]; uint64_t flips; } xform_t;
static uint64_t xform_apply(const xform_t *x, uint64_t s) {
    if (x->kind == G_GEN) {
        uint64_t t = 0;
        for (int b = 0; b < x->L; ++b) {
            int occupied = (int)((s >> b) & 1ULL);
            if ((x->flips >> b) & 1ULL) occupied = !occupied;
            if (occupied) t |= 1ULL << x->perm[b];
        }
        return t;
    }
    switch (x->kind) {
    case G_T: return rotl_L(s, x->L, x->a);
    case G_P: return brev_L(s, x->L);
    case G_Z: return s ^ x->full;
    case G_PZ: return brev_L(s, x->L) ^ x->full;
    case G_ZA: return s ^ x->odd;
    default: return s ^ x->even;
    }
}

/* ------------------------------------------------------------------- basis */
typedef struct {
    int L, nup, pauli, reduced;
    int64_t n_parent;
    uint64_t *parent;         /* ascending */
    csc_t P;                  /* n_parent x n */
    int64_t n;
    uint64_t *states;         /* argmax representatives, column order */
    int64_t *row_col;         /* parent row -> column (-1 if none) */
    cx *row_val;              /* parent row -> projector value */
    int64_t *sorted_idx;      /* permutation sorting states ascending */
} ora_basis;

static int64_t find_u64(const uint64_t *a, int64_t n, uint64_t key) {
    int64_t lo = 0, hi = n;
    while (lo < hi) { int64_t mid = lo + (hi - lo) / 2; if (a[mid] < key) lo = mid + 1; else hi = mid; }
    return (lo < n && a[lo] == key) ? lo : -1;
}

static void set_err(char *err, int errlen, const char *msg) {
    if (err && errlen > 0) { strncpy(err, msg, errlen - 1); err[errlen - 1] = 0; }
}

static int64_t binom_i64(int n, int k) {
    if (k < 0 || k > n) return 0;
    int64_t r = 1;
    for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
    return r;
}

static int enumerate_parent(int L, int nup, uint64_t **out, int64_t *count) {
    if (nup < 0) {
        int64_t n = (int64_t)1 << L;
        uint64_t *s = (uint64_t *)malloc(sizeof(uint64_t) * n);
        if (!s) return -1;
        for (int64_t i = 0; i < n; ++i) s[i] = (uint64_t)i;
        *out = s; *count = n; return 0;
    }
    int64_t n = binom_i64(L, nup);
    uint64_t *s = (uint64_t *)malloc(sizeof(uint64_t) * (n ? n : 1));
    if (!s) return -1;
    if (nup == 0) { s[0] = 0; *out = s; *count = 1; return 0; }
    if (nup == L) { s[0] = lmask(L); *out = s; *count = 1; return 0; }
    uint64_t state = (1ULL << nup) - 1ULL;
    for (int64_t i = 0; i < n; ++i) {
        s[i] = state;
        if (i == n - 1) break;
        uint64_t lowest = state & (~state + 1ULL);
        uint64_t next = state + lowest;
        state = next | ((next ^ state) >> (__builtin_ctzll(lowest) + 2));
    }
    *out = s; *count = n; return 0;
}

/* _cyclic_projector (symmetry_basis.jl:57-108) */
static int cyclic_projector(csc_t *out, const uint64_t *st, int64_t n, const xform_t *x, cx eig,
                            char *err, int errlen) {
    char *visited = (char *)calloc(n ? n : 1, 1);
    int64_t cap = n ? n : 1, nt = 0, ncol = 0;
    int64_t *rows = (int64_t *)malloc(sizeof(int64_t) * cap);
    int64_t *cols = (int64_t *)malloc(sizeof(int64_t) * cap);
    cx *vals = (cx *)malloc(sizeof(cx) * cap);
    int64_t *orbit = (int64_t *)malloc(sizeof(int64_t) * 256);
    cx *coef = (cx *)malloc(sizeof(cx) * 256);
    int rc = 0;
    for (int64_t start = 0; start < n; ++start) {
        if (visited[start]) continue;
        int64_t len = 0, cur = start;
        for (;;) {
            orbit[len++] = cur;
            visited[cur] = 1;
            int64_t nxt = find_u64(st, n, xform_apply(x, st[cur]));
            if (nxt < 0) { set_err(err, errlen, "symmetry transformation leaves the selected particle sector"); rc = -2; goto done; }
            if (nxt == start) break;
            for (int64_t q = 0; q < len; ++q)
                if (orbit[q] == nxt) { set_err(err, errlen, "symmetry map produced a non-cyclic orbit"); rc = -2; goto done; }
            if (len >= 256) { set_err(err, errlen, "orbit too long"); rc = -2; goto done; }
            cur = nxt;
        }
        coef[0] = mkc(1.0, 0.0);
        for (int64_t j = 1; j < len; ++j) coef[j] = jl_cdiv(cmul(coef[j - 1], mkc(1.0, 0.0)), eig);
        cx closure = cmul(coef[len - 1], mkc(1.0, 0.0));
        if (!jl_isapprox(closure, cmul(eig, coef[0]), 2e-10, 2e-10)) continue;
        double nrm = jl_norm2(coef, len);
        for (int64_t j = 0; j < len; ++j) {
            rows[nt] = orbit[j]; cols[nt] = ncol; vals[nt] = cdivr(coef[j], nrm); nt++;
        }
        ncol++;
    }
    csc_from_triplets(out, n, ncol, nt, rows, cols, vals);
done:
    free(visited); free(rows); free(cols); free(vals); free(orbit); free(coef);
    return rc;
}

/* _intersect_eigenspace, permutation-like branch (symmetry_basis.jl:110-198) */
static int intersect_eigenspace(csc_t *out, csc_t *P, const uint64_t *st, int64_t n, const xform_t *x,
                                cx eig, char *err, int errlen) {
    if (P->n == 0) { *out = *P; memset(P, 0, sizeof(*P)); return 0; }
    /* _signed_permutation: S[row(T s_col), col] = 1 */
    int64_t *srows = (int64_t *)malloc(sizeof(int64_t) * n);
    int64_t *scols = (int64_t *)malloc(sizeof(int64_t) * n);
    cx *svals = (cx *)malloc(sizeof(cx) * n);
    for (int64_t c = 0; c < n; ++c) {
        int64_t r = find_u64(st, n, xform_apply(x, st[c]));
        if (r < 0) {
            free(srows); free(scols); free(svals);
            set_err(err, errlen, "symmetry transformation leaves the selected particle sector");
            return -2;
        }
        srows[c] = r; scols[c] = c; svals[c] = mkc(1.0, 0.0);
    }
    csc_t S, Pa, PaS, R;
    csc_from_triplets(&S, n, n, n, srows, scols, svals);
    free(srows); free(scols); free(svals);
    csc_adjoint(&Pa, P);
    csc_matmul(&PaS, &Pa, &S);
    csc_matmul(&R, &PaS, P);
    csc_free(&S); csc_free(&Pa); csc_free(&PaS);
    csc_droptol(&R, 5e-12);
    int64_t rd = R.n;
    int64_t *mrow = (int64_t *)malloc(sizeof(int64_t) * rd);
    cx *mph = (cx *)malloc(sizeof(cx) * rd);
    int perm_like = 1;
    for (int64_t c = 0; c < rd; ++c) {
        if (R.colptr[c + 1] - R.colptr[c] != 1) { perm_like = 0; break; }
        int64_t p = R.colptr[c];
        mrow[c] = R.rowval[p]; mph[c] = R.nzval[p];
        if (!jl_isapprox(mkc(jl_cabs(mph[c]), 0.0), mkc(1.0, 0.0), 2e-10, 2e-10)) { perm_like = 0; break; }
    }
    if (perm_like) {
        char *hit = (char *)calloc(rd, 1);
        for (int64_t c = 0; c < rd; ++c) { if (hit[mrow[c]]) { perm_like = 0; break; } hit[mrow[c]] = 1; }
        free(hit);
    }
    csc_free(&R);
    if (!perm_like) {
        free(mrow); free(mph);
        set_err(err, errlen, "symmetry intersection is not permutation-like (dense nullspace fallback is not restated)");
        return -3;
    }
    char *visited = (char *)calloc(rd, 1);
    int64_t *rows = (int64_t *)malloc(sizeof(int64_t) * rd);
    int64_t *cols = (int64_t *)malloc(sizeof(int64_t) * rd);
    cx *vals = (cx *)malloc(sizeof(cx) * rd);
    int64_t *orbit = (int64_t *)malloc(sizeof(int64_t) * (rd + 1));
    cx *ph = (cx *)malloc(sizeof(cx) * (rd + 1));
    cx *coef = (cx *)malloc(sizeof(cx) * (rd + 1));
    int64_t nt = 0, ncol = 0;
    for (int64_t start = 0; start < rd; ++start) {
        if (visited[start]) continue;
        int64_t len = 0, cur = start;
        int broke = 0;
        for (;;) {
            orbit[len] = cur; visited[cur] = 1; ph[len] = mph[cur]; len++;
            int64_t nxt = mrow[cur];
            if (nxt == start) break;
            if (visited[nxt]) { broke = 1; break; }
            cur = nxt;
        }
        if (broke) { perm_like = 0; break; }
        coef[0] = mkc(1.0, 0.0);
        for (int64_t j = 1; j < len; ++j) coef[j] = jl_cdiv(cmul(coef[j - 1], ph[j - 1]), eig);
        cx closure = cmul(coef[len - 1], ph[len - 1]);
        if (!jl_isapprox(closure, cmul(eig, coef[0]), 2e-10, 2e-10)) continue;
        double nrm = jl_norm2(coef, len);
        for (int64_t j = 0; j < len; ++j) { rows[nt] = orbit[j]; cols[nt] = ncol; vals[nt] = cdivr(coef[j], nrm); nt++; }
        ncol++;
    }
    free(visited); free(mrow); free(mph); free(orbit); free(ph); free(coef);
    if (!perm_like) {
        free(rows); free(cols); free(vals);
        set_err(err, errlen, "symmetry intersection is not permutation-like (dense nullspace fallback is not restated)");
        return -3;
    }
    csc_t Rp;
    csc_from_triplets(&Rp, rd, ncol, nt, rows, cols, vals);
    free(rows); free(cols); free(vals);
    csc_matmul(out, P, &Rp);
    csc_free(&Rp);
    csc_droptol(out, 5e-14);
    return 0;
}

ORA_EXPORT void ora_basis_free(ora_basis *b) {
    if (!b) return;
    free(b->parent); csc_free(&b->P); free(b->states); free(b->row_col); free(b->row_val); free(b->sorted_idx);
    free(b);
}

static ora_basis *sorted_states_b;
static int cmp_state_idx(const void *x, const void *y) {
    uint64_t a = sorted_states_b->states[*(const int64_t *)x], c = sorted_states_b->states[*(const int64_t *)y];
    return a < c ? -1 : (a > c);
}

static int finish_reduced(ora_basis *b, csc_t P, ora_basis **out, char *err, int errlen);

/* sym[0..5] = {has_k? k : unused, p, z, pz, zA, zB} with 0 meaning "not given". */
ORA_EXPORT int ora_basis_create(int L, int nup, int pauli, int a, int has_k, int k,
                                int p, int z, int pz, int za, int zb,
                                ora_basis **out, char *err, int errlen) {
    *out = NULL;
    if (L < 1 || L > 40) { set_err(err, errlen, "L outside the oracle's range"); return -1; }
    if (nup >= 0 && nup > L) { set_err(err, errlen, "nup must lie between 0 and L"); return -1; }
    ora_basis *b = (ora_basis *)calloc(1, sizeof(ora_basis));
    b->L = L; b->nup = nup; b->pauli = pauli;
    if (nup < 0 && L > 26) { free(b); set_err(err, errlen, "parent sector too large for the oracle"); return -1; }
    if (nup >= 0 && binom_i64(L, nup) > 40000000) { free(b); set_err(err, errlen, "parent sector too large for the oracle"); return -1; }
    if (enumerate_parent(L, nup, &b->parent, &b->n_parent)) { free(b); set_err(err, errlen, "allocation failed"); return -1; }
    int requested = has_k || p || z || pz || za || zb;
    if (!requested) {
        b->reduced = 0;
        b->n = b->n_parent;
        b->states = (uint64_t *)malloc(sizeof(uint64_t) * b->n);
        memcpy(b->states, b->parent, sizeof(uint64_t) * b->n);
        *out = b; return 0;
    }
    if (a <= 0 || L % a != 0) { ora_basis_free(b); set_err(err, errlen, "a must be a positive divisor of L"); return -1; }
    int order = L / a;
    xform_t xf; xf.L = L; xf.a = a; xf.full = lmask(L); xf.odd = 0; xf.even = 0;
    for (int s = 1; s <= L; s += 2) xf.odd |= 1ULL << (s - 1);
    for (int s = 2; s <= L; s += 2) xf.even |= 1ULL << (s - 1);
    csc_t P; memset(&P, 0, sizeof(P));
    int haveP = 0, rc = 0;
    if (has_k) {
        int mom = ((k % order) + order) % order;
        double arg = 2 * M_PI * (double)mom / (double)order;
        cx eig = mkc(cos(arg), sin(arg));
        xf.kind = G_T;
        rc = cyclic_projector(&P, b->parent, b->n_parent, &xf, eig, err, errlen);
        if (rc) { ora_basis_free(b); return rc; }
        haveP = 1;
        if (p) {
            if (!(mom == 0 || (order % 2 == 0 && mom == order / 2))) {
                csc_free(&P); ora_basis_free(b);
                set_err(err, errlen, "pblock can be combined with kblock only at k=0 or pi");
                return -1;
            }
        }
    }
    int vals[5] = {p, z, pz, za, zb};
    int kinds[5] = {G_P, G_Z, G_PZ, G_ZA, G_ZB};
    for (int g = 0; g < 5; ++g) {
        if (!vals[g]) continue;
        if (vals[g] != 1 && vals[g] != -1) { if (haveP) csc_free(&P); ora_basis_free(b); set_err(err, errlen, "block must be +1 or -1"); return -1; }
        xf.kind = kinds[g];
        cx eig = mkc((double)vals[g], 0.0);
        if (!haveP) {
            rc = cyclic_projector(&P, b->parent, b->n_parent, &xf, eig, err, errlen);
            haveP = 1;
        } else {
            csc_t Q;
            rc = intersect_eigenspace(&Q, &P, b->parent, b->n_parent, &xf, eig, err, errlen);
            if (!rc) { csc_free(&P); P = Q; }
        }
        if (rc) { if (haveP) csc_free(&P); ora_basis_free(b); return rc; }
    }
    return finish_reduced(b, P, out, err, errlen);
}

/* The reduced basis from its projector: argmax representatives in column
 * order and the row -> column map (src/symmetry_basis.jl:215-255). */
static int finish_reduced(ora_basis *b, csc_t P, ora_basis **out, char *err, int errlen) {
    if (P.n == 0) { csc_free(&P); ora_basis_free(b); set_err(err, errlen, "the requested symmetry sector is empty"); return -4; }
    b->reduced = 1;
    b->P = P;
    b->n = P.n;
    b->states = (uint64_t *)malloc(sizeof(uint64_t) * b->n);
    b->row_col = (int64_t *)malloc(sizeof(int64_t) * b->n_parent);
    b->row_val = (cx *)malloc(sizeof(cx) * b->n_parent);
    for (int64_t r = 0; r < b->n_parent; ++r) { b->row_col[r] = -1; b->row_val[r] = mkc(0, 0); }
    int64_t ncols_kept = 0;
    for (int64_t c = 0; c < P.n; ++c) {
        int64_t p0 = P.colptr[c], p1 = P.colptr[c + 1];
        for (int64_t q = p0; q < p1; ++q) { b->row_col[P.rowval[q]] = c; b->row_val[P.rowval[q]] = P.nzval[q]; }
        if (p1 == p0) continue;
        int64_t largest = p0;
        for (int64_t q = p0 + 1; q < p1; ++q)
            if (jl_cabs(P.nzval[q]) > jl_cabs(P.nzval[largest])) largest = q;
        b->states[ncols_kept++] = b->parent[P.rowval[largest]];
    }
    b->n = ncols_kept;
    b->sorted_idx = (int64_t *)malloc(sizeof(int64_t) * (b->n ? b->n : 1));
    for (int64_t i = 0; i < b->n; ++i) b->sorted_idx[i] = i;
    sorted_states_b = b;
    qsort(b->sorted_idx, b->n, sizeof(int64_t), cmp_state_idx);
    *out = b;
    return 0;
}

/* SpinBasisGeneral (src/basis.jl:455-600) for spin 1/2: nmaps blocks in
 * intersection order; perms[i * L + b] is the 0-based target of source site b,
 * flips[i * L + b] marks a flipped spin.  Order and eigenvalue as
 * _general_spin_map_order (src/basis.jl:305-323) and cis(2 pi mod(q, order) / order). */
ORA_EXPORT int ora_basis_create_general(int L, int nup, int pauli, int nmaps, const int *perms, const int *flips,
                                        const int *qnums, ora_basis **out, char *err, int errlen) {
    *out = NULL;
    if (L < 1 || L > 40) { set_err(err, errlen, "L outside the oracle's range"); return -1; }
    if (nup >= 0 && nup > L) { set_err(err, errlen, "nup must lie between 0 and L"); return -1; }
    ora_basis *b = (ora_basis *)calloc(1, sizeof(ora_basis));
    b->L = L; b->nup = nup; b->pauli = pauli;
    if (nup < 0 && L > 26) { free(b); set_err(err, errlen, "parent sector too large for the oracle"); return -1; }
    if (nup >= 0 && binom_i64(L, nup) > 40000000) { free(b); set_err(err, errlen, "parent sector too large for the oracle"); return -1; }
    if (enumerate_parent(L, nup, &b->parent, &b->n_parent)) { free(b); set_err(err, errlen, "allocation failed"); return -1; }
    if (nmaps == 0) {
        b->reduced = 0;
        b->n = b->n_parent;
        b->states = (uint64_t *)malloc(sizeof(uint64_t) * b->n);
        memcpy(b->states, b->parent, sizeof(uint64_t) * b->n);
        *out = b; return 0;
    }
    csc_t P; memset(&P, 0, sizeof(P));
    for (int i = 0; i < nmaps; ++i) {
        xform_t xf; memset(&xf, 0, sizeof(xf));
        xf.kind = G_GEN; xf.L = L;
        for (int s = 0; s < L; ++s) {
            xf.perm[s] = perms[i * L + s];
            if (flips[i * L + s]) xf.flips |= 1ULL << s;
        }
        long order = 1;
        char seen[64] = {0};
        for (int st = 0; st < L; ++st) {
            if (seen[st]) continue;
            int len = 0, par = 0, cur = st;
            while (!seen[cur]) { seen[cur] = 1; ++len; par ^= (int)((xf.flips >> cur) & 1ULL); cur = xf.perm[cur]; }
            long c = par ? 2L * len : (long)len, a = order, bb = c;
            while (bb) { long t = a % bb; a = bb; bb = t; }
            order = order / a * c;
        }
        long q = ((long)qnums[i] % order + order) % order;
        double arg = 2 * M_PI * (double)q / (double)order;
        cx eig = mkc(cos(arg), sin(arg));
        int rc;
        if (i == 0) {
            rc = cyclic_projector(&P, b->parent, b->n_parent, &xf, eig, err, errlen);
        } else {
            csc_t Q;
            rc = intersect_eigenspace(&Q, &P, b->parent, b->n_parent, &xf, eig, err, errlen);
            if (!rc) { csc_free(&P); P = Q; }
        }
        if (rc) { csc_free(&P); ora_basis_free(b); return rc; }
    }
    return finish_reduced(b, P, out, err, errlen);
}

ORA_EXPORT int64_t ora_basis_size(const ora_basis *b) { return b->n; }
ORA_EXPORT int64_t ora_basis_parent_size(const ora_basis *b) { return b->n_parent; }
ORA_EXPORT int ora_basis_reduced(const ora_basis *b) { return b->reduced; }
ORA_EXPORT void ora_basis_states(const ora_basis *b, uint64_t *out) { memcpy(out, b->states, sizeof(uint64_t) * b->n); }
ORA_EXPORT void ora_basis_parent_states(const ora_basis *b, uint64_t *out) { memcpy(out, b->parent, sizeof(uint64_t) * b->n_parent); }
ORA_EXPORT int64_t ora_basis_projector_nnz(const ora_basis *b) { return b->reduced ? b->P.colptr[b->P.n] : 0; }
/* CSC export: colptr (n+1), rowval (nnz), values (2*nnz interleaved re,im) */
ORA_EXPORT void ora_basis_projector(const ora_basis *b, int64_t *colptr, int64_t *rowval, double *vals) {
    if (!b->reduced) return;
    int64_t nnz = b->P.colptr[b->P.n];
    memcpy(colptr, b->P.colptr, sizeof(int64_t) * (b->P.n + 1));
    memcpy(rowval, b->P.rowval, sizeof(int64_t) * nnz);
    memcpy(vals, b->P.nzval, sizeof(cx) * nnz);
}
/* state_index (basis.jl:1016-1022): 0-based column of a representative, -1 if absent. */
ORA_EXPORT int64_t ora_state_index(const ora_basis *b, uint64_t s) {
    int64_t lo = 0, hi = b->n;
    while (lo < hi) { int64_t mid = lo + (hi - lo) / 2; if (b->states[b->sorted_idx ? b->sorted_idx[mid] : mid] < s) lo = mid + 1; else hi = mid; }
    if (lo < b->n) { int64_t c = b->sorted_idx ? b->sorted_idx[lo] : lo; if (b->states[c] == s) return c; }
    return -1;
}
/* representative / normalization / get_amp (discrete_basis.jl:2386-2422).
 * Returns 0 on success, -1 outside the parent sector, -2 zero weight. */
ORA_EXPORT int ora_representative(const ora_basis *b, uint64_t s, uint64_t *rep, double *norm, double *amp) {
    if (!b->reduced) { *rep = s; *norm = 1.0; amp[0] = 1.0; amp[1] = 0.0; return 0; }
    int64_t r = find_u64(b->parent, b->n_parent, s);
    if (r < 0) return -1;
    int64_t c = b->row_col[r];
    if (c < 0) return -2;
    cx v = b->row_val[r];
    *rep = b->states[c];
    *norm = 1.0 / cabs2(v);
    amp[0] = v.re; amp[1] = v.im;
    return 0;
}

/* ------------------------------------------------------------ term program */
/* Terms are passed flattened: for term t, op string ops[t*8 .. t*8+oplen[t]),
 * couplings coup_off[t] .. coup_off[t+1] with coefficient coef[2*c], coef[2*c+1]
 * and one-based sites sites[c*8 + i]. */
typedef struct {
    int nterms;
    const char *ops; const int *oplen; const int64_t *coup_off;
    const double *coef; const int *sites;
} terms_t;

/* _apply_local (operators.jl:343-379) */
static int apply_local(int pauli, uint64_t *state, char op, int site, cx *factor) {
    uint64_t mask = 1ULL << (site - 1);
    int occ = (*state & mask) != 0;
    switch (op) {
    case 'I': *factor = mkc(1.0, 0.0); return 1;
    case 'z': { double sc = pauli ? 1.0 : 0.5; *factor = mkc(occ ? sc : -sc, 0.0); return 1; }
    case '+': if (occ) return 0; *state |= mask; *factor = mkc(pauli ? 2.0 : 1.0, 0.0); return 1;
    case '-': if (!occ) return 0; *state &= ~mask; *factor = mkc(pauli ? 2.0 : 1.0, 0.0); return 1;
    case 'x': *state ^= mask; *factor = mkc(pauli ? 1.0 : 0.5, 0.0); return 1;
    case 'y': { double sc = pauli ? 1.0 : 0.5; *state ^= mask; *factor = occ ? mkc(0.0, -sc) : mkc(0.0, sc); return 1; }
    default: return -1;
    }
}
static int is_diag_op(const char *op, int len) {
    for (int i = 0; i < len; ++i) if (op[i] != 'I' && op[i] != 'z' && op[i] != 'n' && op[i] != '|') return 0;
    return 1;
}

/* Scatter one term list over `states` (operators.jl:2554-2589).  `dst += alpha *
 * A x` with A the (optionally transposed / conjugated) term matrix. */
static int apply_terms_scatter(int pauli, const uint64_t *states, int64_t n, const terms_t *T,
                               const char *use_term, const cx *x, cx *dst, cx alpha, int transposed, int conjugated) {
    for (int t = 0; t < T->nterms; ++t) {
        if (use_term && !use_term[t]) continue;
        const char *op = T->ops + 8 * t; int len = T->oplen[t];
        for (int64_t c = T->coup_off[t]; c < T->coup_off[t + 1]; ++c) {
            cx coefficient = cmul(alpha, mkc(T->coef[2 * c], T->coef[2 * c + 1]));
            const int *sites = T->sites + 8 * c;
            for (int64_t col = 0; col < n; ++col) {
                cx amp = coefficient; uint64_t st = states[col]; int alive = 1;
                for (int i = len - 1; i >= 0; --i) {
                    cx f; int r = apply_local(pauli, &st, op[i], sites[i], &f);
                    if (r < 0) return -1;
                    if (!r) { alive = 0; break; }
                    amp = cmul(amp, f);
                }
                if (!alive) continue;
                int64_t row = find_u64(states, n, st);
                if (row < 0) continue;
                cx tr = conjugated ? cconj(amp) : amp;
                int64_t src = transposed ? row : col, dstix = transposed ? col : row;
                cx in = x[src];
                if (in.re == 0.0 && in.im == 0.0) continue;
                dst[dstix] = cadd(dst[dstix], cmul(tr, in));
            }
        }
    }
    return 0;
}

/* Extracted diagonal (operators.jl:2372-2429): parent diagonal of structurally
 * diagonal terms, projected with |P|^2.  out has length n (complex). */
ORA_EXPORT int ora_extract_diagonal(const ora_basis *b, int nterms, const char *ops, const int *oplen,
                                    const int64_t *coup_off, const double *coef, const int *sites, double *out) {
    terms_t T = {nterms, ops, oplen, coup_off, coef, sites};
    int64_t np = b->n_parent;
    cx *d = (cx *)calloc(np, sizeof(cx));
    for (int t = 0; t < nterms; ++t) {
        const char *op = ops + 8 * t; int len = oplen[t];
        if (!is_diag_op(op, len)) continue;
        for (int64_t c = coup_off[t]; c < coup_off[t + 1]; ++c) {
            const int *st8 = sites + 8 * c;
            for (int64_t col = 0; col < np; ++col) {
                cx amp = mkc(coef[2 * c], coef[2 * c + 1]); uint64_t st = b->parent[col]; int alive = 1;
                for (int i = len - 1; i >= 0; --i) {
                    cx f; int r = apply_local(b->pauli, &st, op[i], st8[i], &f);
                    if (r < 0) { free(d); return -1; }
                    if (!r) { alive = 0; break; }
                    amp = cmul(amp, f);
                }
                if (alive) d[col] = cadd(d[col], amp);
            }
        }
    }
    (void)T;
    cx *o = (cx *)out;
    if (!b->reduced) { memcpy(o, d, sizeof(cx) * np); free(d); return 0; }
    for (int64_t c = 0; c < b->P.n; ++c) {
        cx acc = mkc(0, 0);
        for (int64_t q = b->P.colptr[c]; q < b->P.colptr[c + 1]; ++q) {
            double w = cabs2(b->P.nzval[q]);
            acc = cadd(acc, cmul(mkc(w, 0.0), d[b->P.rowval[q]]));
        }
        o[c] = acc;
    }
    free(d);
    return 0;
}

/* QuantumLinearOperator mul!(y, op, x, alpha, beta) (operators.jl:3147-3179)
 * with the reference's symmetric path (lift by P, scatter on the parent,
 * project by P').  `extract` = 1 when diagonal terms were extracted at
 * construction (they are then skipped here and `diag` holds user + extracted
 * diagonal).  Vectors are complex interleaved. */
ORA_EXPORT int ora_qlo_matvec(const ora_basis *b, int nterms, const char *ops, const int *oplen,
                              const int64_t *coup_off, const double *coef, const int *sites,
                              int extract, const double *diag, int transposed, int conjugated,
                              const double *alpha_, const double *beta_, const double *x_, double *y_) {
    terms_t T = {nterms, ops, oplen, coup_off, coef, sites};
    const cx *x = (const cx *)x_; cx *y = (cx *)y_;
    cx alpha = mkc(alpha_[0], alpha_[1]), beta = mkc(beta_[0], beta_[1]);
    int64_t n = b->n;
    char *use = (char *)malloc(nterms ? nterms : 1);
    for (int t = 0; t < nterms; ++t) use[t] = extract ? !is_diag_op(ops + 8 * t, oplen[t]) : 1;
    for (int64_t i = 0; i < n; ++i) y[i] = (beta.re == 0.0 && beta.im == 0.0) ? mkc(0, 0) : cmul(beta, y[i]);
    int rc = 0;
    if (!b->reduced) {
        rc = apply_terms_scatter(b->pauli, b->states, n, &T, use, x, y, alpha, transposed, conjugated);
    } else {
        int64_t np = b->n_parent;
        int ordinary = (transposed == conjugated);
        cx *lift = (cx *)calloc(np, sizeof(cx));
        cx *acted = (cx *)calloc(np, sizeof(cx));
        for (int64_t c = 0; c < b->P.n; ++c)
            for (int64_t q = b->P.colptr[c]; q < b->P.colptr[c + 1]; ++q) {
                cx pv = ordinary ? b->P.nzval[q] : cconj(b->P.nzval[q]);
                lift[b->P.rowval[q]] = cadd(lift[b->P.rowval[q]], cmul(pv, x[c]));
            }
        rc = apply_terms_scatter(b->pauli, b->parent, np, &T, use, lift, acted, mkc(1.0, 0.0), transposed, conjugated);
        for (int64_t c = 0; c < b->P.n; ++c) {
            cx acc = mkc(0, 0);
            for (int64_t q = b->P.colptr[c]; q < b->P.colptr[c + 1]; ++q) {
                cx pv = ordinary ? cconj(b->P.nzval[q]) : b->P.nzval[q];
                acc = cadd(acc, cmul(pv, acted[b->P.rowval[q]]));
            }
            y[c] = cadd(y[c], cmul(alpha, acc));
        }
        free(lift); free(acted);
    }
    if (diag) {
        const cx *d = (const cx *)diag;
        for (int64_t i = 0; i < n; ++i) {
            cx dc = conjugated ? cconj(d[i]) : d[i];
            y[i] = cadd(y[i], cmul(cmul(alpha, dc), x[i]));
        }
    }
    free(use);
    return rc;
}

static uint64_t gosper_next(uint64_t s) {
    uint64_t lowest = s & (~s + 1ULL);
    uint64_t next = s + lowest;
    return next | (((next ^ s) >> 2) >> __builtin_ctzll(lowest));
}
/* state of combinadic rank r among the L-bit states of weight nup */
static uint64_t unrank_fixed(int64_t r, int L, int nup) {
    uint64_t s = 0;
    int b = L - 1;
    for (int p = nup; p >= 1; --p) {
        while (binom_i64(b, p) > r) --b;
        s |= 1ULL << b;
        r -= binom_i64(b, p);
        --b;
    }
    return s;
}

/* ==================================================================
 * (2) Representative-space restatement.
 * ================================================================== */
typedef struct { uint64_t img[65]; int shift, refl; uint64_t mask; cx chi; } gelem_t;

typedef struct {
    int L, nup, pauli;
    int ng;
    gelem_t *g;            /* group elements: s -> rotl(R^refl s, shift) ^ mask */
    int64_t n;
    uint64_t *reps;        /* ascending orbit minima with trivial character on the stabiliser */
    int32_t *orbit;        /* orbit size of each representative */
} ora_rbasis;

static uint64_t gapply(const gelem_t *e, uint64_t s, int L) {
    uint64_t r = e->refl ? brev_L(s, L) : s;
    return rotl_L(r, L, e->shift) ^ e->mask;
}
static int gsame(const gelem_t *a, const gelem_t *b, int L) {
    for (int i = 0; i <= L; ++i) if (a->img[i] != b->img[i]) return 0;
    return 1;
}
static void gfill(gelem_t *e, int L) {
    e->img[0] = gapply(e, 0, L);
    for (int bit = 0; bit < L; ++bit) e->img[bit + 1] = gapply(e, 1ULL << bit, L);
}
/* e2 o e1 */
static gelem_t gcompose(const gelem_t *e2, const gelem_t *e1, int L) {
    gelem_t r; memset(&r, 0, sizeof(r));
    int sh1 = e2->refl ? -e1->shift : e1->shift;
    r.shift = (((e2->shift + sh1) % L) + L) % L;
    r.refl = e1->refl ^ e2->refl;
    uint64_t m1 = e2->refl ? brev_L(e1->mask, L) : e1->mask;
    r.mask = rotl_L(m1, L, e2->shift) ^ e2->mask;
    r.chi = cmul(e2->chi, e1->chi);
    gfill(&r, L);
    return r;
}

ORA_EXPORT void ora_rbasis_free(ora_rbasis *b) {
    if (!b) return;
    free(b->g); free(b->reps); free(b->orbit); free(b);
}

static int rep_scan(const ora_rbasis *b, uint64_t t, uint64_t *minv, cx *chi, int *stab) {
    uint64_t best = ~0ULL; cx bc = mkc(1, 0); int cnt = 0;
    for (int i = 0; i < b->ng; ++i) {
        uint64_t v = gapply(&b->g[i], t, b->L);
        if (v < best) { best = v; bc = b->g[i].chi; cnt = 1; }
        else if (v == best) cnt++;
    }
    *minv = best; *chi = bc; *stab = cnt;
    return 0;
}

/* Builds the group by closure and the sorted representative list. */
ORA_EXPORT int ora_rbasis_create(int L, int nup, int pauli, int a, int has_k, int k,
                                 int p, int z, int pz, int za, int zb, int nthreads,
                                 ora_rbasis **out, char *err, int errlen) {
    *out = NULL;
    if (L < 1 || L > 40) { set_err(err, errlen, "L outside the oracle's range"); return -1; }
    ora_rbasis *b = (ora_rbasis *)calloc(1, sizeof(ora_rbasis));
    b->L = L; b->nup = nup; b->pauli = pauli;
    uint64_t full = lmask(L), odd = 0, even = 0;
    for (int s = 1; s <= L; s += 2) odd |= 1ULL << (s - 1);
    for (int s = 2; s <= L; s += 2) even |= 1ULL << (s - 1);
    gelem_t gens[6]; int ngen = 0;
    memset(gens, 0, sizeof(gens));
    int order = L / (a > 0 ? a : 1);
    if (has_k) {
        if (a <= 0 || L % a) { ora_rbasis_free(b); set_err(err, errlen, "a must be a positive divisor of L"); return -1; }
        int mom = ((k % order) + order) % order;
        double arg = 2 * M_PI * (double)mom / (double)order;
        gens[ngen].shift = a % L; gens[ngen].chi = mkc(cos(arg), sin(arg)); ngen++;
        if (p && !(mom == 0 || (order % 2 == 0 && mom == order / 2))) {
            ora_rbasis_free(b); set_err(err, errlen, "pblock can be combined with kblock only at k=0 or pi"); return -1;
        }
    }
    if (p) { gens[ngen].refl = 1; gens[ngen].chi = mkc(p, 0); ngen++; }
    if (z) { gens[ngen].mask = full; gens[ngen].chi = mkc(z, 0); ngen++; }
    if (pz) { gens[ngen].refl = 1; gens[ngen].mask = full; gens[ngen].chi = mkc(pz, 0); ngen++; }
    if (za) { gens[ngen].mask = odd; gens[ngen].chi = mkc(za, 0); ngen++; }
    if (zb) { gens[ngen].mask = even; gens[ngen].chi = mkc(zb, 0); ngen++; }
    for (int i = 0; i < ngen; ++i) gfill(&gens[i], L);
    /* sector checks: flips must preserve the particle number */
    if (nup >= 0) {
        for (int i = 0; i < ngen; ++i) {
            if (gens[i].mask == 0) continue;
            if (gens[i].mask == full && 2 * nup == L) continue;
            ora_rbasis_free(b); set_err(err, errlen, "symmetry transformation leaves the selected particle sector"); return -2;
        }
    }
    int cap = 1024;
    b->g = (gelem_t *)calloc(cap, sizeof(gelem_t));
    memset(&b->g[0], 0, sizeof(gelem_t)); b->g[0].chi = mkc(1, 0); gfill(&b->g[0], L);
    b->ng = 1;
    for (int i = 0; i < b->ng; ++i) {
        for (int j = 0; j < ngen; ++j) {
            gelem_t c = gcompose(&gens[j], &b->g[i], L);
            int found = -1;
            for (int q = 0; q < b->ng; ++q) if (gsame(&b->g[q], &c, L)) { found = q; break; }
            if (found >= 0) {
                if (!jl_isapprox(b->g[found].chi, c.chi, 1e-9, 1e-9)) {
                    ora_rbasis_free(b); set_err(err, errlen, "the requested symmetry sector is empty"); return -4;
                }
                continue;
            }
            if (b->ng >= cap) { ora_rbasis_free(b); set_err(err, errlen, "group too large"); return -1; }
            b->g[b->ng++] = c;
        }
    }
    /* enumerate candidates in ascending order (chunks of consecutive ranks,
     * unranked then stepped with Gosper's rule), keep orbit minima whose
     * stabiliser carries a trivial character */
    int64_t np = nup < 0 ? ((int64_t)1 << L) : binom_i64(L, nup);
    const int64_t chunk = 1 << 14;
    int64_t nch = (np + chunk - 1) / chunk;
    int64_t *cnt = (int64_t *)calloc(nch + 1, sizeof(int64_t));
    for (int pass = 0; pass < 2; ++pass) {
#ifdef _OPENMP
        if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 4)
#endif
        for (int64_t c = 0; c < nch; ++c) {
            int64_t r0 = c * chunk, r1 = r0 + chunk < np ? r0 + chunk : np;
            uint64_t s = nup < 0 ? (uint64_t)r0 : unrank_fixed(r0, L, nup);
            int64_t w = pass ? cnt[c] : 0, k = 0;
            for (int64_t r = r0; r < r1; ++r) {
                int ok = 1, st = 0;
                for (int q = 0; q < b->ng && ok; ++q) {
                    uint64_t v = gapply(&b->g[q], s, L);
                    if (v < s) ok = 0;
                    else if (v == s) {
                        st++;
                        if (!jl_isapprox(b->g[q].chi, mkc(1, 0), 1e-9, 1e-9)) ok = 0;
                    }
                }
                if (ok) {
                    if (pass) { b->reps[w] = s; b->orbit[w] = b->ng / st; w++; }
                    else k++;
                }
                if (r + 1 < r1) s = nup < 0 ? (uint64_t)(r + 1) : gosper_next(s);
            }
            if (!pass) cnt[c] = k;
        }
        if (!pass) {
            int64_t tot = 0;
            for (int64_t c = 0; c < nch; ++c) { int64_t t = cnt[c]; cnt[c] = tot; tot += t; }
            if (tot == 0) { free(cnt); ora_rbasis_free(b); set_err(err, errlen, "the requested symmetry sector is empty"); return -4; }
            b->n = tot;
            b->reps = (uint64_t *)malloc(sizeof(uint64_t) * tot);
            b->orbit = (int32_t *)malloc(sizeof(int32_t) * tot);
        }
    }
    free(cnt);
    *out = b;
    return 0;
}
ORA_EXPORT int64_t ora_rbasis_size(const ora_rbasis *b) { return b->n; }
ORA_EXPORT int ora_rbasis_group_order(const ora_rbasis *b) { return b->ng; }
ORA_EXPORT void ora_rbasis_states(const ora_rbasis *b, uint64_t *out, int32_t *orbit) {
    memcpy(out, b->reps, sizeof(uint64_t) * b->n);
    if (orbit) memcpy(orbit, b->orbit, sizeof(int32_t) * b->n);
}

/* Pull-form representative-space matvec for operators that commute with the
 * group:  y[r'] = beta y[r'] + alpha * ( sum_t A[s_r', t] chi(g)^{-1}...
 * sqrt(|orb r'| / |orb rep t|) x[rep t] + d[r'] x[r'] ).  The transitions
 * from s_r' are generated with the transposed term chain (A[s,t] = <t|A^T|s>).
 * `rows` restricts the work to rows [row0, row1) (bounded CPU samples). */
ORA_EXPORT int ora_rbasis_matvec(const ora_rbasis *b, int nterms, const char *ops, const int *oplen,
                                 const int64_t *coup_off, const double *coef, const int *sites,
                                 const double *diag, const double *alpha_, const double *beta_,
                                 const double *x_, double *y_, int64_t row0, int64_t row1, int nthreads) {
    const cx *x = (const cx *)x_; cx *y = (cx *)y_;
    const cx *d = (const cx *)diag;
    cx alpha = mkc(alpha_[0], alpha_[1]), beta = mkc(beta_[0], beta_[1]);
    int L = b->L;
    int bad = 0;
    if (row1 > b->n) row1 = b->n;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1024) reduction(|:bad)
#endif
    for (int64_t r = row0; r < row1; ++r) {
        uint64_t s = b->reps[r];
        double orb_r = (double)b->orbit[r];
        cx acc = mkc(0, 0);
        for (int t = 0; t < nterms; ++t) {
            const char *op = ops + 8 * t; int len = oplen[t];
            if (is_diag_op(op, len)) continue;
            for (int64_t c = coup_off[t]; c < coup_off[t + 1]; ++c) {
                const int *st8 = sites + 8 * c;
                cx amp = mkc(coef[2 * c], coef[2 * c + 1]);
                uint64_t st = s; int alive = 1;
                /* transposed chain: leftmost operator first, each transposed */
                for (int i = 0; i < len; ++i) {
                    char o = op[i]; cx f; int rr;
                    if (o == '+') o = '-'; else if (o == '-') o = '+';
                    rr = apply_local(b->pauli, &st, o, st8[i], &f);
                    if (rr < 0) { bad = 1; alive = 0; break; }
                    if (!rr) { alive = 0; break; }
                    if (op[i] == 'y') f = mkc(-f.re, -f.im);
                    amp = cmul(amp, f);
                }
                if (!alive) continue;
                uint64_t m; cx chi; int stab;
                rep_scan(b, st, &m, &chi, &stab);
                int64_t idx = find_u64(b->reps, b->n, m);
                if (idx < 0) continue;
                double orb_c = (double)b->orbit[idx];
                cx w = cmul(amp, chi);
                double sc = sqrt(orb_r / orb_c);
                acc = cadd(acc, cmul(mkc(w.re * sc, w.im * sc), x[idx]));
            }
        }
        if (d) acc = cadd(acc, cmul(d[r], x[r]));
        cx yr = (beta.re == 0.0 && beta.im == 0.0) ? mkc(0, 0) : cmul(beta, y[r]);
        y[r] = cadd(yr, cmul(alpha, acc));
    }
    (void)L;
    return bad ? -1 : 0;
}

/* Diagonal of the structurally diagonal terms on the representatives. */
ORA_EXPORT int ora_rbasis_diagonal(const ora_rbasis *b, int nterms, const char *ops, const int *oplen,
                                   const int64_t *coup_off, const double *coef, const int *sites, double *out) {
    cx *o = (cx *)out;
    for (int64_t r = 0; r < b->n; ++r) {
        cx acc = mkc(0, 0);
        for (int t = 0; t < nterms; ++t) {
            const char *op = ops + 8 * t; int len = oplen[t];
            if (!is_diag_op(op, len)) continue;
            for (int64_t c = coup_off[t]; c < coup_off[t + 1]; ++c) {
                const int *st8 = sites + 8 * c;
                cx amp = mkc(coef[2 * c], coef[2 * c + 1]); uint64_t st = b->reps[r]; int alive = 1;
                for (int i = len - 1; i >= 0; --i) {
                    cx f; int rr = apply_local(b->pauli, &st, op[i], st8[i], &f);
                    if (rr < 0) return -1;
                    if (!rr) { alive = 0; break; }
                    amp = cmul(amp, f);
                }
                if (alive) acc = cadd(acc, amp);
            }
        }
        o[r] = acc;
    }
    return 0;
}

ORA_EXPORT int ora_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
