// qs_common.h -- definitions shared by host and device code of libqsgpu.
#pragma once

#include <cstdint>
#include <cmath>
#include <cfloat>

#ifdef __CUDACC__
#define QS_HD __host__ __device__ __forceinline__
#else
#define QS_HD inline
#endif

namespace qs {

constexpr int kMaxGroup = 512;   // |G| <= 2 (parity) * 63 (translations) * 4 (flip masks)
constexpr int kMaxPerm = 128;    // (reflection, shift) pairs
constexpr int kMaxOps = 8;       // characters of one operator string
constexpr int kMaxGens = 6;      // T, P, Z, PZ, ZA, ZB

// Symmetry group of a sector.  Element e acts on a state s as
//     g_e(s) = rotl_L(R^refl(s), shift) ^ mask[e]
// where R reverses the L site bits (parity, site i -> L+1-i) and rotl_L
// rotates left inside L bits (translation, site i -> i+shift).  Elements are
// grouped by their (refl, shift) permutation so that the rotation is computed
// once per permutation: elements perm_begin[p] .. perm_begin[p+1]-1 share it.
struct GroupDesc {
    int32_t L;
    int32_t ng;
    int32_t nperm;
    int32_t real_chars;          // 1 if every character is +-1
    uint64_t lmask;
    int8_t perm_refl[kMaxPerm];
    int8_t perm_shift[kMaxPerm];
    int16_t perm_begin[kMaxPerm + 1];
    uint64_t mask[kMaxGroup];
    double chi_re[kMaxGroup];
    double chi_im[kMaxGroup];
    // general site permutations (SpinBasisGeneral): permutation p maps the
    // state through gtab[(p * 8 + k) * 256 + byte k of the state], OR-ed over
    // the nbytes bytes; perm_refl / perm_shift are unused then
    int32_t general;
    int32_t nbytes;
    const uint64_t* gtab;
};

// The image of t under general permutation p (tables of a GroupDesc).
QS_HD uint64_t gperm_apply(const uint64_t* tab, int p, int nbytes, uint64_t t) {
    uint64_t r = 0;
    const uint64_t* base = tab + (size_t)p * 8 * 256;
    for (int k = 0; k < nbytes; ++k) r |= base[k * 256 + ((t >> (8 * k)) & 255u)];
    return r;
}

// One transition program: the operator string of one coupling, ops applied in
// array order, sites as 0-based bit positions.  When all sites are distinct the
// program is also compiled to masks: the state survives iff (s & need1) ==
// need1 and (s & need0) == 0, becomes s ^ flip, and picks up
// amp0 * (-1)^(popc(~s & zmask) + popc(s & ymask)).
struct TermProg {
    int32_t nops;
    int32_t distinct;
    char ops[kMaxOps];
    int8_t sites[kMaxOps];
    double coef_re, coef_im;
    double amp0_re, amp0_im;
    uint64_t need0, need1, flip, zmask, ymask;
};

// ---------------------------------------------------------------- bit ops
QS_HD uint64_t low_mask(int L) { return L >= 64 ? ~0ull : ((1ull << L) - 1ull); }

template <typename U>
QS_HD U rotl_bits(U x, int k, int L, U m) {
    return k == 0 ? x : (U)(((x << k) | (x >> (L - k))) & m);
}

#ifdef __CUDACC__
__device__ __forceinline__ uint32_t brev_bits(uint32_t x, int L) { return __brev(x) >> (32 - L); }
__device__ __forceinline__ uint64_t brev_bits(uint64_t x, int L) { return __brevll(x) >> (64 - L); }
#endif

inline uint64_t brev_host(uint64_t x, int L) {
    uint64_t r = 0;
    for (int b = 0; b < L; ++b)
        if ((x >> b) & 1ull) r |= 1ull << (L - 1 - b);
    return r;
}

// ------------------------------------------------- IEEE-exact scalar algebra
// These restate Julia's ComplexF64 arithmetic operation for operation, so the
// reference's projector coefficients (and therefore its argmax representatives
// and 1/|amp|^2 normalisations) are reproduced bit for bit.  Device builds of
// this code use the explicitly rounded intrinsics so nothing is contracted.
struct cplx { double re, im; };

#ifdef __CUDA_ARCH__
#define QS_ADD(a, b) __dadd_rn((a), (b))
#define QS_SUB(a, b) __dsub_rn((a), (b))
#define QS_MUL(a, b) __dmul_rn((a), (b))
#define QS_DIV(a, b) __ddiv_rn((a), (b))
#define QS_SQRT(a) __dsqrt_rn(a)
#define QS_FMA(a, b, c) __fma_rn((a), (b), (c))
#else
#define QS_ADD(a, b) ((a) + (b))
#define QS_SUB(a, b) ((a) - (b))
#define QS_MUL(a, b) ((a) * (b))
#define QS_DIV(a, b) ((a) / (b))
#define QS_SQRT(a) std::sqrt(a)
#define QS_FMA(a, b, c) std::fma((a), (b), (c))
#endif

QS_HD cplx cx(double r, double i) { cplx z; z.re = r; z.im = i; return z; }
QS_HD cplx cx_mul(cplx z, cplx w) {
    return cx(QS_SUB(QS_MUL(z.re, w.re), QS_MUL(z.im, w.im)), QS_ADD(QS_MUL(z.re, w.im), QS_MUL(z.im, w.re)));
}
QS_HD cplx cx_add(cplx a, cplx b) { return cx(QS_ADD(a.re, b.re), QS_ADD(a.im, b.im)); }
QS_HD cplx cx_conj(cplx z) { return cx(z.re, -z.im); }
QS_HD cplx cx_divr(cplx z, double x) { return cx(QS_DIV(z.re, x), QS_DIV(z.im, x)); }
QS_HD double cx_abs2(cplx z) { return QS_ADD(QS_MUL(z.re, z.re), QS_MUL(z.im, z.im)); }

// Robust complex division: Baudin & Smith, "A Robust Complex Division in
// Scilab" (2012).
QS_HD double rcdiv2(double a, double b, double c, double d, double r, double t) {
    if (r != 0) {
        double br = QS_MUL(b, r);
        return (br != 0) ? QS_MUL(QS_ADD(a, br), t) : QS_ADD(QS_MUL(a, t), QS_MUL(QS_MUL(b, t), r));
    }
    return QS_MUL(QS_ADD(a, QS_MUL(d, QS_DIV(b, c))), t);
}
QS_HD void rcdiv1(double a, double b, double c, double d, double* p, double* q) {
    double r = QS_DIV(d, c);
    double t = QS_DIV(1.0, QS_ADD(c, QS_MUL(d, r)));
    *p = rcdiv2(a, b, c, d, r, t);
    *q = rcdiv2(b, -a, c, d, r, t);
}
QS_HD cplx cx_div(cplx z, cplx w) {
    double a = z.re, b = z.im, c = w.re, d = w.im;
    double absa = fabs(a), absb = fabs(b);
    double ab = absa >= absb ? absa : absb;
    double absc = fabs(c), absd = fabs(d);
    double cd = absc >= absd ? absc : absd;
    const double halfov = 0.5 * DBL_MAX;
    const double twoune = DBL_MIN * 2.0 / DBL_EPSILON;
    const double bs = 2.0 / (DBL_EPSILON * DBL_EPSILON);
    double s = 1.0, p, q;
    if (ab >= halfov) { a = QS_MUL(0.5, a); b = QS_MUL(0.5, b); s = 2.0; }
    if (cd >= halfov) { c = QS_MUL(0.5, c); d = QS_MUL(0.5, d); s = QS_MUL(s, 0.5); }
    if (ab <= twoune) { a = QS_MUL(a, bs); b = QS_MUL(b, bs); s = QS_DIV(s, bs); }
    if (cd <= twoune) { c = QS_MUL(c, bs); d = QS_MUL(d, bs); s = QS_MUL(s, bs); }
    if (absd <= absc) {
        rcdiv1(a, b, c, d, &p, &q);
    } else {
        rcdiv1(b, a, d, c, &p, &q);
        q = -q;
    }
    return cx(QS_MUL(p, s), QS_MUL(q, s));
}

// Correctly rounded hypot: Borges, "An Improved Algorithm for hypot(a,b)",
// ACM TOMS 45 (2019), FMA-corrected variant.
QS_HD double hypot_cr(double x, double y) {
    double ax = fabs(x), ay = fabs(y);
    if (ax > DBL_MAX || ay > DBL_MAX) return INFINITY;
    if (ay > ax) { double t = ax; ax = ay; ay = t; }
    const double small_ratio = 1.0536712127723509e-08;  // sqrt(eps/2), eps = 2^-52
    if (ay <= QS_MUL(ax, small_ratio)) return ax;
    double scale = 1.0;
    const double big = 9.480751908109176e+153;          // sqrt(DBL_MAX / 2)
    const double tiny = 1.4916681462400413e-154;        // sqrt(DBL_MIN)
    const double sc = 3.3121686421112381e-170;          // eps * sqrt(DBL_MIN)
    if (ax > big) {
        ax = QS_MUL(ax, sc); ay = QS_MUL(ay, sc); scale = QS_DIV(1.0, sc);
    } else if (ay < tiny) {
        ax = QS_DIV(ax, sc); ay = QS_DIV(ay, sc); scale = sc;
    }
    double h = QS_SQRT(QS_FMA(ax, ax, QS_MUL(ay, ay)));
    double hsq = QS_MUL(h, h);
    double axsq = QS_MUL(ax, ax);
    double corr = QS_SUB(QS_ADD(QS_FMA(-ay, ay, QS_SUB(hsq, axsq)), QS_FMA(h, h, -hsq)), QS_FMA(ax, ax, -axsq));
    h = QS_SUB(h, QS_DIV(corr, QS_MUL(2.0, h)));
    return QS_MUL(h, scale);
}
QS_HD double cx_abs(cplx z) { return hypot_cr(z.re, z.im); }

// 2-norm of a short complex vector: maximum magnitude, then sqrt of the
// running sum of abs2 (no scaling in the normal range).
QS_HD double norm2_short(const cplx* v, int n) {
    if (n == 0) return 0.0;
    double maxabs = 0.0;
    for (int i = 0; i < n; ++i) {
        double a = cx_abs(v[i]);
        if (a > maxabs) maxabs = a;
    }
    if (maxabs == 0.0 || maxabs > DBL_MAX) return maxabs;
    double sum = cx_abs2(v[0]);
    for (int i = 1; i < n; ++i) sum = QS_ADD(sum, cx_abs2(v[i]));
    return QS_SQRT(sum);
}

}  // namespace qs
