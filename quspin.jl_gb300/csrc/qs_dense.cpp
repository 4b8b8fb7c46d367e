// qs_dense.cpp -- small dense FP64 linear algebra for the Krylov drivers
// (projected matrices of order <= ~100).  Written from published algorithms:
//   * Householder tridiagonalisation and the implicit symmetric QR step with
//     a Wilkinson shift (Golub & Van Loan, Matrix Computations, 4th ed.,
//     section 8.3);
//   * scaling and squaring with the [13/13] Pade approximant for exp(A)
//     (Higham, SIAM J. Matrix Anal. Appl. 26 (2005) 1179-1193);
//   * the complex Schur form: Householder reduction to Hessenberg form, then
//     the implicit single-shift QR iteration with Wilkinson shifts and
//     deflation, reordering of the Schur form by adjacent Givens swaps, and
//     eigenvectors of the triangular factor by back substitution (Golub &
//     Van Loan, sections 7.4-7.7).
#include "qs_dense.h"

#include <algorithm>
#include <cmath>
#include <stdexcept>

namespace qs {

namespace {

// One implicit symmetric QR step with a Wilkinson shift on the unreduced block
// lo..hi of the tridiagonal (d, e), chasing the bulge with Givens rotations
// G = [c -s; s c] (T <- G^T T G) that are accumulated into Q <- Q G.
void qr_step(std::vector<double>& d, std::vector<double>& e, int lo, int hi, std::vector<double>& Q, int n) {
    const double a = d[hi - 1], b = e[hi - 1], cc = d[hi];
    const double delta = 0.5 * (a - cc);
    const double mu = cc - b * b / (delta + std::copysign(std::hypot(delta, b), delta));
    double x = d[lo] - mu, z = e[lo];
    for (int k = lo; k < hi; ++k) {
        double r = std::hypot(x, z), c = 1.0, s = 0.0;
        if (r != 0.0) {
            c = x / r;
            s = z / r;
        }
        if (k > lo) e[k - 1] = r;   // the previous bulge is annihilated
        const double dk = d[k], dk1 = d[k + 1], ek = e[k];
        d[k] = c * c * dk + 2.0 * c * s * ek + s * s * dk1;
        d[k + 1] = s * s * dk - 2.0 * c * s * ek + c * c * dk1;
        e[k] = c * s * (dk1 - dk) + (c * c - s * s) * ek;
        if (k + 1 < hi) {
            const double bulge = s * e[k + 1];
            e[k + 1] *= c;
            x = e[k];
            z = bulge;
        }
        for (int i = 0; i < n; ++i) {
            double* q = &Q[(size_t)i * n];
            const double qk = q[k], qk1 = q[k + 1];
            q[k] = c * qk + s * qk1;
            q[k + 1] = -s * qk + c * qk1;
        }
    }
}

}  // namespace

// Householder reduction to tridiagonal form, then implicit QR steps with
// Wilkinson shifts (Golub & Van Loan, Matrix Computations, 4th ed.,
// algorithms 8.3.1 and 8.3.2), eigenvectors accumulated throughout.
void sym_eig(int n, const std::vector<double>& A_in, std::vector<double>& w, std::vector<double>& Z) {
    std::vector<double> A(A_in), Q((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) Q[(size_t)i * n + i] = 1.0;
    auto a = [&](int i, int j) -> double& { return A[(size_t)i * n + j]; };
    std::vector<double> v(n), p(n), q(n);
    for (int k = 0; k + 2 < n; ++k) {
        double alpha2 = 0;
        for (int i = k + 1; i < n; ++i) alpha2 += a(i, k) * a(i, k);
        if (alpha2 == 0.0) continue;
        const double alpha = -std::copysign(std::sqrt(alpha2), a(k + 1, k));
        double vv = 0;
        for (int i = k + 1; i < n; ++i) {
            v[i] = a(i, k) - (i == k + 1 ? alpha : 0.0);
            vv += v[i] * v[i];
        }
        if (vv == 0.0) continue;
        const double beta = 2.0 / vv;
        // H S H on the trailing block S = A[k+1:, k+1:] with H = I - beta v v^T
        double vp = 0;
        for (int i = k + 1; i < n; ++i) {
            double t = 0;
            for (int j = k + 1; j < n; ++j) t += a(i, j) * v[j];
            p[i] = beta * t;
            vp += v[i] * p[i];
        }
        const double K = 0.5 * beta * vp;
        for (int i = k + 1; i < n; ++i) q[i] = p[i] - K * v[i];
        for (int i = k + 1; i < n; ++i)
            for (int j = k + 1; j < n; ++j) a(i, j) -= v[i] * q[j] + q[i] * v[j];
        a(k + 1, k) = a(k, k + 1) = alpha;
        for (int i = k + 2; i < n; ++i) a(i, k) = a(k, i) = 0.0;
        for (int r = 0; r < n; ++r) {
            double* qr = &Q[(size_t)r * n];
            double t = 0;
            for (int j = k + 1; j < n; ++j) t += qr[j] * v[j];
            t *= beta;
            for (int j = k + 1; j < n; ++j) qr[j] -= t * v[j];
        }
    }
    std::vector<double> d(n), e(std::max(n - 1, 1), 0.0);
    for (int i = 0; i < n; ++i) d[i] = a(i, i);
    for (int i = 0; i + 1 < n; ++i) e[i] = a(i + 1, i);
    const double eps = 2.220446049250313e-16;
    int hi = n - 1, iters = 0;
    while (hi > 0) {
        if (std::fabs(e[hi - 1]) <= eps * (std::fabs(d[hi - 1]) + std::fabs(d[hi]))) {
            e[hi - 1] = 0.0;
            --hi;
            continue;
        }
        int lo = hi - 1;
        while (lo > 0 && std::fabs(e[lo - 1]) > eps * (std::fabs(d[lo - 1]) + std::fabs(d[lo]))) --lo;
        if (lo > 0) e[lo - 1] = 0.0;
        qr_step(d, e, lo, hi, Q, n);
        if (++iters > 50 * n) throw std::runtime_error("symmetric eigensolver did not converge");
    }
    std::vector<int> idx(n);
    for (int i = 0; i < n; ++i) idx[i] = i;
    std::sort(idx.begin(), idx.end(), [&](int x, int y) { return d[x] < d[y]; });
    w.resize(n);
    Z.assign((size_t)n * n, 0.0);
    for (int c = 0; c < n; ++c) {
        w[c] = d[idx[c]];
        for (int r = 0; r < n; ++r) Z[(size_t)r * n + c] = Q[(size_t)r * n + idx[c]];
    }
}

namespace {

using cd = std::complex<double>;
using CMat = std::vector<cd>;  // row-major n x n

CMat cmatmul(int n, const CMat& A, const CMat& B) {
    CMat C((size_t)n * n, cd(0, 0));
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < n; ++k) {
            cd aik = A[(size_t)i * n + k];
            if (aik == cd(0, 0)) continue;
            for (int j = 0; j < n; ++j) C[(size_t)i * n + j] += aik * B[(size_t)k * n + j];
        }
    return C;
}

// Solve P X = Q (n x n) by Gaussian elimination with partial pivoting.
CMat csolve(int n, CMat P, CMat Q) {
    for (int c = 0; c < n; ++c) {
        int piv = c;
        double best = std::abs(P[(size_t)c * n + c]);
        for (int r = c + 1; r < n; ++r) {
            double v = std::abs(P[(size_t)r * n + c]);
            if (v > best) { best = v; piv = r; }
        }
        if (best == 0.0) throw std::runtime_error("singular Pade denominator");
        if (piv != c)
            for (int j = 0; j < n; ++j) {
                std::swap(P[(size_t)c * n + j], P[(size_t)piv * n + j]);
                std::swap(Q[(size_t)c * n + j], Q[(size_t)piv * n + j]);
            }
        cd inv = 1.0 / P[(size_t)c * n + c];
        for (int r = c + 1; r < n; ++r) {
            cd f = P[(size_t)r * n + c] * inv;
            if (f == cd(0, 0)) continue;
            for (int j = c; j < n; ++j) P[(size_t)r * n + j] -= f * P[(size_t)c * n + j];
            for (int j = 0; j < n; ++j) Q[(size_t)r * n + j] -= f * Q[(size_t)c * n + j];
        }
    }
    for (int c = n - 1; c >= 0; --c) {
        cd inv = 1.0 / P[(size_t)c * n + c];
        for (int j = 0; j < n; ++j) {
            cd s = Q[(size_t)c * n + j];
            for (int k = c + 1; k < n; ++k) s -= P[(size_t)c * n + k] * Q[(size_t)k * n + j];
            Q[(size_t)c * n + j] = s * inv;
        }
    }
    return Q;
}

}  // namespace

void expm_complex(int n, const std::vector<std::complex<double>>& A_in, std::vector<std::complex<double>>& E) {
    static const double b[14] = {64764752532480000.0, 32382376266240000.0, 7771770303897600.0,
                                 1187353796428800.0,  129060195264000.0,   10559470521600.0,
                                 670442572800.0,      33522128640.0,       1323241920.0,
                                 40840800.0,          960960.0,            16380.0,
                                 182.0,               1.0};
    const double theta13 = 5.371920351148152;
    double norm1 = 0.0;
    for (int j = 0; j < n; ++j) {
        double s = 0.0;
        for (int i = 0; i < n; ++i) s += std::abs(A_in[(size_t)i * n + j]);
        norm1 = std::max(norm1, s);
    }
    int sq = 0;
    if (norm1 > theta13) sq = std::max(0, (int)std::ceil(std::log2(norm1 / theta13)));
    double scale = std::ldexp(1.0, -sq);
    CMat A(A_in);
    for (auto& v : A) v *= scale;
    CMat I((size_t)n * n, cd(0, 0));
    for (int i = 0; i < n; ++i) I[(size_t)i * n + i] = 1.0;
    CMat A2 = cmatmul(n, A, A), A4 = cmatmul(n, A2, A2), A6 = cmatmul(n, A4, A2);
    CMat U1((size_t)n * n), V1((size_t)n * n), U2((size_t)n * n), V2((size_t)n * n);
    for (size_t k = 0; k < U1.size(); ++k) {
        U1[k] = b[13] * A6[k] + b[11] * A4[k] + b[9] * A2[k];
        V1[k] = b[12] * A6[k] + b[10] * A4[k] + b[8] * A2[k];
    }
    U1 = cmatmul(n, A6, U1);
    V1 = cmatmul(n, A6, V1);
    for (size_t k = 0; k < U1.size(); ++k) {
        U2[k] = U1[k] + b[7] * A6[k] + b[5] * A4[k] + b[3] * A2[k] + b[1] * I[k];
        V2[k] = V1[k] + b[6] * A6[k] + b[4] * A4[k] + b[2] * A2[k] + b[0] * I[k];
    }
    CMat U = cmatmul(n, A, U2);
    CMat P((size_t)n * n), Q((size_t)n * n);
    for (size_t k = 0; k < U.size(); ++k) {
        P[k] = V2[k] - U[k];
        Q[k] = V2[k] + U[k];
    }
    CMat R = csolve(n, P, Q);
    for (int s = 0; s < sq; ++s) R = cmatmul(n, R, R);
    E.swap(R);
}


// ------------------------------------------------------------- complex Schur
namespace {

using cx = std::complex<double>;

// Givens rotation [c s; -conj(s) c] with c real that maps (x, y) to (r, 0)
void cgivens(cx x, cx y, double& c, cx& s) {
    const double ax = std::abs(x), ay = std::abs(y);
    if (ay == 0.0) {
        c = 1.0;
        s = 0.0;
        return;
    }
    if (ax == 0.0) {
        c = 0.0;
        s = std::conj(y) / ay;
        return;
    }
    const double nr = std::hypot(ax, ay);
    c = ax / nr;
    s = (x / ax) * std::conj(y) / nr;
}

// rows k, k+1 of A (columns c0 .. n-1) <- G rows; columns k, k+1 of A (rows
// 0 .. r1-1) and of Q <- times G^H
void rot_rows(std::vector<cx>& A, int n, int k, int c0, double c, cx s) {
    for (int j = c0; j < n; ++j) {
        const cx a = A[(size_t)k * n + j], b = A[(size_t)(k + 1) * n + j];
        A[(size_t)k * n + j] = c * a + s * b;
        A[(size_t)(k + 1) * n + j] = -std::conj(s) * a + c * b;
    }
}
void rot_cols(std::vector<cx>& A, int n, int k, int r1, double c, cx s) {
    for (int i = 0; i < r1; ++i) {
        const cx a = A[(size_t)i * n + k], b = A[(size_t)i * n + k + 1];
        A[(size_t)i * n + k] = c * a + std::conj(s) * b;
        A[(size_t)i * n + k + 1] = -s * a + c * b;
    }
}

}  // namespace

void complex_schur(int n, std::vector<cx>& A, std::vector<cx>& Q) {
    Q.assign((size_t)n * n, cx(0, 0));
    for (int i = 0; i < n; ++i) Q[(size_t)i * n + i] = 1.0;
    // Householder reduction to upper Hessenberg form, A <- P^H A P, Q <- Q P
    for (int k = 0; k + 2 < n; ++k) {
        double alpha2 = 0.0;
        for (int i = k + 1; i < n; ++i) alpha2 += std::norm(A[(size_t)i * n + k]);
        const double alpha = std::sqrt(alpha2);
        if (alpha == 0.0) continue;
        const cx x0 = A[(size_t)(k + 1) * n + k];
        const cx ph = std::abs(x0) > 0 ? x0 / std::abs(x0) : cx(1, 0);
        std::vector<cx> v(n, cx(0, 0));
        v[k + 1] = x0 + ph * alpha;
        for (int i = k + 2; i < n; ++i) v[i] = A[(size_t)i * n + k];
        double vn = 0.0;
        for (int i = k + 1; i < n; ++i) vn += std::norm(v[i]);
        if (vn == 0.0) continue;
        // A <- (I - 2 v v^H / vn) A (I - 2 v v^H / vn)
        for (int j = 0; j < n; ++j) {
            cx t = 0;
            for (int i = k + 1; i < n; ++i) t += std::conj(v[i]) * A[(size_t)i * n + j];
            t *= 2.0 / vn;
            for (int i = k + 1; i < n; ++i) A[(size_t)i * n + j] -= v[i] * t;
        }
        for (int i = 0; i < n; ++i) {
            cx t = 0;
            for (int j = k + 1; j < n; ++j) t += A[(size_t)i * n + j] * v[j];
            t *= 2.0 / vn;
            for (int j = k + 1; j < n; ++j) A[(size_t)i * n + j] -= t * std::conj(v[j]);
            cx u = 0;
            for (int j = k + 1; j < n; ++j) u += Q[(size_t)i * n + j] * v[j];
            u *= 2.0 / vn;
            for (int j = k + 1; j < n; ++j) Q[(size_t)i * n + j] -= u * std::conj(v[j]);
        }
        for (int i = k + 2; i < n; ++i) A[(size_t)i * n + k] = 0.0;
    }
    // implicit single-shift QR on the active window [lo, hi]
    const double eps = 2.220446049250313e-16;
    int hi = n - 1, iter = 0;
    while (hi > 0) {
        int lo = hi;
        while (lo > 0) {
            const double sub = std::abs(A[(size_t)lo * n + lo - 1]);
            const double dn = std::abs(A[(size_t)lo * n + lo]) + std::abs(A[(size_t)(lo - 1) * n + lo - 1]);
            if (sub <= eps * (dn > 0 ? dn : 1.0)) {
                A[(size_t)lo * n + lo - 1] = 0.0;
                break;
            }
            --lo;
        }
        if (lo == hi) {
            --hi;
            iter = 0;
            continue;
        }
        if (++iter > 60 * n) throw std::runtime_error("complex Schur iteration did not converge");
        // Wilkinson shift from the trailing 2 x 2 block (exceptional shift now and then)
        const cx a = A[(size_t)(hi - 1) * n + hi - 1], b = A[(size_t)(hi - 1) * n + hi];
        const cx c2 = A[(size_t)hi * n + hi - 1], d = A[(size_t)hi * n + hi];
        cx mu;
        if (iter % 11 == 10) {
            mu = d + std::abs(A[(size_t)hi * n + hi - 1]) * 0.75;
        } else {
            const cx tr = 0.5 * (a + d), det = a * d - b * c2;
            const cx disc = std::sqrt(tr * tr - det);
            const cx l1 = tr + disc, l2 = tr - disc;
            mu = std::abs(l1 - d) < std::abs(l2 - d) ? l1 : l2;
        }
        cx x = A[(size_t)lo * n + lo] - mu, y = A[(size_t)(lo + 1) * n + lo];
        for (int k = lo; k < hi; ++k) {
            double c;
            cx sn;
            cgivens(x, y, c, sn);
            rot_rows(A, n, k, k > lo ? k - 1 : k, c, sn);
            rot_cols(A, n, k, std::min(k + 3, hi + 1), c, sn);
            rot_cols(Q, n, k, n, c, sn);
            if (k > lo) A[(size_t)(k + 1) * n + k - 1] = 0.0;
            if (k + 1 < hi) {
                x = A[(size_t)(k + 1) * n + k];
                y = A[(size_t)(k + 2) * n + k];
            }
        }
    }
}

void schur_swap(int n, std::vector<cx>& T, std::vector<cx>& Q, int k) {
    const cx a = T[(size_t)k * n + k], b = T[(size_t)k * n + k + 1], d = T[(size_t)(k + 1) * n + k + 1];
    double c;
    cx s;
    cgivens(b, d - a, c, s);   // rotates the eigenvector (b, d - a) of d onto e_1
    rot_rows(T, n, k, k, c, s);
    rot_cols(T, n, k, n, c, s);
    rot_cols(Q, n, k, n, c, s);
    T[(size_t)(k + 1) * n + k] = 0.0;
    T[(size_t)k * n + k] = d;
    T[(size_t)(k + 1) * n + k + 1] = a;
}

void schur_vector(int n, const std::vector<cx>& T, int i, std::vector<cx>& y) {
    y.assign(n, cx(0, 0));
    y[i] = 1.0;
    const cx lam = T[(size_t)i * n + i];
    double tn = 0.0;
    for (const cx& v : T) tn = std::max(tn, std::abs(v));
    const double small = 2.220446049250313e-16 * std::max(tn, 1e-300);
    for (int j = i - 1; j >= 0; --j) {
        cx sacc = 0;
        for (int l = j + 1; l <= i; ++l) sacc += T[(size_t)j * n + l] * y[l];
        cx den = T[(size_t)j * n + j] - lam;
        if (std::abs(den) < small) den = small;
        y[j] = -sacc / den;
    }
    double nr = 0.0;
    for (const cx& v : y) nr += std::norm(v);
    nr = std::sqrt(nr);
    for (cx& v : y) v /= nr;
}

}  // namespace qs
