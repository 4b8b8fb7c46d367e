// qs_dense.cpp -- small dense FP64 linear algebra for the Krylov drivers
// (projected matrices of order <= ~100).  Written from published algorithms:
//   * Householder tridiagonalisation and the implicit symmetric QR step with
//     a Wilkinson shift (Golub & Van Loan, Matrix Computations, 4th ed.,
//     section 8.3);
//   * scaling and squaring with the [13/13] Pade approximant for exp(A)
//     (Higham, SIAM J. Matrix Anal. Appl. 26 (2005) 1179-1193).
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

}  // namespace qs
