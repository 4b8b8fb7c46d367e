// qs_dense.cpp -- small dense FP64 linear algebra for the Krylov drivers
// (projected matrices of order <= ~100).  Written from published algorithms:
//   * cyclic Jacobi eigenvalue method for real symmetric matrices
//     (Golub & Van Loan, Matrix Computations, 4th ed., section 8.5);
//   * scaling and squaring with the [13/13] Pade approximant for exp(A)
//     (Higham, SIAM J. Matrix Anal. Appl. 26 (2005) 1179-1193).
#include "qs_dense.h"

#include <algorithm>
#include <cmath>
#include <stdexcept>

namespace qs {

void sym_eig(int n, const std::vector<double>& A_in, std::vector<double>& w, std::vector<double>& Z) {
    std::vector<double> A(A_in);
    Z.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) Z[(size_t)i * n + i] = 1.0;
    auto a = [&](int i, int j) -> double& { return A[(size_t)i * n + j]; };
    auto z = [&](int i, int j) -> double& { return Z[(size_t)i * n + j]; };
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0, tot = 0.0;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                double v = a(i, j) * a(i, j);
                tot += v;
                if (i != j) off += v;
            }
        if (off <= 1e-34 * tot || off == 0.0) break;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                double apq = a(p, q);
                if (apq == 0.0) continue;
                double app = a(p, p), aqq = a(q, q);
                double theta = (aqq - app) / (2.0 * apq);
                double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; ++k) {
                    double akp = a(k, p), akq = a(k, q);
                    a(k, p) = c * akp - s * akq;
                    a(k, q) = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {
                    double apk = a(p, k), aqk = a(q, k);
                    a(p, k) = c * apk - s * aqk;
                    a(q, k) = s * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    double zkp = z(k, p), zkq = z(k, q);
                    z(k, p) = c * zkp - s * zkq;
                    z(k, q) = s * zkp + c * zkq;
                }
            }
    }
    // sort ascending
    std::vector<int> idx(n);
    for (int i = 0; i < n; ++i) idx[i] = i;
    std::sort(idx.begin(), idx.end(), [&](int x, int y) { return a(x, x) < a(y, y); });
    w.resize(n);
    std::vector<double> Zs((size_t)n * n);
    for (int c = 0; c < n; ++c) {
        w[c] = a(idx[c], idx[c]);
        for (int r = 0; r < n; ++r) Zs[(size_t)r * n + c] = Z[(size_t)r * n + idx[c]];
    }
    Z.swap(Zs);
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
