// qs_dense.h -- small dense FP64 helpers for the Krylov drivers.
#pragma once

#include <algorithm>
#include <cmath>
#include <complex>
#include <numeric>
#include <vector>

namespace qs {

// Eigen-decomposition of a real symmetric n x n matrix (row-major).  w
// ascending; Z row-major with eigenvectors in its columns.
void sym_eig(int n, const std::vector<double>& A, std::vector<double>& w, std::vector<double>& Z);

// Ranking of the Ritz values w (ascending, as sym_eig returns them) for
// eigsh's `which` (src/operators.jl:3376-3401): 0 SA, 1 LA, 2 LM, 3 SM, 4 BE.
// The first min(k, n) entries are the wanted values in output order (SA
// ascending, LA descending, LM by decreasing and SM by increasing magnitude);
// the rest follow in the order a thick restart keeps them.  BE wants
// floor(k/2) values from the low end and ceil(k/2) from the high end (ARPACK's
// convention, as the reference's dense branch selects them,
// src/operators.jl:1592-1596), keeps Ritz values alternately from both ends,
// and lists its wanted values in descending algebraic order.
inline std::vector<int> ritz_order(const std::vector<double>& w, int which, int k) {
    const int n = (int)w.size();
    std::vector<int> o(n);
    std::iota(o.begin(), o.end(), 0);
    switch (which) {
        case 1: std::reverse(o.begin(), o.end()); break;
        case 2:
            std::stable_sort(o.begin(), o.end(), [&](int a, int b) { return std::fabs(w[a]) > std::fabs(w[b]); });
            break;
        case 3:
            std::stable_sort(o.begin(), o.end(), [&](int a, int b) { return std::fabs(w[a]) < std::fabs(w[b]); });
            break;
        case 4: {
            std::vector<int> il;
            for (int lo = 0, hi = n - 1; lo <= hi;) {
                il.push_back(hi--);
                if (lo <= hi) il.push_back(lo++);
            }
            const int kk = std::min(k, n);
            std::sort(il.begin(), il.begin() + kk, [&](int a, int b) { return w[a] > w[b]; });
            o = il;
            break;
        }
        default: break;
    }
    return o;
}

// Complex Schur form of a general n x n matrix (row-major): on return A holds
// the upper-triangular T and Q the unitary factor, A_in = Q T Q^H.
void complex_schur(int n, std::vector<std::complex<double>>& A, std::vector<std::complex<double>>& Q);
// Swaps the diagonal entries k and k + 1 of the Schur form (T, Q), keeping
// A_in = Q T Q^H.
void schur_swap(int n, std::vector<std::complex<double>>& T, std::vector<std::complex<double>>& Q, int k);
// Unit eigenvector y of the upper-triangular T for its diagonal entry i.
void schur_vector(int n, const std::vector<std::complex<double>>& T, int i, std::vector<std::complex<double>>& y);

// exp(A) for a complex n x n matrix (row-major).
void expm_complex(int n, const std::vector<std::complex<double>>& A, std::vector<std::complex<double>>& E);

}  // namespace qs
