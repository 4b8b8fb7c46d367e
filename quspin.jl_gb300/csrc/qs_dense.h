// qs_dense.h -- small dense FP64 helpers for the Krylov drivers.
#pragma once

#include <complex>
#include <vector>

namespace qs {

// Eigen-decomposition of a real symmetric n x n matrix (row-major).  w
// ascending; Z row-major with eigenvectors in its columns.
void sym_eig(int n, const std::vector<double>& A, std::vector<double>& w, std::vector<double>& Z);

// exp(A) for a complex n x n matrix (row-major).
void expm_complex(int n, const std::vector<std::complex<double>>& A, std::vector<std::complex<double>>& E);

}  // namespace qs
