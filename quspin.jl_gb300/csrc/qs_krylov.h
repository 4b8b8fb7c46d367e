// qs_krylov.h -- Krylov solver entry points (host drivers over device vectors).
#pragma once

#include <complex>

#include "qs_internal.h"

namespace qs {

double eps23();
void eigsh(Op& op, const qs_eigsh_opts& o, double* values, void* vectors, qs_eigsh_info* info);
// eigsh of a non-Hermitian operator: k complex eigenvalues (values: 2k
// doubles) and complex Ritz vectors (n x k ComplexF64)
void eigs_general(Op& op, const qs_eigsh_opts& o, double* values, void* vectors, qs_eigsh_info* info);
void eigsh_batch(Op** ops, int nops, const qs_eigsh_opts& o, double* values, void** vectors, qs_eigsh_info* infos);
void expm_multiply(Op& op, std::complex<double> a, const double* v, double* out, double tol, int krylov_dim,
                   int precision);
void evolve(Op& op, const double* v0, double t0, const double* times, int nt, int imag_time, double tol,
            int krylov_dim, int precision, double* out);

}  // namespace qs
