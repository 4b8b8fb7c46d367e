// qs_tools.h -- the Krylov tools of QuSpin.jl's tools.jl on the batched
// engine: Lanczos bases of many start vectors at once, kept on the device,
// and the products the finite- and low-temperature Lanczos estimates need.
#pragma once

#include <memory>
#include <vector>

#include "qs_engine.h"

namespace qs {

// Lanczos recurrences of one Hermitian operator from nstart start vectors
// (src/tools.jl:2742-2843 lanczos_full / _lanczos_coefficients), one engine
// slot each, stepped together.  The bases stay in the slots' device storage.
struct LanczosSet {
    Op* op = nullptr;
    std::unique_ptr<Engine> E;
    std::vector<int> ids;
    int m = 0;                 // requested Lanczos dimension
    bool cv = false;           // complex vectors
    int64_t n = 0;
    std::vector<std::vector<double>> alphas, betas;
    std::vector<int> used;     // rows kept per start (m, or fewer after a breakdown)
    std::vector<double> norms; // ||v0|| per start
};

// Runs the recurrences: m steps (m <= 256), stopping a start's basis where
// beta <= eps (the reference's breakdown test); full_ortho adds classical
// Gram-Schmidt against every kept vector, twice.
std::unique_ptr<LanczosSet> lanczos_run(Op& op, const qs_lanczos_opts& o, int nstart, const double* v0);
// FP64 copy of start s's rows (used x n; real or interleaved complex).
void lanczos_rows(LanczosSet& L, int s, double* out, bool device);
// out[:, c] = sum_i coeff[i + c used] q_i (complex coefficients, complex out, n x ncoef).
void lanczos_combine(LanczosSet& L, int s, const double* coeff, int ncoef, double* out, bool device);
// out[s][i] = <q_i^(s), O q_0^(s)> for every start (complex, nstart x used_max).
void lanczos_overlaps(LanczosSet& L, Op& obs, double* out);
// out = R^* O R with R = Q^T Y (Y used x nv real, column-major); complex nv x nv column-major.
void lanczos_ritz_matrix(LanczosSet& L, int s, Op& obs, const double* Y, int nv, double* out);

// exp(s_i A) applied to every column of V (n x ncol complex): out[:, c, i]
// (n x ncol x nscales, column-major complex), the columns' Krylov recursions
// (_krylov_expmv_times, src/operators.jl:1805-1949) stepping together on one
// engine, in waves that fit in memory; `normalise` scales every state to norm 1
// (imaginary-time evolution).
void expm_columns(Op& op, const double* V, int ncol, const std::vector<cd>& scales, double tol, int krylov_dim,
                  int precision, bool normalise, double* out, bool device);

// evolve(BlockOps, psi, t0, times) / block_expm (src/tools.jl:2445-2719) for
// static block operators: c_b = P_b^H psi for every block with a nonzero
// projection, exp(s_i H_b) c_b for every scale with all blocks' Krylov
// recursions on one engine, out[:, i] = sum_b P_b state_b(i).  psi: rows
// complex; out: rows x nscales complex (host, or device with `device`).
void block_expm(const std::vector<Op*>& ops, bool pcon, const double* psi, const std::vector<cd>& scales, double tol,
                int krylov_dim, int precision, double* out, bool device);

// This GPU's FP64 fused multiply-add throughput (FMA/s): eight independent
// chains per thread over a full grid, best of three CUDA-event timings.
double fp64_fma_rate();

}  // namespace qs
