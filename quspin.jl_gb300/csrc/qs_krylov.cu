// qs_krylov.cu -- Krylov solvers driven from the host over device vectors.
//
//  * eigsh: thick-restart Lanczos (Wu & Simon, SIAM J. Matrix Anal. Appl. 22
//    (2000) 602-616) with full CGS2 reorthogonalisation, replacing the ARPACK
//    implicitly restarted Lanczos the reference calls (src/operators.jl:
//    3367-3408 via Arpack.eigs).  Convergence uses ARPACK's Ritz bound test
//    |beta_m y_m,i| <= tol * max(eps^(2/3), |theta_i|).  The single-precision
//    form runs the same iteration on FP32 vectors with FP64 alpha/beta,
//    reorthogonalisation coefficients and projected eigensolve, then polishes
//    in FP64 (Rayleigh quotient, FP64 Lanczos refinement if the bound needs it).
//  * Krylov exponential action: the reference's algorithm step for step
//    (_krylov_factorization 1655-1731, _krylov_project 1733-1756,
//    _krylov_expmv_vector 1758-1803, _krylov_expmv_times 1805-1893), used by
//    evolve (2073-2164) and ExpmMultiplyParallel (tools.jl:1662-1708).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <random>
#include <vector>

#include "qs_blas.cuh"
#include "qs_dense.h"
#include "qs_internal.h"
#include "qs_engine.h"
#include "qs_krylov.h"

namespace qs {

namespace {

constexpr double kEps = 2.220446049250313e-16;

struct Ctx {
    Op& op;
    int64_t n;
    VKind vk;
    cudaStream_t s;
    Blas blas;
    int64_t matvecs = 0;
    bool df = false;   // double-float products of an assembled operator
    Ctx(Op& o, VKind k, bool df_ = false)
        : op(o), n(o.basis->n), vk(k), s(o.stream), blas(k, o.basis->n, o.stream), df(df_) {}
    void* col(DevBuf& V, int j) const { return (char*)V.p + (size_t)j * n * vk_bytes(vk); }
    void matvec(const void* x, void* y) {
        MatvecCall c;
        c.x = x;
        c.y = y;
        c.x_complex = c.y_complex = vk_complex(vk);
        c.single = vk_single(vk);
        c.df_io = vk_df(vk);
        c.df = (df || c.df_io) && !c.single;
        op_matvec_device(op, c, s);
        ++matvecs;
    }
};

// Storage of the Krylov vectors for a precision code: 0 FP64, 1 FP32, 2
// double-float (DF storage needs the sliced assembled layout, else FP64
// vectors with double-float products where the operator is assembled).
VKind krylov_kind(const Op& op, bool cpx, int precision) {
    if (precision == 1) return cpx ? VKind::C64 : VKind::F32;
    if (precision == 2 && op.assembled && op.asm_.has_sell) return cpx ? VKind::CDF64 : VKind::DF64;
    return cpx ? VKind::C128 : VKind::F64;
}

// Deterministic pseudo-random start vector (normal entries, generated on the device).
void random_vector(Ctx& c, void* dst, uint64_t seed) {
    fill_normal(dst, c.vk, c.n, seed, c.s);
    QS_CUDA(cudaStreamSynchronize(c.s));
}

// CGS2 of w against V[:, 0:m); returns the summed coefficients.
std::vector<cd> orthogonalize(Ctx& c, DevBuf& V, int m, void* w) {
    std::vector<cd> h, h2;
    c.blas.dots(V.p, c.n, m, w, h);
    c.blas.update(w, V.p, c.n, m, h);
    c.blas.dots(V.p, c.n, m, w, h2);
    c.blas.update(w, V.p, c.n, m, h2);
    for (int i = 0; i < m; ++i) h[i] += h2[i];
    return h;
}

struct TRResult {
    std::vector<double> theta;
    int nconv = 0;
    int restarts = 0;
    double max_rel = 0.0;
};

// Thick-restart Lanczos.  On return X (n x k, storage c.vk) holds the Ritz
// vectors of the wanted values.
TRResult trlan(Ctx& c, int k, int which, double tol, int ncv, int maxiter, const void* v0, void* X) {
    const int64_t n = c.n;
    int m = std::min<int64_t>(ncv, n);
    DevBuf V((size_t)n * (m + 1) * vk_bytes(c.vk));
    DevBuf tmp((size_t)n * m * vk_bytes(c.vk));
    c.blas.copy(V.p, v0);
    double nv0 = c.blas.norm(V.p);
    if (!(nv0 > 0)) throw Error(QS_ERR_ARGUMENT, "starting vector must be nonzero");
    c.blas.scale(V.p, V.p, cd(1.0 / nv0, 0));
    std::vector<double> T((size_t)m * m, 0.0);
    auto Tij = [&](int i, int j) -> double& { return T[(size_t)i * m + j]; };
    int j0 = 0;
    double beta = 0.0;
    const double eps23 = std::pow(kEps, 2.0 / 3.0);
    TRResult R;
    std::vector<double> w, Y;
    int m_eff = m;
    for (int iter = 0; iter < maxiter; ++iter) {
        R.restarts = iter;
        m_eff = m;
        for (int j = j0; j < m; ++j) {
            void* wv = c.col(V, j + 1);
            c.matvec(c.col(V, j), wv);
            std::vector<cd> h = orthogonalize(c, V, j + 1, wv);
            Tij(j, j) = h[j].real();
            beta = c.blas.norm(wv);
            double tnorm = 0.0;
            for (int q = 0; q <= j; ++q) tnorm = std::max(tnorm, std::fabs(Tij(q, q)));
            if (beta <= 1e-13 * std::max(1.0, tnorm)) {
                // invariant subspace: continue with a random vector orthogonal to V
                bool refilled = false;
                if (j + 1 < n) {
                    random_vector(c, wv, 0x9e3779b97f4a7c15ull + (uint64_t)iter * 131 + j);
                    orthogonalize(c, V, j + 1, wv);
                    double nb = c.blas.norm(wv);
                    if (nb > 1e-8) {
                        c.blas.scale(wv, wv, cd(1.0 / nb, 0));
                        refilled = true;
                    }
                }
                beta = 0.0;
                if (!refilled) {
                    m_eff = j + 1;
                    break;
                }
            } else {
                c.blas.scale(wv, wv, cd(1.0 / beta, 0));
            }
            if (j + 1 < m) Tij(j, j + 1) = Tij(j + 1, j) = beta;
        }
        std::vector<double> Te((size_t)m_eff * m_eff);
        for (int i = 0; i < m_eff; ++i)
            for (int j = 0; j < m_eff; ++j) Te[(size_t)i * m_eff + j] = Tij(i, j);
        sym_eig(m_eff, Te, w, Y);
        auto yv = [&](int r, int col) { return Y[(size_t)r * m_eff + col]; };
        const std::vector<int> order = ritz_order(w, which, k);
        int kk = std::min(k, m_eff);
        int nconv = 0;
        double maxrel = 0.0;
        for (int q = 0; q < kk; ++q) {
            int i = order[q];
            double bound = std::fabs(beta * yv(m_eff - 1, i));
            double rel = bound / std::max(eps23, std::fabs(w[i]));
            maxrel = std::max(maxrel, rel);
            if (bound <= tol * std::max(eps23, std::fabs(w[i]))) ++nconv;
        }
        R.nconv = nconv;
        R.max_rel = maxrel;
        bool done = (nconv >= k) || (m_eff < m) || (iter == maxiter - 1);
        if (done) {
            std::vector<double> Ysel((size_t)m_eff * kk);
            R.theta.resize(kk);
            for (int q = 0; q < kk; ++q) {
                R.theta[q] = w[order[q]];
                for (int r = 0; r < m_eff; ++r) Ysel[(size_t)q * m_eff + r] = yv(r, order[q]);
            }
            c.blas.rotate(V.p, n, m_eff, kk, Ysel, tmp.p);
            QS_CUDA(cudaMemcpyAsync(X, V.p, (size_t)n * kk * vk_bytes(c.vk), cudaMemcpyDeviceToDevice, c.s));
            QS_CUDA(cudaStreamSynchronize(c.s));
            if (m_eff < m && nconv < k) R.nconv = kk;  // exact invariant subspace
            return R;
        }
        // restart: keep p Ritz vectors (the wanted end of the spectrum)
        int p = std::min(m - 2, k + (m - k) / 2);
        p = std::max(p, std::min(k, m - 1));
        std::vector<double> Ysel((size_t)m * p);
        std::vector<double> th(p), sc(p);
        for (int q = 0; q < p; ++q) {
            int i = order[q];
            th[q] = w[i];
            sc[q] = beta * yv(m - 1, i);
            for (int r = 0; r < m; ++r) Ysel[(size_t)q * m + r] = yv(r, i);
        }
        c.blas.rotate(V.p, n, m, p, Ysel, tmp.p);
        c.blas.copy(c.col(V, p), c.col(V, m));
        std::fill(T.begin(), T.end(), 0.0);
        for (int q = 0; q < p; ++q) {
            Tij(q, q) = th[q];
            Tij(q, p) = Tij(p, q) = sc[q];
        }
        j0 = p;
    }
    return R;
}


// Ranking of complex Ritz values for a non-Hermitian eigsh: SA / LA by real
// part (the reference asks ARPACK for :SR / :LR, src/operators.jl:3383),
// LM / SM by magnitude; stable, wanted values first in output order.
std::vector<int> ritz_order_complex(const std::vector<cd>& w, int which) {
    std::vector<int> o(w.size());
    for (size_t i = 0; i < o.size(); ++i) o[i] = (int)i;
    auto key = [&](int i) -> double {
        switch (which) {
            case 0: return w[i].real();
            case 1: return -w[i].real();
            case 2: return -std::abs(w[i]);
            default: return std::abs(w[i]);
        }
    };
    std::stable_sort(o.begin(), o.end(), [&](int a, int b) { return key(a) < key(b); });
    return o;
}

struct KSResult {
    std::vector<cd> theta;
    int nconv = 0;
    int restarts = 0;
    double max_rel = 0.0;
};

// Krylov-Schur restarted Arnoldi (Stewart, SIAM J. Matrix Anal. Appl. 23
// (2001) 601-614) for a non-Hermitian operator, in place of the reference's
// ARPACK znaupd / dnaupd run (src/operators.jl:3384-3390): Arnoldi steps with
// CGS2, the complex Schur form of the projected matrix reordered so that the
// wanted Ritz values lead, truncation to p of them (V <- V Q_p, the residual
// direction follows), ARPACK's Ritz bound |beta (Q y)_m| <= tol max(eps^(2/3),
// |theta|) as the convergence test.  Complex vectors (C128) throughout.
KSResult krylov_schur(Ctx& c, int k, int which, double tol, int ncv, int maxiter, const void* v0, void* X) {
    const int64_t n = c.n;
    const int m = (int)std::min<int64_t>(ncv, n);
    DevBuf V((size_t)n * (m + 1) * 16), tmp((size_t)n * m * 16);
    c.blas.copy(V.p, v0);
    const double nv0 = c.blas.norm(V.p);
    if (!(nv0 > 0)) throw Error(QS_ERR_ARGUMENT, "starting vector must be nonzero");
    c.blas.scale(V.p, V.p, cd(1.0 / nv0, 0));
    std::vector<cd> H((size_t)(m + 1) * m, cd(0, 0));
    auto Hij = [&](int i, int j) -> cd& { return H[(size_t)i * m + j]; };
    const double e23 = std::pow(kEps, 2.0 / 3.0);
    int j0 = 0;
    KSResult R;
    for (int iter = 0; iter < maxiter; ++iter) {
        R.restarts = iter;
        int me = m;
        double beta = 0.0;
        for (int j = j0; j < m; ++j) {
            void* wv = c.col(V, j + 1);
            c.matvec(c.col(V, j), wv);
            const std::vector<cd> h = orthogonalize(c, V, j + 1, wv);
            for (int i = 0; i <= j; ++i) Hij(i, j) += h[i];
            beta = c.blas.norm(wv);
            double hn = 0.0;
            for (int i = 0; i <= j; ++i) hn = std::max(hn, std::abs(Hij(i, j)));
            if (beta <= 1e-13 * std::max(1.0, hn)) {
                me = j + 1;   // an invariant subspace: its Ritz values are exact
                beta = 0.0;
                break;
            }
            c.blas.scale(wv, wv, cd(1.0 / beta, 0));
            Hij(j + 1, j) = beta;
        }
        std::vector<cd> T((size_t)me * me), Q;
        for (int i = 0; i < me; ++i)
            for (int j = 0; j < me; ++j) T[(size_t)i * me + j] = Hij(i, j);
        complex_schur(me, T, Q);
        // bring the wanted values to the front, in ranking order
        const int kk = std::min(k, me);
        int p = std::max(kk, std::min(me - 2, kk + (me - kk) / 2));
        if (me < m) p = me;
        std::vector<cd> diag(me);
        for (int i = 0; i < me; ++i) diag[i] = T[(size_t)i * me + i];
        const std::vector<int> order = ritz_order_complex(diag, which);
        std::vector<int> at(me);   // at[pos] = original index now at pos
        for (int i = 0; i < me; ++i) at[i] = i;
        for (int q = 0; q < p; ++q) {
            int pos = q;
            while (at[pos] != order[q]) ++pos;
            for (int s2 = pos - 1; s2 >= q; --s2) {
                schur_swap(me, T, Q, s2);
                std::swap(at[s2], at[s2 + 1]);
            }
        }
        int nconv = 0;
        double maxrel = 0.0;
        std::vector<std::vector<cd>> Y(kk);
        for (int q = 0; q < kk; ++q) {
            schur_vector(me, T, q, Y[q]);
            cd last = 0;
            for (int l = 0; l <= q; ++l) last += Q[(size_t)(me - 1) * me + l] * Y[q][l];
            const double th = std::abs(T[(size_t)q * me + q]);
            const double bound = beta * std::abs(last);
            maxrel = std::max(maxrel, bound / std::max(e23, th));
            if (bound <= tol * std::max(e23, th)) ++nconv;
        }
        R.nconv = nconv;
        R.max_rel = maxrel;
        if (nconv >= kk || me < m || iter == maxiter - 1) {
            R.theta.resize(kk);
            for (int q = 0; q < kk; ++q) {
                R.theta[q] = T[(size_t)q * me + q];
                std::vector<cd> z(me, cd(0, 0));
                for (int r = 0; r < me; ++r)
                    for (int l = 0; l <= q; ++l) z[r] += Q[(size_t)r * me + l] * Y[q][l];
                c.blas.combine((char*)X + (size_t)q * n * 16, V.p, n, me, z);
            }
            if (me < m) R.nconv = kk;
            QS_CUDA(cudaStreamSynchronize(c.s));
            return R;
        }
        // truncate to the p leading Schur vectors; the residual direction follows
        for (int q = 0; q < p; ++q) {
            std::vector<cd> z(me);
            for (int r = 0; r < me; ++r) z[r] = Q[(size_t)r * me + q];
            c.blas.combine(c.col(tmp, q), V.p, n, me, z);
        }
        QS_CUDA(cudaMemcpyAsync(V.p, tmp.p, (size_t)n * p * 16, cudaMemcpyDeviceToDevice, c.s));
        c.blas.copy(c.col(V, p), c.col(V, m));
        std::fill(H.begin(), H.end(), cd(0, 0));
        for (int i = 0; i < p; ++i)
            for (int j = i; j < p; ++j) Hij(i, j) = T[(size_t)i * me + j];
        for (int j = 0; j < p; ++j) Hij(p, j) = beta * Q[(size_t)(me - 1) * me + j];
        j0 = p;
    }
    return R;
}

}  // namespace

// ----------------------------------------------------- non-Hermitian eigsh
void eigs_general(Op& op, const qs_eigsh_opts& o, double* values, void* vectors, qs_eigsh_info* info) {
    auto t0 = std::chrono::steady_clock::now();
    const int64_t n = op.basis->n;
    const int k = o.k;
    if (k < 1 || k > n) throw Error(QS_ERR_ARGUMENT, "k must lie in 1:Ns");
    if (o.which < 0 || o.which > 3)
        throw Error(QS_ERR_ARGUMENT, "which must be SA, LA, SM or LM for a non-Hermitian operator");
    const bool dev = o.mem == QS_MEM_DEVICE;
    const size_t esz = op.complex_mat ? 16 : 8;   // dtype of v0
    Ctx c(op, VKind::C128);
    std::vector<cd> theta;
    DevBuf X((size_t)n * k * 16);
    int64_t mv = 0;
    int nconv = k, restarts = 0;
    double maxrel = 0.0;
    if (k >= n - 1) {
        // dense branch: the matrix column by column, its complex Schur form
        const int N = (int)n;
        std::vector<cd> A((size_t)N * N), hcol(N);
        DevBuf e(n * 16), col(n * 16);
        for (int j = 0; j < N; ++j) {
            std::vector<cd> h(N, cd(0, 0));
            h[j] = 1.0;
            QS_CUDA(cudaMemcpyAsync(e.p, h.data(), n * 16, cudaMemcpyHostToDevice, op.stream));
            c.matvec(e.p, col.p);
            QS_CUDA(cudaMemcpyAsync(hcol.data(), col.p, n * 16, cudaMemcpyDeviceToHost, op.stream));
            QS_CUDA(cudaStreamSynchronize(op.stream));
            for (int i = 0; i < N; ++i) A[(size_t)i * N + j] = hcol[i];
        }
        std::vector<cd> Q;
        complex_schur(N, A, Q);
        std::vector<cd> diag(N);
        for (int i = 0; i < N; ++i) diag[i] = A[(size_t)i * N + i];
        const std::vector<int> order = ritz_order_complex(diag, o.which);
        std::vector<cd> out((size_t)N * k);
        for (int q = 0; q < k; ++q) {
            std::vector<cd> y;
            schur_vector(N, A, order[q], y);
            for (int r = 0; r < N; ++r) {
                cd z = 0;
                for (int l = 0; l < N; ++l) z += Q[(size_t)r * N + l] * y[l];
                out[(size_t)q * N + r] = z;
            }
            theta.push_back(diag[order[q]]);
        }
        QS_CUDA(cudaMemcpyAsync(X.p, out.data(), out.size() * 16, cudaMemcpyHostToDevice, op.stream));
        mv = n;
    } else {
        TransientAssembly ta(op);
        int ncv = o.ncv > 0 ? o.ncv : std::max(20, 2 * k + 1);
        ncv = std::min(ncv, 128);
        if (ncv <= k) ncv = (int)std::min<int64_t>(n, k + 2);
        const double tol = o.tol > 0 ? o.tol : kEps;
        const int maxiter = o.maxiter > 0 ? o.maxiter : 300;
        DevBuf v0((size_t)n * 16);
        if (o.v0) {
            std::vector<cd> h(n);
            if (dev) {
                std::vector<char> raw(n * esz);
                QS_CUDA(cudaMemcpyAsync(raw.data(), o.v0, n * esz, cudaMemcpyDeviceToHost, op.stream));
                QS_CUDA(cudaStreamSynchronize(op.stream));
                for (int64_t i = 0; i < n; ++i)
                    h[i] = esz == 16 ? ((const cd*)raw.data())[i] : cd(((const double*)raw.data())[i], 0.0);
            } else {
                for (int64_t i = 0; i < n; ++i) h[i] = esz == 16 ? ((const cd*)o.v0)[i] : cd(o.v0[i], 0.0);
            }
            QS_CUDA(cudaMemcpyAsync(v0.p, h.data(), n * 16, cudaMemcpyHostToDevice, op.stream));
            QS_CUDA(cudaStreamSynchronize(op.stream));
        } else {
            random_vector(c, v0.p, 20261203ull);
        }
        KSResult R = krylov_schur(c, k, o.which, tol, ncv, maxiter, v0.p, X.p);
        if (R.nconv < k) throw Error(QS_ERR_NOT_CONVERGED, "eigsh did not converge within maxiter restarts");
        theta = R.theta;
        nconv = R.nconv;
        restarts = R.restarts;
        maxrel = R.max_rel;
        mv = c.matvecs;
    }
    for (int q = 0; q < k; ++q) {
        values[2 * q] = theta[q].real();
        values[2 * q + 1] = theta[q].imag();
    }
    if (o.want_vectors && vectors) {
        QS_CUDA(cudaMemcpyAsync(vectors, X.p, (size_t)n * k * 16, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                op.stream));
    }
    QS_CUDA(cudaStreamSynchronize(op.stream));
    if (info) {
        info->nconv = nconv;
        info->restarts = restarts;
        info->matvecs = mv;
        info->max_rel_residual = maxrel;
        info->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
}

// --------------------------------------------------------------------- eigsh
void eigsh(Op& op, const qs_eigsh_opts& o, double* values, void* vectors, qs_eigsh_info* info) {
    auto t0 = std::chrono::steady_clock::now();
    const int64_t n = op.basis->n;
    const int k = o.k;
    if (k < 1 || k > n) throw Error(QS_ERR_ARGUMENT, "k must lie in 1:Ns");
    if (o.which < 0 || o.which > 4) throw Error(QS_ERR_ARGUMENT, "which must be SA, LA, SM, LM, or BE");
    if (!op.hermitian)
        throw Error(QS_ERR_ARGUMENT, "a non-Hermitian operator returns complex eigenvalues: use qs_eigs");
    const bool cpx = op.complex_mat;
    const VKind k64 = cpx ? VKind::C128 : VKind::F64;
    const size_t esz = cpx ? 16 : 8;
    if (k >= n - 1) {
        // dense path (src/operators.jl:3379-3382): materialise and diagonalise
        int N = (int)n;
        std::vector<double> A((size_t)(cpx ? 2 * N : N) * (cpx ? 2 * N : N), 0.0);
        DevBuf e(n * esz), col(n * esz);
        std::vector<double> h(n * (cpx ? 2 : 1));
        Ctx c(op, k64);
        for (int j = 0; j < N; ++j) {
            std::fill(h.begin(), h.end(), 0.0);
            h[cpx ? 2 * j : j] = 1.0;
            QS_CUDA(cudaMemcpyAsync(e.p, h.data(), n * esz, cudaMemcpyHostToDevice, op.stream));
            c.matvec(e.p, col.p);
            QS_CUDA(cudaMemcpyAsync(h.data(), col.p, n * esz, cudaMemcpyDeviceToHost, op.stream));
            QS_CUDA(cudaStreamSynchronize(op.stream));
            for (int i = 0; i < N; ++i) {
                if (!cpx) {
                    A[(size_t)i * N + j] = h[i];
                } else {
                    double re = h[2 * i], im = h[2 * i + 1];
                    int M = 2 * N;
                    A[(size_t)i * M + j] = re;
                    A[(size_t)(i + N) * M + (j + N)] = re;
                    A[(size_t)(i + N) * M + j] = im;
                    A[(size_t)i * M + (j + N)] = -im;
                }
            }
        }
        int M = cpx ? 2 * N : N;
        for (int i = 0; i < M; ++i)
            for (int j = i + 1; j < M; ++j) {
                double avg = 0.5 * (A[(size_t)i * M + j] + A[(size_t)j * M + i]);
                A[(size_t)i * M + j] = A[(size_t)j * M + i] = avg;
            }
        std::vector<double> w, Z;
        sym_eig(M, A, w, Z);
        // complex Hermitian: eigenvalues appear twice in the real embedding
        std::vector<int> pick;
        if (!cpx) {
            for (int i = 0; i < M; ++i) pick.push_back(i);
        } else {
            std::vector<char> used(M, 0);
            for (int i = 0; i < M && (int)pick.size() < N; ++i) {
                if (used[i]) continue;
                pick.push_back(i);
                used[i] = 1;
                // skip the partner (closest unused eigenvalue)
                int best = -1;
                for (int q = i + 1; q < M; ++q)
                    if (!used[q]) { best = q; break; }
                if (best >= 0) used[best] = 1;
            }
        }
        std::vector<double> wp(pick.size());
        for (size_t q = 0; q < pick.size(); ++q) wp[q] = w[pick[q]];
        const std::vector<int> rank = ritz_order(wp, o.which, k);
        std::vector<int> sel;
        for (int q = 0; q < k; ++q) sel.push_back(pick[rank[q]]);
        for (int q = 0; q < k; ++q) values[q] = w[sel[q]];
        if (o.want_vectors && vectors) {
            double* out = (double*)vectors;
            for (int q = 0; q < k; ++q) {
                int ci = sel[q];
                if (!cpx) {
                    for (int i = 0; i < N; ++i) out[(size_t)q * N + i] = Z[(size_t)i * M + ci];
                } else {
                    double nrm = 0.0;
                    for (int i = 0; i < N; ++i) {
                        double re = Z[(size_t)i * M + ci], im = Z[(size_t)(i + N) * M + ci];
                        nrm += re * re + im * im;
                    }
                    nrm = std::sqrt(nrm);
                    for (int i = 0; i < N; ++i) {
                        out[2 * ((size_t)q * N + i)] = Z[(size_t)i * M + ci] / nrm;
                        out[2 * ((size_t)q * N + i) + 1] = Z[(size_t)(i + N) * M + ci] / nrm;
                    }
                }
            }
        }
        if (info) {
            info->nconv = k;
            info->restarts = 0;
            info->matvecs = n;
            info->max_rel_residual = 0;
            info->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        }
        return;
    }
    TransientAssembly ta(op);
    if (op.assembled && op.asm_.has_sell && k < n - 1) {
        // assembled operators: the batched engine with one slot (graph-replayed
        // steps, device-resident Lanczos coefficients, ARPACK's DGKS test)
        Op* one = &op;
        void* vec = vectors;
        eigsh_batch(&one, 1, o, values, o.want_vectors ? &vec : nullptr, info);
        if (info) info->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        return;
    }
    int ncv = o.ncv > 0 ? o.ncv : std::max(20, 2 * k + 1);
    ncv = std::min(ncv, 64);
    if (ncv <= k) ncv = std::min<int64_t>(n, k + 1);
    double tol = o.tol > 0 ? o.tol : kEps;
    int maxiter = o.maxiter > 0 ? o.maxiter : 300;
    const VKind vk = krylov_kind(op, cpx, o.precision);
    // reduced-precision vectors get an FP64 Rayleigh-quotient polish
    const bool single = vk != k64;
    Ctx c(op, vk, o.precision == 2);
    DevBuf v0((size_t)n * vk_bytes(vk));
    const bool dev = o.mem == QS_MEM_DEVICE;
    if (o.v0) {
        if (dev) {
            convert_vec(o.v0, k64, v0.p, vk, n, op.stream);
        } else {
            DevBuf t(n * esz);
            QS_CUDA(cudaMemcpyAsync(t.p, o.v0, n * esz, cudaMemcpyHostToDevice, op.stream));
            convert_vec(t.p, k64, v0.p, vk, n, op.stream);
            QS_CUDA(cudaStreamSynchronize(op.stream));
        }
    } else {
        random_vector(c, v0.p, 20261203ull);
    }
    DevBuf X((size_t)n * k * vk_bytes(vk));
    double tol_run = vk_single(vk) ? std::max(tol, 2e-6) : tol;
    TRResult R = trlan(c, k, o.which, tol_run, ncv, maxiter, v0.p, X.p);
    int64_t mv = c.matvecs;
    std::vector<double> theta = R.theta;
    DevBuf X64;
    if (single) {
        // FP64 polish: promote the Ritz vectors, Rayleigh quotient per vector,
        // and FP64 Lanczos refinement when the quadratic error bound
        // ||r||^2 / gap does not meet tol.
        X64.alloc((size_t)n * k * esz);
        for (int q = 0; q < k; ++q)
            convert_vec((char*)X.p + (size_t)q * n * vk_bytes(vk), vk, (char*)X64.p + (size_t)q * n * esz, k64, n,
                        op.stream);
        Ctx c64(op, k64);
        DevBuf Ax(n * esz);
        bool need_refine = false;
        double maxrel = 0.0;
        for (int q = 0; q < k; ++q) {
            void* xq = (char*)X64.p + (size_t)q * n * esz;
            double nx = c64.blas.norm(xq);
            c64.blas.scale(xq, xq, cd(1.0 / nx, 0));
            c64.matvec(xq, Ax.p);
            double th = c64.blas.dot(xq, Ax.p).real();
            c64.blas.axpy(Ax.p, xq, cd(-th, 0));
            double rn = c64.blas.norm(Ax.p);
            double gap = 1e300;
            for (int q2 = 0; q2 < (int)R.theta.size(); ++q2)
                if (q2 != q) gap = std::min(gap, std::fabs(R.theta[q2] - th));
            if (gap == 1e300) gap = std::max(1e-300, std::fabs(th));
            double bound = rn * rn / gap;
            theta[q] = th;
            maxrel = std::max(maxrel, rn / std::max(eps23(), std::fabs(th)));
            if (bound > tol * std::max(1.0, std::fabs(th))) need_refine = true;
        }
        mv += c64.matvecs;
        R.max_rel = maxrel;
        if (need_refine) {
            // FP64 thick-restart Lanczos started from the promoted first Ritz vector
            TRResult R2 = trlan(c64, k, o.which, tol, ncv, maxiter, X64.p, X64.p);
            mv += c64.matvecs;
            theta = R2.theta;
            R.nconv = R2.nconv;
            R.max_rel = R2.max_rel;
        } else {
            R.nconv = k;
        }
    }
    if (R.nconv < k) throw Error(QS_ERR_NOT_CONVERGED, "eigsh did not converge within maxiter restarts");
    for (int q = 0; q < k; ++q) values[q] = theta[q];
    if (o.want_vectors && vectors) {
        const void* src = single ? X64.p : X.p;
        QS_CUDA(cudaMemcpyAsync(vectors, src, (size_t)n * k * esz,
                                dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, op.stream));
        QS_CUDA(cudaStreamSynchronize(op.stream));
    }
    if (info) {
        info->nconv = R.nconv;
        info->restarts = R.restarts;
        info->matvecs = mv;
        info->max_rel_residual = R.max_rel;
        info->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
}

double eps23() { return std::pow(kEps, 2.0 / 3.0); }

// ------------------------------------------------------ Krylov exponential
namespace {

struct Fact {
    DevBuf V;
    std::vector<cd> H;  // (steps+1) x steps row-major
    double beta = 0;
    int completed = 0, steps = 0;
    double terminal = 0;
    bool hermitian = true;
    cd h(int i, int j) const { return H[(size_t)i * steps + j]; }
};

double hnorm(const std::vector<cd>& H) {
    double s = 0;
    for (const cd& v : H) s += std::norm(v);
    return std::sqrt(s);
}

// _krylov_factorization (src/operators.jl:1655-1731)
void factorize(Ctx& c, const void* v, int krylov_dim, Fact& F) {
    const int64_t n = c.n;
    F.beta = c.blas.norm(v);
    F.steps = (int)std::min<int64_t>(krylov_dim, n);
    F.V.alloc((size_t)n * (F.steps + 1) * vk_bytes(c.vk));
    F.H.assign((size_t)(F.steps + 1) * F.steps, cd(0, 0));
    F.hermitian = c.op.hermitian;
    F.completed = F.steps;
    F.terminal = 0;
    c.blas.scale(c.col(F.V, 0), v, cd(1.0 / F.beta, 0));
    auto H = [&](int i, int j) -> cd& { return F.H[(size_t)i * F.steps + j]; };
    double prev = 0;
    for (int col = 0; col < F.steps; ++col) {
        void* r = c.col(F.V, col + 1);
        c.matvec(c.col(F.V, col), r);
        if (F.hermitian) {
            if (col > 0) c.blas.axpy(r, c.col(F.V, col - 1), cd(-prev, 0));
            cd a = c.blas.dot(c.col(F.V, col), r);
            H(col, col) = a;
            c.blas.axpy(r, c.col(F.V, col), -a);
        } else {
            std::vector<cd> h = orthogonalize(c, F.V, col + 1, r);
            for (int row = 0; row <= col; ++row) H(row, col) = h[row];
        }
        double tn = c.blas.norm(r);
        F.terminal = tn;
        H(col + 1, col) = tn;
        if (F.hermitian && col < F.steps - 1) H(col, col + 1) = tn;
        if (tn <= 100 * kEps * std::max(1.0, hnorm(F.H))) {
            F.completed = col + 1;
            break;
        } else if (col < F.steps - 1) {
            c.blas.scale(r, r, cd(1.0 / tn, 0));
        }
        prev = tn;
    }
}

// Eigen-decomposition of the Hermitian projection (real symmetric tridiagonal).
void herm_eig(const Fact& F, std::vector<double>& w, std::vector<double>& U) {
    int m = F.completed;
    std::vector<double> T((size_t)m * m, 0.0);
    for (int i = 0; i < m; ++i) {
        T[(size_t)i * m + i] = F.h(i, i).real();
        if (i + 1 < m) T[(size_t)i * m + i + 1] = T[(size_t)(i + 1) * m + i] = F.h(i, i + 1).real();
    }
    sym_eig(m, T, w, U);
}

// _krylov_project: exp(scale * H) e_1 (Pade), result = beta V E[:,0].
double project(Ctx& c, const Fact& F, cd scale, void* out) {
    int m = F.completed;
    std::vector<cd> A((size_t)m * m), E;
    for (int i = 0; i < m; ++i)
        for (int j = 0; j < m; ++j) A[(size_t)i * m + j] = scale * F.h(i, j);
    expm_complex(m, A, E);
    std::vector<cd> coef(m);
    for (int i = 0; i < m; ++i) coef[i] = E[(size_t)i * m] * F.beta;
    c.blas.combine(out, F.V.p, c.n, m, coef);
    bool est_on = (F.completed == F.steps) && (F.completed < c.n);
    return est_on ? std::abs(scale) * F.terminal * F.beta * std::abs(E[(size_t)(m - 1) * m]) : 0.0;
}

// _krylov_expmv_vector (src/operators.jl:1758-1803)
void expmv_vector(Ctx& c, const void* v, cd scale, double tol, int krylov_dim, int depth, void* out) {
    if (scale == cd(0, 0)) {
        c.blas.copy(out, v);
        return;
    }
    double nv = c.blas.norm(v);
    if (nv == 0) {
        c.blas.copy(out, v);
        return;
    }
    Fact F;
    factorize(c, v, krylov_dim, F);
    double est = project(c, F, scale, out);
    double nr = c.blas.norm(out);
    if (est > tol * std::max(1.0, nr)) {
        if (depth >= 14)
            throw Error(QS_ERR_NOT_CONVERGED, "Krylov exponential action did not converge; increase krylov_dim");
        DevBuf mid((size_t)c.n * vk_bytes(c.vk)), init((size_t)c.n * vk_bytes(c.vk));
        c.blas.copy(init.p, v);
        expmv_vector(c, init.p, scale / 2.0, tol / 2, krylov_dim, depth + 1, mid.p);
        expmv_vector(c, mid.p, scale / 2.0, tol / 2, krylov_dim, depth + 1, out);
    }
}

}  // namespace

void expm_multiply(Op& op, cd a, const double* v, double* out, double tol, int krylov_dim, int precision) {
    const int64_t n = op.basis->n;
    if (tol <= 0) throw Error(QS_ERR_ARGUMENT, "tol must be positive");
    if (krylov_dim <= 0) throw Error(QS_ERR_ARGUMENT, "krylov_dim must be positive");
    TransientAssembly ta(op);
    if (op.assembled && op.asm_.has_sell && precision != 1 && krylov_dim <= 64 && n >= 2) {
        evolve_engine(op, v, {a}, tol, krylov_dim, precision, false, out);
        return;
    }
    VKind vk = krylov_kind(op, true, precision);
    Ctx c(op, vk, precision == 2);
    DevBuf d64(n * 16), dv((size_t)n * vk_bytes(vk)), dout((size_t)n * vk_bytes(vk));
    QS_CUDA(cudaMemcpyAsync(d64.p, v, n * 16, cudaMemcpyHostToDevice, op.stream));
    convert_vec(d64.p, VKind::C128, dv.p, vk, n, op.stream);
    expmv_vector(c, dv.p, a, tol, krylov_dim, 0, dout.p);
    convert_vec(dout.p, vk, d64.p, VKind::C128, n, op.stream);
    QS_CUDA(cudaMemcpyAsync(out, d64.p, n * 16, cudaMemcpyDeviceToHost, op.stream));
    QS_CUDA(cudaStreamSynchronize(op.stream));
}

// _krylov_expmv_times (src/operators.jl:1805-1893) + evolve's post-processing
void evolve(Op& op, const double* v0, double t0, const double* times, int nt, int imag_time, double tol, int krylov_dim,
            int precision, double* out) {
    const int64_t n = op.basis->n;
    if (tol <= 0) throw Error(QS_ERR_ARGUMENT, "tol must be positive");
    if (krylov_dim <= 0) throw Error(QS_ERR_ARGUMENT, "krylov_dim must be positive");
    TransientAssembly ta(op);
    if (op.assembled && op.asm_.has_sell && precision != 1 && krylov_dim <= 64 && n >= 2) {
        std::vector<cd> sc(nt);
        for (int i = 0; i < nt; ++i) {
            const double off = times[i] - t0;
            sc[i] = imag_time ? cd(-off, 0) : cd(0, -off);
        }
        evolve_engine(op, v0, sc, tol, krylov_dim, precision, imag_time != 0, out);
        return;
    }
    VKind vk = krylov_kind(op, true, precision);
    Ctx c(op, vk, precision == 2);
    DevBuf d64(n * 16), dv((size_t)n * vk_bytes(vk)), st((size_t)n * vk_bytes(vk));
    QS_CUDA(cudaMemcpyAsync(d64.p, v0, n * 16, cudaMemcpyHostToDevice, op.stream));
    convert_vec(d64.p, VKind::C128, dv.p, vk, n, op.stream);
    std::vector<cd> scales(nt);
    bool all_zero = true;
    for (int i = 0; i < nt; ++i) {
        double off = times[i] - t0;
        scales[i] = imag_time ? cd(-off, 0) : cd(0, -off);
        if (off != 0) all_zero = false;
    }
    auto emit = [&](int col, const void* state) {
        const void* src = state;
        if (imag_time) {
            double nr = c.blas.norm(state);
            c.blas.scale(st.p, state, cd(1.0 / nr, 0));
            src = st.p;
        }
        convert_vec(src, vk, d64.p, VKind::C128, n, op.stream);
        QS_CUDA(cudaMemcpyAsync(out + (size_t)col * 2 * n, d64.p, n * 16, cudaMemcpyDeviceToHost, op.stream));
        QS_CUDA(cudaStreamSynchronize(op.stream));
    };
    if (nt == 0) return;
    double nv = c.blas.norm(dv.p);
    if (nv == 0 || all_zero) {
        for (int i = 0; i < nt; ++i) emit(i, dv.p);
        return;
    }
    Fact F;
    factorize(c, dv.p, krylov_dim, F);
    DevBuf state((size_t)n * vk_bytes(vk));
    if (F.hermitian) {
        std::vector<double> w, U;
        herm_eig(F, w, U);
        int m = F.completed;
        for (int i = 0; i < nt; ++i) {
            cd s = scales[i];
            if (s == cd(0, 0)) {
                emit(i, dv.p);
                continue;
            }
            std::vector<cd> coef(m, cd(0, 0));
            for (int r = 0; r < m; ++r) {
                cd acc(0, 0);
                for (int q = 0; q < m; ++q) acc += U[(size_t)r * m + q] * (std::exp(s * w[q]) * U[q]);
                coef[r] = acc;
            }
            std::vector<cd> cb(m);
            for (int r = 0; r < m; ++r) cb[r] = coef[r] * F.beta;
            c.blas.combine(state.p, F.V.p, n, m, cb);
            bool est_on = (F.completed == F.steps) && (F.completed < n);
            double est = est_on ? std::abs(s) * F.terminal * F.beta * std::abs(coef[m - 1]) : 0.0;
            double nr = c.blas.norm(state.p);
            if (est > tol * std::max(1.0, nr)) expmv_vector(c, dv.p, s, tol, krylov_dim, 0, state.p);
            emit(i, state.p);
        }
    } else {
        for (int i = 0; i < nt; ++i) {
            cd s = scales[i];
            if (s == cd(0, 0)) {
                emit(i, dv.p);
                continue;
            }
            double est = project(c, F, s, state.p);
            double nr = c.blas.norm(state.p);
            if (est > tol * std::max(1.0, nr)) expmv_vector(c, dv.p, s, tol, krylov_dim, 0, state.p);
            emit(i, state.p);
        }
    }
}

}  // namespace qs
