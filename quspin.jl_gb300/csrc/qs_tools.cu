// qs_tools.cu -- tools.jl's Lanczos tools on the batched engine.
//
// The recurrences of many start vectors (the random vectors of a finite- or
// low-temperature Lanczos estimate, or the one v0 of lanczos_full) run as
// slots of one engine: each step is the engine's captured launch sequence
// over all starts.  The bases stay in the slots' FP64 storage; the tools read
// them in place:
//   * combine: out[:, c] = sum_i Y[i, c] q_i, rows streamed once per group of
//     eight output columns (HBM-bound, one read of the used basis per group);
//   * dots:    h_i = <q_i, w>, block partials over a fixed grid summed in a
//     fixed order (deterministic, no atomics).
#include <algorithm>
#include <cmath>

#include "qs_blas.cuh"
#include "qs_tools.h"

namespace qs {

namespace {

constexpr int kTT = 256;               // threads per tool block
constexpr int kDotBlocks = 152 * 4;    // row blocks of a dots launch (4 per SM)
constexpr int kDotV = 8;               // vectors per dots block
constexpr int kCombC = 8;              // output columns per combine launch
constexpr int kMaxLanczos = 256;

template <bool C>
__device__ __forceinline__ double2 ld2(const void* p, int64_t r) {
    if (C) return static_cast<const double2*>(p)[r];
    return make_double2(static_cast<const double*>(p)[r], 0.0);
}

// partial[b * nv + i] = sum over block b's rows of conj(V_i[r]) w[r], i in the
// block's group of kDotV vectors.
template <bool VC, bool WC>
__global__ void __launch_bounds__(kTT) tool_dots(const void* __restrict__ V, int64_t n, int nv,
                                                 const void* __restrict__ w, double2* __restrict__ partial) {
    const int i0 = blockIdx.y * kDotV;
    double re[kDotV], im[kDotV];
#pragma unroll
    for (int q = 0; q < kDotV; ++q) re[q] = im[q] = 0.0;
    const size_t cs = (size_t)n * (VC ? 2 : 1);
    const double* Vd = static_cast<const double*>(V);
    for (int64_t r = (int64_t)blockIdx.x * kTT + threadIdx.x; r < n; r += (int64_t)gridDim.x * kTT) {
        const double2 x = ld2<WC>(w, r);
#pragma unroll
        for (int q = 0; q < kDotV; ++q) {
            if (i0 + q < nv) {
                const double2 v = ld2<VC>(Vd + (size_t)(i0 + q) * cs, r);
                re[q] = fma(v.x, x.x, re[q]);
                im[q] = fma(v.x, x.y, im[q]);
                if (VC) {
                    re[q] = fma(v.y, x.y, re[q]);
                    im[q] = fma(-v.y, x.x, im[q]);
                }
            }
        }
    }
    __shared__ double sr[kDotV][kTT / 32], si[kDotV][kTT / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < kDotV; ++q) {
        double a = re[q], b = im[q];
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, o);
            b += __shfl_xor_sync(0xffffffffu, b, o);
        }
        if (lane == 0) {
            sr[q][wid] = a;
            si[q][wid] = b;
        }
    }
    __syncthreads();
    if (threadIdx.x < kDotV && i0 + (int)threadIdx.x < nv) {
        const int q = threadIdx.x;
        double a = 0, b = 0;
        for (int k = 0; k < kTT / 32; ++k) {
            a += sr[q][k];
            b += si[q][k];
        }
        partial[(size_t)blockIdx.x * nv + i0 + q] = make_double2(a, b);
    }
}

// out[i] = sum_b partial[b * nv + i], one block per vector, fixed order.
__global__ void __launch_bounds__(kTT) tool_dots_reduce(const double2* __restrict__ partial, int nb, int nv,
                                                        double2* __restrict__ out) {
    const int i = blockIdx.x;
    double a = 0, b = 0;
    for (int k = threadIdx.x; k < nb; k += kTT) {
        const double2 p = partial[(size_t)k * nv + i];
        a += p.x;
        b += p.y;
    }
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    __shared__ double sa[kTT / 32], sb[kTT / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        sa[wid] = a;
        sb[wid] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        a = b = 0;
        for (int k = 0; k < kTT / 32; ++k) {
            a += sa[k];
            b += sb[k];
        }
        out[i] = make_double2(a, b);
    }
}

// out[c0 + c][r] = sum_{i < nin} Y[(c0 + c) * nin + i] V_i[r] for c < kCombC
// (complex Y and out); the launch's coefficient group is staged in shared memory.
template <bool VC>
__global__ void __launch_bounds__(kTT) tool_combine(const void* __restrict__ V, int64_t n, int nin,
                                                    const double2* __restrict__ Y, int nc, double2* __restrict__ out) {
    __shared__ double2 ys[kMaxLanczos * kCombC];
    const int c0 = blockIdx.y * kCombC;
    const int cn = min(kCombC, nc - c0);
    for (int t = threadIdx.x; t < nin * kCombC; t += kTT) {
        const int i = t / kCombC, c = t % kCombC;
        ys[t] = c < cn ? Y[(size_t)(c0 + c) * nin + i] : make_double2(0.0, 0.0);
    }
    __syncthreads();
    const size_t cs = (size_t)n * (VC ? 2 : 1);
    const double* Vd = static_cast<const double*>(V);
    for (int64_t r = (int64_t)blockIdx.x * kTT + threadIdx.x; r < n; r += (int64_t)gridDim.x * kTT) {
        double ar[kCombC], ai[kCombC];
#pragma unroll
        for (int c = 0; c < kCombC; ++c) ar[c] = ai[c] = 0.0;
        for (int i = 0; i < nin; ++i) {
            const double2 v = ld2<VC>(Vd + (size_t)i * cs, r);
#pragma unroll
            for (int c = 0; c < kCombC; ++c) {
                const double2 y = ys[i * kCombC + c];
                ar[c] = fma(y.x, v.x, ar[c]);
                ai[c] = fma(y.y, v.x, ai[c]);
                if (VC) {
                    ar[c] = fma(-y.y, v.y, ar[c]);
                    ai[c] = fma(y.x, v.y, ai[c]);
                }
            }
        }
#pragma unroll
        for (int c = 0; c < kCombC; ++c)
            if (c < cn) out[(size_t)(c0 + c) * n + r] = make_double2(ar[c], ai[c]);
    }
}

__global__ void tool_promote(const double* __restrict__ x, int64_t n, double2* __restrict__ y) {
    for (int64_t r = (int64_t)blockIdx.x * kTT + threadIdx.x; r < n; r += (int64_t)gridDim.x * kTT)
        y[r] = make_double2(x[r], 0.0);
}

int row_grid(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + kTT - 1) / kTT, kDotBlocks)); }

// h[i] = <V_i, w> for i < nv (V: nv columns of n, real or complex), into host h.
void dots(const void* V, bool vc, int64_t n, int nv, const void* w, bool wc, std::vector<cd>& h, cudaStream_t s) {
    const int nb = row_grid(n);
    PoolBuf part((size_t)nb * nv * sizeof(double2), s), res((size_t)nv * sizeof(double2), s);
    dim3 g(nb, (nv + kDotV - 1) / kDotV);
    double2* pp = part.as<double2>();
    if (vc && wc) tool_dots<true, true><<<g, kTT, 0, s>>>(V, n, nv, w, pp);
    else if (vc) tool_dots<true, false><<<g, kTT, 0, s>>>(V, n, nv, w, pp);
    else if (wc) tool_dots<false, true><<<g, kTT, 0, s>>>(V, n, nv, w, pp);
    else tool_dots<false, false><<<g, kTT, 0, s>>>(V, n, nv, w, pp);
    QS_CUDA(cudaGetLastError());
    tool_dots_reduce<<<nv, kTT, 0, s>>>(pp, nb, nv, res.as<double2>());
    QS_CUDA(cudaGetLastError());
    note_launches(2);
    h.resize(nv);
    QS_CUDA(cudaMemcpyAsync(h.data(), res.p, (size_t)nv * sizeof(double2), cudaMemcpyDeviceToHost, s));
    QS_CUDA(cudaStreamSynchronize(s));
}

// out (device, n x nc complex) = V[:, 0:nin] Y (Y device, nin x nc complex).
void combine(const void* V, bool vc, int64_t n, int nin, const double2* Y, int nc, double2* out, cudaStream_t s) {
    dim3 g(row_grid(n), (nc + kCombC - 1) / kCombC);
    if (vc) tool_combine<true><<<g, kTT, 0, s>>>(V, n, nin, Y, nc, out);
    else tool_combine<false><<<g, kTT, 0, s>>>(V, n, nin, Y, nc, out);
    QS_CUDA(cudaGetLastError());
    note_launches(1);
}

const void* column(const LanczosSet& L, int s, int j) {
    const SlotDev& d = L.E->slot(L.ids[s]);
    return (const char*)d.V + (size_t)j * L.n * (L.cv ? 16 : 8);
}

void check_start(const LanczosSet& L, int s) {
    if (s < 0 || s >= (int)L.ids.size()) throw Error(QS_ERR_ARGUMENT, "start index outside the Lanczos set");
}

}  // namespace

std::unique_ptr<LanczosSet> lanczos_run(Op& op, const qs_lanczos_opts& o, int nstart, const double* v0) {
    if (nstart < 1 || !v0) throw Error(QS_ERR_ARGUMENT, "at least one start vector is required");
    const int64_t n = op.basis->n;
    if (o.m < 1 || o.m >= n) throw Error(QS_ERR_ARGUMENT, "Lanczos dimension m must satisfy 1 <= m < length(v0)");
    if (o.m > kMaxLanczos) throw Error(QS_ERR_ARGUMENT, "Lanczos dimension m must be at most 256");
    if (!op.hermitian) throw Error(QS_ERR_ARGUMENT, "the Lanczos recurrence needs a Hermitian operator");
    auto L = std::make_unique<LanczosSet>();
    L->op = &op;
    L->m = o.m;
    L->n = n;
    L->cv = op.complex_mat || o.complex_vectors;
    // the engine's basis holds m + 1 columns; m = 1 still takes two steps'
    // storage and reads only the first coefficient
    const int mm = std::max(2, o.m);
    L->E.reset(new Engine(Store::F64, op.stream));
    Engine& E = *L->E;
    const int comps = L->cv ? 2 : 1;
    // host start vectors travel in one copy, then load from device memory
    PoolBuf staged;
    const double* src = v0;
    if (o.mem != QS_MEM_DEVICE) {
        staged.alloc((size_t)nstart * n * comps * sizeof(double), op.stream);
        QS_CUDA(cudaMemcpyAsync(staged.p, v0, staged.bytes, cudaMemcpyHostToDevice, op.stream));
        src = staged.as<double>();
    }
    for (int s = 0; s < nstart; ++s) {
        // three-term recurrence as the reference; full_ortho: CGS2 against every kept vector
        const int id = E.add(op, mm, L->cv, true, 1, o.full_ortho ? 0 : 2);
        E.load(id, 0, src + (size_t)s * n * comps, true);
        L->ids.push_back(id);
    }
    L->norms = E.normalize(L->ids);
    for (double nr : L->norms)
        if (!(nr > 0)) throw Error(QS_ERR_ARGUMENT, "initial Lanczos vector must be nonzero");
    for (int id : L->ids) E.start(id, 0);
    for (int steps = E.steps_to_event(); steps > 0; steps = E.steps_to_event()) E.run(steps);
    std::vector<std::vector<cd>> H;
    E.records(L->ids, H);
    const double tol = o.eps > 0 ? o.eps : 2.220446049250313e-16;
    const int ld = mm + 1;
    for (int s = 0; s < nstart; ++s) {
        std::vector<double> a(o.m, 0.0), b(std::max(0, o.m - 1), 0.0);
        int used = o.m;
        for (int j = 0; j < o.m; ++j) {
            a[j] = H[s][(size_t)j * ld + j].real();
            if (j == o.m - 1) break;
            const double bj = H[s][(size_t)j * ld + j + 1].real();
            if (bj <= tol) {
                used = j + 1;
                break;
            }
            b[j] = bj;
        }
        L->alphas.push_back(std::move(a));
        L->betas.push_back(std::move(b));
        L->used.push_back(used);
    }
    note_launches(E.launches());
    return L;
}

void lanczos_rows(LanczosSet& L, int s, double* out, bool device) {
    check_start(L, s);
    const int comps = L.cv ? 2 : 1;
    for (int j = 0; j < L.used[s]; ++j) L.E->store(L.ids[s], j, out + (size_t)j * L.n * comps, device);
    note_launches(L.used[s]);
}

void lanczos_combine(LanczosSet& L, int s, const double* coeff, int ncoef, double* out, bool device) {
    check_start(L, s);
    if (ncoef < 1 || !coeff || !out) throw Error(QS_ERR_ARGUMENT, "one coefficient column at least is required");
    cudaStream_t st = L.E->stream();
    const int used = L.used[s];
    PoolBuf Y((size_t)used * ncoef * sizeof(double2), st);
    QS_CUDA(cudaMemcpyAsync(Y.p, coeff, Y.bytes, cudaMemcpyHostToDevice, st));
    PoolBuf tmp;
    double2* o = reinterpret_cast<double2*>(out);
    if (!device) {
        tmp.alloc((size_t)L.n * ncoef * sizeof(double2), st);
        o = tmp.as<double2>();
    }
    combine(column(L, s, 0), L.cv, L.n, used, Y.as<double2>(), ncoef, o, st);
    if (!device) QS_CUDA(cudaMemcpyAsync(out, tmp.p, tmp.bytes, cudaMemcpyDeviceToHost, st));
    QS_CUDA(cudaStreamSynchronize(st));
}

void lanczos_overlaps(LanczosSet& L, Op& obs, double* out) {
    if (obs.basis->n != L.n) throw Error(QS_ERR_DIMENSION, "the observable must act on a basis of the same size");
    cudaStream_t st = L.E->stream();
    const bool wc = L.cv || obs.complex_mat;
    PoolBuf w((size_t)L.n * (wc ? 16 : 8), st), xc;
    if (wc && !L.cv) xc.alloc((size_t)L.n * 16, st);
    std::vector<cd> h;
    for (int s = 0; s < (int)L.ids.size(); ++s) {
        MatvecCall c;
        c.x = column(L, s, 0);
        if (xc.p) {
            tool_promote<<<row_grid(L.n), kTT, 0, st>>>(static_cast<const double*>(c.x), L.n, xc.as<double2>());
            QS_CUDA(cudaGetLastError());
            note_launches(1);
            c.x = xc.p;
        }
        c.y = w.p;
        c.x_complex = c.y_complex = wc;
        op_matvec_device(obs, c, st);
        dots(column(L, s, 0), L.cv, L.n, L.used[s], w.p, wc, h, st);
        for (int i = 0; i < L.m; ++i) {
            const cd v = i < L.used[s] ? h[i] : cd(0, 0);
            out[((size_t)s * L.m + i) * 2] = v.real();
            out[((size_t)s * L.m + i) * 2 + 1] = v.imag();
        }
    }
}

void lanczos_ritz_matrix(LanczosSet& L, int s, Op& obs, const double* Y, int nv, double* out) {
    check_start(L, s);
    if (obs.basis->n != L.n) throw Error(QS_ERR_DIMENSION, "the observable must act on a basis of the same size");
    if (nv < 1 || nv > L.used[s] || !Y || !out) throw Error(QS_ERR_ARGUMENT, "nv must lie in 1:used");
    cudaStream_t st = L.E->stream();
    const int used = L.used[s];
    std::vector<double2> yc((size_t)used * nv);
    for (size_t t = 0; t < yc.size(); ++t) yc[t] = make_double2(Y[t], 0.0);
    PoolBuf Yd(yc.size() * sizeof(double2), st), R((size_t)L.n * nv * sizeof(double2), st),
        w((size_t)L.n * sizeof(double2), st);
    QS_CUDA(cudaMemcpyAsync(Yd.p, yc.data(), Yd.bytes, cudaMemcpyHostToDevice, st));
    combine(column(L, s, 0), L.cv, L.n, used, Yd.as<double2>(), nv, R.as<double2>(), st);
    std::vector<cd> h;
    for (int c = 0; c < nv; ++c) {
        MatvecCall mc;
        mc.x = R.as<double2>() + (size_t)c * L.n;
        mc.y = w.p;
        mc.x_complex = mc.y_complex = true;
        op_matvec_device(obs, mc, st);
        dots(R.p, true, L.n, nv, w.p, true, h, st);
        for (int a = 0; a < nv; ++a) {
            out[((size_t)c * nv + a) * 2] = h[a].real();
            out[((size_t)c * nv + a) * 2 + 1] = h[a].imag();
        }
    }
}

void expm_columns(Op& op, const double* V, int ncol, const std::vector<cd>& scales, double tol, int krylov_dim,
                  int precision, bool normalise, double* out, bool device) {
    if (ncol < 1 || scales.empty()) throw Error(QS_ERR_ARGUMENT, "at least one column and one scale are required");
    const int64_t n = op.basis->n;
    const int nt = (int)scales.size();
    cudaStream_t st = op.stream;
    const size_t col_bytes = (size_t)n * 16;
    PoolBuf dV;
    const double* v = V;
    if (!device) {
        dV.alloc(col_bytes * ncol, st);
        QS_CUDA(cudaMemcpyAsync(dV.p, V, dV.bytes, cudaMemcpyHostToDevice, st));
        QS_CUDA(cudaStreamSynchronize(st));
        v = dV.as<double>();
    }
    // columns in waves whose Krylov slots fit in half the free memory
    size_t fr = 0, tot = 0;
    QS_CUDA(cudaMemGetInfo(&fr, &tot));
    const int m = (int)std::max<int64_t>(2, std::min<int64_t>(krylov_dim, n));
    const size_t per = Engine::slot_bytes(n, m, true, 1, precision == 0 ? Store::F64 : Store::DF) + col_bytes * nt;
    const int wave = (int)std::max<size_t>(1, std::min<size_t>(ncol, (fr / 2) / std::max<size_t>(per, 1)));
    for (int c0 = 0; c0 < ncol; c0 += wave) {
        const int c1 = std::min(ncol, c0 + wave);
        PoolBuf states(col_bytes * nt * (c1 - c0), st);
        std::vector<Op*> ops(c1 - c0, &op);
        std::vector<const double*> v0s;
        std::vector<double*> outs;
        for (int c = c0; c < c1; ++c) {
            v0s.push_back(v + (size_t)c * n * 2);
            outs.push_back(states.as<double>() + (size_t)(c - c0) * n * 2 * nt);
        }
        evolve_blocks(ops, v0s, scales, tol, krylov_dim, precision, outs);
        Blas B(VKind::C128, n, st);
        for (int c = c0; c < c1; ++c)
            for (int i = 0; i < nt; ++i) {
                double* src = outs[c - c0] + (size_t)i * n * 2;
                if (normalise) {
                    const double nr = B.norm(src);
                    if (nr > 0) B.scale(src, src, cd(1.0 / nr, 0));
                }
                double* dst = out + ((size_t)i * ncol + c) * n * 2;   // out[:, c, i]
                QS_CUDA(cudaMemcpyAsync(dst, src, col_bytes, device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                        st));
            }
        QS_CUDA(cudaStreamSynchronize(st));
    }
}

void block_expm(const std::vector<Op*>& ops, bool pcon, const double* psi, const std::vector<cd>& scales, double tol,
                int krylov_dim, int precision, double* out, bool device) {
    if (ops.empty()) throw Error(QS_ERR_ARGUMENT, "at least one block is required");
    const int64_t rows = basis_projection_rows(*ops[0]->basis, pcon);
    for (Op* op : ops)
        if (basis_projection_rows(*op->basis, pcon) != rows)
            throw Error(QS_ERR_DIMENSION, "the blocks must share one projection space");
    cudaStream_t st = ops[0]->stream;
    const int nt = (int)scales.size();
    PoolBuf dpsi, dout;
    const double* p = psi;
    double* o = out;
    if (!device) {
        dpsi.alloc((size_t)rows * 16, st);
        QS_CUDA(cudaMemcpyAsync(dpsi.p, psi, dpsi.bytes, cudaMemcpyHostToDevice, st));
        dout.alloc((size_t)rows * nt * 16, st);
        p = dpsi.as<double>();
        o = dout.as<double>();
    }
    QS_CUDA(cudaStreamSynchronize(st));
    // c_b = P_b^H psi; blocks where it vanishes (norm <= 1000 eps) are left out,
    // as the reference's _active_block_entries does (tools.jl:2445-2477)
    std::vector<PoolBuf> coef(ops.size()), states(ops.size());
    std::vector<Op*> act;
    std::vector<const double*> v0s;
    std::vector<double*> outs;
    std::vector<size_t> which;
    for (size_t b = 0; b < ops.size(); ++b) {
        Basis& B = *ops[b]->basis;
        coef[b].alloc((size_t)B.n * 16, B.stream);
        basis_project(B, pcon, 1, p, coef[b].as<double>(), false, true);
        Blas nrm(VKind::C128, B.n, B.stream);
        if (!(nrm.norm(coef[b].p) > 1000 * 2.220446049250313e-16)) continue;
        states[b].alloc((size_t)B.n * nt * 16, st);
        act.push_back(ops[b]);
        v0s.push_back(coef[b].as<double>());
        outs.push_back(states[b].as<double>());
        which.push_back(b);
    }
    if (act.empty()) throw Error(QS_ERR_ARGUMENT, "initial state has no projection onto the selected blocks");
    evolve_blocks(act, v0s, scales, tol, krylov_dim, precision, outs);
    // out[:, i] = sum_b P_b state_b(i), blocks in the given order, all times
    // of a block in one launch
    QS_CUDA(cudaMemsetAsync(o, 0, (size_t)rows * nt * 16, st));
    QS_CUDA(cudaStreamSynchronize(st));
    for (size_t q = 0; q < act.size(); ++q)
        basis_project(*act[q]->basis, pcon, 0, outs[q], o, true, true, nt);
    if (!device) {
        QS_CUDA(cudaMemcpyAsync(out, o, (size_t)rows * nt * 16, cudaMemcpyDeviceToHost, st));
        QS_CUDA(cudaStreamSynchronize(st));
    }
}

}  // namespace qs

namespace qs {
namespace {

// Eight independent FP64 FMA chains per thread; the result is written so the
// chains are not removed.
__global__ void __launch_bounds__(256) fma_probe_kernel(double* __restrict__ out, double a, double b, int iters) {
    double x[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) x[u] = threadIdx.x + u;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 8; ++u) x[u] = fma(x[u], a, b);
    }
    double t = 0;
#pragma unroll
    for (int u = 0; u < 8; ++u) t += x[u];
    out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = t;
}

}  // namespace

double fp64_fma_rate() {
    int dev = 0, sms = 152;
    QS_CUDA(cudaGetDevice(&dev));
    QS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = sms * 8, threads = 256, iters = 4096;
    DevBuf out((size_t)blocks * threads * sizeof(double));
    cudaStream_t s = nullptr;
    QS_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    cudaEvent_t e0, e1;
    QS_CUDA(cudaEventCreate(&e0));
    QS_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {
        QS_CUDA(cudaEventRecord(e0, s));
        fma_probe_kernel<<<blocks, threads, 0, s>>>(out.as<double>(), 0.999999, 1e-7, iters);
        QS_CUDA(cudaEventRecord(e1, s));
        QS_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        QS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        best = std::min(best, ms);
    }
    note_launches(3);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(s);
    return (double)blocks * threads * 8 * iters / (best * 1e-3);
}

}  // namespace qs
