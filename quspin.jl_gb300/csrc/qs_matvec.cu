// qs_matvec.cu -- the fused matrix-free Hamiltonian action y = alpha*op(A)x + beta*y.
//
// Replaces the reference's serial scatter (_apply_spin_term!, src/operators.jl:
// 2554-2589) and its symmetric lift -> parent apply -> project path
// (_apply_spin_terms!, 2591-2636) with a row-wise pull form in representative
// space.  One thread owns one output row r (its representative s_r):
//
//   y[r] = beta*y[r] + alpha*( d[r] x[r] +
//          sum_progs  A[s_r, t] * chi(h_t) * sqrt(stab(m_t) / stab(s_r)) * x[rank(m_t)] )
//
// where t runs over the states reached from s_r by the transposed term chain
// (A[s,t] = <t|A^T|s>), m_t = h_t(t) is the orbit minimum of t, chi the sector
// character and stab the stabiliser order.  This equals (P'AP)[r, :] x for the
// reference's projector P (columns P_chi|s_min>/norm) when A commutes with the
// group.  No scatter, no atomics: every row is written once, and the summation
// order per row is fixed, so repeated calls are bit-identical.
//
// Rank lookups: full 2^L space -> the state itself; fixed-weight sector
// without spatial symmetry -> combinadic rank (src/discrete_basis.jl:1879-1906);
// symmetric sector -> search of the sorted representatives with a
// shared-memory splitter stage.
#include <cuda_runtime.h>

#include <cstdlib>
#include <cstring>

#include <algorithm>
#include <atomic>

#include "qs_device.cuh"
#include "qs_df.cuh"
#include "qs_internal.h"

namespace qs {

namespace {

constexpr int kMvThreads = 256;
constexpr int kMaxSplit = 2048;
constexpr int kSmemProgs = 160;

template <typename T> struct V2;
template <> struct V2<double> { using t = double2; };
template <> struct V2<float> { using t = float2; };

struct MvArgs {
    const void* reps;
    const uint16_t* stab;
    const void* split;
    int64_t n, nsplit, stride;
    const GroupDesc* group;
    const uint64_t* binom;
    int L, nup, pauli;
    const TermProg* progs;
    int nprog;
    const int32_t* index;    // direct rank -> column table (mode 3)
    FastGroup fast;          // zero-run orbit search when enabled
    const double* fast_chi;  // complex character per fast element code
    const void* diag;        // complex, precision of the call
    int conj_amp, conj_chi;
    double ar, ai, br, bi;
    int beta_zero;
    const void* x;
    void* y;
};

// Applies one transition program to s (operator characters as in
// src/operators.jl:343-379).  Returns false when an operator annihilates the
// state.  Distinct-site programs use their compiled masks; programs that touch
// a site twice run the character interpreter.
template <typename U, typename T>
__device__ __forceinline__ bool run_prog(const TermProg& p, int pauli, U s, U& t, T& ar, T& ai) {
    if (p.distinct) {
        if ((s & (U)p.need1) != (U)p.need1 || (s & (U)p.need0) != (U)0) return false;
        t = s ^ (U)p.flip;
        int par = __popcll((unsigned long long)(~s & (U)p.zmask)) + __popcll((unsigned long long)(s & (U)p.ymask));
        T re = (T)p.amp0_re, im = (T)p.amp0_im;
        if (par & 1) {
            re = -re;
            im = -im;
        }
        ar = re;
        ai = im;
        return true;
    }
    double re = p.coef_re, im = p.coef_im;
    const double zs = pauli ? 1.0 : 0.5;
    const double pm = pauli ? 2.0 : 1.0;
    t = s;
    for (int i = 0; i < p.nops; ++i) {
        const U bit = (U)1 << p.sites[i];
        const bool occ = (t & bit) != 0;
        switch (p.ops[i]) {
            case 'I':
                break;
            case 'z':
                re *= occ ? zs : -zs;
                im *= occ ? zs : -zs;
                break;
            case '+':
                if (occ) return false;
                t |= bit;
                re *= pm;
                im *= pm;
                break;
            case '-':
                if (!occ) return false;
                t &= ~bit;
                re *= pm;
                im *= pm;
                break;
            case 'x':
                t ^= bit;
                re *= zs;
                im *= zs;
                break;
            case 'y': {
                // occupied -> -i*scale, empty -> +i*scale
                t ^= bit;
                double f = occ ? -zs : zs;
                double nre = -im * f, nim = re * f;
                re = nre;
                im = nim;
                break;
            }
            default:
                return false;
        }
    }
    ar = (T)re;
    ai = (T)im;
    return true;
}

template <typename U>
__device__ __forceinline__ U row_state(const MvArgs& a, int mode, int64_t r) {
    if (mode == 2) return ((const U*)a.reps)[r];
    if (mode == 0) return (U)r;
    // unrank a fixed-weight state (inverse of the combinadic rank)
    U s = 0;
    int b = a.L - 1;
    int64_t rem = r;
    for (int p = a.nup; p >= 1; --p) {
        while ((int64_t)__ldg(a.binom + b * 65 + p) > rem) --b;
        s |= (U)1 << b;
        rem -= (int64_t)__ldg(a.binom + b * 65 + p);
        --b;
    }
    return s;
}

// The fixed-weight state of combinadic rank r (inverse of combinadic_rank32),
// with the C(bit, p) table in shared memory.
__device__ __forceinline__ uint32_t unrank32(int64_t r, const uint32_t* binom32, int L, int nup) {
    uint32_t s = 0, rem = (uint32_t)r;
    int b = L - 1;
    for (int p = nup; p >= 1; --p) {
        while (binom32[b * 33 + p] > rem) --b;
        s |= 1u << b;
        rem -= binom32[b * 33 + p];
        --b;
    }
    return s;
}

// rank(t) from rank(s) = rs for fixed-weight states of equal weight that
// differ only in bits lo .. hi: the set bits below lo and above hi keep their
// particle numbers, so only the set bits inside the span change their terms
// C(bit, particle).  A short span (a bond, a plaquette) costs a few table
// reads instead of the nup of a full rank; a long one (the periodic bond of a
// chain) takes the full rank of t.
__device__ __forceinline__ int64_t rank_from32(uint32_t s, int64_t rs, uint32_t t, const uint32_t* binom32) {
    const uint32_t f = s ^ t;
    if (!f) return rs;
    const int lo = __ffs((int)f) - 1, hi = 31 - __clz((int)f);
    if (hi - lo > 8) return combinadic_rank32(t, binom32);
    const uint32_t span = (hi == 31 ? 0xffffffffu : ((1u << (hi + 1)) - 1u)) & ~((1u << lo) - 1u);
    const int m0 = __popc(s & ((1u << lo) - 1u));
    int64_t d = 0;
    uint32_t bs = s & span, bt = t & span;
    for (int p = m0 + 1; bs; ++p) {
        d -= binom32[(__ffs((int)bs) - 1) * 33 + p];
        bs &= bs - 1;
    }
    for (int p = m0 + 1; bt; ++p) {
        d += binom32[(__ffs((int)bt) - 1) * 33 + p];
        bt &= bt - 1;
    }
    return rs + d;
}

template <typename T, bool kCV>
__device__ __forceinline__ void load_x(const MvArgs& a, int64_t i, T& xr, T& xi) {
    if (kCV) {
        typename V2<T>::t v = ((const typename V2<T>::t*)a.x)[i];
        xr = v.x;
        xi = v.y;
    } else {
        xr = ((const T*)a.x)[i];
        xi = 0;
    }
}

template <typename U, int kMode, bool kCM, bool kCV, typename T>
__global__ void __launch_bounds__(kMvThreads) matvec_kernel(MvArgs a) {
    constexpr bool kSym = kMode >= 2;
    __shared__ GroupSmem g;
    __shared__ U spl[kMode == 2 ? kMaxSplit : 1];
    constexpr bool kB32 = (kMode == 3 || kMode == 1) && sizeof(U) == 4;
    __shared__ uint32_t binom32[kB32 ? 32 * 33 : 1];
    __shared__ TermProg progs[kSmemProgs];
    __shared__ double sqrt_stab[kMaxGroup + 1];
    if (kSym) {
        load_group_smem(g, a.group);
        if (kMode == 2)
            for (int i = threadIdx.x; i < a.nsplit; i += blockDim.x) spl[i] = ((const U*)a.split)[i];
        for (int i = threadIdx.x; i <= kMaxGroup; i += blockDim.x) sqrt_stab[i] = sqrt((double)i);
    }
    // C(bit, p) for bit < 32, p <= 32: all below 2^32
    if (kB32 && a.nup >= 0)
        for (int i = threadIdx.x; i < 32 * 33; i += blockDim.x)
            binom32[i] = (uint32_t)a.binom[(i / 33) * 65 + (i % 33)];
    const int np_smem = a.nprog < kSmemProgs ? a.nprog : kSmemProgs;
    for (int i = threadIdx.x; i < np_smem; i += blockDim.x) progs[i] = a.progs[i];
    __syncthreads();
    const double* chi_re = a.group->chi_re;
    const double* chi_im = a.group->chi_im;

    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < a.n; r += (int64_t)gridDim.x * blockDim.x) {
        const U s = (kB32 && kMode == 1) ? (U)unrank32(r, binom32, a.L, a.nup) : row_state<U>(a, kSym ? 2 : kMode, r);
        T inv_sr = 1;
        if (kSym) inv_sr = (T)1 / (T)sqrt_stab[a.stab[r]];
        T acc_r = 0, acc_i = 0;
        for (int k = 0; k < a.nprog; ++k) {
            const TermProg& p = (k < kSmemProgs) ? progs[k] : a.progs[k];
            U t;
            T wr, wi;
            if (!run_prog<U, T>(p, a.pauli, s, t, wr, wi)) continue;
            int64_t idx;
            if (a.conj_amp) wi = -wi;
            if (kSym) {
                U m;
                int bi, st;
                const double* chr = chi_re;
                const double* chi = chi_im;
                int cstride = 1;
                if (a.fast.enabled) {
                    orbit_min_fast<U>(a.fast, t, m, bi, st);
                    chr = a.fast_chi;
                    chi = a.fast_chi + 1;
                    cstride = 2;
                } else {
                    orbit_min<U>(g, t, m, bi, st);
                }
                if (kMode == 3) {
                    int64_t rk;
                    if (a.nup < 0) rk = (int64_t)m;
                    else if (sizeof(U) == 4) rk = combinadic_rank32((uint32_t)m, binom32);
                    else rk = combinadic_rank<U>(m, a.binom, 65);
                    idx = __ldg(a.index + rk);
                } else {
                    idx = rank_search<U>((const U*)a.reps, a.n, spl, (int)a.nsplit, a.stride, m);
                }
                if (idx < 0) continue;
                const T f = (T)sqrt_stab[st] * inv_sr;
                if (kCM) {
                    T cr = (T)__ldg(chr + bi * cstride), ci = (T)__ldg(chi + bi * cstride);
                    if (a.conj_chi) ci = -ci;
                    T nr = wr * cr - wi * ci, ni = wr * ci + wi * cr;
                    wr = nr * f;
                    wi = ni * f;
                } else {
                    wr *= (T)__ldg(chr + bi * cstride) * f;
                }
            } else if (kMode == 1) {
                if (__popcll((unsigned long long)t) != a.nup) continue;
                if (kB32) idx = rank_from32((uint32_t)s, r, (uint32_t)t, binom32);
                else idx = combinadic_rank<U>(t, a.binom, 65);
            } else {
                idx = (int64_t)t;
            }
            T xr, xi;
            load_x<T, kCV>(a, idx, xr, xi);
            if (kCM) {
                acc_r += wr * xr - wi * xi;
                acc_i += wr * xi + wi * xr;
            } else if (kCV) {
                acc_r += wr * xr;
                acc_i += wr * xi;
            } else {
                acc_r += wr * xr;
            }
        }
        // diagonal (user + extracted), conjugated with the operator
        {
            typename V2<T>::t d = ((const typename V2<T>::t*)a.diag)[r];
            T dr = d.x, di = a.conj_amp ? -d.y : d.y;
            T xr, xi;
            load_x<T, kCV>(a, r, xr, xi);
            if (kCV) {
                acc_r += dr * xr - di * xi;
                acc_i += dr * xi + di * xr;
            } else {
                acc_r += dr * xr;
            }
        }
        if (kCV) {
            typename V2<T>::t* y = (typename V2<T>::t*)a.y;
            T yr = 0, yi = 0;
            if (!a.beta_zero) {
                typename V2<T>::t yo = y[r];
                yr = (T)a.br * yo.x - (T)a.bi * yo.y;
                yi = (T)a.br * yo.y + (T)a.bi * yo.x;
            }
            typename V2<T>::t out;
            out.x = yr + (T)a.ar * acc_r - (T)a.ai * acc_i;
            out.y = yi + (T)a.ar * acc_i + (T)a.ai * acc_r;
            y[r] = out;
        } else {
            T* y = (T*)a.y;
            T yr = a.beta_zero ? (T)0 : (T)a.br * y[r];
            y[r] = yr + (T)a.ar * acc_r;
        }
    }
}


// ----------------------------------------------------- warp-cooperative rank
// First index in [a, b) whose value is >= q (b when none), with all 32 lanes
// of the warp probing together: each round reads 32 evenly spaced entries and
// a ballot keeps the one stride that holds the bound, so a range shrinks
// 32-fold per round.  q and the range are the same in every lane.
template <typename U, class Get>
__device__ __forceinline__ int64_t warp_lower_bound(int64_t a, int64_t b, U q, Get get) {
    const int lane = threadIdx.x & 31;
    while (b - a > 32) {
        const int64_t step = (b - a + 31) / 32;
        const int64_t idx = a + (int64_t)lane * step;
        const unsigned below = __ballot_sync(0xffffffffu, idx < b && get(idx) < q);
        const int c = __popc(below);   // probes are ascending, so the ones below q are a prefix
        if (c == 0) return a;
        const int64_t nb = a + (int64_t)c * step;
        a = a + (int64_t)(c - 1) * step + 1;
        b = nb < b ? nb : b;
    }
    const int64_t idx = a + lane;
    return a + __popc(__ballot_sync(0xffffffffu, idx < b && get(idx) < q));
}

// Column of the representative `key` of every lane that wants one (-1: not a
// representative), resolved for one lane after another by the whole warp: two
// rounds over the shared-memory splitters (splitter i = reps[i * stride]),
// then rounds over the splitter's segment of the sorted representatives in
// global memory.  Every lane of the warp must call it.
template <typename U>
__device__ __forceinline__ int64_t rank_warp(const U* __restrict__ reps, int64_t n, const U* spl, int nsplit,
                                             int64_t stride, U key, bool want) {
    const int lane = threadIdx.x & 31;
    int64_t out = -1;
    unsigned pend = __ballot_sync(0xffffffffu, want);
    while (pend) {
        const int j = __ffs(pend) - 1;
        pend &= pend - 1;
        const U q = __shfl_sync(0xffffffffu, key, j);
        const int64_t ls = warp_lower_bound<U>(0, nsplit, q, [&](int64_t i) { return spl[i]; });
        int64_t idx = -1;
        if (ls < nsplit && spl[ls] == q) {
            idx = ls * stride;
        } else if (ls > 0) {
            const int64_t sa = (ls - 1) * stride, sb = sa + stride < n ? sa + stride : n;
            const int64_t lb = warp_lower_bound<U>(sa, sb, q, [&](int64_t i) { return __ldg(reps + i); });
            if (lb < sb && __ldg(reps + lb) == q) idx = lb;
        }
        if (lane == j) out = idx;
    }
    return out;
}

// The symmetric-sector product of matvec_kernel with the rank of every
// generated state found by rank_warp (QS_RANK_MODE=warp): rows are taken a
// warp at a time so that all 32 lanes reach every lookup together.
template <typename U, bool kCM, bool kCV, typename T>
__global__ void __launch_bounds__(kMvThreads) matvec_warp_rank_kernel(MvArgs a) {
    __shared__ GroupSmem g;
    __shared__ U spl[kMaxSplit];
    __shared__ TermProg progs[kSmemProgs];
    __shared__ double sqrt_stab[kMaxGroup + 1];
    load_group_smem(g, a.group);
    for (int i = threadIdx.x; i < a.nsplit; i += blockDim.x) spl[i] = ((const U*)a.split)[i];
    for (int i = threadIdx.x; i <= kMaxGroup; i += blockDim.x) sqrt_stab[i] = sqrt((double)i);
    const int np_smem = a.nprog < kSmemProgs ? a.nprog : kSmemProgs;
    for (int i = threadIdx.x; i < np_smem; i += blockDim.x) progs[i] = a.progs[i];
    __syncthreads();
    const double* chi_re = a.group->chi_re;
    const double* chi_im = a.group->chi_im;
    const int lane = threadIdx.x & 31;
    const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = blockIdx.x * (int64_t)blockDim.x + (threadIdx.x & ~31); base < a.n; base += nthreads) {
        const int64_t r = base + lane;
        const bool rv = r < a.n;
        const U s = rv ? ((const U*)a.reps)[r] : (U)0;
        const T inv_sr = rv ? (T)1 / (T)sqrt_stab[a.stab[r]] : (T)0;
        T acc_r = 0, acc_i = 0;
        for (int k = 0; k < a.nprog; ++k) {
            const TermProg& p = (k < kSmemProgs) ? progs[k] : a.progs[k];
            U t = 0, m = 0;
            T wr = 0, wi = 0;
            int bi = 0, st = 0;
            const bool alive = rv && run_prog<U, T>(p, a.pauli, s, t, wr, wi);
            const double* chr = chi_re;
            const double* chi = chi_im;
            int cstride = 1;
            if (alive) {
                if (a.conj_amp) wi = -wi;
                if (a.fast.enabled) {
                    orbit_min_fast<U>(a.fast, t, m, bi, st);
                    chr = a.fast_chi;
                    chi = a.fast_chi + 1;
                    cstride = 2;
                } else {
                    orbit_min<U>(g, t, m, bi, st);
                }
            }
            const int64_t idx = rank_warp<U>((const U*)a.reps, a.n, spl, (int)a.nsplit, a.stride, m, alive);
            if (!alive || idx < 0) continue;
            const T f = (T)sqrt_stab[st] * inv_sr;
            if (kCM) {
                T cr = (T)__ldg(chr + bi * cstride), ci = (T)__ldg(chi + bi * cstride);
                if (a.conj_chi) ci = -ci;
                const T nr = wr * cr - wi * ci, ni = wr * ci + wi * cr;
                wr = nr * f;
                wi = ni * f;
            } else {
                wr *= (T)__ldg(chr + bi * cstride) * f;
            }
            T xr, xi;
            load_x<T, kCV>(a, idx, xr, xi);
            if (kCM) {
                acc_r += wr * xr - wi * xi;
                acc_i += wr * xi + wi * xr;
            } else if (kCV) {
                acc_r += wr * xr;
                acc_i += wr * xi;
            } else {
                acc_r += wr * xr;
            }
        }
        if (!rv) continue;
        typename V2<T>::t d = ((const typename V2<T>::t*)a.diag)[r];
        const T dr = d.x, di = a.conj_amp ? -d.y : d.y;
        T xr, xi;
        load_x<T, kCV>(a, r, xr, xi);
        if (kCV) {
            acc_r += dr * xr - di * xi;
            acc_i += dr * xi + di * xr;
        } else {
            acc_r += dr * xr;
        }
        if (kCV) {
            typename V2<T>::t* y = (typename V2<T>::t*)a.y;
            T yr = 0, yi = 0;
            if (!a.beta_zero) {
                typename V2<T>::t yo = y[r];
                yr = (T)a.br * yo.x - (T)a.bi * yo.y;
                yi = (T)a.br * yo.y + (T)a.bi * yo.x;
            }
            typename V2<T>::t o;
            o.x = yr + (T)a.ar * acc_r - (T)a.ai * acc_i;
            o.y = yi + (T)a.ar * acc_i + (T)a.ai * acc_r;
            y[r] = o;
        } else {
            T* y = (T*)a.y;
            const T yr = a.beta_zero ? (T)0 : (T)a.br * y[r];
            y[r] = yr + (T)a.ar * acc_r;
        }
    }
}

// General path for operators that do not commute with the group (reference:
// check_symm=false on a symmetric basis, src/operators.jl:2500-2506): the full
// P' A P with both projector sides expanded over the group,
//   y[r] = (1/stab_r) sum_e chi'(g_e)/sqrt|orb r| sum_t A[g_e s_r, t] chi'(h_t)/sqrt|orb m_t| x[m_t]
template <typename U, bool kCV>
__global__ void __launch_bounds__(kMvThreads) matvec_general_kernel(MvArgs a) {
    __shared__ GroupSmem g;
    __shared__ U spl[kMaxSplit];
    load_group_smem(g, a.group);
    for (int i = threadIdx.x; i < a.nsplit; i += blockDim.x) spl[i] = ((const U*)a.split)[i];
    __syncthreads();
    const GroupDesc* G = a.group;
    const int L = g.L;
    const U lm = (U)g.lmask;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < a.n; r += (int64_t)gridDim.x * blockDim.x) {
        const U s = ((const U*)a.reps)[r];
        const int stab_r = a.stab[r];
        const double orb_r = (double)g.ng / (double)stab_r;
        double acc_r = 0, acc_i = 0;
        U base[2] = {s, brev_bits(s, L)};
        for (int p = 0; p < g.nperm; ++p) {
            U rot = g.general ? (U)gperm_apply(g.gtab, p, g.nbytes, (uint64_t)s)
                              : rotl_bits<U>(base[g.refl[p]], g.shift[p], L, lm);
            for (int e = g.begin[p]; e < g.begin[p + 1]; ++e) {
                const U tp = rot ^ (U)g.mask[e];
                double er = G->chi_re[e], ei = a.conj_chi ? -G->chi_im[e] : G->chi_im[e];
                for (int k = 0; k < a.nprog; ++k) {
                    U t;
                    double are, aim;
                    if (!run_prog<U, double>(a.progs[k], a.pauli, tp, t, are, aim)) continue;
                    if (a.conj_amp) aim = -aim;
                    U m;
                    int bi, st;
                    orbit_min<U>(g, t, m, bi, st);
                    int64_t idx = rank_search<U>((const U*)a.reps, a.n, spl, (int)a.nsplit, a.stride, m);
                    if (idx < 0) continue;
                    double hr = G->chi_re[bi], hi = a.conj_chi ? -G->chi_im[bi] : G->chi_im[bi];
                    double orb_m = (double)g.ng / (double)st;
                    double f = 1.0 / ((double)stab_r * sqrt(orb_r * orb_m));
                    // w = chi(g_e) * A * chi(h) * f
                    double t1r = er * are - ei * aim, t1i = er * aim + ei * are;
                    double wr = (t1r * hr - t1i * hi) * f, wi = (t1r * hi + t1i * hr) * f;
                    double xr, xi;
                    if (kCV) {
                        double2 v = ((const double2*)a.x)[idx];
                        xr = v.x;
                        xi = v.y;
                    } else {
                        xr = ((const double*)a.x)[idx];
                        xi = 0;
                    }
                    acc_r += wr * xr - wi * xi;
                    acc_i += wr * xi + wi * xr;
                }
            }
        }
        double2 d = ((const double2*)a.diag)[r];
        double dr = d.x, di = a.conj_amp ? -d.y : d.y;
        double xr, xi;
        if (kCV) {
            double2 v = ((const double2*)a.x)[r];
            xr = v.x;
            xi = v.y;
        } else {
            xr = ((const double*)a.x)[r];
            xi = 0;
        }
        acc_r += dr * xr - di * xi;
        acc_i += dr * xi + di * xr;
        if (kCV) {
            double2* y = (double2*)a.y;
            double yr = 0, yi = 0;
            if (!a.beta_zero) {
                double2 yo = y[r];
                yr = a.br * yo.x - a.bi * yo.y;
                yi = a.br * yo.y + a.bi * yo.x;
            }
            y[r] = make_double2(yr + a.ar * acc_r - a.ai * acc_i, yi + a.ar * acc_i + a.ai * acc_r);
        } else {
            double* y = (double*)a.y;
            double yr = a.beta_zero ? 0.0 : a.br * y[r];
            y[r] = yr + a.ar * acc_r;
        }
    }
}

// Diagonal of the structurally diagonal programs on each row's representative.
template <typename U>
__global__ void diag_kernel(MvArgs a, const double* user, double* out) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < a.n; r += (int64_t)gridDim.x * blockDim.x) {
        int mode = a.reps ? 2 : (a.nup >= 0 ? 1 : 0);
        U s = row_state<U>(a, mode, r);
        // extracted diagonal summed from zero in term order, then added to the
        // user diagonal (diagonal + extracted_diagonal, src/operators.jl:3103-3106)
        double dr = 0.0, di = 0.0;
        for (int k = 0; k < a.nprog; ++k) {
            U t;
            double are, aim;
            if (!run_prog<U, double>(a.progs[k], a.pauli, s, t, are, aim)) continue;
            dr += are;
            di += aim;
        }
        out[2 * r] = (user ? user[2 * r] : 0.0) + dr;
        out[2 * r + 1] = (user ? user[2 * r + 1] : 0.0) + di;
    }
}

__global__ void diag_df_kernel(const double* in, float4* out, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        DF a = df_from_double(in[2 * i]), b = df_from_double(in[2 * i + 1]);
        out[i] = make_float4(a.h, a.l, b.h, b.l);
    }
}

__global__ void real_part_kernel(const double* in, double* out, float* out32, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        out[i] = in[2 * i];
        out32[i] = (float)in[2 * i];
    }
}

__global__ void to_single_kernel(const double* in, float* out, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (float)in[i];
}

int mv_grid(int64_t n) {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int64_t blocks = (n + kMvThreads - 1) / kMvThreads;
    int64_t cap = (int64_t)sms * 8;
    return (int)std::max<int64_t>(1, std::min(blocks, cap));
}

MvArgs base_args(const Op& op) {
    const Basis& b = *op.basis;
    MvArgs a{};
    a.reps = b.symmetric ? b.d_reps.p : nullptr;
    a.stab = b.d_stab.as<uint16_t>();
    a.split = b.d_split.p;
    a.n = b.n;
    a.nsplit = b.nsplit;
    a.stride = b.split_stride;
    a.group = b.d_group.as<GroupDesc>();
    a.binom = b.d_binom.as<uint64_t>();
    a.L = b.L;
    a.nup = b.nup;
    a.pauli = b.spec.pauli;
    a.index = b.has_index ? b.d_index.as<int32_t>() : nullptr;
    a.fast = b.fast;
    a.fast_chi = b.fast.enabled ? b.d_fast_chi.as<double>() : nullptr;
    return a;
}

template <typename U, int kMode, typename T>
void launch_mode(const MvArgs& a, bool cm, bool cv, cudaStream_t s) {
    int grid = mv_grid(a.n);
    if (cm) matvec_kernel<U, kMode, true, true, T><<<grid, kMvThreads, 0, s>>>(a);
    else if (cv) matvec_kernel<U, kMode, false, true, T><<<grid, kMvThreads, 0, s>>>(a);
    else matvec_kernel<U, kMode, false, false, T><<<grid, kMvThreads, 0, s>>>(a);
}

// QS_RANK_MODE picks the rank lookup of a symmetric sector's generated states
// (read on every product): "direct" (the rank -> column table, when built),
// "search" (per-thread binary search behind shared-memory splitters) or
// "warp" (the warp-cooperative search); default: direct when built, else search.
int rank_mode_env() {
    const char* e = std::getenv("QS_RANK_MODE");
    if (!e || !e[0]) return -1;
    if (!std::strcmp(e, "direct")) return 3;
    if (!std::strcmp(e, "search")) return 2;
    if (!std::strcmp(e, "warp")) return 4;
    return -1;
}

template <typename T>
void launch_matvec(const Basis& b, const MvArgs& a, bool cm, bool cv, cudaStream_t s) {
    const int rm = b.symmetric ? rank_mode_env() : -1;
    if (rm == 4) {
        const int grid = mv_grid(a.n);
        if (b.wide) {
            if (cm) matvec_warp_rank_kernel<uint64_t, true, true, T><<<grid, kMvThreads, 0, s>>>(a);
            else if (cv) matvec_warp_rank_kernel<uint64_t, false, true, T><<<grid, kMvThreads, 0, s>>>(a);
            else matvec_warp_rank_kernel<uint64_t, false, false, T><<<grid, kMvThreads, 0, s>>>(a);
        } else {
            if (cm) matvec_warp_rank_kernel<uint32_t, true, true, T><<<grid, kMvThreads, 0, s>>>(a);
            else if (cv) matvec_warp_rank_kernel<uint32_t, false, true, T><<<grid, kMvThreads, 0, s>>>(a);
            else matvec_warp_rank_kernel<uint32_t, false, false, T><<<grid, kMvThreads, 0, s>>>(a);
        }
        return;
    }
    if (b.symmetric && rm == 2) {
        if (b.wide) launch_mode<uint64_t, 2, T>(a, cm, cv, s);
        else launch_mode<uint32_t, 2, T>(a, cm, cv, s);
        return;
    }
    if (b.symmetric && b.has_index) {
        if (b.wide) launch_mode<uint64_t, 3, T>(a, cm, cv, s);
        else launch_mode<uint32_t, 3, T>(a, cm, cv, s);
    } else if (b.symmetric) {
        if (b.wide) launch_mode<uint64_t, 2, T>(a, cm, cv, s);
        else launch_mode<uint32_t, 2, T>(a, cm, cv, s);
    } else if (b.nup >= 0) {
        // up to 32 sites: 32-bit states, the binomial table in shared memory
        // and ranks updated from the row's own rank
        if (b.wide) launch_mode<uint64_t, 1, T>(a, cm, cv, s);
        else launch_mode<uint32_t, 1, T>(a, cm, cv, s);
    } else {
        launch_mode<uint64_t, 0, T>(a, cm, cv, s);
    }
}

}  // namespace

namespace {
std::atomic<int64_t> g_launches{0};
std::atomic<int64_t> g_device_allocs{0};
}
void note_launches(int64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
int64_t launches() { return g_launches.load(std::memory_order_relaxed); }
void note_device_alloc() { g_device_allocs.fetch_add(1, std::memory_order_relaxed); }
int64_t device_allocs() { return g_device_allocs.load(std::memory_order_relaxed); }

Op::~Op() {
    if (copy_stream) {
        cudaStreamSynchronize(copy_stream);
        cudaStreamDestroy(copy_stream);
        for (cudaEvent_t e : range_done)
            if (e) cudaEventDestroy(e);
    }
    if (own_stream) cudaStreamDestroy(own_stream);
}

void op_prepare_device(Op& op) {
    Basis& b = *op.basis;
    if (!op.own_stream) {
        QS_CUDA(cudaStreamCreateWithFlags(&op.own_stream, cudaStreamNonBlocking));
        op.stream = op.own_stream;
    }
    size_t np = std::max<size_t>(1, op.progs.size());
    op.d_progs.alloc(np * sizeof(TermProg));
    if (!op.progs.empty())
        QS_CUDA(cudaMemcpy(op.d_progs.p, op.progs.data(), op.progs.size() * sizeof(TermProg), cudaMemcpyHostToDevice));
    // diagonal: user diagonal plus, when extracted, the diagonal programs
    DevBuf user(2 * b.n * sizeof(double));
    if (!op.user_diag.empty())
        QS_CUDA(cudaMemcpy(user.p, op.user_diag.data(), 2 * b.n * sizeof(double), cudaMemcpyHostToDevice));
    else
        QS_CUDA(cudaMemset(user.p, 0, 2 * b.n * sizeof(double)));
    op.d_diag.alloc(2 * b.n * sizeof(double));
    DevBuf dprogs(std::max<size_t>(1, op.diag_progs.size()) * sizeof(TermProg));
    if (!op.diag_progs.empty())
        QS_CUDA(cudaMemcpy(dprogs.p, op.diag_progs.data(), op.diag_progs.size() * sizeof(TermProg),
                           cudaMemcpyHostToDevice));
    MvArgs a = base_args(op);
    a.progs = dprogs.as<TermProg>();
    a.nprog = (int)op.diag_progs.size();
    if (b.symmetric && !b.wide)
        diag_kernel<uint32_t><<<mv_grid(b.n), kMvThreads, 0, op.stream>>>(a, user.as<double>(), op.d_diag.as<double>());
    else
        diag_kernel<uint64_t><<<mv_grid(b.n), kMvThreads, 0, op.stream>>>(a, user.as<double>(), op.d_diag.as<double>());
    QS_CUDA(cudaGetLastError());
    op.d_diag32.alloc(2 * b.n * sizeof(float));
    to_single_kernel<<<mv_grid(2 * b.n), kMvThreads, 0, op.stream>>>(op.d_diag.as<double>(), op.d_diag32.as<float>(),
                                                                      2 * b.n);
    QS_CUDA(cudaGetLastError());
    op.d_diag_df.alloc(b.n * 4 * sizeof(float));
    diag_df_kernel<<<mv_grid(b.n), kMvThreads, 0, op.stream>>>(op.d_diag.as<double>(), op.d_diag_df.as<float4>(), b.n);
    QS_CUDA(cudaGetLastError());
    op.d_diag_re.alloc(b.n * sizeof(double));
    op.d_diag32_re.alloc(b.n * sizeof(float));
    real_part_kernel<<<mv_grid(b.n), kMvThreads, 0, op.stream>>>(op.d_diag.as<double>(), op.d_diag_re.as<double>(),
                                                                  op.d_diag32_re.as<float>(), b.n);
    QS_CUDA(cudaGetLastError());
    QS_CUDA(cudaStreamSynchronize(op.stream));
}

void op_matvec_device(Op& op, const MatvecCall& c, cudaStream_t s) {
    if (op.dense) {
        op_matvec_dense(op, c, s);
        return;
    }
    const Basis& b = *op.basis;
    MvArgs a = base_args(op);
    a.progs = op.d_progs.as<TermProg>();
    a.nprog = (int)op.progs.size();
    const bool T = (c.flags & QS_TRANSPOSE) != 0, C = (c.flags & QS_CONJUGATE) != 0;
    a.conj_amp = C;
    a.conj_chi = T != C;
    a.ar = c.alpha.re;
    a.ai = c.alpha.im;
    a.br = c.beta.re;
    a.bi = c.beta.im;
    a.beta_zero = (c.beta.re == 0.0 && c.beta.im == 0.0);
    a.x = c.x;
    a.y = c.y;
    // the pull form of op(A) runs the chain of op(A)^T; a transposed call runs
    // A's own chain (programs are stored for both)
    if (T) a.progs = op.d_progs.as<TermProg>() + op.progs.size() / 2;
    a.nprog = (int)op.progs.size() / 2;
    const bool cm = op.complex_mat;
    const bool cv = c.y_complex;
    if (c.x_complex && !c.y_complex) throw Error(QS_ERR_ARGUMENT, "a complex input needs a complex output");
    if (cm && !cv) throw Error(QS_ERR_ARGUMENT, "a complex operator needs a complex output");
    if (!cv && c.x_complex) throw Error(QS_ERR_ARGUMENT, "a complex input needs a complex output");
    if (c.x_complex != cv) throw Error(QS_ERR_UNSUPPORTED, "input and output must share a dtype at the device boundary");
    if (!op.commuting) {
        if (c.single) throw Error(QS_ERR_UNSUPPORTED, "the single-precision form needs a symmetry-commuting operator");
        a.diag = op.d_diag.p;
        int grid = mv_grid(b.n);
        if (b.wide) {
            if (cv) matvec_general_kernel<uint64_t, true><<<grid, kMvThreads, 0, s>>>(a);
            else matvec_general_kernel<uint64_t, false><<<grid, kMvThreads, 0, s>>>(a);
        } else {
            if (cv) matvec_general_kernel<uint32_t, true><<<grid, kMvThreads, 0, s>>>(a);
            else matvec_general_kernel<uint32_t, false><<<grid, kMvThreads, 0, s>>>(a);
        }
        QS_CUDA(cudaGetLastError());
        note_launches(1);
        return;
    }
    if (op.assembled && (!T || op.hermitian)) {
        op_spmv_device(op, c, s);
        return;
    }
    if (c.df_io) throw Error(QS_ERR_UNSUPPORTED, "double-float vectors need an assembled operator");
    if (c.single) {
        a.diag = op.d_diag32.p;
        launch_matvec<float>(b, a, cm, cv, s);
    } else {
        a.diag = op.d_diag.p;
        launch_matvec<double>(b, a, cm, cv, s);
    }
    QS_CUDA(cudaGetLastError());
    note_launches(1);
}

}  // namespace qs
