// qs_engine.cu -- kernels and host side of the batched Krylov engine
// (qs_engine.h), and the batched eigsh built on it.
//
// The reference solves symmetry sectors one at a time (block_diag_hamiltonian
// / BlockOps, tools.jl:2213-2420, each an ARPACK run through eigsh,
// src/operators.jl:1558-1640).  Here every sector is a slot and one launch of
// each step kernel serves all of them.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <random>
#include <tuple>
#include <type_traits>

#include "qs_blas.cuh"
#include "qs_tc.cuh"
#include "qs_dense.h"
#include "qs_df.cuh"
#include "qs_engine.h"
#include "qs_krylov.h"

namespace qs {

namespace {

constexpr int kT = 256;       // threads per block
// vectors per dots block (eight measured slower than four for FP64 on GB300:
// the dots are FP64-pipe bound, and the larger tile needs twice the
// registers)
template <class A>
__host__ __device__ constexpr int jt() { return 4; }
constexpr int kMaxM = 256;    // largest Krylov basis of a slot

// ------------------------------------------------------------ arithmetic
// The same kernel source runs on FP64 values (A = double) and on
// double-float values (A = DF); a complex value is a pair of A.
template <class A>
struct CA {
    A re, im;
};

__device__ __forceinline__ void mac(double& acc, double a, double b) { acc = fma(a, b, acc); }
__device__ __forceinline__ void mac(DF& acc, DF a, DF b) { df_mac(acc, a.h, a.l, b.h, b.l); }
__device__ __forceinline__ void msub(double& acc, double a, double b) { acc = fma(-a, b, acc); }
__device__ __forceinline__ void msub(DF& acc, DF a, DF b) { df_mac(acc, -a.h, -a.l, b.h, b.l); }
__device__ __forceinline__ double sub(double a, double b) { return a - b; }
__device__ __forceinline__ DF sub(DF a, DF b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ double add(double a, double b) { return a + b; }
__device__ __forceinline__ DF add(DF a, DF b) { return df_add(a, b); }
__device__ __forceinline__ double mul(double a, double b) { return a * b; }
__device__ __forceinline__ DF mul(DF a, DF b) { return df_mul(a, b); }
__device__ __forceinline__ double to_d(double a) { return a; }
__device__ __forceinline__ double to_d(DF a) { return df_to_double(a); }
__device__ __forceinline__ double shfl(double v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ DF shfl(DF v, int o) { return df_shfl_xor(v, o, 32); }
// FP32 storage and arithmetic (the FP32 form)
__device__ __forceinline__ void mac(float& acc, float a, float b) { acc = fmaf(a, b, acc); }
__device__ __forceinline__ void msub(float& acc, float a, float b) { acc = fmaf(-a, b, acc); }
__device__ __forceinline__ float sub(float a, float b) { return a - b; }
__device__ __forceinline__ float add(float a, float b) { return a + b; }
__device__ __forceinline__ float mul(float a, float b) { return a * b; }
__device__ __forceinline__ double to_d(float a) { return (double)a; }
__device__ __forceinline__ float shfl(float v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }

template <class A> __device__ __forceinline__ A zero();
template <> __device__ __forceinline__ double zero<double>() { return 0.0; }
template <> __device__ __forceinline__ DF zero<DF>() { return DF{0.f, 0.f}; }
template <> __device__ __forceinline__ float zero<float>() { return 0.f; }
template <class A> __device__ __forceinline__ A one();
template <> __device__ __forceinline__ double one<double>() { return 1.0; }
template <> __device__ __forceinline__ DF one<DF>() { return DF{1.f, 0.f}; }
template <> __device__ __forceinline__ float one<float>() { return 1.f; }
template <class A> __device__ __forceinline__ A from_d(double v);
template <> __device__ __forceinline__ double from_d<double>(double v) { return v; }
template <> __device__ __forceinline__ DF from_d<DF>(double v) { return df_from_double(v); }
template <> __device__ __forceinline__ float from_d<float>(double v) { return (float)v; }

// vector element i; 8 bytes per real component in both storages
template <class A, bool CV> __device__ __forceinline__ CA<A> ldv(const void* p, int64_t i);
template <> __device__ __forceinline__ CA<double> ldv<double, false>(const void* p, int64_t i) {
    return CA<double>{((const double*)p)[i], 0.0};
}
template <> __device__ __forceinline__ CA<double> ldv<double, true>(const void* p, int64_t i) {
    const double2 v = ((const double2*)p)[i];
    return CA<double>{v.x, v.y};
}
template <> __device__ __forceinline__ CA<DF> ldv<DF, false>(const void* p, int64_t i) {
    const float2 v = ((const float2*)p)[i];
    return CA<DF>{DF{v.x, v.y}, DF{0.f, 0.f}};
}
template <> __device__ __forceinline__ CA<DF> ldv<DF, true>(const void* p, int64_t i) {
    const float4 v = ((const float4*)p)[i];
    return CA<DF>{DF{v.x, v.y}, DF{v.z, v.w}};
}
template <> __device__ __forceinline__ CA<float> ldv<float, false>(const void* p, int64_t i) {
    return CA<float>{((const float*)p)[i], 0.f};
}
template <> __device__ __forceinline__ CA<float> ldv<float, true>(const void* p, int64_t i) {
    const float2 v = ((const float2*)p)[i];
    return CA<float>{v.x, v.y};
}
template <class A, bool CV> __device__ __forceinline__ void stv(void* p, int64_t i, CA<A> v);
template <> __device__ __forceinline__ void stv<float, false>(void* p, int64_t i, CA<float> v) {
    ((float*)p)[i] = v.re;
}
template <> __device__ __forceinline__ void stv<float, true>(void* p, int64_t i, CA<float> v) {
    ((float2*)p)[i] = make_float2(v.re, v.im);
}
template <> __device__ __forceinline__ void stv<double, false>(void* p, int64_t i, CA<double> v) {
    ((double*)p)[i] = v.re;
}
template <> __device__ __forceinline__ void stv<double, true>(void* p, int64_t i, CA<double> v) {
    ((double2*)p)[i] = make_double2(v.re, v.im);
}
template <> __device__ __forceinline__ void stv<DF, false>(void* p, int64_t i, CA<DF> v) {
    ((float2*)p)[i] = make_float2(v.re.h, v.re.l);
}
template <> __device__ __forceinline__ void stv<DF, true>(void* p, int64_t i, CA<DF> v) {
    ((float4*)p)[i] = make_float4(v.re.h, v.re.l, v.im.h, v.im.l);
}

// matrix value of a code and diagonal of a row
template <class A> __device__ __forceinline__ CA<A> ldtab(const SlotDev& S, int c);
template <> __device__ __forceinline__ CA<double> ldtab<double>(const SlotDev& S, int c) {
    const double2 v = __ldg(S.tab64 + c);
    return CA<double>{v.x, v.y};
}
template <> __device__ __forceinline__ CA<DF> ldtab<DF>(const SlotDev& S, int c) {
    const float4 v = __ldg(S.tabdf + c);
    return CA<DF>{DF{v.x, v.y}, DF{v.z, v.w}};
}
template <> __device__ __forceinline__ CA<float> ldtab<float>(const SlotDev& S, int c) {
    const float2 v = __ldg(S.tab32 + c);
    return CA<float>{v.x, v.y};
}
template <class A> __device__ __forceinline__ CA<A> lddiag(const SlotDev& S, int64_t r);
template <> __device__ __forceinline__ CA<double> lddiag<double>(const SlotDev& S, int64_t r) {
    const double2 v = S.diag64[r];
    return CA<double>{v.x, v.y};
}
template <> __device__ __forceinline__ CA<DF> lddiag<DF>(const SlotDev& S, int64_t r) {
    const float4 v = S.diagdf[r];
    return CA<DF>{DF{v.x, v.y}, DF{v.z, v.w}};
}
template <> __device__ __forceinline__ CA<float> lddiag<float>(const SlotDev& S, int64_t r) {
    const float2 v = S.diag32[r];
    return CA<float>{v.x, v.y};
}
template <class A> __device__ __forceinline__ A ldrsq(const void* t, int i);
template <> __device__ __forceinline__ double ldrsq<double>(const void* t, int i) { return ((const double*)t)[i]; }
template <> __device__ __forceinline__ DF ldrsq<DF>(const void* t, int i) {
    const float2 v = ((const float2*)t)[i];
    return DF{v.x, v.y};
}
template <> __device__ __forceinline__ float ldrsq<float>(const void* t, int i) { return ((const float*)t)[i]; }

// bytes of one vector element: 8 per real component in FP64 and double-float,
// 4 in FP32
template <class A, bool CV> __host__ __device__ constexpr size_t vbytes() { return sizeof(A) * (CV ? 2 : 1); }
template <class A> __device__ __forceinline__ char* colp(const SlotDev& S, int c) {
    return (char*)S.V + (size_t)c * S.n * (S.cv ? vbytes<A, true>() : vbytes<A, false>());
}

// ------------------------------------------------------------ SpMV
// y = col(j + 1) = H col(j) on every stepping slot: sliced ELL, one thread per
// row, the slot's value table staged in shared memory.
template <class A, bool CV, bool CM, bool PACKED>
__device__ __forceinline__ void spmv_rows(const SlotDev& S, int64_t s0, int64_t s1, const CA<A>* tab, bool smem_tab,
                                          const A* rsq) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const int64_t n = S.n;
    const void* x = colp<A>(S, S.j);
    void* y = colp<A>(S, S.j + 1);
    const int cb = S.code_bits;
    const uint32_t cmask = S.code_mask;
    const uint16_t* __restrict__ len = S.len;
    const uint16_t* __restrict__ stab = S.stab;
    for (int64_t sl = s0 + warp; sl < s1; sl += nw) {
        const int64_t r = sl * kSellSlice + lane;
        if (r >= n) continue;
        const int cnt = len[r];
        const int64_t base = S.sptr[sl] + lane;
        A ar = zero<A>(), ai = zero<A>();
        sell_row<4, PACKED, false>(S.words, S.cols, S.codes, base, cnt, cb, cmask,
                            [&](uint32_t c) { return ldv<A, CV>(x, c); },
                            [&](uint32_t code, CA<A> xv) {
                                const CA<A> v = smem_tab ? tab[code] : ldtab<A>(S, code);
                                mac(ar, v.re, xv.re);
                                if (CV) {
                                    mac(ai, v.re, xv.im);
                                    if (CM) {
                                        msub(ar, v.im, xv.im);
                                        mac(ai, v.im, xv.re);
                                    }
                                }
                            });
        const A sc = stab ? rsq[stab[r]] : one<A>();
        CA<A> out;
        out.re = mul(ar, sc);
        out.im = CV ? mul(ai, sc) : zero<A>();
        const CA<A> d = lddiag<A>(S, r);
        const CA<A> xr = ldv<A, CV>(x, r);
        mac(out.re, d.re, xr.re);
        if (CV) {
            msub(out.re, d.im, xr.im);
            mac(out.im, d.re, xr.im);
            mac(out.im, d.im, xr.re);
        }
        stv<A, CV>(y, r, out);
    }
}

// the slot's slices [s0, s1) of y = col(j + 1) = H col(j)
template <class A>
__device__ __forceinline__ void spmv_slices(const SlotDev& S, int64_t s0, int64_t s1, const CA<A>* tab, bool smem_tab,
                                            const A* rsq) {
    if (S.packed) {
        if (!S.cv) spmv_rows<A, false, false, true>(S, s0, s1, tab, smem_tab, rsq);
        else if (!S.cm) spmv_rows<A, true, false, true>(S, s0, s1, tab, smem_tab, rsq);
        else spmv_rows<A, true, true, true>(S, s0, s1, tab, smem_tab, rsq);
    } else {
        if (!S.cv) spmv_rows<A, false, false, false>(S, s0, s1, tab, smem_tab, rsq);
        else if (!S.cm) spmv_rows<A, true, false, false>(S, s0, s1, tab, smem_tab, rsq);
        else spmv_rows<A, true, true, false>(S, s0, s1, tab, smem_tab, rsq);
    }
}

template <class A>
__device__ __forceinline__ void spmv_block(const SlotDev* sl, const int* __restrict__ smap,
                                           const void* __restrict__ rsqt, int bx) {
    __shared__ CA<A> tab[1024];
    __shared__ A rsq[kMaxGroup + 1];
    const SlotDev& S = sl[smap[bx]];
    if (S.state != kSlotStep) return;
    const bool smem_tab = S.ncodes <= 1024;
    if (smem_tab)
        for (int i = threadIdx.x; i < S.ncodes; i += blockDim.x) tab[i] = ldtab<A>(S, i);
    if (S.stab)
        for (int i = threadIdx.x; i <= S.max_stab; i += blockDim.x) rsq[i] = ldrsq<A>(rsqt, i);
    __syncthreads();
    const int64_t lb = bx - S.sb_begin;
    spmv_slices<A>(S, lb * S.spb, min(S.nslices, lb * S.spb + S.spb), tab, smem_tab, rsq);
}

template <class A>
__global__ void __launch_bounds__(kT) eng_spmv(const SlotDev* __restrict__ sl, const int* __restrict__ smap,
                                               const void* __restrict__ rsqt) {
    spmv_block<A>(sl, smap, rsqt, blockIdx.x);
}

// ------------------------------------------------------------ dots
// Partial sums per row block b live at partial[(b * P + i) * 2 + {re, im}],
// P = mmax + 1; index mmax holds norms.
// mode 0 (first pass): i in [first, j] with first = j for the three-term
//   recurrence, else 0; DGKS slots also accumulate ||w||^2 at index mmax;
// mode 1 (second pass, only where the step's flag asks): i in [0, j] (the step
//   itself takes these dots from the first update, see eng_update);
// mode 2 (normalise): partial[b][0] = <col ncol, col ncol>.
template <class A, bool CV>
__device__ __forceinline__ void dots_rows(const SlotDev& S, int64_t r0, int64_t r1, int i0, int nv, const void* w,
                                          A* re, A* im, bool want_wn, A& wn) {
    const int64_t n = S.n;
    const char* V = (const char*)S.V;
    const size_t cs = (size_t)n * vbytes<A, CV>();
    const int64_t step = blockDim.x;
    if (nv - i0 == 1) {
        // one vector (a three-term step, a normalisation, the first CGS step):
        // four rows' loads of w and the column in flight, nothing else read
        const void* c0 = V + (size_t)i0 * cs;
        auto acc = [&](const CA<A>& wv, const CA<A>& v) {
            mac(re[0], v.re, wv.re);
            if (CV) {
                mac(re[0], v.im, wv.im);
                mac(im[0], v.re, wv.im);
                msub(im[0], v.im, wv.re);
            }
            if (want_wn) {
                mac(wn, wv.re, wv.re);
                if (CV) mac(wn, wv.im, wv.im);
            }
        };
        int64_t r = r0 + threadIdx.x;
        for (; r + 3 * step < r1; r += 4 * step) {
            CA<A> wv[4], v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                wv[u] = ldv<A, CV>(w, r + u * step);
                v[u] = ldv<A, CV>(c0, r + u * step);
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) acc(wv[u], v[u]);
        }
        for (; r < r1; r += step) acc(ldv<A, CV>(w, r), ldv<A, CV>(c0, r));
        return;
    }
    // columns past nv repeat the last one (cached) so that every load of a row
    // is issued before the arithmetic
    const char* col[jt<A>()];
#pragma unroll
    for (int q = 0; q < jt<A>(); ++q) col[q] = V + (size_t)min(i0 + q, nv - 1) * cs;
    auto row = [&](const CA<A>& wv, const CA<A>* v) {
#pragma unroll
        for (int q = 0; q < jt<A>(); ++q) {
            if (i0 + q < nv) {
                mac(re[q], v[q].re, wv.re);
                if (CV) {
                    mac(re[q], v[q].im, wv.im);
                    mac(im[q], v[q].re, wv.im);
                    msub(im[q], v[q].im, wv.re);
                }
            }
        }
        if (want_wn) {
            mac(wn, wv.re, wv.re);
            if (CV) mac(wn, wv.im, wv.im);
        }
    };
    // real vectors: two rows per iteration, 2 (jt<A>() + 1) loads issued before the
    // arithmetic; complex vectors hold twice the data per row, one row at a time
    int64_t r = r0 + threadIdx.x;
    for (; !CV && r + step < r1; r += 2 * step) {
        const CA<A> w0 = ldv<A, CV>(w, r), w1 = ldv<A, CV>(w, r + step);
        CA<A> v0[jt<A>()], v1[jt<A>()];
#pragma unroll
        for (int q = 0; q < jt<A>(); ++q) {
            v0[q] = ldv<A, CV>(col[q], r);
            v1[q] = ldv<A, CV>(col[q], r + step);
        }
        row(w0, v0);
        row(w1, v1);
    }
    for (; r < r1; r += step) {
        const CA<A> w0 = ldv<A, CV>(w, r);
        CA<A> v0[jt<A>()];
#pragma unroll
        for (int q = 0; q < jt<A>(); ++q) v0[q] = ldv<A, CV>(col[q], r);
        row(w0, v0);
    }
}

template <class A>
__device__ __forceinline__ double block_sum(A v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v = add(v, shfl(v, o));
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[wid] = to_d(v);
    __syncthreads();
    double t = 0;
    for (int q = 0; q < kT / 32; ++q) t += sh[q];
    return t;
}

// Block sums of the jt<A>() accumulators into row[(base + q) * 2 + {re, im}] for
// the vectors i0 + q < nv (row: the block's slice of the partial buffer).
template <class A>
__device__ __forceinline__ void dots_epilogue(A* re, A* im, bool cv, int i0, int nv, int base, double* row) {
    __shared__ double sh[kT / 32][2 * jt<A>()];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < jt<A>(); ++q) {
        for (int o = 16; o > 0; o >>= 1) {
            re[q] = add(re[q], shfl(re[q], o));
            if (cv) im[q] = add(im[q], shfl(im[q], o));
        }
        if (lane == 0) {
            sh[wid][2 * q] = to_d(re[q]);
            sh[wid][2 * q + 1] = cv ? to_d(im[q]) : 0.0;
        }
    }
    __syncthreads();
    if (threadIdx.x < 2 * jt<A>()) {
        double t = 0;
        for (int q = 0; q < kT / 32; ++q) t += sh[q][threadIdx.x];
        const int q = threadIdx.x / 2;
        if (i0 + q < nv) row[(base + q) * 2 + (threadIdx.x & 1)] = t;
    }
    __syncthreads();   // sh is reused by the next call
}

template <class A>
__device__ __forceinline__ void dots_block(const SlotDev* sl, const int* __restrict__ rmap, int mmax, int mode,
                                           double* partial, int bx, int by) {
    const SlotDev& S = sl[rmap[bx]];
    if (S.state != (mode == 2 ? kSlotNormalize : kSlotStep)) return;
    if (mode == 1 && S.nrm[4] == 0.0) return;
    const int P = mmax + 1;
    int first, nv;
    const void* w;
    if (mode == 2) {
        first = S.ncol;
        nv = S.ncol + 1;
        w = colp<A>(S, S.ncol);
    } else {
        first = (mode == 0 && S.orth == 2) ? S.j : 0;
        nv = S.j + 1;
        w = colp<A>(S, S.j + 1);
    }
    const int i0 = first + by * jt<A>();
    if (i0 >= nv) return;
    const bool want_wn = mode == 0 && S.orth == 1 && by == 0;
    const int64_t lb = bx - S.rb_begin;
    const int64_t r0 = lb * S.rpb, r1 = min(S.n, r0 + S.rpb);
    A re[jt<A>()], im[jt<A>()], wn = zero<A>();
#pragma unroll
    for (int q = 0; q < jt<A>(); ++q) re[q] = im[q] = zero<A>();
    if (S.cv) dots_rows<A, true>(S, r0, r1, i0, nv, w, re, im, want_wn, wn);
    else dots_rows<A, false>(S, r0, r1, i0, nv, w, re, im, want_wn, wn);
    dots_epilogue<A>(re, im, S.cv, i0, nv, mode == 2 ? 0 : i0, partial + (size_t)bx * P * 2);
    if (want_wn) {
        __shared__ double sw[kT / 32];
        const double t = block_sum(wn, sw);
        if (threadIdx.x == 0) {
            partial[((size_t)bx * P + mmax) * 2] = t;
            partial[((size_t)bx * P + mmax) * 2 + 1] = 0.0;
        }
    }
}

template <class A>
__global__ void __launch_bounds__(kT, std::is_same<A, DF>::value ? 4 : 3) eng_dots(const SlotDev* __restrict__ sl, const int* __restrict__ rmap, int mmax,
                                               int mode, double* __restrict__ partial) {
    dots_block<A>(sl, rmap, mmax, mode, partial, blockIdx.x, blockIdx.y);
}

// First-pass dots of a real Gram-Schmidt slot with 2 <= nv <= 20 vectors in
// one block per row block: each row's w and nv vector entries are loaded once
// (all loads before the arithmetic) and every column's sum advances, where
// eng_dots reads w once per tile of jt columns.  Per thread the rows and the
// multiply-add order of each column's sum and of ||w||^2 are those of
// dots_rows, and the block sums go through dots_epilogue / block_sum, so the
// partials are bit-identical to dots_block's.
template <class A, int NV>
__device__ __forceinline__ void dots_fused_rows(const SlotDev& S, int64_t r0, int64_t r1, int nv, const void* w,
                                                bool want_wn, int mmax, double* partial, int bx) {
    const char* V = (const char*)S.V;
    const size_t cs = (size_t)S.n * vbytes<A, false>();
    A acc[NV];
#pragma unroll
    for (int t = 0; t < NV; ++t) acc[t] = zero<A>();
    A wn = zero<A>();
    for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        A v[NV];
#pragma unroll
        for (int t = 0; t < NV; ++t)
            if (t < nv) v[t] = ldv<A, false>(V + (size_t)t * cs, r).re;
        const A wr = ldv<A, false>(w, r).re;
#pragma unroll
        for (int t = 0; t < NV; ++t)
            if (t < nv) mac(acc[t], v[t], wr);
        if (want_wn) mac(wn, wr, wr);
    }
    const int P = mmax + 1;
    double* row = partial + (size_t)bx * P * 2;
#pragma unroll
    for (int c0 = 0; c0 < NV; c0 += jt<A>()) {
        if (c0 < nv) {
            A re[jt<A>()], im[jt<A>()];
#pragma unroll
            for (int q = 0; q < jt<A>(); ++q) {
                re[q] = c0 + q < NV ? acc[c0 + q < NV ? c0 + q : 0] : zero<A>();
                im[q] = zero<A>();
            }
            dots_epilogue<A>(re, im, false, c0, nv, c0, row);
        }
    }
    if (want_wn) {
        __shared__ double sw[kT / 32];
        const double t = block_sum(wn, sw);
        if (threadIdx.x == 0) {
            partial[((size_t)bx * P + mmax) * 2] = t;
            partial[((size_t)bx * P + mmax) * 2 + 1] = 0.0;
        }
    }
}

template <class A>
__global__ void __launch_bounds__(kT, 2) eng_dots_fused(const SlotDev* __restrict__ sl, const int* __restrict__ rmap,
                                                        int mmax, double* __restrict__ partial) {
    const int bx = blockIdx.x, by = blockIdx.y;
    const SlotDev& S = sl[rmap[bx]];
    if (S.state != kSlotStep) return;
    const int nv = S.j + 1;
    if (S.cv || S.orth == 2 || nv < 2 || nv > 20) {
        dots_block<A>(sl, rmap, mmax, 0, partial, bx, by);
        return;
    }
    if (by) return;
    const int64_t lb = bx - S.rb_begin;
    const int64_t r0 = lb * S.rpb, r1 = min(S.n, r0 + S.rpb);
    const void* w = colp<A>(S, S.j + 1);
    const bool want_wn = S.orth == 1;
    if (nv <= 12) dots_fused_rows<A, 12>(S, r0, r1, nv, w, want_wn, mmax, partial, bx);
    else dots_fused_rows<A, 20>(S, r0, r1, nv, w, want_wn, mmax, partial, bx);
}

// ------------------------------------------------------------ reduce
// Per slot and vector, the block partials summed in a fixed order, then:
// mode 0: h1 (and ||w||^2; the three-term recurrence takes beta_{j-1} from the record)
// mode 1: ||w'||^2 after the first pass; decides the second pass; without it the
//         step's record column and norm are final
// mode 2: h2 and the record column h1 + h2 (second pass only)
// mode 3: ||w''||^2 (second pass only)
// mode 4: norm of the normalised column
__device__ __forceinline__ void reduce_block(const SlotDev* sl, int mmax, int mode, const double* partial, int dy,
                                             int bx, int by) {
    const SlotDev& S = sl[bx];
    int i = by;
    if (mode == 4) {
        if (S.state != kSlotNormalize || i) return;
    } else {
        if (S.state != kSlotStep) return;
        if ((mode == 2 || mode == 3) && S.nrm[4] == 0.0) return;
        if (mode == 0) {
            // blocks y < dy cover the step's vectors from `first`; y = dy the
            // DGKS norm (kept at partial index mmax)
            const int first = S.orth == 2 ? S.j : 0;
            if (i == dy) {
                if (S.orth != 1) return;
                i = mmax;
            } else {
                i += first;
                if (i > S.j) return;
            }
        } else if (mode == 1 || mode == 3) {
            if (i) return;
            i = mmax;
        } else if (i > S.j) {
            return;
        }
    }
    const int P = mmax + 1;
    double re = 0, im = 0;
    for (int b = threadIdx.x; b < S.rb_count; b += blockDim.x) {
        re += partial[((size_t)(S.rb_begin + b) * P + i) * 2];
        im += partial[((size_t)(S.rb_begin + b) * P + i) * 2 + 1];
    }
    for (int o = 16; o > 0; o >>= 1) {
        re += __shfl_xor_sync(0xffffffffu, re, o);
        im += __shfl_xor_sync(0xffffffffu, im, o);
    }
    __shared__ double sr[kT / 32], si[kT / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        sr[wid] = re;
        si[wid] = im;
    }
    __syncthreads();
    if (threadIdx.x) return;
    re = im = 0;
    for (int q = 0; q < kT / 32; ++q) {
        re += sr[q];
        im += si[q];
    }
    const int ld = S.m + 1;
    const int j = S.j;
    double2* col = S.rec + (size_t)j * ld;
    if (mode == 0) {
        if (i == mmax) {
            S.nrm[3] = re;
        } else {
            S.h1[i] = make_double2(re, im);
            if (S.orth == 2) S.h1[j - 1 >= 0 ? j - 1 : 0] = j > 0 ? S.rec[(size_t)(j - 1) * ld + j] : S.h1[0];
        }
    } else if (mode == 1) {
        const double nb = sqrt(fmax(re, 0.0));
        const bool second = S.orth == 0 || (S.orth == 1 && nb < 0.717 * sqrt(fmax(S.nrm[3], 0.0)));
        S.nrm[4] = second ? 1.0 : 0.0;
        if (!second) {
            // the first pass is final: record column j and the new norm
            const int first = S.orth == 2 ? (j > 0 ? j - 1 : 0) : 0;
            for (int q = first; q <= j; ++q) col[q] = S.h1[q];
            col[j + 1] = make_double2(nb, 0.0);
            S.nrm[0] = re;
            S.nrm[1] = nb > 0 ? 1.0 / nb : 0.0;
        }
    } else if (mode == 2) {
        S.h2[i] = make_double2(re, im);
        const double2 a = S.h1[i];
        col[i] = make_double2(a.x + re, a.y + im);
    } else {
        const double nb = sqrt(fmax(re, 0.0));
        S.nrm[0] = re;
        S.nrm[1] = nb > 0 ? 1.0 / nb : 0.0;
        if (mode == 3) col[j + 1] = make_double2(nb, 0.0);
        else S.nrm[2] = nb;
    }
}

__global__ void __launch_bounds__(kT) eng_reduce(const SlotDev* __restrict__ sl, int mmax, int mode,
                                                 const double* __restrict__ partial, int dy = 0) {
    reduce_block(sl, mmax, mode, partial, dy, blockIdx.x, blockIdx.y);
}

// ------------------------------------------------------------ update
// col(j+1) -= sum_i col(i) h_i over the pass's vectors (pass 0: h1 from
// `first`, pass 1: h2 over 0..j, only where the step's flag asks), leaving the
// block's part of ||col(j+1)||^2 at partial[b][mmax]; pass 0 of a Gram-Schmidt
// slot also leaves the second-pass dots at partial[b][0..j].
template <class A, bool CV>
__device__ __forceinline__ A update_rows(const SlotDev& S, int64_t r0, int64_t r1, int first, int nv, const CA<A>* hs) {
    const char* V = (const char*)S.V;
    const size_t cs = (size_t)S.n * vbytes<A, CV>();
    void* w = (void*)(V + (size_t)(S.j + 1) * cs);
    A nacc = zero<A>();
    auto term = [&](A& ar, A& ai, const CA<A>& v, const CA<A>& h) {
        mac(ar, v.re, h.re);
        if (CV) {
            msub(ar, v.im, h.im);
            mac(ai, v.re, h.im);
            mac(ai, v.im, h.re);
        }
    };
    if (nv - first <= 2) {
        // the three-term update (or a first step): two rows per iteration, all
        // their loads issued before either row's store
        const int two = nv - first == 2;
        const char* va = V + (size_t)first * cs;
        const char* vb = V + (size_t)(first + two) * cs;
        const CA<A> ha = hs[first], hb = two ? hs[first + 1] : CA<A>{zero<A>(), zero<A>()};
        auto one = [&](CA<A> o, const CA<A>& a, const CA<A>& b) {
            A ar = zero<A>(), ai = zero<A>();
            term(ar, ai, a, ha);
            if (two) term(ar, ai, b, hb);
            o.re = sub(o.re, ar);
            if (CV) o.im = sub(o.im, ai);
            mac(nacc, o.re, o.re);
            if (CV) mac(nacc, o.im, o.im);
            return o;
        };
        const int64_t step = blockDim.x;
        int64_t r = r0 + threadIdx.x;
        for (; r + step < r1; r += 2 * step) {
            const CA<A> o0 = ldv<A, CV>(w, r), o1 = ldv<A, CV>(w, r + step);
            const CA<A> a0 = ldv<A, CV>(va, r), a1 = ldv<A, CV>(va, r + step);
            const CA<A> b0 = ldv<A, CV>(vb, r), b1 = ldv<A, CV>(vb, r + step);
            const CA<A> n0 = one(o0, a0, b0), n1 = one(o1, a1, b1);
            stv<A, CV>(w, r, n0);
            stv<A, CV>(w, r + step, n1);
        }
        for (; r < r1; r += step) stv<A, CV>(w, r, one(ldv<A, CV>(w, r), ldv<A, CV>(va, r), ldv<A, CV>(vb, r)));
        return nacc;
    }
    for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        A ar = zero<A>(), ai = zero<A>();
        int t = first;
        // four vector loads in flight before their arithmetic
        for (; t + 4 <= nv; t += 4) {
            CA<A> v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) v[u] = ldv<A, CV>(V + (size_t)(t + u) * cs, r);
#pragma unroll
            for (int u = 0; u < 4; ++u) term(ar, ai, v[u], hs[t + u]);
        }
        for (; t < nv; ++t) term(ar, ai, ldv<A, CV>(V + (size_t)t * cs, r), hs[t]);
        CA<A> o = ldv<A, CV>(w, r);
        o.re = sub(o.re, ar);
        if (CV) o.im = sub(o.im, ai);
        stv<A, CV>(w, r, o);
        mac(nacc, o.re, o.re);
        if (CV) mac(nacc, o.im, o.im);
    }
    return nacc;
}

template <class A>
__device__ __forceinline__ void update_block(const SlotDev* sl, const int* __restrict__ rmap, int mmax, int pass,
                                             double* partial, int bx) {
    const SlotDev& S = sl[rmap[bx]];
    if (S.state != kSlotStep) return;
    if (pass == 1 && S.nrm[4] == 0.0) return;
    __shared__ CA<A> hs[kMaxM];
    const int nv = S.j + 1;
    const int first = (pass == 0 && S.orth == 2) ? (S.j > 0 ? S.j - 1 : 0) : 0;
    const double2* h = pass ? S.h2 : S.h1;
    for (int t = first + threadIdx.x; t < nv; t += blockDim.x) {
        const double2 v = h[t];
        hs[t] = CA<A>{from_d<A>(v.x), from_d<A>(v.y)};
    }
    __syncthreads();
    const int64_t lb = bx - S.rb_begin;
    const int64_t r0 = lb * S.rpb, r1 = min(S.n, r0 + S.rpb);
    A nacc = S.cv ? update_rows<A, true>(S, r0, r1, first, nv, hs) : update_rows<A, false>(S, r0, r1, first, nv, hs);
    __shared__ double sh[kT / 32];
    const double t = block_sum(nacc, sh);
    const int P = mmax + 1;
    if (threadIdx.x == 0) {
        partial[((size_t)bx * P + mmax) * 2] = t;
        partial[((size_t)bx * P + mmax) * 2 + 1] = 0.0;
    }
    if (pass == 0 && S.orth != 2) {
        // the Gram-Schmidt slots' second-pass dots V^* w' over this block's rows,
        // while V and w' are still in cache; used when the DGKS test asks for
        // the second pass
        const void* w = colp<A>(S, S.j + 1);
        double* row = partial + (size_t)bx * P * 2;
        for (int c0 = 0; c0 < nv; c0 += jt<A>()) {
            A re[jt<A>()], im[jt<A>()], dummy = zero<A>();
#pragma unroll
            for (int q = 0; q < jt<A>(); ++q) re[q] = im[q] = zero<A>();
            if (S.cv) dots_rows<A, true>(S, r0, r1, c0, nv, w, re, im, false, dummy);
            else dots_rows<A, false>(S, r0, r1, c0, nv, w, re, im, false, dummy);
            dots_epilogue<A>(re, im, S.cv, c0, nv, c0, row);
        }
    }
}

template <class A>
__global__ void __launch_bounds__(kT, std::is_same<A, DF>::value ? 4 : 3) eng_update(const SlotDev* __restrict__ sl, const int* __restrict__ rmap, int mmax,
                                                 int pass, double* __restrict__ partial) {
    update_block<A>(sl, rmap, mmax, pass, partial, blockIdx.x);
}

// Pass 0 of a real Gram-Schmidt slot with nv <= NV vectors, each row's nv
// vector entries held in registers: w'[r] = w[r] - sum_t V[r, t] h_t, then
// the second-pass dots acc[t] += V[r, t] w'[r] from the same registers (no
// second read of V).  Per thread the rows, the terms and the argument order
// of every multiply-add are those of update_rows followed by dots_rows, and
// the block sums go through the same dots_epilogue, so the results are
// bit-identical to update_block's.
__device__ __forceinline__ double ld_volatile(const volatile double* p) { return *p; }
__device__ __forceinline__ float ld_volatile(const volatile float* p) { return *p; }
__device__ __forceinline__ DF ld_volatile(const volatile DF* p) { return DF{p->h, p->l}; }

template <class A, int NV>
__device__ __forceinline__ void update_fused_rows(const SlotDev& S, int64_t r0, int64_t r1, int nv, const CA<A>* hs,
                                                  int mmax, double* partial, int bx) {
    const char* V = (const char*)S.V;
    const size_t cs = (size_t)S.n * vbytes<A, false>();
    void* w = (void*)(V + (size_t)(S.j + 1) * cs);
    A acc[NV];
#pragma unroll
    for (int t = 0; t < NV; ++t) acc[t] = zero<A>();
    A nacc = zero<A>();
    for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        A v[NV];
#pragma unroll
        for (int t = 0; t < NV; ++t)
            if (t < nv) v[t] = ldv<A, false>(V + (size_t)t * cs, r).re;
        A ar = zero<A>();
        // h from shared memory at each use (held in registers across the row
        // loop it would take NV more of them)
        const volatile A* hv = (const volatile A*)hs;
#pragma unroll
        for (int t = 0; t < NV; ++t)
            if (t < nv) mac(ar, v[t], ld_volatile(hv + 2 * t));
        A o = ldv<A, false>(w, r).re;
        o = sub(o, ar);
        stv<A, false>(w, r, CA<A>{o, zero<A>()});
        mac(nacc, o, o);
#pragma unroll
        for (int t = 0; t < NV; ++t)
            if (t < nv) mac(acc[t], v[t], o);
    }
    __shared__ double sh[kT / 32];
    const double tn = block_sum(nacc, sh);
    const int P = mmax + 1;
    if (threadIdx.x == 0) {
        partial[((size_t)bx * P + mmax) * 2] = tn;
        partial[((size_t)bx * P + mmax) * 2 + 1] = 0.0;
    }
    double* row = partial + (size_t)bx * P * 2;
#pragma unroll
    for (int c0 = 0; c0 < NV; c0 += jt<A>()) {
        if (c0 < nv) {
            A re[jt<A>()], im[jt<A>()];
#pragma unroll
            for (int q = 0; q < jt<A>(); ++q) {
                re[q] = c0 + q < NV ? acc[c0 + q < NV ? c0 + q : 0] : zero<A>();
                im[q] = zero<A>();
            }
            dots_epilogue<A>(re, im, false, c0, nv, c0, row);
        }
    }
}

template <class A>
__global__ void __launch_bounds__(kT, 2) eng_update_fused(const SlotDev* __restrict__ sl, const int* __restrict__ rmap,
                                                          int mmax, double* __restrict__ partial) {
    const int bx = blockIdx.x;
    const SlotDev& S = sl[rmap[bx]];
    if (S.state != kSlotStep) return;
    const int nv = S.j + 1;
    if (S.cv || S.orth == 2 || nv < 3 || nv > 20) {
        update_block<A>(sl, rmap, mmax, 0, partial, bx);
        return;
    }
    __shared__ CA<A> hs[20];
    for (int t = threadIdx.x; t < nv; t += blockDim.x) {
        const double2 v = S.h1[t];
        hs[t] = CA<A>{from_d<A>(v.x), from_d<A>(v.y)};
    }
    __syncthreads();
    const int64_t lb = bx - S.rb_begin;
    const int64_t r0 = lb * S.rpb, r1 = min(S.n, r0 + S.rpb);
    if (nv <= 12) update_fused_rows<A, 12>(S, r0, r1, nv, hs, mmax, partial, bx);
    else update_fused_rows<A, 20>(S, r0, r1, nv, hs, mmax, partial, bx);
}

// ------------------------------------------------------------ scale / advance
// w[r] *= f over rows r0..r1, four rows' loads in flight before their stores
template <class A, bool CV>
__device__ __forceinline__ void scale_rows(void* w, int64_t r0, int64_t r1, A f) {
    const int64_t step = blockDim.x;
    auto sc = [&](CA<A> v) {
        v.re = mul(v.re, f);
        if (CV) v.im = mul(v.im, f);
        return v;
    };
    int64_t r = r0 + threadIdx.x;
    for (; r + 3 * step < r1; r += 4 * step) {
        CA<A> v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) v[u] = ldv<A, CV>(w, r + u * step);
#pragma unroll
        for (int u = 0; u < 4; ++u) stv<A, CV>(w, r + u * step, sc(v[u]));
    }
    for (; r < r1; r += step) stv<A, CV>(w, r, sc(ldv<A, CV>(w, r)));
}
// mode 0: col(j+1) *= 1/beta on stepping slots; mode 1: col ncol on normalising slots
template <class A>
__device__ __forceinline__ void scale_block(const SlotDev* sl, const int* __restrict__ rmap, int mode, int bx) {
    const SlotDev& S = sl[rmap[bx]];
    if (S.state != (mode == 0 ? kSlotStep : kSlotNormalize)) return;
    const A f = from_d<A>(S.nrm[1]);
    void* w = colp<A>(S, mode == 0 ? S.j + 1 : S.ncol);
    const int64_t lb = bx - S.rb_begin;
    const int64_t r0 = lb * S.rpb, r1 = min(S.n, r0 + S.rpb);
    if (S.cv) scale_rows<A, true>(w, r0, r1, f);
    else scale_rows<A, false>(w, r0, r1, f);
}

template <class A>
__global__ void __launch_bounds__(kT) eng_scale(const SlotDev* __restrict__ sl, const int* __restrict__ rmap, int mode) {
    scale_block<A>(sl, rmap, mode, blockIdx.x);
}

__global__ void eng_advance(SlotDev* sl, int nslots) {
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= nslots) return;
    SlotDev& S = sl[id];
    if (S.state != kSlotStep) return;
    S.j += 1;
    if (S.j >= S.m) S.state = kSlotHold;
}

// ------------------------------------------------------------ rotate
// V[:, out0 + c] = sum_{i < rot_in} V[:, i] Y[i, c] for c < p (through tmp),
// then V[:, cdst] = V[:, carry]; rows are independent, each thread owns its rows.
template <class A, bool CV>
__device__ __forceinline__ void rotate_rows(const SlotDev& S, int64_t r0, int64_t r1) {
    char* V = (char*)S.V;
    char* T = (char*)S.tmp;
    const size_t cs = (size_t)S.n * vbytes<A, CV>();
    const CA<A>* Y = (const CA<A>*)S.y;
    const int nin = S.rot_in, p = S.p;
    const bool yreal = S.yreal;
    for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        auto term = [&](A& ar, A& ai, const CA<A>& v, const CA<A>& y) {
            mac(ar, v.re, y.re);
            if (CV) mac(ai, v.im, y.re);
            if (!yreal) {
                msub(ar, v.im, y.im);
                if (CV) mac(ai, v.re, y.im);
            }
        };
        for (int c = 0; c < p; ++c) {
            A ar = zero<A>(), ai = zero<A>();
            const CA<A>* Yc = Y + (size_t)c * nin;
            int i = 0;
            for (; i + 4 <= nin; i += 4) {
                CA<A> v[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) v[u] = ldv<A, CV>(V + (size_t)(i + u) * cs, r);
#pragma unroll
                for (int u = 0; u < 4; ++u) term(ar, ai, v[u], Yc[i + u]);
            }
            for (; i < nin; ++i) term(ar, ai, ldv<A, CV>(V + (size_t)i * cs, r), Yc[i]);
            stv<A, CV>(T + (size_t)c * cs, r, CA<A>{ar, ai});
        }
        for (int c = 0; c < p; ++c) stv<A, CV>(V + (size_t)(S.out0 + c) * cs, r, ldv<A, CV>(T + (size_t)c * cs, r));
        if (S.carry >= 0) stv<A, CV>(V + (size_t)S.cdst * cs, r, ldv<A, CV>(V + (size_t)S.carry * cs, r));
    }
}

// The same rotation when p <= PT: a row's p outputs stay in registers while
// its inputs stream past once (PT multiply-adds per load), then go straight
// into V (every input of the row has been read by then), then the carry copy.
template <class A, bool CV, int PT>
__device__ __forceinline__ void rotate_rows_tile(const SlotDev& S, int64_t r0, int64_t r1) {
    char* V = (char*)S.V;
    const size_t cs = (size_t)S.n * vbytes<A, CV>();
    const CA<A>* __restrict__ Y = (const CA<A>*)S.y;
    const int nin = S.rot_in, p = S.p;
    const bool yreal = S.yreal;
    for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        A ar[PT], ai[PT];
#pragma unroll
        for (int c = 0; c < PT; ++c) ar[c] = ai[c] = zero<A>();
        auto fold = [&](const CA<A>& v, int i) {
#pragma unroll
            for (int c = 0; c < PT; ++c) {
                if (c < p) {
                    const CA<A> y = Y[(size_t)c * nin + i];
                    mac(ar[c], v.re, y.re);
                    if (CV) mac(ai[c], v.im, y.re);
                    if (!yreal) {
                        msub(ar[c], v.im, y.im);
                        if (CV) mac(ai[c], v.re, y.im);
                    }
                }
            }
        };
        int i = 0;
        for (; i + 2 <= nin; i += 2) {
            const CA<A> v0 = ldv<A, CV>(V + (size_t)i * cs, r), v1 = ldv<A, CV>(V + (size_t)(i + 1) * cs, r);
            fold(v0, i);
            fold(v1, i + 1);
        }
        if (i < nin) fold(ldv<A, CV>(V + (size_t)i * cs, r), i);
#pragma unroll
        for (int c = 0; c < PT; ++c)
            if (c < p) stv<A, CV>(V + (size_t)(S.out0 + c) * cs, r, CA<A>{ar[c], ai[c]});
        if (S.carry >= 0) stv<A, CV>(V + (size_t)S.cdst * cs, r, ldv<A, CV>(V + (size_t)S.carry * cs, r));
    }
}

template <class A>
__global__ void __launch_bounds__(kT, 2) eng_rotate(const SlotDev* __restrict__ sl, const int* __restrict__ rmap) {
    const SlotDev& S = sl[rmap[blockIdx.x]];
    if (S.state != kSlotRotate || S.rot_tc) return;
    const int64_t lb = blockIdx.x - S.rb_begin;
    const int64_t r0 = lb * S.rpb, r1 = min(S.n, r0 + S.rpb);
    if (S.p <= 8) {
        if (S.cv) rotate_rows_tile<A, true, 8>(S, r0, r1);
        else rotate_rows_tile<A, false, 8>(S, r0, r1);
    } else if (!std::is_same<A, DF>::value && S.p <= 16) {
        // (double-float accumulators for 16 outputs would not fit in registers)
        if constexpr (!std::is_same<A, DF>::value) {
            if (S.cv) rotate_rows_tile<A, true, 16>(S, r0, r1);
            else rotate_rows_tile<A, false, 16>(S, r0, r1);
        }
    } else {
        if (S.cv) rotate_rows<A, true>(S, r0, r1);
        else rotate_rows<A, false>(S, r0, r1);
    }
}


// ------------------------------------------------------------ rotate on the tensor cores
// The thick-restart rotation V[:, out0 + c] = sum_{i < rot_in} V[:, i] Y[i, c]
// as an exact sliced integer product on the FP16 tensor cores (qs_tc.cuh) for
// the FP64 storage.  A slot takes it (rot_tc) when its
// coefficients are real with |Y| <= 1, 2 <= p <= 16 and rot_in <= 32 (the
// restarts of eigsh, whose V columns are orthonormal); eng_rotate skips those
// slots.  Each block keeps its row range: tiles of 128 real components (a
// complex row is two), thread t owns component t of the tile.  One thread
// issues the MMAs; every wait is bounded and a timeout sets *err.
constexpr int kTcRows = 128, kTcK = 32, kTcN = 16, kTcDigits = 8, kTcGroups = 9;
constexpr uint32_t kTcCols = 256;   // TMEM columns: nine accumulators of kTcN columns
constexpr int kTcATile = kTcRows * kTcK * 2;   // bytes of one digit matrix of V's tile
constexpr int kTcBTile = kTcN * kTcK * 2;      // bytes of one digit matrix of Y
constexpr size_t kTcSmemUsed = (size_t)kTcDigits * (kTcATile + kTcBTile) + 1024;
// requested so that at most two blocks share an SM (2 x 256 TMEM columns: an
// allocation never has to wait for another block)
constexpr size_t kTcSmem = 100 * 1024;
static_assert(kTcSmemUsed <= kTcSmem, "tensor-core rotation tiles exceed their shared memory");
constexpr long long kTcWaitCycles = 2000000000LL;   // about one second

// real component (8 bytes) as trunc(v 2^61), from its raw bits
template <class A> __device__ __forceinline__ long long tc_fix_bits(unsigned long long b);
template <> __device__ __forceinline__ long long tc_fix_bits<double>(unsigned long long b) {
    return fix61(__longlong_as_double((long long)b));
}
// stores v 2^scale into real component e
template <class A> __device__ __forceinline__ void tc_store(char* col, int64_t e, long long v, int scale);
template <> __device__ __forceinline__ void tc_store<double>(char* col, int64_t e, long long v, int scale) {
    ((double*)col)[e] = f64_of_i64(v, scale);
}
// real part of the rotation coefficient e (column-major rot_in x p)
template <class A> __device__ __forceinline__ long long tc_fix_y(const void* y, int e);
template <> __device__ __forceinline__ long long tc_fix_y<double>(const void* y, int e) {
    return fix61(((const CA<double>*)y)[e].re);
}

template <class A>
__global__ void __launch_bounds__(kTcRows, 1) eng_rotate_tc(const SlotDev* __restrict__ sl,
                                                           const int* __restrict__ rmap, int* __restrict__ err) {
    const SlotDev& S = sl[rmap[blockIdx.x]];
    if (S.state != kSlotRotate || !S.rot_tc) return;
    extern __shared__ unsigned char tc_raw[];
    unsigned char* sa = (unsigned char*)(((uintptr_t)tc_raw + 1023) & ~(uintptr_t)1023);
    unsigned char* sb = sa + kTcDigits * kTcATile;
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tbase;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int nin = S.rot_in, p = S.p;
    // zero both operand areas (the K padding beyond rot_in and the rows of Y
    // beyond p stay zero), then the digits of Y: row c of B_b is digit b of
    // Y[:, c] along K
    for (int w = tid; w < kTcDigits * (kTcATile + kTcBTile) / 16; w += kTcRows)
        ((uint4*)sa)[w] = make_uint4(0u, 0u, 0u, 0u);
    __syncthreads();
    for (int e = tid; e < nin * p; e += kTcRows) {
        const int i = e % nin, c = e / nin;
        const long long X = tc_fix_y<A>(S.y, e);
        const uint32_t sg = X < 0 ? 0x8000u : 0u;
        const unsigned long long m = X < 0 ? (unsigned long long)(-X) : (unsigned long long)X;
#pragma unroll
        for (int a = 0; a < kTcDigits; ++a)
            *(uint16_t*)(sb + a * kTcBTile + tc_off(c, i, kTcK)) =
                (uint16_t)f16_of_byte((uint32_t)(m >> (8 * (kTcDigits - 1 - a))) & 0xffu, sg);
    }
    if (warp == 0) tc_alloc(&tbase, kTcCols);
    if (tid == 0) mbar_init(&mbar, 1);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tbase;
    const int comps = S.cv ? 2 : 1;
    const int64_t lb = blockIdx.x - S.rb_begin;
    // blockIdx.y: this block's share of the row block (gridDim.y shares of
    // whole tiles), so that a small engine still fills the GPU
    const int64_t rb0 = lb * S.rpb, rb1 = min(S.n, rb0 + S.rpb);
    const int64_t share = ((rb1 - rb0 + gridDim.y - 1) / gridDim.y + kTcRows - 1) / kTcRows * kTcRows;
    const int64_t r0 = min(rb1, rb0 + (int64_t)blockIdx.y * share), r1 = min(rb1, r0 + share);
    const int64_t e0 = r0 * comps, e1 = r1 * comps;
    char* V = (char*)S.V;
    const size_t cs = (size_t)S.n * comps * 8;   // bytes of one column
    const int ksteps = (nin + 15) / 16;
    uint32_t phase = 0;
    // raw inputs of this thread's component, the next tile's loaded while the
    // tensor cores work on the current one
    unsigned long long raw[kTcK];
    auto load_tile = [&](int64_t t0) {
        const int64_t e = t0 + tid;
        const bool live = e < e1;
#pragma unroll
        for (int i = 0; i < kTcK; ++i)
            raw[i] = (live && i < nin) ? ((const unsigned long long*)(V + (size_t)i * cs))[e] : 0ull;
    };
    if (e0 < e1) load_tile(e0);
    for (int64_t t0 = e0; t0 < e1; t0 += kTcRows) {
        const int64_t e = t0 + tid;
        const bool live = e < e1;
        // the inputs as fixed-point integers, eight per K core matrix, and
        // their bytes as FP16 into the digit matrices
#pragma unroll
        for (int kc = 0; kc < kTcK / 8; ++kc) {
            if (kc * 8 >= nin) break;
            unsigned long long mag[8];
            uint32_t sg[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const long long X = tc_fix_bits<A>(raw[kc * 8 + u]);
                sg[u] = X < 0 ? 0x8000u : 0u;
                mag[u] = X < 0 ? (unsigned long long)(-X) : (unsigned long long)X;
            }
            uint32_t sg2[4], lo[8], hi[8];
#pragma unroll
            for (int u = 0; u < 4; ++u) sg2[u] = sg[2 * u] | (sg[2 * u + 1] << 16);
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                lo[u] = (uint32_t)mag[u];
                hi[u] = (uint32_t)(mag[u] >> 32);
            }
            // digit a is byte 7 - a of the magnitude
            auto put = [&](int a, const uint32_t (&w)[4]) {
                *(uint4*)(sa + a * kTcATile + tc_off(tid, kc * 8, kTcK)) = make_uint4(w[0], w[1], w[2], w[3]);
            };
#define QS_TC_DIGIT(A_, WORD_, BB_)                                                                  \
            {                                                                                       \
                uint32_t w[4];                                                                      \
                _Pragma("unroll") for (int u = 0; u < 4; ++u)                                       \
                    w[u] = f16x2_of_bytes<BB_>(WORD_[2 * u], WORD_[2 * u + 1], sg2[u]);             \
                put(A_, w);                                                                         \
            }
            QS_TC_DIGIT(0, hi, 3)
            QS_TC_DIGIT(1, hi, 2)
            QS_TC_DIGIT(2, hi, 1)
            QS_TC_DIGIT(3, hi, 0)
            QS_TC_DIGIT(4, lo, 3)
            QS_TC_DIGIT(5, lo, 2)
            QS_TC_DIGIT(6, lo, 1)
            QS_TC_DIGIT(7, lo, 0)
#undef QS_TC_DIGIT
        }
        tc_fence_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
            constexpr uint32_t idesc = tc_idesc_f16(kTcRows, kTcN);
            const uint32_t abase = smem_addr(sa), bbase = smem_addr(sb);
            constexpr uint32_t sbo = (kTcK / 8) * 128;
            // accumulator s: sum over digit pairs a + b = s of A_a B_b
            for (int s = 0; s < kTcGroups; ++s) {
                uint32_t acc = 0;
                const int alo = s > kTcDigits - 1 ? s - (kTcDigits - 1) : 0, ahi = s < kTcDigits - 1 ? s : kTcDigits - 1;
                for (int a = alo; a <= ahi; ++a)
                    for (int kk = 0; kk < ksteps; ++kk) {
                        const uint64_t ad = tc_sdesc(abase + a * kTcATile + kk * 256, 128, sbo);
                        const uint64_t bd = tc_sdesc(bbase + (s - a) * kTcBTile + kk * 256, 128, sbo);
                        tc_mma_f16(tmem + (uint32_t)(s * kTcN), ad, bd, idesc, acc);
                        acc = 1;
                    }
            }
            tc_commit(&mbar);
        }
        // the digits are in shared memory: fetch the next tile meanwhile
        if (t0 + kTcRows < e1) load_tile(t0 + kTcRows);
        const bool ok = __syncthreads_and(mbar_wait(&mbar, phase, kTcWaitCycles) ? 1 : 0);
        phase ^= 1u;
        tc_fence_after();
        if (!ok) {
            if (tid == 0) atomicExch(err, 1);
            break;
        }
        // epilogue: row t of the tile is TMEM lane t; warp w reads lanes 32w..32w+31
        const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
        for (int c0 = 0; c0 < p; c0 += 4) {
            uint32_t v[kTcGroups][4];
#pragma unroll
            for (int s = 0; s < kTcGroups; ++s) tc_ld4(trow + (uint32_t)(s * kTcN + c0), v[s]);
            tc_wait_ld();
            long long hi[4] = {0, 0, 0, 0}, lo[4] = {0, 0, 0, 0};
#pragma unroll
            for (int s = 0; s < kTcGroups; ++s) {
                // a new definition after the wait: no use of the loaded
                // registers can move above it
                asm volatile("" : "+r"(v[s][0]), "+r"(v[s][1]), "+r"(v[s][2]), "+r"(v[s][3]));
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const long long d = (long long)__float2int_rn(__uint_as_float(v[s][u]));   // exact: |D_s| < 2^24
                    if (s <= 3) hi[u] += d << (8 * (3 - s));
                    else lo[u] += d << (8 * (8 - s));
                }
            }
            if (live) {
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (c0 + u < p) {
                        // sum = 2^-122 sum_s 256^(14-s) D_s = 2^-74 (hi 2^40 + lo); kept at 2^-62
                        const long long T = (hi[u] << 28) + (lo[u] >> 12);
                        tc_store<A>(V + (size_t)(S.out0 + c0 + u) * cs, e, T, -62);
                    }
            }
        }
        if (live && S.carry >= 0)
            ((unsigned long long*)(V + (size_t)S.cdst * cs))[e] = ((const unsigned long long*)(V + (size_t)S.carry * cs))[e];
        tc_fence_before();
        __syncthreads();   // the next tile overwrites the digits and the accumulators
        tc_fence_after();
    }
    __syncthreads();
    if (warp == 0) tc_dealloc(tmem, kTcCols);
}

// Runs f with a value of the step arithmetic's type for storage st.
template <class F>
void with_store(Store st, F&& f) {
    if (st == Store::DF) f(DF{0.f, 0.f});
    else if (st == Store::F32) f(0.0f);
    else f(0.0);
}

VKind store_kind(Store st, bool cv) {
    if (st == Store::DF) return cv ? VKind::CDF64 : VKind::DF64;
    if (st == Store::F32) return cv ? VKind::C64 : VKind::F32;
    return cv ? VKind::C128 : VKind::F64;
}

// ------------------------------------------------------------ autotuner
struct TuneKey {
    int st;
    bool cv, cm;
    int size_class;
    bool operator<(const TuneKey& o) const {
        return std::tie(st, cv, cm, size_class) < std::tie(o.st, o.cv, o.cm, o.size_class);
    }
};
std::mutex g_tune_mu;
std::map<TuneKey, Tiles> g_tuned;

int size_class(int64_t n) { return (int)std::floor(2.0 * std::log2((double)std::max<int64_t>(n, 1))); }

}  // namespace

// ====================================================================== Engine
Engine::Engine(Store st, cudaStream_t s) : st_(st), s_(s) {
    std::vector<double> r64(kMaxGroup + 1, 0.0);
    std::vector<float> rdf(2 * (kMaxGroup + 1), 0.f), r32(kMaxGroup + 1, 0.f);
    for (int i = 1; i <= kMaxGroup; ++i) {
        r64[i] = 1.0 / std::sqrt((double)i);
        df_split_host(r64[i], rdf[2 * i], rdf[2 * i + 1]);
        r32[i] = (float)r64[i];
    }
    rsq64_.alloc(r64.size() * sizeof(double));
    rsqdf_.alloc(rdf.size() * sizeof(float));
    rsq32_.alloc(r32.size() * sizeof(float));
    QS_CUDA(cudaMemcpy(rsq64_.p, r64.data(), r64.size() * sizeof(double), cudaMemcpyHostToDevice));
    QS_CUDA(cudaMemcpy(rsqdf_.p, rdf.data(), rdf.size() * sizeof(float), cudaMemcpyHostToDevice));
    QS_CUDA(cudaMemcpy(rsq32_.p, r32.data(), r32.size() * sizeof(float), cudaMemcpyHostToDevice));
    const char* tc = std::getenv("QS_TC_ROTATE");
    tc_rotate_ = !(tc && tc[0] == '0');
    tc_err_.alloc(sizeof(int));
    QS_CUDA(cudaMemset(tc_err_.p, 0, sizeof(int)));
}

Engine::~Engine() {
    cudaStreamSynchronize(s_);
    if (side_) {
        cudaStreamSynchronize(side_);
        cudaStreamDestroy(side_);
    }
    if (fork_) cudaEventDestroy(fork_);
    if (join_) cudaEventDestroy(join_);
    if (exec_) cudaGraphExecDestroy(exec_);
    if (graph_) cudaGraphDestroy(graph_);
}

Tiles Engine::tune(Op& op, int m, bool cv) {
    const TuneKey key{(int)st_, cv, op.complex_mat, size_class(op.basis->n)};
    {
        std::lock_guard<std::mutex> g(g_tune_mu);
        auto it = g_tuned.find(key);
        if (it != g_tuned.end()) return it->second;
    }
    // time a few steps of this operator alone for every candidate tile pair
    const int mt = std::min(m, 12);
    Engine E(st_, s_);
    int id = E.add(op, mt, cv, false);
    E.seed(id, 1);
    E.normalize({id});
    cudaEvent_t e0, e1;
    QS_CUDA(cudaEventCreate(&e0));
    QS_CUDA(cudaEventCreate(&e1));
    Tiles best;
    float best_ms = 1e30f;
    // only the SpMV's slices per block are timed: a row's product does not
    // depend on them, while the BLAS row block fixes the order of every
    // reduction and stays at its default (results repeat from run to run)
    const int rpb = best.rpb;
    for (int spb : {16, 64, 256}) {
        E.slots_[id].d.rpb = rpb;
        E.slots_[id].d.spb = spb;
        E.maps_dirty_ = true;
        E.start(id, 0);
        E.run(2);  // captures the graph, warms up
        E.start(id, 2);
        QS_CUDA(cudaEventRecord(e0, s_));
        E.run(std::min(6, mt - 2));
        QS_CUDA(cudaEventRecord(e1, s_));
        QS_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        QS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best_ms) {
            best_ms = ms;
            best.rpb = rpb;
            best.spb = spb;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    launches_ += E.launches();
    std::lock_guard<std::mutex> g(g_tune_mu);
    g_tuned[key] = best;
    return best;
}

size_t Engine::slot_bytes(int64_t n, int m, bool cv, int tmp_cols, Store st) {
    const size_t es = store_bytes(st, cv);
    const int tc = tmp_cols > 0 ? tmp_cols : m - 1;
    return (size_t)(m + 1 + tc) * n * es + ((size_t)2 * m + (size_t)(m + 1) * m + (size_t)m * m) * 16 + 128;
}

int Engine::add(Op& op, int m, bool cv, bool tune_tiles, int tmp_cols, int orth) {
    if (orth < 0 || orth > 2 || (orth == 2 && !op.hermitian))
        throw Error(QS_ERR_ARGUMENT, "the three-term recurrence needs a Hermitian operator");
    if (m < 2 || m > kMaxM) throw Error(QS_ERR_ARGUMENT, "Krylov basis size must lie in 2:256");
    if (op.complex_mat && !cv) throw Error(QS_ERR_ARGUMENT, "complex operators need complex vectors");
    if (!op.assembled) op_assemble(op);
    const Assembled& M = op.asm_;
    if (!M.has_sell) throw Error(QS_ERR_UNSUPPORTED, "the batched engine needs the sliced assembled layout");
    QS_CUDA(cudaStreamSynchronize(op.stream));
    const int64_t n = op.basis->n;
    Slot sl;
    sl.op = &op;
    SlotDev& d = sl.d;
    d.sptr = M.sell_ptr.as<int64_t>();
    d.len = M.sell_len.as<uint16_t>();
    d.words = M.sell_words.as<uint32_t>();
    d.cols = M.sell_cols.as<int32_t>();
    d.codes = M.sell_codes.as<uint16_t>();
    d.tab64 = M.table64.as<double2>();
    d.tabdf = M.table_df.as<float4>();
    d.stab = op.basis->symmetric ? op.basis->d_stab.as<uint16_t>() : nullptr;
    d.diag64 = op.d_diag.as<double2>();
    d.diagdf = op.d_diag_df.as<float4>();
    d.tab32 = M.table32.as<float2>();
    d.diag32 = op.d_diag32.as<float2>();
    d.code_mask = M.code_bits >= 32 ? 0xffffffffu : ((1u << M.code_bits) - 1u);
    d.packed = M.packed;
    d.code_bits = M.code_bits;
    d.ncodes = M.ncodes;
    d.max_stab = std::min(kMaxGroup, std::max(1, op.basis->group.ng));
    d.cm = op.complex_mat;
    d.cv = cv;
    d.n = n;
    d.nslices = M.nslices;
    const size_t es = store_bytes(st_, cv);
    sl.V.alloc((size_t)(m + 1) * n * es, s_);
    const int tc = tmp_cols > 0 ? std::min(tmp_cols, m) : m - 1;
    sl.tmp.alloc((size_t)tc * n * es, s_);
    QS_CUDA(cudaMemsetAsync(sl.V.p, 0, sl.V.bytes, s_));
    // h1 (m), h2 (m), rec ((m+1) m) as double2, nrm (4 doubles)
    const size_t nsmall = (size_t)2 * m + (size_t)(m + 1) * m;
    sl.small.alloc(nsmall * sizeof(double2) + 8 * sizeof(double), s_);
    QS_CUDA(cudaMemsetAsync(sl.small.p, 0, sl.small.bytes, s_));
    d.V = sl.V.p;
    d.tmp = sl.tmp.p;
    d.h1 = sl.small.as<double2>();
    d.h2 = d.h1 + m;
    d.rec = d.h2 + m;
    d.nrm = (double*)(d.rec + (size_t)(m + 1) * m);
    d.y = nullptr;
    d.m = m;
    d.j = 0;
    d.state = kSlotIdle;
    d.carry = -1;
    d.orth = orth;
    sl.tcols = tc;
    Tiles t;
    // (a slot on the cluster step splits its slices by CTA, not by the tile)
    if (tune_tiles && n >= 4096 && m >= 4 && cluster_size_for(d) == 0) t = tune(op, m, cv);
    d.rpb = t.rpb;
    d.spb = t.spb;
    sl.live = true;
    // reuse a dead slot index
    int id = -1;
    for (int i = 0; i < (int)slots_.size(); ++i)
        if (!slots_[i].live) { id = i; break; }
    if (id < 0) {
        id = (int)slots_.size();
        slots_.emplace_back();
    }
    slots_[id] = std::move(sl);
    maps_dirty_ = dirty_ = true;
    return id;
}

void Engine::remove(int id) {
    if (!alive(id)) return;
    slots_[id] = Slot();   // pooled buffers wait for this stream's work before reuse
    maps_dirty_ = dirty_ = true;
}

void Engine::build_maps() {
    nrb_ = nsb_ = 0;
    mmax_ = dmax_ = 1;
    cgs_ = false;
    for (auto& sl : slots_) {
        SlotDev& d = sl.d;
        if (!sl.live) {
            d.state = kSlotIdle;
            d.rb_begin = d.rb_count = d.sb_begin = d.sb_count = 0;
            continue;
        }
        d.rb_begin = nrb_;
        d.rb_count = (int)((d.n + d.rpb - 1) / d.rpb);
        d.sb_begin = nsb_;
        d.sb_count = (int)((d.nslices + d.spb - 1) / d.spb);
        nrb_ += d.rb_count;
        nsb_ += d.sb_count;
        mmax_ = std::max(mmax_, d.m);
        dmax_ = std::max(dmax_, d.orth == 2 ? 1 : d.m);
        cgs_ = cgs_ || d.orth != 2;
    }
    std::vector<int> rm(std::max(1, nrb_)), sm(std::max(1, nsb_));
    for (int i = 0; i < (int)slots_.size(); ++i) {
        const SlotDev& d = slots_[i].d;
        for (int b = 0; b < d.rb_count; ++b) rm[d.rb_begin + b] = i;
        for (int b = 0; b < d.sb_count; ++b) sm[d.sb_begin + b] = i;
    }
    if (rm.size() * sizeof(int) > cap_rmap_) {
        cap_rmap_ = rm.size() * sizeof(int) * 2;
        rmap_.alloc(cap_rmap_);
    }
    if (sm.size() * sizeof(int) > cap_smap_) {
        cap_smap_ = sm.size() * sizeof(int) * 2;
        smap_.alloc(cap_smap_);
    }
    const size_t pb = (size_t)std::max(1, nrb_) * (mmax_ + 1) * 2 * sizeof(double);
    if (pb > cap_partial_) {
        cap_partial_ = pb * 2;
        partial_.alloc(cap_partial_);
    }
    if ((int)slots_.size() > cap_slots_) {
        cap_slots_ = std::max<int>(8, (int)slots_.size() * 2);
        dslots_.alloc((size_t)cap_slots_ * sizeof(SlotDev));
    }
    QS_CUDA(cudaMemcpyAsync(rmap_.p, rm.data(), rm.size() * sizeof(int), cudaMemcpyHostToDevice, s_));
    QS_CUDA(cudaMemcpyAsync(smap_.p, sm.data(), sm.size() * sizeof(int), cudaMemcpyHostToDevice, s_));
    QS_CUDA(cudaStreamSynchronize(s_));
    if (exec_) {
        cudaGraphExecDestroy(exec_);
        exec_ = nullptr;
    }
    if (graph_) {
        cudaGraphDestroy(graph_);
        graph_ = nullptr;
    }
    maps_dirty_ = false;
    dirty_ = true;
}

void Engine::sync_table() {
    if (maps_dirty_) build_maps();
    if (!dirty_) return;
    std::vector<SlotDev> h(slots_.size());
    for (size_t i = 0; i < slots_.size(); ++i) h[i] = slots_[i].d;
    if (!h.empty())
        QS_CUDA(cudaMemcpyAsync(dslots_.p, h.data(), h.size() * sizeof(SlotDev), cudaMemcpyHostToDevice, s_));
    QS_CUDA(cudaStreamSynchronize(s_));
    dirty_ = false;
}

// One step of every stepping slot; returns the number of launches.  The dots
// and reduce grids cover the most vectors a slot dots against (dmax), so
// three-term slots cost one block row however large their basis; without
// Gram-Schmidt slots the second-pass launches are left out.
// QS_FUSED_UPDATE=0 keeps the first-pass dots on eng_dots and pass 0 on
// eng_update (the fused kernels give the same bits; the switch exists to time
// the two)
static bool fused_update_on() {
    const char* e = std::getenv("QS_FUSED_UPDATE");
    return !(e && e[0] == '0');
}

template <class A>
static int launch_step_t(const SlotDev* ds, SlotDev* dsw, const int* rm, const int* sm, double* pa, const void* rsq,
                         int nrb, int nsb, int mmax, int dmax, bool cgs, int ns, cudaStream_t s) {
    const dim3 gd(nrb, (dmax + jt<A>() - 1) / jt<A>());
    eng_spmv<A><<<nsb, kT, 0, s>>>(ds, sm, rsq);
    if (fused_update_on()) eng_dots_fused<A><<<gd, kT, 0, s>>>(ds, rm, mmax, pa);
    else eng_dots<A><<<gd, kT, 0, s>>>(ds, rm, mmax, 0, pa);
    eng_reduce<<<dim3(ns, dmax + 1), kT, 0, s>>>(ds, mmax, 0, pa, dmax);
    if (fused_update_on()) eng_update_fused<A><<<nrb, kT, 0, s>>>(ds, rm, mmax, pa);
    else eng_update<A><<<nrb, kT, 0, s>>>(ds, rm, mmax, 0, pa);
    eng_reduce<<<dim3(ns, 1), kT, 0, s>>>(ds, mmax, 1, pa);
    int n = 5;
    if (cgs) {
        eng_reduce<<<dim3(ns, mmax), kT, 0, s>>>(ds, mmax, 2, pa);
        eng_update<A><<<nrb, kT, 0, s>>>(ds, rm, mmax, 1, pa);
        eng_reduce<<<dim3(ns, 1), kT, 0, s>>>(ds, mmax, 3, pa);
        n += 3;
    }
    eng_scale<A><<<nrb, kT, 0, s>>>(ds, rm, 0);
    eng_advance<<<(ns + 127) / 128, 128, 0, s>>>(dsw, ns);
    return n + 2;
}

// ------------------------------------------------------------ cluster step
// The Lanczos steps of every stepping slot, one thread-block cluster per
// slot, in one launch that runs the steps up to the next Hold event: the
// cluster's CTAs split the slot's slices (and so its rows), every phase
// works on the CTA's own rows, and the per-step reductions (the first-pass
// dots and ||w||^2, ||w'||^2 and the second-pass dots, ||w''||^2) cross the
// cluster through distributed shared memory: each CTA leaves its block sums
// in its shared memory, a cluster barrier (barrier.cluster, release /
// acquire) separates the phases, and every CTA adds the CTAs' sums in rank
// order, so all of them hold the same coefficients and take the same DGKS
// decision without a broadcast.  CTA 0 writes the step's record column; the
// slot's row range ends on a cluster barrier before the next product gathers
// from it.  Nothing crosses clusters, so a slot's result does not depend on
// the others; the reduction order (one partial per CTA) differs from the
// graph replay's (one per row block), so results agree to rounding.
__device__ __forceinline__ uint32_t cl_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t cl_size() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t cl_id() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
    return r;
}
__device__ __forceinline__ void cl_sync() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// a double in CTA `rank`'s shared memory at the address of p in this CTA's
__device__ __forceinline__ double cl_ld(const double* p, uint32_t rank) {
    uint32_t ra;
    double v;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(smem_addr(p)), "r"(rank));
    asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(ra) : "memory");
    return v;
}

template <class A, bool CV>
__device__ __forceinline__ void cluster_steps(SlotDev& Ls, SlotDev* Sg, int nsteps, const CA<A>* tab, bool smem_tab,
                                              const A* rsq, double* part1, double* part2, double* h1, double* h2,
                                              CA<A>* hs, double* scal, double* shb) {
    const uint32_t C = cl_size(), rank = cl_rank();
    const int m = Ls.m, orth = Ls.orth, ld = m + 1;
    const int64_t s0 = Ls.nslices * (int64_t)rank / C, s1 = Ls.nslices * (int64_t)(rank + 1) / C;
    const int64_t r0 = min(Ls.n, s0 * kSellSlice), r1 = min(Ls.n, s1 * kSellSlice);
    int j = Ls.j;
    for (int step = 0; step < nsteps && j < m; ++step) {
        if (threadIdx.x == 0) Ls.j = j;
        __syncthreads();
        // product over this CTA's slices: col(j + 1) = H col(j)
        spmv_slices<A>(Ls, s0, s1, tab, smem_tab, rsq);
        __syncthreads();
        // first-pass dots over this CTA's rows (and ||w||^2 for DGKS)
        const int nv = j + 1;
        const int first = orth == 2 ? j : 0;
        const bool want_wn = orth == 1;
        const void* w = colp<A>(Ls, j + 1);
        A wn = zero<A>();
        for (int i0 = first; i0 < nv; i0 += jt<A>()) {
            A re[jt<A>()], im[jt<A>()];
#pragma unroll
            for (int q = 0; q < jt<A>(); ++q) re[q] = im[q] = zero<A>();
            dots_rows<A, CV>(Ls, r0, r1, i0, nv, w, re, im, want_wn && i0 == first, wn);
            dots_epilogue<A>(re, im, CV, i0, nv, i0, part1);
        }
        {
            const double t = block_sum(wn, shb);
            if (threadIdx.x == 0) part1[m * 2] = t;
        }
        cl_sync();
        // the cluster's sums, in rank order, in every CTA
        for (int i = first + threadIdx.x; i <= j; i += blockDim.x) {
            double re = 0, im = 0;
            for (uint32_t r = 0; r < C; ++r) {
                re += cl_ld(&part1[i * 2], r);
                im += cl_ld(&part1[i * 2 + 1], r);
            }
            h1[i * 2] = re;
            h1[i * 2 + 1] = im;
        }
        if (threadIdx.x == 0) {
            double t = 0;
            for (uint32_t r = 0; r < C; ++r) t += cl_ld(&part1[m * 2], r);
            scal[0] = t;
            // the three-term recurrence takes beta_{j-1} from the record
            if (orth == 2 && j > 0) {
                const double2 b = Ls.rec[(size_t)(j - 1) * ld + j];
                h1[(j - 1) * 2] = b.x;
                h1[(j - 1) * 2 + 1] = b.y;
            }
        }
        __syncthreads();
        // pass 0: w' = w - V h1 over this CTA's rows, ||w'||^2 and the
        // second-pass dots V^* w'
        const int first_u = orth == 2 ? (j > 0 ? j - 1 : 0) : 0;
        for (int t = first_u + threadIdx.x; t < nv; t += blockDim.x)
            hs[t] = CA<A>{from_d<A>(h1[t * 2]), from_d<A>(h1[t * 2 + 1])};
        __syncthreads();
        {
            const A nacc = update_rows<A, CV>(Ls, r0, r1, first_u, nv, hs);
            const double t = block_sum(nacc, shb);
            if (threadIdx.x == 0) part2[m * 2] = t;
        }
        if (orth != 2)
            for (int c0 = 0; c0 < nv; c0 += jt<A>()) {
                A re[jt<A>()], im[jt<A>()], dummy = zero<A>();
#pragma unroll
                for (int q = 0; q < jt<A>(); ++q) re[q] = im[q] = zero<A>();
                dots_rows<A, CV>(Ls, r0, r1, c0, nv, w, re, im, false, dummy);
                dots_epilogue<A>(re, im, CV, c0, nv, c0, part2);
            }
        cl_sync();
        if (threadIdx.x == 0) {
            double t = 0;
            for (uint32_t r = 0; r < C; ++r) t += cl_ld(&part2[m * 2], r);
            const double nb = sqrt(fmax(t, 0.0));
            const bool second = orth == 0 || (orth == 1 && nb < 0.717 * sqrt(fmax(scal[0], 0.0)));
            scal[1] = nb;
            scal[2] = second ? 1.0 : 0.0;
        }
        if (orth != 2)
            for (int i = threadIdx.x; i <= j; i += blockDim.x) {
                double re = 0, im = 0;
                for (uint32_t r = 0; r < C; ++r) {
                    re += cl_ld(&part2[i * 2], r);
                    im += cl_ld(&part2[i * 2 + 1], r);
                }
                h2[i * 2] = re;
                h2[i * 2 + 1] = im;
            }
        __syncthreads();
        double2* col = Ls.rec + (size_t)j * ld;
        double nb = scal[1];
        if (scal[2] == 0.0) {
            if (rank == 0 && threadIdx.x == 0) {
                for (int q = first_u; q <= j; ++q) col[q] = make_double2(h1[q * 2], h1[q * 2 + 1]);
                col[j + 1] = make_double2(nb, 0.0);
            }
        } else {
            // second pass: w'' = w' - V h2, the record column h1 + h2
            if (rank == 0)
                for (int i = threadIdx.x; i <= j; i += blockDim.x)
                    col[i] = make_double2(h1[i * 2] + h2[i * 2], h1[i * 2 + 1] + h2[i * 2 + 1]);
            for (int t = threadIdx.x; t < nv; t += blockDim.x)
                hs[t] = CA<A>{from_d<A>(h2[t * 2]), from_d<A>(h2[t * 2 + 1])};
            __syncthreads();
            const A nacc = update_rows<A, CV>(Ls, r0, r1, 0, nv, hs);
            const double t3 = block_sum(nacc, shb);
            if (threadIdx.x == 0) part1[m * 2] = t3;
            cl_sync();
            if (threadIdx.x == 0) {
                double t = 0;
                for (uint32_t r = 0; r < C; ++r) t += cl_ld(&part1[m * 2], r);
                scal[1] = sqrt(fmax(t, 0.0));
                if (rank == 0) col[j + 1] = make_double2(scal[1], 0.0);
            }
            __syncthreads();
            nb = scal[1];
        }
        // col(j + 1) /= beta over this CTA's rows
        const A f = from_d<A>(nb > 0 ? 1.0 / nb : 0.0);
        scale_rows<A, CV>(colp<A>(Ls, j + 1), r0, r1, f);
        cl_sync();
        ++j;
    }
    if (rank == 0 && threadIdx.x == 0) {
        Sg->j = j;
        if (j >= m) Sg->state = kSlotHold;
    }
}

template <class A>
__global__ void __launch_bounds__(kT, 2) eng_cluster(SlotDev* sl, const int* __restrict__ cmap, int nsteps,
                                                     const void* __restrict__ rsqt) {
    __shared__ SlotDev Ls;
    __shared__ CA<A> tab[1024];
    __shared__ A rsq[kMaxGroup + 1];
    __shared__ double part1[(kMaxM + 1) * 2], part2[(kMaxM + 1) * 2], h1[kMaxM * 2], h2[kMaxM * 2];
    __shared__ CA<A> hs[kMaxM];
    __shared__ double scal[4], shb[kT / 32];
    SlotDev* Sg = &sl[cmap[cl_id()]];
    if (threadIdx.x == 0) Ls = *Sg;
    __syncthreads();
    if (Ls.state == kSlotStepCluster) {
        const bool smem_tab = Ls.ncodes <= 1024;
        if (smem_tab)
            for (int i = threadIdx.x; i < Ls.ncodes; i += blockDim.x) tab[i] = ldtab<A>(Ls, i);
        if (Ls.stab)
            for (int i = threadIdx.x; i <= Ls.max_stab; i += blockDim.x) rsq[i] = ldrsq<A>(rsqt, i);
        __syncthreads();
        if (Ls.cv)
            cluster_steps<A, true>(Ls, Sg, nsteps, tab, smem_tab, rsq, part1, part2, h1, h2, hs, scal, shb);
        else
            cluster_steps<A, false>(Ls, Sg, nsteps, tab, smem_tab, rsq, part1, part2, h1, h2, hs, scal, shb);
    }
    cl_sync();   // no CTA leaves while another may still read its shared memory
}

// ------------------------------------------------------------ persistent step
// The same step as launch_step_t in one cooperative launch: every phase runs
// the kernels' block bodies over the same virtual block indices (so each
// slot's arithmetic, and its result, is the one of the graph replay), and a
// grid-wide barrier separates the phases.  The launch runs nsteps steps.
//
// Barrier: arrival counter + generation word.  Thread 0 of each block
// releases the block's writes, arrives, and the last arrival resets the
// counter and publishes the next generation; the others wait for it with an
// acquire load (which also drops stale L1 lines of other blocks' data).  Each
// wait gives up after limit_ns of global time: it then sets the shared error
// word and returns false, every block leaves the kernel at its next barrier,
// and the host reads the word (QS_ERR_TIMEOUT).
// Two levels: a block arrives at its group's counter (block index mod
// kBarGroups, one 128-byte line each); the last arrival of a group arrives at
// the top counter, and the last group publishes the next generation.  At most
// ceil(blocks / kBarGroups) atomics meet on one address.
constexpr int kBarGroups = 16;
struct GridBar {
    unsigned group[kBarGroups][32];
    unsigned top, gen;
    int err, pad[29];
};

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_gpu(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// `expected` blocks with indices 0..expected-1 take part (blockIdx.x is one);
// group g holds the indices i with i mod kBarGroups == g.
__device__ __noinline__ bool grid_barrier(GridBar* b, unsigned expected, unsigned long long limit_ns) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int good = 1;
        const unsigned g = ld_acquire_gpu(&b->gen);
        const unsigned grp = blockIdx.x % kBarGroups;
        const unsigned ngroups = expected < (unsigned)kBarGroups ? expected : (unsigned)kBarGroups;
        const unsigned in_grp = expected / kBarGroups + (grp < expected % kBarGroups ? 1u : 0u);
        __threadfence();
        bool last = false;
        if (atomicAdd(&b->group[grp][0], 1u) == in_grp - 1) {
            atomicExch(&b->group[grp][0], 0u);
            __threadfence();
            last = atomicAdd(&b->top, 1u) == ngroups - 1;
        }
        if (last) {
            atomicExch(&b->top, 0u);
            __threadfence();
            st_release_gpu(&b->gen, g + 1);
        } else {
            const unsigned long long t0 = global_ns();
            while (ld_acquire_gpu(&b->gen) == g) {
                if (*(volatile int*)&b->err) {
                    good = 0;
                    break;
                }
                if (global_ns() - t0 > limit_ns) {
                    atomicExch(&b->err, 1);
                    good = 0;
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
        ok = good && *(volatile int*)&b->err == 0;
    }
    __syncthreads();
    return ok != 0;
}

constexpr unsigned long long kBarrierLimitNs = 2000000000ull;   // 2 s of global time

template <class A>
__global__ void __launch_bounds__(kT, std::is_same<A, DF>::value ? 4 : 3)
    eng_persist(SlotDev* sl, const int* __restrict__ rm, const int* __restrict__ sm, double* pa, const void* rsq,
                int nrb, int nsb, int mmax, int dmax, int cgs, int ns, int nsteps, GridBar* bar,
                unsigned long long limit_ns) {
    const int nb = gridDim.x;
    const unsigned expected = gridDim.x;
    const int ydots = (dmax + jt<A>() - 1) / jt<A>();
#define QS_PHASE(count, body)                                 \
    for (int v = blockIdx.x; v < (count); v += nb) {          \
        body;                                                 \
        __syncthreads();                                      \
    }                                                         \
    if (!grid_barrier(bar, expected, limit_ns)) return;
    for (int step = 0; step < nsteps; ++step) {
        QS_PHASE(nsb, spmv_block<A>(sl, sm, rsq, v));
        QS_PHASE(nrb * ydots, dots_block<A>(sl, rm, mmax, 0, pa, v % nrb, v / nrb));
        QS_PHASE(ns * (dmax + 1), reduce_block(sl, mmax, 0, pa, dmax, v % ns, v / ns));
        QS_PHASE(nrb, update_block<A>(sl, rm, mmax, 0, pa, v));
        QS_PHASE(ns, reduce_block(sl, mmax, 1, pa, 0, v, 0));
        if (cgs) {
            QS_PHASE(ns * mmax, reduce_block(sl, mmax, 2, pa, 0, v % ns, v / ns));
            QS_PHASE(nrb, update_block<A>(sl, rm, mmax, 1, pa, v));
            QS_PHASE(ns, reduce_block(sl, mmax, 3, pa, 0, v, 0));
        }
        QS_PHASE(nrb, scale_block<A>(sl, rm, 0, v));
        if (blockIdx.x == 0)
            for (int id = threadIdx.x; id < ns; id += blockDim.x) {
                SlotDev& S = sl[id];
                if (S.state != kSlotStep) continue;
                S.j += 1;
                if (S.j >= S.m) S.state = kSlotHold;
            }
        if (!grid_barrier(bar, expected, limit_ns)) return;
    }
#undef QS_PHASE
}

// A few barriers of a cooperative grid that expects `phantom` more blocks
// than it has: with phantom > 0 the first barrier can never complete, so
// every wait runs into its limit (the bounded-wait check of the barrier).
__global__ void eng_barrier_check(GridBar* bar, int phantom, unsigned long long limit_ns, int rounds) {
    for (int r = 0; r < rounds; ++r)
        if (!grid_barrier(bar, gridDim.x + (unsigned)phantom, limit_ns)) return;
}

void Engine::launch_step() {
    const int ns = (int)slots_.size();
    const void* rsq = st_ == Store::DF ? rsqdf_.p : (st_ == Store::F32 ? rsq32_.p : rsq64_.p);
    with_store(st_, [&](auto tag) {
        using A = decltype(tag);
        step_launches_ = launch_step_t<A>(dslots_.as<SlotDev>(), dslots_.as<SlotDev>(), rmap_.as<int>(),
                                          smap_.as<int>(), partial_.as<double>(), rsq, nrb_, nsb_, mmax_, dmax_,
                                          cgs_, ns, s_);
    });
}

void Engine::capture() {
    QS_CUDA(cudaStreamBeginCapture(s_, cudaStreamCaptureModeRelaxed));
    launch_step();
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(s_, &g);
    if (e != cudaSuccess) throw Error(QS_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    graph_ = g;
    QS_CUDA(cudaGraphInstantiate(&exec_, graph_, 0));
}

void Engine::start(int id, int j) {
    SlotDev& d = slots_[id].d;
    if (j < 0 || j >= d.m) throw Error(QS_ERR_ARGUMENT, "start column outside the Krylov basis");
    d.j = j;
    d.state = kSlotStep;
    dirty_ = true;
}

int Engine::steps_to_event() const {
    int best = 0;
    for (const auto& sl : slots_)
        if (sl.live && sl.d.state == kSlotStep) {
            const int left = sl.d.m - sl.d.j;
            best = best == 0 ? left : std::min(best, left);
        }
    return best;
}

// Resident blocks of the persistent step (cooperative grid), once per device
// and storage; 0 when the device cannot run it.
static int persist_capacity(Store st) {
    static std::mutex mu;
    static std::map<std::pair<int, int>, int> cap;
    int dev = 0;
    QS_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> g(mu);
    const auto key = std::make_pair(dev, (int)st);
    auto it = cap.find(key);
    if (it != cap.end()) return it->second;
    int coop = 0, nsm = 0, per_sm = 0;
    QS_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    QS_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    with_store(st, [&](auto tag) {
        using A = decltype(tag);
        QS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, eng_persist<A>, kT, 0));
    });
    const int c = coop ? per_sm * nsm : 0;
    cap[key] = c;
    return c;
}

bool Engine::persistent_wanted() const {
    const char* e = std::getenv("QS_PERSISTENT_STEP");
    if (e && e[0] == '0') return false;
    const int cap = persist_capacity(st_);
    if (cap <= 0) return false;
    if (e && e[0] == '1') return true;
    // off unless asked for: on GB300 the graph replay measured faster at every
    // size (the launch gaps between graph nodes cost less than the barriers)
    return false;
}

void Engine::run_persistent(int nsteps) {
    const int ns = (int)slots_.size();
    const int ydots = (dmax_ + jt<double>() - 1) / jt<double>();
    // as many blocks as the widest product / vector phase has virtual blocks,
    // at most the resident capacity (fewer blocks make cheaper barriers; the
    // reductions' small virtual blocks loop)
    int widest = std::max(nsb_, nrb_ * ydots);
    const int grid = std::max(1, std::min(persist_capacity(st_), widest));
    if (!bar_.p) bar_.alloc(sizeof(GridBar));
    QS_CUDA(cudaMemsetAsync(bar_.p, 0, sizeof(GridBar), s_));
    const void* rsq = st_ == Store::DF ? rsqdf_.p : (st_ == Store::F32 ? rsq32_.p : rsq64_.p);
    SlotDev* ds = dslots_.as<SlotDev>();
    const int* rm = rmap_.as<int>();
    const int* sm = smap_.as<int>();
    double* pa = partial_.as<double>();
    GridBar* bar = bar_.as<GridBar>();
    int cgs = cgs_ ? 1 : 0;
    unsigned long long limit = kBarrierLimitNs;
    void* args[] = {&ds, &rm, &sm, &pa, &rsq, &nrb_, &nsb_, &mmax_, &dmax_, &cgs, (void*)&ns, &nsteps, &bar, &limit};
    with_store(st_, [&](auto tag) {
        using A = decltype(tag);
        QS_CUDA(cudaLaunchCooperativeKernel((const void*)eng_persist<A>, dim3(grid), dim3(kT), args, 0, s_));
    });
    ++launches_;
    GridBar h{};
    QS_CUDA(cudaMemcpyAsync(&h, bar_.p, sizeof(GridBar), cudaMemcpyDeviceToHost, s_));
    QS_CUDA(cudaStreamSynchronize(s_));
    if (h.err) throw Error(QS_ERR_TIMEOUT, "a grid barrier of the persistent Lanczos step timed out");
}

void grid_barrier_check(int phantom, double limit_ms, int blocks) {
    if (phantom < 0 || blocks < 1 || !(limit_ms > 0) || limit_ms > 2000)
        throw Error(QS_ERR_ARGUMENT, "phantom >= 0, blocks >= 1 and 0 < limit_ms <= 2000 required");
    int dev = 0, coop = 0, nsm = 0, per_sm = 0;
    QS_CUDA(cudaGetDevice(&dev));
    QS_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    QS_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    QS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, eng_barrier_check, kT, 0));
    if (!coop || blocks > per_sm * nsm) throw Error(QS_ERR_UNSUPPORTED, "cooperative grid too large for this device");
    cudaStream_t s = nullptr;
    QS_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    DevBuf bar(sizeof(GridBar));
    GridBar h{};
    cudaError_t e = cudaMemsetAsync(bar.p, 0, sizeof(GridBar), s);
    GridBar* b = bar.as<GridBar>();
    unsigned long long limit = (unsigned long long)(limit_ms * 1e6);
    int rounds = 8;
    void* args[] = {&b, &phantom, &limit, &rounds};
    if (e == cudaSuccess)
        e = cudaLaunchCooperativeKernel((const void*)eng_barrier_check, dim3(blocks), dim3(kT), args, 0, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, bar.p, sizeof(GridBar), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    if (e != cudaSuccess) throw Error(QS_ERR_CUDA, cudaGetErrorString(e));
    note_launches(1);
    if (h.err) throw Error(QS_ERR_TIMEOUT, "grid barrier wait ran out");
    if (h.gen != (unsigned)rounds) throw Error(QS_ERR_CUDA, "grid barrier completed a wrong number of rounds");
}

// Which stepping slots take the cluster step, and with how many CTAs: by the
// slot's own size only, so that a slot's result is the same alone and in any
// batch.  Measured on GB300 against the graph replay: eight CTAs per slot
// 1.3-2.2x faster for slots of 700 to 9,300 rows; sixteen CTAs for 8,400 to
// 29,000 rows (1.9x at 8,400, 1.23x at 29,000 rows alone, even for the 22
// sectors of J1-J2 L=22 at 32,000 rows); larger slots are faster on the graph
// replay (0.6-0.7x for the 26 sectors of L=24 at 104,000 rows), whose kernels
// spread a slot over the whole GPU.
constexpr int64_t kClusterRows8 = 8192, kClusterRows16 = 32768;

int Engine::cluster_size_for(const SlotDev& d) const {
    const char* e = std::getenv("QS_CLUSTER_STEP");
    if (e && e[0] == '0') return 0;
    if (!(e && e[0] == '1') && persistent_wanted()) return 0;
    if (d.n <= kClusterRows8) return 8;
    if (d.n <= kClusterRows16 || (e && e[0] == '1')) return cluster16_ok() ? 16 : 8;
    return 0;
}

// Sixteen CTAs per cluster are a non-portable size: allowed per kernel, and
// used where the device can place such a cluster
bool Engine::cluster16_ok() const {
    static std::mutex mu;
    static std::map<std::pair<int, int>, bool> ok;
    int dev = 0;
    QS_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> g(mu);
    const auto key = std::make_pair(dev, (int)st_);
    auto it = ok.find(key);
    if (it != ok.end()) return it->second;
    bool good = false;
    with_store(st_, [&](auto tag) {
        using A = decltype(tag);
        if (cudaFuncSetAttribute(eng_cluster<A>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
            cudaGetLastError();
            return;
        }
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(16);
        cfg.blockDim = dim3(kT);
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = 16;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int nclusters = 0;
        if (cudaOccupancyMaxActiveClusters(&nclusters, eng_cluster<A>, &cfg) == cudaSuccess) good = nclusters > 0;
        else cudaGetLastError();
    });
    ok[key] = good;
    return good;
}

void Engine::run_cluster(const std::vector<int>& ids, int nsteps, int C, cudaStream_t st) {
    if (ids.empty()) return;
    // one map per cluster size: [0, half) for eight CTAs, [half, ...) for sixteen
    const size_t half = slots_.size();
    if (2 * half * sizeof(int) > cap_cmap_) {
        cap_cmap_ = std::max<size_t>(64, 2 * half * sizeof(int) * 2);
        cmap_.alloc(cap_cmap_);
    }
    int* cmd = cmap_.as<int>() + (C == 16 ? half : 0);
    QS_CUDA(cudaMemcpyAsync(cmd, ids.data(), ids.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    const void* rsq = st_ == Store::DF ? rsqdf_.p : (st_ == Store::F32 ? rsq32_.p : rsq64_.p);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(ids.size() * C));
    cfg.blockDim = dim3(kT);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    SlotDev* ds = dslots_.as<SlotDev>();
    const int* cm = cmd;
    with_store(st_, [&](auto tag) {
        using A = decltype(tag);
        QS_CUDA(cudaLaunchKernelEx(&cfg, eng_cluster<A>, ds, cm, nsteps, rsq));
    });
    ++launches_;
}

void Engine::run(int nsteps) {
    if (nsteps <= 0) return;
    // small slots step in the cluster step, marked so that the graph-replayed
    // kernels skip them; the others in the graph replay (or the persistent step)
    std::vector<int> cl8, cl16;
    bool rest = false;
    for (int i = 0; i < (int)slots_.size(); ++i) {
        Slot& sl = slots_[i];
        if (!sl.live || sl.d.state != kSlotStep) continue;
        const int C = cluster_size_for(sl.d);
        if (C) {
            sl.d.state = kSlotStepCluster;
            (C == 16 ? cl16 : cl8).push_back(i);
            dirty_ = true;
        } else {
            rest = true;
        }
    }
    const bool cl = !cl8.empty() || !cl16.empty();
    sync_table();
    if (nrb_ == 0) return;
    // with large slots too, the cluster step runs on the side stream beside
    // their graph replay (the two touch different slots and partial rows);
    // never beside the cooperative step, whose blocks must all be resident
    cudaStream_t cs = s_;
    if (cl && rest && !persistent_wanted()) {
        if (!side_) {
            QS_CUDA(cudaStreamCreateWithFlags(&side_, cudaStreamNonBlocking));
            QS_CUDA(cudaEventCreateWithFlags(&fork_, cudaEventDisableTiming));
            QS_CUDA(cudaEventCreateWithFlags(&join_, cudaEventDisableTiming));
        }
        QS_CUDA(cudaEventRecord(fork_, s_));
        QS_CUDA(cudaStreamWaitEvent(side_, fork_, 0));
        cs = side_;
    }
    run_cluster(cl8, nsteps, 8, cs);
    run_cluster(cl16, nsteps, 16, cs);
    if (rest) {
        if (!exec_ && !persistent_wanted()) capture();
        if (persistent_wanted()) {
            run_persistent(nsteps);
        } else {
            for (int t = 0; t < nsteps; ++t) QS_CUDA(cudaGraphLaunch(exec_, s_));
            launches_ += step_launches_ * (int64_t)nsteps;
        }
    }
    if (cs != s_) {
        QS_CUDA(cudaEventRecord(join_, side_));
        QS_CUDA(cudaStreamWaitEvent(s_, join_, 0));
    }
    // mirror the device step counters (the cluster step leaves its slots in
    // kSlotStepCluster or Hold on the device; the next table upload restores Step)
    for (auto& sl : slots_) {
        if (!sl.live || (sl.d.state != kSlotStep && sl.d.state != kSlotStepCluster)) continue;
        const int adv = std::min(nsteps, sl.d.m - sl.d.j);
        sl.d.j += adv;
        sl.matvecs += adv;
        sl.d.state = sl.d.j >= sl.d.m ? kSlotHold : kSlotStep;
        dirty_ = dirty_ || cl;
    }
}

void Engine::seed(int id, uint64_t sd) {
    const SlotDev& d = slots_[id].d;
    fill_normal(d.V, store_kind(st_, d.cv), d.n, sd, s_);
    ++launches_;
}

void Engine::load(int id, int col, const double* v, bool device) {
    const SlotDev& d = slots_[id].d;
    const VKind k64 = d.cv ? VKind::C128 : VKind::F64;
    const VKind ks = store_kind(st_, d.cv);
    const size_t bytes = (size_t)d.n * (d.cv ? 16 : 8);   // FP64 input
    char* dst = (char*)d.V + (size_t)col * d.n * store_bytes(st_, d.cv);
    PoolBuf st;
    const void* src = v;
    if (!device) {
        st.alloc(bytes, s_);
        QS_CUDA(cudaMemcpyAsync(st.p, v, bytes, cudaMemcpyHostToDevice, s_));
        src = st.p;
    }
    convert_vec(src, k64, dst, ks, d.n, s_);
    ++launches_;
    QS_CUDA(cudaStreamSynchronize(s_));
}

void Engine::store(int id, int col, double* out, bool device) {
    const SlotDev& d = slots_[id].d;
    const VKind k64 = d.cv ? VKind::C128 : VKind::F64;
    const VKind ks = store_kind(st_, d.cv);
    const size_t bytes = (size_t)d.n * (d.cv ? 16 : 8);   // FP64 output
    const char* src = (const char*)d.V + (size_t)col * d.n * store_bytes(st_, d.cv);
    if (device) {
        convert_vec(src, ks, out, k64, d.n, s_);
    } else {
        PoolBuf st(bytes, s_);
        convert_vec(src, ks, st.p, k64, d.n, s_);
        QS_CUDA(cudaMemcpyAsync(out, st.p, bytes, cudaMemcpyDeviceToHost, s_));
    }
    ++launches_;
    QS_CUDA(cudaStreamSynchronize(s_));
}

std::vector<double> Engine::normalize(const std::vector<int>& ids, int col, bool scale) {
    std::vector<int> saved(ids.size());
    for (size_t q = 0; q < ids.size(); ++q) {
        SlotDev& d = slots_[ids[q]].d;
        if (col < 0 || col > d.m) throw Error(QS_ERR_ARGUMENT, "normalised column outside the Krylov basis");
        saved[q] = d.state;
        d.state = kSlotNormalize;
        d.ncol = col;
    }
    dirty_ = true;
    sync_table();
    const SlotDev* ds = dslots_.as<SlotDev>();
    const int* rm = rmap_.as<int>();
    double* pa = partial_.as<double>();
    const int ns = (int)slots_.size();
    if (nrb_ > 0 && !ids.empty()) {
        with_store(st_, [&](auto tag) {
            using A = decltype(tag);
            eng_dots<A><<<dim3(nrb_, 1), kT, 0, s_>>>(ds, rm, mmax_, 2, pa);
            eng_reduce<<<dim3(ns, 1), kT, 0, s_>>>(ds, mmax_, 4, pa);
            if (scale) eng_scale<A><<<nrb_, kT, 0, s_>>>(ds, rm, 1);
        });
        QS_CUDA(cudaGetLastError());
        launches_ += scale ? 3 : 2;
    }
    std::vector<double> out(ids.size());
    for (size_t q = 0; q < ids.size(); ++q)
        QS_CUDA(cudaMemcpyAsync(&out[q], slots_[ids[q]].d.nrm + 2, sizeof(double), cudaMemcpyDeviceToHost, s_));
    QS_CUDA(cudaStreamSynchronize(s_));
    for (size_t q = 0; q < ids.size(); ++q) slots_[ids[q]].d.state = saved[q];
    dirty_ = true;
    return out;
}

void Engine::rotate(const std::vector<RotReq>& reqs) {
    if (reqs.empty()) return;
    // every slot's coefficients in the storage's complex format (double2,
    // float4 hi/lo pairs, or float2), packed into one upload
    const size_t eb = st_ == Store::F32 ? 8 : 16;
    size_t total = 0;
    for (const RotReq& R : reqs) total += R.Y.size();
    if (total * eb > cap_y_) {
        cap_y_ = std::max<size_t>(total * eb * 2, 1 << 16);
        QS_CUDA(cudaStreamSynchronize(s_));
        ybuf_.alloc(cap_y_);
    }
    std::vector<double> c64;
    std::vector<float> c32;
    if (st_ == Store::F64) c64.resize(2 * total);
    else c32.resize((st_ == Store::DF ? 4 : 2) * total);
    std::vector<int> saved(reqs.size());
    size_t off = 0;
    bool any_tc = false;
    for (size_t q = 0; q < reqs.size(); ++q) {
        const RotReq& R = reqs[q];
        Slot& sl = slots_[R.id];
        SlotDev& d = sl.d;
        const bool bad = R.nin < 0 || R.nin > d.m || R.p < 0 || R.p > sl.tcols || (R.p > 0 && R.nin < 1) ||
                         R.out0 < 0 || R.out0 + R.p > d.m + 1 || R.Y.size() != (size_t)R.nin * R.p ||
                         (R.carry >= 0 && (R.carry > d.m || R.cdst < 0 || R.cdst > d.m));
        if (bad) throw Error(QS_ERR_ARGUMENT, "rotation shape outside the Krylov basis");
        bool yreal = true;
        for (size_t i = 0; i < R.Y.size(); ++i) {
            const double re = R.Y[i].real(), im = R.Y[i].imag();
            const size_t e = off + i;
            if (im != 0.0) yreal = false;
            if (st_ == Store::DF) {
                df_split_host(re, c32[4 * e], c32[4 * e + 1]);
                df_split_host(im, c32[4 * e + 2], c32[4 * e + 3]);
            } else if (st_ == Store::F32) {
                c32[2 * e] = (float)re;
                c32[2 * e + 1] = (float)im;
            } else {
                c64[2 * e] = re;
                c64[2 * e + 1] = im;
            }
        }
        // the tensor-core path: real coefficients |Y| <= 1 (the Ritz vectors of
        // a thick restart), 2 <= p <= 16 outputs, at most 32 inputs
        double ymax = 0.0;
        for (const cd& v : R.Y) ymax = std::max(ymax, std::abs(v.real()));
        // (the double-float rotation runs on the FP32 pipe near its memory
        // bound, and measured no slower than the tensor-core form: only the
        // FP64 storage takes it)
        const bool tc = tc_rotate_ && st_ == Store::F64 && yreal && R.p >= 2 && R.p <= 16 && R.nin >= 1 &&
                        R.nin <= 32 && ymax <= 1.0 + 1e-9;
        any_tc = any_tc || tc;
        saved[q] = d.state;
        d.state = kSlotRotate;
        d.rot_tc = tc ? 1 : 0;
        d.y = (char*)ybuf_.p + off * eb;
        d.yreal = yreal;
        d.rot_in = R.nin;
        d.p = R.p;
        d.out0 = R.out0;
        d.carry = R.carry;
        d.cdst = R.cdst;
        off += R.Y.size();
    }
    if (total)
        QS_CUDA(cudaMemcpyAsync(ybuf_.p, st_ == Store::F64 ? (const void*)c64.data() : (const void*)c32.data(),
                                total * eb, cudaMemcpyHostToDevice, s_));
    dirty_ = true;
    sync_table();
    if (nrb_ > 0) {
        with_store(st_, [&](auto tag) {
            using A = decltype(tag);
            eng_rotate<A><<<nrb_, kT, 0, s_>>>(dslots_.as<SlotDev>(), rmap_.as<int>());
        });
        QS_CUDA(cudaGetLastError());
        ++launches_;
        if (any_tc) {
            // the shared-memory size, once per device
            static thread_local int attr_dev = -1;
            int dev = 0;
            QS_CUDA(cudaGetDevice(&dev));
            if (attr_dev != dev) {
                QS_CUDA(cudaFuncSetAttribute(eng_rotate_tc<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)kTcSmem));
                attr_dev = dev;
            }
            // at least two blocks per SM: row blocks split into shares
            int nsm = 152;
            QS_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
            const int split = std::max(1, std::min(8, (2 * nsm + nrb_ - 1) / std::max(1, nrb_)));
            eng_rotate_tc<double><<<dim3(nrb_, split), kTcRows, kTcSmem, s_>>>(dslots_.as<SlotDev>(), rmap_.as<int>(),
                                                                   tc_err_.as<int>());
            QS_CUDA(cudaGetLastError());
            ++launches_;
            int err = 0;
            QS_CUDA(cudaMemcpyAsync(&err, tc_err_.p, sizeof(int), cudaMemcpyDeviceToHost, s_));
            QS_CUDA(cudaStreamSynchronize(s_));
            if (err) {
                QS_CUDA(cudaMemsetAsync(tc_err_.p, 0, sizeof(int), s_));
                throw Error(QS_ERR_TIMEOUT, "the tensor-core rotation timed out waiting for its MMAs");
            }
        }
    }
    for (size_t q = 0; q < reqs.size(); ++q) {
        SlotDev& d = slots_[reqs[q].id].d;
        d.state = saved[q] == kSlotRotate ? kSlotIdle : saved[q];
        d.carry = -1;
        d.p = 0;
        d.rot_tc = 0;
    }
    dirty_ = true;
}

void Engine::record(int id, std::vector<cd>& H) {
    std::vector<std::vector<cd>> all;
    records({id}, all);
    H = std::move(all[0]);
}

void Engine::records(const std::vector<int>& ids, std::vector<std::vector<cd>>& H) {
    H.assign(ids.size(), {});
    for (size_t q = 0; q < ids.size(); ++q) {
        const SlotDev& d = slots_[ids[q]].d;
        H[q].resize((size_t)(d.m + 1) * d.m);   // std::complex<double> is two doubles
        QS_CUDA(cudaMemcpyAsync(H[q].data(), d.rec, H[q].size() * sizeof(cd), cudaMemcpyDeviceToHost, s_));
    }
    QS_CUDA(cudaStreamSynchronize(s_));
}

// ================================================================ eigsh task
void EigTask::init(int k_, int which_, double tol_, int m_, int maxiter_) {
    k = k_;
    which = which_;
    m = m_;
    tol = tol_ > 0 ? tol_ : 2.220446049250313e-16;
    maxiter = maxiter_ > 0 ? maxiter_ : 300;
    p = std::max(std::min(m - 2, k + (m - k) / 2), std::min(k, m - 1));
    T.assign((size_t)m * m, 0.0);
    theta.assign(k, 0.0);
    beta = maxrel = 0;
    nconv = restarts = j0 = 0;
}

bool EigTask::on_hold(const std::vector<cd>& H, int id, RotReq& rot) {
    static const double eps23 = std::pow(2.220446049250313e-16, 2.0 / 3.0);
    for (int j = j0; j < m; ++j) {
        T[(size_t)j * m + j] = H[(size_t)j * (m + 1) + j].real();
        const double b = H[(size_t)j * (m + 1) + j + 1].real();
        if (j + 1 < m) T[(size_t)j * m + j + 1] = T[(size_t)(j + 1) * m + j] = b;
        else beta = b;
    }
    std::vector<double> w, Y;
    sym_eig(m, T, w, Y);
    const std::vector<int> order = ritz_order(w, which, k);
    int nc = 0;
    double mr = 0;
    for (int q = 0; q < k; ++q) {
        const int c = order[q];
        const double bound = std::fabs(beta * Y[(size_t)(m - 1) * m + c]);
        mr = std::max(mr, bound / std::max(eps23, std::fabs(w[c])));
        if (bound <= tol * std::max(eps23, std::fabs(w[c]))) ++nc;
    }
    nconv = nc;
    maxrel = mr;
    for (int q = 0; q < k; ++q) theta[q] = w[order[q]];
    const bool fin = nc >= k || restarts >= maxiter - 1;
    const int keep = fin ? k : p;
    rot.id = id;
    rot.Y.assign((size_t)m * keep, cd(0, 0));
    for (int q = 0; q < keep; ++q)
        for (int r = 0; r < m; ++r) rot.Y[(size_t)q * m + r] = cd(Y[(size_t)r * m + order[q]], 0.0);
    rot.nin = m;
    rot.p = keep;
    rot.out0 = 0;
    rot.carry = fin ? -1 : m;   // thick restart: the residual direction follows the Ritz vectors
    rot.cdst = keep;
    if (!fin) {
        std::fill(T.begin(), T.end(), 0.0);
        for (int q = 0; q < p; ++q) {
            T[(size_t)q * m + q] = w[order[q]];
            const double c = beta * Y[(size_t)(m - 1) * m + order[q]];
            T[(size_t)q * m + p] = T[(size_t)p * m + q] = c;
        }
        j0 = p;
        ++restarts;
    }
    return fin;
}

// ================================================================ batched eigsh
// Thick-restart Lanczos (the iteration of eigsh in qs_krylov.cu) on every
// operator at once; values: nops * k per operator, in the order of `which`
// (ritz_order).
void eigsh_batch(Op** ops, int nops, const qs_eigsh_opts& o, double* values, void** vectors, qs_eigsh_info* infos) {
    auto t0 = std::chrono::steady_clock::now();
    if (nops <= 0) throw Error(QS_ERR_ARGUMENT, "no operators");
    const int k = o.k;
    if (o.which < 0 || o.which > 4) throw Error(QS_ERR_ARGUMENT, "which must be SA, LA, SM, LM, or BE");
    int m = o.ncv > 0 ? o.ncv : std::max(20, 2 * k + 1);
    m = std::min(m, kMaxM);
    for (int i = 0; i < nops; ++i) {
        Op& op = *ops[i];
        if (!op.hermitian) throw Error(QS_ERR_UNSUPPORTED, "eigsh on this engine needs Hermitian operators");
        const int64_t n = op.basis->n;
        if (k < 1 || k >= n - 1) throw Error(QS_ERR_ARGUMENT, "batched eigsh needs 1 <= k < Ns - 1 for every operator");
        m = (int)std::min<int64_t>(m, n);
    }
    if (m <= k) throw Error(QS_ERR_ARGUMENT, "ncv must exceed k");
    const bool fp32 = o.precision == 1;
    Engine E(o.precision == 0 ? Store::F64 : (fp32 ? Store::F32 : Store::DF), ops[0]->stream);
    std::vector<int> id(nops);
    std::vector<EigTask> task(nops);
    const bool dev = o.mem == QS_MEM_DEVICE;
    // the FP32 form converges to what FP32 vectors resolve, then an FP64 polish
    const double tol_run = fp32 ? std::max(o.tol > 0 ? o.tol : 2.220446049250313e-16, 2e-6) : o.tol;
    for (int i = 0; i < nops; ++i) {
        id[i] = E.add(*ops[i], m, ops[i]->complex_mat);
        if (o.v0 && nops == 1) E.load(id[i], 0, o.v0, dev);   // a start vector only for a single operator
        else E.seed(id[i], 20261203ull);
        task[i].init(k, o.which, tol_run, m, o.maxiter);
    }
    std::vector<PoolBuf> promoted(fp32 ? nops : 0);   // FP64 Ritz vectors of the FP32 form
    E.normalize(id);
    for (int i = 0; i < nops; ++i) E.start(id[i], 0);
    std::vector<char> done(nops, 0);
    int left = nops;
    while (left > 0) {
        const int steps = E.steps_to_event();
        if (steps <= 0) throw Error(QS_ERR_CUDA, "batched eigsh lost its stepping slots");
        E.run(steps);
        std::vector<RotReq> rot;
        std::vector<int> fin, hold, hold_ids;
        for (int i = 0; i < nops; ++i)
            if (!done[i] && E.slot(id[i]).state == kSlotHold) {
                hold.push_back(i);
                hold_ids.push_back(id[i]);
            }
        std::vector<std::vector<cd>> H;
        E.records(hold_ids, H);
        for (size_t q = 0; q < hold.size(); ++q) {
            const int i = hold[q];
            RotReq R;
            if (task[i].on_hold(H[q], id[i], R)) fin.push_back(i);
            rot.push_back(std::move(R));
        }
        E.rotate(rot);
        for (const RotReq& R : rot)
            if (R.carry >= 0) E.start(R.id, task[0].p);
        for (int i : fin) {
            const EigTask& t = task[i];
            done[i] = 1;
            --left;
            if (t.nconv < k) throw Error(QS_ERR_NOT_CONVERGED, "batched eigsh did not converge within maxiter restarts");
            for (int q = 0; q < k; ++q) values[(size_t)i * k + q] = t.theta[q];
            const int64_t n = ops[i]->basis->n;
            const int comps = ops[i]->complex_mat ? 2 : 1;
            if (fp32) {
                promoted[i].alloc((size_t)k * n * comps * sizeof(double), E.stream());
                for (int q = 0; q < k; ++q) E.store(id[i], q, promoted[i].as<double>() + (size_t)q * n * comps, true);
            } else if (vectors && vectors[i]) {
                for (int q = 0; q < k; ++q) E.store(id[i], q, (double*)vectors[i] + (size_t)q * n * comps, dev);
            }
            if (infos) {
                infos[i].nconv = t.nconv;
                infos[i].restarts = t.restarts;
                infos[i].matvecs = E.matvecs(id[i]);
                infos[i].max_rel_residual = t.maxrel;
                infos[i].seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            }
            // parked, not removed: removing would rebuild the block maps and
            // recapture the step graph; the slot's blocks exit at once
            E.slot_mut(id[i]).state = kSlotIdle;
        }
    }
    for (int i = 0; i < nops; ++i) E.remove(id[i]);
    QS_CUDA(cudaStreamSynchronize(E.stream()));
    note_launches(E.launches());
    if (!fp32) return;
    // FP64 polish of the FP32 form: the Rayleigh quotient of every promoted Ritz
    // vector with the FP64 product; where the quadratic bound ||r||^2 / gap
    // misses the tolerance, a double-float thick-restart solve from the
    // promoted ground vector finishes the job
    const double tol = o.tol > 0 ? o.tol : 2.220446049250313e-16;
    const double eps23 = std::pow(2.220446049250313e-16, 2.0 / 3.0);
    for (int i = 0; i < nops; ++i) {
        Op& op = *ops[i];
        const int64_t n = op.basis->n;
        const bool cpx = op.complex_mat;
        const int comps = cpx ? 2 : 1;
        const VKind k64 = cpx ? VKind::C128 : VKind::F64;
        Blas B(k64, n, op.stream);
        PoolBuf Ax((size_t)n * comps * sizeof(double), op.stream);
        std::vector<double> th(k);
        bool refine = false;
        double maxrel = 0;
        for (int q = 0; q < k; ++q) {
            double* xq = promoted[i].as<double>() + (size_t)q * n * comps;
            const double nx = B.norm(xq);
            B.scale(xq, xq, cd(1.0 / nx, 0));
            MatvecCall c;
            c.x = xq;
            c.y = Ax.p;
            c.x_complex = c.y_complex = cpx;
            op_matvec_device(op, c, op.stream);
            th[q] = B.dot(xq, Ax.p).real();
            B.axpy(Ax.p, xq, cd(-th[q], 0));
            const double rn = B.norm(Ax.p);
            double gap = 1e300;
            for (int q2 = 0; q2 < k; ++q2)
                if (q2 != q) gap = std::min(gap, std::fabs(values[(size_t)i * k + q2] - th[q]));
            if (gap == 1e300) gap = std::max(1e-300, std::fabs(th[q]));
            maxrel = std::max(maxrel, rn / std::max(eps23, std::fabs(th[q])));
            if (rn * rn / gap > tol * std::max(1.0, std::fabs(th[q]))) refine = true;
        }
        if (refine) {
            qs_eigsh_opts r = o;
            r.precision = 2;
            r.v0 = promoted[i].as<double>();
            r.mem = QS_MEM_DEVICE;
            r.want_vectors = vectors && vectors[i];
            std::vector<double> vals(k);
            void* vec = (vectors && vectors[i]) ? vectors[i] : nullptr;
            PoolBuf vdev;
            if (vec && !dev) {
                vdev.alloc((size_t)k * n * comps * sizeof(double), op.stream);
                vec = vdev.p;
            }
            qs_eigsh_info inf{};
            Op* one = &op;
            eigsh_batch(&one, 1, r, vals.data(), vec ? &vec : nullptr, &inf);
            for (int q = 0; q < k; ++q) values[(size_t)i * k + q] = vals[q];
            if (vectors && vectors[i] && !dev)
                QS_CUDA(cudaMemcpy(vectors[i], vdev.p, vdev.bytes, cudaMemcpyDeviceToHost));
            if (infos) {
                infos[i].matvecs += inf.matvecs;
                infos[i].restarts += inf.restarts;
                infos[i].max_rel_residual = inf.max_rel_residual;
            }
        } else {
            for (int q = 0; q < k; ++q) values[(size_t)i * k + q] = th[q];
            if (vectors && vectors[i])
                QS_CUDA(cudaMemcpyAsync(vectors[i], promoted[i].p, promoted[i].bytes,
                                        dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, op.stream));
            if (infos) {
                infos[i].matvecs += k;
                infos[i].max_rel_residual = maxrel;
            }
        }
        QS_CUDA(cudaStreamSynchronize(op.stream));
        if (infos) infos[i].seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
}

// ================================================================ Krylov exponential
void krylov_project(const std::vector<cd>& H, int m, bool hermitian, cd scale, int& c, std::vector<cd>& coef,
                    double& terminal) {
    const int ld = m + 1;
    auto h = [&](int i, int j) { return H[(size_t)j * ld + i]; };
    // completed steps: the reference stops when the new norm is below
    // 100 eps max(1, ||H||_F) of the Hessenberg matrix built so far
    c = m;
    double hn2 = 0;
    for (int j = 0; j < m; ++j) {
        const double tn = std::abs(h(j + 1, j));
        if (hermitian) {
            hn2 += std::norm(h(j, j)) + tn * tn + (j < m - 1 ? tn * tn : 0.0);
        } else {
            for (int i = 0; i <= j; ++i) hn2 += std::norm(h(i, j));
            hn2 += tn * tn;
        }
        if (tn <= 100 * 2.220446049250313e-16 * std::max(1.0, std::sqrt(hn2))) {
            c = j + 1;
            break;
        }
    }
    terminal = std::abs(h(c, c - 1));
    coef.assign(c, cd(0, 0));
    if (hermitian) {
        std::vector<double> T((size_t)c * c, 0.0), w, U;
        for (int i = 0; i < c; ++i) {
            T[(size_t)i * c + i] = h(i, i).real();
            if (i + 1 < c) T[(size_t)i * c + i + 1] = T[(size_t)(i + 1) * c + i] = h(i + 1, i).real();
        }
        sym_eig(c, T, w, U);
        for (int r = 0; r < c; ++r) {
            cd acc(0, 0);
            for (int q = 0; q < c; ++q) acc += U[(size_t)r * c + q] * (std::exp(scale * w[q]) * U[q]);
            coef[r] = acc;
        }
    } else {
        std::vector<cd> A((size_t)c * c), E;
        for (int i = 0; i < c; ++i)
            for (int j = 0; j < c; ++j) A[(size_t)i * c + j] = scale * h(i, j);
        expm_complex(c, A, E);
        for (int r = 0; r < c; ++r) coef[r] = E[(size_t)r * c];
    }
}

void EvoTask::init(int m_, int64_t n_, bool herm, cd scale, double tol, double beta0, bool split) {
    m = m_;
    n = n_;
    hermitian = herm;
    beta = beta0;
    err = 0;
    halvings = 0;
    segs.clear();
    if (beta0 == 0 || scale == cd(0, 0)) return;
    if (split) {
        segs.push_back(Seg{scale / 2.0, tol / 2, 1});
        segs.push_back(Seg{scale / 2.0, tol / 2, 1});
        halvings = 1;
    } else {
        segs.push_back(Seg{scale, tol, 0});
    }
}

void EvoTask::on_hold(const std::vector<cd>& Hrec, int id, RotReq& rot) {
    H = Hrec;
    project(id, rot);
}

void EvoTask::project(int id, RotReq& rot) {
    const Seg sg = segs.front();
    int c;
    std::vector<cd> coef;
    double terminal;
    krylov_project(H, m, hermitian, sg.scale, c, coef, terminal);
    rot = RotReq();
    rot.id = id;
    rot.nin = c;
    rot.p = 1;
    rot.out0 = m;   // the candidate goes to column m; column 0 keeps the segment's start
    rot.Y.resize(c);
    for (int i = 0; i < c; ++i) rot.Y[i] = coef[i] * beta;
    const bool est_on = c == m && m < n;
    err = est_on ? std::abs(sg.scale) * terminal * beta * std::abs(coef[c - 1]) : 0.0;
}

int EvoTask::after_norm(double nr, int id, RotReq& copy) {
    const Seg sg = segs.front();
    if (err <= sg.tol * std::max(1.0, nr)) {
        segs.pop_front();
        beta = nr;
        copy = RotReq();
        copy.id = id;
        copy.carry = m;
        copy.cdst = 0;
        return 1;
    }
    if (sg.depth >= 14) return -1;
    segs.pop_front();
    segs.push_front(Seg{sg.scale / 2.0, sg.tol / 2, sg.depth + 1});
    segs.push_front(Seg{sg.scale / 2.0, sg.tol / 2, sg.depth + 1});
    ++halvings;
    return 0;
}

// Runs EvoTasks on their slots until all are done; out_cols[i] receives
// beta * column 0 (host, Ns complex) of task i.
// Runs the EvoTasks of the listed slots to completion and writes beta * the
// accepted state of each to outs (host, or device with `device`).  Slots may
// have different Krylov sizes (different operators).
static void run_evo_slots(Engine& E, std::vector<int>& ids, std::vector<EvoTask>& tasks,
                          const std::vector<double*>& outs, bool device = false) {
    const size_t nt = tasks.size();
    std::vector<char> fin(nt, 0);
    size_t left = 0;
    for (size_t i = 0; i < nt; ++i) {
        if (tasks[i].done()) fin[i] = 1;
        else {
            E.start(ids[i], 0);
            ++left;
        }
    }
    auto emit = [&](size_t i) {
        const int64_t n = tasks[i].n;
        const double b = tasks[i].beta;
        if (device) {
            E.store(ids[i], 0, outs[i], true);
            Blas B(VKind::C128, n, E.stream());
            B.scale(outs[i], outs[i], cd(b, 0));
            QS_CUDA(cudaStreamSynchronize(E.stream()));
            return;
        }
        E.store(ids[i], 0, outs[i], false);
        for (int64_t q = 0; q < 2 * n; ++q) outs[i][q] *= b;
    };
    for (size_t i = 0; i < nt; ++i)
        if (fin[i]) emit(i);
    while (left > 0) {
        const int steps = E.steps_to_event();
        if (steps <= 0) throw Error(QS_ERR_CUDA, "Krylov exponential lost its stepping slots");
        E.run(steps);
        std::vector<size_t> hold;
        std::vector<int> hold_ids;
        for (size_t i = 0; i < nt; ++i)
            if (!fin[i] && E.slot(ids[i]).state == kSlotHold) {
                hold.push_back(i);
                hold_ids.push_back(ids[i]);
            }
        std::vector<std::vector<cd>> H;
        E.records(hold_ids, H);
        std::vector<RotReq> rot(hold.size());
        for (size_t q = 0; q < hold.size(); ++q) tasks[hold[q]].on_hold(H[q], ids[hold[q]], rot[q]);
        std::vector<size_t> proj = hold, done_now, restart;
        // project, measure, decide; rejected slots project their half step from
        // the same basis until every slot is accepted
        while (!proj.empty()) {
            E.rotate(rot);
            // the candidates sit in column m of each slot: one normalisation per Krylov size
            std::vector<double> nr(proj.size());
            std::map<int, std::vector<size_t>> by_m;
            for (size_t q = 0; q < proj.size(); ++q) by_m[tasks[proj[q]].m].push_back(q);
            for (const auto& kv : by_m) {
                std::vector<int> pid;
                for (size_t q : kv.second) pid.push_back(ids[proj[q]]);
                const std::vector<double> g = E.normalize(pid, kv.first);
                for (size_t t = 0; t < kv.second.size(); ++t) nr[kv.second[t]] = g[t];
            }
            std::vector<RotReq> copies, next_rot;
            std::vector<size_t> next;
            for (size_t q = 0; q < proj.size(); ++q) {
                const size_t i = proj[q];
                RotReq cp;
                const int r = tasks[i].after_norm(nr[q], ids[i], cp);
                if (r < 0)
                    throw Error(QS_ERR_NOT_CONVERGED, "Krylov exponential action did not converge; increase krylov_dim");
                if (r == 1) {
                    copies.push_back(std::move(cp));
                    (tasks[i].done() ? done_now : restart).push_back(i);
                } else {
                    RotReq R;
                    tasks[i].project(ids[i], R);
                    next_rot.push_back(std::move(R));
                    next.push_back(i);
                }
            }
            E.rotate(copies);
            rot.swap(next_rot);
            proj.swap(next);
        }
        for (size_t i : done_now) {
            emit(i);
            fin[i] = 1;
            --left;
            E.remove(ids[i]);
        }
        for (size_t i : restart) E.start(ids[i], 0);
    }
}

void evolve_engine(Op& op, const double* v0, const std::vector<cd>& scales, double tol, int krylov_dim, int precision,
                   bool normalise, double* out) {
    const int64_t n = op.basis->n;
    const int nt = (int)scales.size();
    if (nt == 0) return;
    const int m = (int)std::min<int64_t>(std::min(krylov_dim, kMaxM), n);
    if (m < 2) throw Error(QS_ERR_UNSUPPORTED, "the engine needs a Krylov dimension of at least 2");
    const bool herm = op.hermitian;
    const int orth = herm ? 2 : 0;
    auto copy_v0 = [&](int i) { std::copy(v0, v0 + 2 * n, out + (size_t)i * 2 * n); };
    Engine E(precision == 0 ? Store::F64 : Store::DF, op.stream);
    // one factorisation from v0 serves every time whose estimate passes
    const int f = E.add(op, m, true, true, 1, orth);
    E.load(f, 0, v0, false);
    const double beta = E.normalize({f})[0];
    bool all_zero = true;
    for (const cd& sc : scales) all_zero = all_zero && sc == cd(0, 0);
    if (beta == 0 || all_zero) {
        for (int i = 0; i < nt; ++i) copy_v0(i);
        return;
    }
    E.start(f, 0);
    E.run(m);
    std::vector<cd> H;
    E.record(f, H);
    std::vector<int> failing;
    for (int i = 0; i < nt; ++i) {
        if (scales[i] == cd(0, 0)) {
            copy_v0(i);
            continue;
        }
        int c;
        std::vector<cd> coef;
        double terminal;
        krylov_project(H, m, herm, scales[i], c, coef, terminal);
        RotReq R;
        R.id = f;
        R.nin = c;
        R.p = 1;
        R.out0 = m;
        R.Y.resize(c);
        for (int r = 0; r < c; ++r) R.Y[r] = coef[r] * beta;
        E.rotate({R});
        const double nr = E.normalize({f}, m, false)[0];
        const bool est_on = c == m && m < n;
        const double est = est_on ? std::abs(scales[i]) * terminal * beta * std::abs(coef[c - 1]) : 0.0;
        if (est > tol * std::max(1.0, nr)) failing.push_back(i);
        else E.store(f, m, out + (size_t)i * 2 * n, false);
    }
    E.remove(f);
    // the failing times: the recursion from v0, concurrently, in waves that fit in memory
    if (!failing.empty()) {
        size_t fr = 0, tot = 0;
        QS_CUDA(cudaMemGetInfo(&fr, &tot));
        const size_t per = Engine::slot_bytes(n, m, true, 1, E.store());
        const int wave = (int)std::max<size_t>(1, std::min<size_t>(failing.size(), (fr / 2) / std::max<size_t>(per, 1)));
        for (size_t w0 = 0; w0 < failing.size(); w0 += wave) {
            const size_t w1 = std::min(failing.size(), w0 + wave);
            std::vector<int> ids;
            std::vector<EvoTask> tasks;
            std::vector<double*> outs;
            for (size_t q = w0; q < w1; ++q) {
                const int i = failing[q];
                const int id = E.add(op, m, true, true, 1, orth);
                E.load(id, 0, v0, false);
                ids.push_back(id);
                outs.push_back(out + (size_t)i * 2 * n);
            }
            std::vector<double> b0 = E.normalize(ids);
            for (size_t q = w0; q < w1; ++q) {
                EvoTask t;
                // the recursion's first attempt is the shared factorisation, which failed
                t.init(m, n, herm, scales[failing[q]], tol, b0[q - w0], true);
                tasks.push_back(t);
            }
            run_evo_slots(E, ids, tasks, outs);
        }
    }
    if (normalise)
        for (int i = 0; i < nt; ++i) {
            double* o = out + (size_t)i * 2 * n;
            double s2 = 0;
            for (int64_t q = 0; q < 2 * n; ++q) s2 += o[q] * o[q];
            const double inv = s2 > 0 ? 1.0 / std::sqrt(s2) : 0.0;
            for (int64_t q = 0; q < 2 * n; ++q) o[q] *= inv;
        }
    QS_CUDA(cudaStreamSynchronize(E.stream()));
    note_launches(E.launches());
}

void evolve_stepwise(Op& op, const double* v0, const std::vector<double>& offsets, bool imag_time, double tol,
                     int krylov_dim, int precision, double* out) {
    const int64_t n = op.basis->n;
    const int nt = (int)offsets.size();
    if (nt == 0) return;
    const int m = (int)std::max<int64_t>(2, std::min<int64_t>(std::min(krylov_dim, kMaxM), n));
    const bool herm = op.hermitian;
    Engine E(precision == 0 ? Store::F64 : Store::DF, op.stream);
    cudaStream_t st = E.stream();
    const size_t bytes = (size_t)n * 16;
    PoolBuf cur(bytes, st);
    QS_CUDA(cudaMemcpyAsync(cur.p, v0, bytes, cudaMemcpyHostToDevice, st));
    // the times in order of their offset from t0, propagated one from the next
    std::vector<int> order(nt);
    for (int i = 0; i < nt; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return offsets[a] < offsets[b]; });
    int steps = 0;
    double prev = 0.0;
    for (int i : order)
        if (offsets[i] != prev) {
            ++steps;
            prev = offsets[i];
        }
    // the steps' errors add up: each gets an equal share of the tolerance
    const double tol_step = tol / std::max(1, steps);
    Blas B(VKind::C128, n, st);
    prev = 0.0;
    for (int i : order) {
        const double d = offsets[i] - prev;
        if (d != 0.0) {
            const int id = E.add(op, m, true, true, 1, herm ? 2 : 0);
            E.load(id, 0, cur.as<double>(), true);
            const double beta = E.normalize({id})[0];
            if (beta > 0) {
                std::vector<int> ids{id};
                std::vector<EvoTask> tasks(1);
                tasks[0].init(m, n, herm, imag_time ? cd(-d, 0) : cd(0, -d), tol_step, beta, false);
                std::vector<double*> outs{cur.as<double>()};
                run_evo_slots(E, ids, tasks, outs, true);
            } else {
                E.remove(id);
            }
            if (imag_time) {
                // exp(-tau H) shrinks or grows the state: carry it at norm 1, as
                // the reference normalises every imaginary-time state
                const double nr = B.norm(cur.p);
                if (nr > 0) B.scale(cur.p, cur.p, cd(1.0 / nr, 0));
            }
            prev = offsets[i];
        }
        QS_CUDA(cudaMemcpyAsync(out + (size_t)i * 2 * n, cur.p, bytes, cudaMemcpyDeviceToHost, st));
    }
    QS_CUDA(cudaStreamSynchronize(st));
    note_launches(E.launches());
}

void evolve_blocks(const std::vector<Op*>& ops, const std::vector<const double*>& v0s, const std::vector<cd>& scales,
                   double tol, int krylov_dim, int precision, const std::vector<double*>& outs) {
    const size_t nb = ops.size();
    const int nt = (int)scales.size();
    if (nb == 0 || nt == 0) return;
    Engine E(precision == 0 ? Store::F64 : Store::DF, ops[0]->stream);
    cudaStream_t st = E.stream();
    std::vector<int64_t> n(nb);
    std::vector<int> m(nb), f(nb, -1);
    std::vector<char> herm(nb);
    auto copy_v0 = [&](size_t b, int i) {
        QS_CUDA(cudaMemcpyAsync(outs[b] + (size_t)i * 2 * n[b], v0s[b], (size_t)n[b] * 16, cudaMemcpyDeviceToDevice,
                                st));
    };
    // phase 1: one factorisation per block from its start vector (a 1-state
    // block still takes two columns; its second direction is zero and the
    // breakdown test stops the projection at c = 1)
    std::vector<int> fid;
    for (size_t b = 0; b < nb; ++b) {
        n[b] = ops[b]->basis->n;
        m[b] = (int)std::max<int64_t>(2, std::min<int64_t>(std::min(krylov_dim, kMaxM), n[b]));
        herm[b] = ops[b]->hermitian;
        f[b] = E.add(*ops[b], m[b], true, true, 1, herm[b] ? 2 : 0);
        E.load(f[b], 0, v0s[b], true);
        fid.push_back(f[b]);
    }
    const std::vector<double> beta = E.normalize(fid);
    std::vector<char> active(nb, 0);
    for (size_t b = 0; b < nb; ++b) {
        bool all_zero = true;
        for (const cd& sc : scales) all_zero = all_zero && sc == cd(0, 0);
        if (beta[b] == 0 || all_zero) {
            for (int i = 0; i < nt; ++i) copy_v0(b, i);
            E.remove(f[b]);
        } else {
            active[b] = 1;
            E.start(f[b], 0);
        }
    }
    for (int steps = E.steps_to_event(); steps > 0; steps = E.steps_to_event()) E.run(steps);
    std::vector<size_t> act;
    std::vector<int> act_ids;
    for (size_t b = 0; b < nb; ++b)
        if (active[b]) {
            act.push_back(b);
            act_ids.push_back(f[b]);
        }
    std::vector<std::vector<cd>> H;
    E.records(act_ids, H);
    // every time of every block from its shared factorisation: one rotation
    // launch and one normalisation per Krylov size for all blocks at a time
    std::vector<std::pair<size_t, int>> failing;
    for (int i = 0; i < nt; ++i) {
        std::vector<RotReq> rot;
        std::vector<size_t> who;
        std::vector<int> cs;
        std::vector<double> terms;
        for (size_t q = 0; q < act.size(); ++q) {
            const size_t b = act[q];
            if (scales[i] == cd(0, 0)) {
                copy_v0(b, i);
                continue;
            }
            int c;
            std::vector<cd> coef;
            double terminal;
            krylov_project(H[q], m[b], herm[b], scales[i], c, coef, terminal);
            RotReq R;
            R.id = f[b];
            R.nin = c;
            R.p = 1;
            R.out0 = m[b];
            R.Y.resize(c);
            for (int r = 0; r < c; ++r) R.Y[r] = coef[r] * beta[b];
            rot.push_back(std::move(R));
            who.push_back(b);
            cs.push_back(c);
            terms.push_back(std::abs(scales[i]) * terminal * beta[b] * std::abs(coef[c - 1]));
        }
        if (rot.empty()) continue;
        E.rotate(rot);
        std::map<int, std::vector<size_t>> by_m;
        for (size_t q = 0; q < who.size(); ++q) by_m[m[who[q]]].push_back(q);
        std::vector<double> nr(who.size());
        for (const auto& kv : by_m) {
            std::vector<int> ids;
            for (size_t q : kv.second) ids.push_back(f[who[q]]);
            const std::vector<double> g = E.normalize(ids, kv.first, false);
            for (size_t t = 0; t < kv.second.size(); ++t) nr[kv.second[t]] = g[t];
        }
        for (size_t q = 0; q < who.size(); ++q) {
            const size_t b = who[q];
            const bool est_on = cs[q] == m[b] && m[b] < n[b];
            const double est = est_on ? terms[q] : 0.0;
            if (est > tol * std::max(1.0, nr[q])) failing.push_back({b, i});
            else E.store(f[b], m[b], outs[b] + (size_t)i * 2 * n[b], true);
        }
    }
    for (size_t b : act) E.remove(f[b]);
    // phase 2: the failing (block, time) pairs run the reference's recursion
    // from their start vectors, concurrently, in waves that fit in memory
    size_t fr = 0, tot = 0;
    QS_CUDA(cudaMemGetInfo(&fr, &tot));
    for (size_t w0 = 0; w0 < failing.size();) {
        std::vector<int> ids;
        std::vector<EvoTask> tasks;
        std::vector<double*> wouts;
        std::vector<size_t> blk;
        size_t used = 0, w1 = w0;
        for (; w1 < failing.size(); ++w1) {
            const size_t b = failing[w1].first;
            const size_t per = Engine::slot_bytes(n[b], m[b], true, 1, E.store());
            if (w1 > w0 && used + per > fr / 2) break;
            used += per;
            const int id = E.add(*ops[b], m[b], true, true, 1, herm[b] ? 2 : 0);
            E.load(id, 0, v0s[b], true);
            ids.push_back(id);
            wouts.push_back(outs[b] + (size_t)failing[w1].second * 2 * n[b]);
            blk.push_back(b);
        }
        const std::vector<double> b0 = E.normalize(ids);
        for (size_t q = 0; q < ids.size(); ++q) {
            EvoTask t;
            // the recursion's first attempt is the shared factorisation, which failed
            t.init(m[blk[q]], n[blk[q]], herm[blk[q]], scales[failing[w0 + q].second], tol, b0[q], true);
            tasks.push_back(t);
        }
        run_evo_slots(E, ids, tasks, wouts, true);
        w0 = w1;
    }
    QS_CUDA(cudaStreamSynchronize(st));
    note_launches(E.launches());
}

}  // namespace qs
