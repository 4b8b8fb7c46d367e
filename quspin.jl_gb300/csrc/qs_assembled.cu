// qs_assembled.cu -- the assembled (compiled-transition) form of an operator.
//
// The reference's static Hamiltonian assembles H.data as a CSC matrix at
// construction (_assemble, src/operators.jl:461-576) and its matvec is a
// SparseArrays SpMV (754-766).  Here the assembled form is built on the device
// by one pass of the fused row kernel that records, for every surviving
// transition, its column and a small value code, packed into one 32-bit word
// (column in the high bits, code in the low bits).  Every matrix element is a
// product  A_class * (+-1) * chi_class * sqrt(stab_col) / sqrt(stab_row),  so a
// table of a few hundred values replaces the 8-16 bytes of a stored element and
// the SpMV streams 4 bytes per nonzero.  Rows are sub-warp owned; no atomics.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <cmath>
#include <complex>
#include <vector>

#include "qs_device.cuh"
#include "qs_df.cuh"
#include "qs_internal.h"

namespace qs {

namespace {

constexpr int kThreads = 256;
constexpr int kMaxSplit = 2048;

struct BuildArgs {
    const void* reps;
    const uint16_t* stab;
    const void* split;
    int64_t n, nsplit, stride;
    const GroupDesc* group;
    const uint64_t* binom;
    const int32_t* index;
    int L, nup, mode;      // mode: 0 full space, 1 combinadic, 2 search, 3 direct index
    const TermProg* progs;
    int nprog;
    const uint16_t* prog_code;   // (aclass * 2 + sign) per program
    const uint16_t* elem_code;   // (cclass * 2 + sign) per group element
    const uint8_t* stab_class;   // dclass per stabiliser order
    FastGroup fast;              // zero-run orbit search when enabled
    const uint16_t* fast_code;   // (cclass * 2 + sign) per fast element code
    int nC, nD, code_bits;
    int32_t* counts;             // pass 1
    const int64_t* rowptr;       // pass 2
    uint32_t* words;
    uint16_t* codes;             // unpacked layout: code per nonzero
    int32_t* cols;               // unpacked layout: column per nonzero
    int packed;
};

template <typename U>
__device__ __forceinline__ U build_row_state(const BuildArgs& a, int64_t r) {
    if (a.mode >= 2) return ((const U*)a.reps)[r];
    if (a.mode == 0) return (U)r;
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

template <typename U, bool kWrite>
__global__ void __launch_bounds__(kThreads) build_kernel(BuildArgs a) {
    __shared__ GroupSmem g;
    __shared__ U spl[kMaxSplit];
    if (a.mode >= 2) {
        load_group_smem(g, a.group);
        if (a.mode == 2)
            for (int i = threadIdx.x; i < a.nsplit; i += blockDim.x) spl[i] = ((const U*)a.split)[i];
        __syncthreads();
    }
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < a.n; r += (int64_t)gridDim.x * blockDim.x) {
        const U s = build_row_state<U>(a, r);
        int64_t out = kWrite ? a.rowptr[r] : 0;
        int32_t cnt = 0;
        for (int k = 0; k < a.nprog; ++k) {
            const TermProg& p = a.progs[k];
            if ((s & (U)p.need1) != (U)p.need1 || (s & (U)p.need0) != (U)0) continue;
            U t = s ^ (U)p.flip;
            int sign = (__popcll((unsigned long long)(~s & (U)p.zmask)) + __popcll((unsigned long long)(s & (U)p.ymask))) & 1;
            int64_t idx;
            int cclass = 0, dclass = 0;
            if (a.mode >= 2) {
                U m;
                int bi, st;
                int ec;
                if (a.fast.enabled) {
                    orbit_min_fast<U>(a.fast, t, m, bi, st);
                    ec = a.fast_code[bi];
                } else {
                    orbit_min<U>(g, t, m, bi, st);
                    ec = a.elem_code[bi];
                }
                if (a.mode == 3) {
                    int64_t rk = a.nup >= 0 ? combinadic_rank<U>(m, a.binom, 65) : (int64_t)m;
                    idx = __ldg(a.index + rk);
                } else {
                    idx = rank_search<U>((const U*)a.reps, a.n, spl, (int)a.nsplit, a.stride, m);
                }
                if (idx < 0) continue;
                cclass = ec >> 1;
                sign ^= ec & 1;
                dclass = a.stab_class[st];
            } else if (a.mode == 1) {
                if (__popcll((unsigned long long)t) != a.nup) continue;
                idx = combinadic_rank<U>(t, a.binom, 65);
            } else {
                idx = (int64_t)t;
            }
            if (kWrite) {
                int pc = a.prog_code[k];
                sign ^= pc & 1;
                uint32_t code = (uint32_t)((((pc >> 1) * a.nC + cclass) * a.nD + dclass) * 2 + sign);
                if (a.packed) a.words[out] = ((uint32_t)idx << a.code_bits) | code;
                else {
                    a.cols[out] = (int32_t)idx;
                    a.codes[out] = (uint16_t)code;
                }
                ++out;
            } else {
                ++cnt;
            }
        }
        if (!kWrite) a.counts[r] = cnt;
    }
}

__global__ void counts_to_i64(const int32_t* c, int64_t* o, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        o[i] = c[i];
}

template <typename T> struct V2;
template <> struct V2<double> { using t = double2; };
template <> struct V2<float> { using t = float2; };

struct SpmvArgs {
    const int64_t* rowptr;
    const uint32_t* words;
    const int32_t* cols;
    const uint16_t* codes;
    int packed;
    uint32_t code_mask;
    int code_bits;
    const void* table;       // value per code (T or complex T)
    int ncodes;
    const uint16_t* stab;    // row stabiliser order (null: 1)
    const void* diag;        // complex T per row
    int64_t n;
    double ar, ai, br, bi;
    int beta_zero;
    int conj;                // use the conjugated value table and diagonal
    const void* x;
    void* y;
};

// y = beta*y + alpha*( d.*x + (1/sqrt(stab_r)) * sum_j table[code_j] x[col_j] ),
// kG lanes per row.
template <int kG, bool kCM, bool kCV, typename T>
__global__ void __launch_bounds__(kThreads) spmv_kernel(SpmvArgs a) {
    using T2 = typename V2<T>::t;
    __shared__ T2 tab[1024];
    __shared__ T rsq[kMaxGroup + 1];
    const bool smem_tab = a.ncodes <= 1024;
    if (smem_tab)
        for (int i = threadIdx.x; i < a.ncodes; i += blockDim.x) {
            T2 v = ((const T2*)a.table)[i];
            if (a.conj) v.y = -v.y;
            tab[i] = v;
        }
    for (int i = threadIdx.x; i <= kMaxGroup; i += blockDim.x) rsq[i] = i ? (T)(1.0 / sqrt((double)i)) : (T)0;
    __syncthreads();
    const int lane = threadIdx.x % kG;
    constexpr int kRowsPerWarp = 32 / kG;
    const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / 32;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) / 32;
    const int sub = (threadIdx.x % 32) / kG;
    // every lane of a warp runs the same number of iterations (shuffles below)
    for (int64_t base = warp0 * kRowsPerWarp; base < a.n; base += nwarps * kRowsPerWarp) {
        const int64_t r = base + sub;
        const bool live = r < a.n;
        const int64_t j0 = live ? a.rowptr[r] : 0, j1 = live ? a.rowptr[r + 1] : 0;
        T acc_r = 0, acc_i = 0;
        for (int64_t j = j0 + lane; j < j1; j += kG) {
            uint32_t col, code;
            if (a.packed) {
                uint32_t w = __ldg(a.words + j);
                col = w >> a.code_bits;
                code = w & a.code_mask;
            } else {
                col = (uint32_t)__ldg(a.cols + j);
                code = __ldg(a.codes + j);
            }
            T2 v;
            if (smem_tab) v = tab[code];
            else {
                v = ((const T2*)a.table)[code];
                if (a.conj) v.y = -v.y;
            }
            if (kCV) {
                T2 xv = ((const T2*)a.x)[col];
                if (kCM) {
                    acc_r += v.x * xv.x - v.y * xv.y;
                    acc_i += v.x * xv.y + v.y * xv.x;
                } else {
                    acc_r += v.x * xv.x;
                    acc_i += v.x * xv.y;
                }
            } else {
                acc_r += v.x * ((const T*)a.x)[col];
            }
        }
#pragma unroll
        for (int o = kG / 2; o > 0; o >>= 1) {
            acc_r += __shfl_xor_sync(0xffffffffu, acc_r, o, kG);
            if (kCV) acc_i += __shfl_xor_sync(0xffffffffu, acc_i, o, kG);
        }
        if (lane == 0 && live) {
            T sc = a.stab ? rsq[a.stab[r]] : (T)1;
            acc_r *= sc;
            acc_i *= sc;
            T2 d = ((const T2*)a.diag)[r];
            T dr = d.x, di = a.conj ? -d.y : d.y;
            if (kCV) {
                T2 xv = ((const T2*)a.x)[r];
                acc_r += dr * xv.x - di * xv.y;
                acc_i += dr * xv.y + di * xv.x;
                T2* y = (T2*)a.y;
                T yr = 0, yi = 0;
                if (!a.beta_zero) {
                    T2 yo = y[r];
                    yr = (T)a.br * yo.x - (T)a.bi * yo.y;
                    yi = (T)a.br * yo.y + (T)a.bi * yo.x;
                }
                T2 o;
                o.x = yr + (T)a.ar * acc_r - (T)a.ai * acc_i;
                o.y = yi + (T)a.ar * acc_i + (T)a.ai * acc_r;
                y[r] = o;
            } else {
                acc_r += dr * ((const T*)a.x)[r];
                T* y = (T*)a.y;
                T yr = a.beta_zero ? (T)0 : (T)a.br * y[r];
                y[r] = yr + (T)a.ar * acc_r;
            }
        }
    }
}

// ---------------------------------------------------------- double-float form
// GB300's FP64 pipe, not HBM, bounds the FP64 product above (one DFMA per
// nonzero).  This form keeps every per-nonzero operation on the FP32 pipe:
// x is split once per row into hi + lo floats, the value table holds hi + lo
// pairs, and products and sums are carried as unevaluated float pairs with
// the error-free transformations TwoProd (via fma) and TwoSum (Knuth), i.e.
// about 48 significand bits.  Only the per-row combination runs in FP64.

__device__ __forceinline__ float2 df_split(double v) {
    float h = __double2float_rn(v);
    float l = __double2float_rn(v - (double)h);
    return make_float2(h, l);
}

// x (double, or double2 when complex) -> (hi, lo) float pairs per component
template <bool kCV>
__global__ void split_kernel(const void* x, float4* out_c, float2* out_r, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (kCV) {
            double2 v = ((const double2*)x)[i];
            float2 a = df_split(v.x), b = df_split(v.y);
            out_c[i] = make_float4(a.x, a.y, b.x, b.y);
        } else {
            out_r[i] = df_split(((const double*)x)[i]);
        }
    }
}

struct SpmvDFArgs {
    SpmvArgs s;
    const float4* tab_df;    // per code: re(hi, lo), im(hi, lo)
    const void* xs;          // split x: float2 (real) or float4 (complex)
};

template <int kG, bool kCM, bool kCV>
__global__ void __launch_bounds__(kThreads) spmv_df_kernel(SpmvDFArgs da) {
    const SpmvArgs& a = da.s;
    __shared__ float4 tab[1024];
    __shared__ double rsq[kMaxGroup + 1];
    const bool smem_tab = a.ncodes <= 1024;
    if (smem_tab)
        for (int i = threadIdx.x; i < a.ncodes; i += blockDim.x) {
            float4 v = da.tab_df[i];
            if (a.conj) { v.z = -v.z; v.w = -v.w; }
            tab[i] = v;
        }
    for (int i = threadIdx.x; i <= kMaxGroup; i += blockDim.x) rsq[i] = i ? 1.0 / sqrt((double)i) : 0.0;
    __syncthreads();
    const int lane = threadIdx.x % kG;
    constexpr int kRowsPerWarp = 32 / kG;
    const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / 32;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) / 32;
    const int sub = (threadIdx.x % 32) / kG;
    for (int64_t base = warp0 * kRowsPerWarp; base < a.n; base += nwarps * kRowsPerWarp) {
        const int64_t r = base + sub;
        const bool live = r < a.n;
        const int64_t j0 = live ? a.rowptr[r] : 0, j1 = live ? a.rowptr[r + 1] : 0;
        DF ar{0.f, 0.f}, ai{0.f, 0.f};
        for (int64_t j = j0 + lane; j < j1; j += kG) {
            uint32_t col, code;
            if (a.packed) {
                uint32_t w = __ldg(a.words + j);
                col = w >> a.code_bits;
                code = w & a.code_mask;
            } else {
                col = (uint32_t)__ldg(a.cols + j);
                code = __ldg(a.codes + j);
            }
            float4 v;
            if (smem_tab) v = tab[code];
            else {
                v = da.tab_df[code];
                if (a.conj) { v.z = -v.z; v.w = -v.w; }
            }
            if (kCV) {
                float4 xv = ((const float4*)da.xs)[col];
                df_mac(ar, v.x, v.y, xv.x, xv.y);
                df_mac(ai, v.x, v.y, xv.z, xv.w);
                if (kCM) {
                    df_mac(ar, -v.z, -v.w, xv.z, xv.w);
                    df_mac(ai, v.z, v.w, xv.x, xv.y);
                }
            } else {
                float2 xv = ((const float2*)da.xs)[col];
                df_mac(ar, v.x, v.y, xv.x, xv.y);
            }
        }
#pragma unroll
        for (int o = kG / 2; o > 0; o >>= 1) {
            DF br{__shfl_xor_sync(0xffffffffu, ar.h, o, kG), __shfl_xor_sync(0xffffffffu, ar.l, o, kG)};
            ar = df_add(ar, br);
            if (kCV) {
                DF bi{__shfl_xor_sync(0xffffffffu, ai.h, o, kG), __shfl_xor_sync(0xffffffffu, ai.l, o, kG)};
                ai = df_add(ai, bi);
            }
        }
        if (lane == 0 && live) {
            double sc = a.stab ? rsq[a.stab[r]] : 1.0;
            double acc_r = df_to_double(ar) * sc, acc_i = kCV ? df_to_double(ai) * sc : 0.0;
            double2 d = ((const double2*)a.diag)[r];
            double dr = d.x, di = a.conj ? -d.y : d.y;
            if (kCV) {
                double2 xv = ((const double2*)a.x)[r];
                acc_r += dr * xv.x - di * xv.y;
                acc_i += dr * xv.y + di * xv.x;
                double2* y = (double2*)a.y;
                double yr = 0, yi = 0;
                if (!a.beta_zero) {
                    double2 yo = y[r];
                    yr = a.br * yo.x - a.bi * yo.y;
                    yi = a.br * yo.y + a.bi * yo.x;
                }
                y[r] = make_double2(yr + a.ar * acc_r - a.ai * acc_i, yi + a.ar * acc_i + a.ai * acc_r);
            } else {
                acc_r += dr * ((const double*)a.x)[r];
                double* y = (double*)a.y;
                double yr = a.beta_zero ? 0.0 : a.br * y[r];
                y[r] = yr + a.ar * acc_r;
            }
        }
    }
}

// ----------------------------------------------------------- sliced ELL
constexpr int kSlice = kSellSlice;

__global__ void sell_fill_kernel(const int64_t* rowptr, const uint32_t* words, const int32_t* cols,
                                 const uint16_t* codes, int packed, const int32_t* perm, const int64_t* sptr,
                                 int64_t npos, uint32_t* swords, int32_t* scols, uint16_t* scodes) {
    for (int64_t pos = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; pos < npos; pos += (int64_t)gridDim.x * blockDim.x) {
        const int r = perm[pos];
        if (r < 0) continue;
        const int64_t s = pos / kSlice, l = pos % kSlice;
        const int64_t j0 = rowptr[r], j1 = rowptr[r + 1];
        const int64_t base = sptr[s] + l;
        for (int64_t j = j0; j < j1; ++j) {
            const int64_t o = base + (j - j0) * kSlice;
            if (packed) swords[o] = words[j];
            else {
                scols[o] = cols[j];
                scodes[o] = codes[j];
            }
        }
    }
}

// Explicitly rounded multiply-adds: the single product and the several-column
// product run the same operations in the same order, whatever the compiler
// would have contracted.
__device__ __forceinline__ double fma_t(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float fma_t(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double mul_t(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_t(float a, float b) { return __fmul_rn(a, b); }

// acc += value * x (complex value when kCM, complex x when kCV)
template <bool kCM, bool kCV, typename T, typename T2>
__device__ __forceinline__ void sell_mac(T& acc_r, T& acc_i, T2 v, T xr, T xi) {
    if (kCM) {
        acc_r = fma_t(v.x, xr, acc_r);
        acc_r = fma_t(-v.y, xi, acc_r);
        acc_i = fma_t(v.x, xi, acc_i);
        acc_i = fma_t(v.y, xr, acc_i);
    } else {
        acc_r = fma_t(v.x, xr, acc_r);
        if (kCV) acc_i = fma_t(v.x, xi, acc_i);
    }
}

// y[r] = beta y[r] + alpha (d[r] x[r] + sc acc) for one row of one column
template <bool kCV, typename T, typename T2>
__device__ __forceinline__ void sell_tail(T acc_r, T acc_i, T sc, T dr, T di, T xr, T xi, T2* y2, T* y1, int64_t r,
                                          double br, double bi, double ar, double ai, bool beta_zero) {
    acc_r = mul_t(acc_r, sc);
    acc_i = mul_t(acc_i, sc);
    if (kCV) {
        acc_r = fma_t(dr, xr, acc_r);
        acc_r = fma_t(-di, xi, acc_r);
        acc_i = fma_t(dr, xi, acc_i);
        acc_i = fma_t(di, xr, acc_i);
        T yr = 0, yi = 0;
        if (!beta_zero) {
            const T2 yo = y2[r];
            yr = mul_t((T)br, yo.x);
            yr = fma_t(-(T)bi, yo.y, yr);
            yi = mul_t((T)br, yo.y);
            yi = fma_t((T)bi, yo.x, yi);
        }
        T2 o;
        o.x = fma_t((T)ar, acc_r, yr);
        o.x = fma_t(-(T)ai, acc_i, o.x);
        o.y = fma_t((T)ar, acc_i, yi);
        o.y = fma_t((T)ai, acc_r, o.y);
        y2[r] = o;
    } else {
        acc_r = fma_t(dr, xr, acc_r);
        const T yr = beta_zero ? (T)0 : mul_t((T)br, y1[r]);
        y1[r] = fma_t((T)ar, acc_r, yr);
    }
}

struct SellArgs {
    const int64_t* sptr;
    const int32_t* perm;
    const uint16_t* len;
    const uint32_t* words;
    const int32_t* cols;
    const uint16_t* codes;
    int packed;
    uint32_t code_mask;
    int code_bits;
    const void* table;
    int ncodes;
    const uint16_t* stab;
    const void* diag;
    const void* diag_re;     // real diagonal (real operators)
    int64_t nslices, n;      // slices slice0 .. nslices - 1 are computed
    int64_t slice0;
    double ar, ai, br, bi;
    int beta_zero;
    int conj;
    const void* x;
    void* y;
};

// One thread per row: y[r] = beta y[r] + alpha (d[r] x[r] + rs(stab[r]) sum_j T[code_j] x[col_j])
template <bool kCM, bool kCV, typename T, bool kPacked, int U, int MINB, bool kHint>
__global__ void __launch_bounds__(kThreads, MINB) sell_kernel(SellArgs a) {
    using T2 = typename V2<T>::t;
    __shared__ T2 tab[1024];
    __shared__ T rsq[kMaxGroup + 1];
    const bool smem_tab = a.ncodes <= 1024;
    if (smem_tab)
        for (int i = threadIdx.x; i < a.ncodes; i += blockDim.x) {
            T2 v = ((const T2*)a.table)[i];
            if (a.conj) v.y = -v.y;
            tab[i] = v;
        }
    for (int i = threadIdx.x; i <= kMaxGroup; i += blockDim.x) rsq[i] = i ? (T)(1.0 / sqrt((double)i)) : (T)0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const T2* __restrict__ gtab = (const T2*)a.table;
    const bool conj = a.conj;
    for (int64_t s = a.slice0 + warp0; s < a.nslices; s += nwarps) {
        const int64_t r = s * kSlice + lane;
        if (r >= a.n) continue;
        const int len = a.len[r];
        const int64_t base = a.sptr[s] + lane;
        T acc_r = 0, acc_i = 0;
        auto value = [&](uint32_t code) -> T2 {
            if (smem_tab) return tab[code];
            T2 v = gtab[code];
            if (conj) v.y = -v.y;
            return v;
        };
        if (kCV) {
            const T2* __restrict__ x = (const T2*)a.x;
            sell_row<U, kPacked, kHint>(a.words, a.cols, a.codes, base, len, a.code_bits, a.code_mask,
                                 [&](uint32_t c) { return ld_gather<kHint>(x + c); },
                                 [&](uint32_t code, T2 xv) { sell_mac<kCM, true>(acc_r, acc_i, value(code), xv.x, xv.y); });
        } else {
            const T* __restrict__ x = (const T*)a.x;
            sell_row<U, kPacked, kHint>(a.words, a.cols, a.codes, base, len, a.code_bits, a.code_mask,
                                 [&](uint32_t c) { return ld_gather<kHint>(x + c); },
                                 [&](uint32_t code, T xv) { sell_mac<false, false>(acc_r, acc_i, value(code), xv, (T)0); });
        }
        const T sc = a.stab ? rsq[a.stab[r]] : (T)1;
        T dr, di = 0;
        if (kCM) {
            const T2 d = ((const T2*)a.diag)[r];
            dr = d.x;
            di = a.conj ? -d.y : d.y;
        } else {
            dr = ((const T*)a.diag_re)[r];
        }
        T xr, xi = 0;
        if (kCV) {
            const T2 xv = ((const T2*)a.x)[r];
            xr = xv.x;
            xi = xv.y;
        } else {
            xr = ((const T*)a.x)[r];
        }
        sell_tail<kCV>(acc_r, acc_i, sc, dr, di, xr, xi, (T2*)a.y, (T*)a.y, r, a.br, a.bi, a.ar, a.ai, a.beta_zero);
    }
}

// ------------------------------------------------ several right-hand sides
// mul!(Y, op, X) with X and Y column-major n x ncols (src/operators.jl:
// 3185-3208, a column loop in the reference), up to R = 8 columns per launch.
// X is first interleaved into Xt (row r holds its R values contiguously, the
// unused columns zero), so that one gather brings every column's x[col]
// (64 bytes in FP64) where separate products would gather R times; one
// thread per row walks the row's packed words once.  Per column the sum runs
// over the row's nonzeros in the order of sell_kernel and the row tail is the
// same, so each column of Y is bit-identical to a single product.
template <typename E, int R>
__global__ void interleave_kernel(const E* __restrict__ X, E* __restrict__ Xt, int64_t n, int ncols) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        E v[R];
#pragma unroll
        for (int c = 0; c < R; ++c) {
            if (c < ncols) v[c] = X[(int64_t)c * n + r];
            else memset(&v[c], 0, sizeof(E));
        }
#pragma unroll
        for (int c = 0; c < R; ++c) Xt[r * R + c] = v[c];
    }
}

// R values of type T starting at p (16-byte aligned), read 16 bytes at a time
template <typename T, int R>
__device__ __forceinline__ void ld_row(const T* p, T (&v)[R]) {
    static_assert((R * sizeof(T)) % 16 == 0, "rows of whole 16-byte units");
    if (sizeof(T) == 8) {
#pragma unroll
        for (int c = 0; c < R; c += 2) {
            const double2 d = ld_gather<true>((const double2*)(p + c));
            memcpy(&v[c], &d, 16);
        }
    } else {
#pragma unroll
        for (int c = 0; c < R; c += 4) {
            const float4 f = ld_gather<true>((const float4*)(p + c));
            memcpy(&v[c], &f, 16);
        }
    }
}

template <bool kCM, bool kCV, typename T, bool kPacked, int R>
__global__ void __launch_bounds__(kThreads, 2) sell_mm_kernel(SellArgs a, int ncols, int64_t ldy) {
    using T2 = typename V2<T>::t;
    __shared__ T2 tab[1024];
    __shared__ T rsq[kMaxGroup + 1];
    const bool smem_tab = a.ncodes <= 1024;
    if (smem_tab)
        for (int i = threadIdx.x; i < a.ncodes; i += blockDim.x) {
            T2 v = ((const T2*)a.table)[i];
            if (a.conj) v.y = -v.y;
            tab[i] = v;
        }
    for (int i = threadIdx.x; i <= kMaxGroup; i += blockDim.x) rsq[i] = i ? (T)(1.0 / sqrt((double)i)) : (T)0;
    __syncthreads();
    constexpr int W = kCV ? 2 * R : R;   // reals per interleaved row
    const T* __restrict__ Xt = (const T*)a.x;
    const int lane = threadIdx.x & 31;
    const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const T2* __restrict__ gtab = (const T2*)a.table;
    const bool conj = a.conj;
    for (int64_t s = a.slice0 + warp0; s < a.nslices; s += nwarps) {
        const int64_t r = s * kSlice + lane;
        if (r >= a.n) continue;
        const int len = a.len[r];
        const int64_t base = a.sptr[s] + lane;
        T acc_r[R], acc_i[R];
#pragma unroll
        for (int c = 0; c < R; ++c) acc_r[c] = acc_i[c] = 0;
        for (int j = 0; j < len; ++j) {
            const int64_t o = base + (int64_t)j * kSellSlice;
            uint32_t col, code;
            if (kPacked) {
                const uint32_t w = ld_word<true>(a.words + o);
                col = w >> a.code_bits;
                code = w & a.code_mask;
            } else {
                col = (uint32_t)ld_word<true>(a.cols + o);
                code = ld_word<true>(a.codes + o);
            }
            T xv[W];
            ld_row<T, W>(Xt + (int64_t)col * W, xv);
            T2 v;
            if (smem_tab) {
                v = tab[code];
            } else {
                v = gtab[code];
                if (conj) v.y = -v.y;
            }
#pragma unroll
            for (int c = 0; c < R; ++c) {
                if (kCV) sell_mac<kCM, true>(acc_r[c], acc_i[c], v, xv[2 * c], xv[2 * c + 1]);
                else sell_mac<false, false>(acc_r[c], acc_i[c], v, xv[c], (T)0);
            }
        }
        const T sc = a.stab ? rsq[a.stab[r]] : (T)1;
        T dr, di = 0;
        if (kCM) {
            const T2 d = ((const T2*)a.diag)[r];
            dr = d.x;
            di = a.conj ? -d.y : d.y;
        } else {
            dr = ((const T*)a.diag_re)[r];
        }
        T xr_row[W];
        ld_row<T, W>(Xt + r * W, xr_row);
#pragma unroll
        for (int c = 0; c < R; ++c) {
            if (c >= ncols) break;
            const T xr = kCV ? xr_row[2 * c] : xr_row[c], xi = kCV ? xr_row[2 * c + 1] : (T)0;
            sell_tail<kCV>(acc_r[c], acc_i[c], sc, dr, di, xr, xi, (T2*)a.y + c * ldy, (T*)a.y + c * ldy, r, a.br,
                           a.bi, a.ar, a.ai, a.beta_zero);
        }
    }
}

// Double-float products, one thread per row; FP64 only in the per-row tail,
// where all 32 lanes of a warp work on 32 rows.
template <bool kCM, bool kCV, bool kPacked, int U, int MINB, bool kHint>
__global__ void __launch_bounds__(kThreads, MINB) sell_df_kernel(SellArgs a, const float4* __restrict__ tab_df,
                                                           const void* __restrict__ xs) {
    __shared__ float4 tab[1024];
    __shared__ double rsq[kMaxGroup + 1];
    const bool smem_tab = a.ncodes <= 1024;
    if (smem_tab)
        for (int i = threadIdx.x; i < a.ncodes; i += blockDim.x) {
            float4 v = tab_df[i];
            if (a.conj) { v.z = -v.z; v.w = -v.w; }
            tab[i] = v;
        }
    for (int i = threadIdx.x; i <= kMaxGroup; i += blockDim.x) rsq[i] = i ? 1.0 / sqrt((double)i) : 0.0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const bool conj = a.conj;
    for (int64_t s = a.slice0 + warp0; s < a.nslices; s += nwarps) {
        const int64_t r = s * kSlice + lane;
        if (r >= a.n) continue;
        const int len = a.len[r];
        const int64_t base = a.sptr[s] + lane;
        DF ar{0.f, 0.f}, ai{0.f, 0.f};
        auto value = [&](uint32_t code) -> float4 {
            if (smem_tab) return tab[code];
            float4 v = tab_df[code];
            if (conj) { v.z = -v.z; v.w = -v.w; }
            return v;
        };
        if (kCV) {
            const float4* __restrict__ x = (const float4*)xs;
            sell_row<U, kPacked, kHint>(a.words, a.cols, a.codes, base, len, a.code_bits, a.code_mask,
                                 [&](uint32_t c) { return ld_gather<kHint>(x + c); },
                                 [&](uint32_t code, float4 xv) {
                                     const float4 v = value(code);
                                     df_mac(ar, v.x, v.y, xv.x, xv.y);
                                     df_mac(ai, v.x, v.y, xv.z, xv.w);
                                     if (kCM) {
                                         df_mac(ar, -v.z, -v.w, xv.z, xv.w);
                                         df_mac(ai, v.z, v.w, xv.x, xv.y);
                                     }
                                 });
        } else {
            const float2* __restrict__ x = (const float2*)xs;
            sell_row<U, kPacked, kHint>(a.words, a.cols, a.codes, base, len, a.code_bits, a.code_mask,
                                 [&](uint32_t c) { return ld_gather<kHint>(x + c); },
                                 [&](uint32_t code, float2 xv) {
                                     const float4 v = value(code);
                                     df_mac(ar, v.x, v.y, xv.x, xv.y);
                                 });
        }
        const double sc = a.stab ? rsq[a.stab[r]] : 1.0;
        double acc_r = df_to_double(ar) * sc, acc_i = kCV ? df_to_double(ai) * sc : 0.0;
        double dr, di = 0;
        if (kCM) {
            const double2 d = ((const double2*)a.diag)[r];
            dr = d.x;
            di = a.conj ? -d.y : d.y;
        } else {
            dr = ((const double*)a.diag_re)[r];
        }
        if (kCV) {
            const double2 xv = ((const double2*)a.x)[r];
            acc_r += dr * xv.x - di * xv.y;
            acc_i += dr * xv.y + di * xv.x;
            double2* y = (double2*)a.y;
            double yr = 0, yi = 0;
            if (!a.beta_zero) {
                const double2 yo = y[r];
                yr = a.br * yo.x - a.bi * yo.y;
                yi = a.br * yo.y + a.bi * yo.x;
            }
            y[r] = make_double2(yr + a.ar * acc_r - a.ai * acc_i, yi + a.ar * acc_i + a.ai * acc_r);
        } else {
            acc_r += dr * ((const double*)a.x)[r];
            double* y = (double*)a.y;
            const double yr = a.beta_zero ? 0.0 : a.br * y[r];
            y[r] = yr + a.ar * acc_r;
        }
    }
}

// Double-float storage in and out (the Krylov solvers' double-float vectors):
// y = d .* x + rs(stab) * sum_j T[code_j] x[col_j], entirely on the FP32 pipe.
template <bool kCM, bool kCV, bool kPacked, int U, int MINB, bool kHint>
__global__ void __launch_bounds__(kThreads, MINB) sell_dfio_kernel(SellArgs a, const float4* __restrict__ tab_df,
                                                                const float4* __restrict__ diag_df,
                                                                const float2* __restrict__ rsq_df) {
    __shared__ float4 tab[1024];
    __shared__ float2 rsq[kMaxGroup + 1];
    const bool smem_tab = a.ncodes <= 1024;
    if (smem_tab)
        for (int i = threadIdx.x; i < a.ncodes; i += blockDim.x) {
            float4 v = tab_df[i];
            if (a.conj) { v.z = -v.z; v.w = -v.w; }
            tab[i] = v;
        }
    for (int i = threadIdx.x; i <= kMaxGroup; i += blockDim.x) rsq[i] = rsq_df[i];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const bool conj = a.conj;
    for (int64_t s = a.slice0 + warp0; s < a.nslices; s += nwarps) {
        const int64_t r = s * kSlice + lane;
        if (r >= a.n) continue;
        const int len = a.len[r];
        const int64_t base = a.sptr[s] + lane;
        DF ar{0.f, 0.f}, ai{0.f, 0.f};
        auto value = [&](uint32_t code) -> float4 {
            if (smem_tab) return tab[code];
            float4 v = tab_df[code];
            if (conj) { v.z = -v.z; v.w = -v.w; }
            return v;
        };
        if (kCV) {
            const float4* __restrict__ x = (const float4*)a.x;
            sell_row<U, kPacked, kHint>(a.words, a.cols, a.codes, base, len, a.code_bits, a.code_mask,
                                 [&](uint32_t c) { return ld_gather<kHint>(x + c); },
                                 [&](uint32_t code, float4 xv) {
                                     const float4 v = value(code);
                                     df_mac(ar, v.x, v.y, xv.x, xv.y);
                                     df_mac(ai, v.x, v.y, xv.z, xv.w);
                                     if (kCM) {
                                         df_mac(ar, -v.z, -v.w, xv.z, xv.w);
                                         df_mac(ai, v.z, v.w, xv.x, xv.y);
                                     }
                                 });
        } else {
            const float2* __restrict__ x = (const float2*)a.x;
            sell_row<U, kPacked, kHint>(a.words, a.cols, a.codes, base, len, a.code_bits, a.code_mask,
                                 [&](uint32_t c) { return ld_gather<kHint>(x + c); },
                                 [&](uint32_t code, float2 xv) {
                                     const float4 v = value(code);
                                     df_mac(ar, v.x, v.y, xv.x, xv.y);
                                 });
        }
        const float2 sc = a.stab ? rsq[a.stab[r]] : make_float2(1.f, 0.f);
        DF out_r = df_mul(ar, DF{sc.x, sc.y});
        const float4 d = diag_df[r];   // re hi, re lo, im hi, im lo
        const float dih = a.conj ? -d.z : d.z, dil = a.conj ? -d.w : d.w;
        if (kCV) {
            DF out_i = df_mul(ai, DF{sc.x, sc.y});
            const float4 xv = ((const float4*)a.x)[r];
            df_mac(out_r, d.x, d.y, xv.x, xv.y);
            df_mac(out_r, -dih, -dil, xv.z, xv.w);
            df_mac(out_i, d.x, d.y, xv.z, xv.w);
            df_mac(out_i, dih, dil, xv.x, xv.y);
            ((float4*)a.y)[r] = make_float4(out_r.h, out_r.l, out_i.h, out_i.l);
        } else {
            const float2 xv = ((const float2*)a.x)[r];
            df_mac(out_r, d.x, d.y, xv.x, xv.y);
            ((float2*)a.y)[r] = make_float2(out_r.h, out_r.l);
        }
    }
}

// ------------------------------------------------ exact fixed-point row sums
// When every stored value is real and, with the column's sqrt(stab) taken
// out, one of at most four amplitudes (value = +-A_c sqrt(stab_col)), a row
// sum needs no multiply per nonzero:
//     sum_j value_j x_j = sum_c A_c sum_{j in c} +-x'_j,  x'_j = x_j sqrt(stab_j).
// x' is scaled by a power of two 2^K and rounded to 64-bit integers once per
// product (K from a bound of max |x'| within a factor of two and from the
// longest row, so that no sum of a row can overflow), the inner sums are
// exact integer adds on the integer pipe, and FP64 runs only per row: one
// conversion and one multiply-add per class, the row scale and the diagonal
// term.  Besides the FP64 product x_j sqrt(stab_j), the only rounding before
// the row tail is that of each x'_j to a multiple of 2^-K, at most
// 2^(len_bits - 61) max|x'|, so a row sum of at most 2^len_bits terms is
// within 2^(2 len_bits - 61) max|x'| of exact: normwise the accuracy of an
// FP64 row sum.  Elements far
// below max|x'| do not keep their relative accuracy, which is why the form is
// requested explicitly (QS_FIXED_POINT) and the FP64 product stays the default.

constexpr int kFxParts = 4096;   // blocks of the max pass, at most
// kFxCodes (256) bounds the value codes: four classes x 2 signs x the divisor
// count of |G| (at most 24 for |G| <= 512) is 192 at most

struct FxArgs {
    const uint32_t* cls;                // per code: class << 1 | sign
    const double* amp;                  // per class: A_c
    const double* sq;                   // sqrt(i), i = 0 .. kMaxGroup
    unsigned long long* part;           // per block of the max pass: max |x'_j| as its IEEE bit pattern
    unsigned long long* maxbits;        // max |x'_j| over all of x
    int len_bits;                       // ceil(log2(longest row))
    void* xq;                           // round(x' 2^K): int64, or int64 pairs for complex x
};

// 2^k for -1022 <= k <= 1023, from its bit pattern
__device__ __forceinline__ double fx_pow2(int k) { return __longlong_as_double((long long)(1023 + k) << 52); }

__device__ __forceinline__ bool fx_finite(unsigned long long mb) { return mb < 0x7ff0000000000000ull; }

// With max |x'| < 2^E (E from the biased exponent; subnormals count as
// 2^-1022), |x'_j| 2^K <= 2^(62 - len_bits): a sum of at most 2^len_bits of
// them stays within 2^62.  -978 <= K <= 1083.
__device__ __forceinline__ int fx_shift(unsigned long long mb, int len_bits) {
    const int e = (int)(mb >> 52);
    return 62 - ((e > 0 ? e : 1) - 1022) - len_bits;
}

// GB300 runs FP64 at ~1/70 of its FP32 rate, so both passes over x stay on
// the integer pipe but for one FP64 multiply x_j sqrt(stab_j) per element
// (an integer 53 x 64-bit product in its place measured slower).

// ceil(log2(sqrt(st))) for st >= 1: sqrt(st) <= 2^c
__device__ __forceinline__ int fx_sqrt_exp(unsigned st) { return (32 - __clz(st - 1u) + 1) >> 1; }

// An upper bound of |x sqrt(st)| within a factor of two, as an IEEE bit
// pattern: |x| times 2^c added in the exponent field.  Infinities and NaNs
// stay at or above the infinity pattern; a finite value whose bound passes
// it is treated as non-finite (the product then runs as FP64).
__device__ __forceinline__ unsigned long long fx_bound_bits(double v, int c) {
    return ((unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull) + ((unsigned long long)c << 52);
}

// round(v 2^K) to the nearest integer, ties to even, from v's bit pattern;
// |v 2^K| <= 2^62 by the choice of K
__device__ __forceinline__ long long fx_round_scaled(double v, int K) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const int e = (int)((b >> 52) & 0x7ff);
    const unsigned long long mant = (b & 0xfffffffffffffull) | (e ? (1ull << 52) : 0ull);
    const int t = (e ? e : 1) - 1075 + K;   // v 2^K = mant 2^t
    unsigned long long q;
    if (t >= 0) {
        q = mant << t;
    } else if (t < -63) {
        q = 0;
    } else {
        const int sh = -t;
        q = mant >> sh;
        const unsigned long long rem = mant & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
        q += (rem > half || (rem == half && (q & 1ull))) ? 1ull : 0ull;
    }
    return (b >> 63) ? -(long long)q : (long long)q;
}

// rows i + u st, u = 0 .. R-1: x and stab loads first (the passes are bound
// by memory latency with one load chain per thread)
template <bool kCV, int R>
__device__ __forceinline__ void fx_load(const void* __restrict__ x, const uint16_t* __restrict__ stab, int64_t i,
                                        int64_t st, double (&re)[R], double (&im)[R], unsigned (&k)[R]) {
#pragma unroll
    for (int u = 0; u < R; ++u) {
        if (kCV) {
            const double2 v = ((const double2*)x)[i + u * st];
            re[u] = v.x;
            im[u] = v.y;
        } else {
            re[u] = ((const double*)x)[i + u * st];
            im[u] = 0.0;
        }
        k[u] = stab ? (unsigned)stab[i + u * st] : 1u;
    }
}

// max of v over the block (bit patterns of non-negative doubles order as the values)
__device__ __forceinline__ unsigned long long fx_block_max(unsigned long long m) {
    __shared__ unsigned long long wm[kThreads / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
    __syncthreads();
    m = threadIdx.x < kThreads / 32 ? wm[threadIdx.x] : 0ull;
    if (threadIdx.x < 32) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    }
    return m;   // valid in thread 0
}

// pass 1: per block, a bound of max |x_j sqrt(stab_j)| within a factor of two
template <bool kCV>
__global__ void __launch_bounds__(kThreads) fx_max_kernel(const void* __restrict__ x, const uint16_t* __restrict__ stab,
                                                          int64_t n, unsigned long long* __restrict__ part) {
    unsigned long long m = 0;
    const int64_t st = (int64_t)gridDim.x * blockDim.x;
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    auto take = [&](double re, double im, unsigned k) {
        const int c = fx_sqrt_exp(k);
        m = max(m, fx_bound_bits(re, c));
        if (kCV) m = max(m, fx_bound_bits(im, c));
    };
    for (; i + 3 * st < n; i += 4 * st) {
        double re[4], im[4];
        unsigned k[4];
        fx_load<kCV, 4>(x, stab, i, st, re, im, k);
#pragma unroll
        for (int u = 0; u < 4; ++u) take(re[u], im[u], k[u]);
    }
    for (; i < n; i += st) {
        double re[1], im[1];
        unsigned k[1];
        fx_load<kCV, 1>(x, stab, i, st, re, im, k);
        take(re[0], im[0], k[0]);
    }
    m = fx_block_max(m);
    if (threadIdx.x == 0) part[blockIdx.x] = m;
}

// pass 2: every block reduces the partial bounds (a few KB from L2), block 0
// publishes the total for the product kernel, and round(x_j sqrt(stab_j) 2^K)
// is stored as int64 (one FP64 multiply, the rounding in integers)
template <bool kCV>
__global__ void __launch_bounds__(kThreads) fx_quant_kernel(const void* __restrict__ x, const uint16_t* __restrict__ stab,
                                                            const double* __restrict__ sq, int64_t n,
                                                            const unsigned long long* __restrict__ part, int nparts,
                                                            unsigned long long* __restrict__ maxbits, int len_bits,
                                                            void* __restrict__ xq) {
    __shared__ double sqs[kMaxGroup + 1];
    __shared__ unsigned long long total;
    for (int i = threadIdx.x; i <= kMaxGroup; i += blockDim.x) sqs[i] = sq[i];
    unsigned long long m = 0;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) m = max(m, part[i]);
    m = fx_block_max(m);
    if (threadIdx.x == 0) {
        total = m;
        if (blockIdx.x == 0) *maxbits = m;
    }
    __syncthreads();
    const unsigned long long mb = total;
    if (!fx_finite(mb)) return;   // the product kernel takes the FP64 path
    const int K = fx_shift(mb, len_bits);
    auto store = [&](int64_t r, double re, double im, unsigned k) {
        const double s = sqs[k];
        if (kCV) {
            longlong2 q;
            q.x = fx_round_scaled(stab ? re * s : re, K);
            q.y = fx_round_scaled(stab ? im * s : im, K);
            ((longlong2*)xq)[r] = q;
        } else {
            ((long long*)xq)[r] = fx_round_scaled(stab ? re * s : re, K);
        }
    };
    const int64_t st = (int64_t)gridDim.x * blockDim.x;
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    for (; i + 3 * st < n; i += 4 * st) {
        double re[4], im[4];
        unsigned k[4];
        fx_load<kCV, 4>(x, stab, i, st, re, im, k);
#pragma unroll
        for (int u = 0; u < 4; ++u) store(i + u * st, re[u], im[u], k[u]);
    }
    for (; i < n; i += st) {
        double re[1], im[1];
        unsigned k[1];
        fx_load<kCV, 1>(x, stab, i, st, re, im, k);
        store(i, re[0], im[0], k[0]);
    }
}

// y[r] = beta y[r] + alpha (d[r] x[r] + acc) for a real diagonal
template <bool kCV>
__device__ __forceinline__ void fx_store_row(const SellArgs& a, int64_t r, double acc_r, double acc_i) {
    const double dr = ((const double*)a.diag_re)[r];
    if (kCV) {
        const double2 xv = ((const double2*)a.x)[r];
        acc_r += dr * xv.x;
        acc_i += dr * xv.y;
        double2* y = (double2*)a.y;
        double yr = 0, yi = 0;
        if (!a.beta_zero) {
            const double2 yo = y[r];
            yr = a.br * yo.x - a.bi * yo.y;
            yi = a.br * yo.y + a.bi * yo.x;
        }
        double2 o;
        o.x = yr + a.ar * acc_r - a.ai * acc_i;
        o.y = yi + a.ar * acc_i + a.ai * acc_r;
        y[r] = o;
    } else {
        acc_r += dr * ((const double*)a.x)[r];
        double* y = (double*)a.y;
        const double yr = a.beta_zero ? 0.0 : a.br * y[r];
        y[r] = yr + a.ar * acc_r;
    }
}

// One thread per row: integer sums per amplitude class, FP64 per row.  NC is
// the number of class accumulators (the operator's classes, rounded up).
// kHint marks only the word stream here: the kernel runs at 32 registers, and
// an x cache-policy operand on top spills.
// x that holds a NaN or an infinity has no fixed-point scale: then every row
// is computed as by the FP64 product, so non-finite values propagate alike.
template <bool kCV, bool kPacked, int NC, int U, int MINB, bool kHint>
__global__ void __launch_bounds__(kThreads, MINB) sell_fx_kernel(SellArgs a, FxArgs f) {
    __shared__ uint32_t ccls[kFxCodes];
    __shared__ double rsk[kMaxGroup + 1];
    __shared__ double amp[NC];
    const unsigned long long mb = *f.maxbits;
    const int K = fx_shift(mb, f.len_bits);
    // 2^-K folds into the row scale unless it leaves the normal range
    const bool fold = K >= -900 && K <= 900;
    for (int i = threadIdx.x; i < a.ncodes; i += blockDim.x) ccls[i] = f.cls[i];
    for (int i = threadIdx.x; i <= kMaxGroup; i += blockDim.x) {
        const double r = i ? 1.0 / sqrt((double)i) : 0.0;
        rsk[i] = fold ? r * fx_pow2(-K) : r;
    }
    if (threadIdx.x < NC) amp[threadIdx.x] = f.amp[threadIdx.x];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t warp0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    if (!fx_finite(mb)) {
        // the FP64 product's arithmetic
        const double2* __restrict__ tab = (const double2*)a.table;
        for (int64_t s = a.slice0 + warp0; s < a.nslices; s += nwarps) {
            const int64_t r = s * kSlice + lane;
            if (r >= a.n) continue;
            double acc_r = 0, acc_i = 0;
            if (kCV) {
                const double2* __restrict__ x = (const double2*)a.x;
                sell_row<1, kPacked, kHint>(a.words, a.cols, a.codes, a.sptr[s] + lane, a.len[r], a.code_bits, a.code_mask,
                                     [&](uint32_t c) { return ld_gather<kHint>(x + c); },
                                     [&](uint32_t code, double2 xv) {
                                         const double v = __ldg(&tab[code].x);
                                         acc_r += v * xv.x;
                                         acc_i += v * xv.y;
                                     });
            } else {
                const double* __restrict__ x = (const double*)a.x;
                sell_row<1, kPacked, kHint>(a.words, a.cols, a.codes, a.sptr[s] + lane, a.len[r], a.code_bits, a.code_mask,
                                     [&](uint32_t c) { return ld_gather<kHint>(x + c); },
                                     [&](uint32_t code, double xv) { acc_r += __ldg(&tab[code].x) * xv; });
            }
            const double sc = a.stab ? 1.0 / sqrt((double)a.stab[r]) : 1.0;
            fx_store_row<kCV>(a, r, acc_r * sc, acc_i * sc);
        }
        return;
    }
    // rows and slices fit in 32 bits (columns are 32-bit): fewer registers
    const int nsl = (int)a.nslices, nrows = (int)a.n, step = (int)nwarps;
    for (int s = (int)(a.slice0 + warp0); s < nsl; s += step) {
        const int r = s * kSlice + lane;
        if (r >= nrows) continue;
        const int len = a.len[r];
        const int64_t base = a.sptr[s] + lane;
        double acc_r = 0, acc_i = 0;
        // all classes' signed sum (the sign applied as a mask), and the sums of
        // classes 1 .. NC-1 by mask; class 0 is their difference (exact in two's
        // complement)
        if (kCV) {
            long long tr = 0, ti = 0, sr[NC], si[NC];
#pragma unroll
            for (int c = 1; c < NC; ++c) sr[c] = si[c] = 0;
            const longlong2* __restrict__ xq = (const longlong2*)f.xq;
            sell_row<U, kPacked, kHint>(a.words, a.cols, a.codes, base, len, a.code_bits, a.code_mask,
                                 [&](uint32_t c) { return ld_gather<false>(xq + c); },
                                 [&](uint32_t code, longlong2 q) {
                                     const uint32_t w = ccls[code];
                                     const long long m = -(long long)(w & 1u);
                                     const long long vr = (q.x ^ m) - m, vi = (q.y ^ m) - m;
                                     tr += vr;
                                     ti += vi;
#pragma unroll
                                     for (int c = 1; c < NC; ++c) {
                                         const long long cm = -(long long)((w >> 1) == (uint32_t)c);
                                         sr[c] += vr & cm;
                                         si[c] += vi & cm;
                                     }
                                 });
            long long r0 = tr, i0 = ti;
#pragma unroll
            for (int c = 1; c < NC; ++c) {
                r0 -= sr[c];
                i0 -= si[c];
                acc_r = fma(amp[c], __ll2double_rn(sr[c]), acc_r);
                acc_i = fma(amp[c], __ll2double_rn(si[c]), acc_i);
            }
            acc_r = fma(amp[0], __ll2double_rn(r0), acc_r);
            acc_i = fma(amp[0], __ll2double_rn(i0), acc_i);
        } else {
            long long t = 0, sr[NC];
#pragma unroll
            for (int c = 1; c < NC; ++c) sr[c] = 0;
            const long long* __restrict__ xq = (const long long*)f.xq;
            sell_row<U, kPacked, kHint>(a.words, a.cols, a.codes, base, len, a.code_bits, a.code_mask,
                                 [&](uint32_t c) { return ld_gather<false>(xq + c); },
                                 [&](uint32_t code, long long q) {
                                     const uint32_t w = ccls[code];
                                     const long long m = -(long long)(w & 1u);
                                     const long long v = (q ^ m) - m;
                                     t += v;
#pragma unroll
                                     for (int c = 1; c < NC; ++c) sr[c] += v & -(long long)((w >> 1) == (uint32_t)c);
                                 });
            long long r0 = t;
#pragma unroll
            for (int c = 1; c < NC; ++c) {
                r0 -= sr[c];
                acc_r = fma(amp[c], __ll2double_rn(sr[c]), acc_r);
            }
            acc_r = fma(amp[0], __ll2double_rn(r0), acc_r);
        }
        const double sc = rsk[a.stab ? a.stab[r] : 1];
        acc_r *= sc;
        acc_i *= sc;
        if (!fold) {
            const int k1 = K / 2;
            const double u1 = fx_pow2(-k1), u2 = fx_pow2(k1 - K);
            acc_r = acc_r * u1 * u2;
            acc_i = acc_i * u1 * u2;
        }
        fx_store_row<kCV>(a, r, acc_r, acc_i);
    }
}

// the fixed-point product's variants (gathers in flight, resident blocks):
// complex vectors and four classes hold more accumulators, so fewer blocks
template <bool kCV, bool kPacked, int NC>
void launch_fx(int v, int grid, cudaStream_t s, const SellArgs& a, const FxArgs& f) {
    constexpr int B0 = kCV ? 4 : (NC <= 2 ? 8 : 6);
    constexpr int B1 = (kCV || NC > 2) ? 4 : 6;
    switch (v) {
        case 0: sell_fx_kernel<kCV, kPacked, NC, 1, B0, false><<<grid, kThreads, 0, s>>>(a, f); break;
        case 1: sell_fx_kernel<kCV, kPacked, NC, 2, B1, false><<<grid, kThreads, 0, s>>>(a, f); break;
        case 2: sell_fx_kernel<kCV, kPacked, NC, 4, 4, false><<<grid, kThreads, 0, s>>>(a, f); break;
        case 3: sell_fx_kernel<kCV, kPacked, NC, 1, B0, true><<<grid, kThreads, 0, s>>>(a, f); break;
        case 4: sell_fx_kernel<kCV, kPacked, NC, 2, B1, true><<<grid, kThreads, 0, s>>>(a, f); break;
        default: sell_fx_kernel<kCV, kPacked, NC, 4, 4, true><<<grid, kThreads, 0, s>>>(a, f); break;
    }
}

// six sliced-ELL variants: three (gathers in flight, blocks per SM) shapes,
// each with plain loads and with the evict-first / evict-last hints
constexpr int kSellVariants = 6;

// QS_TUNE_VERBOSE=1 prints the variant timings of each tuning to stderr
bool tune_verbose() {
    static const bool on = [] {
        const char* e = std::getenv("QS_TUNE_VERBOSE");
        return e && e[0] && e[0] != '0';
    }();
    return on;
}

// QS_SELL_VARIANT=v (0 .. kSellVariants - 1) runs variant v instead of the
// timed choice (read on every product; the tests run every variant with it)
int forced_variant() {
    const char* e = std::getenv("QS_SELL_VARIANT");
    if (!e || !e[0]) return -1;
    const int v = std::atoi(e);
    return (v >= 0 && v < kSellVariants) ? v : -1;
}

int grid_rows(int64_t threads_needed) {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int64_t blocks = (threads_needed + kThreads - 1) / kThreads;
    int64_t cap = (int64_t)sms * 8;
    return (int)std::max<int64_t>(1, std::min(blocks, cap));
}

}  // namespace

// Sliced-ELL copy of the CSR words: slices of kSlice consecutive rows, words
// column-major inside a slice; every row keeps its own length, so the padding
// of a slice is allocated but never read.
void build_sell(const Basis& b, Assembled& M, cudaStream_t s) {
    const int64_t n = b.n;
    std::vector<int64_t> rp(n + 1);
    QS_CUDA(cudaMemcpy(rp.data(), M.rowptr.p, (n + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost));
    int64_t maxlen = 0;
    for (int64_t r = 0; r < n; ++r) maxlen = std::max<int64_t>(maxlen, rp[r + 1] - rp[r]);
    if (maxlen > 65535) return;  // keep the CSR path
    M.len_bits = 0;
    while (((int64_t)1 << M.len_bits) < maxlen) ++M.len_bits;
    M.nslices = (n + kSlice - 1) / kSlice;
    const int64_t npos = M.nslices * kSlice;
    std::vector<int32_t> perm(npos, -1);
    std::vector<uint16_t> len(npos, 0);
    // Rows stay in their natural order: each thread loops over its own row
    // only, so a slice's padding is never read, while the natural order keeps
    // y, the diagonal and x[r] coalesced and the x gathers of neighbouring
    // rows close together (sorting by length inside windows measured slower).
    for (int64_t r = 0; r < n; ++r) {
        perm[r] = (int32_t)r;
        len[r] = (uint16_t)(rp[r + 1] - rp[r]);
    }
    std::vector<int64_t> sptr(M.nslices + 1, 0);
    for (int64_t sl = 0; sl < M.nslices; ++sl) {
        int mx = 0;
        for (int l = 0; l < kSlice; ++l) mx = std::max<int>(mx, len[sl * kSlice + l]);
        sptr[sl + 1] = sptr[sl] + (int64_t)mx * kSlice;
    }
    const int64_t total = std::max<int64_t>(1, sptr[M.nslices]);
    M.sell_ptr.alloc((M.nslices + 1) * sizeof(int64_t));
    M.sell_perm.alloc(npos * sizeof(int32_t));
    M.sell_len.alloc(npos * sizeof(uint16_t));
    QS_CUDA(cudaMemcpy(M.sell_ptr.p, sptr.data(), (M.nslices + 1) * sizeof(int64_t), cudaMemcpyHostToDevice));
    QS_CUDA(cudaMemcpy(M.sell_perm.p, perm.data(), npos * sizeof(int32_t), cudaMemcpyHostToDevice));
    QS_CUDA(cudaMemcpy(M.sell_len.p, len.data(), npos * sizeof(uint16_t), cudaMemcpyHostToDevice));
    if (M.packed) {
        M.sell_words.alloc(total * sizeof(uint32_t));
    } else {
        M.sell_cols.alloc(total * sizeof(int32_t));
        M.sell_codes.alloc(total * sizeof(uint16_t));
    }
    sell_fill_kernel<<<grid_rows(npos), kThreads, 0, s>>>(M.rowptr.as<int64_t>(), M.words.as<uint32_t>(),
                                                         M.cols.as<int32_t>(), M.codes.as<uint16_t>(), M.packed,
                                                         M.sell_perm.as<int32_t>(), M.sell_ptr.as<int64_t>(), npos,
                                                         M.sell_words.as<uint32_t>(), M.sell_cols.as<int32_t>(),
                                                         M.sell_codes.as<uint16_t>());
    QS_CUDA(cudaGetLastError());
    QS_CUDA(cudaStreamSynchronize(s));
    note_launches(1);
    M.has_sell = true;
}

void op_assemble(Op& op) {
    Basis& b = *op.basis;
    if (op.assembled) return;
    if (!op.commuting) throw Error(QS_ERR_UNSUPPORTED, "only symmetry-commuting operators are assembled");
    const size_t nfwd = op.progs.size() / 2;
    std::vector<TermProg> fwd(op.progs.begin(), op.progs.begin() + nfwd);
    for (const TermProg& p : fwd)
        if (!p.distinct) throw Error(QS_ERR_UNSUPPORTED, "operators acting twice on one site are not assembled");
    // value classes
    using cd = std::complex<double>;
    auto canon = [](cd v, int& sign) {
        sign = 0;
        if (v.real() < 0 || (v.real() == 0 && v.imag() < 0)) { v = -v; sign = 1; }
        return v;
    };
    std::vector<cd> A, C;
    std::vector<uint16_t> prog_code(std::max<size_t>(1, nfwd));
    for (size_t k = 0; k < nfwd; ++k) {
        int sg;
        cd v = canon(cd(fwd[k].amp0_re, fwd[k].amp0_im), sg);
        size_t c = 0;
        while (c < A.size() && A[c] != v) ++c;
        if (c == A.size()) A.push_back(v);
        prog_code[k] = (uint16_t)(c * 2 + sg);
    }
    if (A.empty()) A.push_back(cd(0, 0));
    const GroupDesc& G = b.group;
    std::vector<uint16_t> elem_code(kMaxGroup, 0);
    std::vector<uint8_t> stab_class(kMaxGroup + 1, 0);
    std::vector<double> D;
    if (b.symmetric) {
        for (int e = 0; e < G.ng; ++e) {
            int sg;
            cd v = canon(cd(G.chi_re[e], G.chi_im[e]), sg);
            size_t c = 0;
            while (c < C.size() && std::abs(C[c] - v) > 1e-14) ++c;
            if (c == C.size()) C.push_back(v);
            elem_code[e] = (uint16_t)(c * 2 + sg);
        }
        for (int st = 1; st <= G.ng; ++st)
            if (G.ng % st == 0) {
                stab_class[st] = (uint8_t)D.size();
                D.push_back(std::sqrt((double)st));
            }
    } else {
        C.push_back(cd(1, 0));
        D.push_back(1.0);
    }
    const int nA = (int)A.size(), nC = (int)C.size(), nD = (int)D.size();
    const int64_t ncodes = (int64_t)nA * nC * nD * 2;
    if (ncodes > 65536) throw Error(QS_ERR_UNSUPPORTED, "too many distinct matrix elements to assemble");
    int col_bits = 1;
    while (((int64_t)1 << col_bits) < b.n) ++col_bits;
    int code_bits = 1;
    while (((int64_t)1 << code_bits) < ncodes) ++code_bits;
    const bool packed = col_bits + code_bits <= 32;
    if (packed) code_bits = 32 - col_bits;
    std::vector<cd> table(ncodes);
    for (int a = 0; a < nA; ++a)
        for (int c = 0; c < nC; ++c)
            for (int d = 0; d < nD; ++d)
                for (int sg = 0; sg < 2; ++sg) {
                    cd v = A[a] * C[c] * D[d];
                    table[(((int64_t)a * nC + c) * nD + d) * 2 + sg] = sg ? -v : v;
                }
    Assembled& M = op.asm_;
    M.ncodes = (int)ncodes;
    M.code_bits = code_bits;
    M.packed = packed;
    M.table64.alloc(ncodes * sizeof(cd));
    QS_CUDA(cudaMemcpy(M.table64.p, table.data(), ncodes * sizeof(cd), cudaMemcpyHostToDevice));
    std::vector<std::complex<float>> t32(ncodes);
    for (int64_t i = 0; i < ncodes; ++i) t32[i] = std::complex<float>((float)table[i].real(), (float)table[i].imag());
    M.table32.alloc(ncodes * sizeof(std::complex<float>));
    QS_CUDA(cudaMemcpy(M.table32.p, t32.data(), ncodes * sizeof(std::complex<float>), cudaMemcpyHostToDevice));
    std::vector<float> tdf(4 * ncodes);
    for (int64_t i = 0; i < ncodes; ++i) {
        double re = table[i].real(), im = table[i].imag();
        float rh = (float)re, ih = (float)im;
        tdf[4 * i] = rh;
        tdf[4 * i + 1] = (float)(re - (double)rh);
        tdf[4 * i + 2] = ih;
        tdf[4 * i + 3] = (float)(im - (double)ih);
    }
    M.table_df.alloc(ncodes * 4 * sizeof(float));
    QS_CUDA(cudaMemcpy(M.table_df.p, tdf.data(), ncodes * 4 * sizeof(float), cudaMemcpyHostToDevice));
    {
        // fixed-point row sums: value(code) = +-amp[class] * D[d], with class =
        // a * nC + c real and at most four of them
        const int ncls = nA * nC;
        bool ok = !op.complex_mat && ncls <= 4 && ncodes <= kFxCodes;
        std::vector<double> amp(4, 0.0);
        for (int a = 0; ok && a < nA; ++a)
            for (int c = 0; c < nC; ++c) {
                const cd v = A[a] * C[c];
                if (v.imag() != 0.0) ok = false;
                amp[a * nC + c] = v.real();
            }
        M.fx_classes = 0;
        if (ok) {
            // per code: class << 1 | sign
            std::vector<uint32_t> cls(ncodes);
            for (int64_t code = 0; code < ncodes; ++code)
                cls[code] = (uint32_t)((((code >> 1) / nD) << 1) | (code & 1));
            std::vector<double> sq(kMaxGroup + 1);
            for (int i = 0; i <= kMaxGroup; ++i) sq[i] = std::sqrt((double)i);
            M.fx_cls.alloc(cls.size() * sizeof(uint32_t));
            QS_CUDA(cudaMemcpy(M.fx_cls.p, cls.data(), cls.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
            M.fx_amp.alloc(4 * sizeof(double));
            QS_CUDA(cudaMemcpy(M.fx_amp.p, amp.data(), 4 * sizeof(double), cudaMemcpyHostToDevice));
            M.fx_sq.alloc(sq.size() * sizeof(double));
            QS_CUDA(cudaMemcpy(M.fx_sq.p, sq.data(), sq.size() * sizeof(double), cudaMemcpyHostToDevice));
            M.fx_max.alloc((1 + kFxParts) * sizeof(unsigned long long));
            M.fx_classes = ncls;
        }
    }
    {
        std::vector<float> rq(2 * (kMaxGroup + 1), 0.f);
        for (int i = 1; i <= kMaxGroup; ++i) df_split_host(1.0 / std::sqrt((double)i), rq[2 * i], rq[2 * i + 1]);
        M.rsq_df.alloc(rq.size() * sizeof(float));
        QS_CUDA(cudaMemcpy(M.rsq_df.p, rq.data(), rq.size() * sizeof(float), cudaMemcpyHostToDevice));
    }
    M.xsplit.alloc((size_t)b.n * 4 * sizeof(float));

    cudaStream_t s = op.stream;
    std::vector<uint16_t> fast_code(std::max<size_t>(1, b.fast_to_elem.size()), 0);
    for (size_t i = 0; i < b.fast_to_elem.size(); ++i) fast_code[i] = elem_code[b.fast_to_elem[i]];
    DevBuf d_prog(fwd.size() * sizeof(TermProg) + 1), d_pc(prog_code.size() * 2), d_ec(kMaxGroup * 2),
        d_sc(kMaxGroup + 1), d_fc(fast_code.size() * 2);
    QS_CUDA(cudaMemcpy(d_fc.p, fast_code.data(), fast_code.size() * 2, cudaMemcpyHostToDevice));
    if (!fwd.empty())
        QS_CUDA(cudaMemcpy(d_prog.p, fwd.data(), fwd.size() * sizeof(TermProg), cudaMemcpyHostToDevice));
    QS_CUDA(cudaMemcpy(d_pc.p, prog_code.data(), prog_code.size() * 2, cudaMemcpyHostToDevice));
    QS_CUDA(cudaMemcpy(d_ec.p, elem_code.data(), kMaxGroup * 2, cudaMemcpyHostToDevice));
    QS_CUDA(cudaMemcpy(d_sc.p, stab_class.data(), kMaxGroup + 1, cudaMemcpyHostToDevice));
    BuildArgs a{};
    a.reps = b.d_reps.p;
    a.stab = b.d_stab.as<uint16_t>();
    a.split = b.d_split.p;
    a.n = b.n;
    a.nsplit = b.nsplit;
    a.stride = b.split_stride;
    a.group = b.d_group.as<GroupDesc>();
    a.binom = b.d_binom.as<uint64_t>();
    a.index = b.has_index ? b.d_index.as<int32_t>() : nullptr;
    a.L = b.L;
    a.nup = b.nup;
    a.mode = b.symmetric ? (b.has_index ? 3 : 2) : (b.nup >= 0 ? 1 : 0);
    a.progs = d_prog.as<TermProg>();
    a.nprog = (int)fwd.size();
    a.prog_code = d_pc.as<uint16_t>();
    a.elem_code = d_ec.as<uint16_t>();
    a.stab_class = d_sc.as<uint8_t>();
    a.fast = b.fast;
    a.fast_code = d_fc.as<uint16_t>();
    a.nC = nC;
    a.nD = nD;
    a.code_bits = code_bits;
    a.packed = packed;
    DevBuf cnt32(b.n * sizeof(int32_t)), cnt64(b.n * sizeof(int64_t));
    M.rowptr.alloc((b.n + 1) * sizeof(int64_t));
    a.counts = cnt32.as<int32_t>();
    int grid = grid_rows(b.n);
    const bool wide = b.symmetric ? b.wide : true;
    if (wide) build_kernel<uint64_t, false><<<grid, kThreads, 0, s>>>(a);
    else build_kernel<uint32_t, false><<<grid, kThreads, 0, s>>>(a);
    QS_CUDA(cudaGetLastError());
    counts_to_i64<<<grid, kThreads, 0, s>>>(cnt32.as<int32_t>(), cnt64.as<int64_t>(), b.n);
    QS_CUDA(cudaGetLastError());
    scan_i64(cnt64.as<int64_t>(), M.rowptr.as<int64_t>(), b.n, s);
    int64_t last = 0, lastc = 0;
    QS_CUDA(cudaMemcpyAsync(&last, M.rowptr.as<int64_t>() + b.n - 1, 8, cudaMemcpyDeviceToHost, s));
    QS_CUDA(cudaMemcpyAsync(&lastc, cnt64.as<int64_t>() + b.n - 1, 8, cudaMemcpyDeviceToHost, s));
    QS_CUDA(cudaStreamSynchronize(s));
    M.nnz = last + lastc;
    QS_CUDA(cudaMemcpy(M.rowptr.as<int64_t>() + b.n, &M.nnz, 8, cudaMemcpyHostToDevice));
    if (packed) {
        M.words.alloc(std::max<int64_t>(1, M.nnz) * sizeof(uint32_t));
        a.words = M.words.as<uint32_t>();
    } else {
        M.cols.alloc(std::max<int64_t>(1, M.nnz) * sizeof(int32_t));
        M.codes.alloc(std::max<int64_t>(1, M.nnz) * sizeof(uint16_t));
        a.cols = M.cols.as<int32_t>();
        a.codes = M.codes.as<uint16_t>();
    }
    a.rowptr = M.rowptr.as<int64_t>();
    if (wide) build_kernel<uint64_t, true><<<grid, kThreads, 0, s>>>(a);
    else build_kernel<uint32_t, true><<<grid, kThreads, 0, s>>>(a);
    QS_CUDA(cudaGetLastError());
    QS_CUDA(cudaStreamSynchronize(s));
    note_launches(4);
    // lanes per row: the power of two nearest a quarter of the mean row length
    double mean = b.n ? (double)M.nnz / (double)b.n : 0.0;
    M.lanes = mean > 48 ? 16 : (mean > 12 ? 8 : 4);
    build_sell(b, M, s);
    op.assembled = true;
}

void op_spmv_device(Op& op, const MatvecCall& c, cudaStream_t s) {
    const Basis& b = *op.basis;
    const Assembled& M = op.asm_;
    if (c.df_io && !M.has_sell) throw Error(QS_ERR_UNSUPPORTED, "double-float vectors need the sliced layout");
    if (M.has_sell) {
        SellArgs a{};
        a.sptr = M.sell_ptr.as<int64_t>();
        a.perm = M.sell_perm.as<int32_t>();
        a.len = M.sell_len.as<uint16_t>();
        a.words = M.sell_words.as<uint32_t>();
        a.cols = M.sell_cols.as<int32_t>();
        a.codes = M.sell_codes.as<uint16_t>();
        a.packed = M.packed;
        a.code_bits = M.code_bits;
        a.code_mask = M.code_bits >= 32 ? 0xffffffffu : ((1u << M.code_bits) - 1u);
        a.ncodes = M.ncodes;
        a.stab = b.symmetric ? b.d_stab.as<uint16_t>() : nullptr;
        a.nslices = c.slice1 >= 0 ? std::min<int64_t>(c.slice1, M.nslices) : M.nslices;
        a.slice0 = c.slice0;
        a.n = b.n;
        a.ar = c.alpha.re;
        a.ai = c.alpha.im;
        a.br = c.beta.re;
        a.bi = c.beta.im;
        a.beta_zero = (c.beta.re == 0.0 && c.beta.im == 0.0);
        const bool T = (c.flags & QS_TRANSPOSE) != 0, C = (c.flags & QS_CONJUGATE) != 0;
        a.conj = T != C;
        a.x = c.x;
        a.y = c.y;
        const bool cm = op.complex_mat, cv = c.y_complex;
        const int grid = grid_rows(std::max<int64_t>(1, a.nslices - a.slice0) * kSlice);
        // variants: (gathers in flight per thread, resident blocks per SM) x
        // (plain loads, or the word stream evict-first and x evict-last)
#define QS_VARIANTS(LAUNCH, v)                         \
    do {                                               \
        switch (v) {                                   \
            case 0: LAUNCH(1, 8, false); break;        \
            case 1: LAUNCH(2, 6, false); break;        \
            case 2: LAUNCH(4, 4, false); break;        \
            case 3: LAUNCH(1, 8, true); break;         \
            case 4: LAUNCH(2, 6, true); break;         \
            default: LAUNCH(4, 4, true); break;        \
        }                                              \
    } while (0)
#define QS_SHAPES(K, U_, B_, H_, ...)                                                        \
    do {                                                                                     \
        if (a.packed) {                                                                      \
            if (cm) K<true, true, true, U_, B_, H_><<<grid, kThreads, 0, s>>>(__VA_ARGS__);        \
            else if (cv) K<false, true, true, U_, B_, H_><<<grid, kThreads, 0, s>>>(__VA_ARGS__);  \
            else K<false, false, true, U_, B_, H_><<<grid, kThreads, 0, s>>>(__VA_ARGS__);         \
        } else {                                                                             \
            if (cm) K<true, true, false, U_, B_, H_><<<grid, kThreads, 0, s>>>(__VA_ARGS__);       \
            else if (cv) K<false, true, false, U_, B_, H_><<<grid, kThreads, 0, s>>>(__VA_ARGS__); \
            else K<false, false, false, U_, B_, H_><<<grid, kThreads, 0, s>>>(__VA_ARGS__);        \
        }                                                                                    \
    } while (0)
        int kind;
        std::function<void(int)> launch;
        const float4* td = M.table_df.as<float4>();
        if (c.df_io) {
            kind = 3;
            const float4* dd = op.d_diag_df.as<float4>();
            const float2* rq = M.rsq_df.as<float2>();
            launch = [&, td, dd, rq](int v) {
#define L_DFIO(U_, B_, H_) QS_SHAPES(sell_dfio_kernel, U_, B_, H_, a, td, dd, rq)
                QS_VARIANTS(L_DFIO, v);
#undef L_DFIO
            };
        } else if (c.fx && !c.single && M.fx_classes > 0) {
            kind = 4;
            a.table = M.table64.p;
            a.diag = op.d_diag.p;
            a.diag_re = op.d_diag_re.p;
            FxArgs f{};
            f.cls = M.fx_cls.as<uint32_t>();
            f.amp = M.fx_amp.as<double>();
            f.sq = M.fx_sq.as<double>();
            f.part = M.fx_max.as<unsigned long long>() + 1;
            f.maxbits = M.fx_max.as<unsigned long long>();
            f.len_bits = M.len_bits;
            f.xq = M.xsplit.p;
            if (!c.fx_ready) {
                // max |x sqrt(stab)| per block, then the total and the scaled integer copy
                const int sg = std::min(grid_rows(b.n), kFxParts);
                if (cv) {
                    fx_max_kernel<true><<<sg, kThreads, 0, s>>>(c.x, a.stab, b.n, f.part);
                    fx_quant_kernel<true><<<sg, kThreads, 0, s>>>(c.x, a.stab, f.sq, b.n, f.part, sg, f.maxbits,
                                                                  f.len_bits, f.xq);
                } else {
                    fx_max_kernel<false><<<sg, kThreads, 0, s>>>(c.x, a.stab, b.n, f.part);
                    fx_quant_kernel<false><<<sg, kThreads, 0, s>>>(c.x, a.stab, f.sq, b.n, f.part, sg, f.maxbits,
                                                                   f.len_bits, f.xq);
                }
                QS_CUDA(cudaGetLastError());
                note_launches(2);
            }
            const int nc = M.fx_classes;
            launch = [&, f, nc](int v) {
                if (a.packed) {
                    if (cv) (nc <= 2 ? launch_fx<true, true, 2> : launch_fx<true, true, 4>)(v, grid, s, a, f);
                    else (nc <= 2 ? launch_fx<false, true, 2> : launch_fx<false, true, 4>)(v, grid, s, a, f);
                } else {
                    if (cv) (nc <= 2 ? launch_fx<true, false, 2> : launch_fx<true, false, 4>)(v, grid, s, a, f);
                    else (nc <= 2 ? launch_fx<false, false, 2> : launch_fx<false, false, 4>)(v, grid, s, a, f);
                }
            };
        } else if (c.df && !c.single) {
            kind = 2;
            a.table = M.table64.p;
            a.diag = op.d_diag.p;
            a.diag_re = op.d_diag_re.p;
            const int sg = grid_rows(b.n);
            if (cv) split_kernel<true><<<sg, kThreads, 0, s>>>(c.x, M.xsplit.as<float4>(), nullptr, b.n);
            else split_kernel<false><<<sg, kThreads, 0, s>>>(c.x, nullptr, M.xsplit.as<float2>(), b.n);
            QS_CUDA(cudaGetLastError());
            note_launches(1);
            const void* xs = M.xsplit.p;
            launch = [&, td, xs](int v) {
#define L_DF(U_, B_, H_) QS_SHAPES(sell_df_kernel, U_, B_, H_, a, td, xs)
                QS_VARIANTS(L_DF, v);
#undef L_DF
            };
        } else if (c.single) {
            kind = 1;
            a.table = M.table32.p;
            a.diag = op.d_diag32.p;
            a.diag_re = op.d_diag32_re.p;
            launch = [&](int v) {
#define L_32(U_, B_, H_)                                                                           \
    do {                                                                                           \
        if (a.packed) {                                                                            \
            if (cm) sell_kernel<true, true, float, true, U_, B_, H_><<<grid, kThreads, 0, s>>>(a);       \
            else if (cv) sell_kernel<false, true, float, true, U_, B_, H_><<<grid, kThreads, 0, s>>>(a); \
            else sell_kernel<false, false, float, true, U_, B_, H_><<<grid, kThreads, 0, s>>>(a);        \
        } else {                                                                                   \
            if (cm) sell_kernel<true, true, float, false, U_, B_, H_><<<grid, kThreads, 0, s>>>(a);      \
            else if (cv) sell_kernel<false, true, float, false, U_, B_, H_><<<grid, kThreads, 0, s>>>(a);\
            else sell_kernel<false, false, float, false, U_, B_, H_><<<grid, kThreads, 0, s>>>(a);       \
        }                                                                                          \
    } while (0)
                QS_VARIANTS(L_32, v);
#undef L_32
            };
        } else {
            kind = 0;
            a.table = M.table64.p;
            a.diag = op.d_diag.p;
            a.diag_re = op.d_diag_re.p;
            launch = [&](int v) {
#define L_64(U_, B_, H_)                                                                           \
    do {                                                                                           \
        if (a.packed) {                                                                            \
            if (cm) sell_kernel<true, true, double, true, U_, B_, H_><<<grid, kThreads, 0, s>>>(a);       \
            else if (cv) sell_kernel<false, true, double, true, U_, B_, H_><<<grid, kThreads, 0, s>>>(a); \
            else sell_kernel<false, false, double, true, U_, B_, H_><<<grid, kThreads, 0, s>>>(a);        \
        } else {                                                                                   \
            if (cm) sell_kernel<true, true, double, false, U_, B_, H_><<<grid, kThreads, 0, s>>>(a);      \
            else if (cv) sell_kernel<false, true, double, false, U_, B_, H_><<<grid, kThreads, 0, s>>>(a);\
            else sell_kernel<false, false, double, false, U_, B_, H_><<<grid, kThreads, 0, s>>>(a);       \
        }                                                                                          \
    } while (0)
                QS_VARIANTS(L_64, v);
#undef L_64
            };
        }
#undef QS_SHAPES
#undef QS_VARIANTS
        int& var = op.asm_.sell_variant[kind];
        if (var < 0 && !c.no_tune && forced_variant() < 0) {
            // choose the variant by timing, when repeating the product is harmless
            // (beta = 0) and the stream is not being captured into a graph
            cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
            QS_CUDA(cudaStreamIsCapturing(s, &cap));
            if (a.beta_zero && cap == cudaStreamCaptureStatusNone) {
                cudaEvent_t e0, e1;
                QS_CUDA(cudaEventCreate(&e0));
                QS_CUDA(cudaEventCreate(&e1));
                float best = 1e30f;
                int bv = 2;
                float ms_v[kSellVariants] = {};
                for (int v = 0; v < kSellVariants; ++v) {
                    launch(v);
                    QS_CUDA(cudaGetLastError());
                    QS_CUDA(cudaEventRecord(e0, s));
                    for (int r = 0; r < 3; ++r) launch(v);
                    QS_CUDA(cudaEventRecord(e1, s));
                    QS_CUDA(cudaEventSynchronize(e1));
                    float ms = 0;
                    QS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                    ms_v[v] = ms / 3;
                    if (ms < best) {
                        best = ms;
                        bv = v;
                    }
                }
                cudaEventDestroy(e0);
                cudaEventDestroy(e1);
                note_launches(4 * kSellVariants);
                if (tune_verbose()) {
                    std::fprintf(stderr, "qsgpu: sliced-ELL product kind %d, n=%lld: variant ms", kind, (long long)b.n);
                    for (int v = 0; v < kSellVariants; ++v) std::fprintf(stderr, " %d:%.4f", v, ms_v[v]);
                    std::fprintf(stderr, " -> %d\n", bv);
                }
                var = bv;
            }
        }
        const int fv = forced_variant();
        launch(fv >= 0 ? fv : (var < 0 ? 2 : var));
        QS_CUDA(cudaGetLastError());
        note_launches(1);
        return;
    }
    SpmvArgs a{};
    a.rowptr = M.rowptr.as<int64_t>();
    a.words = M.words.as<uint32_t>();
    a.cols = M.cols.as<int32_t>();
    a.codes = M.codes.as<uint16_t>();
    a.packed = M.packed;
    a.code_bits = M.code_bits;
    a.code_mask = M.code_bits >= 32 ? 0xffffffffu : ((1u << M.code_bits) - 1u);
    a.ncodes = M.ncodes;
    a.stab = b.symmetric ? b.d_stab.as<uint16_t>() : nullptr;
    a.n = b.n;
    a.ar = c.alpha.re;
    a.ai = c.alpha.im;
    a.br = c.beta.re;
    a.bi = c.beta.im;
    a.beta_zero = (c.beta.re == 0.0 && c.beta.im == 0.0);
    const bool T = (c.flags & QS_TRANSPOSE) != 0, C = (c.flags & QS_CONJUGATE) != 0;
    // transpose of a Hermitian operator is its conjugate
    a.conj = T != C;
    a.x = c.x;
    a.y = c.y;
    const bool cm = op.complex_mat, cv = c.y_complex;
    const int64_t thr = b.n * M.lanes;
    const int grid = grid_rows(thr);
#define QS_SPMV(G, T_)                                                                          \
    do {                                                                                        \
        if (cm) spmv_kernel<G, true, true, T_><<<grid, kThreads, 0, s>>>(a);                    \
        else if (cv) spmv_kernel<G, false, true, T_><<<grid, kThreads, 0, s>>>(a);              \
        else spmv_kernel<G, false, false, T_><<<grid, kThreads, 0, s>>>(a);                     \
    } while (0)
    if (c.df && !c.single) {
        a.diag = op.d_diag.p;
        SpmvDFArgs da{};
        da.s = a;
        da.tab_df = M.table_df.as<float4>();
        da.xs = M.xsplit.p;
        const int sg = grid_rows(b.n);
        if (cv) split_kernel<true><<<sg, kThreads, 0, s>>>(c.x, M.xsplit.as<float4>(), nullptr, b.n);
        else split_kernel<false><<<sg, kThreads, 0, s>>>(c.x, nullptr, M.xsplit.as<float2>(), b.n);
        QS_CUDA(cudaGetLastError());
#define QS_SPMV_DF(G)                                                                           \
        do {                                                                                    \
            if (cm) spmv_df_kernel<G, true, true><<<grid, kThreads, 0, s>>>(da);                \
            else if (cv) spmv_df_kernel<G, false, true><<<grid, kThreads, 0, s>>>(da);          \
            else spmv_df_kernel<G, false, false><<<grid, kThreads, 0, s>>>(da);                 \
        } while (0)
        if (M.lanes == 16) QS_SPMV_DF(16);
        else if (M.lanes == 8) QS_SPMV_DF(8);
        else QS_SPMV_DF(4);
#undef QS_SPMV_DF
        QS_CUDA(cudaGetLastError());
        note_launches(2);
        return;
    }
    if (c.single) {
        a.table = M.table32.p;
        a.diag = op.d_diag32.p;
        if (M.lanes == 16) QS_SPMV(16, float);
        else if (M.lanes == 8) QS_SPMV(8, float);
        else QS_SPMV(4, float);
    } else {
        a.table = M.table64.p;
        a.diag = op.d_diag.p;
        if (M.lanes == 16) QS_SPMV(16, double);
        else if (M.lanes == 8) QS_SPMV(8, double);
        else QS_SPMV(4, double);
    }
#undef QS_SPMV
    QS_CUDA(cudaGetLastError());
    note_launches(1);
}


bool op_spmm_device(Op& op, const MatvecCall& c, int64_t nrhs, cudaStream_t s) {
    const Basis& b = *op.basis;
    const Assembled& M = op.asm_;
    const bool T = (c.flags & QS_TRANSPOSE) != 0, C = (c.flags & QS_CONJUGATE) != 0;
    if (nrhs < 2 || !op.commuting || !op.assembled || !M.has_sell || (T && !op.hermitian) || c.df || c.fx ||
        c.df_io || c.slice1 >= 0 || c.slice0 != 0)
        return false;
    SellArgs a{};
    a.sptr = M.sell_ptr.as<int64_t>();
    a.perm = M.sell_perm.as<int32_t>();
    a.len = M.sell_len.as<uint16_t>();
    a.words = M.sell_words.as<uint32_t>();
    a.cols = M.sell_cols.as<int32_t>();
    a.codes = M.sell_codes.as<uint16_t>();
    a.packed = M.packed;
    a.code_bits = M.code_bits;
    a.code_mask = M.code_bits >= 32 ? 0xffffffffu : ((1u << M.code_bits) - 1u);
    a.ncodes = M.ncodes;
    a.stab = b.symmetric ? b.d_stab.as<uint16_t>() : nullptr;
    a.nslices = M.nslices;
    a.slice0 = 0;
    a.n = b.n;
    a.ar = c.alpha.re;
    a.ai = c.alpha.im;
    a.br = c.beta.re;
    a.bi = c.beta.im;
    a.beta_zero = (c.beta.re == 0.0 && c.beta.im == 0.0);
    a.conj = T != C;
    const bool cm = op.complex_mat, cv = c.y_complex;
    if (c.single) {
        a.table = M.table32.p;
        a.diag = op.d_diag32.p;
        a.diag_re = op.d_diag32_re.p;
    } else {
        a.table = M.table64.p;
        a.diag = op.d_diag.p;
        a.diag_re = op.d_diag_re.p;
    }
    constexpr int R = 8;
    const size_t eb = (c.single ? 4 : 8) * (cv ? 2 : 1);
    const int grid = grid_rows(std::max<int64_t>(1, a.nslices) * kSlice);
    PoolBuf xt((size_t)b.n * R * eb, s);   // the interleaved columns
    const int ig = grid_rows(b.n);
    for (int64_t j0 = 0; j0 < nrhs; j0 += R) {
        const int nc = (int)std::min<int64_t>(R, nrhs - j0);
        const void* xs = (const char*)c.x + (size_t)j0 * b.n * eb;
        if (eb == 4) interleave_kernel<float, R><<<ig, kThreads, 0, s>>>((const float*)xs, xt.as<float>(), b.n, nc);
        else if (eb == 8) interleave_kernel<double, R><<<ig, kThreads, 0, s>>>((const double*)xs, xt.as<double>(), b.n, nc);
        else interleave_kernel<double2, R><<<ig, kThreads, 0, s>>>((const double2*)xs, xt.as<double2>(), b.n, nc);
        a.x = xt.p;
        a.y = (char*)c.y + (size_t)j0 * b.n * eb;
#define QS_MM(TT)                                                                                        \
        do {                                                                                             \
            if (a.packed) {                                                                              \
                if (cm) sell_mm_kernel<true, true, TT, true, R><<<grid, kThreads, 0, s>>>(a, nc, b.n);      \
                else if (cv) sell_mm_kernel<false, true, TT, true, R><<<grid, kThreads, 0, s>>>(a, nc, b.n); \
                else sell_mm_kernel<false, false, TT, true, R><<<grid, kThreads, 0, s>>>(a, nc, b.n);        \
            } else {                                                                                     \
                if (cm) sell_mm_kernel<true, true, TT, false, R><<<grid, kThreads, 0, s>>>(a, nc, b.n);     \
                else if (cv) sell_mm_kernel<false, true, TT, false, R><<<grid, kThreads, 0, s>>>(a, nc, b.n); \
                else sell_mm_kernel<false, false, TT, false, R><<<grid, kThreads, 0, s>>>(a, nc, b.n);       \
            }                                                                                            \
        } while (0)
        if (c.single) QS_MM(float);
        else QS_MM(double);
#undef QS_MM
        QS_CUDA(cudaGetLastError());
        note_launches(2);
    }
    return true;
}

namespace {

// Element values of the assembled CSR form: value k of row r is
// table[code_k] / sqrt(stab_r) (the row scale the products apply after the
// sum), column col_k.
__global__ void export_kernel(const int64_t* __restrict__ rowptr, const uint32_t* __restrict__ words,
                              const int32_t* __restrict__ cols, const uint16_t* __restrict__ codes, int packed,
                              int cb, uint32_t cmask, const double2* __restrict__ table,
                              const uint16_t* __restrict__ stab, int64_t n, int64_t* __restrict__ ocol,
                              double2* __restrict__ oval) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        const double sc = stab ? 1.0 / sqrt((double)stab[r]) : 1.0;
        for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k) {
            uint32_t col, code;
            if (packed) {
                col = words[k] >> cb;
                code = words[k] & cmask;
            } else {
                col = (uint32_t)cols[k];
                code = codes[k];
            }
            const double2 v = table[code];
            ocol[k] = col;
            oval[k] = make_double2(v.x * sc, v.y * sc);
        }
    }
}

}  // namespace

void op_export_csr(Op& op, int64_t* rowptr, int64_t* cols, double* values, double* diag) {
    if (!op.assembled) op_assemble(op);
    const Assembled& M = op.asm_;
    Basis& b = *op.basis;
    const int64_t n = b.n;
    cudaStream_t s = op.stream;
    PoolBuf dcol((size_t)std::max<int64_t>(1, M.nnz) * sizeof(int64_t), s),
        dval((size_t)std::max<int64_t>(1, M.nnz) * sizeof(double2), s);
    const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16));
    export_kernel<<<grid, 256, 0, s>>>(M.rowptr.as<int64_t>(), M.words.as<uint32_t>(), M.cols.as<int32_t>(),
                                       M.codes.as<uint16_t>(), M.packed ? 1 : 0, M.code_bits,
                                       M.code_bits >= 32 ? 0xffffffffu : ((1u << M.code_bits) - 1u),
                                       M.table64.as<double2>(), b.symmetric ? b.d_stab.as<uint16_t>() : nullptr, n,
                                       dcol.as<int64_t>(), dval.as<double2>());
    QS_CUDA(cudaGetLastError());
    note_launches(1);
    QS_CUDA(cudaMemcpyAsync(rowptr, M.rowptr.p, (size_t)(n + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    if (M.nnz) {
        QS_CUDA(cudaMemcpyAsync(cols, dcol.p, (size_t)M.nnz * sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        QS_CUDA(cudaMemcpyAsync(values, dval.p, (size_t)M.nnz * sizeof(double2), cudaMemcpyDeviceToHost, s));
    }
    QS_CUDA(cudaMemcpyAsync(diag, op.d_diag.p, (size_t)n * sizeof(double2), cudaMemcpyDeviceToHost, s));
    QS_CUDA(cudaStreamSynchronize(s));
}


void op_release_assembly(Op& op) {
    if (!op.assembled) return;
    QS_CUDA(cudaStreamSynchronize(op.stream));
    op.asm_ = Assembled();
    op.assembled = false;
}

TransientAssembly::TransientAssembly(Op& o) : op(o) {
    if (op.assembled || !op.commuting) return;
    // in small sectors a solve is dominated by per-call setup, not by
    // products: XXZ L=16 (12,870 rows) eigsh k=4 takes 9.3 ms assembled for
    // the call (0.8 ms of it the assembly, the steps on the cluster step)
    // against 12.3 ms matrix-free; below 4,096 rows the operator stays
    // matrix-free
    if (op.basis->n < 4096) return;
    const char* e = std::getenv("QS_TRANSIENT_ASSEMBLY");
    if (e && e[0] == '0') return;
    // an upper bound of the assembled form (both layouts): a packed word per
    // program and row, twice, with the row tables; a quarter of free memory at most
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    const double bound = (double)op.basis->n * ((double)op.progs.size() / 2 * 4.0 * 2 + 64);
    if (bound > 0.25 * (double)free_b) return;
    try {
        op_assemble(op);
        made = true;
    } catch (const Error& err) {
        if (err.status != QS_ERR_UNSUPPORTED) throw;   // programs that cannot be assembled stay matrix-free
    }
}

TransientAssembly::~TransientAssembly() {
    if (!made) return;
    try {
        op_release_assembly(op);
    } catch (...) {
    }
}

bool op_matvec_host_overlap(Op& op, const MatvecCall& c0, void* y_host, size_t eb) {
    const Assembled& M = op.asm_;
    const bool T = (c0.flags & QS_TRANSPOSE) != 0;
    const bool fx = c0.fx && !c0.single && M.fx_classes > 0;
    if (!op.commuting || !op.assembled || !M.has_sell || (T && !op.hermitian) || (c0.df && !fx) || c0.df_io)
        return false;
    if (!(c0.beta.re == 0.0 && c0.beta.im == 0.0)) return false;   // y is not read
    // the first product of a kind times the kernel variants on the full range
    if (M.sell_variant[fx ? 4 : (c0.single ? 1 : 0)] < 0) return false;
    constexpr int K = 4;
    if (M.nslices < 4 * K) return false;
    if (!op.copy_stream) {
        QS_CUDA(cudaStreamCreateWithFlags(&op.copy_stream, cudaStreamNonBlocking));
        for (cudaEvent_t& e : op.range_done) QS_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    const int64_t n = op.basis->n;
    for (int k = 0; k < K; ++k) {
        MatvecCall c = c0;
        c.slice0 = M.nslices * k / K;
        c.slice1 = M.nslices * (k + 1) / K;
        c.fx_ready = k > 0;   // the first range makes the integer copy of x for all
        op_spmv_device(op, c, op.stream);
        QS_CUDA(cudaEventRecord(op.range_done[k], op.stream));
        QS_CUDA(cudaStreamWaitEvent(op.copy_stream, op.range_done[k], 0));
        const int64_t r0 = c.slice0 * kSellSlice, r1 = std::min<int64_t>(n, c.slice1 * kSellSlice);
        if (r1 > r0)
            QS_CUDA(cudaMemcpyAsync((char*)y_host + (size_t)r0 * eb, (const char*)c0.y + (size_t)r0 * eb,
                                    (size_t)(r1 - r0) * eb, cudaMemcpyDeviceToHost, op.copy_stream));
    }
    QS_CUDA(cudaStreamSynchronize(op.copy_stream));
    return true;
}

}  // namespace qs
