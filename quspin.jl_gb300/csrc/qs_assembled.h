// qs_assembled.h -- device storage of an assembled operator (see qs_assembled.cu).
#pragma once

#include <cstdint>

namespace qs {

constexpr int kSellSlice = 32;   // rows per slice of the sliced-ELL layout
constexpr int kFxCodes = 256;    // value codes of an operator with fixed-point row sums, at most

#ifdef __CUDACC__
// Cache policies of the sliced-ELL walk.  kHint = false: plain read-only
// loads (__ldg).  kHint = true: the packed words, read once per product, skip
// L1 and leave L2 first (an L2::evict_first cache policy), and the x gathers
// leave L2 last (L2::evict_last), so the word stream (hundreds of MB) does
// not evict x (tens of MB) between its reuses.  Per-instruction cache-policy
// operands only (createpolicy): no device or context setting changes.
__device__ __forceinline__ unsigned long long l2_evict_first() {
    unsigned long long p;
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ unsigned long long l2_evict_last() {
    unsigned long long p;
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}
template <bool kHint> __device__ __forceinline__ uint32_t ld_word(const uint32_t* p) {
    if (!kHint) return __ldg(p);
    uint32_t v;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(l2_evict_first()));
    return v;
}
template <bool kHint> __device__ __forceinline__ int32_t ld_word(const int32_t* p) {
    if (!kHint) return __ldg(p);
    int32_t v;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.s32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(l2_evict_first()));
    return v;
}
template <bool kHint> __device__ __forceinline__ uint16_t ld_word(const uint16_t* p) {
    if (!kHint) return __ldg(p);
    unsigned short v;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.u16 %0, [%1], %2;" : "=h"(v) : "l"(p), "l"(l2_evict_first()));
    return v;
}
template <bool kHint> __device__ __forceinline__ double ld_gather(const double* p) {
    if (!kHint) return __ldg(p);
    double v;
    asm("ld.global.nc.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(p), "l"(l2_evict_last()));
    return v;
}
template <bool kHint> __device__ __forceinline__ double2 ld_gather(const double2* p) {
    if (!kHint) return __ldg(p);
    double2 v;
    asm("ld.global.nc.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;" : "=d"(v.x), "=d"(v.y) : "l"(p), "l"(l2_evict_last()));
    return v;
}
template <bool kHint> __device__ __forceinline__ float ld_gather(const float* p) {
    if (!kHint) return __ldg(p);
    float v;
    asm("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(l2_evict_last()));
    return v;
}
template <bool kHint> __device__ __forceinline__ float2 ld_gather(const float2* p) {
    if (!kHint) return __ldg(p);
    float2 v;
    asm("ld.global.nc.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;" : "=f"(v.x), "=f"(v.y) : "l"(p), "l"(l2_evict_last()));
    return v;
}
template <bool kHint> __device__ __forceinline__ float4 ld_gather(const float4* p) {
    if (!kHint) return __ldg(p);
    float4 v;
    asm("ld.global.nc.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
        : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(p), "l"(l2_evict_last()));
    return v;
}
template <bool kHint> __device__ __forceinline__ long long ld_gather(const long long* p) {
    if (!kHint) return __ldg(p);
    long long v;
    asm("ld.global.nc.L2::cache_hint.s64 %0, [%1], %2;" : "=l"(v) : "l"(p), "l"(l2_evict_last()));
    return v;
}
template <bool kHint> __device__ __forceinline__ longlong2 ld_gather(const longlong2* p) {
    if (!kHint) return __ldg(p);
    longlong2 v;
    asm("ld.global.nc.L2::cache_hint.v2.s64 {%0, %1}, [%2], %3;" : "=l"(v.x), "=l"(v.y) : "l"(p), "l"(l2_evict_last()));
    return v;
}

// The nonzeros of one sliced-ELL row (`len` of them from `base`, stride
// kSellSlice), fed to acc(code, x[col]) with U words and then U gathers in
// flight before any arithmetic: the product is bound by the latency of the
// x gathers, and this keeps U of them outstanding per thread.
template <int U, bool kPacked, bool kHint, class LoadX, class Acc>
__device__ __forceinline__ void sell_row(const uint32_t* __restrict__ words, const int32_t* __restrict__ cols,
                                         const uint16_t* __restrict__ codes, int64_t base, int len, int cb,
                                         uint32_t cmask, LoadX ldx, Acc acc) {
    int j = 0;
    for (; j + U <= len; j += U) {
        uint32_t col[U], code[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int64_t o = base + (int64_t)(j + u) * kSellSlice;
            if (kPacked) {
                const uint32_t w = ld_word<kHint>(words + o);
                col[u] = w >> cb;
                code[u] = w & cmask;
            } else {
                col[u] = (uint32_t)ld_word<kHint>(cols + o);
                code[u] = ld_word<kHint>(codes + o);
            }
        }
        decltype(ldx(0u)) xv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) xv[u] = ldx(col[u]);
#pragma unroll
        for (int u = 0; u < U; ++u) acc(code[u], xv[u]);
    }
    for (; j < len; ++j) {
        const int64_t o = base + (int64_t)j * kSellSlice;
        uint32_t col, code;
        if (kPacked) {
            const uint32_t w = ld_word<kHint>(words + o);
            col = w >> cb;
            code = w & cmask;
        } else {
            col = (uint32_t)ld_word<kHint>(cols + o);
            code = ld_word<kHint>(codes + o);
        }
        acc(code, ldx(col));
    }
}
#endif

struct Assembled {
    DevBuf rowptr;     // int64, n + 1
    DevBuf words;      // uint32 (column << code_bits) | code, when packed
    DevBuf cols;       // int32 column per nonzero, when not packed
    DevBuf codes;      // uint16 code per nonzero, when not packed
    DevBuf table64;    // complex double value per code
    DevBuf table32;    // complex float value per code
    DevBuf table_df;   // per code: re hi, re lo, im hi, im lo (float)
    DevBuf xsplit;     // x split into float pairs for the double-float product
    DevBuf rsq_df;     // 1/sqrt(stab) as float pairs, stab = 0 .. kMaxGroup
    int64_t nnz = 0;
    int ncodes = 0;
    int code_bits = 0;
    bool packed = true;
    int lanes = 8;     // threads per row in the CSR SpMV
    // sliced-ELL copy: slices of kSellSlice consecutive rows in natural
    // order, words column-major inside a slice (one thread per row), each
    // row with its own length
    DevBuf sell_words;  // uint32 packed (or int32 column + uint16 code pairs as uint32/uint16 arrays)
    DevBuf sell_cols, sell_codes;
    DevBuf sell_ptr;    // int64 start of each slice
    DevBuf sell_perm;   // int32 row of each slice position (-1 past the end)
    DevBuf sell_len;    // uint16 length of each slice position's row
    int64_t nslices = 0;
    bool has_sell = false;
    // exact fixed-point row sums (FP64 vectors): usable when every stored
    // value is real and is +-A_c sqrt(stab_col) for at most four amplitude
    // classes c; fx_classes = 0 otherwise
    int fx_classes = 0;
    int len_bits = 0;   // ceil(log2(longest row)), at least 0
    DevBuf fx_cls;      // uint32 per code: class << 1 | sign
    DevBuf fx_amp;      // double per class: A_c
    DevBuf fx_sq;       // double sqrt(i), i = 0 .. kMaxGroup
    DevBuf fx_max;      // uint64: max |x_j sqrt(stab_j)| of the current product (bit pattern), then per-block maxima
    // sliced-ELL kernel variant (gathers in flight x resident blocks) per
    // product kind (FP64, FP32, double-float with FP64 vectors, double-float
    // vectors, fixed-point row sums), chosen by timing on the first product
    // that allows it (-1: not yet)
    int sell_variant[5] = {-1, -1, -1, -1, -1};
};

}  // namespace qs
