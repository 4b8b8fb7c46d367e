// qs_tc.cuh -- fifth-generation tensor cores (tcgen05) from inline PTX, and the
// exact integer slicing that lets them carry FP64-class products.
//
// The Krylov restart rotation V[:, 0:p] = V[:, 0:m] Y is the one dense
// contraction of the solvers (N x m by m x p, m <= 32).  GB300 has no fast
// FP64 tensor path, so the FP64 engine runs it as an exact integer product on
// the FP16 tensor cores, after Ozaki et al. ("Error-free
// transformations of matrix multiplication by using fast routines of matrix
// multiplication and its applications", Numer. Algorithms 2012): every entry
// (|v| <= 2) is scaled to a 61-bit fixed-point integer X = trunc(v 2^61),
// whose magnitude splits into eight bytes d_0 (most significant) .. d_7, each
// exact in FP16 with the entry's sign.  A product of two digits is below 2^16,
// so the sum over the m <= 32 terms of every digit pair (a, b) with the same
// a + b = s (at most nine pairs) stays below 2^24 and accumulates exactly in
// the FP32 tensor accumulator; the nine sums D_s (s = 0 .. 8) are combined in
// 64-bit integers, and the pairs with a + b > 8 (weight below 2^-59 of the
// largest entry) are dropped.  Normwise the result is as accurate as an FP64
// product (measured against the FP64 rotation in the tests).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace qs {

#ifdef __CUDACC__

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor of tcgen05.mma: K-major, no swizzle
// (core matrices of 8 rows x 16 bytes, stored as 128 contiguous bytes).
// lbo: bytes between core matrices adjacent in K; sbo: bytes between core
// matrices adjacent in M (or N).  Bits 46-47 hold the descriptor version (1).
__device__ __forceinline__ uint64_t tc_sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo & 0x3FFFFu) >> 4) << 16;
    d |= (uint64_t)((sbo & 0x3FFFFu) >> 4) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor of kind::f16 with FP16 A and B (both K-major) and
// an FP32 accumulator, M x N.
__host__ __device__ constexpr uint32_t tc_idesc_f16(int M, int N) {
    return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Byte offset of element (row, k) of a K-major no-swizzle tile whose rows
// hold kp elements of 2 bytes.
__host__ __device__ constexpr uint32_t tc_off(int row, int k, int kp) {
    return (uint32_t)((row >> 3) * (kp / 8) * 128 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ void tc_alloc(uint32_t* dst_smem, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst_smem)),
                 "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void tc_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols));
}
__device__ __forceinline__ void tc_mma_f16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                            uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}
// arrive on the mbarrier once every tcgen05 operation issued so far by this
// thread has completed
__device__ __forceinline__ void tc_commit(uint64_t* mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
        smem_addr(mbar)));
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;"); }
// generic-proxy shared-memory writes become visible to the tensor cores
__device__ __forceinline__ void tc_fence_smem() { asm volatile("fence.proxy.async.shared::cta;"); }

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(mbar)), "r"(count));
    asm volatile("fence.mbarrier_init.release.cluster;");
}
// Waits for phase `parity` of the mbarrier to complete, for at most `limit`
// clock cycles; false when the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, long long limit) {
    const long long t0 = clock64();
    uint32_t done = 0;
    while (true) {
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smem_addr(mbar)), "r"(parity));
        if (done) return true;
        if (clock64() - t0 > limit) return false;
        __nanosleep(64);
    }
}

// 32 lanes x 4 consecutive 32-bit columns of TMEM (this warp's lane quarter)
__device__ __forceinline__ void tc_ld4(uint32_t taddr, uint32_t (&v)[4]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3])
                 : "r"(taddr));
}
__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;"); }

// trunc(v 2^61) for |v| < 2, from the bit pattern (zero for subnormals)
__device__ __forceinline__ long long fix61(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const int e = (int)((b >> 52) & 0x7ff);
    const unsigned long long mant = (b & 0xfffffffffffffull) | (1ull << 52);
    const int sh = e - 1014;   // v 2^61 = mant 2^(e - 1075 + 61)
    unsigned long long q = 0;
    if (e != 0) q = sh >= 0 ? mant << (sh > 9 ? 9 : sh) : (sh > -64 ? mant >> -sh : 0ull);
    return (b >> 63) ? -(long long)q : (long long)q;
}
// Two FP16 digits at once: byte bb (0..3) of x and of y, each below 256 and
// exact in FP16, with the signs sg (0x8000 in either half), as one f16x2
// word: a byte permutation puts each byte under the exponent of 1024
// (FP16 0x6400 + b is 1024 + b exactly), one packed subtraction removes the
// 1024.
template <int bb>
__device__ __forceinline__ uint32_t f16x2_of_bytes(uint32_t x, uint32_t y, uint32_t sg) {
    constexpr uint32_t sel = (uint32_t)bb | ((uint32_t)(4 + bb) << 8);
    const uint32_t t = (__byte_perm(x, y, sel) & 0x00FF00FFu) | 0x64006400u;
    uint32_t r;
    asm("sub.rn.f16x2 %0, %1, %2;" : "=r"(r) : "r"(t), "r"(0x64006400u));
    return r | sg;
}
// FP16 bits of sign * byte
__device__ __forceinline__ uint32_t f16_of_byte(uint32_t byte, uint32_t sign) {
    uint32_t r;
    asm("sub.rn.f16x2 %0, %1, %2;" : "=r"(r) : "r"(0x6400u | byte), "r"(0x6400u));
    return (r & 0xffffu) | sign;
}

// v 2^scale rounded to the nearest double (ties to even); v 2^scale in the
// normal range
__device__ __forceinline__ double f64_of_i64(long long v, int scale) {
    if (v == 0) return 0.0;
    const unsigned long long sgn = v < 0 ? (1ull << 63) : 0ull;
    unsigned long long m = v < 0 ? (unsigned long long)(-v) : (unsigned long long)v;
    const int lz = __clzll((long long)m);
    int e = 63 - lz;
    m <<= lz;
    unsigned long long mant = m >> 11;
    const unsigned long long rem = m & 0x7ffull;
    if (rem > 0x400ull || (rem == 0x400ull && (mant & 1ull))) {
        mant += 1;
        if (mant >> 53) {
            mant >>= 1;
            e += 1;
        }
    }
    return __longlong_as_double((long long)(sgn | ((unsigned long long)(e + scale + 1023) << 52) |
                                            (mant & 0xfffffffffffffull)));
}
#endif

}  // namespace qs
