// qs_device.cuh -- device-side building blocks shared by the basis and matvec
// kernels: group scans, representative search and rank lookups.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "qs_common.h"

namespace qs {

// Shared-memory image of the permutation/mask tables of a GroupDesc (the
// characters stay in global memory: only the winning element's is read).
struct GroupSmem {
    int32_t L, ng, nperm;
    int32_t general, nbytes;
    const uint64_t* gtab;
    uint64_t lmask;
    int8_t refl[kMaxPerm];
    int8_t shift[kMaxPerm];
    int16_t begin[kMaxPerm + 1];
    uint64_t mask[kMaxGroup];
};

__device__ __forceinline__ void load_group_smem(GroupSmem& s, const GroupDesc* __restrict__ g) {
    if (threadIdx.x == 0) {
        s.L = g->L;
        s.ng = g->ng;
        s.nperm = g->nperm;
        s.lmask = g->lmask;
        s.general = g->general;
        s.nbytes = g->nbytes;
        s.gtab = g->gtab;
    }
    for (int i = threadIdx.x; i < g->nperm; i += blockDim.x) {
        s.refl[i] = g->perm_refl[i];
        s.shift[i] = g->perm_shift[i];
    }
    for (int i = threadIdx.x; i <= g->nperm; i += blockDim.x) s.begin[i] = g->perm_begin[i];
    for (int i = threadIdx.x; i < g->ng; i += blockDim.x) s.mask[i] = g->mask[i];
    __syncthreads();
}

// Minimum of the orbit of t, the element reaching it and the number of
// elements reaching it (= order of the stabiliser of the minimum).
template <typename U>
__device__ __forceinline__ void orbit_min(const GroupSmem& g, U t, U& best, int& bidx, int& stab) {
    const int L = g.L;
    const U m = (U)g.lmask;
    U base[2];
    base[0] = t;
    base[1] = brev_bits(t, L);
    best = (U)~(U)0;
    bidx = 0;
    stab = 0;
    for (int p = 0; p < g.nperm; ++p) {
        U r = g.general ? (U)gperm_apply(g.gtab, p, g.nbytes, (uint64_t)t)
                        : rotl_bits<U>(base[g.refl[p]], g.shift[p], L, m);
        const int e1 = g.begin[p + 1];
        for (int e = g.begin[p]; e < e1; ++e) {
            U c = r ^ (U)g.mask[e];
            if (c < best) {
                best = c;
                bidx = e;
                stab = 1;
            } else if (c == best) {
                ++stab;
            }
        }
    }
}

// Lower-bound search over the sorted representatives: a shared-memory stage of
// nsplit splitters (splitter i = reps[i * stride]) narrows the key to one
// stride-long segment, then a binary search finishes in global memory.
template <typename U>
__device__ __forceinline__ int64_t rank_search(const U* __restrict__ reps, int64_t n, const U* spl, int nsplit,
                                               int64_t stride, U key) {
    int lo = 0, hi = nsplit;  // find last splitter <= key
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (spl[mid] <= key) lo = mid;
        else hi = mid;
    }
    int64_t a = (int64_t)lo * stride;
    int64_t b = a + stride;
    if (b > n) b = n;
    while (a < b) {
        int64_t mid = (a + b) >> 1;
        U v = __ldg(reps + mid);
        if (v < key) a = mid + 1;
        else b = mid;
    }
    return (a < n && __ldg(reps + a) == key) ? a : -1;
}

// Combinadic rank of a fixed-weight state: sum over set bits (ascending) of
// C(bit, particle), particle = 1, 2, ...  (matches Gosper order).
template <typename U>
__device__ __forceinline__ int64_t combinadic_rank(U s, const uint64_t* binom, int stride_p) {
    int64_t r = 0;
    int particle = 1;
    while (s) {
        int bit = (sizeof(U) == 8) ? __ffsll((long long)s) - 1 : __ffs((int)s) - 1;
        r += (int64_t)binom[bit * stride_p + particle];
        ++particle;
        s &= s - 1;
    }
    return r;
}

// Combinadic rank of a state of at most 32 sites with the C(bit, p) table in
// shared memory (32 x 33 uint32 entries).
__device__ __forceinline__ int64_t combinadic_rank32(uint32_t s, const uint32_t* binom32) {
    uint32_t r = 0;
    int particle = 1;
    while (s) {
        int bit = __ffs((int)s) - 1;
        r += binom32[bit * 33 + particle];
        ++particle;
        s &= s - 1;
    }
    return (int64_t)r;
}

}  // namespace qs
