// qs_orbit.cuh -- orbit minimum for the translation x parity x spin-flip groups
// of a chain, without visiting every group element.
//
// For a group G = {s -> F^f( rotl_L( P^r(s), a*j ) )}, j < L/a, r in R, f in M,
// (P: site reversal, F: complement of all L bits, rotl_L: rotation by whole
// sites) the minimum of the orbit of t is the minimum over the |R| * |M| bases
// b = F^f(P^r(t)) of the least allowed rotation of b.  A rotation of b by k
// puts bit p = L-1-k of b on top, so its value is smallest when the run of
// zeros that descends from p (cyclically) is longest.  The positions that start
// a maximal descending zero run are found bit-parallel:
//     R_1 = ~b,   R_{t+s} = R_t & rotl(R_s, t)      (R_t: a zero run of length >= t starts here)
// with powers of two and binary lifting, restricted to positions reachable by
// allowed rotations.  Only those candidates (usually one or two per base) are
// compared as full values.  Every group element that reaches the minimum is
// among the candidates, so the stabiliser order is the number of candidates
// whose rotation equals the minimum.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "qs_common.h"

namespace qs {

struct FastGroup {
    int32_t enabled;
    int32_t L, a, nT;
    int32_t has_refl, has_flip;
    uint64_t lmask;
    uint64_t allowed;    // bit p set when L-1-p is a multiple of a
};

#ifdef __CUDACC__
template <typename U>
__device__ __forceinline__ U rot_sites(U x, int k, int L, U lm) {
    if (sizeof(U) == 4 && L == 32) return __funnelshift_l((uint32_t)x, (uint32_t)x, k);
    return k == 0 ? x : (U)(((x << k) | (x >> (L - k))) & lm);
}

// Returns the length of the longest descending zero run of b that starts at an
// allowed position, and the mask of those starting positions.
template <typename U>
__device__ __forceinline__ int zero_run_starts(U b, int L, U lm, U allowed, U& starts) {
    const U y = (U)(~b) & lm;
    if ((y & allowed) == (U)0) {
        starts = allowed;
        return 0;
    }
    U R[6];
    R[0] = y;
    int kmax = 0;
#pragma unroll
    for (int k = 1; k < 6; ++k) {
        if ((1 << k) <= L) {
            R[k] = R[k - 1] & rot_sites<U>(R[k - 1], 1 << (k - 1), L, lm);
            kmax = k;
        }
    }
    U cur = y;
    int t = 1;
#pragma unroll
    for (int k = 5; k >= 0; --k) {
        if (k > kmax) continue;
        const int s = 1 << k;
        if (t + s > L) continue;
        const U c = cur & rot_sites<U>(R[k], t % L, L, lm);
        if ((c & allowed) != (U)0) {
            cur = c;
            t += s;
        }
    }
    starts = cur & allowed;
    return t;
}

// Orbit minimum of t.  elem = (r * 2 + f) * nT + j identifies the element that
// reaches it (its character is looked up by the caller); stab counts elements.
template <typename U>
__device__ __forceinline__ void orbit_min_fast(const FastGroup& G, U t, U& best, int& elem, int& stab) {
    const int L = G.L;
    const U lm = (U)G.lmask;
    const U allowed = (U)G.allowed;
    U base[4];
    int nb = 0;
    int code[4];
    const U tr = G.has_refl ? brev_bits(t, L) : t;
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        if (r && !G.has_refl) break;
        const U b0 = r ? tr : t;
#pragma unroll
        for (int f = 0; f < 2; ++f) {
            if (f && !G.has_flip) break;
            base[nb] = f ? ((U)(~b0) & lm) : b0;
            code[nb] = r * 2 + f;
            ++nb;
        }
    }
    int tb[4];
    U st[4];
    int tmax = -1;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        if (i < nb) {
            tb[i] = zero_run_starts<U>(base[i], L, lm, allowed, st[i]);
            tmax = tb[i] > tmax ? tb[i] : tmax;
        }
    }
    best = (U)~(U)0;
    elem = 0;
    stab = 0;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        if (i >= nb || tb[i] != tmax) continue;
        U c = st[i];
        while (c) {
            const int p = (sizeof(U) == 8) ? (63 - __clzll((long long)c)) : (31 - __clz((int)c));
            c &= ~((U)1 << p);
            const int k = L - 1 - p;
            const U v = rot_sites<U>(base[i], k, L, lm);
            if (v < best) {
                best = v;
                elem = code[i] * G.nT + k / G.a;
                stab = 1;
            } else if (v == best) {
                ++stab;
            }
        }
    }
}

#endif  // __CUDACC__

}  // namespace qs
