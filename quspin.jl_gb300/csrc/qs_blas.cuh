// qs_blas.cuh -- Krylov vector kernels (BLAS-1 / tall-skinny) with FP64
// accumulation, for real or complex vectors stored in double or single
// precision.  Vector sets V are column-major with leading dimension ld.
#pragma once

#include <cuda_runtime.h>

#include <complex>
#include <cstdint>
#include <vector>

#include "qs_internal.h"

namespace qs {

// Storage of a Krylov vector: scalar type and real/complex.
// DF64 / CDF64: double-float storage, hi + lo float per real component.
enum class VKind { F64 = 0, C128 = 1, F32 = 2, C64 = 3, DF64 = 4, CDF64 = 5 };
inline bool vk_complex(VKind k) { return k == VKind::C128 || k == VKind::C64 || k == VKind::CDF64; }
inline bool vk_single(VKind k) { return k == VKind::F32 || k == VKind::C64; }
inline bool vk_df(VKind k) { return k == VKind::DF64 || k == VKind::CDF64; }
inline size_t vk_bytes(VKind k) {
    switch (k) {
        case VKind::F64: return 8;
        case VKind::C128: return 16;
        case VKind::F32: return 4;
        case VKind::C64: return 8;
        case VKind::DF64: return 8;
        default: return 16;
    }
}

using cd = std::complex<double>;

// All functions launch on stream s; those returning host values synchronise.
struct Blas {
    VKind kind;
    int64_t n;
    cudaStream_t s;
    DevBuf partial;   // block partials for reductions
    DevBuf coeffs;    // small coefficient vectors on the device
    DevBuf result;    // reduced dot products
    std::vector<double> hbuf;
    std::vector<float> fbuf;
    Blas(VKind k, int64_t n_, cudaStream_t st);
    void upload_df(const std::vector<cd>& h, int m);
    // h_j = <V_j, w>, j < m
    void dots(const void* V, int64_t ld, int m, const void* w, std::vector<cd>& h);
    // w -= sum_j V_j h_j
    void update(void* w, const void* V, int64_t ld, int m, const std::vector<cd>& h);
    // out = sum_j V_j c_j  (out may not alias V)
    void combine(void* out, const void* V, int64_t ld, int m, const std::vector<cd>& c);
    double norm(const void* w);
    cd dot(const void* a, const void* b);
    // dst = a * src
    void scale(void* dst, const void* src, cd a);
    // y += a * x
    void axpy(void* y, const void* x, cd a);
    void copy(void* dst, const void* src);
    // V[:, 0:p] = V[:, 0:m] * Y[0:m, 0:p] (Y column-major m x p, real), using tmp (n x p)
    void rotate(void* V, int64_t ld, int m, int p, const std::vector<double>& Y, void* tmp);
};

// Conversions between storage precisions (same real/complex-ness).
void convert_vec(const void* src, VKind ks, void* dst, VKind kd, int64_t n, cudaStream_t s);

// dst = n elements of kind k with independent standard normal components, a
// pure function of (seed, component index): the same vector on every run and
// whatever else shares the device.
void fill_normal(void* dst, VKind k, int64_t n, uint64_t seed, cudaStream_t s);

}  // namespace qs
