// qs_blas.cu -- Krylov vector kernels with FP64 accumulation (warp-shuffle
// block reductions).  Replaces the BLAS-1 calls of the reference's Krylov
// loop (dot / axpy! / norm in _krylov_factorization, src/operators.jl:
// 1681-1726) and the reorthogonalisation ARPACK performs internally.
#include "qs_blas.cuh"
#include "qs_df.cuh"

#include <algorithm>

namespace qs {

namespace {

constexpr int kThreads = 256;
constexpr int kJT = 8;          // vectors per dot tile
constexpr int kMaxBlocks = 1216;

template <typename S, bool C> struct El;
template <> struct El<double, false> { using t = double; };
template <> struct El<double, true> { using t = double2; };
template <> struct El<float, false> { using t = float; };
template <> struct El<float, true> { using t = float2; };

template <typename S, bool C>
__device__ __forceinline__ void ld(const void* p, int64_t i, double& re, double& im) {
    if constexpr (C) {
        auto v = ((const typename El<S, C>::t*)p)[i];
        re = (double)v.x;
        im = (double)v.y;
    } else {
        re = (double)((const S*)p)[i];
        im = 0.0;
    }
}
template <typename S, bool C>
__device__ __forceinline__ void st(void* p, int64_t i, double re, double im) {
    if constexpr (C) {
        typename El<S, C>::t v;
        v.x = (S)re;
        v.y = (S)im;
        ((typename El<S, C>::t*)p)[i] = v;
    } else {
        ((S*)p)[i] = (S)re;
    }
}

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-sum of kJT complex values; result valid in thread 0.
__device__ __forceinline__ void block_sum(double (&re)[kJT], double (&im)[kJT]) {
    __shared__ double sh[kThreads / 32][2 * kJT];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < kJT; ++j) {
        re[j] = warp_sum(re[j]);
        im[j] = warp_sum(im[j]);
    }
    if (lane == 0)
#pragma unroll
        for (int j = 0; j < kJT; ++j) {
            sh[wid][2 * j] = re[j];
            sh[wid][2 * j + 1] = im[j];
        }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int j = 0; j < kJT; ++j) {
            double a = lane < kThreads / 32 ? sh[lane][2 * j] : 0.0;
            double b = lane < kThreads / 32 ? sh[lane][2 * j + 1] : 0.0;
            re[j] = warp_sum(a);
            im[j] = warp_sum(b);
        }
    }
}

template <typename S, bool C>
__global__ void __launch_bounds__(kThreads) dots_kernel(const void* V, int64_t ldv, int m, const void* w, int64_t n,
                                                        double* partial) {
    const int j0 = blockIdx.y * kJT;
    double re[kJT], im[kJT];
#pragma unroll
    for (int j = 0; j < kJT; ++j) re[j] = im[j] = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kThreads) {
        double wr, wi;
        ld<S, C>(w, i, wr, wi);
#pragma unroll
        for (int j = 0; j < kJT; ++j) {
            if (j0 + j < m) {
                double vr, vi;
                ld<S, C>(V, (int64_t)(j0 + j) * ldv + i, vr, vi);
                re[j] = fma(vr, wr, re[j]);
                if (C) {
                    re[j] = fma(vi, wi, re[j]);
                    im[j] = fma(vr, wi, im[j]);
                    im[j] = fma(-vi, wr, im[j]);
                }
            }
        }
    }
    block_sum(re, im);
    if (threadIdx.x == 0)
#pragma unroll
        for (int j = 0; j < kJT; ++j)
            if (j0 + j < m) {
                partial[((int64_t)blockIdx.x * m + j0 + j) * 2] = re[j];
                partial[((int64_t)blockIdx.x * m + j0 + j) * 2 + 1] = im[j];
            }
}

__global__ void reduce_partials_kernel(const double* partial, int nblocks, int m, double* out) {
    int j = blockIdx.x;
    double re = 0.0, im = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
        re += partial[((int64_t)b * m + j) * 2];
        im += partial[((int64_t)b * m + j) * 2 + 1];
    }
    __shared__ double sr[32], si[32];
    re = warp_sum(re);
    im = warp_sum(im);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { sr[wid] = re; si[wid] = im; }
    __syncthreads();
    if (wid == 0) {
        int nw = blockDim.x / 32;
        re = lane < nw ? sr[lane] : 0.0;
        im = lane < nw ? si[lane] : 0.0;
        re = warp_sum(re);
        im = warp_sum(im);
        if (lane == 0) { out[2 * j] = re; out[2 * j + 1] = im; }
    }
}

// w -= sum_j V_j h_j   (mode 0)   or   out = sum_j V_j h_j   (mode 1)
template <typename S, bool C, int kMode>
__global__ void __launch_bounds__(kThreads) update_kernel(void* w, const void* V, int64_t ldv, int m, const double* h,
                                                          int64_t n) {
    __shared__ double hs[2 * 128];
    for (int j = threadIdx.x; j < 2 * m; j += blockDim.x) hs[j] = h[j];
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kThreads) {
        double ar = 0.0, ai = 0.0;
        for (int j = 0; j < m; ++j) {
            double vr, vi;
            ld<S, C>(V, (int64_t)j * ldv + i, vr, vi);
            double hr = hs[2 * j], hi = hs[2 * j + 1];
            ar = fma(vr, hr, ar);
            if (C) {
                ar = fma(-vi, hi, ar);
                ai = fma(vr, hi, ai);
                ai = fma(vi, hr, ai);
            }
        }
        if (kMode == 0) {
            double wr, wi;
            ld<S, C>(w, i, wr, wi);
            st<S, C>(w, i, wr - ar, wi - ai);
        } else {
            st<S, C>(w, i, ar, ai);
        }
    }
}

template <typename S, bool C>
__global__ void axpby_kernel(void* y, const void* x, double ar, double ai, double br, int64_t n) {
    // y = a*x + br*y
    for (int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kThreads) {
        double xr, xi, yr = 0.0, yi = 0.0;
        ld<S, C>(x, i, xr, xi);
        if (br != 0.0) ld<S, C>(y, i, yr, yi);
        st<S, C>(y, i, br * yr + ar * xr - ai * xi, br * yi + ar * xi + ai * xr);
    }
}

// Vt[:, c] = sum_j V[:, j] Y[j, c] for c < p into tmp, Y column-major m x p.
template <typename S, bool C>
__global__ void __launch_bounds__(kThreads) rotate_kernel(void* tmp, const void* V, int64_t ldv, int m, int p,
                                                          const double* Y, int64_t n) {
    extern __shared__ double ys[];
    for (int k = threadIdx.x; k < m * p; k += blockDim.x) ys[k] = Y[k];
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kThreads) {
        for (int c = 0; c < p; ++c) {
            double ar = 0.0, ai = 0.0;
            for (int j = 0; j < m; ++j) {
                double vr, vi;
                ld<S, C>(V, (int64_t)j * ldv + i, vr, vi);
                double y = ys[c * m + j];
                ar = fma(vr, y, ar);
                if (C) ai = fma(vi, y, ai);
            }
            st<S, C>(tmp, (int64_t)c * n + i, ar, ai);
        }
    }
}

template <typename S, bool C>
__global__ void copy_cols_kernel(void* V, int64_t ldv, const void* tmp, int p, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kThreads)
        for (int c = 0; c < p; ++c) {
            double r, im;
            ld<S, C>(tmp, (int64_t)c * n + i, r, im);
            st<S, C>(V, (int64_t)c * ldv + i, r, im);
        }
}

template <typename SA, typename SB, bool C>
__global__ void convert_kernel(const void* src, void* dst, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kThreads) {
        double r, im;
        ld<SA, C>(src, i, r, im);
        st<SB, C>(dst, i, r, im);
    }
}

// ------------------------------------------------- double-float storage
template <bool C>
__device__ __forceinline__ void ld_df(const void* p, int64_t i, DF& re, DF& im) {
    if (C) {
        float4 v = ((const float4*)p)[i];
        re = DF{v.x, v.y};
        im = DF{v.z, v.w};
    } else {
        float2 v = ((const float2*)p)[i];
        re = DF{v.x, v.y};
        im = DF{0.f, 0.f};
    }
}
template <bool C>
__device__ __forceinline__ void st_df(void* p, int64_t i, DF re, DF im) {
    if (C) ((float4*)p)[i] = make_float4(re.h, re.l, im.h, im.l);
    else ((float2*)p)[i] = make_float2(re.h, re.l);
}

// partial[b][j] = sum over the block of conj(V_j) w, in double-float; only the
// per-warp totals are converted to double.
template <bool C>
__global__ void __launch_bounds__(kThreads) dots_df_kernel(const void* V, int64_t ldv, int m, const void* w, int64_t n,
                                                           double* partial) {
    const int j0 = blockIdx.y * kJT;
    DF re[kJT], im[kJT];
#pragma unroll
    for (int j = 0; j < kJT; ++j) re[j] = im[j] = DF{0.f, 0.f};
    for (int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kThreads) {
        DF wr, wi;
        ld_df<C>(w, i, wr, wi);
#pragma unroll
        for (int j = 0; j < kJT; ++j) {
            if (j0 + j < m) {
                DF vr, vi;
                ld_df<C>(V, (int64_t)(j0 + j) * ldv + i, vr, vi);
                df_mac(re[j], vr.h, vr.l, wr.h, wr.l);
                if (C) {
                    df_mac(re[j], vi.h, vi.l, wi.h, wi.l);
                    df_mac(im[j], vr.h, vr.l, wi.h, wi.l);
                    df_mac(im[j], -vi.h, -vi.l, wr.h, wr.l);
                }
            }
        }
    }
    __shared__ double sh[kThreads / 32][2 * kJT];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < kJT; ++j) {
        for (int o = 16; o > 0; o >>= 1) {
            re[j] = df_add(re[j], df_shfl_xor(re[j], o, 32));
            if (C) im[j] = df_add(im[j], df_shfl_xor(im[j], o, 32));
        }
        if (lane == 0) {
            sh[wid][2 * j] = df_to_double(re[j]);
            sh[wid][2 * j + 1] = C ? df_to_double(im[j]) : 0.0;
        }
    }
    __syncthreads();
    if (threadIdx.x < 2 * kJT) {
        double t = 0;
        for (int q = 0; q < kThreads / 32; ++q) t += sh[q][threadIdx.x];
        const int j = threadIdx.x / 2;
        if (j0 + j < m) partial[((int64_t)blockIdx.x * m + j0 + j) * 2 + (threadIdx.x & 1)] = t;
    }
}

// w -= sum_j V_j h_j (mode 0) or out = sum_j V_j h_j (mode 1); hs holds each
// complex h_j as four floats (re hi, re lo, im hi, im lo)
template <bool C, int kMode>
__global__ void __launch_bounds__(kThreads) update_df_kernel(void* w, const void* V, int64_t ldv, int m,
                                                             const float4* h, int64_t n) {
    __shared__ float4 hs[128];
    for (int j = threadIdx.x; j < m; j += blockDim.x) hs[j] = h[j];
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kThreads) {
        DF ar{0.f, 0.f}, ai{0.f, 0.f};
        for (int j = 0; j < m; ++j) {
            DF vr, vi;
            ld_df<C>(V, (int64_t)j * ldv + i, vr, vi);
            const float4 hj = hs[j];
            df_mac(ar, vr.h, vr.l, hj.x, hj.y);
            if (C) {
                df_mac(ar, -vi.h, -vi.l, hj.z, hj.w);
                df_mac(ai, vr.h, vr.l, hj.z, hj.w);
                df_mac(ai, vi.h, vi.l, hj.x, hj.y);
            }
        }
        if (kMode == 0) {
            DF wr, wi;
            ld_df<C>(w, i, wr, wi);
            st_df<C>(w, i, df_add(wr, df_neg(ar)), df_add(wi, df_neg(ai)));
        } else {
            st_df<C>(w, i, ar, ai);
        }
    }
}

// y = a x + b y, a complex and b real, both split into float pairs
template <bool C>
__global__ void axpby_df_kernel(void* y, const void* x, float4 a, float2 b, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kThreads) {
        DF xr, xi, yr{0.f, 0.f}, yi{0.f, 0.f};
        ld_df<C>(x, i, xr, xi);
        if (b.x != 0.f) ld_df<C>(y, i, yr, yi);
        DF orr = df_mul(yr, DF{b.x, b.y}), oi = df_mul(yi, DF{b.x, b.y});
        df_mac(orr, a.x, a.y, xr.h, xr.l);
        if (C) {
            df_mac(orr, -a.z, -a.w, xi.h, xi.l);
            df_mac(oi, a.x, a.y, xi.h, xi.l);
            df_mac(oi, a.z, a.w, xr.h, xr.l);
        }
        st_df<C>(y, i, orr, oi);
    }
}

// tmp[:, c] = sum_j V[:, j] Y[j, c], Y (m x p, column-major) as float pairs
template <bool C>
__global__ void __launch_bounds__(kThreads) rotate_df_kernel(void* tmp, const void* V, int64_t ldv, int m, int p,
                                                             const float2* Y, int64_t n) {
    extern __shared__ float2 ysf[];
    for (int k = threadIdx.x; k < m * p; k += blockDim.x) ysf[k] = Y[k];
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kThreads) {
        for (int c = 0; c < p; ++c) {
            DF ar{0.f, 0.f}, ai{0.f, 0.f};
            for (int j = 0; j < m; ++j) {
                DF vr, vi;
                ld_df<C>(V, (int64_t)j * ldv + i, vr, vi);
                const float2 y = ysf[c * m + j];
                df_mac(ar, vr.h, vr.l, y.x, y.y);
                if (C) df_mac(ai, vi.h, vi.l, y.x, y.y);
            }
            st_df<C>(tmp, (int64_t)c * n + i, ar, ai);
        }
    }
}

template <bool C>
__global__ void copy_cols_df_kernel(void* V, int64_t ldv, const void* tmp, int p, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kThreads)
        for (int c = 0; c < p; ++c) {
            DF r, im;
            ld_df<C>(tmp, (int64_t)c * n + i, r, im);
            st_df<C>(V, (int64_t)c * ldv + i, r, im);
        }
}

// double <-> double-float storage (same real/complex-ness)
template <bool C>
__global__ void to_df_kernel(const double* in, void* out, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kThreads) {
        if (C) {
            DF a = df_from_double(in[2 * i]), b = df_from_double(in[2 * i + 1]);
            ((float4*)out)[i] = make_float4(a.h, a.l, b.h, b.l);
        } else {
            DF a = df_from_double(in[i]);
            ((float2*)out)[i] = make_float2(a.h, a.l);
        }
    }
}
template <bool C>
__global__ void from_df_kernel(const void* in, double* out, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x; i < n; i += (int64_t)gridDim.x * kThreads) {
        if (C) {
            float4 v = ((const float4*)in)[i];
            out[2 * i] = df_to_double(DF{v.x, v.y});
            out[2 * i + 1] = df_to_double(DF{v.z, v.w});
        } else {
            float2 v = ((const float2*)in)[i];
            out[i] = df_to_double(DF{v.x, v.y});
        }
    }
}

// ------------------------------------------------------- seeded normals
// splitmix64 (Steele, Lea & Flood 2014) of (seed, index) gives two uniforms;
// Box-Muller turns them into a standard normal.
__device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

__global__ void fill_normal_kernel(void* dst, int kind, int64_t ncomp, uint64_t seed) {
    for (int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x; i < ncomp; i += (int64_t)gridDim.x * kThreads) {
        const uint64_t a = splitmix64(seed ^ splitmix64((uint64_t)i));
        const uint64_t b = splitmix64(a);
        const float u1 = (float)((a >> 40) + 1) * 5.9604644775390625e-8f;   // (0, 1]
        const float u2 = (float)(b >> 40) * 5.9604644775390625e-8f;         // [0, 1)
        const float g = sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
        if (kind == 0) {
            ((double*)dst)[i] = (double)g;
        } else if (kind == 1) {
            ((float*)dst)[i] = g;
        } else {
            ((float2*)dst)[i] = make_float2(g, 0.f);
        }
    }
}

int nblocks(int64_t n) {
    int64_t b = (n + kThreads - 1) / kThreads;
    return (int)std::max<int64_t>(1, std::min<int64_t>(b, kMaxBlocks));
}

#define QS_DISPATCH(kind, FN, ...)                                       \
    switch (kind) {                                                      \
        case VKind::F64: FN<double, false>(__VA_ARGS__); break;          \
        case VKind::C128: FN<double, true>(__VA_ARGS__); break;          \
        case VKind::F32: FN<float, false>(__VA_ARGS__); break;           \
        default: FN<float, true>(__VA_ARGS__); break;                    \
    }

template <typename S, bool C>
void launch_dots(const void* V, int64_t ldv, int m, const void* w, int64_t n, double* partial, int nb, cudaStream_t s) {
    dim3 grid(nb, (m + kJT - 1) / kJT);
    dots_kernel<S, C><<<grid, kThreads, 0, s>>>(V, ldv, m, w, n, partial);
}
template <typename S, bool C>
void launch_update(void* w, const void* V, int64_t ldv, int m, const double* h, int64_t n, int mode, cudaStream_t s) {
    if (mode == 0) update_kernel<S, C, 0><<<nblocks(n), kThreads, 0, s>>>(w, V, ldv, m, h, n);
    else update_kernel<S, C, 1><<<nblocks(n), kThreads, 0, s>>>(w, V, ldv, m, h, n);
}
template <typename S, bool C>
void launch_axpby(void* y, const void* x, double ar, double ai, double br, int64_t n, cudaStream_t s) {
    axpby_kernel<S, C><<<nblocks(n), kThreads, 0, s>>>(y, x, ar, ai, br, n);
}
template <typename S, bool C>
void launch_rotate(void* tmp, void* V, int64_t ldv, int m, int p, const double* Y, int64_t n, cudaStream_t s) {
    rotate_kernel<S, C><<<nblocks(n), kThreads, (size_t)m * p * sizeof(double), s>>>(tmp, V, ldv, m, p, Y, n);
    copy_cols_kernel<S, C><<<nblocks(n), kThreads, 0, s>>>(V, ldv, tmp, p, n);
}

}  // namespace

Blas::Blas(VKind k, int64_t n_, cudaStream_t st) : kind(k), n(n_), s(st) {
    partial.alloc((size_t)kMaxBlocks * 128 * 2 * sizeof(double));
    coeffs.alloc(128 * 128 * sizeof(double));
    result.alloc(2 * 128 * sizeof(double));
}

void Blas::dots(const void* V, int64_t ldv, int m, const void* w, std::vector<cd>& h) {
    if (m > 128) throw Error(QS_ERR_UNSUPPORTED, "Krylov basis larger than 128 vectors");
    int nb = nblocks(n);
    if (vk_df(kind)) {
        dim3 grid(nb, (m + kJT - 1) / kJT);
        if (kind == VKind::CDF64) dots_df_kernel<true><<<grid, kThreads, 0, s>>>(V, ldv, m, w, n, partial.as<double>());
        else dots_df_kernel<false><<<grid, kThreads, 0, s>>>(V, ldv, m, w, n, partial.as<double>());
    } else {
        QS_DISPATCH(kind, launch_dots, V, ldv, m, w, n, partial.as<double>(), nb, s);
    }
    QS_CUDA(cudaGetLastError());
    reduce_partials_kernel<<<m, 256, 0, s>>>(partial.as<double>(), nb, m, result.as<double>());
    QS_CUDA(cudaGetLastError());
    note_launches(2);
    hbuf.resize(2 * m);
    QS_CUDA(cudaMemcpyAsync(hbuf.data(), result.p, 2 * m * sizeof(double), cudaMemcpyDeviceToHost, s));
    QS_CUDA(cudaStreamSynchronize(s));
    h.resize(m);
    for (int j = 0; j < m; ++j) h[j] = cd(hbuf[2 * j], hbuf[2 * j + 1]);
}

void Blas::upload_df(const std::vector<cd>& h, int m) {
    fbuf.resize(4 * m);
    for (int j = 0; j < m; ++j) {
        df_split_host(h[j].real(), fbuf[4 * j], fbuf[4 * j + 1]);
        df_split_host(h[j].imag(), fbuf[4 * j + 2], fbuf[4 * j + 3]);
    }
    QS_CUDA(cudaMemcpyAsync(coeffs.p, fbuf.data(), 4 * m * sizeof(float), cudaMemcpyHostToDevice, s));
}

void Blas::update(void* w, const void* V, int64_t ldv, int m, const std::vector<cd>& h) {
    if (m == 0) return;
    if (vk_df(kind)) {
        upload_df(h, m);
        if (kind == VKind::CDF64) update_df_kernel<true, 0><<<nblocks(n), kThreads, 0, s>>>(w, V, ldv, m, coeffs.as<float4>(), n);
        else update_df_kernel<false, 0><<<nblocks(n), kThreads, 0, s>>>(w, V, ldv, m, coeffs.as<float4>(), n);
        QS_CUDA(cudaGetLastError());
        note_launches(1);
        QS_CUDA(cudaStreamSynchronize(s));
        return;
    }
    hbuf.resize(2 * m);
    for (int j = 0; j < m; ++j) { hbuf[2 * j] = h[j].real(); hbuf[2 * j + 1] = h[j].imag(); }
    QS_CUDA(cudaMemcpyAsync(coeffs.p, hbuf.data(), 2 * m * sizeof(double), cudaMemcpyHostToDevice, s));
    QS_DISPATCH(kind, launch_update, w, V, ldv, m, coeffs.as<double>(), n, 0, s);
    QS_CUDA(cudaGetLastError());
    note_launches(1);
    QS_CUDA(cudaStreamSynchronize(s));
}

void Blas::combine(void* out, const void* V, int64_t ldv, int m, const std::vector<cd>& c) {
    if (vk_df(kind)) {
        upload_df(c, m);
        if (kind == VKind::CDF64) update_df_kernel<true, 1><<<nblocks(n), kThreads, 0, s>>>(out, V, ldv, m, coeffs.as<float4>(), n);
        else update_df_kernel<false, 1><<<nblocks(n), kThreads, 0, s>>>(out, V, ldv, m, coeffs.as<float4>(), n);
        QS_CUDA(cudaGetLastError());
        note_launches(1);
        QS_CUDA(cudaStreamSynchronize(s));
        return;
    }
    hbuf.resize(2 * m);
    for (int j = 0; j < m; ++j) { hbuf[2 * j] = c[j].real(); hbuf[2 * j + 1] = c[j].imag(); }
    QS_CUDA(cudaMemcpyAsync(coeffs.p, hbuf.data(), 2 * m * sizeof(double), cudaMemcpyHostToDevice, s));
    QS_DISPATCH(kind, launch_update, out, V, ldv, m, coeffs.as<double>(), n, 1, s);
    QS_CUDA(cudaGetLastError());
    note_launches(1);
    QS_CUDA(cudaStreamSynchronize(s));
}

double Blas::norm(const void* w) {
    std::vector<cd> h;
    dots(w, n, 1, w, h);
    return std::sqrt(std::max(0.0, h[0].real()));
}

cd Blas::dot(const void* a, const void* b) {
    std::vector<cd> h;
    dots(a, n, 1, b, h);
    return h[0];
}

static float4 split4(std::complex<double> a) {
    float4 r;
    df_split_host(a.real(), r.x, r.y);
    df_split_host(a.imag(), r.z, r.w);
    return r;
}

void Blas::scale(void* dst, const void* src, cd a) {
    if (vk_df(kind)) {
        if (kind == VKind::CDF64) axpby_df_kernel<true><<<nblocks(n), kThreads, 0, s>>>(dst, src, split4(a), make_float2(0.f, 0.f), n);
        else axpby_df_kernel<false><<<nblocks(n), kThreads, 0, s>>>(dst, src, split4(a), make_float2(0.f, 0.f), n);
        QS_CUDA(cudaGetLastError());
        note_launches(1);
        return;
    }
    QS_DISPATCH(kind, launch_axpby, dst, src, a.real(), a.imag(), 0.0, n, s);
    QS_CUDA(cudaGetLastError());
    note_launches(1);
}

void Blas::axpy(void* y, const void* x, cd a) {
    if (vk_df(kind)) {
        if (kind == VKind::CDF64) axpby_df_kernel<true><<<nblocks(n), kThreads, 0, s>>>(y, x, split4(a), make_float2(1.f, 0.f), n);
        else axpby_df_kernel<false><<<nblocks(n), kThreads, 0, s>>>(y, x, split4(a), make_float2(1.f, 0.f), n);
        QS_CUDA(cudaGetLastError());
        note_launches(1);
        return;
    }
    QS_DISPATCH(kind, launch_axpby, y, x, a.real(), a.imag(), 1.0, n, s);
    QS_CUDA(cudaGetLastError());
    note_launches(1);
}

void Blas::copy(void* dst, const void* src) {
    QS_CUDA(cudaMemcpyAsync(dst, src, n * vk_bytes(kind), cudaMemcpyDeviceToDevice, s));
}

void Blas::rotate(void* V, int64_t ldv, int m, int p, const std::vector<double>& Y, void* tmp) {
    if (vk_df(kind)) {
        fbuf.resize(2 * (size_t)m * p);
        for (size_t k = 0; k < (size_t)m * p; ++k) df_split_host(Y[k], fbuf[2 * k], fbuf[2 * k + 1]);
        QS_CUDA(cudaMemcpyAsync(coeffs.p, fbuf.data(), fbuf.size() * sizeof(float), cudaMemcpyHostToDevice, s));
        const size_t sm = (size_t)m * p * sizeof(float2);
        if (kind == VKind::CDF64) {
            rotate_df_kernel<true><<<nblocks(n), kThreads, sm, s>>>(tmp, V, ldv, m, p, coeffs.as<float2>(), n);
            copy_cols_df_kernel<true><<<nblocks(n), kThreads, 0, s>>>(V, ldv, tmp, p, n);
        } else {
            rotate_df_kernel<false><<<nblocks(n), kThreads, sm, s>>>(tmp, V, ldv, m, p, coeffs.as<float2>(), n);
            copy_cols_df_kernel<false><<<nblocks(n), kThreads, 0, s>>>(V, ldv, tmp, p, n);
        }
        QS_CUDA(cudaGetLastError());
        note_launches(2);
        QS_CUDA(cudaStreamSynchronize(s));
        return;
    }
    QS_CUDA(cudaMemcpyAsync(coeffs.p, Y.data(), (size_t)m * p * sizeof(double), cudaMemcpyHostToDevice, s));
    QS_DISPATCH(kind, launch_rotate, tmp, V, ldv, m, p, coeffs.as<double>(), n, s);
    QS_CUDA(cudaGetLastError());
    note_launches(2);
    QS_CUDA(cudaStreamSynchronize(s));
}

void fill_normal(void* dst, VKind k, int64_t n, uint64_t seed, cudaStream_t s) {
    const int64_t ncomp = n * (vk_complex(k) ? 2 : 1);
    const int kind = vk_df(k) ? 2 : (vk_single(k) ? 1 : 0);
    fill_normal_kernel<<<nblocks(ncomp), kThreads, 0, s>>>(dst, kind, ncomp, seed);
    QS_CUDA(cudaGetLastError());
    note_launches(1);
}

void convert_vec(const void* src, VKind ks, void* dst, VKind kd, int64_t n, cudaStream_t s) {
    bool c = vk_complex(ks);
    if (c != vk_complex(kd)) throw Error(QS_ERR_ARGUMENT, "real/complex mismatch in a precision conversion");
    if (vk_df(ks) || vk_df(kd)) {
        if (ks == kd) {
            QS_CUDA(cudaMemcpyAsync(dst, src, n * vk_bytes(ks), cudaMemcpyDeviceToDevice, s));
        } else if (vk_df(kd) && (ks == VKind::F64 || ks == VKind::C128)) {
            if (c) to_df_kernel<true><<<nblocks(n), kThreads, 0, s>>>((const double*)src, dst, n);
            else to_df_kernel<false><<<nblocks(n), kThreads, 0, s>>>((const double*)src, dst, n);
        } else if (vk_df(ks) && (kd == VKind::F64 || kd == VKind::C128)) {
            if (c) from_df_kernel<true><<<nblocks(n), kThreads, 0, s>>>(src, (double*)dst, n);
            else from_df_kernel<false><<<nblocks(n), kThreads, 0, s>>>(src, (double*)dst, n);
        } else {
            throw Error(QS_ERR_UNSUPPORTED, "double-float vectors convert to and from FP64 only");
        }
        QS_CUDA(cudaGetLastError());
        note_launches(1);
        return;
    }
    bool s1 = vk_single(ks), s2 = vk_single(kd);
    if (s1 == s2) {
        QS_CUDA(cudaMemcpyAsync(dst, src, n * vk_bytes(ks), cudaMemcpyDeviceToDevice, s));
        return;
    }
    if (c) {
        if (s1) convert_kernel<float, double, true><<<nblocks(n), kThreads, 0, s>>>(src, dst, n);
        else convert_kernel<double, float, true><<<nblocks(n), kThreads, 0, s>>>(src, dst, n);
    } else {
        if (s1) convert_kernel<float, double, false><<<nblocks(n), kThreads, 0, s>>>(src, dst, n);
        else convert_kernel<double, float, false><<<nblocks(n), kThreads, 0, s>>>(src, dst, n);
    }
    QS_CUDA(cudaGetLastError());
    note_launches(1);
}

}  // namespace qs
