// qs_batch.cu -- many independent eigsh solves in lockstep, one launch per step.
//
// The reference solves sector by sector (block_diag_hamiltonian / BlockOps,
// tools.jl:2213-2420, each an ARPACK run).  Here the vectors of all sectors
// live in one concatenated space (sector s owns rows [off_s, off_s + n_s)),
// and every Lanczos step is one launch of each kernel for all sectors: a
// multi-sector SpMV over the assembled operators (block -> sector map, each
// block loads its sector's value table into shared memory) and segmented
// multi-vector dots / updates for the reorthogonalisation.  Each sector keeps
// its own thick-restart state on the host; converged sectors drop out of the
// launches.  Complex vectors are used for all sectors when any sector is
// complex.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstring>
#include <random>
#include <vector>

#include "qs_dense.h"
#include "qs_internal.h"
#include "qs_krylov.h"

namespace qs {

namespace {

constexpr int kThreads = 256;
constexpr int kRowsPerBlock = 1024;   // rows of one sector per block (SpMV and BLAS)
constexpr int kJT = 8;

struct SectorDev {
    const int64_t* rowptr;
    const uint32_t* words;
    const int32_t* cols;
    const uint16_t* codes;
    const double2* table;     // complex value per code
    const float4* table_df;   // double-float value per code
    const uint16_t* stab;     // null without symmetry
    const double2* diag;      // complex diagonal
    int64_t off, n;
    int32_t packed, code_bits, ncodes, lanes;
    uint32_t code_mask;
    int32_t block_begin, nblocks;
    int32_t active;
    int32_t cm;               // complex matrix elements
};

// y = H_s x on every active sector; complex (kC) or real vectors.
template <bool kC, bool kDF>
__global__ void __launch_bounds__(kThreads) batch_spmv_kernel(const SectorDev* __restrict__ sec,
                                                              const int* __restrict__ bmap, const void* x, void* y) {
    __shared__ double2 tab[1024];
    __shared__ double rsq[kMaxGroup + 1];
    const int s = bmap[blockIdx.x];
    const SectorDev& S = sec[s];
    if (!S.active) return;
    const bool smem = S.ncodes <= 1024;
    if (smem)
        for (int i = threadIdx.x; i < S.ncodes; i += blockDim.x) tab[i] = S.table[i];
    for (int i = threadIdx.x; i <= kMaxGroup; i += blockDim.x) rsq[i] = i ? 1.0 / sqrt((double)i) : 0.0;
    __syncthreads();
    const int G = S.lanes;
    const int lane = threadIdx.x % G;
    const int sub = threadIdx.x / G;
    const int rows_per_pass = blockDim.x / G;
    const int64_t lb = blockIdx.x - S.block_begin;
    const int64_t r0 = lb * kRowsPerBlock;
    const int64_t r1 = min(S.n, r0 + kRowsPerBlock);
    // rounds are uniform across the block (shuffles inside)
    for (int64_t base = r0; base < r1; base += rows_per_pass) {
        const int64_t r = base + sub;
        const bool live = r < r1;
        const int64_t j0 = live ? S.rowptr[r] : 0, j1 = live ? S.rowptr[r + 1] : 0;
        double ar = 0, ai = 0;
        for (int64_t j = j0 + lane; j < j1; j += G) {
            uint32_t col, code;
            if (S.packed) {
                uint32_t w = __ldg(S.words + j);
                col = w >> S.code_bits;
                code = w & S.code_mask;
            } else {
                col = (uint32_t)__ldg(S.cols + j);
                code = __ldg(S.codes + j);
            }
            double2 v = smem ? tab[code] : S.table[code];
            if (kC) {
                double2 xv = ((const double2*)x)[S.off + col];
                ar += v.x * xv.x - v.y * xv.y;
                ai += v.x * xv.y + v.y * xv.x;
            } else {
                ar += v.x * ((const double*)x)[S.off + col];
            }
        }
        for (int o = G / 2; o > 0; o >>= 1) {
            ar += __shfl_xor_sync(0xffffffffu, ar, o, G);
            if (kC) ai += __shfl_xor_sync(0xffffffffu, ai, o, G);
        }
        if (lane == 0 && live) {
            double sc = S.stab ? rsq[S.stab[r]] : 1.0;
            double2 d = S.diag[r];
            if (kC) {
                double2 xv = ((const double2*)x)[S.off + r];
                double2 out;
                out.x = ar * sc + d.x * xv.x - d.y * xv.y;
                out.y = ai * sc + d.x * xv.y + d.y * xv.x;
                ((double2*)y)[S.off + r] = out;
            } else {
                ((double*)y)[S.off + r] = ar * sc + d.x * ((const double*)x)[S.off + r];
            }
        }
    }
}

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// partial[b][j] = sum over the block's rows of conj(V_j) w; V_j column-major
// with leading dimension ld (the concatenated length).
template <bool kC>
__global__ void __launch_bounds__(kThreads) batch_dots_kernel(const SectorDev* __restrict__ sec, const int* bmap,
                                                               const void* V, int64_t ld, int m, const void* w,
                                                               double* partial) {
    const int s = bmap[blockIdx.x];
    const SectorDev& S = sec[s];
    const int j0 = blockIdx.y * kJT;
    double re[kJT], im[kJT];
#pragma unroll
    for (int j = 0; j < kJT; ++j) re[j] = im[j] = 0.0;
    if (S.active) {
        const int64_t lb = blockIdx.x - S.block_begin;
        const int64_t r0 = lb * kRowsPerBlock, r1 = min(S.n, r0 + kRowsPerBlock);
        for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
            const int64_t i = S.off + r;
            double wr, wi = 0;
            if (kC) {
                double2 t = ((const double2*)w)[i];
                wr = t.x;
                wi = t.y;
            } else {
                wr = ((const double*)w)[i];
            }
#pragma unroll
            for (int j = 0; j < kJT; ++j) {
                if (j0 + j < m) {
                    if (kC) {
                        double2 v = ((const double2*)V)[(int64_t)(j0 + j) * ld + i];
                        re[j] = fma(v.x, wr, fma(v.y, wi, re[j]));
                        im[j] = fma(v.x, wi, fma(-v.y, wr, im[j]));
                    } else {
                        re[j] = fma(((const double*)V)[(int64_t)(j0 + j) * ld + i], wr, re[j]);
                    }
                }
            }
        }
    }
    __shared__ double sh[kThreads / 32][2 * kJT];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int j = 0; j < kJT; ++j) {
        double a = warp_sum(re[j]), b = warp_sum(im[j]);
        if (lane == 0) {
            sh[wid][2 * j] = a;
            sh[wid][2 * j + 1] = b;
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

// per sector and vector: sum the block partials
__global__ void batch_reduce_kernel(const SectorDev* __restrict__ sec, int m, const double* partial, double* out) {
    const int s = blockIdx.x, j = blockIdx.y;
    const SectorDev& S = sec[s];
    double re = 0, im = 0;
    if (S.active)
        for (int b = threadIdx.x; b < S.nblocks; b += blockDim.x) {
            re += partial[((int64_t)(S.block_begin + b) * m + j) * 2];
            im += partial[((int64_t)(S.block_begin + b) * m + j) * 2 + 1];
        }
    __shared__ double sr[32], si[32];
    re = warp_sum(re);
    im = warp_sum(im);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { sr[wid] = re; si[wid] = im; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0, b = 0;
        for (int q = 0; q < (int)(blockDim.x / 32); ++q) { a += sr[q]; b += si[q]; }
        out[((int64_t)s * m + j) * 2] = a;
        out[((int64_t)s * m + j) * 2 + 1] = b;
    }
}

// w -= sum_j V_j h[s][j] (mode 0), out = sum_j V_j h[s][j] (mode 1), on active sectors
template <bool kC, int kMode>
__global__ void __launch_bounds__(kThreads) batch_update_kernel(const SectorDev* __restrict__ sec, const int* bmap,
                                                                 void* w, const void* V, int64_t ld, int m,
                                                                 const double* h) {
    const int s = bmap[blockIdx.x];
    const SectorDev& S = sec[s];
    if (!S.active) return;
    __shared__ double hs[2 * 128];
    for (int j = threadIdx.x; j < 2 * m; j += blockDim.x) hs[j] = h[(int64_t)s * 2 * m + j];
    __syncthreads();
    const int64_t lb = blockIdx.x - S.block_begin;
    const int64_t r0 = lb * kRowsPerBlock, r1 = min(S.n, r0 + kRowsPerBlock);
    for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        const int64_t i = S.off + r;
        double ar = 0, ai = 0;
        for (int j = 0; j < m; ++j) {
            double hr = hs[2 * j], hi = hs[2 * j + 1];
            if (kC) {
                double2 v = ((const double2*)V)[(int64_t)j * ld + i];
                ar = fma(v.x, hr, fma(-v.y, hi, ar));
                ai = fma(v.x, hi, fma(v.y, hr, ai));
            } else {
                ar = fma(((const double*)V)[(int64_t)j * ld + i], hr, ar);
            }
        }
        if (kC) {
            double2* wp = (double2*)w + i;
            double2 o = kMode == 0 ? *wp : make_double2(0, 0);
            *wp = kMode == 0 ? make_double2(o.x - ar, o.y - ai) : make_double2(ar, ai);
        } else {
            double* wp = (double*)w + i;
            *wp = kMode == 0 ? *wp - ar : ar;
        }
    }
}

// w *= a[s] (real) on active sectors
template <bool kC>
__global__ void batch_scale_kernel(const SectorDev* __restrict__ sec, const int* bmap, void* w, const double* a) {
    const int s = bmap[blockIdx.x];
    const SectorDev& S = sec[s];
    if (!S.active) return;
    const double f = a[s];
    const int64_t lb = blockIdx.x - S.block_begin;
    const int64_t r0 = lb * kRowsPerBlock, r1 = min(S.n, r0 + kRowsPerBlock);
    for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        const int64_t i = S.off + r;
        if (kC) {
            double2 v = ((double2*)w)[i];
            ((double2*)w)[i] = make_double2(v.x * f, v.y * f);
        } else {
            ((double*)w)[i] *= f;
        }
    }
}

// V[:, c] (c < p) = sum_j V[:, j] Y_s[j, c] through tmp (ld-strided, p columns), Y per sector m x p
template <bool kC>
__global__ void __launch_bounds__(kThreads) batch_rotate_kernel(const SectorDev* __restrict__ sec, const int* bmap,
                                                                 void* V, int64_t ld, int m, int p, const double* Y,
                                                                 void* tmp) {
    const int s = bmap[blockIdx.x];
    const SectorDev& S = sec[s];
    if (!S.active) return;
    const double* Ys = Y + (int64_t)s * m * p;
    const int64_t lb = blockIdx.x - S.block_begin;
    const int64_t r0 = lb * kRowsPerBlock, r1 = min(S.n, r0 + kRowsPerBlock);
    for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        const int64_t i = S.off + r;
        for (int c = 0; c < p; ++c) {
            double ar = 0, ai = 0;
            for (int j = 0; j < m; ++j) {
                double y = Ys[(int64_t)c * m + j];
                if (kC) {
                    double2 v = ((const double2*)V)[(int64_t)j * ld + i];
                    ar = fma(v.x, y, ar);
                    ai = fma(v.y, y, ai);
                } else {
                    ar = fma(((const double*)V)[(int64_t)j * ld + i], y, ar);
                }
            }
            if (kC) ((double2*)tmp)[(int64_t)c * ld + i] = make_double2(ar, ai);
            else ((double*)tmp)[(int64_t)c * ld + i] = ar;
        }
        for (int c = 0; c < p; ++c) {
            if (kC) ((double2*)V)[(int64_t)c * ld + i] = ((const double2*)tmp)[(int64_t)c * ld + i];
            else ((double*)V)[(int64_t)c * ld + i] = ((const double*)tmp)[(int64_t)c * ld + i];
        }
    }
}

template <bool kC>
__global__ void batch_copy_col_kernel(const SectorDev* __restrict__ sec, const int* bmap, void* dst, const void* src) {
    const int s = bmap[blockIdx.x];
    const SectorDev& S = sec[s];
    if (!S.active) return;
    const int64_t lb = blockIdx.x - S.block_begin;
    const int64_t r0 = lb * kRowsPerBlock, r1 = min(S.n, r0 + kRowsPerBlock);
    for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        const int64_t i = S.off + r;
        if (kC) ((double2*)dst)[i] = ((const double2*)src)[i];
        else ((double*)dst)[i] = ((const double*)src)[i];
    }
}

using cd = std::complex<double>;

struct Batch {
    std::vector<Op*> ops;
    std::vector<SectorDev> hsec;
    DevBuf dsec, dmap, partial, hbufd, ybuf;
    int nblocks = 0;
    int64_t ntot = 0;
    bool cplx = false;
    cudaStream_t s = nullptr;
    int64_t launches = 0;
    size_t esz() const { return cplx ? 16 : 8; }

    void upload_active() {
        QS_CUDA(cudaMemcpyAsync(dsec.p, hsec.data(), hsec.size() * sizeof(SectorDev), cudaMemcpyHostToDevice, s));
    }
    void spmv(const void* x, void* y) {
        if (cplx) batch_spmv_kernel<true, false><<<nblocks, kThreads, 0, s>>>(dsec.as<SectorDev>(), dmap.as<int>(), x, y);
        else batch_spmv_kernel<false, false><<<nblocks, kThreads, 0, s>>>(dsec.as<SectorDev>(), dmap.as<int>(), x, y);
        QS_CUDA(cudaGetLastError());
        ++launches;
    }
    // h[s][j] = <V_j, w>_s for all sectors
    void dots(const void* V, int m, const void* w, std::vector<cd>& h) {
        dim3 grid(nblocks, (m + kJT - 1) / kJT);
        if (cplx) batch_dots_kernel<true><<<grid, kThreads, 0, s>>>(dsec.as<SectorDev>(), dmap.as<int>(), V, ntot, m, w, partial.as<double>());
        else batch_dots_kernel<false><<<grid, kThreads, 0, s>>>(dsec.as<SectorDev>(), dmap.as<int>(), V, ntot, m, w, partial.as<double>());
        QS_CUDA(cudaGetLastError());
        batch_reduce_kernel<<<dim3((unsigned)hsec.size(), m), 256, 0, s>>>(dsec.as<SectorDev>(), m, partial.as<double>(),
                                                                          hbufd.as<double>());
        QS_CUDA(cudaGetLastError());
        launches += 2;
        std::vector<double> tmp(hsec.size() * m * 2);
        QS_CUDA(cudaMemcpyAsync(tmp.data(), hbufd.p, tmp.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
        QS_CUDA(cudaStreamSynchronize(s));
        h.resize(hsec.size() * m);
        for (size_t i = 0; i < h.size(); ++i) h[i] = cd(tmp[2 * i], tmp[2 * i + 1]);
    }
    void update(void* w, const void* V, int m, const std::vector<cd>& h, int mode) {
        std::vector<double> tmp(hsec.size() * m * 2);
        for (size_t i = 0; i < h.size(); ++i) { tmp[2 * i] = h[i].real(); tmp[2 * i + 1] = h[i].imag(); }
        QS_CUDA(cudaMemcpyAsync(hbufd.p, tmp.data(), tmp.size() * sizeof(double), cudaMemcpyHostToDevice, s));
        if (cplx) {
            if (mode == 0) batch_update_kernel<true, 0><<<nblocks, kThreads, 0, s>>>(dsec.as<SectorDev>(), dmap.as<int>(), w, V, ntot, m, hbufd.as<double>());
            else batch_update_kernel<true, 1><<<nblocks, kThreads, 0, s>>>(dsec.as<SectorDev>(), dmap.as<int>(), w, V, ntot, m, hbufd.as<double>());
        } else {
            if (mode == 0) batch_update_kernel<false, 0><<<nblocks, kThreads, 0, s>>>(dsec.as<SectorDev>(), dmap.as<int>(), w, V, ntot, m, hbufd.as<double>());
            else batch_update_kernel<false, 1><<<nblocks, kThreads, 0, s>>>(dsec.as<SectorDev>(), dmap.as<int>(), w, V, ntot, m, hbufd.as<double>());
        }
        QS_CUDA(cudaGetLastError());
        ++launches;
    }
    void scale(void* w, const std::vector<double>& a) {
        QS_CUDA(cudaMemcpyAsync(hbufd.p, a.data(), a.size() * sizeof(double), cudaMemcpyHostToDevice, s));
        if (cplx) batch_scale_kernel<true><<<nblocks, kThreads, 0, s>>>(dsec.as<SectorDev>(), dmap.as<int>(), w, hbufd.as<double>());
        else batch_scale_kernel<false><<<nblocks, kThreads, 0, s>>>(dsec.as<SectorDev>(), dmap.as<int>(), w, hbufd.as<double>());
        QS_CUDA(cudaGetLastError());
        ++launches;
    }
    void rotate(void* V, int m, int p, const std::vector<double>& Y, void* tmp) {
        QS_CUDA(cudaMemcpyAsync(ybuf.p, Y.data(), Y.size() * sizeof(double), cudaMemcpyHostToDevice, s));
        if (cplx) batch_rotate_kernel<true><<<nblocks, kThreads, 0, s>>>(dsec.as<SectorDev>(), dmap.as<int>(), V, ntot, m, p, ybuf.as<double>(), tmp);
        else batch_rotate_kernel<false><<<nblocks, kThreads, 0, s>>>(dsec.as<SectorDev>(), dmap.as<int>(), V, ntot, m, p, ybuf.as<double>(), tmp);
        QS_CUDA(cudaGetLastError());
        ++launches;
    }
    void copy_col(void* dst, const void* src) {
        if (cplx) batch_copy_col_kernel<true><<<nblocks, kThreads, 0, s>>>(dsec.as<SectorDev>(), dmap.as<int>(), dst, src);
        else batch_copy_col_kernel<false><<<nblocks, kThreads, 0, s>>>(dsec.as<SectorDev>(), dmap.as<int>(), dst, src);
        QS_CUDA(cudaGetLastError());
        ++launches;
    }
};

}  // namespace

// Thick-restart Lanczos (same iteration as eigsh in qs_krylov.cu) on every
// operator at once; values: nops * k, ascending per operator.
void eigsh_batch(Op** ops, int nops, const qs_eigsh_opts& o, double* values, void** vectors, qs_eigsh_info* infos) {
    auto t0 = std::chrono::steady_clock::now();
    if (nops <= 0) throw Error(QS_ERR_ARGUMENT, "no operators");
    const int k = o.k;
    if (o.which != 0 && o.which != 1) throw Error(QS_ERR_UNSUPPORTED, "which must be SA or LA on this engine");
    Batch B;
    B.s = ops[0]->stream;
    int64_t off = 0;
    int maxn = 0;
    for (int i = 0; i < nops; ++i) {
        Op& op = *ops[i];
        if (!op.assembled) op_assemble(op);
        if (!op.hermitian) throw Error(QS_ERR_UNSUPPORTED, "eigsh on this engine needs Hermitian operators");
        if (op.complex_mat) B.cplx = true;
        const int64_t n = op.basis->n;
        if (k < 1 || k >= n - 1) throw Error(QS_ERR_ARGUMENT, "batched eigsh needs 1 <= k < Ns - 1 for every operator");
        maxn = (int)std::max<int64_t>(maxn, n);
        SectorDev d{};
        const Assembled& M = op.asm_;
        d.rowptr = M.rowptr.as<int64_t>();
        d.words = M.words.as<uint32_t>();
        d.cols = M.cols.as<int32_t>();
        d.codes = M.codes.as<uint16_t>();
        d.table = M.table64.as<double2>();
        d.table_df = M.table_df.as<float4>();
        d.stab = op.basis->symmetric ? op.basis->d_stab.as<uint16_t>() : nullptr;
        d.diag = op.d_diag.as<double2>();
        d.off = off;
        d.n = n;
        d.packed = M.packed;
        d.code_bits = M.code_bits;
        d.code_mask = M.code_bits >= 32 ? 0xffffffffu : ((1u << M.code_bits) - 1u);
        d.ncodes = M.ncodes;
        d.lanes = M.lanes;
        d.block_begin = B.nblocks;
        d.nblocks = (int)((n + kRowsPerBlock - 1) / kRowsPerBlock);
        d.active = 1;
        d.cm = op.complex_mat;
        B.nblocks += d.nblocks;
        off += n;
        B.hsec.push_back(d);
        B.ops.push_back(&op);
    }
    B.ntot = off;
    const int nsec = nops;
    std::vector<int> bmap(B.nblocks);
    for (int s = 0; s < nsec; ++s)
        for (int b = 0; b < B.hsec[s].nblocks; ++b) bmap[B.hsec[s].block_begin + b] = s;
    B.dsec.alloc(nsec * sizeof(SectorDev));
    B.dmap.alloc(B.nblocks * sizeof(int));
    QS_CUDA(cudaMemcpy(B.dmap.p, bmap.data(), bmap.size() * sizeof(int), cudaMemcpyHostToDevice));
    B.upload_active();
    int m = o.ncv > 0 ? o.ncv : std::max(20, 2 * k + 1);
    m = std::min(m, 64);
    m = (int)std::min<int64_t>(m, maxn);
    for (int s = 0; s < nsec; ++s) m = (int)std::min<int64_t>(m, B.hsec[s].n);
    if (m <= k) throw Error(QS_ERR_ARGUMENT, "ncv must exceed k");
    const double tol = o.tol > 0 ? o.tol : 2.220446049250313e-16;
    const int maxiter = o.maxiter > 0 ? o.maxiter : 300;
    B.partial.alloc((size_t)B.nblocks * m * 2 * sizeof(double));
    B.hbufd.alloc((size_t)nsec * std::max(m, 1) * 2 * sizeof(double));
    B.ybuf.alloc((size_t)nsec * m * m * sizeof(double));
    const size_t es = B.esz();
    DevBuf V((size_t)B.ntot * (m + 1) * es), tmp((size_t)B.ntot * m * es);
    auto col = [&](int j) { return (char*)V.p + (size_t)j * B.ntot * es; };
    // start vectors: seeded normal entries (or one v0 per operator, host, op dtype)
    {
        std::vector<double> h((B.cplx ? 2 : 1) * B.ntot);
        std::mt19937_64 rng(20261203ull);
        std::normal_distribution<double> nd(0.0, 1.0);
        for (auto& v : h) v = nd(rng);
        QS_CUDA(cudaMemcpy(V.p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
    std::vector<cd> h, h2;
    B.dots(col(0), 1, col(0), h);
    std::vector<double> sc(nsec);
    for (int s = 0; s < nsec; ++s) sc[s] = 1.0 / std::sqrt(h[s].real());
    B.scale(col(0), sc);
    // per-sector Lanczos state
    std::vector<std::vector<double>> T(nsec, std::vector<double>((size_t)m * m, 0.0));
    std::vector<double> beta(nsec, 0.0);
    std::vector<std::vector<double>> theta(nsec);
    std::vector<int> nconv(nsec, 0), restarts(nsec, 0);
    std::vector<double> maxrel(nsec, 0.0);
    std::vector<char> done(nsec, 0);
    const double eps23 = std::pow(2.220446049250313e-16, 2.0 / 3.0);
    int j0 = 0;
    int64_t matvecs = 0;
    for (int iter = 0; iter < maxiter; ++iter) {
        for (int j = j0; j < m; ++j) {
            void* wv = col(j + 1);
            B.spmv(col(j), wv);
            ++matvecs;
            B.dots(V.p, j + 1, wv, h);
            B.update(wv, V.p, j + 1, h, 0);
            B.dots(V.p, j + 1, wv, h2);
            B.update(wv, V.p, j + 1, h2, 0);
            B.dots(wv, 1, wv, h2);  // norms
            for (int s = 0; s < nsec; ++s) {
                if (done[s]) continue;
                T[s][(size_t)j * m + j] = (h[(size_t)s * (j + 1) + j]).real();
                beta[s] = std::sqrt(std::max(0.0, h2[s].real()));
                if (j + 1 < m) T[s][(size_t)j * m + j + 1] = T[s][(size_t)(j + 1) * m + j] = beta[s];
                sc[s] = beta[s] > 0 ? 1.0 / beta[s] : 0.0;
            }
            B.scale(wv, sc);
        }
        // Ritz values per sector; restart or finish
        std::vector<double> Yall((size_t)nsec * m * m, 0.0);
        int p = std::min(m - 2, k + (m - k) / 2);
        p = std::max(p, std::min(k, m - 1));
        bool any_active = false;
        std::vector<std::vector<double>> Ysave(nsec);
        for (int s = 0; s < nsec; ++s) {
            if (done[s]) continue;
            std::vector<double> w, Y;
            sym_eig(m, T[s], w, Y);
            std::vector<int> order(m);
            for (int i = 0; i < m; ++i) order[i] = o.which == 0 ? i : m - 1 - i;
            int nc = 0;
            double mr = 0;
            for (int q = 0; q < k; ++q) {
                int i = order[q];
                double bound = std::fabs(beta[s] * Y[(size_t)(m - 1) * m + i]);
                mr = std::max(mr, bound / std::max(eps23, std::fabs(w[i])));
                if (bound <= tol * std::max(eps23, std::fabs(w[i]))) ++nc;
            }
            nconv[s] = nc;
            maxrel[s] = mr;
            restarts[s] = iter;
            theta[s].assign(k, 0.0);
            for (int q = 0; q < k; ++q) theta[s][q] = w[order[q]];
            const bool fin = nc >= k || iter == maxiter - 1;
            const int keep = fin ? k : p;
            Ysave[s].assign((size_t)m * keep, 0.0);
            for (int q = 0; q < keep; ++q)
                for (int r = 0; r < m; ++r) Ysave[s][(size_t)q * m + r] = Y[(size_t)r * m + order[q]];
            if (!fin) {
                std::fill(T[s].begin(), T[s].end(), 0.0);
                for (int q = 0; q < p; ++q) {
                    T[s][(size_t)q * m + q] = w[order[q]];
                    double c = beta[s] * Y[(size_t)(m - 1) * m + order[q]];
                    T[s][(size_t)q * m + p] = T[s][(size_t)p * m + q] = c;
                }
                any_active = true;
            }
        }
        // finished sectors: Ritz vectors into V[:, 0:k] and output, then drop out
        for (int pass = 0; pass < 2; ++pass) {
            // pass 0: rotate finishing sectors with keep = k; pass 1: continuing with keep = p
            const int keep = pass == 0 ? k : p;
            std::vector<char> act(nsec, 0);
            bool anyp = false;
            for (int s = 0; s < nsec; ++s) {
                if (done[s] || Ysave[s].empty()) continue;
                const bool fin = nconv[s] >= k || iter == maxiter - 1;
                if ((pass == 0) != fin) continue;
                act[s] = 1;
                anyp = true;
                std::copy(Ysave[s].begin(), Ysave[s].end(), Yall.begin() + (size_t)s * m * keep);
            }
            if (!anyp) continue;
            for (int s = 0; s < nsec; ++s) B.hsec[s].active = act[s];
            B.upload_active();
            B.rotate(V.p, m, keep, Yall, tmp.p);
            if (pass == 1) B.copy_col(col(p), col(m));
            if (pass == 0)
                for (int s = 0; s < nsec; ++s)
                    if (act[s]) done[s] = 1;
        }
        for (int s = 0; s < nsec; ++s) B.hsec[s].active = !done[s];
        B.upload_active();
        j0 = p;
        if (!any_active) break;
    }
    QS_CUDA(cudaStreamSynchronize(B.s));
    for (int s = 0; s < nsec; ++s) {
        if (nconv[s] < k) throw Error(QS_ERR_NOT_CONVERGED, "batched eigsh did not converge within maxiter restarts");
        for (int q = 0; q < k; ++q) values[(size_t)s * k + q] = theta[s][q];
        if (vectors && vectors[s]) {
            const Op& op = *B.ops[s];
            const bool ocx = op.complex_mat;
            std::vector<double> hb((size_t)B.hsec[s].n * (B.cplx ? 2 : 1));
            for (int q = 0; q < k; ++q) {
                QS_CUDA(cudaMemcpy(hb.data(), (char*)V.p + ((size_t)q * B.ntot + B.hsec[s].off) * es,
                                   (size_t)B.hsec[s].n * es, cudaMemcpyDeviceToHost));
                double* out = (double*)vectors[s] + (size_t)q * B.hsec[s].n * (ocx ? 2 : 1);
                if (B.cplx && !ocx)
                    for (int64_t i = 0; i < B.hsec[s].n; ++i) out[i] = hb[2 * i];
                else
                    std::memcpy(out, hb.data(), hb.size() * sizeof(double));
            }
        }
        if (infos) {
            infos[s].nconv = nconv[s];
            infos[s].restarts = restarts[s];
            infos[s].matvecs = matvecs;
            infos[s].max_rel_residual = maxrel[s];
            infos[s].seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        }
    }
    note_launches(B.launches);
}

}  // namespace qs
