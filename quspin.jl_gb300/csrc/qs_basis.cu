// qs_basis.cu -- symmetry-reduced spin-1/2 basis on the device.
//
// Replaces SpinBasis1D (src/basis.jl:622-777) and the projector machinery of
// src/symmetry_basis.jl.  The reference enumerates the whole parent sector,
// hashes it and builds an explicit sparse projector; here every candidate state
// is tested independently on the device ("is it the minimum of its orbit, and
// is the sector's character trivial on its stabiliser?"), survivors are
// compacted in ascending order -- exactly the reference's column order -- and
// only the representatives (plus a 16-bit stabiliser order) stay in HBM.
//
// The reference's public representative of a column is the argmax-|coef| entry
// of its floating-point projector column (src/symmetry_basis.jl:215-232), which
// is not always the orbit minimum.  basis_compute_refrep replays the reference's
// projector arithmetic per column (qs_common.h primitives) to reproduce it bit
// for bit, and basis_representative does the same for normalization/get_amp.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

#include "qs_device.cuh"
#include "qs_internal.h"

namespace qs {

Basis::~Basis() {
    if (stream) cudaStreamDestroy(stream);
}

// ----------------------------------------------------------- group closure
namespace {

struct Elem {
    int refl, shift;
    uint64_t mask;
    int j;        // translation count (character exponent)
    int sign;     // product of involution characters
    std::vector<uint64_t> img;
};

uint64_t elem_apply(const Elem& e, uint64_t s, int L) {
    uint64_t r = e.refl ? brev_host(s, L) : s;
    return rotl_bits<uint64_t>(r, e.shift % L, L, low_mask(L)) ^ e.mask;
}

void elem_fill(Elem& e, int L) {
    e.img.resize(L + 1);
    e.img[0] = elem_apply(e, 0, L);
    for (int b = 0; b < L; ++b) e.img[b + 1] = elem_apply(e, 1ull << b, L);
}

// e2 o e1
Elem elem_compose(const Elem& e2, const Elem& e1, int L, int nT) {
    Elem r;
    int sh1 = e2.refl ? -e1.shift : e1.shift;
    r.shift = (((e2.shift + sh1) % L) + L) % L;
    r.refl = e1.refl ^ e2.refl;
    uint64_t m1 = e2.refl ? brev_host(e1.mask, L) : e1.mask;
    r.mask = rotl_bits<uint64_t>(m1, e2.shift % L, L, low_mask(L)) ^ e2.mask;
    r.j = nT > 0 ? ((e1.j + e2.j) % nT) : 0;
    r.sign = e1.sign * e2.sign;
    elem_fill(r, L);
    return r;
}

struct Closure {
    std::vector<Elem> elems;
    std::map<std::vector<uint64_t>, int> index;
};

cplx char_value(const Elem& e, int kmom, int nT) {
    double re = 1.0, im = 0.0;
    if (nT > 0 && kmom != 0) {
        long q = ((long)kmom * (long)e.j) % nT;
        double arg = 2.0 * M_PI * (double)q / (double)nT;
        re = std::cos(arg);
        im = std::sin(arg);
    }
    return cx(re * e.sign, im * e.sign);
}

// Closure of the generators; returns false when the requested character is not
// a character of the generated group (the sector is then empty).
bool close_group(const std::vector<Elem>& gens, int L, int kmom, int nT, Closure& C) {
    Elem id{0, 0, 0, 0, 1, {}};
    elem_fill(id, L);
    C.elems.push_back(id);
    C.index[id.img] = 0;
    for (size_t i = 0; i < C.elems.size(); ++i) {
        for (const Elem& g : gens) {
            Elem c = elem_compose(g, C.elems[i], L, nT);
            auto it = C.index.find(c.img);
            if (it != C.index.end()) {
                cplx a = char_value(C.elems[it->second], kmom, nT), b = char_value(c, kmom, nT);
                if (std::fabs(a.re - b.re) > 1e-9 || std::fabs(a.im - b.im) > 1e-9) return false;
                continue;
            }
            if ((int)C.elems.size() >= kMaxGroup) throw Error(QS_ERR_UNSUPPORTED, "symmetry group too large");
            C.index[c.img] = (int)C.elems.size();
            C.elems.push_back(c);
        }
    }
    return true;
}

void fill_desc(GroupDesc& d, const Closure& C, int L, int kmom, int nT) {
    std::memset(&d, 0, sizeof(d));
    d.L = L;
    d.lmask = low_mask(L);
    std::vector<int> order(C.elems.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        const Elem &x = C.elems[a], &y = C.elems[b];
        if (x.refl != y.refl) return x.refl < y.refl;
        return x.shift < y.shift;
    });
    d.ng = (int)order.size();
    d.nperm = 0;
    d.real_chars = 1;
    int prev_refl = -1, prev_shift = -1;
    for (int k = 0; k < d.ng; ++k) {
        const Elem& e = C.elems[order[k]];
        if (e.refl != prev_refl || e.shift != prev_shift) {
            if (d.nperm >= kMaxPerm) throw Error(QS_ERR_UNSUPPORTED, "symmetry group too large");
            d.perm_refl[d.nperm] = (int8_t)e.refl;
            d.perm_shift[d.nperm] = (int8_t)e.shift;
            d.perm_begin[d.nperm] = (int16_t)k;
            d.nperm++;
            prev_refl = e.refl;
            prev_shift = e.shift;
        }
        d.mask[k] = e.mask;
        cplx ch = char_value(e, kmom, nT);
        d.chi_re[k] = ch.re;
        d.chi_im[k] = ch.im;
        if (std::fabs(ch.im) > 1e-12) d.real_chars = 0;
    }
    d.perm_begin[d.nperm] = (int16_t)d.ng;
}

int64_t binom_host(int n, int k) {
    if (k < 0 || k > n) return 0;
    int64_t r = 1;
    for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
    return r;
}

}  // namespace

// ------------------------------------------------- general site maps
namespace {

// One element of a group of general site maps: t = perm(s) ^ mask, with its
// character; keyed, like Elem, by the images of 0 and of every single bit.
struct GElem {
    std::vector<int> perm;
    uint64_t mask = 0;
    cplx chi = cx(1.0, 0.0);
    std::vector<uint64_t> img;
};

uint64_t gelem_apply(const GElem& e, uint64_t s, int L) {
    uint64_t r = 0;
    for (int b = 0; b < L; ++b)
        if ((s >> b) & 1ull) r |= 1ull << e.perm[b];
    return r ^ e.mask;
}

void gelem_fill(GElem& e, int L) {
    e.img.resize(L + 1);
    e.img[0] = gelem_apply(e, 0, L);
    for (int b = 0; b < L; ++b) e.img[b + 1] = gelem_apply(e, 1ull << b, L);
}

// e2 o e1 (e1 first)
GElem gelem_compose(const GElem& e2, const GElem& e1, int L) {
    GElem r;
    r.perm.resize(L);
    uint64_t pm = 0;
    for (int b = 0; b < L; ++b) {
        r.perm[b] = e2.perm[e1.perm[b]];
        if ((e1.mask >> b) & 1ull) pm |= 1ull << e2.perm[b];
    }
    r.mask = pm ^ e2.mask;
    r.chi = cx_mul(e1.chi, e2.chi);
    gelem_fill(r, L);
    return r;
}

GElem gelem_identity(int L) {
    GElem e;
    e.perm.resize(L);
    for (int b = 0; b < L; ++b) e.perm[b] = b;
    gelem_fill(e, L);
    return e;
}

struct GClosure {
    std::vector<GElem> elems;
    std::map<std::vector<uint64_t>, int> index;
};

// Closure of the generators; false when the characters contradict each other
// (the sector is then empty).
bool close_general(const std::vector<GElem>& gens, int L, GClosure& C) {
    GElem id = gelem_identity(L);
    C.elems.push_back(id);
    C.index[id.img] = 0;
    for (size_t i = 0; i < C.elems.size(); ++i) {
        for (const GElem& g : gens) {
            GElem c = gelem_compose(g, C.elems[i], L);
            auto it = C.index.find(c.img);
            if (it != C.index.end()) {
                const cplx a = C.elems[it->second].chi;
                if (std::fabs(a.re - c.chi.re) > 1e-9 || std::fabs(a.im - c.chi.im) > 1e-9) return false;
                continue;
            }
            if ((int)C.elems.size() >= kMaxGroup) throw Error(QS_ERR_UNSUPPORTED, "symmetry group too large");
            C.index[c.img] = (int)C.elems.size();
            C.elems.push_back(c);
        }
    }
    return true;
}

// GroupDesc of a general group: elements grouped by permutation, one set of
// byte tables per distinct permutation (appended to `tables`).
void fill_desc_general(GroupDesc& d, const GClosure& C, int L, std::vector<uint64_t>& tables,
                       std::vector<std::vector<int>>* perms = nullptr) {
    std::memset(&d, 0, sizeof(d));
    d.L = L;
    d.lmask = low_mask(L);
    d.general = 1;
    d.nbytes = (L + 7) / 8;
    std::vector<int> order(C.elems.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return C.elems[a].perm < C.elems[b].perm; });
    d.ng = (int)order.size();
    d.real_chars = 1;
    const std::vector<int>* prev = nullptr;
    tables.clear();
    for (int k = 0; k < d.ng; ++k) {
        const GElem& e = C.elems[order[k]];
        if (!prev || *prev != e.perm) {
            if (d.nperm >= kMaxPerm) throw Error(QS_ERR_UNSUPPORTED, "symmetry group has too many site permutations");
            d.perm_begin[d.nperm] = (int16_t)k;
            d.nperm++;
            prev = &e.perm;
            if (perms) perms->push_back(e.perm);
            for (int byte = 0; byte < 8; ++byte)
                for (int v = 0; v < 256; ++v) {
                    uint64_t img = 0;
                    for (int i = 0; i < 8; ++i) {
                        const int b = 8 * byte + i;
                        if (b < L && ((v >> i) & 1)) img |= 1ull << e.perm[b];
                    }
                    tables.push_back(img);
                }
        }
        d.mask[k] = e.mask;
        d.chi_re[k] = e.chi.re;
        d.chi_im[k] = e.chi.im;
        if (std::fabs(e.chi.im) > 1e-12) d.real_chars = 0;
    }
    d.perm_begin[d.nperm] = (int16_t)d.ng;
}

}  // namespace

// ------------------------------------------------------------ enumeration
namespace {

constexpr int kChunk = 64;        // candidates per thread
constexpr int kEnumThreads = 256;

// Group scan with early exit: is s the minimum of its orbit, and is the
// character trivial on its stabiliser?
template <typename U>
__device__ __forceinline__ int is_rep(const GroupSmem& g, const int8_t* chi_one, U s) {
    const int L = g.L;
    const U m = (U)g.lmask;
    U base[2];
    base[0] = s;
    base[1] = brev_bits(s, L);
    int stab = 0;
    for (int p = 0; p < g.nperm; ++p) {
        U r = g.general ? (U)gperm_apply(g.gtab, p, g.nbytes, (uint64_t)s)
                        : rotl_bits<U>(base[g.refl[p]], g.shift[p], L, m);
        const int e1 = g.begin[p + 1];
        for (int e = g.begin[p]; e < e1; ++e) {
            U c = r ^ (U)g.mask[e];
            if (c < s) return 0;
            if (c == s) {
                if (!chi_one[e]) return 0;
                ++stab;
            }
        }
    }
    return stab;
}

template <typename U>
__device__ __forceinline__ U unrank_fixed(int64_t r, int L, int nup, const uint64_t* binom, int bstride) {
    U s = 0;
    int b = L - 1;
    for (int p = nup; p >= 1; --p) {
        while ((int64_t)binom[b * bstride + p] > r) --b;
        s |= (U)1 << b;
        r -= (int64_t)binom[b * bstride + p];
        --b;
    }
    return s;
}

template <typename U>
__device__ __forceinline__ U gosper_next(U s) {
    U lowest = s & (~s + 1);
    U next = s + lowest;
    int tz = (sizeof(U) == 8) ? __ffsll((long long)lowest) - 1 : __ffs((int)lowest) - 1;
    return next | (((next ^ s) >> 2) >> tz);
}

struct EnumArgs {
    const GroupDesc* group;
    const int8_t* chi_one;
    const uint64_t* binom;
    int bstride;
    int L, nup;
    int64_t total;      // candidates
    int64_t nchunks;
    int64_t* counts;    // per chunk
    const int64_t* offsets;
    void* reps;
    uint16_t* stab;
};

template <typename U, bool kWrite>
__global__ void __launch_bounds__(kEnumThreads) enum_kernel(EnumArgs a) {
    __shared__ GroupSmem g;
    __shared__ int8_t chi_one[kMaxGroup];
    load_group_smem(g, a.group);
    for (int i = threadIdx.x; i < g.ng; i += blockDim.x) chi_one[i] = a.chi_one[i];
    __syncthreads();
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < a.nchunks;
         c += (int64_t)gridDim.x * blockDim.x) {
        int64_t r0 = c * kChunk;
        int64_t r1 = r0 + kChunk;
        if (r1 > a.total) r1 = a.total;
        U s = (a.nup >= 0) ? unrank_fixed<U>(r0, a.L, a.nup, a.binom, a.bstride) : (U)r0;
        int64_t cnt = 0;
        int64_t out = kWrite ? a.offsets[c] : 0;
        for (int64_t r = r0; r < r1; ++r) {
            int st = is_rep<U>(g, chi_one, s);
            if (st) {
                if (kWrite) {
                    ((U*)a.reps)[out] = s;
                    a.stab[out] = (uint16_t)st;
                    ++out;
                } else {
                    ++cnt;
                }
            }
            if (r + 1 < r1) s = (a.nup >= 0) ? gosper_next<U>(s) : (U)(r + 1);
        }
        if (!kWrite) a.counts[c] = cnt;
    }
}

// ---- device-wide exclusive scan of int64 counts (three-phase, recursive)
constexpr int kScanThreads = 1024;

__global__ void scan_block_kernel(const int64_t* in, int64_t* out, int64_t* block_sums, int64_t n) {
    __shared__ int64_t s[kScanThreads];
    int64_t i = blockIdx.x * (int64_t)kScanThreads + threadIdx.x;
    int64_t v = (i < n) ? in[i] : 0;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < kScanThreads; off <<= 1) {
        int64_t t = (threadIdx.x >= off) ? s[threadIdx.x - off] : 0;
        __syncthreads();
        s[threadIdx.x] += t;
        __syncthreads();
    }
    if (i < n) out[i] = s[threadIdx.x] - v;
    if (threadIdx.x == kScanThreads - 1 && block_sums) block_sums[blockIdx.x] = s[threadIdx.x];
}

__global__ void scan_add_kernel(int64_t* out, const int64_t* block_offsets, int64_t n) {
    int64_t i = blockIdx.x * (int64_t)kScanThreads + threadIdx.x;
    if (i < n) out[i] += block_offsets[blockIdx.x];
}

void exclusive_scan(const int64_t* in, int64_t* out, int64_t n, cudaStream_t s) {
    int64_t nb = (n + kScanThreads - 1) / kScanThreads;
    if (nb <= 1) {
        scan_block_kernel<<<1, kScanThreads, 0, s>>>(in, out, nullptr, n);
        QS_CUDA(cudaGetLastError());
        return;
    }
    DevBuf sums(nb * sizeof(int64_t)), sums_scan(nb * sizeof(int64_t));
    scan_block_kernel<<<(unsigned)nb, kScanThreads, 0, s>>>(in, out, sums.as<int64_t>(), n);
    QS_CUDA(cudaGetLastError());
    exclusive_scan(sums.as<int64_t>(), sums_scan.as<int64_t>(), nb, s);
    scan_add_kernel<<<(unsigned)nb, kScanThreads, 0, s>>>(out, sums_scan.as<int64_t>(), n);
    QS_CUDA(cudaGetLastError());
    QS_CUDA(cudaStreamSynchronize(s));
}

template <typename U>
__global__ void splitter_kernel(const U* reps, U* spl, int64_t nsplit, int64_t stride) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < nsplit) spl[i] = reps[i * stride];
}

// Direct index: column of every representative at its parent-sector rank
// (combinadic rank for a fixed-weight sector, the state itself otherwise).
template <typename U>
__global__ void index_fill_kernel(const U* reps, int64_t n, const uint64_t* binom, int nup, int32_t* index) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        U s = reps[i];
        int64_t rk = nup >= 0 ? combinadic_rank<U>(s, binom, 65) : (int64_t)s;
        index[rk] = (int32_t)i;
    }
}

int grid_for(int64_t work, int threads) {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int64_t blocks = (work + threads - 1) / threads;
    int64_t cap = (int64_t)sms * 8;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    return (int)blocks;
}

template <typename U>
void enumerate_sector(Basis& b, DevBuf& d_chi_one) {
    cudaStream_t s = b.stream;
    int64_t total = b.n_parent;
    int64_t nchunks = (total + kChunk - 1) / kChunk;
    DevBuf counts(nchunks * sizeof(int64_t)), offs(nchunks * sizeof(int64_t));
    EnumArgs a{};
    a.group = b.d_group.as<GroupDesc>();
    a.chi_one = d_chi_one.as<int8_t>();
    a.binom = b.d_binom.as<uint64_t>();
    a.bstride = 65;
    a.L = b.L;
    a.nup = b.nup;
    a.total = total;
    a.nchunks = nchunks;
    a.counts = counts.as<int64_t>();
    int grid = grid_for(nchunks, kEnumThreads);
    enum_kernel<U, false><<<grid, kEnumThreads, 0, s>>>(a);
    QS_CUDA(cudaGetLastError());
    exclusive_scan(counts.as<int64_t>(), offs.as<int64_t>(), nchunks, s);
    int64_t last_off = 0, last_cnt = 0;
    QS_CUDA(cudaMemcpyAsync(&last_off, offs.as<int64_t>() + nchunks - 1, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    QS_CUDA(cudaMemcpyAsync(&last_cnt, counts.as<int64_t>() + nchunks - 1, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    QS_CUDA(cudaStreamSynchronize(s));
    b.n = last_off + last_cnt;
    if (b.n == 0) throw Error(QS_ERR_ARGUMENT, "the requested symmetry sector is empty");
    b.d_reps.alloc(b.n * sizeof(U));
    b.d_stab.alloc(b.n * sizeof(uint16_t));
    a.offsets = offs.as<int64_t>();
    a.reps = b.d_reps.p;
    a.stab = b.d_stab.as<uint16_t>();
    enum_kernel<U, true><<<grid, kEnumThreads, 0, s>>>(a);
    QS_CUDA(cudaGetLastError());
    // splitters for the rank search
    b.nsplit = std::min<int64_t>(b.n, 2048);
    b.split_stride = (b.n + b.nsplit - 1) / b.nsplit;
    b.nsplit = (b.n + b.split_stride - 1) / b.split_stride;
    b.d_split.alloc(b.nsplit * sizeof(U));
    splitter_kernel<U><<<(unsigned)((b.nsplit + 255) / 256), 256, 0, s>>>(b.d_reps.as<U>(), b.d_split.as<U>(),
                                                                          b.nsplit, b.split_stride);
    QS_CUDA(cudaGetLastError());
    // Direct rank -> column table when it fits in a quarter of free memory and
    // every column fits an int32: one HBM load replaces the search.
    size_t free_b = 0, total_b = 0;
    QS_CUDA(cudaMemGetInfo(&free_b, &total_b));
    size_t need = (size_t)b.n_parent * sizeof(int32_t);
    if (b.n < INT32_MAX && need <= free_b / 4) {
        b.d_index.alloc(need);
        QS_CUDA(cudaMemsetAsync(b.d_index.p, 0xFF, need, s));
        index_fill_kernel<U><<<grid_for(b.n, 256), 256, 0, s>>>(b.d_reps.as<U>(), b.n, b.d_binom.as<uint64_t>(),
                                                                 b.nup, b.d_index.as<int32_t>());
        QS_CUDA(cudaGetLastError());
        b.has_index = true;
    }
    QS_CUDA(cudaStreamSynchronize(s));
}

}  // namespace

void scan_i64(const int64_t* in, int64_t* out, int64_t n, cudaStream_t s) { exclusive_scan(in, out, n, s); }

namespace {

// Recognises G = translations by multiples of a x {1, parity} x {1, full flip}
// (every combination present and distinct) and builds the per-element tables
// the zero-run orbit search (qs_orbit.cuh) needs.
void detect_fast_group(Basis& b, const Closure& C, int kmom, int nT) {
    b.fast = FastGroup{};
    b.fast_chi.clear();
    b.fast_to_elem.clear();
    if (!b.symmetric) return;
    const int L = b.L;
    const uint64_t lm = low_mask(L);
    std::map<std::tuple<int, int, uint64_t>, int> where;
    for (size_t i = 0; i < C.elems.size(); ++i) {
        const Elem& e = C.elems[i];
        if (e.mask != 0 && e.mask != lm) return;
        where[std::make_tuple(e.refl, e.shift, e.mask)] = (int)i;
    }
    int a = L;
    for (const Elem& e : C.elems)
        if (!e.refl && !e.mask && e.shift > 0) a = std::min(a, e.shift);
    if (L % a) return;
    const int nt = L / a;
    const int has_refl = where.count(std::make_tuple(1, 0, (uint64_t)0)) ? 1 : 0;
    const int has_flip = where.count(std::make_tuple(0, 0, lm)) ? 1 : 0;
    if ((size_t)nt * (1 + has_refl) * (1 + has_flip) != C.elems.size()) return;
    // map fast codes to generic elements (the group order of fill_desc)
    std::vector<int> gidx(C.elems.size());
    {
        std::vector<int> order(C.elems.size());
        for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
        std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
            if (C.elems[x].refl != C.elems[y].refl) return C.elems[x].refl < C.elems[y].refl;
            return C.elems[x].shift < C.elems[y].shift;
        });
        for (size_t k = 0; k < order.size(); ++k) gidx[order[k]] = (int)k;
    }
    b.fast_chi.assign(4 * nt, cx(0, 0));
    b.fast_to_elem.assign(4 * nt, 0);
    for (int r = 0; r <= has_refl; ++r)
        for (int f = 0; f <= has_flip; ++f)
            for (int j = 0; j < nt; ++j) {
                auto it = where.find(std::make_tuple(r, (a * j) % L, f ? lm : (uint64_t)0));
                if (it == where.end()) return;
                int code = (r * 2 + f) * nt + j;
                b.fast_chi[code] = char_value(C.elems[it->second], kmom, nT);
                b.fast_to_elem[code] = gidx[it->second];
            }
    b.fast.enabled = 1;
    b.fast.L = L;
    b.fast.a = a;
    b.fast.nT = nt;
    b.fast.has_refl = has_refl;
    b.fast.has_flip = has_flip;
    b.fast.lmask = lm;
    uint64_t allowed = 0;
    for (int p = 0; p < L; ++p)
        if (((L - 1 - p) % a) == 0) allowed |= 1ull << p;
    b.fast.allowed = allowed;
}

}  // namespace

// ----------------------------------------------------------- basis_build
void basis_build(Basis& b) {
    const qs_basis_spec& sp = b.spec;
    if (sp.L < 1 || sp.L > 63) throw Error(QS_ERR_ARGUMENT, "L must be between 1 and 63");
    if (sp.nup >= 0 && sp.nup > sp.L) throw Error(QS_ERR_ARGUMENT, "nup must lie between 0 and L");
    if (sp.nup < -1) throw Error(QS_ERR_ARGUMENT, "nup must lie between 0 and L");
    b.L = sp.L;
    b.nup = sp.nup;
    b.wide = b.L > 32;
    int L = b.L;
    const int vals[5] = {sp.pblock, sp.zblock, sp.pzblock, sp.zAblock, sp.zBblock};
    const char* names[5] = {"pblock", "zblock", "pzblock", "zAblock", "zBblock"};
    bool requested = sp.has_kblock != 0;
    for (int i = 0; i < 5; ++i) requested = requested || vals[i] != 0;
    b.symmetric = requested;
    if (b.nup < 0 && L > 40) throw Error(QS_ERR_UNSUPPORTED, "a full 2^L space above L=40 does not fit in device memory");
    b.n_parent = b.nup >= 0 ? binom_host(L, b.nup) : (int64_t)1 << L;

    std::vector<Elem> gens;
    int kmom = 0, nT = 0;
    uint64_t full = low_mask(L), odd = 0, even = 0;
    for (int st = 1; st <= L; st += 2) odd |= 1ull << (st - 1);
    for (int st = 2; st <= L; st += 2) even |= 1ull << (st - 1);
    if (requested) {
        if (sp.a <= 0 || L % sp.a != 0) throw Error(QS_ERR_ARGUMENT, "a must be a positive divisor of L");
        nT = L / sp.a;
        if (sp.has_kblock) {
            kmom = ((sp.kblock % nT) + nT) % nT;
            Elem t{0, sp.a % L, 0, 1, 1, {}};
            elem_fill(t, L);
            gens.push_back(t);
            Generator G;
            G.kind = GEN_T; G.shift = sp.a % L; G.refl = 0; G.mask = 0; G.order = nT;
            double arg = 2 * M_PI * (double)kmom / (double)nT;
            G.eig = cx(std::cos(arg), std::sin(arg));
            b.gens.push_back(G);
            if (sp.pblock != 0 && !(kmom == 0 || (nT % 2 == 0 && kmom == nT / 2)))
                throw Error(QS_ERR_ARGUMENT, "pblock can be combined with kblock only at k=0 or pi");
        }
        const int kinds[5] = {GEN_P, GEN_Z, GEN_PZ, GEN_ZA, GEN_ZB};
        for (int i = 0; i < 5; ++i) {
            if (!vals[i]) continue;
            if (vals[i] != 1 && vals[i] != -1) throw Error(QS_ERR_ARGUMENT, std::string(names[i]) + " must be +1 or -1");
            Elem e{0, 0, 0, 0, vals[i], {}};
            if (kinds[i] == GEN_P || kinds[i] == GEN_PZ) e.refl = 1;
            if (kinds[i] == GEN_Z || kinds[i] == GEN_PZ) e.mask = full;
            if (kinds[i] == GEN_ZA) e.mask = odd;
            if (kinds[i] == GEN_ZB) e.mask = even;
            if (b.nup >= 0 && e.mask != 0) {
                int c = __builtin_popcountll(e.mask);
                if (!(c == L && 2 * b.nup == L))
                    throw Error(QS_ERR_ARGUMENT, "symmetry transformation leaves the selected particle sector");
            }
            elem_fill(e, L);
            gens.push_back(e);
            Generator G;
            G.kind = kinds[i]; G.shift = 0; G.refl = e.refl; G.mask = e.mask; G.order = 2;
            G.eig = cx((double)vals[i], 0.0);
            b.gens.push_back(G);
        }
    }
    Closure C;
    if (!close_group(gens, L, kmom, nT, C)) throw Error(QS_ERR_ARGUMENT, "the requested symmetry sector is empty");
    fill_desc(b.group, C, L, kmom, nT);
    b.complex_chars = !b.group.real_chars;

    // The reference intersects one generator at a time and needs every later
    // generator to map each column onto one column (its permutation-like
    // branch, src/symmetry_basis.jl:116-198).  That holds when each generator
    // normalises the group of the earlier ones and keeps their character.
    b.level_groups.clear();
    for (size_t lvl = 0; lvl < gens.size(); ++lvl) {
        std::vector<Elem> sub(gens.begin(), gens.begin() + lvl + 1);
        Closure H;
        if (!close_group(sub, L, kmom, nT, H)) throw Error(QS_ERR_ARGUMENT, "the requested symmetry sector is empty");
        GroupDesc d;
        fill_desc(d, H, L, kmom, nT);
        b.level_groups.push_back(d);
        if (lvl + 1 < gens.size()) {
            const Elem& g = gens[lvl + 1];
            for (const Elem& h : H.elems) {
                Elem c = elem_compose(g, elem_compose(h, g, L, nT), L, nT);
                auto it = H.index.find(c.img);
                bool ok = it != H.index.end();
                if (ok) {
                    cplx a = char_value(h, kmom, nT), bb = char_value(H.elems[it->second], kmom, nT);
                    ok = std::fabs(a.re - bb.re) < 1e-9 && std::fabs(a.im - bb.im) < 1e-9;
                }
                if (!ok) {
                    // the reference's intersection of this generator is not
                    // permutation-like on the eigenvectors of the earlier ones:
                    // build the sector level by level with explicit projectors
                    // (qs_projector.cu)
                    std::vector<ProjMap> maps;
                    std::vector<cplx> eigs;
                    for (size_t q = 0; q < gens.size(); ++q) {
                        const Elem e = gens[q];
                        maps.push_back([e, L](uint64_t st) { return elem_apply(e, st, L); });
                        eigs.push_back(b.gens[q].eig);
                    }
                    basis_build_projector(b, maps, eigs, (int64_t)H.elems.size());
                    return;
                }
            }
        }
    }
    // level-0 coefficient table: orbit of length n under the first generator
    // has coefficients c_j = c_{j-1} * 1 / eig, normalised by norm(c)
    // (src/symmetry_basis.jl:90-104).
    b.level0_table.assign(64 * 64, cx(0, 0));
    if (!b.gens.empty()) {
        const Generator& g0 = b.gens[0];
        for (int n = 1; n <= std::min(g0.order, 63); ++n) {
            if (g0.order % n) continue;
            cplx c[64];
            c[0] = cx(1.0, 0.0);
            for (int j = 1; j < n; ++j) c[j] = cx_div(cx_mul(c[j - 1], cx(1.0, 0.0)), g0.eig);
            double nrm = norm2_short(c, n);
            for (int j = 0; j < n; ++j) b.level0_table[n * 64 + j] = cx_divr(c[j], nrm);
        }
    }

    // everything above is host-side validation; device work starts here
    QS_CUDA(cudaStreamCreateWithFlags(&b.stream, cudaStreamNonBlocking));
    // combinadic table C(bit, p) for bit < 64, p <= 64
    std::vector<uint64_t> binom(64 * 65, 0);
    for (int n = 0; n < 64; ++n)
        for (int k = 0; k <= 64; ++k) binom[n * 65 + k] = (uint64_t)binom_host(n, k);
    b.d_binom.alloc(binom.size() * sizeof(uint64_t));
    QS_CUDA(cudaMemcpy(b.d_binom.p, binom.data(), binom.size() * sizeof(uint64_t), cudaMemcpyHostToDevice));
    b.d_group.alloc(sizeof(GroupDesc));
    QS_CUDA(cudaMemcpy(b.d_group.p, &b.group, sizeof(GroupDesc), cudaMemcpyHostToDevice));
    detect_fast_group(b, C, kmom, nT);
    if (b.fast.enabled) {
        b.d_fast_chi.alloc(b.fast_chi.size() * sizeof(cplx));
        QS_CUDA(cudaMemcpy(b.d_fast_chi.p, b.fast_chi.data(), b.fast_chi.size() * sizeof(cplx), cudaMemcpyHostToDevice));
    }

    if (!b.symmetric) {
        b.n = b.n_parent;
        return;
    }
    std::vector<int8_t> chi_one(kMaxGroup, 0);
    for (int e = 0; e < b.group.ng; ++e)
        chi_one[e] = (std::fabs(b.group.chi_re[e] - 1.0) < 1e-9 && std::fabs(b.group.chi_im[e]) < 1e-9) ? 1 : 0;
    DevBuf d_chi_one(kMaxGroup);
    QS_CUDA(cudaMemcpy(d_chi_one.p, chi_one.data(), kMaxGroup, cudaMemcpyHostToDevice));
    if (b.wide) enumerate_sector<uint64_t>(b, d_chi_one);
    else enumerate_sector<uint32_t>(b, d_chi_one);
}

// ------------------------------------------------- basis_build_general
void basis_build_general(Basis& b, const qs_general_spec& gs) {
    const int L = gs.L;
    if (L < 1 || L > 63) throw Error(QS_ERR_UNSUPPORTED, "general symmetry maps are supported for L <= 63");
    if (gs.nup < -1 || gs.nup > L) throw Error(QS_ERR_ARGUMENT, "nup must lie between 0 and L");
    if (gs.nmaps < 0 || (gs.nmaps > 0 && (!gs.maps || !gs.flips || !gs.qnums)))
        throw Error(QS_ERR_ARGUMENT, "general symmetry blocks must be (map, quantum_number)");
    std::memset(&b.spec, 0, sizeof(b.spec));
    b.spec.L = L;
    b.spec.nup = gs.nup;
    b.spec.pauli = gs.pauli;
    b.spec.a = 1;
    b.L = L;
    b.nup = gs.nup;
    b.wide = L > 32;
    b.general = true;
    b.symmetric = gs.nmaps > 0;
    if (b.nup < 0 && L > 40) throw Error(QS_ERR_UNSUPPORTED, "a full 2^L space above L=40 does not fit in device memory");
    b.n_parent = b.nup >= 0 ? binom_host(L, b.nup) : (int64_t)1 << L;
    std::vector<GElem> gens;
    b.gens.clear();
    for (int i = 0; i < gs.nmaps; ++i) {
        GElem g;
        g.perm.resize(L);
        std::vector<char> seen(L, 0);
        uint64_t flips = 0;
        for (int src = 0; src < L; ++src) {
            const int t = gs.maps[(size_t)i * L + src];
            if (t < 0 || t >= L || seen[t]) throw Error(QS_ERR_ARGUMENT, "a general symmetry map must be a site permutation");
            seen[t] = 1;
            g.perm[src] = t;
            if (gs.flips[(size_t)i * L + src]) flips |= 1ull << src;
        }
        for (int src = 0; src < L; ++src)
            if ((flips >> src) & 1ull) g.mask |= 1ull << g.perm[src];
        if (b.nup >= 0 && flips != 0 && !(__builtin_popcountll(flips) == L && 2 * b.nup == L))
            throw Error(QS_ERR_ARGUMENT, "symmetry transformation leaves the selected particle sector");
        // order: lcm of the cycle lengths, a cycle with an odd number of flips counting twice
        // (src/basis.jl:305-323)
        int64_t order = 1;
        std::vector<char> vis(L, 0);
        for (int st = 0; st < L; ++st) {
            if (vis[st]) continue;
            int len = 0, parity = 0, cur = st;
            while (!vis[cur]) {
                vis[cur] = 1;
                ++len;
                parity ^= (int)((flips >> cur) & 1ull);
                cur = g.perm[cur];
            }
            const int64_t c = parity ? 2 * len : len;
            int64_t a = order, bb = c;
            while (bb) {
                const int64_t t = a % bb;
                a = bb;
                bb = t;
            }
            order = order / a * c;
        }
        if (order > 63) throw Error(QS_ERR_UNSUPPORTED, "symmetry map order above 63");
        const int64_t q = ((int64_t)gs.qnums[i] % order + order) % order;
        const double th = 2.0 * M_PI * (double)q / (double)order;
        g.chi = cx(std::cos(th), std::sin(th));
        gelem_fill(g, L);
        gens.push_back(g);
        Generator G;
        G.kind = GEN_GENERAL;
        G.shift = 0;
        G.refl = 0;
        G.mask = g.mask;
        G.eig = g.chi;
        G.order = (int)order;
        G.perm = g.perm;
        b.gens.push_back(G);
    }
    GClosure C;
    if (!close_general(gens, L, C)) throw Error(QS_ERR_ARGUMENT, "the requested symmetry sector is empty");
    // as for the 1D generators, every later map must permute the columns of
    // the earlier ones and keep their character (the reference's
    // permutation-like intersection, src/symmetry_basis.jl:116-198)
    for (size_t lvl = 0; lvl + 1 < gens.size(); ++lvl) {
        std::vector<GElem> sub(gens.begin(), gens.begin() + lvl + 1);
        GClosure H;
        if (!close_general(sub, L, H)) throw Error(QS_ERR_ARGUMENT, "the requested symmetry sector is empty");
        const GElem& g = gens[lvl + 1];
        GElem ginv = gelem_identity(L);
        for (int k = 1; k < b.gens[lvl + 1].order; ++k) ginv = gelem_compose(g, ginv, L);
        for (const GElem& h : H.elems) {
            GElem c = gelem_compose(g, gelem_compose(h, ginv, L), L);
            auto it = H.index.find(c.img);
            bool ok = it != H.index.end();
            if (ok) {
                const cplx a = h.chi, bb = H.elems[it->second].chi;
                ok = std::fabs(a.re - bb.re) < 1e-9 && std::fabs(a.im - bb.im) < 1e-9;
            }
            if (!ok) {
                // not permutation-like: the dense nullspace intersection (qs_projector.cu)
                std::vector<ProjMap> maps;
                std::vector<cplx> eigs;
                for (size_t q = 0; q < gens.size(); ++q) {
                    const GElem e = gens[q];
                    maps.push_back([e, L](uint64_t st) { return gelem_apply(e, st, L); });
                    eigs.push_back(b.gens[q].eig);
                }
                b.group.ng = (int)C.elems.size();   // the group order the sector reports
                basis_build_projector(b, maps, eigs, (int64_t)H.elems.size());
                return;
            }
        }
    }
    std::vector<uint64_t> tables;
    std::vector<std::vector<int>> perms;
    fill_desc_general(b.group, C, L, tables, &perms);
    b.complex_chars = !b.group.real_chars;
    b.gen_perm_index.clear();
    for (const GElem& g : gens) {
        const auto it = std::find(perms.begin(), perms.end(), g.perm);
        b.gen_perm_index.push_back((int)(it - perms.begin()));
    }
    // the reference-exact column replay holds at most 32 first-generator orbits
    // per column: the later generators' cycle lengths multiply to at most that
    int64_t leaves = 1;
    for (size_t l = 1; l < b.gens.size(); ++l) leaves *= b.gens[l].order;
    b.replay = b.symmetric && (int)b.gens.size() <= kMaxGens && leaves <= (1 << (kMaxGens - 1));
    std::vector<std::vector<uint64_t>> level_tables;
    b.level_groups.clear();
    if (b.replay) {
        for (size_t lvl = 0; lvl < gens.size(); ++lvl) {
            std::vector<GElem> sub(gens.begin(), gens.begin() + lvl + 1);
            GClosure H;
            close_general(sub, L, H);
            GroupDesc d;
            std::vector<uint64_t> t;
            fill_desc_general(d, H, L, t);
            b.level_groups.push_back(d);
            level_tables.push_back(std::move(t));
        }
        // level-0 coefficient table of the first map, as for the 1D generators
        b.level0_table.assign(64 * 64, cx(0, 0));
        const Generator& g0 = b.gens[0];
        for (int n = 1; n <= std::min(g0.order, 63); ++n) {
            if (g0.order % n) continue;
            cplx c[64];
            c[0] = cx(1.0, 0.0);
            for (int j = 1; j < n; ++j) c[j] = cx_div(cx_mul(c[j - 1], cx(1.0, 0.0)), g0.eig);
            double nrm = norm2_short(c, n);
            for (int j = 0; j < n; ++j) b.level0_table[n * 64 + j] = cx_divr(c[j], nrm);
        }
    }
    // device work
    QS_CUDA(cudaStreamCreateWithFlags(&b.stream, cudaStreamNonBlocking));
    std::vector<uint64_t> binom(64 * 65, 0);
    for (int n = 0; n < 64; ++n)
        for (int k = 0; k <= 64; ++k) binom[n * 65 + k] = (uint64_t)binom_host(n, k);
    b.d_binom.alloc(binom.size() * sizeof(uint64_t));
    QS_CUDA(cudaMemcpy(b.d_binom.p, binom.data(), binom.size() * sizeof(uint64_t), cudaMemcpyHostToDevice));
    b.d_gtab.alloc(std::max<size_t>(1, tables.size()) * sizeof(uint64_t));
    if (!tables.empty())
        QS_CUDA(cudaMemcpy(b.d_gtab.p, tables.data(), tables.size() * sizeof(uint64_t), cudaMemcpyHostToDevice));
    b.group.gtab = b.d_gtab.as<uint64_t>();
    b.d_level_gtab.clear();
    for (size_t lvl = 0; lvl < level_tables.size(); ++lvl) {
        b.d_level_gtab.emplace_back(level_tables[lvl].size() * sizeof(uint64_t));
        QS_CUDA(cudaMemcpy(b.d_level_gtab.back().p, level_tables[lvl].data(), level_tables[lvl].size() * sizeof(uint64_t),
                           cudaMemcpyHostToDevice));
        b.level_groups[lvl].gtab = b.d_level_gtab.back().as<uint64_t>();
    }
    b.d_group.alloc(sizeof(GroupDesc));
    QS_CUDA(cudaMemcpy(b.d_group.p, &b.group, sizeof(GroupDesc), cudaMemcpyHostToDevice));
    b.fast = FastGroup{};
    if (!b.symmetric) {
        b.n = b.n_parent;
        return;
    }
    std::vector<int8_t> chi_one(kMaxGroup, 0);
    for (int e = 0; e < b.group.ng; ++e)
        chi_one[e] = (std::fabs(b.group.chi_re[e] - 1.0) < 1e-9 && std::fabs(b.group.chi_im[e]) < 1e-9) ? 1 : 0;
    DevBuf d_chi_one(kMaxGroup);
    QS_CUDA(cudaMemcpy(d_chi_one.p, chi_one.data(), kMaxGroup, cudaMemcpyHostToDevice));
    if (b.wide) enumerate_sector<uint64_t>(b, d_chi_one);
    else enumerate_sector<uint32_t>(b, d_chi_one);
}

// ------------------------------------------------------------- index_of
namespace {

struct IndexArgs {
    const GroupDesc* group;
    const void* reps;
    const void* split;
    int64_t n, nsplit, stride;
    const uint64_t* binom;
    const uint64_t* refrep;   // device reference representatives (symmetric only)
    int L, nup, symmetric;
    const uint64_t* q;
    int64_t nq;
    int64_t* out;
};

template <typename U>
__global__ void index_kernel(IndexArgs a) {
    __shared__ GroupSmem g;
    load_group_smem(g, a.group);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.nq; i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t s64 = a.q[i];
        int64_t res = -1;
        if ((s64 & ~low_mask(a.L)) == 0) {
            U s = (U)s64;
            if (!a.symmetric) {
                if (a.nup < 0) res = (int64_t)s64;
                else if (__popcll(s64) == a.nup) res = combinadic_rank<U>(s, a.binom, 65);
            } else {
                if (a.nup < 0 || __popcll(s64) == a.nup) {
                    U m; int bi, st;
                    orbit_min<U>(g, s, m, bi, st);
                    int64_t r = rank_search<U>((const U*)a.reps, a.n, (const U*)a.split, (int)a.nsplit, a.stride, m);
                    if (r >= 0 && a.refrep[r] == s64) res = r;
                }
            }
        }
        a.out[i] = res;
    }
}

}  // namespace

// ---------------------------------------------- reference projector replay
namespace {

struct REnt {
    uint64_t s;
    double re, im;
};

struct ReplayCtx {
    const GroupDesc* levels;   // subgroup H_l for l = 0..m-1
    const cplx* table0;        // level-0 coefficients [n * 64 + j]
    int m;                     // number of generators
    int L;
    int g0_shift, g0_refl;     // first generator's action
    uint64_t g0_mask;
    int g0_order;
    int refl[kMaxGens];
    int shift[kMaxGens];
    uint64_t mask[kMaxGens];
    double eig_re[kMaxGens];
    double eig_im[kMaxGens];   // 0 for every 1D generator after the first
    // general site maps: generator l is permutation gidx[l] of the group's tables
    int general, nbytes;
    const uint64_t* gtab;
    int gidx[kMaxGens];
};

__host__ __device__ inline uint64_t brev_any(uint64_t x, int L) {
#ifdef __CUDA_ARCH__
    return __brevll(x) >> (64 - L);
#else
    return brev_host(x, L);
#endif
}

__host__ __device__ inline uint64_t gen_apply(const ReplayCtx& c, int l, uint64_t s) {
    if (c.general) return gperm_apply(c.gtab, c.gidx[l], c.nbytes, s) ^ c.mask[l];
    uint64_t r = c.refl[l] ? brev_any(s, c.L) : s;
    return rotl_bits<uint64_t>(r, c.shift[l], c.L, low_mask(c.L)) ^ c.mask[l];
}

__host__ __device__ inline uint64_t sub_orbit_min(const GroupDesc& g, uint64_t t) {
    uint64_t base[2] = {t, brev_any(t, g.L)};
    uint64_t best = ~0ull;
    for (int p = 0; p < g.nperm; ++p) {
        uint64_t r = g.general ? gperm_apply(g.gtab, p, g.nbytes, t)
                               : rotl_bits<uint64_t>(base[g.perm_refl[p]], g.perm_shift[p], g.L, g.lmask);
        for (int e = g.perm_begin[p]; e < g.perm_begin[p + 1]; ++e) {
            uint64_t v = r ^ g.mask[e];
            if (v < best) best = v;
        }
    }
    return best;
}

__host__ __device__ inline void sort_ents(REnt* a, int n) {
    for (int i = 1; i < n; ++i) {
        REnt x = a[i];
        int j = i - 1;
        while (j >= 0 && a[j].s > x.s) { a[j + 1] = a[j]; --j; }
        a[j + 1] = x;
    }
}

__host__ __device__ inline int find_ent(const REnt* a, int n, uint64_t s) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (a[mid].s < s) lo = mid + 1;
        else hi = mid;
    }
    return (lo < n && a[lo].s == s) ? lo : -1;
}

// Column of the last level with anchor a, values exactly as the reference's
// projector holds them, sorted by state into buf (tmp: scratch, same size).
// The column is a binary tree of first-generator orbits: level l joins the
// level-(l-1) column of a with that of min_{H_(l-1)}(g_l a) when they differ.
// The tree is laid out top-down, then evaluated bottom-up.
__host__ __device__ int replay_column(const ReplayCtx& c, uint64_t a, REnt* buf, REnt* tmp) {
    constexpr int kLeaves = 1 << (kMaxGens - 1);
    uint64_t anc[kMaxGens][kLeaves];
    int8_t cyc[kMaxGens][kLeaves];   // cycle length of each level-l column's join (1: fixed)
    int cnt[kMaxGens];
    int off[kLeaves + 1], len[kLeaves];
    const int m = c.m;
    anc[m - 1][0] = a;
    cnt[m - 1] = 1;
    for (int l = m - 1; l >= 1; --l) {
        int k = 0;
        for (int i = 0; i < cnt[l]; ++i) {
            // the columns x, min g(x), min g(min g(x)), ... up to the return to x
            const uint64_t x = anc[l][i];
            uint64_t y = x;
            int d = 0;
            do {
                if (k >= kLeaves) return -1;   // the host keeps trees within kLeaves
                anc[l - 1][k++] = y;
                ++d;
                y = sub_orbit_min(c.levels[l - 1], gen_apply(c, l, y));
            } while (y != x && d < 64);
            cyc[l][i] = (int8_t)d;
        }
        cnt[l - 1] = k;
    }
    int pos = 0;
    for (int i = 0; i < cnt[0]; ++i) {
        int n = 0;
        uint64_t u = anc[0][i];
        REnt* seg = buf + pos;
        do {
            seg[n].s = u;
            ++n;
            u = gen_apply(c, 0, u);
        } while (u != anc[0][i] && n < 64);
        for (int j = 0; j < n; ++j) {
            cplx v = c.table0[n * 64 + j];
            seg[j].re = v.re;
            seg[j].im = v.im;
        }
        sort_ents(seg, n);
        off[i] = pos;
        len[i] = n;
        pos += n;
    }
    for (int l = 1; l < m; ++l) {
        int j = 0;
        const cplx e = cx(c.eig_re[l], c.eig_im[l]);
        for (int i = 0; i < cnt[l]; ++i) {
            const int d = cyc[l][i];
            REnt* A = buf + off[j];
            const int n0 = len[j];
            const int o0 = off[j];
            if (d == 1) {
                // fixed column: one-element orbit, coefficient 1, norm 1
                for (int q = 0; q < n0; ++q) {
                    cplx v = cx_mul(cx(A[q].re, A[q].im), cx(1.0, 0.0));
                    A[q].re = v.re;
                    A[q].im = v.im;
                }
                ++j;
                off[i] = o0;
                len[i] = n0;
                continue;
            }
            // coef_0 = 1, coef_k = coef_(k-1) ph_(k-1) / e with ph_k = (P' S P)[C_(k+1), C_k]
            // accumulated over the rows of C_k in ascending order
            // (src/symmetry_basis.jl:116-198, the permutation-like branch)
            cplx coef[64];
            coef[0] = cx(1.0, 0.0);
            for (int k = 0; k + 1 < d; ++k) {
                const REnt* Ck = buf + off[j + k];
                const int nk = len[j + k];
                const REnt* Cn = buf + off[j + k + 1];
                const int nn = len[j + k + 1];
                cplx phi = cx(0, 0);
                for (int q = 0; q < nk; ++q) {
                    int kk = find_ent(Cn, nn, gen_apply(c, l, Ck[q].s));
                    cplx pr = kk >= 0 ? cx(Cn[kk].re, Cn[kk].im) : cx(0, 0);
                    cplx prod = cx_mul(cx_conj(pr), cx(Ck[q].re, Ck[q].im));
                    phi = (q == 0) ? prod : cx_add(phi, prod);
                }
                coef[k + 1] = cx_div(cx_mul(coef[k], phi), e);
            }
            const double nu = norm2_short(coef, d);
            int total = 0;
            for (int k = 0; k < d; ++k) {
                REnt* Ck = buf + off[j + k];
                const cplx r = cx_divr(coef[k], nu);
                for (int q = 0; q < len[j + k]; ++q) {
                    cplx v = cx_mul(cx(Ck[q].re, Ck[q].im), r);
                    Ck[q].re = v.re;
                    Ck[q].im = v.im;
                }
                total += len[j + k];
            }
            // merge the d sorted segments (contiguous from o0) by state
            int head[64];
            for (int k = 0; k < d; ++k) head[k] = 0;
            for (int q = 0; q < total; ++q) {
                int best = -1;
                for (int k = 0; k < d; ++k) {
                    if (head[k] >= len[j + k]) continue;
                    if (best < 0 || buf[off[j + k] + head[k]].s < buf[off[j + best] + head[best]].s) best = k;
                }
                tmp[q] = buf[off[j + best] + head[best]];
                ++head[best];
            }
            for (int q = 0; q < total; ++q) A[q] = tmp[q];
            j += d;
            off[i] = o0;
            len[i] = total;
        }
    }
    return len[0];
}

__host__ __device__ inline int argmax_abs(const REnt* a, int n) {
    int best = 0;
    double bv = cx_abs(cx(a[0].re, a[0].im));
    for (int i = 1; i < n; ++i) {
        double v = cx_abs(cx(a[i].re, a[i].im));
        if (v > bv) { bv = v; best = i; }
    }
    return best;
}


struct RefrepArgs {
    ReplayCtx ctx;
    const void* reps;
    int64_t n;
    int wide;
    uint64_t* out;
    REnt* scratch;   // per-thread 2 * cap entries
    int64_t cap;
    int64_t nthreads;
};

__global__ void refrep_kernel(RefrepArgs a) {
    int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (tid >= a.nthreads) return;
    REnt* buf = a.scratch + tid * 2 * a.cap;
    REnt* tmp = buf + a.cap;
    for (int64_t i = tid; i < a.n; i += a.nthreads) {
        uint64_t s = a.wide ? ((const uint64_t*)a.reps)[i] : ((const uint32_t*)a.reps)[i];
        int cnt = replay_column(a.ctx, s, buf, tmp);
        a.out[i] = buf[argmax_abs(buf, cnt)].s;
    }
}

struct QueryArgs {
    ReplayCtx ctx;
    const GroupDesc* group;
    const void* reps;
    const void* split;
    int64_t n, nsplit, stride;
    int wide, nup, L;
    const uint64_t* q;
    int64_t nq;
    const uint64_t* refrep;
    uint64_t* rep;
    double* norm;
    double* amp;
    int32_t* status;
    REnt* scratch;
    int64_t cap;
    int64_t nthreads;
};

template <typename U>
__global__ void query_kernel(QueryArgs a) {
    __shared__ GroupSmem g;
    load_group_smem(g, a.group);
    int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (tid >= a.nthreads) return;
    REnt* buf = a.scratch + tid * 2 * a.cap;
    REnt* tmp = buf + a.cap;
    for (int64_t i = tid; i < a.nq; i += a.nthreads) {
        uint64_t s64 = a.q[i];
        a.rep[i] = 0; a.norm[i] = 0; a.amp[2 * i] = 0; a.amp[2 * i + 1] = 0;
        if ((s64 & ~low_mask(a.L)) != 0 || (a.nup >= 0 && __popcll(s64) != a.nup)) { a.status[i] = 1; continue; }
        U m; int bi, st;
        orbit_min<U>(g, (U)s64, m, bi, st);
        int64_t col = rank_search<U>((const U*)a.reps, a.n, (const U*)a.split, (int)a.nsplit, a.stride, m);
        if (col < 0) { a.status[i] = 2; continue; }
        int cnt = replay_column(a.ctx, (uint64_t)m, buf, tmp);
        int k = find_ent(buf, cnt, s64);
        cplx v = k >= 0 ? cx(buf[k].re, buf[k].im) : cx(0, 0);
        a.rep[i] = a.refrep[col];
        a.norm[i] = QS_DIV(1.0, cx_abs2(v));
        a.amp[2 * i] = v.re;
        a.amp[2 * i + 1] = v.im;
        a.status[i] = 0;
    }
}

// project_from / project_to over the columns of a basis: one thread per
// column replays the reference's projector column (states ascending) and
// either scatters out[row(s)] += P[s, j] c_j (every parent state lies in one
// column, so the scatter has no conflicts) or gathers c_j = sum_s
// conj(P[s, j]) psi[row(s)] in ascending state order.  Products and sums are
// rounded one by one (no contraction), as Julia's sparse products round them.
struct ProjArgs {
    ReplayCtx ctx;
    const void* reps;      // column keys: orbit minima (or the states themselves)
    int64_t n;
    int symmetric;
    int nup, pcon;
    const uint64_t* binom;
    int mode;              // 0: out += P in; 1: out = P^H in
    const double2* in;
    double2* out;
    int ncols;             // vectors, column c at in + c * in_ld, out + c * out_ld
    int64_t in_ld, out_ld;
    REnt* scratch;
    int64_t cap, nthreads;
};

template <typename U>
__device__ __forceinline__ int64_t proj_row(const ProjArgs& a, uint64_t s) {
    if (a.pcon && a.nup >= 0) return combinadic_rank<U>((U)s, a.binom, 65);
    return (int64_t)s;
}

template <typename U>
__global__ void project_kernel(ProjArgs a) {
    int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (tid >= a.nthreads) return;
    REnt* buf = a.scratch + tid * 2 * a.cap;
    REnt* tmp = buf + a.cap;
    for (int64_t j = tid; j < a.n; j += a.nthreads) {
        const uint64_t key = (uint64_t)((const U*)a.reps)[j];
        int cnt = 1;
        if (a.symmetric) {
            cnt = replay_column(a.ctx, key, buf, tmp);
        } else {
            buf[0].s = key;
            buf[0].re = 1.0;
            buf[0].im = 0.0;
        }
        for (int col = 0; col < a.ncols; ++col) {
            const double2* in = a.in + (size_t)col * a.in_ld;
            double2* out = a.out + (size_t)col * a.out_ld;
            if (a.mode == 0) {
                const double2 c = in[j];
                for (int k = 0; k < cnt; ++k) {
                    const int64_t row = proj_row<U>(a, buf[k].s);
                    const double vr = buf[k].re, vi = buf[k].im;
                    double2 o = out[row];
                    o.x = __dadd_rn(o.x, __dsub_rn(__dmul_rn(vr, c.x), __dmul_rn(vi, c.y)));
                    o.y = __dadd_rn(o.y, __dadd_rn(__dmul_rn(vr, c.y), __dmul_rn(vi, c.x)));
                    out[row] = o;
                }
            } else {
                double ar = 0.0, ai = 0.0;
                for (int k = 0; k < cnt; ++k) {
                    const double2 x = in[proj_row<U>(a, buf[k].s)];
                    const double vr = buf[k].re, vi = -buf[k].im;   // conj(P[s, j])
                    ar = __dadd_rn(ar, __dsub_rn(__dmul_rn(vr, x.x), __dmul_rn(vi, x.y)));
                    ai = __dadd_rn(ai, __dadd_rn(__dmul_rn(vr, x.y), __dmul_rn(vi, x.x)));
                }
                out[j] = make_double2(ar, ai);
            }
        }
    }
}

// The projector of a basis without symmetry is an embedding: row s of the
// 2^L space holds column rank(s) when popcount(s) = nup (rank: the position
// among the ascending fixed-weight states), column s of a full basis, and the
// parent-sector projector (pcon) is the identity.  One thread per row.
struct EmbedArgs {
    int64_t rows;
    int nup, pcon;
    const uint64_t* binom;
    int mode;              // 0: out += P in; 1: out = P^H in
    const double2* in;
    double2* out;
    int ncols;
    int64_t in_ld, out_ld;
};

template <typename U>
__global__ void embed_kernel(EmbedArgs a) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < a.rows;
         r += (int64_t)gridDim.x * blockDim.x) {
        int64_t j = r;
        if (!a.pcon && a.nup >= 0) {
            if (__popcll((unsigned long long)r) != a.nup) continue;
            j = combinadic_rank<U>((U)r, a.binom, 65);
        }
        for (int col = 0; col < a.ncols; ++col) {
            const double2* in = a.in + (size_t)col * a.in_ld;
            double2* out = a.out + (size_t)col * a.out_ld;
            if (a.mode == 0) {
                double2 o = out[r];
                const double2 c = in[j];
                o.x = __dadd_rn(o.x, c.x);
                o.y = __dadd_rn(o.y, c.y);
                out[r] = o;
            } else {
                out[j] = in[r];
            }
        }
    }
}

// Bases of general site maps carry no replay: a column is the orbit state of
// its minimum m, P[s, col] = sqrt(stab / |G|) chi(g) for the element g taking
// s to m (real positive at m), as the reference's cyclic projector and
// permutation-like intersections anchor it.
struct GenArgs {
    const GroupDesc* group;
    const void* reps;
    const void* split;
    int64_t n, nsplit, stride;
    int L, nup, pcon;
    const uint64_t* binom;
    // queries
    const uint64_t* q;
    int64_t nq;
    uint64_t* rep;
    double* norm;
    double* amp;
    int32_t* status;
    // projections: mode 0 out += P in (per row), mode 1 out = P^H in (per column)
    int mode;
    int64_t rows;
    const double2* in;
    double2* out;
    int ncols;
    int64_t in_ld, out_ld;
};

template <typename U>
__device__ __forceinline__ bool gen_column(const GroupSmem& g, const GenArgs& a, U s, int64_t& col, double2& amp) {
    U m;
    int bidx, stab;
    orbit_min<U>(g, s, m, bidx, stab);
    col = rank_search<U>((const U*)a.reps, a.n, (const U*)a.split, (int)a.nsplit, a.stride, m);
    if (col < 0) return false;
    const double w = sqrt((double)stab / (double)g.ng);
    amp = make_double2(w * a.group->chi_re[bidx], w * a.group->chi_im[bidx]);
    return true;
}

template <typename U>
__global__ void gen_query_kernel(GenArgs a) {
    __shared__ GroupSmem g;
    load_group_smem(g, a.group);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.nq; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t s64 = a.q[i];
        a.rep[i] = 0;
        a.norm[i] = 0;
        a.amp[2 * i] = a.amp[2 * i + 1] = 0;
        if ((s64 & ~low_mask(a.L)) != 0 || (a.nup >= 0 && __popcll(s64) != a.nup)) {
            a.status[i] = 1;
            continue;
        }
        U m;
        int bidx, stab;
        orbit_min<U>(g, (U)s64, m, bidx, stab);
        int64_t col;
        double2 v;
        if (!gen_column<U>(g, a, (U)s64, col, v)) {
            a.status[i] = 2;
            continue;
        }
        a.rep[i] = (uint64_t)m;
        a.amp[2 * i] = v.x;
        a.amp[2 * i + 1] = v.y;
        a.norm[i] = 1.0 / (v.x * v.x + v.y * v.y);
        a.status[i] = 0;
    }
}

// mode 0: one thread per row of the projection space
template <typename U>
__global__ void gen_from_kernel(GenArgs a) {
    __shared__ GroupSmem g;
    load_group_smem(g, a.group);
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < a.rows; r += (int64_t)gridDim.x * blockDim.x) {
        U s;
        if (a.pcon) {
            s = a.nup >= 0 ? unrank_fixed<U>(r, a.L, a.nup, a.binom, 65) : (U)r;
        } else {
            if (a.nup >= 0 && __popcll((unsigned long long)r) != a.nup) continue;
            s = (U)r;
        }
        int64_t col;
        double2 v;
        if (!gen_column<U>(g, a, s, col, v)) continue;
        for (int c = 0; c < a.ncols; ++c) {
            const double2 x = a.in[(size_t)c * a.in_ld + col];
            double2* o = a.out + (size_t)c * a.out_ld + r;
            double2 y = *o;
            y.x += v.x * x.x - v.y * x.y;
            y.y += v.x * x.y + v.y * x.x;
            *o = y;
        }
    }
}

// mode 1: one thread per column, summing over every group element (each orbit
// state is reached stab times) and dividing by stab
template <typename U>
__global__ void gen_to_kernel(GenArgs a, const uint16_t* __restrict__ stabs) {
    __shared__ GroupSmem g;
    load_group_smem(g, a.group);
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < a.n; j += (int64_t)gridDim.x * blockDim.x) {
        const U m = ((const U*)a.reps)[j];
        const double st = (double)stabs[j];
        const double w = sqrt(st / (double)g.ng) / st;
        for (int c = 0; c < a.ncols; ++c) {
            double ar = 0, ai = 0;
            for (int p = 0; p < g.nperm; ++p) {
                const U rp = (U)gperm_apply(g.gtab, p, g.nbytes, (uint64_t)m);
                for (int e = g.begin[p]; e < g.begin[p + 1]; ++e) {
                    const U t = rp ^ (U)g.mask[e];
                    int64_t row = (int64_t)t;
                    if (a.pcon && a.nup >= 0) row = combinadic_rank<U>(t, a.binom, 65);
                    const double2 x = a.in[(size_t)c * a.in_ld + row];
                    // conj(P[t, j]) = w chi(e), e taking m to t
                    const double cr = a.group->chi_re[e], ci = a.group->chi_im[e];
                    ar += cr * x.x - ci * x.y;
                    ai += cr * x.y + ci * x.x;
                }
            }
            a.out[(size_t)c * a.out_ld + j] = make_double2(w * ar, w * ai);
        }
    }
}

ReplayCtx make_ctx(const Basis& b, const DevBuf& lv, const DevBuf& t0) {
    ReplayCtx c{};
    c.levels = lv.as<GroupDesc>();
    c.table0 = t0.as<cplx>();
    c.m = (int)b.gens.size();
    c.L = b.L;
    const Generator& g0 = b.gens[0];
    c.g0_shift = g0.shift;
    c.g0_refl = g0.refl;
    c.g0_mask = g0.mask;
    c.g0_order = g0.order;
    for (int l = 0; l < c.m; ++l) {
        c.refl[l] = b.gens[l].refl;
        c.shift[l] = b.gens[l].shift;
        c.mask[l] = b.gens[l].mask;
        c.eig_re[l] = b.gens[l].eig.re;
        c.eig_im[l] = l == 0 ? 0.0 : b.gens[l].eig.im;
    }
    c.general = b.general;
    if (b.general) {
        c.nbytes = b.group.nbytes;
        c.gtab = b.group.gtab;
        for (int l = 0; l < c.m; ++l) c.gidx[l] = b.gen_perm_index[l];
    }
    return c;
}

void upload_replay(Basis& b) {
    if (b.d_level_groups.p) return;
    b.d_level_groups.alloc(b.level_groups.size() * sizeof(GroupDesc));
    QS_CUDA(cudaMemcpy(b.d_level_groups.p, b.level_groups.data(), b.level_groups.size() * sizeof(GroupDesc),
                       cudaMemcpyHostToDevice));
    b.d_level0.alloc(b.level0_table.size() * sizeof(cplx));
    QS_CUDA(cudaMemcpy(b.d_level0.p, b.level0_table.data(), b.level0_table.size() * sizeof(cplx),
                       cudaMemcpyHostToDevice));
}

int64_t replay_threads(int64_t work) {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int64_t t = (int64_t)sms * 512;
    return std::max<int64_t>(1, std::min(t, work));
}

}  // namespace

void basis_compute_refrep(Basis& b) {
    if (b.refrep_ready) return;
    b.h_refrep.resize(b.n);
    if (!b.symmetric) {
        b.refrep_ready = true;  // states are computed directly by qs_basis_states
        return;
    }
    if (b.general && !b.replay) {
        // without the replay a general basis labels each column by its orbit minimum
        if (b.wide) {
            QS_CUDA(cudaMemcpy(b.h_refrep.data(), b.d_reps.p, b.n * sizeof(uint64_t), cudaMemcpyDeviceToHost));
        } else {
            std::vector<uint32_t> tmp(b.n);
            QS_CUDA(cudaMemcpy(tmp.data(), b.d_reps.p, b.n * sizeof(uint32_t), cudaMemcpyDeviceToHost));
            for (int64_t i = 0; i < b.n; ++i) b.h_refrep[i] = tmp[i];
        }
        b.refrep_ready = true;
        return;
    }
    upload_replay(b);
    DevBuf out(b.n * sizeof(uint64_t));
    int64_t nt = replay_threads(b.n);
    int64_t cap = b.group.ng;
    DevBuf scratch((size_t)nt * 2 * cap * sizeof(REnt));
    RefrepArgs a{};
    a.ctx = make_ctx(b, b.d_level_groups, b.d_level0);
    a.reps = b.d_reps.p;
    a.n = b.n;
    a.wide = b.wide;
    a.out = out.as<uint64_t>();
    a.scratch = scratch.as<REnt>();
    a.cap = cap;
    a.nthreads = nt;
    refrep_kernel<<<(unsigned)((nt + 127) / 128), 128, 0, b.stream>>>(a);
    QS_CUDA(cudaGetLastError());
    QS_CUDA(cudaMemcpyAsync(b.h_refrep.data(), out.p, b.n * sizeof(uint64_t), cudaMemcpyDeviceToHost, b.stream));
    QS_CUDA(cudaStreamSynchronize(b.stream));
    b.refrep_ready = true;
}

void basis_index_of(Basis& b, const uint64_t* states, int64_t n, int64_t* out) {
    if (n == 0) return;
    if (b.symmetric) basis_compute_refrep(b);
    DevBuf dq(n * sizeof(uint64_t)), dout(n * sizeof(int64_t)), dref;
    QS_CUDA(cudaMemcpyAsync(dq.p, states, n * sizeof(uint64_t), cudaMemcpyHostToDevice, b.stream));
    IndexArgs a{};
    a.group = b.d_group.as<GroupDesc>();
    a.reps = b.d_reps.p;
    a.split = b.d_split.p;
    a.n = b.n;
    a.nsplit = b.nsplit;
    a.stride = b.split_stride;
    a.binom = b.d_binom.as<uint64_t>();
    a.L = b.L;
    a.nup = b.nup;
    a.symmetric = b.symmetric;
    a.q = dq.as<uint64_t>();
    a.nq = n;
    a.out = dout.as<int64_t>();
    if (b.symmetric) {
        dref.alloc(b.n * sizeof(uint64_t));
        QS_CUDA(cudaMemcpyAsync(dref.p, b.h_refrep.data(), b.n * sizeof(uint64_t), cudaMemcpyHostToDevice, b.stream));
        a.refrep = dref.as<uint64_t>();
    }
    int grid = grid_for(n, 256);
    if (b.wide) index_kernel<uint64_t><<<grid, 256, 0, b.stream>>>(a);
    else index_kernel<uint32_t><<<grid, 256, 0, b.stream>>>(a);
    QS_CUDA(cudaGetLastError());
    QS_CUDA(cudaMemcpyAsync(out, dout.p, n * sizeof(int64_t), cudaMemcpyDeviceToHost, b.stream));
    QS_CUDA(cudaStreamSynchronize(b.stream));
}

void basis_representative(Basis& b, const uint64_t* states, int64_t n, uint64_t* reps, double* norms, double* amps,
                          int32_t* status) {
    if (n == 0) return;
    if (!b.symmetric) {
        for (int64_t i = 0; i < n; ++i) {
            reps[i] = states[i];
            norms[i] = 1.0;
            amps[2 * i] = 1.0;
            amps[2 * i + 1] = 0.0;
            status[i] = 0;
        }
        return;
    }
    if (b.general && !b.replay) {
        DevBuf dq(n * sizeof(uint64_t)), drep(n * sizeof(uint64_t)), dnorm(n * sizeof(double)),
            damp(2 * n * sizeof(double)), dst(n * sizeof(int32_t));
        QS_CUDA(cudaMemcpyAsync(dq.p, states, n * sizeof(uint64_t), cudaMemcpyHostToDevice, b.stream));
        GenArgs a{};
        a.group = b.d_group.as<GroupDesc>();
        a.reps = b.d_reps.p;
        a.split = b.d_split.p;
        a.n = b.n;
        a.nsplit = b.nsplit;
        a.stride = b.split_stride;
        a.L = b.L;
        a.nup = b.nup;
        a.q = dq.as<uint64_t>();
        a.nq = n;
        a.rep = drep.as<uint64_t>();
        a.norm = dnorm.as<double>();
        a.amp = damp.as<double>();
        a.status = dst.as<int32_t>();
        if (b.wide) gen_query_kernel<uint64_t><<<grid_for(n, 128), 128, 0, b.stream>>>(a);
        else gen_query_kernel<uint32_t><<<grid_for(n, 128), 128, 0, b.stream>>>(a);
        QS_CUDA(cudaGetLastError());
        QS_CUDA(cudaMemcpyAsync(reps, drep.p, n * sizeof(uint64_t), cudaMemcpyDeviceToHost, b.stream));
        QS_CUDA(cudaMemcpyAsync(norms, dnorm.p, n * sizeof(double), cudaMemcpyDeviceToHost, b.stream));
        QS_CUDA(cudaMemcpyAsync(amps, damp.p, 2 * n * sizeof(double), cudaMemcpyDeviceToHost, b.stream));
        QS_CUDA(cudaMemcpyAsync(status, dst.p, n * sizeof(int32_t), cudaMemcpyDeviceToHost, b.stream));
        QS_CUDA(cudaStreamSynchronize(b.stream));
        return;
    }
    basis_compute_refrep(b);
    upload_replay(b);
    DevBuf dq(n * sizeof(uint64_t)), dref(b.n * sizeof(uint64_t)), drep(n * sizeof(uint64_t)),
        dnorm(n * sizeof(double)), damp(2 * n * sizeof(double)), dst(n * sizeof(int32_t));
    QS_CUDA(cudaMemcpyAsync(dq.p, states, n * sizeof(uint64_t), cudaMemcpyHostToDevice, b.stream));
    QS_CUDA(cudaMemcpyAsync(dref.p, b.h_refrep.data(), b.n * sizeof(uint64_t), cudaMemcpyHostToDevice, b.stream));
    int64_t nt = replay_threads(n);
    int64_t cap = b.group.ng;
    DevBuf scratch((size_t)nt * 2 * cap * sizeof(REnt));
    QueryArgs a{};
    a.ctx = make_ctx(b, b.d_level_groups, b.d_level0);
    a.group = b.d_group.as<GroupDesc>();
    a.reps = b.d_reps.p;
    a.split = b.d_split.p;
    a.n = b.n;
    a.nsplit = b.nsplit;
    a.stride = b.split_stride;
    a.wide = b.wide;
    a.nup = b.nup;
    a.L = b.L;
    a.q = dq.as<uint64_t>();
    a.nq = n;
    a.refrep = dref.as<uint64_t>();
    a.rep = drep.as<uint64_t>();
    a.norm = dnorm.as<double>();
    a.amp = damp.as<double>();
    a.status = dst.as<int32_t>();
    a.scratch = scratch.as<REnt>();
    a.cap = cap;
    a.nthreads = nt;
    unsigned grid = (unsigned)((nt + 127) / 128);
    if (b.wide) query_kernel<uint64_t><<<grid, 128, 0, b.stream>>>(a);
    else query_kernel<uint32_t><<<grid, 128, 0, b.stream>>>(a);
    QS_CUDA(cudaGetLastError());
    QS_CUDA(cudaMemcpyAsync(reps, drep.p, n * sizeof(uint64_t), cudaMemcpyDeviceToHost, b.stream));
    QS_CUDA(cudaMemcpyAsync(norms, dnorm.p, n * sizeof(double), cudaMemcpyDeviceToHost, b.stream));
    QS_CUDA(cudaMemcpyAsync(amps, damp.p, 2 * n * sizeof(double), cudaMemcpyDeviceToHost, b.stream));
    QS_CUDA(cudaMemcpyAsync(status, dst.p, n * sizeof(int32_t), cudaMemcpyDeviceToHost, b.stream));
    QS_CUDA(cudaStreamSynchronize(b.stream));
}

int64_t basis_projection_rows(const Basis& b, bool pcon) {
    if (pcon) return b.n_parent;
    if (b.L > 40) throw Error(QS_ERR_UNSUPPORTED, "a full 2^L space above L=40 does not fit in device memory");
    return (int64_t)1 << b.L;
}

void basis_project(Basis& b, bool pcon, int mode, const double* in, double* out, bool accumulate, bool device,
                   int ncols) {
    if (b.dense_proj) {
        basis_project_dense(b, pcon, mode, in, out, accumulate, device, ncols);
        return;
    }
    const int64_t rows = basis_projection_rows(b, pcon);
    const int64_t nin1 = mode == 0 ? b.n : rows, nout1 = mode == 0 ? rows : b.n;
    const int64_t nin = nin1 * ncols, nout = nout1 * ncols;
    if (b.symmetric) upload_replay(b);
    cudaStream_t s = b.stream;
    PoolBuf din, dout;
    const double2* pin = reinterpret_cast<const double2*>(in);
    double2* pout = reinterpret_cast<double2*>(out);
    if (!device) {
        din.alloc((size_t)nin * sizeof(double2), s);
        dout.alloc((size_t)nout * sizeof(double2), s);
        QS_CUDA(cudaMemcpyAsync(din.p, in, din.bytes, cudaMemcpyHostToDevice, s));
        if (mode == 0 && accumulate) QS_CUDA(cudaMemcpyAsync(dout.p, out, dout.bytes, cudaMemcpyHostToDevice, s));
        pin = din.as<double2>();
        pout = dout.as<double2>();
    }
    if (mode == 0 && !accumulate) QS_CUDA(cudaMemsetAsync(pout, 0, (size_t)nout * sizeof(double2), s));
    if (!b.symmetric) {
        EmbedArgs e{};
        e.rows = rows;
        e.nup = b.nup;
        e.pcon = pcon;
        e.binom = b.d_binom.as<uint64_t>();
        e.mode = mode;
        e.in = pin;
        e.out = pout;
        e.ncols = ncols;
        e.in_ld = nin1;
        e.out_ld = nout1;
        const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>((rows + 255) / 256, 152 * 16));
        if (b.wide) embed_kernel<uint64_t><<<grid, 256, 0, s>>>(e);
        else embed_kernel<uint32_t><<<grid, 256, 0, s>>>(e);
        QS_CUDA(cudaGetLastError());
        note_launches(1);
        if (!device) QS_CUDA(cudaMemcpyAsync(out, pout, (size_t)nout * sizeof(double2), cudaMemcpyDeviceToHost, s));
        QS_CUDA(cudaStreamSynchronize(s));
        return;
    }
    if (b.general && !b.replay) {
        GenArgs g{};
        g.group = b.d_group.as<GroupDesc>();
        g.reps = b.d_reps.p;
        g.split = b.d_split.p;
        g.n = b.n;
        g.nsplit = b.nsplit;
        g.stride = b.split_stride;
        g.L = b.L;
        g.nup = b.nup;
        g.pcon = pcon;
        g.binom = b.d_binom.as<uint64_t>();
        g.mode = mode;
        g.rows = rows;
        g.in = pin;
        g.out = pout;
        g.ncols = ncols;
        g.in_ld = nin1;
        g.out_ld = nout1;
        const int64_t work = mode == 0 ? rows : b.n;
        const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>((work + 127) / 128, 152 * 32));
        if (b.wide) {
            if (mode == 0) gen_from_kernel<uint64_t><<<grid, 128, 0, s>>>(g);
            else gen_to_kernel<uint64_t><<<grid, 128, 0, s>>>(g, b.d_stab.as<uint16_t>());
        } else {
            if (mode == 0) gen_from_kernel<uint32_t><<<grid, 128, 0, s>>>(g);
            else gen_to_kernel<uint32_t><<<grid, 128, 0, s>>>(g, b.d_stab.as<uint16_t>());
        }
        QS_CUDA(cudaGetLastError());
        note_launches(1);
        if (!device) QS_CUDA(cudaMemcpyAsync(out, pout, (size_t)nout * sizeof(double2), cudaMemcpyDeviceToHost, s));
        QS_CUDA(cudaStreamSynchronize(s));
        return;
    }
    const int64_t nt = replay_threads(b.n);
    const int64_t cap = b.symmetric ? b.group.ng : 1;
    PoolBuf scratch((size_t)nt * 2 * cap * sizeof(REnt), s);
    ProjArgs a{};
    if (b.symmetric) a.ctx = make_ctx(b, b.d_level_groups, b.d_level0);
    a.reps = b.d_reps.p;
    a.n = b.n;
    a.symmetric = b.symmetric;
    a.nup = b.nup;
    a.pcon = pcon;
    a.binom = b.d_binom.as<uint64_t>();
    a.mode = mode;
    a.in = pin;
    a.out = pout;
    a.ncols = ncols;
    a.in_ld = nin1;
    a.out_ld = nout1;
    a.scratch = scratch.as<REnt>();
    a.cap = cap;
    a.nthreads = nt;
    const unsigned grid = (unsigned)((nt + 127) / 128);
    if (b.wide) project_kernel<uint64_t><<<grid, 128, 0, s>>>(a);
    else project_kernel<uint32_t><<<grid, 128, 0, s>>>(a);
    QS_CUDA(cudaGetLastError());
    note_launches(1);
    if (!device) QS_CUDA(cudaMemcpyAsync(out, pout, (size_t)nout * sizeof(double2), cudaMemcpyDeviceToHost, s));
    QS_CUDA(cudaStreamSynchronize(s));
}

}  // namespace qs
