// qs_internal.h -- host-side structures of libqsgpu (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>

#include <complex>
#include <cstdint>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/qsgpu.h"
#include "qs_common.h"
#include "qs_orbit.cuh"

namespace qs {

// Exception carrying a qs_status; converted to a status code at the C ABI.
struct Error : std::runtime_error {
    int status;
    Error(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};

#define QS_CUDA(call)                                                                        \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) {                                                             \
            int st_ = (e_ == cudaErrorMemoryAllocation) ? QS_ERR_NOMEM : QS_ERR_CUDA;        \
            throw ::qs::Error(st_, std::string("CUDA error: ") + cudaGetErrorString(e_) +    \
                                       " at " + __FILE__ + ":" + std::to_string(__LINE__));  \
        }                                                                                    \
    } while (0)

// Count of device allocations made by the library (every cudaMalloc of a
// DevBuf or of the pool); qs_device_alloc_count reports it.
void note_device_alloc();

// Owning device buffer.
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    explicit DevBuf(size_t n) { alloc(n); }
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : p(o.p), bytes(o.bytes) { o.p = nullptr; o.bytes = 0; }
    DevBuf& operator=(DevBuf&& o) noexcept {
        if (this != &o) { release(); p = o.p; bytes = o.bytes; o.p = nullptr; o.bytes = 0; }
        return *this;
    }
    ~DevBuf() { release(); }
    void alloc(size_t n) {
        release();
        if (n) {
            note_device_alloc();
            QS_CUDA(cudaMalloc(&p, n));
        }
        bytes = n;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <typename T> T* as() const { return static_cast<T*>(p); }
};

// Cached device allocations for buffers that live for one solve (Krylov
// bases, slot storage): freed blocks are kept for reuse up to a cap (a tenth
// of device memory, at most 32 GB), so a solve does not pay cudaMalloc /
// cudaFree for its large buffers.  A block returned with pool_put carries an
// event recorded on the stream that last used it; pool_get waits for that
// event before handing the block out again.  pool_trim() frees every cached
// block.
void* pool_get(size_t bytes);
void pool_put(void* p, size_t bytes, cudaStream_t last_use);
void pool_trim();
// Device address of page-locked host memory (cudaHostAlloc / cudaHostRegister,
// mapped under unified addressing), or null for any other pointer.
void* mapped_host_address(void* p);

struct PoolBuf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaStream_t s = nullptr;   // the stream the buffer is used on
    PoolBuf() = default;
    PoolBuf(size_t n, cudaStream_t st) { alloc(n, st); }
    PoolBuf(const PoolBuf&) = delete;
    PoolBuf& operator=(const PoolBuf&) = delete;
    PoolBuf(PoolBuf&& o) noexcept : p(o.p), bytes(o.bytes), s(o.s) { o.p = nullptr; o.bytes = 0; }
    PoolBuf& operator=(PoolBuf&& o) noexcept {
        if (this != &o) { release(); p = o.p; bytes = o.bytes; s = o.s; o.p = nullptr; o.bytes = 0; }
        return *this;
    }
    ~PoolBuf() { release(); }
    void alloc(size_t n, cudaStream_t st) {
        release();
        s = st;
        if (n) p = pool_get(n);
        bytes = n;
    }
    void release() {
        if (p) pool_put(p, bytes, s);
        p = nullptr;
        bytes = 0;
    }
    template <typename T> T* as() const { return static_cast<T*>(p); }
};

// Symmetry generator in the reference's order (src/basis.jl:691-735).
// GEN_GENERAL: a site permutation with spin flips (SpinBasisGeneral,
// src/basis.jl:282-337, 455-600): source site b goes to perm[b], and the
// flips become `mask` in target coordinates (t = perm(s) ^ mask).
enum GenKind { GEN_T = 0, GEN_P, GEN_Z, GEN_PZ, GEN_ZA, GEN_ZB, GEN_GENERAL };
struct Generator {
    int kind;
    int shift, refl;
    uint64_t mask;
    cplx eig;       // eigenvalue exactly as the reference computes it
    int order;      // cyclic order of the map (L/a for T, 2 otherwise)
    std::vector<int> perm;   // GEN_GENERAL only
};

struct Basis {
    qs_basis_spec spec{};
    int L = 0;
    int nup = -1;
    bool symmetric = false;
    bool general = false;            // general site maps (GEN_GENERAL generators)
    DevBuf d_gtab;                   // their permutation tables (GroupDesc::gtab)
    std::vector<int> gen_perm_index; // each generator's permutation in those tables
    std::vector<DevBuf> d_level_gtab;// the level groups' tables
    bool replay = true;              // the projector replay covers this basis
    bool wide = false;               // states need 64 bits (L > 32)
    bool complex_chars = false;
    int64_t n = 0;
    int64_t n_parent = 0;
    std::vector<Generator> gens;
    GroupDesc group{};               // host copy
    DevBuf d_group;                  // GroupDesc on device
    DevBuf d_reps;                   // ascending orbit minima (uint32 or uint64)
    DevBuf d_stab;                   // uint16 stabiliser order per representative
    DevBuf d_split;                  // search splitters (same type as reps)
    int64_t nsplit = 0, split_stride = 1;
    DevBuf d_binom;                  // uint64 C(b, p) table for combinadic ranks
    DevBuf d_index;                  // int32 column of each parent-sector rank (-1: none)
    FastGroup fast{};                // translation x parity x flip structure, when present
    std::vector<cplx> fast_chi;      // character per fast element code
    std::vector<int> fast_to_elem;   // generic element index per fast element code
    DevBuf d_fast_chi;               // complex double, 4 * nT
    bool has_index = false;          // direct rank -> column table built
    std::vector<uint64_t> h_refrep;  // reference (argmax) representatives
    bool refrep_ready = false;
    // per-level subgroup element lists and the level-0 coefficient table used
    // to replay the reference's projector arithmetic
    std::vector<GroupDesc> level_groups;
    std::vector<cplx> level0_table;  // [len * 64 + j]
    DevBuf d_level_groups, d_level0;
    // a sector from the dense nullspace intersection (qs_projector.cu): the
    // projector P (parent states x n) explicitly, columns in CSC order, the
    // argmax state of each column and the state -> column lookup
    bool dense_proj = false;
    std::vector<uint64_t> proj_parent;
    std::vector<int64_t> proj_colptr, proj_row;
    std::vector<cplx> proj_val;
    std::vector<uint64_t> proj_reps;
    std::unordered_map<uint64_t, int64_t> proj_index;
    DevBuf d_proj_colptr, d_proj_row, d_proj_val;        // CSC
    DevBuf d_proj_rowptr, d_proj_rowcol, d_proj_rowval;  // CSR over parent rows
    DevBuf d_proj_parent;
    cudaStream_t stream = nullptr;
    ~Basis();
};

// a symmetry map on the states of a basis (state -> image state)
using ProjMap = std::function<uint64_t(uint64_t)>;
// Builds b as the reference does when an intersection is not permutation-like
// (qs_projector.cu); maps and eigenvalues in the reference's intersection
// order; group_order_before_dense bounds the parent sector it accepts.
void basis_build_projector(Basis& b, const std::vector<ProjMap>& maps, const std::vector<cplx>& eigs,
                           int64_t group_order_before_dense);
// basis_project (below) for such a basis
void basis_project_dense(Basis& b, bool pcon, int mode, const double* in, double* out, bool accumulate, bool device,
                         int ncols);

}  // namespace qs
#include "qs_assembled.h"
namespace qs {

struct Op {
    Basis* basis = nullptr;
    bool complex_mat = false;       // eltype ComplexF64
    bool hermitian = true;
    bool commuting = true;          // terms commute with the group (fast pull form)
    bool extracted = true;          // diagonal terms folded into the diagonal
    std::vector<TermProg> progs;    // off-diagonal transition programs
    std::vector<TermProg> diag_progs;
    std::vector<std::complex<double>> user_diag;
    DevBuf d_progs;
    DevBuf d_diag;                  // complex diagonal (user + extracted), 2*n doubles
    DevBuf d_diag32;                // single-precision copy
    DevBuf d_diag_re, d_diag32_re;  // real parts (read by real operators)
    DevBuf d_diag_df;               // diagonal as float pairs: re hi, re lo, im hi, im lo
    DevBuf d_x, d_y;                // staging for host vectors
    DevBuf d_x32, d_y32;
    cudaStream_t stream = nullptr;      // stream in use
    cudaStream_t own_stream = nullptr;  // created by the library
    Assembled asm_;                     // assembled (compiled-transition) form
    bool assembled = false;
    int device = 0;                     // device current when the operator was created
    cudaStream_t copy_stream = nullptr; // read-back of host products (op_matvec_host_overlap)
    cudaEvent_t range_done[4] = {};
    // an operator on a dense-nullspace basis: H = P^H A P (n x n complex,
    // column-major) without and with the user diagonal, from the operator on
    // the parent sector
    bool dense = false;
    std::unique_ptr<Basis> dense_parent_basis;
    std::unique_ptr<Op> dense_parent_op;
    DevBuf dense_base, dense_h;
    int64_t dense_offdiag_nnz = 0;
    ~Op();
};

// qs_basis.cu
void basis_build(Basis& b);
// SpinBasisGeneral(L; nup, pauli, blocks...) with the blocks in intersection order
void basis_build_general(Basis& b, const qs_general_spec& gs);
void basis_index_of(Basis& b, const uint64_t* states, int64_t n, int64_t* out);
void basis_compute_refrep(Basis& b);
void basis_representative(Basis& b, const uint64_t* states, int64_t n, uint64_t* reps, double* norms,
                          double* amps, int32_t* status);
// rows of the projection space: 2^L, or the parent particle sector (pcon)
int64_t basis_projection_rows(const Basis& b, bool pcon);
// mode 0: out (rows) = [out +] P in (Ns); mode 1: out (Ns) = P^H in (rows);
// complex vectors, host or device; ncols contiguous vectors at once (one
// replay of each projector column for all of them)
void basis_project(Basis& b, bool pcon, int mode, const double* in, double* out, bool accumulate, bool device,
                   int ncols = 1);

// qs_op.cpp
Op* op_create(Basis* basis, const qs_term* terms, int nterms, const double* diagonal, int checks);

// qs_matvec.cu
struct MatvecCall {
    int flags = 0;
    cplx alpha{1, 0}, beta{0, 0};
    const void* x = nullptr;
    void* y = nullptr;
    bool x_complex = false, y_complex = false;
    bool single = false;            // FP32 vectors and accumulation
    bool df = false;                // FP64 vectors, double-float products (assembled form)
    bool df_io = false;             // double-float vectors in and out, alpha = 1, beta = 0
    bool fx = false;                // FP64 vectors, exact fixed-point row sums where the operator allows
    bool fx_ready = false;          // the scaled integer copy of x is already made (later row ranges)
    bool no_tune = false;           // never time kernel variants inside this call
    int64_t slice0 = 0, slice1 = -1; // sliced-ELL slices [slice0, slice1) only (-1: to the end)
};
void op_prepare_device(Op& op);
// qs_projector.cu: operators on a dense-nullspace basis
void op_build_dense(Op& op, const qs_term* terms, int nterms, int checks);
void op_dense_apply_diagonal(Op& op);
void op_matvec_dense(Op& op, const MatvecCall& c, cudaStream_t s);
// H.data of such an operator: off-diagonal CSR (host) and the diagonal
void op_export_dense(Op& op, int64_t* rowptr, int64_t* cols, double* values, double* diag);
// qs_noalloc.cu
size_t noalloc_vector_bytes();
void op_matvec_noalloc(Op& op, int flags, cplx alpha, const void* x, int x_dtype, cplx beta, void* y, int y_dtype,
                       int64_t nrhs);
// qs_assembled.cu
void op_assemble(Op& op);
// drops the assembled form (the operator runs matrix-free again)
void op_release_assembly(Op& op);
// The Krylov solvers of a matrix-free operator with at least 4,096 rows run
// on its assembled form for the length of one call when the form fits in a
// quarter of free memory:
// assembly is one pass of the product kernel, and each product after it is an
// order of magnitude cheaper than the matrix-free one.  The form is dropped
// when the call returns (QS_TRANSIENT_ASSEMBLY=0 keeps the solvers matrix-free).
struct TransientAssembly {
    Op& op;
    bool made = false;
    explicit TransientAssembly(Op& o);
    ~TransientAssembly();
    TransientAssembly(const TransientAssembly&) = delete;
    TransientAssembly& operator=(const TransientAssembly&) = delete;
};
void op_spmv_device(Op& op, const MatvecCall& c, cudaStream_t s);
// y = op x for nrhs column-major vectors (n apart) with one pass over the
// sliced-ELL words per 8 columns; false (nothing done) when the operator or
// the call does not allow it (then the caller loops over the columns)
bool op_spmm_device(Op& op, const MatvecCall& c, int64_t nrhs, cudaStream_t s);
// y = op x for one host vector with the assembled sliced-ELL product split in
// row ranges, each range's rows of y copied back while later ranges compute;
// false (nothing done) when the operator or the call does not allow it
bool op_matvec_host_overlap(Op& op, const MatvecCall& c, void* y_host, size_t elem_bytes);
// the assembled matrix on the host: CSR off-diagonal part (rowptr n + 1,
// cols and complex values nnz; a row may repeat a column) and the diagonal
void op_export_csr(Op& op, int64_t* rowptr, int64_t* cols, double* values, double* diag);
// device-wide exclusive scan of int64 (qs_basis.cu)
void scan_i64(const int64_t* in, int64_t* out, int64_t n, cudaStream_t s);
// kernel launch accounting (qs_launch_count)
void note_launches(int64_t n);
int64_t launches();
int64_t device_allocs();
void op_matvec_device(Op& op, const MatvecCall& c, cudaStream_t s);

}  // namespace qs
