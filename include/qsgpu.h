/*
 * qsgpu.h -- C ABI of the GB300 (sm_103a) engine for QuSpin.jl's matrix-free
 * Hamiltonian action on symmetry-reduced spin-1/2 bases and the Krylov solvers
 * that consume it.
 *
 * Every entry point takes plain pointers and sizes.  Functions return a
 * qs_status (0 = success); on failure qs_last_error() returns a message that
 * the Julia shim raises as the exception named beside each status code.  The
 * library owns device memory behind opaque handles; host arrays passed in are
 * borrowed for the duration of the call, outputs are caller-allocated (Julia
 * mul! semantics).  Calls on distinct handles may run from different threads;
 * calls on one handle must be serialised by the caller.
 *
 * Complex vectors are interleaved (re, im) doubles, the memory layout of
 * Julia's Vector{ComplexF64}.  Indices are 0-based here; the Julia shim adds 1.
 *
 * Reference citations are paths inside QuSpin.jl.
 */
#ifndef QSGPU_H
#define QSGPU_H

#include <stdint.h>

#if defined(__GNUC__)
#define QS_API __attribute__((visibility("default")))
#else
#define QS_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    QS_OK = 0,
    QS_ERR_ARGUMENT = 1,        /* ArgumentError */
    QS_ERR_DIMENSION = 2,       /* DimensionMismatch */
    QS_ERR_CUDA = 3,            /* ErrorException: device failure */
    QS_ERR_NOMEM = 4,           /* OutOfMemoryError */
    QS_ERR_NOT_CONVERGED = 5,   /* ErrorException: Krylov / Lanczos did not converge */
    QS_ERR_UNSUPPORTED = 6,     /* ArgumentError: outside what this engine implements */
    QS_ERR_TIMEOUT = 7,         /* ErrorException: a bounded device wait ran out */
    QS_PENDING = 8              /* a served request is queued or running */
} qs_status;

typedef enum { QS_F64 = 0, QS_C128 = 1, QS_F32 = 2, QS_C64 = 3 } qs_dtype;
typedef enum { QS_MEM_HOST = 0, QS_MEM_DEVICE = 1 } qs_mem;

typedef struct qs_basis qs_basis;
typedef struct qs_op qs_op;

/* ------------------------------------------------------------------ basis */

/* Keyword arguments of SpinBasis1D(L; nup, pauli, a, kblock, pblock, zblock,
 * pzblock, zAblock, zBblock), src/basis.jl:622-637.  nup = -1 means "not
 * given"; a block of 0 means "not given", otherwise +1 / -1. */
typedef struct {
    int32_t L;
    int32_t nup;
    int32_t pauli;
    int32_t a;
    int32_t has_kblock;
    int32_t kblock;
    int32_t pblock;
    int32_t zblock;
    int32_t pzblock;
    int32_t zAblock;
    int32_t zBblock;
} qs_basis_spec;

/* SpinBasisGeneral(L; nup, pauli, block_order, blocks...) for spin 1/2
 * (src/basis.jl:282-337, 455-600): nmaps symmetry blocks (map, quantum
 * number) in intersection order.  maps[i * L + b] is the 0-based target site
 * of source site b under map i, flips[i * L + b] = 1 where that site's spin is
 * flipped (a negative entry of the reference's map); the map's order is the
 * lcm of its cycle lengths (doubled for a cycle with an odd number of flips)
 * and its eigenvalue cis(2 pi mod(q, order) / order). */
typedef struct {
    int32_t L;
    int32_t nup;              /* -1: not given */
    int32_t pauli;
    int32_t nmaps;
    const int32_t *maps;      /* nmaps x L */
    const int32_t *flips;     /* nmaps x L */
    const int32_t *qnums;     /* nmaps */
} qs_general_spec;

/* Columns are the symmetric orbit states in ascending orbit minimum, each
 * anchored (real positive) at its minimum, labelled by the reference's own
 * representative (its projector is replayed; trees beyond 32 first-map
 * orbits are labelled by the orbit minimum); L <= 63. */
QS_API int qs_basis_create_general(const qs_general_spec *spec, qs_basis **out);

/* Replaces SpinBasis1D(L; ...) (src/basis.jl:622-777): enumerates the sector on
 * the device, keeps one representative per symmetric orbit and orders columns
 * as the reference's projector does (ascending orbit minimum).  When a later
 * block's generator does not map the earlier blocks' eigenvectors onto one
 * another (e.g. zAblock after a one-site translation), the sector comes from
 * the reference's dense nullspace intersection (src/symmetry_basis.jl:199-212,
 * at most 512 reduced columns, else QS_ERR_ARGUMENT with its message): columns
 * are then nullspace vectors over the parent sector, operators on it are
 * P^H A P, and the orbit queries below return QS_ERR_UNSUPPORTED.  The same
 * holds for qs_basis_create_general. */
QS_API int qs_basis_create(const qs_basis_spec *spec, qs_basis **out);
QS_API void qs_basis_destroy(qs_basis *basis);

/* length(basis) / basis.Ns (src/basis.jl:779, 786-799). */
QS_API int64_t qs_basis_size(const qs_basis *basis);

/* 1 if the sector needs a complex projector (src/symmetry_basis.jl:622-629,
 * _basis_requires_complex). */
QS_API int qs_basis_requires_complex(const qs_basis *basis);

/* Order of the symmetry group the sector is reduced by (1 without symmetry). */
QS_API int32_t qs_basis_group_order(const qs_basis *basis);

/* states(basis) / basis.states (src/basis.jl:785): the reference's
 * representative of every column, in column order. */
QS_API int qs_basis_states(const qs_basis *basis, uint64_t *out, int64_t n);

/* Ascending orbit minima of the columns (the device's canonical key). */
QS_API int qs_basis_orbit_minima(const qs_basis *basis, uint64_t *out, int64_t n);

/* Order of the stabiliser of every column's orbit minimum (1 without
 * symmetry); the orbit holds group_order / stab states, and the reference's
 * normalization(basis, s) is that count up to rounding. */
QS_API int qs_basis_stabilizers(const qs_basis *basis, uint16_t *out, int64_t n);

/* state_index(basis, s) (src/basis.jl:1016-1022) for n states at once;
 * out[i] = column or -1 when the state is not represented (the shim raises
 * ArgumentError "state ... is not represented by this basis"). */
QS_API int qs_basis_state_index(const qs_basis *basis, const uint64_t *states, int64_t n, int64_t *out);

/* representative / normalization / get_amp (src/discrete_basis.jl:2386-2422)
 * for n parent states.  status[i] = 0 ok, 1 outside the parent sector,
 * 2 zero weight in this sector.  amps is 2n doubles (complex). */
QS_API int qs_basis_representative(const qs_basis *basis, const uint64_t *states, int64_t n,
                            uint64_t *reps, double *norms, double *amps, int32_t *status);

/* Rows of the projection space: 2^L (pcon = 0) or the parent particle sector
 * (pcon = 1, ascending fixed-weight states), as projection_matrix(basis;
 * pcon) (src/basis.jl:862-880); -1 when 2^L does not fit. */
QS_API int64_t qs_basis_projection_rows(const qs_basis *basis, int32_t pcon);

/* project_from(basis, v; pcon) (src/basis.jl:889-908): out = P v with P the
 * reference's projector (full space or parent sector), v Ns complex, out
 * rows complex; accumulate = 1 adds P v to out.  mem: QS_MEM_HOST or
 * QS_MEM_DEVICE for both vectors.  Bit-for-bit the reference's sparse product. */
QS_API int qs_basis_project_from(qs_basis *basis, int32_t pcon, const double *v, double *out, int32_t accumulate,
                                 int32_t mem);

/* project_to(basis, v; pcon) (src/discrete_basis.jl:2455-2475): out = P^H v,
 * v rows complex, out Ns complex. */
QS_API int qs_basis_project_to(qs_basis *basis, int32_t pcon, const double *v, double *out, int32_t mem);

/* --------------------------------------------------------------- operator */

/* One OperatorTerm (src/operators.jl:42-63): op string over {I,z,+,-,x,y},
 * n_couplings couplings, coefficient c (2 doubles, complex) and one-based
 * sites (strlen(op) ints) each. */
typedef struct {
    const char *op;
    int32_t n_couplings;
    const double *coeffs;   /* 2 * n_couplings */
    const int32_t *sites;   /* strlen(op) * n_couplings, one-based */
    int32_t complex_coeffs; /* 1 if the Julia coefficient type is complex */
} qs_term;

enum {
    QS_CHECK_SYMM = 1,
    QS_CHECK_HERM = 2,
    QS_CHECK_PCON = 4,
    QS_DIAG_COMPLEX = 8     /* the user diagonal has a complex eltype */
};

/* QuantumLinearOperator(basis, static_list; diagonal, check_symm, check_herm,
 * check_pcon), src/operators.jl:2492-2552.  diagonal: NULL or 2*Ns doubles
 * (complex, user diagonal).  check_symm is structural (every generator maps
 * the consolidated term set onto itself) instead of the reference's dense
 * parent-space residual, which does not fit in memory at these sizes. */
QS_API int qs_op_create(qs_basis *basis, const qs_term *terms, int32_t nterms, const double *diagonal,
                 int32_t checks, qs_op **out);
QS_API void qs_op_destroy(qs_op *op);

/* eltype(op): QS_F64 or QS_C128 (src/operators.jl:2523-2529). */
QS_API int qs_op_dtype(const qs_op *op);
/* ishermitian(op) (src/operators.jl:3269). */
QS_API int qs_op_hermitian(const qs_op *op);
/* Launch this operator's kernels (matvec and solvers) on the caller's CUDA
 * stream (a cudaStream_t); NULL returns to the library's own stream.  No
 * reference counterpart: it lets a host runtime that owns streams (CUDA.jl,
 * PyTorch) order the engine's work with its own. */
QS_API int qs_op_set_stream(qs_op *op, void *stream);
/* Assemble the operator on the device, as Hamiltonian(basis, terms) assembles
 * H.data (src/operators.jl:461-614): every surviving transition is recorded
 * once as a packed (column, value-code) word, and later products with this
 * operator (qs_op_matvec and the solvers) stream it instead of regenerating
 * the transitions.  QS_ERR_UNSUPPORTED when the operator cannot be assembled
 * (non-commuting, or a site acted on twice); it then stays matrix-free. */
QS_API int qs_op_assemble(qs_op *op);
/* Stored nonzeros of the assembled form (off-diagonal), -1 if not assembled. */
QS_API int64_t qs_op_nnz(const qs_op *op);
/* Amplitude classes the QS_FIXED_POINT product sums in integers (1 to 4), or 0
 * when the operator is not assembled or QS_FIXED_POINT falls back to the FP64
 * product for it.  No counterpart in the reference. */
QS_API int32_t qs_op_fixed_point_classes(const qs_op *op);
/* H.data / tocsc(H) (src/operators.jl:461-576, 1347) from the device's
 * assembled form: the off-diagonal part in CSR (rowptr Ns + 1, cols and
 * complex values qs_op_nnz(op) each; entries of one row may repeat a column,
 * the element is their sum) and the diagonal (Ns complex).  Host buffers. */
QS_API int qs_op_export_csr(qs_op *op, int64_t *rowptr, int64_t *cols, double *values, double *diag);
/* set_diagonal!(op, d) (src/operators.jl:3298-3307); d is 2*Ns doubles. */
QS_API int qs_op_set_diagonal(qs_op *op, const double *diagonal);

enum {
    QS_TRANSPOSE = 1,
    QS_CONJUGATE = 2,
    /* FP64 vectors, products of an assembled operator carried in double-float
     * (pairs of FP32, ~48-bit significand) to stay off GB300's slow FP64 pipe;
     * ignored for single precision and for matrix-free operators. */
    QS_DOUBLE_FLOAT = 4,
    /* FP64 vectors, row sums of an assembled operator carried exactly in 64-bit
     * fixed point (x sqrt(stab) scaled by one power of two per product), FP64
     * only per row: for real operators whose stored values fall in at most four
     * amplitude classes (e.g. Heisenberg / J1-J2 / XXZ / TFIM couplings in real
     * sectors); otherwise the FP64 product.  Each row sum is within
     * 2^(2 ceil(log2(longest row)) - 61) max|x sqrt(stab)| of exact -- the
     * normwise accuracy of FP64 -- but elements far below the largest do not
     * keep FP64's relative accuracy.  Takes precedence over QS_DOUBLE_FLOAT. */
    QS_FIXED_POINT = 8
};

/* mul!(Y, op, X, alpha, beta) (src/operators.jl:3147-3208) for nrhs column-
 * major right-hand sides with leading dimension Ns:
 *   Y = alpha * op(A) * X + beta * Y,  op() from flags (transpose(op),
 *   conj(op), adjoint(op), src/operators.jl:3283-3295).
 * x_dtype / y_dtype: QS_F64 or QS_C128 (y must be complex if A or x is), or
 * QS_F32 / QS_C64 for the single-precision form (x, y both single, FP32
 * accumulation).  alpha, beta: complex (2 doubles).  mem: where X and Y live;
 * with QS_MEM_DEVICE the call only enqueues work on the operator's stream
 * (qs_op_set_stream) and returns, with QS_MEM_HOST it returns when Y is
 * written back. */
QS_API int qs_op_matvec(qs_op *op, int32_t flags, const double *alpha, const void *x, int32_t x_dtype,
                 const double *beta, void *y, int32_t y_dtype, int64_t nrhs, int32_t mem);

/* Allocation-free form of qs_op_matvec for host buffers (x_dtype == y_dtype),
 * with the same flags (QS_TRANSPOSE, QS_CONJUGATE, QS_DOUBLE_FLOAT,
 * QS_FIXED_POINT; other bits give QS_ERR_ARGUMENT).  No counterpart in the
 * reference: it exists for callers that cannot let a library allocate device
 * memory -- hosts whose device memory belongs to their own pool allocator with
 * a hard limit (CUDA.jl, PyTorch), loops that cannot absorb cudaMalloc's
 * synchronisation.  x and y are staged through one static device array of
 * 2 x 8 MiB (Ns times the element size must not exceed 8 MiB, else
 * QS_ERR_ARGUMENT), which every loaded device holds until the process exits.
 * The device that was current when the operator was created must be current
 * (else QS_ERR_ARGUMENT).  The first call on a device resolves the array's
 * address and must come before any stream capture; calls that overlap on the
 * GPU share the array and race, so the caller serialises them. */
QS_API int qs_op_matvec_noalloc(qs_op *op, int32_t flags, const double *alpha, const void *x, int32_t x_dtype,
                                const double *beta, void *y, int32_t y_dtype, int64_t nrhs);

/* ----------------------------------------------------------------- solvers */

typedef struct {
    int32_t k;            /* number of eigenpairs */
    int32_t which;        /* 0 = SA (smallest algebraic), 1 = LA (largest algebraic), 2 = LM (largest
                             magnitude), 3 = SM (smallest magnitude), 4 = BE (half from each end);
                             values come in the reference's order: SA ascending, LA descending,
                             LM by decreasing and SM by increasing magnitude, BE descending */
    double tol;           /* relative Ritz tolerance, 0 = machine epsilon (ARPACK default) */
    int32_t ncv;          /* Lanczos basis size, 0 = max(20, 2k+1) (Arpack.jl default) */
    int32_t maxiter;      /* restarts, 0 = 300 */
    int32_t precision;    /* 0 = FP64, 1 = FP32 matvec and vectors + FP64 polish,
                             2 = double-float (hi+lo float) Krylov vectors and products on the
                             FP32 pipe + FP64 Rayleigh-quotient polish (assembled operators;
                             matrix-free operators run this as 0) */
    int32_t want_vectors;
    const double *v0;     /* NULL or starting vector, dtype of op */
    int32_t mem;          /* QS_MEM_HOST or QS_MEM_DEVICE for v0 and vectors */
} qs_eigsh_opts;

typedef struct {
    int32_t nconv;
    int32_t restarts;
    int64_t matvecs;
    double max_rel_residual;
    double seconds;
} qs_eigsh_info;

/* eigsh(op; k, which=:SA, v0, tol, ncv, maxiter) (src/operators.jl:3367-3408):
 * values (k doubles) in the order of opts->which; vectors Ns x k column-major in the op dtype
 * (host, or device with opts->mem).  A thick-restart Lanczos with full
 * reorthogonalisation replaces the ARPACK implicitly restarted Lanczos;
 * convergence is ARPACK's test ||r_i|| <= tol * max(eps^(2/3), |theta_i|).
 * Assembled operators (qs_op_assemble) run on the batched engine with one
 * operator (as qs_eigsh_batch).  A matrix-free operator of at least 4,096
 * states whose assembled form fits in a quarter of free device memory is
 * assembled for the length of the call and runs there too (the form is dropped on return; environment
 * QS_TRANSIENT_ASSEMBLY=0 keeps the call matrix-free). */
QS_API int qs_eigsh(qs_op *op, const qs_eigsh_opts *opts, double *values, void *vectors, qs_eigsh_info *info);

/* eigsh(op; k, which, v0, tol, ncv, maxiter) for a non-Hermitian operator
 * (src/operators.jl:3367-3408, where ARPACK's nonsymmetric driver returns
 * complex values, 3402-3404): which = SA / LA select by real part (the
 * reference's :SR / :LR), LM / SM by magnitude (BE is rejected), in the
 * reference's output order.  values: 2k doubles (complex); vectors: Ns x k
 * ComplexF64 column-major (host, or device with opts->mem); v0 in the
 * operator's dtype.  Krylov-Schur restarted Arnoldi on the device. */
QS_API int qs_eigs(qs_op *op, const qs_eigsh_opts *opts, double *values, void *vectors, qs_eigsh_info *info);

/* eigsh on nops Hermitian operators at once (e.g. every momentum / parity
 * sector of one model): the Lanczos iterations of all operators run in
 * lockstep on their assembled forms (assembled here if needed): for
 * operators of more than 32,768 states each step is one launch per kernel
 * over all of them, replayed from a captured CUDA graph; smaller operators
 * run their steps up to each restart in one launch with a thread-block
 * cluster per operator.  Operators that converge drop out.  Replaces the per-sector loop of
 * block_diag_hamiltonian / BlockOps (tools.jl:2213-2420) followed by eigsh on
 * each block.  values: nops * k, ascending per operator; vectors: NULL or nops
 * pointers (each NULL or Ns_i x k in the operator's dtype, host); infos: NULL
 * or nops entries.  opts->precision: 0 FP64 Krylov vectors, 1 FP32 vectors
 * and products then an FP64 Rayleigh-quotient polish (a double-float
 * refinement where the polish misses the tolerance), 2 double-float vectors
 * on the FP32 pipe.  opts->v0 is used when nops is 1,
 * else every operator starts from seeded normal entries (the same seed as
 * qs_eigsh); opts->mem applies to v0 and the vectors. */
QS_API int qs_eigsh_batch(qs_op *const *ops, int32_t nops, const qs_eigsh_opts *opts, double *values, void **vectors,
                          qs_eigsh_info *infos);

/* apply(ExpmMultiplyParallel(A, a), v; tol) (tools.jl:1662-1708) and the
 * Krylov exponential action _krylov_expmv_vector (src/operators.jl:1758-1803):
 * out = exp(a * A) v with complex a.  v, out: Ns complex (host).
 * precision: 0 FP64, 1 FP32 Krylov vectors, 2 double-float Krylov vectors
 * (assembled operators; otherwise FP64).  A matrix-free operator is assembled
 * for the length of the call as in qs_eigsh. */
QS_API int qs_expm_multiply(qs_op *op, const double *a, const double *v, double *out, double tol,
                     int32_t krylov_dim, int32_t precision);

/* evolve(H, v0, t0, times; eom=:SE, imag_time, tol, krylov_dim) for a static
 * Hamiltonian (src/operators.jl:2073-2164 via _krylov_expmv_times
 * 1805-1893): out is Ns x nt column-major complex (host); precision as for
 * qs_expm_multiply. */
QS_API int qs_evolve(qs_op *op, const double *v0, double t0, const double *times, int32_t nt, int32_t imag_time,
              double tol, int32_t krylov_dim, int32_t precision, double *out);

/* evolve(H, v0, t0, times) computed from each time to the next (times taken
 * in order of t - t0): every step runs the reference's Krylov recursion
 * (_krylov_expmv_vector) from the previous state with tol / (number of
 * steps), so the result agrees with qs_evolve to tol while late times cost a
 * single pass over [t0, t] instead of one from v0 each.  An addition for
 * long time series (the reference evaluates every time from v0); arguments
 * and output as qs_evolve, assembled operators. */
QS_API int qs_evolve_stepwise(qs_op *op, const double *v0, double t0, const double *times, int32_t nt,
                              int32_t imag_time, double tol, int32_t krylov_dim, int32_t precision, double *out);

/* The Krylov exponential on a matrix: out[:, c, i] = exp(scales[i] A) V[:, c]
 * (src/operators.jl:1895-1949 _krylov_expmv_times / _krylov_expmv on a
 * matrix; apply(ExpmMultiplyParallel, V) and evolve(H, V0, t0, times) with a
 * matrix of start states).  V: Ns x ncol complex column-major; scales:
 * nscales complex; out: Ns x ncol x nscales complex.  Every column's
 * recursion runs on one batched engine; normalise = 1 scales every state to
 * norm 1 (evolve in imaginary time).  mem applies to V and out. */
QS_API int qs_expm_columns(qs_op *op, const double *V, int32_t ncol, const double *scales, int32_t nscales,
                           double tol, int32_t krylov_dim, int32_t precision, int32_t normalise, double *out,
                           int32_t mem);

/* ------------------------------------------------------------ Krylov tools */

/* Lanczos bases held on the device: the recurrences of tools.jl's
 * lanczos_full / lanczos_iter for one Hermitian operator from nstart start
 * vectors, run together on the batched engine (one FP64 slot per start). */
typedef struct qs_lanczos qs_lanczos;

typedef struct {
    int32_t m;                /* Lanczos dimension, 1 <= m < Ns and m <= 256 */
    int32_t full_ortho;       /* 1: re-orthogonalise against every kept vector */
    double eps;               /* a basis stops where beta <= eps; 0 = machine epsilon */
    int32_t complex_vectors;  /* 1: complex start vectors for a real operator */
    int32_t mem;              /* QS_MEM_HOST or QS_MEM_DEVICE for v0 */
} qs_lanczos_opts;

/* lanczos_full(A, v0, m; full_ortho, eps) (tools.jl:2742-2805) and
 * _lanczos_coefficients (2807-2843) for nstart start vectors at once: v0 is
 * Ns x nstart column-major (real for a real operator unless
 * opts->complex_vectors, else interleaved complex).  ArgumentError codes:
 * m outside 1:Ns-1 or above 256, a zero start vector, a non-Hermitian operator. */
QS_API int qs_lanczos_run(qs_op *op, const qs_lanczos_opts *opts, int32_t nstart, const double *v0,
                          qs_lanczos **out);
QS_API void qs_lanczos_destroy(qs_lanczos *lanczos);
/* The recurrence of start s: alphas (m doubles, `used` valid), betas (m - 1
 * doubles, used - 1 valid) and the number of Lanczos vectors kept (m, or
 * fewer where beta fell to eps). */
QS_API int qs_lanczos_coefficients(const qs_lanczos *lanczos, int32_t s, double *alphas, double *betas,
                                   int32_t *used);
/* 1 when the Lanczos vectors are complex. */
QS_API int qs_lanczos_complex(const qs_lanczos *lanczos);
/* The rows Q_T of start s: used x Ns, each Lanczos vector contiguous (real or
 * interleaved complex per qs_lanczos_complex); host or device per mem. */
QS_API int qs_lanczos_rows(qs_lanczos *lanczos, int32_t s, double *out, int32_t mem);
/* lin_comb_Q_T(coeff, Q_T) (tools.jl:2909-2945), also expm_lanczos
 * (2947-2952) and the Ritz vectors of ltlm_static_iteration: out[:, c] =
 * sum_i coeff[i + c * used] q_i for c < ncoef; coeff complex (used x ncoef,
 * column-major, interleaved), out complex Ns x ncoef (host or device per mem). */
QS_API int qs_lanczos_combine(qs_lanczos *lanczos, int32_t s, const double *coeff, int32_t ncoef, double *out,
                              int32_t mem);
/* The overlaps of ftlm_static_iteration (tools.jl:2966-3013): out[s * m + i] =
 * <q_i, O q_0> of every start s (complex, nstart x m, rows past `used` zero),
 * for an observable on a basis of the same size. */
QS_API int qs_lanczos_overlaps(qs_lanczos *lanczos, qs_op *observable, double *out);
/* The projected observable of ltlm_static_iteration (tools.jl:3015-3068):
 * out = R^* O R with R = sum_i q_i Y[i, :] (Y real, used x nv column-major);
 * out complex nv x nv column-major (host). */
QS_API int qs_lanczos_ritz_matrix(qs_lanczos *lanczos, int32_t s, qs_op *observable, const double *Y, int32_t nv,
                                  double *out);

/* ------------------------------------------------------------ block tools */

/* evolve(BlockOps, psi, t0, times) and block_expm(BlockOps, psi; a, start,
 * stop, num) (tools.jl:2445-2719) for static block Hamiltonians: ops[b] acts
 * on block b's basis; c_b = P_b^H psi for every block (blocks whose
 * projection has norm <= 1000 eps are left out, ArgumentError when none is
 * left), exp(s_i H_b) c_b for the nscales complex scales s_i by the
 * reference's _krylov_expmv_times with every block's Krylov recursions on one
 * batched engine, out[:, i] = sum_b P_b state_b(i).  psi: rows complex (2^L,
 * or the common parent sector with pcon); out: rows x nscales column-major
 * complex; mem applies to both.  precision as for qs_evolve. */
QS_API int qs_block_expm(qs_op *const *ops, int32_t nblocks, int32_t pcon, const double *psi, const double *scales,
                         int32_t nscales, double tol, int32_t krylov_dim, int32_t precision, double *out,
                         int32_t mem);

/* ---------------------------------------------------------------- serving */

/* A request loop for ground-state and time-evolution solves of mixed sizes and
 * sectors on one GPU, with no counterpart in the reference (which runs one
 * solve per call, src/operators.jl:1558-1640, 2073-2164).  Requests are
 * admitted in arrival order against a device-memory budget (basis, assembled
 * operator and Krylov state are all counted), operators are cached by sector
 * and terms, and every running solve advances in the same batched launches;
 * requests arriving while others run join them as soon as they are built
 * (continuous batching).  A result does not depend on what else was running. */
typedef struct qs_server qs_server;

typedef struct {
    double hbm_budget_bytes;   /* device bytes the server may hold, 0 = 150e9 */
    int32_t max_slots;         /* solves running at once, 0 = 64 */
    int32_t precision;         /* 0 FP64 Krylov vectors, 2 double-float (FP32 pipe);
                                  1 eigsh in FP32 with an FP64 polish of each result
                                  (double-float refinement where the polish misses
                                  tol), evolve in double-float */
    int32_t disable_op_cache;  /* 1: free each operator with its last request */
    int32_t chunk_steps;       /* Krylov steps between admissions, 0 = 8 */
    int32_t builders;          /* threads building bases and operators, 0 = 4 */
    int32_t policy;            /* admission order: 0 arrival (FIFO); 1 smallest estimated
                                  work first, a request waiting longer than max_wait_s
                                  going first regardless */
    double max_wait_s;         /* policy 1 aging limit, 0 = 10 s */
    int32_t device;            /* set by the library: the device current at creation */
} qs_server_opts;

typedef enum { QS_REQ_EIGSH = 0, QS_REQ_EVOLVE = 1 } qs_request_kind;

typedef struct {
    int32_t kind;              /* qs_request_kind */
    qs_basis_spec basis;       /* the sector */
    const qs_term *terms;      /* the static Hamiltonian; copied at submission */
    int32_t nterms;
    /* eigsh(H; k, which, tol, ncv, maxiter) */
    int32_t k, which, ncv, maxiter;
    double tol;                /* eigsh: 0 = machine epsilon; evolve: 0 = 1e-12 */
    /* evolve(H, v0, 0, [t]; imag_time, krylov_dim) */
    double t;
    int32_t imag_time, krylov_dim;
    const double *v0;          /* NULL: seeded start vector; evolve: Ns complex, eigsh: op dtype */
    int64_t v0_len;            /* doubles in v0 */
    uint64_t seed;             /* 0 = the seed qs_eigsh uses */
    int32_t want_vector;       /* keep the eigenvectors / evolved state for qs_server_vector */
} qs_request;

typedef struct {
    int32_t status;            /* QS_PENDING, QS_OK or the failure's status */
    int32_t nvalues;
    int64_t Ns;
    double values[8];          /* eigsh: the first min(k, 8) eigenvalues */
    double submit_s, admit_s, done_s;  /* seconds since the server started (-1: not yet) */
    int64_t matvecs;
    int32_t restarts;          /* eigsh: thick restarts; evolve: step halvings */
    double error_estimate;     /* eigsh: max relative Ritz residual; evolve: last step's estimate */
    int64_t vector_len;        /* doubles qs_server_vector returns */
    char message[128];         /* failure text */
} qs_result;

typedef struct {
    int64_t submitted, completed, failed, builds, cache_hits, evictions, steps, launches;
    int64_t cached_ops, running, queued;
    double bytes_in_use, peak_bytes;
} qs_server_counters;

QS_API int qs_server_create(const qs_server_opts *opts, qs_server **out);
QS_API void qs_server_destroy(qs_server *server);
/* Copies the request (terms and v0 included) and returns its ticket. */
QS_API int qs_server_submit(qs_server *server, const qs_request *req, int64_t *ticket);
/* Result so far; returns the request's status (QS_PENDING while running). */
QS_API int qs_server_poll(qs_server *server, int64_t ticket, qs_result *out);
/* Waits up to timeout_s seconds (<= 0: no limit) for the request to finish. */
QS_API int qs_server_wait(qs_server *server, int64_t ticket, double timeout_s, qs_result *out);
/* The kept eigenvectors (Ns x k, op dtype) or evolved state (Ns complex). */
QS_API int qs_server_vector(qs_server *server, int64_t ticket, double *out, int64_t len);
/* Forgets a finished request, or cancels one that is still queued or running. */
QS_API int qs_server_release(qs_server *server, int64_t ticket);
QS_API int qs_server_stats(qs_server *server, qs_server_counters *out);

/* ----------------------------------------------------------------- errors */

/* Message of the last failure on the calling thread (empty if none). */
QS_API const char *qs_last_error(void);

/* The GPU's FP64 fused multiply-add throughput in FMA/s, measured by a short
 * chained-FMA kernel (best of three).  No reference counterpart: the roofline
 * for the FP64-bound kernels (GB300's FP64 rate is far below its memory
 * bandwidth per flop). */
QS_API int qs_fp64_fma_rate(double *fma_per_s);

/* Check of the bounded grid barrier that separates the phases of the
 * persistent Lanczos step: `blocks` co-resident blocks pass eight barriers
 * that expect `phantom` more blocks than run.  phantom = 0: QS_OK.  phantom > 0:
 * the barriers cannot complete, every wait gives up after limit_ms (at most
 * 2000) of device time and the call returns QS_ERR_TIMEOUT with the device
 * still usable.  No reference counterpart: the failure path of the device
 * waits, exercised without a fault. */
QS_API int qs_grid_barrier_check(int32_t phantom, double limit_ms, int32_t blocks);

/* Number of kernels this library has launched in the process so far (all
 * handles).  No reference counterpart: instrumentation for benchmarks. */
QS_API int64_t qs_launch_count(void);

/* Number of device allocations (cudaMalloc calls) this library has made in the
 * process so far, pooled blocks included.  No reference counterpart:
 * instrumentation, e.g. to check that a call allocated nothing. */
QS_API int64_t qs_device_alloc_count(void);

/* Library version string. */
QS_API const char *qs_version(void);

#ifdef __cplusplus
}
#endif

#endif /* QSGPU_H */
