// qs_engine.h -- the batched Krylov engine: many Krylov processes ("slots"),
// each on its own assembled operator and its own vectors, advanced together.
//
// One Lanczos/Arnoldi step of every stepping slot is a fixed sequence of ten
// launches (SpMV; dots + reduce; the update with the norm and the second
// pass's dots fused; the conditional second Gram-Schmidt update; scale;
// advance; seven when every slot runs the three-term recurrence), each
// covering all slots through a block -> slot map.  The step
// counters live on the device, so the sequence is captured once in a CUDA
// graph and replayed; the host only meets the device when a slot has filled
// its basis (restart, convergence test, exponential).  The projected matrix of
// every slot is recorded on the device in FP64 (column j of the Hessenberg
// matrix: the summed CGS2 coefficients and the new norm).
//
// Vectors are stored either in FP64 or as double-float pairs (hi + lo float,
// arithmetic on the FP32 pipe); both take 8 bytes per real component.  Each
// slot has its own real/complex vector flag, so a slot's arithmetic does not
// depend on which other slots share the launches.  The SpMV's slices per
// block are per slot, chosen by a timing autotuner and cached per (storage,
// flags, size class); the BLAS row block is fixed, so every reduction, and
// with it every result, repeats from run to run.
#pragma once

#include <cuda_runtime.h>

#include <complex>
#include <cstdint>
#include <deque>
#include <vector>

#include "qs_internal.h"

namespace qs {

using cd = std::complex<double>;

// kSlotStepCluster: stepping in the cluster step (eng_cluster), which the
// graph-replayed step kernels skip
enum SlotState : int32_t { kSlotIdle = 0, kSlotStep = 1, kSlotRotate = 2, kSlotHold = 3, kSlotNormalize = 4,
                           kSlotStepCluster = 5 };

// Device descriptor of one slot.
struct SlotDev {
    // operator: sliced ELL of the assembled form
    const int64_t* sptr;
    const uint16_t* len;
    const uint32_t* words;
    const int32_t* cols;
    const uint16_t* codes;
    const double2* tab64;   // complex value per code
    const float4* tabdf;    // per code: re hi, re lo, im hi, im lo
    const uint16_t* stab;   // stabiliser order per row (null without symmetry)
    const double2* diag64;  // complex diagonal
    const float4* diagdf;
    const float2* tab32;    // FP32 storage: complex value per code and diagonal
    const float2* diag32;
    uint32_t code_mask;
    int32_t packed, code_bits, ncodes, max_stab;
    int32_t cm, cv;         // complex matrix elements / complex vectors
    int64_t n, nslices;
    // Krylov storage
    void* V;                // m + 1 columns of n
    void* tmp;              // m columns of n (rotation)
    double2* h1;            // m first-pass CGS coefficients
    double2* h2;            // m second-pass CGS coefficients
    double2* rec;           // (m + 1) x m projected matrix, column-major
    void* y;                // rotation coefficients, rot_in x p column-major (storage format)
    // [0] squared norm of the new direction, [1] its inverse norm, [2] norm of
    // a normalised column, [3] ||w||^2 before orthogonalisation, [4] 1 when the
    // second Gram-Schmidt pass runs in this step
    double* nrm;
    int32_t m, j, state;
    // orthogonalisation of a step: 0 classical Gram-Schmidt twice (CGS2);
    // 1 CGS with the DGKS correction only when ||w'|| < 0.717 ||w|| (ARPACK's
    // dsaitr test); 2 Lanczos three-term recurrence (Hermitian operators,
    // the reference's Krylov exponential)
    int32_t orth;
    // rotation: V[:, out0 + c] = sum_{i < rot_in} V[:, i] Y[i, c] for c < p, then
    // V[:, cdst] = V[:, carry] when carry >= 0
    int32_t rot_in, p, out0, carry, cdst;
    int32_t yreal;          // rotation coefficients are real
    int32_t rot_tc;         // the rotation runs on the tensor cores (eng_rotate_tc)
    int32_t ncol;           // column normalised by normalize()
    // tiles
    int32_t rpb, spb;       // rows per BLAS block, slices per SpMV block
    int32_t rb_begin, rb_count, sb_begin, sb_count;
};

// Storage of a slot's Krylov vectors (and the arithmetic of the step kernels).
enum class Store : int32_t { F64 = 0, DF = 1, F32 = 2 };

// rpb: rows per BLAS block (4096 measured best or within 3 % on single and
// batched solves; fixed so that reductions repeat); spb: SELL slices per SpMV
// block (timed per operator size class)
struct Tiles {
    int rpb = 4096, spb = 64;
};

// One slot's part of a rotate() call.
struct RotReq {
    int id = 0;
    std::vector<cd> Y;   // nin x p, column-major
    int nin = 0, p = 0, out0 = 0, carry = -1, cdst = 0;
};

class Engine {
   public:
    Engine(Store st, cudaStream_t s);
    ~Engine();
    Engine(const Engine&) = delete;
    Engine& operator=(const Engine&) = delete;

    Store store() const { return st_; }
    cudaStream_t stream() const { return s_; }
    // Adds a slot of basis size m on an assembled operator (assembled here if
    // needed).  cv: complex vectors (required for complex operators); tmp_cols:
    // most rotation outputs (m - 1 when 0).
    int add(Op& op, int m, bool cv, bool tune = true, int tmp_cols = 0, int orth = 1);
    // device bytes add() would allocate for a slot
    static size_t slot_bytes(int64_t n, int m, bool cv, int tmp_cols = 0, Store st = Store::F64);
    void remove(int id);
    int count() const { return (int)slots_.size(); }
    const SlotDev& slot(int id) const { return slots_[id].d; }
    SlotDev& slot_mut(int id) { dirty_ = true; return slots_[id].d; }
    bool alive(int id) const { return id >= 0 && id < (int)slots_.size() && slots_[id].live; }
    Op& op(int id) { return *slots_[id].op; }

    // column 0 <- seeded normal entries / an FP64 vector (host or device; real
    // for real-vector slots, interleaved complex otherwise)
    void seed(int id, uint64_t seed);
    void load(int id, int col, const double* v, bool device);
    // FP64 copy of a column (host or device destination)
    void store(int id, int col, double* out, bool device);
    // column col /= ||column col|| for the listed slots (scale = false: only
    // measure); returns the norms
    std::vector<double> normalize(const std::vector<int>& ids, int col = 0, bool scale = true);
    // one launch for all listed rotations (RotReq)
    void rotate(const std::vector<RotReq>& reqs);
    // Starts stepping slot id from column j (columns 0..j orthonormal).
    void start(int id, int j);
    // Replays the step graph nsteps times (slots at m stop by themselves).
    void run(int nsteps);
    // Steps left before the first stepping slot fills its basis (0: none stepping).
    int steps_to_event() const;
    // Host copy of the projected matrix record ((m + 1) x m, column-major).
    void record(int id, std::vector<cd>& H);
    // The same for several slots with one synchronisation.
    void records(const std::vector<int>& ids, std::vector<std::vector<cd>>& H);
    int64_t launches() const { return launches_; }
    int64_t matvecs(int id) const { return slots_[id].matvecs; }

   private:
    struct Slot {
        Op* op = nullptr;
        SlotDev d{};
        PoolBuf V, tmp, small;
        int tcols = 0;    // columns of tmp
        bool live = false;
        int64_t matvecs = 0;
    };
    void sync_table();
    void build_maps();
    void capture();
    void launch_step();
    // The step as one cooperative launch of nsteps steps (eng_persist):
    // chosen when every phase fits in one wave of resident blocks, forced by
    // QS_PERSISTENT_STEP=1 and disabled by QS_PERSISTENT_STEP=0
    bool persistent_wanted() const;
    void run_persistent(int nsteps);
    // The steps of the listed slots up to their next Hold event as one launch
    // with a thread-block cluster of C CTAs per slot (eng_cluster): chosen per
    // slot by its size, forced by QS_CLUSTER_STEP=1, disabled by =0
    int cluster_size_for(const SlotDev& d) const;   // 0: not in the cluster step
    bool cluster16_ok() const;
    void run_cluster(const std::vector<int>& ids, int nsteps, int C, cudaStream_t st);
    Tiles tune(Op& op, int m, bool cv);
    Store st_;
    cudaStream_t s_;
    std::vector<Slot> slots_;
    DevBuf dslots_, rmap_, smap_, partial_, rsq64_, rsqdf_, rsq32_, ybuf_;
    DevBuf tc_err_;            // timeout flag of the tensor-core rotation
    DevBuf bar_;               // grid barrier of the persistent step
    DevBuf cmap_;              // stepping slot of each cluster (cluster step)
    size_t cap_cmap_ = 0;
    // the cluster step runs on a side stream beside the graph replay of the
    // large slots when an engine holds both (joined by events)
    cudaStream_t side_ = nullptr;
    cudaEvent_t fork_ = nullptr, join_ = nullptr;
    bool tc_rotate_ = true;    // QS_TC_ROTATE=0 keeps every rotation on eng_rotate
    size_t cap_y_ = 0;
    int nrb_ = 0, nsb_ = 0, mmax_ = 1, cap_slots_ = 0;
    // most vectors any slot dots against in a step (1 for three-term slots,
    // m for Gram-Schmidt ones) and whether any slot takes a second pass
    int dmax_ = 1;
    bool cgs_ = false;
    int step_launches_ = 10;
    size_t cap_partial_ = 0, cap_rmap_ = 0, cap_smap_ = 0;
    bool dirty_ = true, maps_dirty_ = true;
    cudaGraph_t graph_ = nullptr;
    cudaGraphExec_t exec_ = nullptr;
    int64_t launches_ = 0;
    friend struct EngineTuner;
};

// Runs `blocks` cooperative blocks through eight grid barriers (the persistent
// step's barrier) that expect `phantom` blocks more than run: with phantom 0
// they complete, otherwise every wait runs out after limit_ms and this throws
// QS_ERR_TIMEOUT.
void grid_barrier_check(int phantom, double limit_ms, int blocks);

// Thick-restart Lanczos (Wu-Simon) on one slot, ARPACK's convergence test:
// the state kept on the host between the slot's Hold events.
struct EigTask {
    int k = 1, which = 0, m = 20, p = 10, maxiter = 300;
    double tol = 0;
    std::vector<double> T, theta;
    double beta = 0, maxrel = 0;
    int nconv = 0, restarts = 0, j0 = 0;
    void init(int k_, int which_, double tol_, int m_, int maxiter_);
    // Called when the slot has filled its basis, with its record H: Ritz
    // values, then either a thick restart (rot keeps p Ritz vectors and the
    // residual direction; returns false, restart the slot at column p) or the
    // final rotation (k Ritz vectors into columns 0..k-1; returns true).
    bool on_hold(const std::vector<cd>& H, int id, RotReq& rot);
};

// Element bytes of a vector in storage st (cv: complex).
inline size_t store_bytes(Store st, bool cv) { return (st == Store::F32 ? 4 : 8) * (cv ? 2 : 1); }

// Krylov projection of a filled record H ((m + 1) x m, column-major):
// the completed size c (the reference's breakdown test, tn <= 100 eps
// max(1, ||H||_F) on the matrix built so far), coef = exp(s H_c) e_1 (for a
// Hermitian recurrence through the eigen-decomposition of the real
// tridiagonal, as the reference does, else Pade), and the terminal norm
// H(c, c - 1).  src/operators.jl:1655-1756.
void krylov_project(const std::vector<cd>& H, int m, bool hermitian, cd scale, int& c, std::vector<cd>& coef,
                    double& terminal);

// The reference's _krylov_expmv_vector (src/operators.jl:1758-1803) on one
// slot: the recursion is a queue of segments (scale, tol, depth) applied in
// order; column 0 holds the current segment's start / beta.  A rejected step
// is replaced by two half steps whose first starts from the same vector: its
// Krylov factorisation would be the same (the engine is deterministic), so
// the kept record and basis are projected again instead of recomputed, and a
// new factorisation is built only from an accepted state.
struct EvoTask {
    struct Seg {
        cd scale;
        double tol;
        int depth;
    };
    int m = 30;
    int64_t n = 0;
    bool hermitian = true;
    std::deque<Seg> segs;
    double beta = 0, err = 0;
    int halvings = 0;
    std::vector<cd> H;   // record of the factorisation of column 0's state
    // split: the full-scale attempt is known to fail (it was the shared
    // factorisation), so start from the two half steps it would produce
    void init(int m_, int64_t n_, bool herm, cd scale, double tol, double beta0, bool split = false);
    bool done() const { return segs.empty(); }
    // The slot filled its basis: keeps the record and projects the front
    // segment (project).
    void on_hold(const std::vector<cd>& Hrec, int id, RotReq& rot);
    // The candidate beta V_c exp(s H_c) e_1 of the front segment goes to
    // column m (rot); the error estimate is kept.
    void project(int id, RotReq& rot);
    // With the candidate's norm: 1 accepted (copy column m to column 0 through
    // `copy`, beta = nr; a new factorisation is due unless done()), 0 rejected
    // and split (call project again: same basis), -1 depth limit reached.
    int after_norm(double nr, int id, RotReq& copy);
};

// evolve / expm_multiply on an assembled operator through the engine:
// _krylov_expmv_times (src/operators.jl:1805-1893): one factorisation from v0
// for all times, and for every time whose error estimate fails the
// recursion from v0, those running concurrently as slots.  out: Ns x nt
// complex (host).
void evolve_engine(Op& op, const double* v0, const std::vector<cd>& scales, double tol, int krylov_dim, int precision,
                   bool normalise, double* out);
// evolve from each time to the next instead of from v0 every time: the times
// in order of their offset from t0, each step the reference's
// _krylov_expmv_vector recursion from the previous state with tol / steps
// (the steps' errors add), imaginary-time states carried at norm 1.  Far fewer
// products than _krylov_expmv_times for many late times; the results agree
// with it to the tolerance, not bit for bit.  v0, out: host (out Ns x nt).
void evolve_stepwise(Op& op, const double* v0, const std::vector<double>& offsets, bool imag_time, double tol,
                     int krylov_dim, int precision, double* out);
// The reference's _krylov_expmv_times (src/operators.jl:1805-1893) on several
// operators at once (the blocks of tools.jl's BlockOps evolution): v0s[b]
// and outs[b] are device complex vectors (outs[b]: n_b x nscales); the blocks'
// factorisations step together, then the failing (block, time) pairs run
// their recursions concurrently.
void evolve_blocks(const std::vector<Op*>& ops, const std::vector<const double*>& v0s, const std::vector<cd>& scales,
                   double tol, int krylov_dim, int precision, const std::vector<double*>& outs);

}  // namespace qs
