// qs_server.cpp -- the request loop: ground-state (eigsh) and time-evolution
// (evolve) solves of mixed sizes and sectors, continuously batched on one GPU.
//
// Requests arrive through qs_server_submit from any thread.  A builder thread
// admits them in arrival order against a device-memory budget (operator,
// basis and Krylov state are all counted), builds the basis and the assembled
// operator on its own streams (or takes it from a cache of operators keyed by
// sector and terms), and hands it to the engine thread.  The engine thread
// owns one batched Krylov engine (qs_engine.h): new requests become slots as
// soon as they are built, whatever the phase of the running ones, and every
// Krylov step of every running solve is one replay of the captured step
// graph.  A slot's arithmetic depends only on its own operator and vectors,
// so a result is the same alone and in the mix.
//
// eigsh follows the thick-restart Lanczos of qs_eigsh (src/operators.jl:
// 1558-1640 / 3367-3408 through ARPACK); evolve follows _krylov_expmv_vector
// (src/operators.jl:1758-1803): a Krylov projection of krylov_dim steps, the
// error estimate |s| h_{m+1,m} beta |e_m^T exp(sH) e_1|, and on failure the
// same two half steps with half the tolerance, up to depth 14.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <random>
#include <string>
#include <thread>
#include <vector>

#include "../../include/qsgpu.h"
#include "qs_blas.cuh"
#include "qs_dense.h"
#include "qs_engine.h"
#include "qs_internal.h"
#include "qs_server.h"

namespace qs {

namespace {

using Clock = std::chrono::steady_clock;

size_t basis_bytes(const Basis& b) {
    return b.d_group.bytes + b.d_reps.bytes + b.d_stab.bytes + b.d_split.bytes + b.d_binom.bytes + b.d_index.bytes +
           b.d_fast_chi.bytes + b.d_level_groups.bytes + b.d_level0.bytes;
}

size_t op_bytes(const Op& o) {
    const Assembled& M = o.asm_;
    return o.d_progs.bytes + o.d_diag.bytes + o.d_diag32.bytes + o.d_diag_re.bytes + o.d_diag32_re.bytes +
           o.d_diag_df.bytes + o.d_x.bytes + o.d_y.bytes + o.d_x32.bytes + o.d_y32.bytes + M.rowptr.bytes +
           M.words.bytes + M.cols.bytes + M.codes.bytes + M.table64.bytes + M.table32.bytes + M.table_df.bytes +
           M.xsplit.bytes + M.rsq_df.bytes + M.sell_words.bytes + M.sell_cols.bytes + M.sell_codes.bytes +
           M.sell_ptr.bytes + M.sell_perm.bytes + M.sell_len.bytes;
}

double binom(int n, int k) {
    if (k < 0 || k > n) return 0;
    double r = 1;
    for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
    return r;
}

}  // namespace

// ------------------------------------------------------------ server state
struct TermCopy {
    std::string op;
    std::vector<double> coeffs;
    std::vector<int32_t> sites;
    int32_t n = 0, cc = 0;
};

struct CachedOp {
    std::string key;
    std::unique_ptr<Basis> basis;
    Op* op = nullptr;
    size_t bytes = 0;
    int users = 0;
    uint64_t last_use = 0;
    ~CachedOp() {
        delete op;
    }
};

struct Request {
    int64_t ticket = 0;
    qs_request r{};
    std::vector<TermCopy> terms;
    std::vector<double> v0;
    std::string key;
    double t_submit = 0, t_admit = -1, t_done = -1;
    std::atomic<int> status{QS_PENDING};
    std::atomic<bool> cancel{false};
    std::string error;
    std::vector<double> values;
    std::vector<double> vec;
    int64_t n = 0, matvecs = 0;
    int restarts = 0;
    double err = 0;
    // runtime
    std::shared_ptr<CachedOp> op;
    double work = 0;   // estimated work (row-products), for the smallest-first policy
    size_t slot_reserved = 0;
    int slot = -1;
    int lane = 0;            // engine holding the slot (1: the FP32 lane)
    bool polished = false;   // an FP32 solve already went through its FP64 polish
    bool cv = false;
    int m = 0;
    EigTask eig;   // eigsh
    EvoTask evo;   // evolve
};

struct Server {
    qs_server_opts opts{};
    cudaStream_t stream = nullptr;
    Clock::time_point t0 = Clock::now();
    std::mutex mu;
    std::condition_variable cv_build, cv_engine, cv_done;
    std::deque<std::shared_ptr<Request>> pending;   // submitted, not yet admitted
    std::deque<std::shared_ptr<Request>> ready;     // built, waiting for a slot
    std::map<int64_t, std::shared_ptr<Request>> all;
    std::map<std::string, std::shared_ptr<CachedOp>> cache;
    std::map<std::string, int> building;             // keys a builder is working on
    int64_t next_ticket = 1;
    size_t used = 0, peak = 0;
    int running = 0;
    bool stop = false;
    uint64_t use_clock = 0;
    qs_server_counters stats{};
    std::vector<std::shared_ptr<CachedOp>> graveyard;   // evicted, freed outside the lock
    std::vector<std::thread> builders;
    std::thread engine;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

std::string make_key(const qs_request& r, const std::vector<TermCopy>& terms) {
    std::string k;
    auto put = [&](const void* p, size_t n) { k.append((const char*)p, n); };
    put(&r.basis, sizeof(r.basis));
    for (const TermCopy& t : terms) {
        k += t.op;
        k += '|';
        put(&t.n, sizeof(t.n));
        put(&t.cc, sizeof(t.cc));
        put(t.coeffs.data(), t.coeffs.size() * sizeof(double));
        put(t.sites.data(), t.sites.size() * sizeof(int32_t));
    }
    return k;
}

// Upper estimate of the device bytes of a request before anything is built.
size_t estimate_bytes(const Request& q, bool cached, int64_t n_known) {
    const qs_basis_spec& sp = q.r.basis;
    const int L = sp.L;
    const double parent = sp.nup >= 0 ? binom(L, sp.nup) : std::ldexp(1.0, L);
    double order = 1;
    if (sp.has_kblock) order *= std::max(1, L / std::max(1, sp.a));
    for (int b : {sp.pblock, sp.zblock, sp.pzblock, sp.zAblock, sp.zBblock})
        if (b) order *= 2;
    double n = n_known > 0 ? (double)n_known : std::ceil(parent / order * 1.2) + 64;
    double offd = 1;
    for (const TermCopy& t : q.terms)
        if (t.op.find_first_of("+-xy") != std::string::npos) offd += t.n;
    double total = 0;
    if (!cached) {
        total += parent * 4 + n * 32;                    // rank index, representatives, stabilisers
        total += n * offd * 4 * 2.4 + n * (16 * 6 + 8);  // CSR + sliced words, diagonals, staging
    }
    const int m = q.r.kind == QS_REQ_EIGSH ? std::max(20, 2 * q.r.k + 1) : (q.r.krylov_dim > 0 ? q.r.krylov_dim : 30);
    total += (double)Engine::slot_bytes((int64_t)n, std::min(m, 64), true, 0);
    return (size_t)total;
}

void finish(Server& S, const std::shared_ptr<Request>& q, int status, const std::string& err) {
    std::lock_guard<std::mutex> g(S.mu);
    q->t_done = S.now();
    q->error = err;
    if (q->op) {
        q->op->users--;
        q->op->last_use = ++S.use_clock;
        if (S.opts.disable_op_cache && q->op->users == 0 && S.cache.count(q->op->key)) {
            // without the cache an operator's bytes go with its last request
            S.cache.erase(q->op->key);
            S.used -= std::min(S.used, q->op->bytes);
            S.graveyard.push_back(q->op);
        }
        q->op.reset();
    }
    S.used -= std::min(S.used, q->slot_reserved);
    q->slot_reserved = 0;
    if (status == QS_OK) S.stats.completed++;
    else S.stats.failed++;
    S.running--;
    q->status.store(status);
    S.cv_build.notify_all();
    S.cv_done.notify_all();
}

// Frees cached operators nobody uses, oldest first, until `need` more bytes fit.
bool make_room(Server& S, size_t need) {
    while (S.used + need > (size_t)S.opts.hbm_budget_bytes) {
        std::shared_ptr<CachedOp> victim;
        for (auto& kv : S.cache)
            if (kv.second->users == 0 && (!victim || kv.second->last_use < victim->last_use)) victim = kv.second;
        if (!victim) return false;
        S.used -= std::min(S.used, victim->bytes);
        S.cache.erase(victim->key);
        S.graveyard.push_back(victim);
        S.stats.evictions++;
    }
    return true;
}

// ------------------------------------------------------------ builder thread
void builder_loop(Server& S) {
    int dev = S.opts.device;
    cudaSetDevice(dev);
    while (true) {
        std::shared_ptr<Request> q;
        std::shared_ptr<CachedOp> hit;
        size_t est = 0;
        {
            // free evicted operators without holding the lock (cudaFree waits for the device)
            std::vector<std::shared_ptr<CachedOp>> dead;
            {
                std::lock_guard<std::mutex> g(S.mu);
                dead.swap(S.graveyard);
            }
            dead.clear();
        }
        {
            std::unique_lock<std::mutex> g(S.mu);
            // admit the oldest pending request (or, with the smallest-first policy,
            // the least work unless the oldest has waited max_wait_s) whose sector
            // no other builder is building, once its estimate fits the budget
            while (true) {
                if (S.stop) return;
                auto pos = S.pending.begin();
                while (pos != S.pending.end() && !(*pos)->cancel && S.building.count((*pos)->key)) ++pos;
                if (S.opts.policy == 1 && pos != S.pending.end() && !(*pos)->cancel &&
                    S.now() - (*pos)->t_submit < S.opts.max_wait_s) {
                    for (auto it = pos; it != S.pending.end(); ++it) {
                        if ((*it)->cancel) {
                            pos = it;
                            break;
                        }
                        if (!S.building.count((*it)->key) && (*it)->work < (*pos)->work) pos = it;
                    }
                }
                if (pos != S.pending.end()) {
                    q = *pos;
                    if (q->cancel) {
                        S.pending.erase(pos);
                        q->t_done = S.now();
                        q->error = "cancelled";
                        q->status.store(QS_ERR_ARGUMENT);
                        S.stats.failed++;
                        S.cv_done.notify_all();
                        q.reset();
                        continue;
                    }
                    auto it = S.cache.find(q->key);
                    hit = it != S.cache.end() ? it->second : nullptr;
                    est = estimate_bytes(*q, (bool)hit, hit ? hit->basis->n : 0);
                    if (hit) hit->users++;   // pin while waiting for room
                    const bool fits = make_room(S, est);
                    if (hit) hit->users--;
                    if (fits && S.running < S.opts.max_slots) {
                        S.pending.erase(pos);
                        if (!hit) S.building[q->key]++;
                        S.used += est;
                        S.peak = std::max(S.peak, S.used);
                        S.running++;
                        if (hit) hit->users++;
                        break;
                    }
                    if (!fits && S.running == 0) {
                        // nothing will free memory (unused operators were evicted):
                        // the request alone exceeds the budget
                        S.pending.erase(pos);
                        q->t_done = S.now();
                        q->error = "request exceeds the device memory budget";
                        q->status.store(QS_ERR_NOMEM);
                        S.stats.failed++;
                        S.cv_done.notify_all();
                        q.reset();
                        continue;
                    }
                }
                S.cv_build.wait_for(g, std::chrono::milliseconds(50));
            }
            q->t_admit = S.now();
        }
        // build outside the lock
        std::string err;
        int status = QS_OK;
        bool built = false;   // a new operator joined the cache (its bytes stay counted)
        try {
            if (hit) {
                q->op = hit;
                std::lock_guard<std::mutex> g(S.mu);
                S.stats.cache_hits++;
            } else {
                auto c = std::make_shared<CachedOp>();
                c->key = q->key;
                c->basis = std::make_unique<Basis>();
                c->basis->spec = q->r.basis;
                basis_build(*c->basis);
                std::vector<qs_term> tv(q->terms.size());
                for (size_t i = 0; i < q->terms.size(); ++i) {
                    const TermCopy& t = q->terms[i];
                    tv[i] = qs_term{t.op.c_str(), t.n, t.coeffs.data(), t.sites.data(), t.cc};
                }
                c->op = op_create(c->basis.get(), tv.data(), (int)tv.size(), nullptr,
                                  QS_CHECK_SYMM | QS_CHECK_HERM | QS_CHECK_PCON);
                op_assemble(*c->op);
                // the engine reads only the sliced layout: drop the row-compressed copy
                Assembled& M = c->op->asm_;
                M.rowptr.release();
                M.words.release();
                M.cols.release();
                M.codes.release();
                M.xsplit.release();
                QS_CUDA(cudaStreamSynchronize(c->op->stream));
                c->bytes = basis_bytes(*c->basis) + op_bytes(*c->op);
                c->users = 1;
                q->op = c;
                std::lock_guard<std::mutex> g(S.mu);
                S.cache[c->key] = c;
                built = true;
                S.stats.builds++;
            }
            if (!q->op->op->hermitian && q->r.kind == QS_REQ_EIGSH)
                throw Error(QS_ERR_UNSUPPORTED, "eigsh on this engine needs a Hermitian operator");
            q->n = q->op->basis->n;
            const bool cv = q->r.kind == QS_REQ_EVOLVE || q->op->op->complex_mat;
            int m;
            if (q->r.kind == QS_REQ_EIGSH) {
                m = q->r.ncv > 0 ? q->r.ncv : std::max(20, 2 * q->r.k + 1);
                m = (int)std::min<int64_t>(std::min(m, 64), q->n);
                if (q->r.k < 1 || q->r.k >= q->n - 1 || m <= q->r.k)
                    throw Error(QS_ERR_ARGUMENT, "served eigsh needs 1 <= k < Ns - 1");
            } else {
                m = q->r.krylov_dim > 0 ? q->r.krylov_dim : 30;
                m = (int)std::min<int64_t>(std::min(m, 64), q->n);
                if (m < 2) throw Error(QS_ERR_ARGUMENT, "served evolve needs Ns >= 2");
            }
            q->cv = cv;
            q->m = m;
            // replace the estimate by what is really held: the slot, and a new
            // operator (which stays counted while it is cached)
            std::lock_guard<std::mutex> g(S.mu);
            const Store st = S.opts.precision == 0 ? Store::F64 : Store::DF;   // FP32 slots are smaller
            const size_t slot = Engine::slot_bytes(q->n, m, cv, q->r.kind == QS_REQ_EIGSH ? 0 : 1, st);
            S.used = S.used - std::min(S.used, est) + slot + (built ? q->op->bytes : 0);
            S.peak = std::max(S.peak, S.used);
            est = 0;
            built = false;
            q->slot_reserved = slot;
        } catch (const Error& e) {
            status = e.status;
            err = e.what();
        } catch (const std::exception& e) {
            status = QS_ERR_CUDA;
            err = e.what();
        }
        if (!hit) {
            std::lock_guard<std::mutex> g(S.mu);
            if (--S.building[q->key] <= 0) S.building.erase(q->key);
            S.cv_build.notify_all();
        }
        if (status != QS_OK) {
            {
                std::lock_guard<std::mutex> g(S.mu);
                S.used = S.used - std::min(S.used, est) + (built && q->op ? q->op->bytes : 0);
                q->slot_reserved = 0;
            }
            if (q->op) {
                finish(S, q, status, err);
            } else {
                std::lock_guard<std::mutex> g(S.mu);
                q->t_done = S.now();
                q->error = err;
                S.running--;
                S.stats.failed++;
                q->status.store(status);
                S.cv_done.notify_all();
                S.cv_build.notify_all();
            }
            continue;
        }
        std::lock_guard<std::mutex> g(S.mu);
        S.ready.push_back(q);
        S.cv_engine.notify_all();
    }
}

// ------------------------------------------------------------ engine thread
// One engine and the requests whose slots it holds.
struct Lane {
    int id;
    Engine E;
    std::vector<std::shared_ptr<Request>> live;
    Lane(int i, Store st, cudaStream_t s) : id(i), E(st, s) {}
};

void engine_loop(Server& S) {
    cudaSetDevice(S.opts.device);
    // lane 0: FP64 or double-float vectors (evolve; eigsh unless the FP32 form
    // is asked for; the FP32 form's refinements).  Lane 1, with precision 1:
    // eigsh in FP32, each result polished in FP64 before it is returned.
    const bool fp32 = S.opts.precision == 1;
    Lane lane0(0, S.opts.precision == 0 ? Store::F64 : Store::DF, S.stream);
    std::unique_ptr<Lane> lane1;
    cudaStream_t s1 = nullptr;
    if (fp32) {
        QS_CUDA(cudaStreamCreateWithFlags(&s1, cudaStreamNonBlocking));
        lane1.reset(new Lane(1, Store::F32, s1));
    }
    auto lane_of = [&](const Request& q) -> Lane& { return q.lane == 1 ? *lane1 : lane0; };
    auto fail = [&](const std::shared_ptr<Request>& q, int st, const std::string& e) {
        if (q->slot >= 0) lane_of(*q).E.remove(q->slot);
        q->slot = -1;
        finish(S, q, st, e);
    };
    // drops finished requests and those handed to the other lane
    auto prune = [](Lane& ln) {
        ln.live.erase(std::remove_if(ln.live.begin(), ln.live.end(),
                                     [&](const std::shared_ptr<Request>& q) { return q->slot < 0 || q->lane != ln.id; }),
                      ln.live.end());
    };
    // Adds the requests to a lane: slots, start vectors (host v0, device v0, or
    // seeded), one normalisation, then stepping.
    auto admit = [&](Lane& ln, std::vector<std::shared_ptr<Request>>& reqs,
                     const std::vector<const double*>& dev_v0) {
        Engine& E = ln.E;
        std::vector<int> norm_ids;
        std::vector<std::shared_ptr<Request>> norm_q;
        for (size_t r = 0; r < reqs.size(); ++r) {
            auto& q = reqs[r];
            try {
                if (q->cancel) throw Error(QS_ERR_ARGUMENT, "cancelled");
                // eigsh: CGS with ARPACK's DGKS test; evolve: the reference's Krylov
                // recurrence (three-term for Hermitian operators, else CGS2)
                const int orth = q->r.kind == QS_REQ_EIGSH ? 1 : (q->op->op->hermitian ? 2 : 0);
                q->lane = ln.id;
                q->slot = E.add(*q->op->op, q->m, q->cv, true, q->r.kind == QS_REQ_EIGSH ? 0 : 1, orth);
                const int comps = q->cv ? 2 : 1;
                if (!dev_v0.empty() && dev_v0[r]) {
                    E.load(q->slot, 0, dev_v0[r], true);
                } else if (!q->v0.empty()) {
                    if ((int64_t)q->v0.size() != q->n * comps) throw Error(QS_ERR_DIMENSION, "v0 must have length Ns");
                    E.load(q->slot, 0, q->v0.data(), false);
                } else {
                    E.seed(q->slot, q->r.seed ? q->r.seed : 20261203ull);
                }
                if (q->r.kind == QS_REQ_EIGSH) {
                    const double tol = q->r.tol > 0 ? q->r.tol : 2.220446049250313e-16;
                    q->eig.init(q->r.k, q->r.which, ln.id == 1 ? std::max(tol, 2e-6) : q->r.tol, q->m,
                                q->r.maxiter);
                }
                norm_ids.push_back(q->slot);
                norm_q.push_back(q);
                ln.live.push_back(q);
            } catch (const Error& e) {
                fail(q, e.status, e.what());
            } catch (const std::exception& e) {
                fail(q, QS_ERR_CUDA, e.what());
            }
        }
        if (norm_ids.empty()) return;
        std::vector<double> nrm = E.normalize(norm_ids);
        for (size_t i = 0; i < norm_q.size(); ++i) {
            Request& q = *norm_q[i];
            if (q.r.kind == QS_REQ_EVOLVE) {
                const cd sc = q.r.imag_time ? cd(-q.r.t, 0) : cd(0, -q.r.t);
                q.evo.init(q.m, q.n, q.op->op->hermitian, sc, q.r.tol > 0 ? q.r.tol : 1e-12, nrm[i]);
            }
            if (q.r.kind == QS_REQ_EIGSH || !q.evo.done()) E.start(q.slot, 0);
        }
        // evolve requests with nothing to do (t = 0 or v0 = 0) finish at once:
        // exp(0) v = v is the start vector
        for (auto& qp : norm_q) {
            Request& q = *qp;
            if (q.r.kind == QS_REQ_EVOLVE && q.evo.done()) {
                if (q.r.want_vector) {
                    q.vec.resize(q.n * 2);
                    E.store(q.slot, 0, q.vec.data(), false);
                    for (double& v : q.vec) v *= q.evo.beta;
                }
                E.remove(q.slot);
                q.slot = -1;
                finish(S, qp, QS_OK, "");
            }
        }
        prune(ln);
    };
    // FP64 polish of a finished FP32 ground-state solve: the Rayleigh quotient
    // of each promoted Ritz vector with the FP64 product.  Returns true when the
    // quadratic bound meets the tolerance (values and vectors set); otherwise
    // `promoted` holds the FP64 vectors for a refinement.
    auto polish = [&](Request& q, PoolBuf& promoted) -> bool {
        Engine& E = lane1->E;
        Op& op = *q.op->op;
        const int k = q.eig.k;
        const int comps = q.cv ? 2 : 1;
        const VKind k64 = q.cv ? VKind::C128 : VKind::F64;
        promoted.alloc((size_t)k * q.n * comps * sizeof(double), s1);
        for (int i = 0; i < k; ++i) E.store(q.slot, i, promoted.as<double>() + (size_t)i * q.n * comps, true);
        Blas B(k64, q.n, s1);
        PoolBuf Ax((size_t)q.n * comps * sizeof(double), s1);
        const double tol = q.r.tol > 0 ? q.r.tol : 2.220446049250313e-16;
        std::vector<double> th(k);
        bool ok = true;
        for (int i = 0; i < k; ++i) {
            double* xq = promoted.as<double>() + (size_t)i * q.n * comps;
            const double nx = B.norm(xq);
            B.scale(xq, xq, cd(1.0 / nx, 0));
            MatvecCall c;
            c.x = xq;
            c.y = Ax.p;
            c.x_complex = c.y_complex = q.cv;
            c.no_tune = true;   // the operator may be stepping on the other lane
            op_matvec_device(op, c, s1);
            th[i] = B.dot(xq, Ax.p).real();
            B.axpy(Ax.p, xq, cd(-th[i], 0));
            const double rn = B.norm(Ax.p);
            double gap = 1e300;
            for (int i2 = 0; i2 < k; ++i2)
                if (i2 != i) gap = std::min(gap, std::fabs(q.eig.theta[i2] - th[i]));
            if (gap == 1e300) gap = std::max(1e-300, std::fabs(th[i]));
            if (rn * rn / gap > tol * std::max(1.0, std::fabs(th[i]))) ok = false;
        }
        QS_CUDA(cudaStreamSynchronize(s1));
        q.matvecs += k;
        if (!ok) return false;
        q.values = th;
        if (q.r.want_vector) {
            q.vec.resize((size_t)q.n * comps * k);
            QS_CUDA(cudaMemcpy(q.vec.data(), promoted.p, q.vec.size() * sizeof(double), cudaMemcpyDeviceToHost));
        }
        return true;
    };
    // One round of a lane: cancellations, a bounded chunk of steps, the events.
    auto round = [&](Lane& ln) {
        Engine& E = ln.E;
        // requests released while running stop here, between steps
        {
            std::vector<std::shared_ptr<Request>> cancelled;
            {
                std::lock_guard<std::mutex> g(S.mu);
                for (auto& q : ln.live)
                    if (q->cancel && q->slot >= 0) cancelled.push_back(q);
            }
            for (auto& q : cancelled) fail(q, QS_ERR_ARGUMENT, "cancelled");
            if (!cancelled.empty()) prune(ln);
        }
        const int steps = E.steps_to_event();
        if (steps == 0) return;
        // a bounded chunk keeps admission latency low for new arrivals
        E.run(std::min(steps, S.opts.chunk_steps > 0 ? S.opts.chunk_steps : steps));
        {
            std::lock_guard<std::mutex> g(S.mu);
            S.stats.steps++;
        }
        // ---- events: slots that filled their basis
        std::vector<RotReq> rot;
        std::vector<std::shared_ptr<Request>> eig_fin, evo_ev, holding;
        std::vector<int> hold_ids;
        for (auto& qp : ln.live)
            if (qp->slot >= 0 && E.slot(qp->slot).state == kSlotHold) {
                holding.push_back(qp);
                hold_ids.push_back(qp->slot);
            }
        std::vector<std::vector<cd>> Hs;
        if (!hold_ids.empty()) E.records(hold_ids, Hs);
        for (size_t hq = 0; hq < holding.size(); ++hq) {
            auto& qp = holding[hq];
            Request& q = *qp;
            try {
                if (q.r.kind == QS_REQ_EIGSH) {
                    RotReq R;
                    if (q.eig.on_hold(Hs[hq], q.slot, R)) eig_fin.push_back(qp);
                    rot.push_back(std::move(R));
                } else {
                    // Krylov projection exp(s H_m) e_1 of the current segment
                    RotReq R;
                    q.evo.on_hold(Hs[hq], q.slot, R);
                    rot.push_back(std::move(R));
                    evo_ev.push_back(qp);
                }
            } catch (const Error& e) {
                fail(qp, e.status, e.what());
            } catch (const std::exception& e) {
                fail(qp, QS_ERR_CUDA, e.what());
            }
        }
        rot.erase(std::remove_if(rot.begin(), rot.end(), [&](const RotReq& R) { return !E.alive(R.id); }), rot.end());
        E.rotate(rot);
        std::vector<std::shared_ptr<Request>> refine;
        std::vector<PoolBuf> refine_v0;
        for (auto& qp : eig_fin) {
            Request& q = *qp;
            q.values = q.eig.theta;
            q.restarts += q.eig.restarts;
            q.err = q.eig.maxrel;
            q.matvecs += E.matvecs(q.slot);
            int st = QS_OK;
            std::string e;
            if (q.eig.nconv < q.eig.k) {
                st = QS_ERR_NOT_CONVERGED;
                e = "eigsh did not converge within maxiter restarts";
            } else if (q.lane == 1) {
                PoolBuf promoted;
                bool ok = false;
                try {
                    ok = polish(q, promoted);
                } catch (const Error& ex) {
                    st = ex.status;
                    e = ex.what();
                }
                if (st == QS_OK && !ok) {
                    // the polish missed the tolerance: a double-float solve from
                    // the promoted ground vector finishes the job on lane 0
                    E.remove(q.slot);
                    q.slot = -1;
                    q.polished = true;
                    refine.push_back(qp);
                    refine_v0.push_back(std::move(promoted));
                    continue;
                }
            } else if (q.r.want_vector) {
                const int comps = q.cv ? 2 : 1;
                q.vec.resize((size_t)q.n * comps * q.eig.k);
                for (int i = 0; i < q.eig.k; ++i) E.store(q.slot, i, q.vec.data() + (size_t)i * q.n * comps, false);
            }
            E.remove(q.slot);
            q.slot = -1;
            finish(S, qp, st, e);
        }
        for (auto& qp : ln.live) {
            Request& q = *qp;
            if (q.slot >= 0 && q.r.kind == QS_REQ_EIGSH && E.slot(q.slot).state == kSlotHold) E.start(q.slot, q.eig.p);
        }
        if (!refine.empty()) {
            std::vector<const double*> v0s;
            for (auto& b : refine_v0) v0s.push_back(b.as<double>());
            QS_CUDA(cudaStreamSynchronize(s1));
            admit(lane0, refine, v0s);
        }
        // normalise the candidates (column m of each slot, grouped by m), then
        // accept, or split and project the first half step from the same basis
        std::vector<std::shared_ptr<Request>> proj = evo_ev, evo_done, evo_restart, evo_fail;
        bool first_round = true;
        while (!proj.empty()) {
            if (!first_round) {
                std::vector<RotReq> again;
                for (auto& qp : proj) {
                    RotReq R;
                    qp->evo.project(qp->slot, R);
                    again.push_back(std::move(R));
                }
                E.rotate(again);
            }
            first_round = false;
            std::map<int, std::vector<std::shared_ptr<Request>>> by_m;
            for (auto& qp : proj) by_m[qp->m].push_back(qp);
            std::vector<RotReq> copies;
            std::vector<std::shared_ptr<Request>> next;
            for (auto& kv : by_m) {
                std::vector<int> ids;
                for (auto& qp : kv.second) ids.push_back(qp->slot);
                std::vector<double> nr = E.normalize(ids, kv.first);
                for (size_t i = 0; i < kv.second.size(); ++i) {
                    Request& q = *kv.second[i];
                    RotReq cp;
                    const int r = q.evo.after_norm(nr[i], q.slot, cp);
                    q.restarts = q.evo.halvings;
                    q.err = q.evo.err;
                    if (r < 0) {
                        evo_fail.push_back(kv.second[i]);
                    } else if (r == 1) {
                        // accepted: the candidate becomes the next segment's start
                        copies.push_back(std::move(cp));
                        (q.evo.done() ? evo_done : evo_restart).push_back(kv.second[i]);
                    } else {
                        next.push_back(kv.second[i]);
                    }
                }
            }
            E.rotate(copies);
            proj.swap(next);
        }
        for (auto& qp : evo_fail)
            fail(qp, QS_ERR_NOT_CONVERGED, "Krylov exponential action did not converge; increase krylov_dim");
        for (auto& qp : evo_done) {
            Request& q = *qp;
            q.matvecs = E.matvecs(q.slot);
            if (q.r.want_vector) {
                q.vec.resize((size_t)q.n * 2);
                E.store(q.slot, 0, q.vec.data(), false);
                for (double& v : q.vec) v *= q.evo.beta;
            }
            E.remove(q.slot);
            q.slot = -1;
            finish(S, qp, QS_OK, "");
        }
        for (auto& qp : evo_restart) {
            qp->matvecs = E.matvecs(qp->slot);
            E.start(qp->slot, 0);
        }
        prune(ln);
    };
    while (true) {
        std::vector<std::shared_ptr<Request>> fresh;
        {
            std::unique_lock<std::mutex> g(S.mu);
            if (S.stop) break;
            const bool idle = lane0.E.steps_to_event() == 0 && (!lane1 || lane1->E.steps_to_event() == 0);
            if (S.ready.empty() && idle) S.cv_engine.wait_for(g, std::chrono::milliseconds(20));
            if (S.stop) break;
            while (!S.ready.empty()) {
                fresh.push_back(S.ready.front());
                S.ready.pop_front();
            }
        }
        // new slots join between steps, whatever the phase of the others
        std::vector<std::shared_ptr<Request>> to0, to1;
        for (auto& q : fresh) (fp32 && q->r.kind == QS_REQ_EIGSH ? to1 : to0).push_back(q);
        if (!to0.empty()) admit(lane0, to0, {});
        if (!to1.empty()) admit(*lane1, to1, {});
        round(lane0);
        if (lane1) round(*lane1);
        {
            std::lock_guard<std::mutex> g(S.mu);
            S.stats.launches = lane0.E.launches() + (lane1 ? lane1->E.launches() : 0);
        }
    }
    note_launches(lane0.E.launches() + (lane1 ? lane1->E.launches() : 0));
    lane1.reset();
    if (s1) cudaStreamDestroy(s1);
}

}  // namespace

Server* server_create(const qs_server_opts* o) {
    if (o && o->policy != 0 && o->policy != 1) throw Error(QS_ERR_ARGUMENT, "unknown admission policy");
    auto* S = new Server();
    if (o) S->opts = *o;
    if (S->opts.hbm_budget_bytes <= 0) S->opts.hbm_budget_bytes = 150e9;
    if (S->opts.max_slots <= 0) S->opts.max_slots = 64;
    if (S->opts.chunk_steps < 0) S->opts.chunk_steps = 0;
    if (S->opts.chunk_steps == 0) S->opts.chunk_steps = 8;
    if (S->opts.max_wait_s <= 0) S->opts.max_wait_s = 10.0;
    QS_CUDA(cudaGetDevice(&S->opts.device));
    QS_CUDA(cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking));
    if (S->opts.builders <= 0) S->opts.builders = 4;
    for (int i = 0; i < S->opts.builders; ++i) S->builders.emplace_back(builder_loop, std::ref(*S));
    S->engine = std::thread(engine_loop, std::ref(*S));
    return S;
}

void server_destroy(Server* S) {
    {
        std::lock_guard<std::mutex> g(S->mu);
        S->stop = true;
        S->cv_build.notify_all();
        S->cv_engine.notify_all();
    }
    for (auto& t : S->builders)
        if (t.joinable()) t.join();
    if (S->engine.joinable()) S->engine.join();
    cudaStreamSynchronize(S->stream);
    {
        std::lock_guard<std::mutex> g(S->mu);
        for (auto& kv : S->all) kv.second->op.reset();
        S->cache.clear();
    }
    cudaStreamDestroy(S->stream);
    delete S;
}

int64_t server_submit(Server* S, const qs_request* r) {
    if (!r) throw Error(QS_ERR_ARGUMENT, "null request");
    if (r->kind != QS_REQ_EIGSH && r->kind != QS_REQ_EVOLVE) throw Error(QS_ERR_ARGUMENT, "unknown request kind");
    if (r->nterms < 0 || (r->nterms > 0 && !r->terms)) throw Error(QS_ERR_ARGUMENT, "terms missing");
    if (r->kind == QS_REQ_EIGSH && (r->which < 0 || r->which > 4))
        throw Error(QS_ERR_ARGUMENT, "which must be SA, LA, SM, LM, or BE");
    auto q = std::make_shared<Request>();
    q->r = *r;
    q->r.terms = nullptr;
    q->r.v0 = nullptr;
    for (int i = 0; i < r->nterms; ++i) {
        const qs_term& t = r->terms[i];
        if (!t.op) throw Error(QS_ERR_ARGUMENT, "term without an operator string");
        TermCopy c;
        c.op = t.op;
        c.n = t.n_couplings;
        c.cc = t.complex_coeffs;
        int arity = 0;
        for (char ch : c.op)
            if (ch != '|') ++arity;
        c.coeffs.assign(t.coeffs, t.coeffs + 2 * (size_t)std::max(0, t.n_couplings));
        c.sites.assign(t.sites, t.sites + (size_t)arity * std::max(0, t.n_couplings));
        q->terms.push_back(std::move(c));
    }
    if (r->v0) {
        if (r->v0_len <= 0) throw Error(QS_ERR_ARGUMENT, "v0_len must give the length of v0 in doubles");
        q->v0.assign(r->v0, r->v0 + r->v0_len);
    }
    q->key = make_key(q->r, q->terms);
    {
        // rough work estimate: sector size x expected products (a ground state
        // ~150; an exponential ~30 per unit of |t| times the chain length)
        const qs_basis_spec& sp = q->r.basis;
        const double parent = sp.nup >= 0 ? binom(sp.L, sp.nup) : std::ldexp(1.0, sp.L);
        double order = sp.has_kblock ? std::max(1, sp.L / std::max(1, sp.a)) : 1;
        for (int b : {sp.pblock, sp.zblock, sp.pzblock, sp.zAblock, sp.zBblock})
            if (b) order *= 2;
        const double prods = q->r.kind == QS_REQ_EIGSH ? 150.0 : 30.0 * std::max(1.0, std::fabs(q->r.t) * sp.L / 8.0);
        q->work = parent / order * prods;
    }
    std::lock_guard<std::mutex> g(S->mu);
    q->ticket = S->next_ticket++;
    q->t_submit = S->now();
    S->all[q->ticket] = q;
    S->pending.push_back(q);
    S->stats.submitted++;
    S->cv_build.notify_all();
    return q->ticket;
}

static void fill_result(Server* S, const Request& q, qs_result* out) {
    if (!out) return;
    std::memset(out, 0, sizeof(*out));
    out->status = q.status.load();
    out->Ns = q.n;
    const int nv = (int)std::min<size_t>(q.values.size(), 8);
    for (int i = 0; i < nv; ++i) out->values[i] = q.values[i];
    out->nvalues = nv;
    out->submit_s = q.t_submit;
    out->admit_s = q.t_admit;
    out->done_s = q.t_done;
    out->matvecs = q.matvecs;
    out->restarts = q.restarts;
    out->error_estimate = q.err;
    out->vector_len = (int64_t)q.vec.size();
    std::snprintf(out->message, sizeof(out->message), "%s", q.error.c_str());
    (void)S;
}

int server_poll(Server* S, int64_t ticket, qs_result* out) {
    std::lock_guard<std::mutex> g(S->mu);
    auto it = S->all.find(ticket);
    if (it == S->all.end()) throw Error(QS_ERR_ARGUMENT, "unknown ticket");
    fill_result(S, *it->second, out);
    return it->second->status.load();
}

int server_wait(Server* S, int64_t ticket, double timeout_s, qs_result* out) {
    std::unique_lock<std::mutex> g(S->mu);
    auto it = S->all.find(ticket);
    if (it == S->all.end()) throw Error(QS_ERR_ARGUMENT, "unknown ticket");
    std::shared_ptr<Request> q = it->second;
    auto deadline = Clock::now() + std::chrono::duration_cast<Clock::duration>(
                                       std::chrono::duration<double>(timeout_s > 0 ? timeout_s : 1e9));
    while (q->status.load() == QS_PENDING) {
        if (S->cv_done.wait_until(g, deadline) == std::cv_status::timeout) break;
    }
    fill_result(S, *q, out);
    return q->status.load();
}

void server_vector(Server* S, int64_t ticket, double* out, int64_t len) {
    std::lock_guard<std::mutex> g(S->mu);
    auto it = S->all.find(ticket);
    if (it == S->all.end()) throw Error(QS_ERR_ARGUMENT, "unknown ticket");
    const Request& q = *it->second;
    if (q.status.load() != QS_OK) throw Error(QS_ERR_ARGUMENT, "request has no result");
    if (len != (int64_t)q.vec.size()) throw Error(QS_ERR_DIMENSION, "vector length does not match the result");
    std::memcpy(out, q.vec.data(), q.vec.size() * sizeof(double));
}

void server_release(Server* S, int64_t ticket) {
    std::lock_guard<std::mutex> g(S->mu);
    auto it = S->all.find(ticket);
    if (it == S->all.end()) throw Error(QS_ERR_ARGUMENT, "unknown ticket");
    if (it->second->status.load() == QS_PENDING) {
        it->second->cancel = true;
        return;
    }
    S->all.erase(it);
}

void server_stats(Server* S, qs_server_counters* out) {
    std::lock_guard<std::mutex> g(S->mu);
    *out = S->stats;
    out->bytes_in_use = (double)S->used;
    out->peak_bytes = (double)S->peak;
    out->cached_ops = (int64_t)S->cache.size();
    out->running = S->running;
    out->queued = (int64_t)S->pending.size();
}

}  // namespace qs
