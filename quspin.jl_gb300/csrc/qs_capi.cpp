// qs_capi.cpp -- the C ABI (include/qsgpu.h): status codes, last-error text,
// host/device buffer staging.  Every entry point catches exceptions and turns
// them into a qs_status; nothing throws across the boundary.
#include <cstring>
#include <string>
#include <vector>

#include "../../include/qsgpu.h"
#include "qs_internal.h"
#include "qs_krylov.h"
#include "qs_server.h"
#include "qs_tools.h"

struct qs_basis {
    qs::Basis b;
};
struct qs_op {
    qs::Op* op;
};
struct qs_server {
    qs::Server* s;
};
struct qs_lanczos {
    std::unique_ptr<qs::LanczosSet> l;
};

namespace {

thread_local std::string g_last_error;

template <typename F>
int guard(F&& f) {
    try {
        g_last_error.clear();
        f();
        return QS_OK;
    } catch (const qs::Error& e) {
        g_last_error = e.what();
        return e.status;
    } catch (const std::bad_alloc&) {
        g_last_error = "host allocation failed";
        return QS_ERR_NOMEM;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return QS_ERR_CUDA;
    }
}

bool is_complex(int dt) { return dt == QS_C128 || dt == QS_C64; }
bool is_single(int dt) { return dt == QS_F32 || dt == QS_C64; }
size_t dt_bytes(int dt) {
    switch (dt) {
        case QS_F64: return 8;
        case QS_C128: return 16;
        case QS_F32: return 4;
        case QS_C64: return 8;
        default: throw qs::Error(QS_ERR_ARGUMENT, "unknown dtype");
    }
}

}  // namespace

extern "C" {

const char* qs_last_error(void) { return g_last_error.c_str(); }
const char* qs_version(void) { return "qsgpu 0.1.0 (sm_103a)"; }

int qs_basis_create(const qs_basis_spec* spec, qs_basis** out) {
    return guard([&] {
        if (!spec || !out) throw qs::Error(QS_ERR_ARGUMENT, "null argument");
        *out = nullptr;
        qs_basis* h = new qs_basis();
        h->b.spec = *spec;
        try {
            qs::basis_build(h->b);
        } catch (...) {
            delete h;
            throw;
        }
        *out = h;
    });
}

void qs_basis_destroy(qs_basis* basis) { delete basis; }

int64_t qs_basis_size(const qs_basis* basis) { return basis ? basis->b.n : -1; }

int qs_basis_create_general(const qs_general_spec* spec, qs_basis** out) {
    return guard([&] {
        if (!spec || !out) throw qs::Error(QS_ERR_ARGUMENT, "null argument");
        *out = nullptr;
        qs_basis* h = new qs_basis();
        try {
            qs::basis_build_general(h->b, *spec);
        } catch (...) {
            delete h;
            throw;
        }
        *out = h;
    });
}

int qs_basis_requires_complex(const qs_basis* basis) { return basis && basis->b.complex_chars ? 1 : 0; }

int32_t qs_basis_group_order(const qs_basis* basis) { return basis ? basis->b.group.ng : 0; }

// a basis from the dense nullspace intersection has no orbit structure
static void no_orbits(const qs::Basis& b) {
    if (b.dense_proj)
        throw qs::Error(QS_ERR_UNSUPPORTED, "a sector from the dense nullspace intersection has no orbits; its "
                                            "columns are general combinations of parent states");
}

int qs_basis_orbit_minima(const qs_basis* basis, uint64_t* out, int64_t n) {
    return guard([&] {
        const qs::Basis& b = basis->b;
        no_orbits(b);
        if (n != b.n) throw qs::Error(QS_ERR_DIMENSION, "output length must equal Ns");
        if (!b.symmetric) {
            if (b.nup < 0) {
                for (int64_t i = 0; i < n; ++i) out[i] = (uint64_t)i;
                return;
            }
            // Gosper order (src/basis.jl:229-250)
            if (b.nup == 0) { out[0] = 0; return; }
            uint64_t s = (b.nup >= 64) ? ~0ull : ((1ull << b.nup) - 1ull);
            for (int64_t i = 0; i < n; ++i) {
                out[i] = s;
                if (i == n - 1) break;
                uint64_t lowest = s & (~s + 1ull);
                uint64_t next = s + lowest;
                s = next | (((next ^ s) >> 2) >> __builtin_ctzll(lowest));
            }
            return;
        }
        if (b.wide) {
            QS_CUDA(cudaMemcpy(out, b.d_reps.p, n * sizeof(uint64_t), cudaMemcpyDeviceToHost));
        } else {
            std::vector<uint32_t> tmp(n);
            QS_CUDA(cudaMemcpy(tmp.data(), b.d_reps.p, n * sizeof(uint32_t), cudaMemcpyDeviceToHost));
            for (int64_t i = 0; i < n; ++i) out[i] = tmp[i];
        }
    });
}

int qs_basis_stabilizers(const qs_basis* basis, uint16_t* out, int64_t n) {
    return guard([&] {
        const qs::Basis& b = basis->b;
        no_orbits(b);
        if (n != b.n) throw qs::Error(QS_ERR_DIMENSION, "output length must equal Ns");
        if (!b.symmetric) {
            for (int64_t i = 0; i < n; ++i) out[i] = 1;
            return;
        }
        QS_CUDA(cudaMemcpy(out, b.d_stab.p, n * sizeof(uint16_t), cudaMemcpyDeviceToHost));
    });
}

int qs_basis_states(const qs_basis* basis, uint64_t* out, int64_t n) {
    if (!basis) return QS_ERR_ARGUMENT;
    if (basis->b.dense_proj)
        return guard([&] {
            if (n != basis->b.n) throw qs::Error(QS_ERR_DIMENSION, "output length must equal Ns");
            std::memcpy(out, basis->b.proj_reps.data(), n * sizeof(uint64_t));
        });
    if (!basis->b.symmetric) return qs_basis_orbit_minima(basis, out, n);
    return guard([&] {
        qs::Basis& b = const_cast<qs::Basis&>(basis->b);
        if (n != b.n) throw qs::Error(QS_ERR_DIMENSION, "output length must equal Ns");
        qs::basis_compute_refrep(b);
        std::memcpy(out, b.h_refrep.data(), n * sizeof(uint64_t));
    });
}

int qs_basis_state_index(const qs_basis* basis, const uint64_t* states, int64_t n, int64_t* out) {
    return guard([&] {
        const qs::Basis& b = basis->b;
        if (b.dense_proj) {
            for (int64_t i = 0; i < n; ++i) {
                auto it = b.proj_index.find(states[i]);
                out[i] = it == b.proj_index.end() ? -1 : it->second;
            }
            return;
        }
        qs::basis_index_of(const_cast<qs::Basis&>(b), states, n, out);
    });
}

int qs_basis_representative(const qs_basis* basis, const uint64_t* states, int64_t n, uint64_t* reps, double* norms,
                            double* amps, int32_t* status) {
    return guard([&] {
        no_orbits(basis->b);
        qs::basis_representative(const_cast<qs::Basis&>(basis->b), states, n, reps, norms, amps, status);
    });
}

int64_t qs_basis_projection_rows(const qs_basis* basis, int32_t pcon) {
    if (!basis) return -1;
    try {
        return qs::basis_projection_rows(basis->b, pcon != 0);
    } catch (const std::exception&) {
        return -1;
    }
}

int qs_basis_project_from(qs_basis* basis, int32_t pcon, const double* v, double* out, int32_t accumulate,
                          int32_t mem) {
    return guard([&] {
        if (!basis || !v || !out) throw qs::Error(QS_ERR_ARGUMENT, "null argument");
        qs::basis_project(basis->b, pcon != 0, 0, v, out, accumulate != 0, mem == QS_MEM_DEVICE);
    });
}

int qs_basis_project_to(qs_basis* basis, int32_t pcon, const double* v, double* out, int32_t mem) {
    return guard([&] {
        if (!basis || !v || !out) throw qs::Error(QS_ERR_ARGUMENT, "null argument");
        qs::basis_project(basis->b, pcon != 0, 1, v, out, false, mem == QS_MEM_DEVICE);
    });
}

int qs_op_create(qs_basis* basis, const qs_term* terms, int32_t nterms, const double* diagonal, int32_t checks,
                 qs_op** out) {
    return guard([&] {
        if (!basis || !out) throw qs::Error(QS_ERR_ARGUMENT, "null argument");
        *out = nullptr;
        qs::Op* op = qs::op_create(&basis->b, terms, nterms, diagonal, checks);
        *out = new qs_op{op};
    });
}

void qs_op_destroy(qs_op* op) {
    if (!op) return;
    delete op->op;
    delete op;
}

int qs_op_set_stream(qs_op* op, void* stream) {
    return guard([&] {
        qs::Op& o = *op->op;
        QS_CUDA(cudaStreamSynchronize(o.stream));
        o.stream = stream ? (cudaStream_t)stream : o.own_stream;
    });
}

int64_t qs_launch_count(void) { return qs::launches(); }
int64_t qs_device_alloc_count(void) { return qs::device_allocs(); }

int qs_op_assemble(qs_op* op) {
    return guard([&] {
        if (op->op->dense) return;   // held as the dense P^H A P from creation
        qs::op_assemble(*op->op);
    });
}

int64_t qs_op_nnz(const qs_op* op) {
    const qs::Op& o = *op->op;
    if (o.dense) {
        // off-diagonal stored entries of P^H A P, as the export lists them
        return o.dense_offdiag_nnz;
    }
    return o.assembled ? o.asm_.nnz : -1;
}

int32_t qs_op_fixed_point_classes(const qs_op* op) {
    const qs::Op& o = *op->op;
    return o.assembled && o.asm_.has_sell ? o.asm_.fx_classes : 0;
}

int qs_op_export_csr(qs_op* op, int64_t* rowptr, int64_t* cols, double* values, double* diag) {
    return guard([&] {
        if (!op || !rowptr || !diag) throw qs::Error(QS_ERR_ARGUMENT, "null argument");
        if (op->op->dense) {
            qs::op_export_dense(*op->op, rowptr, cols, values, diag);
            return;
        }
        if (!op->op->assembled) throw qs::Error(QS_ERR_ARGUMENT, "assemble the operator first (qs_op_assemble)");
        if (op->op->asm_.nnz && (!cols || !values)) throw qs::Error(QS_ERR_ARGUMENT, "null argument");
        qs::op_export_csr(*op->op, rowptr, cols, values, diag);
    });
}

int qs_op_dtype(const qs_op* op) { return op->op->complex_mat ? QS_C128 : QS_F64; }
int qs_op_hermitian(const qs_op* op) { return op->op->hermitian ? 1 : 0; }

int qs_op_set_diagonal(qs_op* op, const double* diagonal) {
    return guard([&] {
        qs::Op& o = *op->op;
        o.user_diag.resize(o.basis->n);
        for (int64_t i = 0; i < o.basis->n; ++i) o.user_diag[i] = {diagonal[2 * i], diagonal[2 * i + 1]};
        if (o.dense) {
            qs::op_dense_apply_diagonal(o);
            return;
        }
        qs::op_prepare_device(o);
    });
}

int qs_op_matvec(qs_op* op, int32_t flags, const double* alpha, const void* x, int32_t x_dtype, const double* beta,
                 void* y, int32_t y_dtype, int64_t nrhs, int32_t mem) {
    return guard([&] {
        qs::Op& o = *op->op;
        const int64_t n = o.basis->n;
        if (is_single(x_dtype) != is_single(y_dtype))
            throw qs::Error(QS_ERR_ARGUMENT, "input and output must share a precision");
        if (!is_complex(y_dtype) && (is_complex(x_dtype) || o.complex_mat))
            throw qs::Error(QS_ERR_ARGUMENT, "the output must be complex for a complex operator or input");
        if (nrhs < 0) throw qs::Error(QS_ERR_DIMENSION, "nrhs must be nonnegative");
        const bool single = is_single(y_dtype);
        const bool ycx = is_complex(y_dtype);
        const size_t yb = dt_bytes(y_dtype), xb = dt_bytes(x_dtype);
        qs::MatvecCall c;
        c.flags = flags & (QS_TRANSPOSE | QS_CONJUGATE);
        c.df = (flags & QS_DOUBLE_FLOAT) != 0;
        c.fx = (flags & QS_FIXED_POINT) != 0;
        c.alpha = qs::cx(alpha ? alpha[0] : 1.0, alpha ? alpha[1] : 0.0);
        c.beta = qs::cx(beta ? beta[0] : 0.0, beta ? beta[1] : 0.0);
        c.single = single;
        c.x_complex = ycx;
        c.y_complex = ycx;
        const bool beta_zero = c.beta.re == 0.0 && c.beta.im == 0.0;
        if (mem == QS_MEM_DEVICE) {
            if (is_complex(x_dtype) != ycx)
                throw qs::Error(QS_ERR_UNSUPPORTED, "device buffers must share the output dtype");
            c.x = x;
            c.y = y;
            // several columns at once on the sliced-ELL form (one pass over its words)
            if (nrhs > 1 && qs::op_spmm_device(o, c, nrhs, o.stream)) return;
            for (int64_t j = 0; j < nrhs; ++j) {
                c.x = (const char*)x + (size_t)j * n * xb;
                c.y = (char*)y + (size_t)j * n * yb;
                qs::op_matvec_device(o, c, o.stream);
            }
            return;  // asynchronous on the operator's stream
        }
        if (!o.d_x.p || o.d_x.bytes < n * yb) o.d_x.alloc(n * yb);
        if (!o.d_y.p || o.d_y.bytes < n * yb) o.d_y.alloc(n * yb);
        std::vector<char> widen;
        for (int64_t j = 0; j < nrhs; ++j) {
            const char* xs = (const char*)x + (size_t)j * n * xb;
            if (is_complex(x_dtype) == ycx) {
                QS_CUDA(cudaMemcpyAsync(o.d_x.p, xs, n * yb, cudaMemcpyHostToDevice, o.stream));
            } else {
                // real input, complex output: widen on the host
                widen.assign(n * yb, 0);
                for (int64_t i = 0; i < n; ++i) {
                    if (single) ((float*)widen.data())[2 * i] = ((const float*)xs)[i];
                    else ((double*)widen.data())[2 * i] = ((const double*)xs)[i];
                }
                QS_CUDA(cudaMemcpyAsync(o.d_x.p, widen.data(), n * yb, cudaMemcpyHostToDevice, o.stream));
            }
            char* ys = (char*)y + (size_t)j * n * yb;
            c.x = o.d_x.p;
            // page-locked y and nothing to read from it: the product writes it
            // through its mapped address, with no device copy and no read-back
            void* y_mapped = beta_zero ? qs::mapped_host_address(ys) : nullptr;
            if (y_mapped) {
                c.y = y_mapped;
                qs::op_matvec_device(o, c, o.stream);
                QS_CUDA(cudaStreamSynchronize(o.stream));
                continue;
            }
            if (!beta_zero) QS_CUDA(cudaMemcpyAsync(o.d_y.p, ys, n * yb, cudaMemcpyHostToDevice, o.stream));
            c.y = o.d_y.p;
            // the assembled product in row ranges, each range read back while the
            // next computes; otherwise one product and one read-back
            if (!qs::op_matvec_host_overlap(o, c, ys, yb)) {
                qs::op_matvec_device(o, c, o.stream);
                QS_CUDA(cudaMemcpyAsync(ys, o.d_y.p, n * yb, cudaMemcpyDeviceToHost, o.stream));
            }
            QS_CUDA(cudaStreamSynchronize(o.stream));
        }
    });
}

int qs_op_matvec_noalloc(qs_op* op, int32_t flags, const double* alpha, const void* x, int32_t x_dtype,
                         const double* beta, void* y, int32_t y_dtype, int64_t nrhs) {
    return guard([&] {
        qs::op_matvec_noalloc(*op->op, flags, qs::cx(alpha ? alpha[0] : 1.0, alpha ? alpha[1] : 0.0), x, x_dtype,
                              qs::cx(beta ? beta[0] : 0.0, beta ? beta[1] : 0.0), y, y_dtype, nrhs);
    });
}

int qs_eigsh(qs_op* op, const qs_eigsh_opts* opts, double* values, void* vectors, qs_eigsh_info* info) {
    return guard([&] { qs::eigsh(*op->op, *opts, values, vectors, info); });
}

int qs_eigs(qs_op* op, const qs_eigsh_opts* opts, double* values, void* vectors, qs_eigsh_info* info) {
    return guard([&] {
        if (!op || !opts || !values) throw qs::Error(QS_ERR_ARGUMENT, "null argument");
        qs::eigs_general(*op->op, *opts, values, vectors, info);
    });
}

int qs_eigsh_batch(qs_op* const* ops, int32_t nops, const qs_eigsh_opts* opts, double* values, void** vectors,
                   qs_eigsh_info* infos) {
    return guard([&] {
        std::vector<qs::Op*> v(nops);
        for (int i = 0; i < nops; ++i) v[i] = ops[i]->op;
        qs::eigsh_batch(v.data(), nops, *opts, values, vectors, infos);
    });
}

int qs_expm_multiply(qs_op* op, const double* a, const double* v, double* out, double tol, int32_t krylov_dim,
                     int32_t precision) {
    return guard([&] {
        qs::expm_multiply(*op->op, std::complex<double>(a[0], a[1]), v, out, tol, krylov_dim, precision);
    });
}

int qs_evolve(qs_op* op, const double* v0, double t0, const double* times, int32_t nt, int32_t imag_time, double tol,
              int32_t krylov_dim, int32_t precision, double* out) {
    return guard(
        [&] { qs::evolve(*op->op, v0, t0, times, nt, imag_time, tol, krylov_dim, precision, out); });
}

// ------------------------------------------------------------------ Krylov tools
int qs_lanczos_run(qs_op* op, const qs_lanczos_opts* opts, int32_t nstart, const double* v0, qs_lanczos** out) {
    return guard([&] {
        if (!op || !opts || !out) throw qs::Error(QS_ERR_ARGUMENT, "null argument");
        *out = nullptr;
        auto l = qs::lanczos_run(*op->op, *opts, nstart, v0);
        *out = new qs_lanczos{std::move(l)};
    });
}

void qs_lanczos_destroy(qs_lanczos* lanczos) { delete lanczos; }

int qs_lanczos_coefficients(const qs_lanczos* lanczos, int32_t s, double* alphas, double* betas, int32_t* used) {
    return guard([&] {
        if (!lanczos) throw qs::Error(QS_ERR_ARGUMENT, "null argument");
        const qs::LanczosSet& L = *lanczos->l;
        if (s < 0 || s >= (int)L.ids.size()) throw qs::Error(QS_ERR_ARGUMENT, "start index outside the Lanczos set");
        if (alphas) std::memcpy(alphas, L.alphas[s].data(), L.alphas[s].size() * sizeof(double));
        if (betas) std::memcpy(betas, L.betas[s].data(), L.betas[s].size() * sizeof(double));
        if (used) *used = L.used[s];
    });
}

int qs_lanczos_complex(const qs_lanczos* lanczos) { return lanczos && lanczos->l->cv ? 1 : 0; }

int qs_lanczos_rows(qs_lanczos* lanczos, int32_t s, double* out, int32_t mem) {
    return guard([&] {
        if (!lanczos || !out) throw qs::Error(QS_ERR_ARGUMENT, "null argument");
        qs::lanczos_rows(*lanczos->l, s, out, mem == QS_MEM_DEVICE);
    });
}

int qs_lanczos_combine(qs_lanczos* lanczos, int32_t s, const double* coeff, int32_t ncoef, double* out,
                       int32_t mem) {
    return guard([&] {
        if (!lanczos) throw qs::Error(QS_ERR_ARGUMENT, "null argument");
        qs::lanczos_combine(*lanczos->l, s, coeff, ncoef, out, mem == QS_MEM_DEVICE);
    });
}

int qs_lanczos_overlaps(qs_lanczos* lanczos, qs_op* observable, double* out) {
    return guard([&] {
        if (!lanczos || !observable || !out) throw qs::Error(QS_ERR_ARGUMENT, "null argument");
        qs::lanczos_overlaps(*lanczos->l, *observable->op, out);
    });
}

int qs_lanczos_ritz_matrix(qs_lanczos* lanczos, int32_t s, qs_op* observable, const double* Y, int32_t nv,
                           double* out) {
    return guard([&] {
        if (!lanczos || !observable) throw qs::Error(QS_ERR_ARGUMENT, "null argument");
        qs::lanczos_ritz_matrix(*lanczos->l, s, *observable->op, Y, nv, out);
    });
}

int qs_evolve_stepwise(qs_op* op, const double* v0, double t0, const double* times, int32_t nt, int32_t imag_time,
                       double tol, int32_t krylov_dim, int32_t precision, double* out) {
    return guard([&] {
        if (!op || !v0 || !out || (nt > 0 && !times)) throw qs::Error(QS_ERR_ARGUMENT, "null argument");
        if (krylov_dim < 1) throw qs::Error(QS_ERR_ARGUMENT, "krylov_dim must be positive");
        std::vector<double> off(std::max(0, nt));
        for (int i = 0; i < nt; ++i) off[i] = times[i] - t0;
        qs::evolve_stepwise(*op->op, v0, off, imag_time != 0, tol > 0 ? tol : 1e-12, krylov_dim, precision, out);
    });
}

int qs_expm_columns(qs_op* op, const double* V, int32_t ncol, const double* scales, int32_t nscales, double tol,
                    int32_t krylov_dim, int32_t precision, int32_t normalise, double* out, int32_t mem) {
    return guard([&] {
        if (!op || !V || !scales || !out) throw qs::Error(QS_ERR_ARGUMENT, "null argument");
        if (krylov_dim < 1) throw qs::Error(QS_ERR_ARGUMENT, "krylov_dim must be positive");
        std::vector<std::complex<double>> sc(std::max(0, nscales));
        for (int i = 0; i < nscales; ++i) sc[i] = {scales[2 * i], scales[2 * i + 1]};
        qs::expm_columns(*op->op, V, ncol, sc, tol > 0 ? tol : 1e-12, krylov_dim, precision, normalise != 0, out,
                         mem == QS_MEM_DEVICE);
    });
}

int qs_grid_barrier_check(int32_t phantom, double limit_ms, int32_t blocks) {
    return guard([&] { qs::grid_barrier_check(phantom, limit_ms, blocks); });
}

int qs_fp64_fma_rate(double* fma_per_s) {
    return guard([&] {
        if (!fma_per_s) throw qs::Error(QS_ERR_ARGUMENT, "null argument");
        *fma_per_s = qs::fp64_fma_rate();
    });
}

int qs_block_expm(qs_op* const* ops, int32_t nblocks, int32_t pcon, const double* psi, const double* scales,
                  int32_t nscales, double tol, int32_t krylov_dim, int32_t precision, double* out, int32_t mem) {
    return guard([&] {
        if (!ops || nblocks < 1 || !psi || !scales || !out || nscales < 1)
            throw qs::Error(QS_ERR_ARGUMENT, "null argument");
        std::vector<qs::Op*> v(nblocks);
        for (int b = 0; b < nblocks; ++b) v[b] = ops[b]->op;
        std::vector<std::complex<double>> sc(nscales);
        for (int i = 0; i < nscales; ++i) sc[i] = {scales[2 * i], scales[2 * i + 1]};
        if (krylov_dim < 1) throw qs::Error(QS_ERR_ARGUMENT, "krylov_dim must be positive");
        qs::block_expm(v, pcon != 0, psi, sc, tol > 0 ? tol : 1e-12, krylov_dim, precision, out, mem == QS_MEM_DEVICE);
    });
}

}  // extern "C"

// ------------------------------------------------------------------ serving
int qs_server_create(const qs_server_opts* opts, qs_server** out) {
    return guard([&] {
        if (!out) throw qs::Error(QS_ERR_ARGUMENT, "null argument");
        *out = nullptr;
        *out = new qs_server{qs::server_create(opts)};
    });
}

void qs_server_destroy(qs_server* server) {
    if (!server) return;
    qs::server_destroy(server->s);
    delete server;
}

int qs_server_submit(qs_server* server, const qs_request* req, int64_t* ticket) {
    return guard([&] {
        if (!server || !ticket) throw qs::Error(QS_ERR_ARGUMENT, "null argument");
        *ticket = qs::server_submit(server->s, req);
    });
}

int qs_server_poll(qs_server* server, int64_t ticket, qs_result* out) {
    int st = QS_OK;
    int rc = guard([&] {
        if (!server) throw qs::Error(QS_ERR_ARGUMENT, "null argument");
        st = qs::server_poll(server->s, ticket, out);
    });
    return rc != QS_OK ? rc : st;
}

int qs_server_wait(qs_server* server, int64_t ticket, double timeout_s, qs_result* out) {
    int st = QS_OK;
    int rc = guard([&] {
        if (!server) throw qs::Error(QS_ERR_ARGUMENT, "null argument");
        st = qs::server_wait(server->s, ticket, timeout_s, out);
    });
    return rc != QS_OK ? rc : st;
}

int qs_server_vector(qs_server* server, int64_t ticket, double* out, int64_t len) {
    return guard([&] {
        if (!server || !out) throw qs::Error(QS_ERR_ARGUMENT, "null argument");
        qs::server_vector(server->s, ticket, out, len);
    });
}

int qs_server_release(qs_server* server, int64_t ticket) {
    return guard([&] {
        if (!server) throw qs::Error(QS_ERR_ARGUMENT, "null argument");
        qs::server_release(server->s, ticket);
    });
}

int qs_server_stats(qs_server* server, qs_server_counters* out) {
    return guard([&] {
        if (!server || !out) throw qs::Error(QS_ERR_ARGUMENT, "null argument");
        qs::server_stats(server->s, out);
    });
}
