"""ctypes binding of libqsgpu (include/qsgpu.h).

There is no CPU fallback: if the shared library is missing or cannot be loaded
the import fails with the loader's message.
"""
from __future__ import annotations

import ctypes
import os

from .errors import raise_status

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libqsgpu.so")

P = ctypes.c_void_p
i32 = ctypes.c_int32
i64 = ctypes.c_int64
f64 = ctypes.c_double


class BasisSpec(ctypes.Structure):
    _fields_ = [(name, i32) for name in (
        "L", "nup", "pauli", "a", "has_kblock", "kblock", "pblock", "zblock", "pzblock", "zAblock", "zBblock")]


class Term(ctypes.Structure):
    _fields_ = [("op", ctypes.c_char_p), ("n_couplings", i32), ("coeffs", P), ("sites", P),
                ("complex_coeffs", i32)]


class GeneralSpec(ctypes.Structure):
    _fields_ = [("L", i32), ("nup", i32), ("pauli", i32), ("nmaps", i32), ("maps", P), ("flips", P), ("qnums", P)]


class EigshOpts(ctypes.Structure):
    _fields_ = [("k", i32), ("which", i32), ("tol", f64), ("ncv", i32), ("maxiter", i32), ("precision", i32),
                ("want_vectors", i32), ("v0", P), ("mem", i32)]


class EigshInfo(ctypes.Structure):
    _fields_ = [("nconv", i32), ("restarts", i32), ("matvecs", i64), ("max_rel_residual", f64), ("seconds", f64)]


class LanczosOpts(ctypes.Structure):
    _fields_ = [("m", i32), ("full_ortho", i32), ("eps", f64), ("complex_vectors", i32), ("mem", i32)]


class ServerOpts(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", f64), ("max_slots", i32), ("precision", i32), ("disable_op_cache", i32),
                ("chunk_steps", i32), ("builders", i32), ("policy", i32), ("max_wait_s", f64), ("device", i32)]


class Request(ctypes.Structure):
    _fields_ = [("kind", i32), ("basis", BasisSpec), ("terms", ctypes.POINTER(Term)), ("nterms", i32),
                ("k", i32), ("which", i32), ("ncv", i32), ("maxiter", i32), ("tol", f64), ("t", f64),
                ("imag_time", i32), ("krylov_dim", i32), ("v0", P), ("v0_len", i64), ("seed", ctypes.c_uint64),
                ("want_vector", i32)]


class Result(ctypes.Structure):
    _fields_ = [("status", i32), ("nvalues", i32), ("Ns", i64), ("values", f64 * 8), ("submit_s", f64),
                ("admit_s", f64), ("done_s", f64), ("matvecs", i64), ("restarts", i32), ("error_estimate", f64),
                ("vector_len", i64), ("message", ctypes.c_char * 128)]


class ServerCounters(ctypes.Structure):
    _fields_ = [(n, i64) for n in ("submitted", "completed", "failed", "builds", "cache_hits", "evictions", "steps",
                                   "launches", "cached_ops", "running", "queued")] + [
        ("bytes_in_use", f64), ("peak_bytes", f64)]


QS_PENDING = 8
QS_REQ_EIGSH, QS_REQ_EVOLVE = 0, 1
QS_F64, QS_C128, QS_F32, QS_C64 = 0, 1, 2, 3
QS_MEM_HOST, QS_MEM_DEVICE = 0, 1
QS_CHECK_SYMM, QS_CHECK_HERM, QS_CHECK_PCON, QS_DIAG_COMPLEX = 1, 2, 4, 8
QS_TRANSPOSE, QS_CONJUGATE, QS_DOUBLE_FLOAT, QS_FIXED_POINT = 1, 2, 4, 8

# every symbol declared in include/qsgpu.h
EXPORTS = (
    "qs_basis_create", "qs_basis_destroy", "qs_basis_size", "qs_basis_requires_complex", "qs_basis_group_order",
    "qs_basis_states", "qs_basis_orbit_minima", "qs_basis_state_index", "qs_basis_representative",
    "qs_op_create", "qs_op_destroy", "qs_op_dtype", "qs_op_hermitian", "qs_op_set_diagonal", "qs_op_matvec",
    "qs_eigsh", "qs_expm_multiply", "qs_evolve", "qs_last_error", "qs_version", "qs_op_set_stream",
    "qs_launch_count", "qs_op_assemble", "qs_op_nnz", "qs_op_fixed_point_classes", "qs_op_matvec_noalloc",
    "qs_eigsh_batch", "qs_basis_stabilizers",
    "qs_server_create", "qs_server_destroy", "qs_server_submit", "qs_server_poll", "qs_server_wait",
    "qs_server_vector", "qs_server_release", "qs_server_stats",
    "qs_lanczos_run", "qs_lanczos_destroy", "qs_lanczos_coefficients", "qs_lanczos_complex", "qs_lanczos_rows",
    "qs_lanczos_combine", "qs_lanczos_overlaps", "qs_lanczos_ritz_matrix",
    "qs_basis_projection_rows", "qs_basis_project_from", "qs_basis_project_to", "qs_block_expm", "qs_op_export_csr", "qs_fp64_fma_rate", "qs_basis_create_general", "qs_expm_columns", "qs_evolve_stepwise",
    "qs_device_alloc_count", "qs_eigs", "qs_grid_barrier_check",
)

_lib = None


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"libqsgpu.so is not built ({LIB_PATH}); run qsgpu.build.build() first")
    L = ctypes.CDLL(LIB_PATH)
    L.qs_basis_create.argtypes = [ctypes.POINTER(BasisSpec), ctypes.POINTER(P)]
    L.qs_basis_destroy.argtypes = [P]
    L.qs_basis_destroy.restype = None
    L.qs_basis_size.argtypes = [P]
    L.qs_basis_size.restype = i64
    L.qs_basis_requires_complex.argtypes = [P]
    L.qs_basis_group_order.argtypes = [P]
    L.qs_basis_group_order.restype = i32
    L.qs_basis_states.argtypes = [P, P, i64]
    L.qs_basis_orbit_minima.argtypes = [P, P, i64]
    L.qs_basis_stabilizers.argtypes = [P, P, i64]
    L.qs_basis_state_index.argtypes = [P, P, i64, P]
    L.qs_basis_representative.argtypes = [P, P, i64, P, P, P, P]
    L.qs_op_create.argtypes = [P, ctypes.POINTER(Term), i32, P, i32, ctypes.POINTER(P)]
    L.qs_op_destroy.argtypes = [P]
    L.qs_op_destroy.restype = None
    L.qs_op_dtype.argtypes = [P]
    L.qs_op_hermitian.argtypes = [P]
    L.qs_op_set_diagonal.argtypes = [P, P]
    L.qs_op_matvec.argtypes = [P, i32, P, P, i32, P, P, i32, i64, i32]
    L.qs_eigsh.argtypes = [P, ctypes.POINTER(EigshOpts), P, P, ctypes.POINTER(EigshInfo)]
    L.qs_eigs.argtypes = [P, ctypes.POINTER(EigshOpts), P, P, ctypes.POINTER(EigshInfo)]
    L.qs_grid_barrier_check.argtypes = [i32, ctypes.c_double, i32]
    L.qs_grid_barrier_check.restype = ctypes.c_int
    L.qs_expm_multiply.argtypes = [P, P, P, P, f64, i32, i32]
    L.qs_evolve.argtypes = [P, P, f64, P, i32, i32, f64, i32, i32, P]
    L.qs_op_set_stream.argtypes = [P, P]
    L.qs_op_matvec_noalloc.argtypes = [P, i32, P, P, i32, P, P, i32, i64]
    L.qs_eigsh_batch.argtypes = [ctypes.POINTER(P), i32, ctypes.POINTER(EigshOpts), P, ctypes.POINTER(P),
                                 ctypes.POINTER(EigshInfo)]
    L.qs_server_create.argtypes = [ctypes.POINTER(ServerOpts), ctypes.POINTER(P)]
    L.qs_server_destroy.argtypes = [P]
    L.qs_server_destroy.restype = None
    L.qs_server_submit.argtypes = [P, ctypes.POINTER(Request), ctypes.POINTER(i64)]
    L.qs_server_poll.argtypes = [P, i64, ctypes.POINTER(Result)]
    L.qs_server_wait.argtypes = [P, i64, f64, ctypes.POINTER(Result)]
    L.qs_server_vector.argtypes = [P, i64, P, i64]
    L.qs_server_release.argtypes = [P, i64]
    L.qs_server_stats.argtypes = [P, ctypes.POINTER(ServerCounters)]
    L.qs_lanczos_run.argtypes = [P, ctypes.POINTER(LanczosOpts), i32, P, ctypes.POINTER(P)]
    L.qs_lanczos_destroy.argtypes = [P]
    L.qs_lanczos_destroy.restype = None
    L.qs_lanczos_coefficients.argtypes = [P, i32, P, P, ctypes.POINTER(i32)]
    L.qs_lanczos_complex.argtypes = [P]
    L.qs_lanczos_rows.argtypes = [P, i32, P, i32]
    L.qs_lanczos_combine.argtypes = [P, i32, P, i32, P, i32]
    L.qs_lanczos_overlaps.argtypes = [P, P, P]
    L.qs_lanczos_ritz_matrix.argtypes = [P, i32, P, P, i32, P]
    L.qs_basis_projection_rows.argtypes = [P, i32]
    L.qs_basis_projection_rows.restype = i64
    L.qs_basis_project_from.argtypes = [P, i32, P, P, i32, i32]
    L.qs_basis_project_to.argtypes = [P, i32, P, P, i32]
    L.qs_op_export_csr.argtypes = [P, P, P, P, P]
    L.qs_fp64_fma_rate.argtypes = [ctypes.POINTER(f64)]
    L.qs_evolve_stepwise.argtypes = [P, P, f64, P, i32, i32, f64, i32, i32, P]
    L.qs_expm_columns.argtypes = [P, P, i32, P, i32, f64, i32, i32, i32, P, i32]
    L.qs_basis_create_general.argtypes = [ctypes.POINTER(GeneralSpec), ctypes.POINTER(P)]
    L.qs_block_expm.argtypes = [P, i32, i32, P, P, i32, f64, i32, i32, P, i32]
    L.qs_op_assemble.argtypes = [P]
    L.qs_op_nnz.argtypes = [P]
    L.qs_op_nnz.restype = i64
    L.qs_op_fixed_point_classes.argtypes = [P]
    L.qs_op_fixed_point_classes.restype = ctypes.c_int32
    L.qs_launch_count.restype = i64
    L.qs_device_alloc_count.restype = i64
    L.qs_last_error.restype = ctypes.c_char_p
    L.qs_version.restype = ctypes.c_char_p
    for name in EXPORTS:
        getattr(L, name)
    _lib = L
    return L


def check(status: int):
    if status != 0:
        raise_status(status, load().qs_last_error().decode(errors="replace"))


def ptr(a):
    return a.ctypes.data_as(P)
