"""The allocation-free host-buffer matvec against the ordinary one.

qs_op_matvec_noalloc serves callers that cannot let the library allocate device
memory: a host program whose device memory belongs to its own pool allocator
with a hard limit (CUDA.jl, PyTorch), or a loop that cannot absorb
cudaMalloc's synchronisation.  It stages x and y through one fixed static
device array, so it must give what qs_op_matvec gives, also on a second call
that finds the previous call's data still in that array, and the library's
allocation counter must not move across any of its calls.  Collected last so
that a run stopping at the first failure has already run every other test.
"""
import numpy as np
import pytest

import models

pytestmark = pytest.mark.gpu

TOL = {"f64": 1e-13, "c128": 1e-13, "f32": 2e-5, "c64": 2e-5}


def _codes(_lib):
    return {"f64": (_lib.QS_F64, np.float64), "c128": (_lib.QS_C128, np.complex128),
            "f32": (_lib.QS_F32, np.float32), "c64": (_lib.QS_C64, np.complex64)}


def _call(lib, _lib, fn, op, flags, x, y, code, alpha, beta, nrhs):
    a = np.array([complex(alpha).real, complex(alpha).imag])
    b = np.array([complex(beta).real, complex(beta).imag])
    args = [op._h, flags, _lib.ptr(a), _lib.ptr(x), code, _lib.ptr(b), _lib.ptr(y), code, nrhs]
    if fn == "qs_op_matvec":
        args.append(_lib.QS_MEM_HOST)
    _lib.check(getattr(lib, fn)(*args))
    return y


def _vectors(n, nrhs, dt, seed):
    cx = np.issubdtype(dt, np.complexfloating)
    cols = [models.seeded(n, seed=seed + j, complex_=cx) for j in range(nrhs)]
    # column-major n x nrhs, as the C ABI reads it
    return np.ascontiguousarray(np.stack(cols).astype(dt))


def _check_twice(lib, _lib, op, n, kind, nrhs, flags, alpha, beta):
    code, dt = _codes(_lib)[kind]
    for call, seed in enumerate((1, 2)):
        x = _vectors(n, nrhs, dt, seed)
        y0 = _vectors(n, nrhs, dt, seed + 10)
        before = lib.qs_device_alloc_count()
        got = _call(lib, _lib, "qs_op_matvec_noalloc", op, flags, x, y0.copy(), code, alpha, beta, nrhs)
        assert lib.qs_device_alloc_count() == before, "the allocation-free matvec allocated device memory"
        want = _call(lib, _lib, "qs_op_matvec", op, flags, x, y0.copy(), code, alpha, beta, nrhs)
        scale = max(1.0, float(np.abs(want).max()))
        assert np.max(np.abs(got - want)) <= TOL[kind] * scale, (kind, nrhs, flags, call)


@pytest.mark.parametrize("assembled", [False, True])
@pytest.mark.parametrize("kind", ["f64", "c128", "f32", "c64"])
def test_noalloc_matches_matvec_twice(qs, assembled, kind):
    from qsgpu import _lib
    lib = _lib.load()
    L = 16
    b = qs.SpinBasis1D(L, nup=8, pauli=False, kblock=0, pblock=1, zblock=1)
    terms = models.to_terms(qs, models.j1j2(L, 1.0, 0.5))
    op = qs.Hamiltonian(b, terms) if assembled else qs.QuantumLinearOperator(b, terms)
    n = b.Ns
    for nrhs in (1, 3):
        for alpha, beta in ((1.0, 0.0), (0.75, -0.5)):
            if kind in ("c128", "c64"):
                alpha, beta = complex(alpha, 0.25), complex(beta, -0.125)
            _check_twice(lib, _lib, op, n, kind, nrhs, 0, alpha, beta)


def test_noalloc_flags_match_matvec(qs):
    """Double-float products, fixed-point row sums, the transpose of a
    non-Hermitian operator and the conjugate give qs_op_matvec's results."""
    from qsgpu import _lib
    lib = _lib.load()
    L = 16
    b = qs.SpinBasis1D(L, nup=8, pauli=False, kblock=0, pblock=1, zblock=1)
    H = qs.Hamiltonian(b, models.to_terms(qs, models.j1j2(L, 1.0, 0.5)))
    assert H.fixed_point_classes > 0
    for flags in (_lib.QS_DOUBLE_FLOAT, _lib.QS_FIXED_POINT, _lib.QS_FIXED_POINT | _lib.QS_TRANSPOSE):
        _check_twice(lib, _lib, H, b.Ns, "f64", 2, flags, 1.0, 0.0)
        _check_twice(lib, _lib, H, b.Ns, "c128", 1, flags, 0.5 - 0.25j, 0.25j)
    # a non-Hermitian operator (no symmetry): transpose and conjugate
    bn = qs.SpinBasis1D(12, nup=6, pauli=False)
    terms = [qs.OperatorTerm("+-", [(0.7 + 0.2j, i, i % 12 + 1) for i in range(1, 13)]),
             qs.OperatorTerm("zz", [(0.3, i, i % 12 + 1) for i in range(1, 13)])]
    op = qs.QuantumLinearOperator(bn, terms, check_herm=False)
    for flags in (_lib.QS_TRANSPOSE, _lib.QS_CONJUGATE, _lib.QS_TRANSPOSE | _lib.QS_CONJUGATE):
        _check_twice(lib, _lib, op, bn.Ns, "c128", 2, flags, 1.25 - 0.5j, -0.5)


def test_noalloc_rejects_oversized_sector_and_bad_flags(qs):
    from qsgpu import _lib
    lib = _lib.load()
    L = 24
    b = qs.SpinBasis1D(L, nup=12, pauli=False)   # 2,704,156 states: 21.6 MB per FP64 vector
    op = qs.QuantumLinearOperator(b, models.to_terms(qs, models.xxz(L)))
    x = np.zeros(b.Ns)
    y = np.zeros(b.Ns)
    a = np.array([1.0, 0.0])
    z = np.array([0.0, 0.0])
    st = lib.qs_op_matvec_noalloc(op._h, 0, _lib.ptr(a), _lib.ptr(x), _lib.QS_F64, _lib.ptr(z), _lib.ptr(y),
                                  _lib.QS_F64, 1)
    assert st == 1
    assert "at most 8 MiB" in lib.qs_last_error().decode()
    small = qs.SpinBasis1D(8, nup=4, pauli=False)
    op = qs.QuantumLinearOperator(small, models.to_terms(qs, models.xxz(8)))
    x = np.zeros(small.Ns)
    y = np.zeros(small.Ns)
    st = lib.qs_op_matvec_noalloc(op._h, 1 << 10, _lib.ptr(a), _lib.ptr(x), _lib.QS_F64, _lib.ptr(z), _lib.ptr(y),
                                  _lib.QS_F64, 1)
    assert st == 1 and "flag" in lib.qs_last_error().decode()
