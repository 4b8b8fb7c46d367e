"""The allocation-free host-buffer matvec against the ordinary one.

qs_op_matvec_noalloc serves callers that cannot let the library allocate device
memory (CUDA graph capture in progress, hosts whose device memory belongs to
their own pool allocator, loops that cannot absorb cudaMalloc's
synchronisation).  It stages x and y through one fixed static device array, so
it must give exactly what qs_op_matvec gives, including on a second call that
finds the previous call's data still in that array.  Collected last so that a
run stopping at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

import models

pytestmark = pytest.mark.gpu


def _call(lib, _lib, fn, op, x, y, dtype_code, alpha, beta):
    a = np.array([complex(alpha).real, complex(alpha).imag])
    b = np.array([complex(beta).real, complex(beta).imag])
    args = [op._h, 0, _lib.ptr(a), _lib.ptr(x), dtype_code, _lib.ptr(b), _lib.ptr(y), dtype_code, 1]
    if fn == "qs_op_matvec":
        args.append(_lib.QS_MEM_HOST)
    _lib.check(getattr(lib, fn)(*args))
    return y


@pytest.mark.parametrize("assembled", [False, True])
def test_noalloc_matches_matvec_twice(qs, assembled):
    from qsgpu import _lib
    lib = _lib.load()
    L = 16
    sp = models.j1j2(L, 1.0, 0.5)
    b = qs.SpinBasis1D(L, nup=8, pauli=False, kblock=0, pblock=1, zblock=1)
    terms = models.to_terms(qs, sp)
    op = qs.Hamiltonian(b, terms) if assembled else qs.QuantumLinearOperator(b, terms)
    n = b.Ns
    for call, seed in enumerate((1, 2)):
        x = np.ascontiguousarray(models.seeded(n, seed=seed))
        y0 = np.ascontiguousarray(models.seeded(n, seed=seed + 10))
        for alpha, beta in ((1.0, 0.0), (0.75, -0.5)):
            want = _call(lib, _lib, "qs_op_matvec", op, x, y0.copy(), _lib.QS_F64, alpha, beta)
            got = _call(lib, _lib, "qs_op_matvec_noalloc", op, x, y0.copy(), _lib.QS_F64, alpha, beta)
            assert np.allclose(got, want, rtol=1e-13, atol=1e-13 * np.abs(want).max()), (call, alpha, beta)
    # complex vectors through the same static array
    xc = np.ascontiguousarray(models.seeded(n, seed=5, complex_=True))
    want = _call(lib, _lib, "qs_op_matvec", op, xc, np.zeros(n, dtype=np.complex128), _lib.QS_C128, 1.0, 0.0)
    got = _call(lib, _lib, "qs_op_matvec_noalloc", op, xc, np.zeros(n, dtype=np.complex128), _lib.QS_C128, 1.0, 0.0)
    assert np.allclose(got, want, rtol=1e-13, atol=1e-13 * np.abs(want).max())


def test_noalloc_rejects_oversized_sector(qs):
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
