"""mul!(Y, op, X) with several columns on device buffers: one pass over the
sliced-ELL words for up to eight columns (src/operators.jl:3185-3208 is a
column loop).  Every column must be bit-identical to the single-vector product
and match the oracle."""
import ctypes

import numpy as np
import pytest

import models

pytestmark = pytest.mark.gpu

CASES = [
    (16, 8, dict(kblock=0, pblock=1, zblock=1), "f64"),
    (16, 8, dict(kblock=0, pblock=1, zblock=1), "c128"),
    (16, 8, dict(kblock=3), "c128"),
    (16, 8, dict(kblock=0, pblock=1, zblock=1), "f32"),
    (16, 8, dict(kblock=5), "c64"),
]


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("L,nup,sym,kind", CASES)
@pytest.mark.parametrize("nrhs", [2, 3, 8, 11])
def test_multi_rhs_matches_column_loop(qs, ora, L, nup, sym, kind, nrhs):
    torch = pytest.importorskip("torch")
    from qsgpu import _lib
    lib = _lib.load()
    sp = models.j1j2(L, 1.0, 0.5)
    b = qs.SpinBasis1D(L, nup=nup, pauli=False, **sym)
    H = qs.Hamiltonian(b, models.to_terms(qs, sp))
    n = b.Ns
    code, dt = {"f64": (_lib.QS_F64, np.float64), "c128": (_lib.QS_C128, np.complex128),
                "f32": (_lib.QS_F32, np.float32), "c64": (_lib.QS_C64, np.complex64)}[kind]
    cx = np.issubdtype(dt, np.complexfloating)
    X = np.stack([models.seeded(n, seed=40 + j, complex_=cx) for j in range(nrhs)]).astype(dt)   # nrhs x n = column-major n x nrhs
    Y0 = np.stack([models.seeded(n, seed=90 + j, complex_=cx) for j in range(nrhs)]).astype(dt)
    rep = ora.RepBasis(L, nup=nup, pauli=False, **sym)
    for flags, alpha, beta in ((0, 1.0, 0.0), (0, 0.75 - (0.25j if cx else 0), 0.5), (_lib.QS_TRANSPOSE, 1.25, -0.5)):
        a = np.array([complex(alpha).real, complex(alpha).imag])
        bb = np.array([complex(beta).real, complex(beta).imag])
        xd, yd = _dev(torch, X), _dev(torch, Y0)
        _lib.check(lib.qs_op_matvec(H._h, flags, _lib.ptr(a), ctypes.c_void_p(xd.data_ptr()), code, _lib.ptr(bb),
                                    ctypes.c_void_p(yd.data_ptr()), code, nrhs, _lib.QS_MEM_DEVICE))
        torch.cuda.synchronize()
        got = yd.cpu().numpy()
        for j in range(nrhs):
            xj, yj = _dev(torch, X[j]), _dev(torch, Y0[j])
            _lib.check(lib.qs_op_matvec(H._h, flags, _lib.ptr(a), ctypes.c_void_p(xj.data_ptr()), code,
                                        _lib.ptr(bb), ctypes.c_void_p(yj.data_ptr()), code, 1, _lib.QS_MEM_DEVICE))
            torch.cuda.synchronize()
            assert np.array_equal(got[j], yj.cpu().numpy()), (flags, j)
            xc = X[j].astype(np.complex128)
            # a transposed Hermitian operator is its conjugate: A^T x = conj(A conj(x))
            ax = np.conj(rep.matvec(sp, np.conj(xc))) if flags else rep.matvec(sp, xc)
            want = alpha * ax + beta * Y0[j]
            if not cx:
                want = want.real
            tol = 2e-5 if kind in ("f32", "c64") else 1e-13
            assert np.max(np.abs(got[j] - want)) <= tol * max(1.0, np.abs(want).max()), (flags, j)
