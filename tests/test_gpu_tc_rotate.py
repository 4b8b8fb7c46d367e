"""The thick-restart rotation on the tensor cores against the FP64 rotation.

eigsh's restarts rotate the Krylov basis by the Ritz vectors (V[:, :p] = V Y),
which the FP64 engine runs as an exact sliced integer product on the FP16
tensor cores (tcgen05).  QS_TC_ROTATE=0 keeps the rotation on the FP64
arithmetic kernel; both must give the same eigenpairs, and those must match the
dense spectrum (1e-10 relative) with FP64-class residuals.  The double-float
engine keeps its FP32-pipe rotation and must agree as well.
"""
import os

import numpy as np
import pytest

import models

pytestmark = pytest.mark.gpu

CASES = [
    (18, 9, dict(kblock=0, pblock=1, zblock=1), 1),
    (18, 9, dict(kblock=0, pblock=1, zblock=1), 4),
    (16, 8, dict(kblock=3), 2),          # complex vectors, real Ritz coefficients
    (14, None, dict(kblock=0, pblock=1), 3),
    (24, 12, dict(kblock=0, pblock=1, zblock=1), 2),   # many row blocks
]


@pytest.fixture
def tc_env():
    old = os.environ.get("QS_TC_ROTATE")
    yield
    if old is None:
        os.environ.pop("QS_TC_ROTATE", None)
    else:
        os.environ["QS_TC_ROTATE"] = old


@pytest.mark.parametrize("L,nup,sym,k", CASES)
@pytest.mark.parametrize("prec", ["fp64", "fp64df"])
def test_tensor_core_rotation_matches(qs, ora, tc_env, L, nup, sym, k, prec):
    pauli = nup is None
    sp = models.tfim(L, 1.0, 0.7) if pauli else models.j1j2(L, 1.0, 0.5)
    b = qs.SpinBasis1D(L, nup=nup, pauli=pauli, **sym)
    H = qs.Hamiltonian(b, models.to_terms(qs, sp))
    v0 = models.seeded(b.Ns, seed=5, complex_=H.dtype == np.complex128)
    out = {}
    for tc in ("1", "0"):
        os.environ["QS_TC_ROTATE"] = tc
        info = {}
        vals, vecs = qs.eigsh(H, k=k, which="SA", tol=1e-12, v0=v0, ncv=12, precision=prec, info=info)
        assert info["restarts"] >= 1   # the rotation ran
        out[tc] = (vals, vecs)
    va, Va = out["1"]
    vb, Vb = out["0"]
    scale = float(np.abs(vb).max())
    assert np.max(np.abs(va - vb)) <= 1e-11 * scale
    # residuals of the tensor-core run's eigenpairs
    R = np.stack([H.dot(Va[:, j]) for j in range(k)], axis=1) - Va * va
    assert np.max(np.linalg.norm(R, axis=0)) <= 1e-8 * scale
    assert np.allclose(np.linalg.norm(Va, axis=0), 1.0, atol=1e-12)
    rep = ora.RepBasis(L, nup=nup, pauli=pauli, **sym)
    n = b.Ns
    if n <= 3000:
        D = np.zeros((n, n), dtype=np.complex128)
        e = np.zeros(n, dtype=np.complex128)
        for j in range(n):
            e[:] = 0
            e[j] = 1
            D[:, j] = rep.matvec(sp, e)
        w = np.linalg.eigvalsh(D)
        assert np.allclose(va, w[:k], rtol=1e-10, atol=1e-10 * scale)
