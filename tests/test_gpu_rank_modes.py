"""The three rank lookups of the matrix-free product give the same result.

The column of a generated state's representative comes from the direct
rank -> column table, a per-thread binary search behind shared-memory
splitters, or the warp-cooperative search (all 32 lanes probing the splitters
and the sorted representatives together).  QS_RANK_MODE selects one; the
products must be bit-identical and match the oracle.
"""
import os

import numpy as np
import pytest

import models

pytestmark = pytest.mark.gpu

CASES = [
    (16, 8, False, dict(kblock=0, pblock=1, zblock=1), "j1j2"),
    (16, 8, False, dict(kblock=3), "j1j2"),
    (14, None, True, dict(kblock=0, pblock=1), "tfim"),
    (20, 10, False, dict(kblock=0, pblock=-1), "j1j2"),
]


@pytest.fixture
def rank_env():
    old = os.environ.get("QS_RANK_MODE")
    yield
    if old is None:
        os.environ.pop("QS_RANK_MODE", None)
    else:
        os.environ["QS_RANK_MODE"] = old


@pytest.mark.parametrize("L,nup,pauli,sym,model", CASES)
def test_rank_modes_identical(qs, ora, rank_env, L, nup, pauli, sym, model):
    sp = models.tfim(L, 1.0, 0.7) if model == "tfim" else models.j1j2(L, 1.0, 0.5)
    b = qs.SpinBasis1D(L, nup=nup, pauli=pauli, **sym)
    op = qs.QuantumLinearOperator(b, models.to_terms(qs, sp))
    rep = ora.RepBasis(L, nup=nup, pauli=pauli, **sym)
    x = models.seeded(b.Ns, complex_=True)
    want = rep.matvec(sp, x)
    scale = max(1.0, float(np.abs(want).max()))
    first = None
    for mode in ("direct", "search", "warp"):
        os.environ["QS_RANK_MODE"] = mode
        got = op.dot(x)
        assert np.max(np.abs(got - want)) <= 1e-13 * scale, mode
        got32 = op.dot(x.astype(np.complex64), precision="fp32")
        assert np.max(np.abs(got32 - want)) <= 2e-5 * scale, mode
        if first is None:
            first = got
        else:
            assert np.array_equal(got, first), mode
