"""Every sliced-ELL kernel variant gives the same product.

The assembled product picks one of six kernel variants by timing (gathers in
flight per thread x resident blocks, each with plain loads or with the
evict-first word stream / evict-last x gathers).  The variants differ only in
how they load, not in their arithmetic or summation order, so their results
must be bit-identical; QS_SELL_VARIANT runs each in turn here, on a real, a
complex-vector and a complex-operator sector, in FP64, double-float,
fixed-point and FP32 form, against the oracle.
"""
import os

import numpy as np
import pytest

import models

pytestmark = pytest.mark.gpu

NVAR = 6
CASES = [
    (16, 8, dict(kblock=0, pblock=1, zblock=1), False),
    (16, 8, dict(kblock=3), True),
    (14, 7, dict(kblock=0, pblock=-1), True),
]


@pytest.fixture
def variant_env():
    old = os.environ.get("QS_SELL_VARIANT")
    yield
    if old is None:
        os.environ.pop("QS_SELL_VARIANT", None)
    else:
        os.environ["QS_SELL_VARIANT"] = old


@pytest.mark.parametrize("L,nup,sym,cx", CASES)
def test_all_variants_identical(qs, ora, variant_env, L, nup, sym, cx):
    sp = models.j1j2(L, 1.0, 0.5)
    b = qs.SpinBasis1D(L, nup=nup, pauli=False, **sym)
    rep = ora.RepBasis(L, nup=nup, pauli=False, **sym)
    H = qs.Hamiltonian(b, models.to_terms(qs, sp))
    x = models.seeded(b.Ns, complex_=cx)
    want = rep.matvec(sp, x)
    if not cx and H.dtype == np.float64:
        want = want.real
    scale = max(1.0, float(np.abs(want).max()))
    forms = ["fp64", "fp64df", "fp32"] + (["fp64fx"] if H.fixed_point_classes else [])
    first = {}
    for v in range(NVAR):
        os.environ["QS_SELL_VARIANT"] = str(v)
        for prec in forms:
            xin = x.astype(np.complex64 if cx else np.float32) if prec == "fp32" else x
            got = H.dot(xin, precision=prec)
            tol = 2e-5 if prec == "fp32" else 1e-13
            assert np.max(np.abs(got - want)) <= tol * scale, (v, prec)
            if prec in first:
                assert np.array_equal(got, first[prec]), (v, prec)
            else:
                first[prec] = got
        # the double-float Krylov storage runs the double-float-vector kernel
        e = qs.eigsh(H, k=1, which="SA", tol=1e-12, precision="fp64df", return_eigenvectors=False)
        if v == 0:
            e_first = e
        assert abs(e[0] - e_first[0]) <= 1e-11 * abs(e_first[0]), v
