"""tocsc / tocsr / toarray of a Hamiltonian from the device's assembled form
against the oracle's dense restatement of the reference's H.data
(src/operators.jl:461-576) and the reference's XXZ spectrum."""
import numpy as np
import pytest
import scipy.sparse as sp

import models

pytestmark = pytest.mark.gpu

CASES = [
    (12, 6, dict(kblock=0, pblock=1), "j1j2"),
    (12, 6, dict(kblock=5), "j1j2"),
    (12, 6, dict(kblock=6, pblock=-1, zblock=1), "j1j2"),
    (10, 5, dict(), "xxz"),
    (10, None, dict(kblock=3, pblock=None), "tfim"),
    (10, None, dict(kblock=0, zblock=1), "xyz"),
]


def spec_for(name, L):
    return {"j1j2": lambda: models.j1j2(L, 1.0, 0.4), "xxz": lambda: models.xxz(L, 1.0, 0.6),
            "tfim": lambda: models.tfim(L, 1.0, 0.7), "xyz": lambda: models.xyz_field(L)}[name]()


@pytest.mark.parametrize("L,nup,sym,name", CASES)
def test_export_matches_dense(qs, ora, L, nup, sym, name):
    sym = {k: v for k, v in sym.items() if v is not None}
    spec = spec_for(name, L)
    if name == "xyz":
        spec = [t for t in spec if len(t[0]) == 2]   # single-site fields break the spin-flip symmetry
    H = qs.Hamiltonian(qs.SpinBasis1D(L, nup=nup, pauli=False, **sym), models.to_terms(qs, spec))
    rb = ora.RefBasis(L, nup=nup, pauli=False, **sym)
    D = rb.dense(ora.consolidate_terms(spec))
    A = H.toarray()
    assert A.dtype == (np.complex128 if H.dtype == np.complex128 else np.float64)
    assert np.abs(A - D).max() < 1e-13 * max(1.0, np.abs(D).max())
    # the same numerical nonzeros
    assert np.array_equal(np.abs(A) > 1e-12, np.abs(D) > 1e-12)
    C = qs.tocsc(H)
    assert isinstance(C, sp.csc_matrix) and np.abs(C.toarray() - A).max() == 0
    R = qs.tocsr(H)
    assert isinstance(R, sp.csr_matrix) and np.abs(R.toarray() - A).max() == 0
    x = models.seeded(H.Ns, complex_=True)
    assert np.abs(C @ x - H.dot(x)).max() < 1e-12 * np.abs(x).sum() / np.sqrt(H.Ns)
    out = np.empty_like(A)
    assert qs.toarray(H, out=out) is out and np.array_equal(out, A)


def test_export_reference_xxz_spectrum(qs, kats):
    k = kats["xxz_L4_spectrum"]
    jxy = np.sqrt(2.0)
    t = k["terms"]
    terms = [qs.OperatorTerm("+-", [(jxy / 2, a, b) for a, b in t[0][2]]),
             qs.OperatorTerm("-+", [(jxy / 2, a, b) for a, b in t[1][2]]),
             qs.OperatorTerm("zz", [(1.0, a, b) for a, b in t[2][2]]),
             qs.OperatorTerm("z", [(1 / np.sqrt(3.0), s[0]) for s in t[3][2]])]
    H = qs.Hamiltonian(qs.SpinBasis1D(k["L"], nup=k["nup"], pauli=k["pauli"]), terms)
    A = H.toarray()
    assert np.allclose(np.linalg.eigvalsh(A), k["eigenvalues"], atol=k["atol"], rtol=k["atol"])
    assert abs(np.trace(A) - k["trace"]) < k["atol"]
    assert abs(np.linalg.norm(A) - k["frobenius"]) < k["atol"]
