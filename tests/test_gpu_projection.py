"""project_from / project_to on the device against the oracle's restatement
of the reference projector (src/symmetry_basis.jl:366-501): bit for bit,
with every product and sum rounded separately as Julia's sparse products do."""
import numpy as np
import pytest

import models

pytestmark = pytest.mark.gpu

SECTORS = [
    (12, 6, dict(kblock=0, pblock=1)),
    (12, 6, dict(kblock=3)),
    (12, 6, dict(kblock=6, pblock=-1, zblock=1)),
    (12, 5, dict(kblock=2)),
    (12, 6, dict(pzblock=-1)),
    (10, None, dict(zblock=1)),
    (10, None, dict(kblock=4)),
    (12, 6, dict()),
]


def exact_from(P, rows, v, nrows):
    """out[rows[r]] = P[r, j] v[j] for the single nonzero of parent row r,
    (vr cr - vi ci, vr ci + vi cr) with separate roundings."""
    Pc = P.tocoo()
    vr, vi = Pc.data.real, Pc.data.imag
    c = v[Pc.col]
    re = np.subtract(np.multiply(vr, c.real), np.multiply(vi, c.imag))
    im = np.add(np.multiply(vr, c.imag), np.multiply(vi, c.real))
    out = np.zeros(nrows, dtype=np.complex128)
    out[rows[Pc.row]] = re + 1j * im
    return out


def exact_to(P, rows, x):
    """c_j = sum over column j's entries (ascending state) of conj(P) x, summed in order."""
    Pc = P.tocsc()
    Pc.sort_indices()
    n = Pc.shape[1]
    start, cnt = Pc.indptr[:-1], np.diff(Pc.indptr)
    ar, ai = np.zeros(n), np.zeros(n)
    for k in range(int(cnt.max())):
        sel = np.nonzero(cnt > k)[0]
        e = start[sel] + k
        vr, vi = Pc.data[e].real, -Pc.data[e].imag
        xv = x[rows[Pc.indices[e]]]
        ar[sel] = np.add(ar[sel], np.subtract(np.multiply(vr, xv.real), np.multiply(vi, xv.imag)))
        ai[sel] = np.add(ai[sel], np.add(np.multiply(vr, xv.imag), np.multiply(vi, xv.real)))
    return ar + 1j * ai


@pytest.mark.parametrize("L,nup,sym", SECTORS)
def test_projection_bitwise(qs, ora, L, nup, sym):
    b = qs.SpinBasis1D(L, nup=nup, pauli=False, **sym)
    rb = ora.RefBasis(L, nup=nup, pauli=False, **sym)
    assert b.Ns == rb.Ns
    P = rb.projector()
    rng = np.random.default_rng(L * 100 + b.Ns)
    c = rng.standard_normal(b.Ns) + 1j * rng.standard_normal(b.Ns)
    for pcon in (False, True):
        rows = np.arange(rb.n_parent) if pcon else rb.parent_states.astype(np.int64)
        nrows = rb.n_parent if pcon else 1 << L
        got = qs.project_from(b, c, pcon=pcon)
        assert got.shape == (nrows,)
        assert np.array_equal(got, exact_from(P, rows, c, nrows)), pcon
        psi = rng.standard_normal(nrows) + 1j * rng.standard_normal(nrows)
        back = qs.project_to(b, psi, pcon=pcon)
        assert np.array_equal(back, exact_to(P, rows, psi)), pcon
        # P^H P = I on the sector
        assert np.abs(qs.project_to(b, got, pcon=pcon) - c).max() < 1e-13
        assert np.array_equal(qs.get_vec(b, c, pcon=pcon), got)


def test_projection_matrix_columns_and_errors(qs):
    b = qs.SpinBasis1D(8, nup=4, pauli=False, kblock=1)
    with pytest.raises(qs.ArgumentError):
        qs.project_from(b, np.ones(b.Ns))          # a complex sector needs a complex vector
    with pytest.raises(qs.DimensionMismatch):
        qs.project_from(b, np.ones(b.Ns + 1, dtype=complex))
    with pytest.raises(qs.DimensionMismatch):
        qs.project_to(b, np.ones(5, dtype=complex))
    # matrix input: column by column
    C = models.seeded(b.Ns * 3, complex_=True).reshape(b.Ns, 3)
    M = qs.project_from(b, C)
    for j in range(3):
        assert np.array_equal(M[:, j], qs.project_from(b, np.ascontiguousarray(C[:, j])))
    # a real sector keeps real vectors real
    r = qs.SpinBasis1D(8, nup=4, pauli=False, kblock=0, pblock=1)
    out = qs.project_from(r, np.ones(r.Ns))
    assert out.dtype == np.float64 and abs(np.linalg.norm(out) - np.sqrt(r.Ns)) < 1e-12
    sp = qs.project_from(r, np.ones(r.Ns), sparse=True)
    assert sp.shape == (1 << 8, 1) and np.allclose(sp.toarray()[:, 0], out)
