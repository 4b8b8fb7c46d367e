"""Sectors from the reference's dense nullspace intersection.

When a later symmetry generator does not map the eigenvectors of the earlier
ones onto one another (zA or zB after a one-site translation), the reference
takes the nullspace of (represented map - eigenvalue I) from an SVD
(src/symmetry_basis.jl:199-212).  The engine builds these sectors level by
level with explicit projectors and a Jacobi SVD, and runs operators on them as
P^H A P.  A nullspace basis is only fixed up to a unitary mix (the reference's
is LAPACK's), so the checks are the basis-independent ones against the
oracle's numpy restatement (oracle.DenseSector): the dimension, the projector
P P^H onto the sector, the spectrum of the projected operator, eigsh and the
time evolution of a state; plus the engine's own consistency (orthonormal
columns, argmax representatives, the product equal to P^H A P with the
engine's P).
"""
import numpy as np
import pytest
import scipy.linalg as sla

import models

pytestmark = pytest.mark.gpu

SECTORS = [
    dict(L=6, kblock=0, zAblock=1),
    dict(L=6, kblock=0, zAblock=-1),
    dict(L=8, kblock=1, zAblock=1),
    dict(L=8, kblock=2, zBblock=-1),
    dict(L=8, kblock=0, pblock=1, zAblock=1),
    dict(L=8, kblock=4, pblock=-1, zAblock=1),
    dict(L=10, kblock=3, zAblock=-1),
    dict(L=10, kblock=0, pblock=1, zBblock=1),
]


def model(L, h=0.45):
    """x_i x_{i+1} + 0.7 z_i z_{i+2} + h x_i: invariant under T, P, zA, zB."""
    nn = [(i, i % L + 1) for i in range(1, L + 1)]
    nnn = [(i, (i + 1) % L + 1) for i in range(1, L + 1)]
    return [("xx", [(1.0, i, j) for i, j in nn]), ("zz", [(0.7, i, j) for i, j in nnn]),
            ("x", [(h, i) for i in range(1, L + 1)])]


@pytest.mark.parametrize("sym", SECTORS)
def test_dense_sector_against_oracle(qs, ora, sym):
    L = sym["L"]
    kw = {k: v for k, v in sym.items() if k != "L"}
    b = qs.SpinBasis1D(L, pauli=True, **kw)
    ref = ora.DenseSector(L, **kw)
    assert b.Ns == ref.Ns
    with pytest.raises(qs.ArgumentError):
        b.orbit_minima()   # no orbit structure on this branch
    P = qs.project_from(b, np.eye(b.Ns, dtype=np.complex128), pcon=True)   # P, column by column
    assert P.shape == (2 ** L, b.Ns)
    # orthonormal columns spanning the oracle's sector
    assert np.max(np.abs(P.conj().T @ P - np.eye(b.Ns))) < 1e-12
    assert np.max(np.abs(P @ P.conj().T - ref.projector_span())) < 1e-10
    # every column is an eigenvector of every requested generator (G P = lambda P)
    for perm, lam in ref.generators():
        GP = np.zeros_like(P)
        GP[perm, :] = P
        assert np.max(np.abs(GP - lam * P)) < 1e-10
    # the states are the argmax rows of the columns (first wins)
    states = b.states
    for c in range(b.Ns):
        a = np.abs(P[:, c])
        assert states[c] == int(np.flatnonzero(a == a.max())[0]) or a[int(states[c])] >= a.max() * (1 - 1e-15)
    # the basis index of each state: the last column with that state
    last = {int(s): c for c, s in enumerate(states)}
    assert np.array_equal(b.index_array(states), np.array([last[int(s)] for s in states]))
    assert b.requires_complex == bool(np.abs(P.imag).max() > 2e-12)
    # operators: P^H A P with the parent sector's dense matrix from the oracle
    sp = model(L)
    Ap = ora.RefBasis(L, pauli=True).dense(ora.consolidate_terms(sp))
    want = P.conj().T @ Ap @ P
    for op in (qs.QuantumLinearOperator(b, models.to_terms(qs, sp)), qs.Hamiltonian(b, models.to_terms(qs, sp))):
        X = np.eye(b.Ns, dtype=np.complex128)
        got = np.stack([op.dot(X[:, c]) for c in range(b.Ns)], axis=1)
        assert np.max(np.abs(got - want)) < 1e-12 * max(1.0, np.abs(want).max())
        # transpose / adjoint
        gotT = np.stack([op.T.dot(X[:, c]) for c in range(b.Ns)], axis=1)
        assert np.max(np.abs(gotT - want.T)) < 1e-12 * max(1.0, np.abs(want).max())
    # the spectrum against the oracle's own projector
    wref = np.linalg.eigvalsh(ref.P.conj().T @ Ap @ ref.P)
    w = np.linalg.eigvalsh(want)
    assert np.max(np.abs(w - wref)) < 1e-10 * max(1.0, np.abs(wref).max())
    H = qs.Hamiltonian(b, models.to_terms(qs, sp))
    k = min(2, b.Ns - 2) if b.Ns > 3 else 1
    e = qs.eigsh(H, k=k, which="SA", tol=1e-12, return_eigenvectors=False)
    assert np.max(np.abs(np.sort(e) - wref[:k])) < 1e-10 * max(1.0, np.abs(wref).max())
    # evolution: P psi(t) = exp(-i t A) P psi(0) in the parent sector
    psi = models.seeded(b.Ns, seed=9, complex_=True)
    psi /= np.linalg.norm(psi)
    st = qs.evolve(H, psi, 0.0, [0.7], tol=1e-12)
    lifted = P @ st[:, 0]
    exact = sla.expm(-1j * 0.7 * Ap) @ (P @ psi)
    assert np.linalg.norm(lifted - exact) < 1e-9


def test_dense_sector_unsupported_paths(qs):
    from qsgpu import _lib
    b = qs.SpinBasis1D(8, pauli=True, kblock=1, zAblock=1)
    H = qs.Hamiltonian(b, models.to_terms(qs, model(8)))
    x = models.seeded(b.Ns, complex_=True)
    with pytest.raises(qs.ArgumentError):
        b.stabilizers()
    lib = _lib.load()
    y = np.zeros(b.Ns, dtype=np.complex128)
    a = np.array([1.0, 0.0])
    z = np.array([0.0, 0.0])
    st = lib.qs_op_matvec_noalloc(H._h, 0, _lib.ptr(a), _lib.ptr(x), _lib.QS_C128, _lib.ptr(z), _lib.ptr(y),
                                  _lib.QS_C128, 1)
    assert st == 6
    with pytest.raises(qs.ArgumentError):
        qs.eigsh_batch([H], k=1)


def test_general_maps_take_the_same_branch(qs, ora):
    """SpinBasisGeneral with the translation and sublattice-flip maps of a 1D
    dense-nullspace sector gives the same sector (P P^H), through the same
    level-by-level construction."""
    L = 8
    T = [(i % L) + 1 for i in range(1, L + 1)]
    # zero-based map (a negative entry -(t + 1) sends the site to t and flips it):
    # the odd sites 1, 3, ... (one-based) flipped in place
    zA = [-(i + 1) if i % 2 == 0 else i for i in range(L)]
    g = qs.SpinBasisGeneral(L, pauli=True, block_order=["T", "zA"], T=(T, 1), zA=(zA, 0))
    b = qs.SpinBasis1D(L, pauli=True, kblock=1, zAblock=1)
    assert g.Ns == b.Ns
    Pg = qs.project_from(g, np.eye(g.Ns, dtype=np.complex128), pcon=True)
    Pb = qs.project_from(b, np.eye(b.Ns, dtype=np.complex128), pcon=True)
    assert np.max(np.abs(Pg @ Pg.conj().T - Pb @ Pb.conj().T)) < 1e-10
    ref = ora.DenseSector(L, kblock=1, zAblock=1)
    assert np.max(np.abs(Pg @ Pg.conj().T - ref.projector_span())) < 1e-10
