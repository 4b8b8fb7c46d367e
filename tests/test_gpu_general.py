"""SpinBasisGeneral on the device (general site maps: 2D lattices) against
the oracle running the reference's projector algorithm over the same maps
(src/basis.jl:455-600, src/symmetry_basis.jl:57-213)."""
import numpy as np
import pytest
import scipy.linalg as sla

import models

pytestmark = pytest.mark.gpu

SECTORS_4x3 = [
    dict(tx=0, ty=0, z=0),
    dict(tx=1, ty=0, z=1),
    dict(tx=2, ty=1, z=0),
    dict(tx=3, ty=2, z=1),
    dict(tx=0, ty=0, px=0, z=0),
    dict(tx=2, ty=1, px=1, z=1),
]


def blocks_for(maps, q):
    Tx, Ty, Px, Z = maps
    out = [("Tx", Tx, q["tx"]), ("Ty", Ty, q["ty"])]
    if "px" in q:
        out.append(("Px", Px, q["px"]))
    out.append(("Z", Z, q["z"]))
    return out


def make_pair(qs, ora, Lx, Ly, nup, q):
    maps = models.torus_maps(Lx, Ly)
    blk = blocks_for(maps, q)
    b = qs.SpinBasisGeneral(Lx * Ly, nup=nup, pauli=False, **{n: (m, v) for n, m, v in blk})
    rb = ora.general_basis(Lx * Ly, nup=nup, pauli=False, blocks=[(m, v) for _, m, v in blk])
    return b, rb


@pytest.mark.parametrize("q", SECTORS_4x3)
def test_general_sector_matches_reference_algorithm(qs, ora, q):
    Lx, Ly, nup = 4, 3, 6
    b, rb = make_pair(qs, ora, Lx, Ly, nup, q)
    assert b.Ns == rb.Ns
    P = rb.projector().tocsc()
    P.sort_indices()
    mins = np.array([rb.parent_states[P.indices[P.indptr[j]]] for j in range(P.shape[1])], dtype=np.uint64)
    # the replayed projector gives the reference's own (argmax) representatives
    assert np.array_equal(qs.states(b), rb.states)
    assert np.array_equal(b.orbit_minima(), mins)
    spec = models.torus_heisenberg(Lx, Ly, 1.0, 0.35)
    H = qs.Hamiltonian(b, models.to_terms(qs, spec))
    D = rb.dense(ora.consolidate_terms(spec))
    assert np.abs(H.toarray() - D).max() < 1e-13
    x = models.seeded(b.Ns, complex_=True)
    assert np.abs(H.dot(x) - D @ x).max() < 1e-12
    # the projector: P c into the full 2^L space and back
    full = np.zeros(((1 << (Lx * Ly)), b.Ns), dtype=np.complex128)
    full[rb.parent_states.astype(np.int64)] = P.toarray()
    got = qs.project_from(b, x)
    assert np.abs(got - full @ x).max() < 1e-13
    assert np.array_equal(qs.project_from(b, x, pcon=True), exact_from(P, x))   # bit for bit
    psi = models.seeded(1 << (Lx * Ly), seed=4, complex_=True)
    assert np.abs(qs.project_to(b, psi) - full.conj().T @ psi).max() < 1e-12
    # get_amp / representative of every parent state of the sector
    Pr = P.tocsr()
    for s in rb.parent_states[::37]:
        row = int(np.searchsorted(rb.parent_states, s))
        cols = Pr.indices[Pr.indptr[row]:Pr.indptr[row + 1]]
        if len(cols) == 0:
            continue
        amp = qs.get_amp(b, int(s))
        assert amp == Pr[row, cols[0]]
        assert qs.representative(b, int(s)) == int(rb.states[cols[0]])
    # eigenpairs against the dense sector matrix
    w = np.linalg.eigvalsh(D)
    vals = qs.eigsh(H, k=2, tol=1e-12, return_eigenvectors=False)
    assert np.allclose(vals, w[:2], rtol=1e-10, atol=1e-10)


def exact_from(P, v):
    """P v with separately rounded products (parent-sector rows)."""
    Pc = P.tocoo()
    c = v[Pc.col]
    re = np.subtract(np.multiply(Pc.data.real, c.real), np.multiply(Pc.data.imag, c.imag))
    im = np.add(np.multiply(Pc.data.real, c.imag), np.multiply(Pc.data.imag, c.real))
    out = np.zeros(P.shape[0], dtype=np.complex128)
    out[Pc.row] = re + 1j * im
    return out


def test_general_without_replay(qs, ora):
    """Blocks whose later generators' orders multiply past 32 (the replay's
    tree): the columns, the sector matrix and the projector still match the
    reference algorithm (columns labelled by their orbit minima)."""
    Lx, Ly, nup = 4, 3, 6
    Tx, Ty, Px, Z = models.torus_maps(Lx, Ly)
    Py = [(i % Lx) + Lx * ((Ly - 1 - i // Lx) % Ly) for i in range(Lx * Ly)]
    blk = [("Z", Z, 0), ("Tx", Tx, 0), ("Ty", Ty, 0), ("Px", Px, 0), ("Py", Py, 0)]
    b = qs.SpinBasisGeneral(12, nup=nup, pauli=False, block_order=[n for n, _, _ in blk],
                            **{n: (m, q) for n, m, q in blk})
    rb = ora.general_basis(12, nup=nup, pauli=False, blocks=[(m, q) for _, m, q in blk])
    assert b.Ns == rb.Ns
    P = rb.projector().tocsc()
    P.sort_indices()
    mins = np.array([rb.parent_states[P.indices[P.indptr[j]]] for j in range(P.shape[1])], dtype=np.uint64)
    assert np.array_equal(qs.states(b), mins)
    spec = models.torus_heisenberg(Lx, Ly, 1.0, 0.35)
    H = qs.Hamiltonian(b, models.to_terms(qs, spec))
    D = rb.dense(ora.consolidate_terms(spec))
    assert np.abs(H.toarray() - D).max() < 1e-13
    x = models.seeded(b.Ns, complex_=True)
    assert np.abs(qs.project_from(b, x, pcon=True) - P @ x).max() < 1e-13
    psi = models.seeded(rb.n_parent, seed=2, complex_=True)
    assert np.abs(qs.project_to(b, psi, pcon=True) - P.conj().T @ psi).max() < 1e-12


def test_general_sectors_cover_the_full_spectrum(qs, ora):
    """The (kx, ky) sectors of the 4 x 3 torus at nup = 6 hold every eigenvalue
    of the unreduced sector, with multiplicity; their ground energies batch."""
    Lx, Ly, nup = 4, 3, 6
    spec = models.torus_heisenberg(Lx, Ly, 1.0, 0.35)
    terms = models.to_terms(qs, spec)
    Tx, Ty, _, _ = models.torus_maps(Lx, Ly)
    allw, ops = [], []
    for qx in range(Lx):
        for qy in range(Ly):
            b = qs.SpinBasisGeneral(Lx * Ly, nup=nup, pauli=False, Tx=(Tx, qx), Ty=(Ty, qy))
            H = qs.Hamiltonian(b, terms)
            allw.append(np.linalg.eigvalsh(H.toarray()))
            ops.append(H)
    allw = np.sort(np.concatenate(allw))
    full = ora.RefBasis(Lx * Ly, nup=nup, pauli=False)
    wf = np.linalg.eigvalsh(full.dense(ora.consolidate_terms(spec)))
    assert allw.size == wf.size and np.abs(allw - wf).max() < 1e-11
    vals = qs.eigsh_batch(ops, k=1, tol=1e-12)
    assert abs(vals[:, 0].min() - wf[0]) < 1e-10


def test_general_4x4_evolution(qs, ora):
    """4 x 4 torus, nup = 8, k = (0, 0), reflection and flip even: evolution
    against the dense sector exponential."""
    Lx = Ly = 4
    Tx, Ty, Px, Z = models.torus_maps(Lx, Ly)
    blocks = [(Tx, 0), (Ty, 0), (Px, 0), (Z, 0)]
    b = qs.SpinBasisGeneral(16, nup=8, pauli=False, Tx=blocks[0], Ty=blocks[1], Px=blocks[2], Z=blocks[3])
    rb = ora.general_basis(16, nup=8, pauli=False, blocks=blocks)
    assert b.Ns == rb.Ns
    spec = models.torus_heisenberg(Lx, Ly)
    H = qs.Hamiltonian(b, models.to_terms(qs, spec))
    D = rb.dense(ora.consolidate_terms(spec))
    v0 = models.seeded(b.Ns, seed=3, complex_=True)
    got = qs.evolve(H, v0, 0.0, [0.5, 2.0], tol=1e-12)
    for i, t in enumerate((0.5, 2.0)):
        assert np.linalg.norm(got[:, i] - sla.expm(-1j * t * D) @ v0) < 1e-10 * np.linalg.norm(v0)
    assert abs(qs.eigsh(H, k=1, tol=1e-12, return_eigenvectors=False)[0] - np.linalg.eigvalsh(D)[0]) < 1e-10


def test_general_argument_errors(qs):
    Tx, Ty, Px, Z = models.torus_maps(4, 3)
    with pytest.raises(qs.ArgumentError):
        qs.SpinBasisGeneral(12, nup=6, Tx=([0] * 12, 0))                  # not a permutation
    with pytest.raises(qs.ArgumentError):
        qs.SpinBasisGeneral(12, nup=5, Z=(Z, 0))                          # the flip leaves nup = 5
    with pytest.raises(qs.ArgumentError):
        qs.SpinBasisGeneral(12, nup=6, block_order=["Ty"], Tx=(Tx, 0))    # unknown block name
    with pytest.raises(qs.ArgumentError):
        qs.SpinBasisGeneral(12, nup=6, Tx=(Tx[:5], 0))                    # wrong length
    # a non-commuting term set is rejected by the symmetry check
    b = qs.SpinBasisGeneral(12, nup=6, pauli=False, Tx=(Tx, 1))
    with pytest.raises(qs.ArgumentError):
        qs.Hamiltonian(b, [qs.OperatorTerm("zz", [(1.0, 1, 2)])])


def test_general_wide_states(qs, ora):
    """L = 34 > 32 (64-bit states): a 17 x 2 torus at nup = 3 against the
    oracle: sizes, representatives, the sector matrix and the ground state."""
    Lx, Ly, nup = 17, 2, 3
    Tx, Ty, Px, Z = models.torus_maps(Lx, Ly)
    for qx, qy in ((0, 0), (3, 1)):
        b = qs.SpinBasisGeneral(Lx * Ly, nup=nup, pauli=False, Tx=(Tx, qx), Ty=(Ty, qy))
        rb = ora.general_basis(Lx * Ly, nup=nup, pauli=False, blocks=[(Tx, qx), (Ty, qy)])
        assert b.Ns == rb.Ns
        assert np.array_equal(qs.states(b), rb.states)
        spec = models.torus_heisenberg(Lx, Ly, 1.0, 0.2)
        H = qs.Hamiltonian(b, models.to_terms(qs, spec))
        D = rb.dense(ora.consolidate_terms(spec))
        assert np.abs(H.toarray() - D).max() < 1e-13
        e0 = qs.eigsh(H, k=1, tol=1e-12, return_eigenvectors=False)[0]
        assert abs(e0 - np.linalg.eigvalsh(D)[0]) < 1e-10
