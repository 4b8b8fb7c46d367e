"""tools.jl's block tools on the device (block_diag_hamiltonian, BlockOps,
evolve on BlockOps, block_expm) against the reference's known answers and
dense FP64 evolution of the full space from the oracle."""
import numpy as np
import pytest
import scipy.linalg as sla

import models

pytestmark = pytest.mark.gpu


def kat_setup(qs, k):
    terms = [qs.OperatorTerm(op, [tuple(c) for c in cs]) for op, cs in k["terms"]]
    blocks = [{"nup": n} for n in k["blocks_nup"]]
    psi = np.array(k["psi_unnormalized"], dtype=np.complex128)
    return terms, blocks, psi / np.linalg.norm(psi)


def test_reference_block_tools(qs, kats):
    """test/runtests.jl:277-325."""
    k = kats["block_tools_L2"]
    terms, blocks, psi = kat_setup(qs, k)
    P, block_H = qs.block_diag_hamiltonian(blocks, terms, [], qs.SpinBasis1D, (k["L"],), np.complex128,
                                           basis_kwargs={"pauli": k["pauli"]})
    full_H = qs.Hamiltonian(qs.SpinBasis1D(k["L"], pauli=k["pauli"]), terms)
    Pm = P.toarray()
    Hf = np.column_stack([full_H.dot(np.eye(4)[:, j].astype(complex)) for j in range(4)])
    assert np.allclose(Pm.conj().T @ Pm, np.eye(4))
    assert np.allclose(block_H.toarray(), Pm.conj().T @ Hf @ Pm)
    assert np.allclose(qs.block_diag_hamiltonian(blocks, terms, [], qs.SpinBasis1D, (k["L"],), np.complex128,
                                                 basis_kwargs={"pauli": k["pauli"]}, get_proj=False).toarray(),
                       block_H.toarray())
    ops = qs.BlockOps(blocks, terms, [], qs.SpinBasis1D, (k["L"],), np.complex128, basis_kwargs={"pauli": k["pauli"]})
    assert len(ops.basis_dict) == 3 and not ops.H_dict
    ops.compute_all_blocks()
    assert len(ops.H_dict) == 3 and len(ops.P_dict) == 3
    times = k["times"]
    got = qs.evolve(ops, psi, 0.0, times)
    want = qs.evolve(full_H, psi, 0.0, times)
    assert np.allclose(got, want, atol=k["evolve_atol"], rtol=0)
    U = sla.expm(-1j * Hf)
    assert np.allclose(qs.block_expm(ops, psi), U @ psi, atol=k["expm_atol"], rtol=0)
    g = k["grid"]
    grid = qs.block_expm(ops, psi, start=g["start"], stop=g["stop"], num=g["num"])
    assert grid.shape == (4, g["num"])
    assert np.allclose(grid[:, 0], psi, atol=k["grid_first_atol"], rtol=0)
    assert np.allclose(grid[:, -1], U @ psi, atol=k["grid_last_atol"], rtol=0)


def dense_full(ora, L, spec):
    rb = ora.RefBasis(L, pauli=False)
    return rb.dense(ora.consolidate_terms(spec))


def test_momentum_blocks_match_dense_full_space(qs, ora):
    """Every (nup, k) sector of an XXZ chain with a field: the blocks cover the
    full 2^L space, so the block evolution equals the dense full evolution."""
    L = 10
    spec = models.xxz(L, 1.0, 0.7) + [("z", [(0.15, i) for i in range(1, L + 1)])]
    terms = models.to_terms(qs, spec)
    blocks = [{"nup": n, "kblock": kb} for n in range(L + 1) for kb in range(L)]
    ops = qs.BlockOps(blocks, terms, [], qs.SpinBasis1D, (L,), np.complex128, basis_kwargs={"pauli": False})
    assert sum(b.Ns for b in ops.basis_dict.values()) == 1 << L
    Hf = dense_full(ora, L, spec)
    w, V = np.linalg.eigh(Hf)
    psi = models.seeded(1 << L, seed=5, complex_=True)
    psi /= np.linalg.norm(psi)
    times = [0.0, 0.4, 1.3, 3.0]
    got = qs.evolve(ops, psi, 0.1, times, tol=1e-12)
    for i, t in enumerate(times):
        want = V @ (np.exp(-1j * (t - 0.1) * w) * (V.conj().T @ psi))
        assert np.linalg.norm(got[:, i] - want) < 1e-10, t
    # imaginary time, and a scalar time gives a vector
    got_im = qs.evolve(ops, psi, 0.0, 0.5, imag_time=True)
    want_im = V @ (np.exp(-0.5 * w) * (V.conj().T @ psi))
    assert got_im.shape == (1 << L,) and np.linalg.norm(got_im - want_im) < 1e-10 * np.linalg.norm(want_im)
    # block_expm with a shift and an open grid
    grid = qs.block_expm(ops, psi, a=-0.5j, start=0.0, stop=2.0, num=4, endpoint=False, shift=0.3)
    for i, s in enumerate(np.linspace(0.0, 2.0, 5)[:-1]):
        want = V @ (np.exp(-0.5j * s * (w + 0.3)) * (V.conj().T @ psi))
        assert np.linalg.norm(grid[:, i] - want) < 1e-10
    states = list(qs.block_expm(ops, psi, a=-0.5j, start=0.0, stop=2.0, num=4, endpoint=False, shift=0.3,
                                iterate=True))
    assert len(states) == 4 and np.array_equal(states[2], grid[:, 2])


def test_blocks_with_projection_only_on_some(qs, ora):
    """A state in one nup sector only touches that sector's momentum blocks;
    a state with no weight on the blocks is an ArgumentError."""
    L = 12
    spec = models.j1j2(L, 1.0, 0.4)
    terms = models.to_terms(qs, spec)
    blocks = [{"kblock": kb} for kb in range(L)]
    ops = qs.BlockOps(blocks, terms, [], qs.SpinBasis1D, (L,), np.complex128,
                      basis_kwargs={"pauli": False, "nup": 6})
    full = qs.SpinBasis1D(L, nup=6, pauli=False)
    Hs = qs.Hamiltonian(full, terms)
    psi_sector = models.seeded(full.Ns, seed=9, complex_=True)
    psi = qs.project_from(full, psi_sector)               # embedded in the 2^L space
    got = qs.evolve(ops, psi, 0.0, [0.7, 2.0])
    want = qs.evolve(Hs, psi_sector, 0.0, [0.7, 2.0])
    for i in range(2):
        assert np.linalg.norm(qs.project_to(full, got[:, i]) - want[:, i]) < 1e-10 * np.linalg.norm(want[:, i])
    outside = np.zeros(1 << L, dtype=np.complex128)
    outside[0] = 1.0                                      # nup = 0: no block holds it
    with pytest.raises(qs.ArgumentError):
        qs.evolve(ops, outside, 0.0, [1.0])
    with pytest.raises(qs.ArgumentError):
        qs.BlockOps(blocks, terms, [("zz", [(1.0, 1, 2)], None, ())], qs.SpinBasis1D, (L,), np.complex128)
