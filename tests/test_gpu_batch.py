"""Batched (lockstep) eigsh over all momentum / parity sectors against the
per-sector solver and dense diagonalisation."""
import numpy as np
import pytest

import models

pytestmark = pytest.mark.gpu


def sectors(qs, L, nup, J2):
    out = []
    order = L
    for k in range(order):
        if k in (0, order // 2):
            for p in (1, -1):
                out.append(dict(kblock=k, pblock=p))
        else:
            out.append(dict(kblock=k))
    return out


def test_batched_ground_states_all_sectors(qs, ora):
    L, nup = 14, 7
    sp = models.j1j2(L, 1.0, 0.3)
    terms = models.to_terms(qs, sp)
    syms = sectors(qs, L, nup, 0.3)
    ops = []
    dense0 = []
    for sym in syms:
        b = qs.SpinBasis1D(L, nup=nup, pauli=False, **sym)
        ops.append(qs.Hamiltonian(b, terms))
        rep = ora.RepBasis(L, nup=nup, pauli=False, **sym)
        n = rep.Ns
        H = np.zeros((n, n), dtype=np.complex128)
        e = np.zeros(n, dtype=np.complex128)
        for j in range(n):
            e[:] = 0
            e[j] = 1
            H[:, j] = rep.matvec(sp, e)
        dense0.append(np.linalg.eigvalsh(H)[:2])
    infos = []
    vals, vecs = qs.eigsh_batch(ops, k=2, tol=1e-12, return_eigenvectors=True, infos=infos)
    for i, op in enumerate(ops):
        assert np.allclose(vals[i], dense0[i], rtol=1e-10, atol=1e-10), (syms[i], vals[i], dense0[i])
        res = op.dot(vecs[i]) - vecs[i] * vals[i]
        assert np.abs(res).max() < 1e-8
        single = qs.eigsh(op, k=2, tol=1e-12, return_eigenvectors=False)
        assert np.allclose(single, vals[i], rtol=1e-10, atol=1e-10)
    # the union of sector ground energies contains the global ground energy
    full = qs.Hamiltonian(qs.SpinBasis1D(L, nup=nup, pauli=False), terms)
    e0 = qs.eigsh(full, k=1, tol=1e-12, return_eigenvectors=False)[0]
    assert abs(vals[:, 0].min() - e0) < 1e-10 * abs(e0)
