"""Pins the oracle's numpy restatement of the reference's level-by-level
intersection (oracle.DenseSector), which checks the engine's dense-nullspace
sectors:

* on sectors where every intersection is permutation-like it must span the
  same space as the C restatement (oracle.RefBasis, itself pinned to the
  reference's vectors): P P^H equal and the same dimension;
* on the dense branch its columns must be orthonormal eigenvectors of every
  requested generator with the requested eigenvalue (G P = lambda P, the
  defining property of the intersection), and the sector must be all of that
  intersection: its dimension equals the nullity of the stacked
  (G_i - lambda_i I), computed independently from the maps."""
import numpy as np
import pytest


def _maps(L, a=1):
    full = (1 << L) - 1
    odd = sum(1 << (s - 1) for s in range(1, L + 1, 2))
    even = sum(1 << (s - 1) for s in range(2, L + 1, 2))

    def perm_map(perm):
        def f(s):
            t = 0
            for site in range(1, L + 1):
                if s >> (site - 1) & 1:
                    t |= 1 << (perm[site - 1] - 1)
            return t
        return f

    trans = perm_map([(site + a - 1) % L + 1 for site in range(1, L + 1)])
    par = perm_map([L - site + 1 for site in range(1, L + 1)])
    return {"T": trans, "P": par, "Z": lambda s: s ^ full, "zA": lambda s: s ^ odd, "zB": lambda s: s ^ even}


@pytest.mark.parametrize("L,nup,sym", [
    (10, 5, dict(kblock=0, pblock=1, zblock=1)),
    (10, 5, dict(kblock=3)),
    (9, None, dict(kblock=2)),
    (8, None, dict(kblock=0, pblock=-1, zblock=1)),
    (8, None, dict(zAblock=1, zBblock=-1)),
])
def test_dense_restatement_matches_c_oracle(ora, L, nup, sym):
    d = ora.DenseSector(L, nup=nup, **sym)
    r = ora.RefBasis(L, nup=nup, pauli=True, **sym)
    assert d.Ns == r.Ns
    Pr = r.projector().toarray()
    assert np.max(np.abs(d.projector_span() - Pr @ Pr.conj().T)) < 1e-12


@pytest.mark.parametrize("L,sym", [
    (6, dict(kblock=0, zAblock=1)),
    (8, dict(kblock=1, zAblock=1)),
    (8, dict(kblock=2, zBblock=-1)),
    (8, dict(kblock=0, pblock=1, zAblock=1)),
    (10, dict(kblock=3, zAblock=-1)),
])
def test_dense_branch_is_the_intersection(ora, L, sym):
    d = ora.DenseSector(L, **sym)
    P = d.P
    st = d.parent_states
    idx = {int(s): i for i, s in enumerate(st)}
    assert np.max(np.abs(P.conj().T @ P - np.eye(d.Ns))) < 1e-12
    maps = _maps(L)
    gens = []
    if "kblock" in sym:
        k = sym["kblock"] % L
        gens.append((maps["T"], np.exp(2j * np.pi * k / L)))
    for name, key in (("pblock", "P"), ("zblock", "Z"), ("zAblock", "zA"), ("zBblock", "zB")):
        if name in sym:
            gens.append((maps[key], float(sym[name])))
    for f, lam in gens:
        perm = np.array([idx[f(int(s))] for s in st])
        GP = np.zeros_like(P)
        GP[perm, :] = P                       # (G P)[f(s)] = P[s]
        assert np.max(np.abs(GP - lam * P)) < 1e-10
    # the whole intersection: its dimension is the nullity of the stacked
    # (G_i - lambda_i I), from dense matrices
    n = len(st)
    rows = []
    for f, lam in gens:
        G = np.zeros((n, n), complex)
        G[[idx[f(int(s))] for s in st], np.arange(n)] = 1
        rows.append(G - lam * np.eye(n))
    sv = np.linalg.svd(np.vstack(rows), compute_uv=False)
    assert int(np.sum(sv <= 1e-9)) == d.Ns
