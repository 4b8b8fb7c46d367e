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


@pytest.mark.parametrize("precision", ["fp64", "fp64df", "fp32"])
def test_batched_ground_states_all_sectors(qs, ora, precision):
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
    vals, vecs = qs.eigsh_batch(ops, k=2, tol=1e-12, return_eigenvectors=True, infos=infos, precision=precision)
    assert all(i["nconv"] >= 2 for i in infos)
    # the FP32 form polishes the eigenvalues to FP64 accuracy (Rayleigh quotient
    # with the FP64 product); its vectors keep FP32-level residuals
    res_tol = 1e-6 if precision == "fp32" else 1e-8
    for i, op in enumerate(ops):
        assert np.allclose(vals[i], dense0[i], rtol=1e-10, atol=1e-10), (syms[i], vals[i], dense0[i])
        res = op.dot(vecs[i]) - vecs[i] * vals[i]
        assert np.abs(res).max() < res_tol
        single = qs.eigsh(op, k=2, tol=1e-12, return_eigenvectors=False)
        assert np.allclose(single, vals[i], rtol=1e-10, atol=1e-10)
    # the union of sector ground energies contains the global ground energy
    full = qs.Hamiltonian(qs.SpinBasis1D(L, nup=nup, pauli=False), terms)
    e0 = qs.eigsh(full, k=1, tol=1e-12, return_eigenvectors=False)[0]
    assert abs(vals[:, 0].min() - e0) < 1e-10 * abs(e0)


def test_batched_result_independent_of_batch(qs):
    """A sector's eigenpairs are the same solved alone and inside a batch: each
    slot's arithmetic and reductions depend only on its own operator."""
    L, nup = 16, 8
    terms = models.to_terms(qs, models.j1j2(L, 1.0, 0.5))
    syms = [dict(kblock=0, pblock=1), dict(kblock=3), dict(kblock=8, pblock=-1), dict(kblock=5)]
    ops = [qs.Hamiltonian(qs.SpinBasis1D(L, nup=nup, pauli=False, **s), terms) for s in syms]
    for precision in ("fp64", "fp64df"):
        together, vt = qs.eigsh_batch(ops, k=1, tol=1e-12, return_eigenvectors=True, precision=precision)
        for i, op in enumerate(ops):
            alone, va = qs.eigsh_batch([op], k=1, tol=1e-12, return_eigenvectors=True, precision=precision)
            assert together[i, 0] == alone[0, 0], (precision, i)
            assert np.array_equal(vt[i], va[0]), (precision, i)


def test_batched_cluster_beside_graph_replay(qs):
    """A batch holding small slots (cluster step, eight and sixteen CTAs) and a
    large one (graph replay) runs the two concurrently on two streams; every
    sector's eigenpairs are the ones it has alone."""
    terms = lambda L: models.to_terms(qs, models.j1j2(L, 1.0, 0.41))
    specs = [(24, dict(kblock=0, pblock=1)), (16, dict(kblock=3)), (20, dict(kblock=3)),
             (16, dict(kblock=0, pblock=-1))]
    ops = [qs.Hamiltonian(qs.SpinBasis1D(L, nup=L // 2, pauli=False, **s), terms(L)) for L, s in specs]
    assert ops[0].Ns > 32768 and 8192 < ops[2].Ns <= 32768 and ops[1].Ns <= 8192
    for precision in ("fp64", "fp32"):
        together, vt = qs.eigsh_batch(ops, k=2, tol=1e-12, return_eigenvectors=True, precision=precision)
        for i, op in enumerate(ops):
            alone, va = qs.eigsh_batch([op], k=2, tol=1e-12, return_eigenvectors=True, precision=precision)
            assert np.array_equal(together[i], alone[0]), (precision, i)
            assert np.array_equal(vt[i], va[0]), (precision, i)


def test_batched_mixed_real_and_complex_sizes(qs, ora):
    """Sectors of very different sizes, real and complex, with k=3."""
    L = 12
    sp = models.xxz(L, 1.0, 0.5)
    terms = models.to_terms(qs, sp)
    syms = [(6, dict()), (6, dict(kblock=1)), (4, dict(kblock=0)),
            (5, dict(kblock=2))]
    ops, dense = [], []
    for nup, sym in syms:
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
        dense.append(np.linalg.eigvalsh(H)[:3])
    for precision in ("fp64", "fp64df", "fp32"):
        vals, vecs = qs.eigsh_batch(ops, k=3, tol=1e-12, return_eigenvectors=True, precision=precision)
        for i, op in enumerate(ops):
            assert np.allclose(vals[i], dense[i], rtol=1e-10, atol=1e-10), (precision, i)
            res_tol = 1e-6 if precision == "fp32" else 1e-8
            assert np.abs(op.dot(vecs[i]) - vecs[i] * vals[i]).max() < res_tol


def test_results_repeat_across_processes(qs):
    """Two processes (each timing its own SpMV tiles) give the same bits: the
    reductions' order is fixed by the BLAS row block, not by the tuner."""
    import json
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = (
        "import json, sys; sys.path.insert(0, 'quspin.jl_gb300'); sys.path.insert(0, 'tests');"
        "import qsgpu as qs, models;"
        "L = 20; terms = models.to_terms(qs, models.j1j2(L, 1.0, 0.3));"
        "ops = [qs.Hamiltonian(qs.SpinBasis1D(L, nup=10, pauli=False, kblock=k), terms) for k in (1, 2, 3)];"
        "out = {p: qs.eigsh_batch(ops, k=1, tol=1e-10, precision=p)[:, 0].tolist() for p in ('fp64', 'fp64df')};"
        "E, V, Q = qs.lanczos_full(ops[0], models.seeded(ops[0].Ns, complex_=True), 40);"
        "out['lanczos'] = E.tolist(); print(json.dumps(out))")
    runs = [subprocess.run([sys.executable, "-c", code], cwd=root, capture_output=True, text=True, check=True)
            for _ in range(2)]
    a, b = (json.loads(r.stdout.strip().splitlines()[-1]) for r in runs)
    assert a == b
