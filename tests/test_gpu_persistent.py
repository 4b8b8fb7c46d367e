"""The persistent Lanczos step against the graph-replayed one.

QS_PERSISTENT_STEP=1 runs each chunk of Lanczos steps as one cooperative
launch whose phases (product, dots, reductions, updates, scaling) are the
graph kernels' block bodies over the same block indices, separated by grid
barriers; QS_PERSISTENT_STEP=0 replays the captured graph of separate
launches.  The arithmetic and its order are the same, so every result must be
bit-identical: batched sectors in the three precision forms, a single solve
with vectors, a Krylov exponential and the batched three-term recurrences.
The barrier's waits are bounded: a grid that waits for a block that never
comes returns QS_ERR_TIMEOUT and leaves the device usable.
"""
import os

import numpy as np
import pytest

import models

pytestmark = pytest.mark.gpu


@pytest.fixture
def mode_env():
    old = {k: os.environ.get(k) for k in ("QS_PERSISTENT_STEP", "QS_CLUSTER_STEP")}
    os.environ["QS_CLUSTER_STEP"] = "0"   # the graph replay and the persistent form
    yield
    for k, v in old.items():
        if v is None:
            os.environ.pop(k, None)
        else:
            os.environ[k] = v


def both_modes(fn):
    out = {}
    for m in ("0", "1"):
        os.environ["QS_PERSISTENT_STEP"] = m
        out[m] = fn()
    return out["0"], out["1"]


def sector_ops(qs, L, nup, J2):
    terms = models.to_terms(qs, models.j1j2(L, 1.0, J2))
    ops = []
    for k in range(L):
        for p in ((1, -1) if k in (0, L // 2) else (0,)):
            sym = dict(kblock=k, pblock=p) if p else dict(kblock=k)
            ops.append(qs.Hamiltonian(qs.SpinBasis1D(L, nup=nup, pauli=False, **sym), terms))
    return ops


@pytest.mark.parametrize("precision", ["fp64", "fp64df", "fp32"])
def test_batched_sectors_bit_identical(qs, mode_env, precision):
    ops = sector_ops(qs, 14, 7, 0.3)
    g, p = both_modes(lambda: qs.eigsh_batch(ops, k=2, tol=1e-12, return_eigenvectors=True, precision=precision))
    assert np.array_equal(g[0], p[0])
    for a, b in zip(g[1], p[1]):
        assert np.array_equal(a, b)


def test_single_solve_evolve_and_recurrences_bit_identical(qs, ora, mode_env):
    L = 20
    sp = models.j1j2(L, 1.0, 0.37)
    sym = dict(kblock=0, pblock=1, zblock=1)
    b = qs.SpinBasis1D(L, nup=10, pauli=False, **sym)
    H = qs.Hamiltonian(b, models.to_terms(qs, sp))
    v0 = models.seeded(b.Ns, seed=7)
    g, p = both_modes(lambda: qs.eigsh(H, k=3, which="SA", tol=1e-12, v0=v0))
    assert np.array_equal(g[0], p[0]) and np.array_equal(g[1], p[1])
    # against the oracle's spectrum
    rep = ora.RepBasis(L, nup=10, pauli=False, **sym)
    want, _ = ora.eigsh_arpack(lambda v: rep.matvec(sp, v).real, b.Ns, 3, np.float64, v0=v0, tol=1e-13)
    assert np.max(np.abs(np.sort(p[0]) - np.sort(want))) <= 1e-10 * np.abs(want).max()
    v = models.seeded(b.Ns, seed=8, complex_=True)
    v /= np.linalg.norm(v)
    g, p = both_modes(lambda: qs.evolve(H, v, 0.0, [0.5, 1.0], tol=1e-10))
    assert np.array_equal(g, p)
    V0 = np.stack([models.seeded(b.Ns, seed=20 + i) for i in range(4)], axis=1)

    def rec():
        out = []
        for E, Vr, Q in qs.lanczos_batch(H, V0, 40):
            out.append((E, Vr, qs.lin_comb_Q_T(np.linspace(0.5, 1.5, Q.used), Q)))
        return out

    g, p = both_modes(rec)
    for a, c in zip(g, p):
        for x, y in zip(a, c):
            assert np.array_equal(x, y)


def test_grid_barrier_wait_is_bounded(qs):
    from qsgpu import _lib
    lib = _lib.load()
    assert lib.qs_grid_barrier_check(0, 200.0, 64) == 0
    st = lib.qs_grid_barrier_check(1, 20.0, 64)
    assert st == 7, lib.qs_last_error()   # QS_ERR_TIMEOUT
    assert "ran out" in lib.qs_last_error().decode()
    # the context is intact: a product still matches the oracle
    L = 12
    b = qs.SpinBasis1D(L, nup=6, pauli=False)
    H = qs.Hamiltonian(b, models.to_terms(qs, models.xxz(L)))
    x = models.seeded(b.Ns)
    y = H.dot(x)
    z = qs.QuantumLinearOperator(b, models.to_terms(qs, models.xxz(L))).dot(x)
    assert np.max(np.abs(y - z)) <= 1e-13 * max(1.0, np.abs(z).max())
    assert lib.qs_grid_barrier_check(0, 200.0, 64) == 0


@pytest.mark.parametrize("precision", ["fp64", "fp64df", "fp32"])
def test_fused_update_bit_identical(qs, precision):
    """The first-pass dots and the pass-0 update with each row's vector
    entries held in registers (the second-pass dots from the values that
    served the update; QS_FUSED_UPDATE=1, the default) against the tiled dots
    and the update followed by a second read of V (QS_FUSED_UPDATE=0)."""
    saved = {k: os.environ.get(k) for k in ("QS_FUSED_UPDATE", "QS_PERSISTENT_STEP", "QS_CLUSTER_STEP")}
    L = 20
    b = qs.SpinBasis1D(L, nup=10, pauli=False, kblock=0, pblock=1, zblock=1)
    H = qs.Hamiltonian(b, models.to_terms(qs, models.j1j2(L, 1.0, 0.37)))
    ops = sector_ops(qs, 14, 7, 0.3)
    got = {}
    try:
        os.environ["QS_PERSISTENT_STEP"] = "0"
        os.environ["QS_CLUSTER_STEP"] = "0"
        for m in ("0", "1"):
            os.environ["QS_FUSED_UPDATE"] = m
            got[m] = (qs.eigsh(H, k=3, which="SA", tol=1e-12, v0=models.seeded(b.Ns, seed=4), precision=precision),
                      qs.eigsh_batch(ops, k=2, tol=1e-12, return_eigenvectors=True, precision=precision))
    finally:
        for k, v in saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    (a0, a1), (b0, b1) = got["0"], got["1"]
    assert np.array_equal(a0[0], b0[0]) and np.array_equal(a0[1], b0[1])
    assert np.array_equal(a1[0], b1[0])
    for x, y in zip(a1[1], b1[1]):
        assert np.array_equal(x, y)


def test_fused_update_at_config_size(qs):
    """The fused kernels on the 4.7 M-state sector (1150 row blocks): the same
    eigenvalue bits as the unfused ones in the three precision forms."""
    saved = os.environ.get("QS_FUSED_UPDATE")
    L = 32
    b = qs.SpinBasis1D(L, nup=16, pauli=False, kblock=0, pblock=1, zblock=1)
    H = qs.Hamiltonian(b, models.to_terms(qs, models.j1j2(L, 1.0, 0.5)))
    v0 = models.seeded(b.Ns, seed=2)
    out = {}
    try:
        for m in ("0", "1"):
            os.environ["QS_FUSED_UPDATE"] = m
            out[m] = [qs.eigsh(H, k=1, which="SA", tol=1e-10, v0=v0, return_eigenvectors=False, precision=p)[0]
                      for p in ("fp64", "fp64df", "fp32")]
    finally:
        if saved is None:
            os.environ.pop("QS_FUSED_UPDATE", None)
        else:
            os.environ["QS_FUSED_UPDATE"] = saved
    assert out["0"] == out["1"]
    assert abs(out["1"][0] + 12.0) < 1e-10 * 12   # the Majumdar-Ghosh energy -3L/8 = -12


@pytest.mark.parametrize("precision", ["fp64", "fp64df", "fp32"])
def test_cluster_step(qs, ora, precision):
    """QS_CLUSTER_STEP=1: a thread-block cluster per slot runs the steps up to
    each Hold event, the reductions crossing the cluster through distributed
    shared memory.  Its reduction order differs from the graph replay's, so
    the eigenvalues agree to rounding; a slot's result does not depend on the
    other slots (bit-identical alone and in the batch); against the dense
    spectrum of every sector."""
    saved = os.environ.get("QS_CLUSTER_STEP")
    ops = sector_ops(qs, 14, 7, 0.3)
    try:
        os.environ["QS_CLUSTER_STEP"] = "0"
        g = qs.eigsh_batch(ops, k=2, tol=1e-12, precision=precision)
        os.environ["QS_CLUSTER_STEP"] = "1"
        c = qs.eigsh_batch(ops, k=2, tol=1e-12, precision=precision)
        alone = [qs.eigsh_batch([op], k=2, tol=1e-12, precision=precision)[0] for op in ops[:4]]
        L = 20
        b = qs.SpinBasis1D(L, nup=10, pauli=False, kblock=0, pblock=1, zblock=1)
        H = qs.Hamiltonian(b, models.to_terms(qs, models.j1j2(L, 1.0, 0.37)))
        v0 = models.seeded(b.Ns, seed=4)
        e1 = qs.eigsh(H, k=3, which="SA", tol=1e-12, v0=v0, precision=precision, return_eigenvectors=False)
        # 8,359 rows: sixteen CTAs per cluster
        b22 = qs.SpinBasis1D(22, nup=11, pauli=False, kblock=0, pblock=1, zblock=1)
        H22 = qs.Hamiltonian(b22, models.to_terms(qs, models.j1j2(22, 1.0, 0.37)))
        w22 = models.seeded(b22.Ns, seed=5)
        os.environ.pop("QS_CLUSTER_STEP", None)
        f1 = qs.eigsh(H22, k=2, which="SA", tol=1e-12, v0=w22, precision=precision, return_eigenvectors=False)
        os.environ["QS_CLUSTER_STEP"] = "0"
        f0 = qs.eigsh(H22, k=2, which="SA", tol=1e-12, v0=w22, precision=precision, return_eigenvectors=False)
        e0 = qs.eigsh(H, k=3, which="SA", tol=1e-12, v0=v0, precision=precision, return_eigenvectors=False)
    finally:
        if saved is None:
            os.environ.pop("QS_CLUSTER_STEP", None)
        else:
            os.environ["QS_CLUSTER_STEP"] = saved
    scale = np.abs(g).max()
    assert np.max(np.abs(c - g)) <= 1e-10 * scale
    for i, a in enumerate(alone):
        assert np.array_equal(a, c[i])
    assert np.max(np.abs(np.sort(e1) - np.sort(e0))) <= 1e-10 * np.abs(e0).max()
    assert np.max(np.abs(np.sort(f1) - np.sort(f0))) <= 1e-10 * np.abs(f0).max()
