"""The request loop (qs_server_*): served eigsh / evolve results against the
direct solvers and dense FP64, the same result alone and in a mix, admission
under a device-memory budget, cancellation."""
import numpy as np
import pytest
import scipy.linalg as sla

import models

pytestmark = pytest.mark.gpu


def j1j2_terms(qs, L, J2=0.5):
    return models.to_terms(qs, models.j1j2(L, 1.0, J2))


def dense(ora, L, nup, sym, sp):
    rep = ora.RepBasis(L, nup=nup, pauli=False, **sym)
    n = rep.Ns
    H = np.zeros((n, n), dtype=np.complex128)
    e = np.zeros(n, dtype=np.complex128)
    for j in range(n):
        e[:] = 0
        e[j] = 1
        H[:, j] = rep.matvec(sp, e)
    return H


@pytest.mark.parametrize("precision", ["fp64", "fp64df", "fp32"])
def test_served_results_match_dense(qs, ora, precision):
    L = 12
    sp = models.j1j2(L, 1.0, 0.3)   # away from J2 = 0.5, where sector ground states are degenerate
    terms = models.to_terms(qs, sp)
    cases = [(6, dict(kblock=0, pblock=1)), (6, dict(kblock=3)), (5, dict(kblock=1)), (4, dict(kblock=6))]
    with qs.Server(hbm_budget_gb=4, precision=precision) as srv:
        tick = []
        for nup, sym in cases:
            basis = dict(L=L, nup=nup, pauli=False, **sym)
            tick.append(("e", nup, sym, srv.submit_eigsh(basis, terms, k=2, tol=1e-12, want_vector=True)))
            v0 = models.seeded(qs.SpinBasis1D(L, nup=nup, pauli=False, **sym).Ns, complex_=True)
            tick.append(("t", nup, sym, srv.submit_evolve(basis, terms, 1.7, v0=v0, tol=1e-11), v0))
        for item in tick:
            kind, nup, sym, t = item[:4]
            D = dense(ora, L, nup, sym, sp)
            res = srv.wait(t, timeout=120)
            if kind == "e":
                w = np.linalg.eigvalsh(D)[:2]
                assert np.allclose(res["values"], w, rtol=1e-10, atol=1e-10), (sym, res["values"], w)
                vec = srv.vector(t)
                # the FP32 form's eigenvalues are polished to FP64 accuracy; its
                # vectors keep FP32-level residuals
                res_tol = 1e-6 if precision == "fp32" else 1e-8
                assert np.abs(D @ vec - vec * np.array(res["values"])).max() < res_tol
            else:
                want = sla.expm(-1j * 1.7 * D) @ item[4]
                got = srv.vector(t)
                assert np.linalg.norm(got - want) < 1e-9 * np.linalg.norm(want), sym
        st = srv.stats()
        assert st["completed"] == len(tick) and st["failed"] == 0
        assert st["cache_hits"] >= len(cases)   # each sector built once, reused by its second request


def test_same_result_alone_and_in_the_mix(qs):
    """Each result is the same whether the request ran alone or among others."""
    L = 16
    terms = j1j2_terms(qs, L)
    probe = [("e", dict(L=L, nup=8, pauli=False, kblock=0, pblock=1)),
             ("t", dict(L=L, nup=7, pauli=False, kblock=2)),
             ("e", dict(L=L, nup=6, pauli=False, kblock=5))]
    others = [dict(L=L, nup=8, pauli=False, kblock=k) for k in (1, 3, 4, 7)] + \
             [dict(L=14, nup=7, pauli=False, kblock=k) for k in (0, 2)]

    def submit(srv, kind, basis, seed):
        tm = terms if basis["L"] == L else j1j2_terms(qs, basis["L"])
        if kind == "e":
            return srv.submit_eigsh(basis, tm, k=1, tol=1e-10, seed=seed, want_vector=True)
        return srv.submit_evolve(basis, tm, 2.3, seed=seed, tol=1e-9)

    for precision in ("fp64", "fp64df", "fp32"):
        with qs.Server(precision=precision) as srv:
            alone = []
            for i, (kind, basis) in enumerate(probe):
                t = submit(srv, kind, basis, 100 + i)
                srv.wait(t, timeout=300)
                alone.append((srv.poll(t), srv.vector(t)))
            ts = []
            for i, b in enumerate(others):
                ts.append(submit(srv, "e" if i % 2 == 0 else "t", b, 500 + i))
                if i == 2:
                    mix = [submit(srv, kind, basis, 100 + j) for j, (kind, basis) in enumerate(probe)]
            for t in ts + mix:
                srv.wait(t, timeout=300)
            for (r0, v0), t, (kind, _) in zip(alone, mix, probe):
                r1, v1 = srv.poll(t), srv.vector(t)
                if kind == "e":
                    assert abs(r1["values"][0] - r0["values"][0]) <= 1e-12 * abs(r0["values"][0])
                    ov = abs(np.vdot(v0[:, 0], v1[:, 0]))
                    assert abs(ov - 1) < 1e-10
                else:
                    assert np.linalg.norm(v1 - v0) < 1e-12
                # bit-for-bit: a slot's arithmetic does not see the other slots
                assert r1["values"] == r0["values"] and np.array_equal(v1, v0), (precision, kind)


def test_admission_under_a_small_budget(qs):
    """With room for only a few solves the server queues the rest and never
    holds more than the budget; a request larger than the budget fails."""
    L = 16
    terms = j1j2_terms(qs, L)
    budget_gb = 0.25
    with qs.Server(hbm_budget_gb=budget_gb, precision="fp64df", op_cache=False) as srv:
        ts = [srv.submit_eigsh(dict(L=L, nup=8, pauli=False, kblock=k), terms, k=1, tol=1e-10) for k in range(8)]
        for t in ts:
            srv.wait(t, timeout=300)
        st = srv.stats()
        assert st["completed"] == 8 and st["peak_bytes"] <= budget_gb * 1e9
        big = srv.submit_eigsh(dict(L=28, nup=14, pauli=False, kblock=1), j1j2_terms(qs, 28), k=1)
        with pytest.raises(MemoryError):
            srv.wait(big, timeout=300)


def test_release_cancels_a_queued_request(qs):
    L = 18
    terms = j1j2_terms(qs, L)
    with qs.Server(max_slots=1, precision="fp64df") as srv:
        first = srv.submit_eigsh(dict(L=L, nup=9, pauli=False, kblock=1), terms, k=1, tol=1e-10)
        queued = srv.submit_eigsh(dict(L=L, nup=9, pauli=False, kblock=2), terms, k=1, tol=1e-10)
        srv.release(queued)
        srv.wait(first, timeout=300)
        r = srv.poll(queued)
        assert r["status"] != 0 or r["values"]   # cancelled, or finished before the release landed
        # a running request stops between steps
        big = srv.submit_evolve(dict(L=26, nup=13, pauli=False, kblock=1), j1j2_terms(qs, 26), 400.0, tol=1e-12)
        import time
        time.sleep(0.3)
        srv.release(big)
        with pytest.raises(qs.ArgumentError):
            srv.wait(big, timeout=300)
        with pytest.raises(qs.ArgumentError):
            srv.poll(123456)


def test_smallest_first_policy_completes_every_request(qs):
    """The smallest-work-first admission order serves the same requests with the
    same results; an unknown policy is an argument error."""
    L = 16
    terms = j1j2_terms(qs, L)
    reqs = [dict(L=L, nup=8, pauli=False, kblock=k) for k in range(6)] + \
           [dict(L=12, nup=6, pauli=False, kblock=k) for k in range(4)]
    results = {}
    for policy in ("fifo", "sjf"):
        with qs.Server(precision="fp64df", policy=policy, max_slots=2) as srv:
            ts = [srv.submit_eigsh(b, terms if b["L"] == L else j1j2_terms(qs, b["L"]), k=1, tol=1e-10, seed=7)
                  for b in reqs]
            results[policy] = [srv.wait(t, timeout=300)["values"][0] for t in ts]
    assert results["fifo"] == results["sjf"]
    with pytest.raises(qs.ArgumentError):
        qs.Server(policy="lifo")
