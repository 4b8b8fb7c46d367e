"""tools.jl's Krylov tools on the device (lanczos_full, lanczos_iter,
lin_comb_Q_T, expm_lanczos, ftlm_static_iteration, ltlm_static_iteration,
and the batched form) against the reference's known answers and the oracle."""
import numpy as np
import pytest

import models

pytestmark = pytest.mark.gpu


def kat_operators(qs, k):
    """The 4 x 4 matrices of test/runtests.jl:130-172 as spin-1/2 operators on
    the full L = 2 basis (states 0..3): A = 0.6 x_1 + 0.4 x_1 z_2 + 0.3 (s+_1
    s-_2 + s-_1 s+_2) + diag(A), B = diag(B)."""
    A = np.array(k["A"])
    basis = qs.SpinBasis1D(2, pauli=False)
    terms = [qs.OperatorTerm("x", [(0.6, 1)]), qs.OperatorTerm("xz", [(0.4, 1, 2)]),
             qs.OperatorTerm("+-", [(0.3, 1, 2)]), qs.OperatorTerm("-+", [(0.3, 1, 2)])]
    opA = qs.QuantumLinearOperator(basis, terms, diagonal=np.diag(A))
    opB = qs.QuantumLinearOperator(basis, [qs.OperatorTerm("z", [(0.0, 1)])], diagonal=np.array(k["B_diagonal"]))
    return A, opA, opB


def test_reference_known_answers(qs, kats):
    k = kats["krylov_tools_4x4"]
    A, opA, opB = kat_operators(qs, k)
    e = np.eye(4)
    assert np.allclose(np.column_stack([opA.dot(e[:, j]) for j in range(4)]), A, atol=1e-15)
    v0 = np.array(k["v0"])
    E, V, Q = qs.lanczos_full(opA, v0, k["m"])
    Qh = np.asarray(Q)
    assert np.allclose(E, k["E"], atol=k["E_atol"], rtol=0)
    assert np.allclose(Qh @ Qh.T, np.eye(k["m"]), atol=k["orthonormal_atol"], rtol=0)
    assert np.allclose(qs.lin_comb_Q_T(k["lin_comb_coeff"], Q), k["lin_comb"], atol=k["lin_comb_atol"], rtol=0)
    assert np.allclose(qs.expm_lanczos(E, V, Q, a=k["expm_a"]), k["expm_lanczos"], atol=k["expm_atol"], rtol=0)
    Ei, Vi, Qi = qs.lanczos_iter(opA, v0, k["m"])
    assert np.allclose(Ei, E, atol=k["iter_atol"], rtol=0)
    assert np.allclose(np.abs(Vi), np.abs(V), atol=k["iter_atol"], rtol=0)
    assert np.allclose(np.array(list(Qi)), Qh, atol=k["iter_atol"], rtol=0)
    obs = {"A": opA, "B": opB}
    f, fi = qs.ftlm_static_iteration(obs, E, V, Q, beta=k["beta"])
    lt, li = qs.ltlm_static_iteration(obs, E, V, Q, beta=k["beta"])
    assert np.allclose(fi, k["ftlm_identity"], atol=k["ftlm_identity_atol"], rtol=0)
    assert np.allclose(f["B"], k["ftlm_B"], atol=k["ftlm_B_atol"], rtol=0)
    assert np.allclose(li, fi, atol=k["ftlm_identity_atol"], rtol=0)
    assert np.allclose(lt["B"], k["ltlm_B"], atol=k["ltlm_B_atol"], rtol=0)


def sector(qs, ora, L, sym, spec):
    basis = qs.SpinBasis1D(L, nup=L // 2, pauli=False, **sym)
    H = qs.Hamiltonian(basis, models.to_terms(qs, spec))
    rep = ora.RepBasis(L, nup=L // 2, pauli=False, **sym)
    return H, (lambda x: rep.matvec(spec, np.asarray(x, dtype=np.complex128))), rep


@pytest.mark.parametrize("sym", [dict(kblock=0, pblock=1), dict(kblock=3)])
def test_full_ortho_matches_oracle(qs, ora, sym):
    L = 14
    spec = models.j1j2(L, 1.0, 0.3)
    H, mv, _ = sector(qs, ora, L, sym, spec)
    v0 = models.seeded(H.Ns, complex_=H.dtype == np.complex128)
    m = 40
    E, V, Q = qs.lanczos_full(H, v0, m, full_ortho=True)
    Eo, Vo, Qo = ora.lanczos_full(mv, v0, m, full_ortho=True)
    assert np.allclose(E, Eo, rtol=1e-10, atol=1e-10)
    Qh = np.asarray(Q)
    assert np.abs(Qh - Qo).max() < 1e-8
    assert np.abs(Qh.conj() @ Qh.T - np.eye(m)).max() < 1e-12


def test_three_term_recurrence_matches_oracle(qs, ora):
    L = 16
    spec = models.j1j2(L, 1.0, 0.3)
    H, mv, _ = sector(qs, ora, L, dict(kblock=0, pblock=1), spec)
    v0 = models.seeded(H.Ns)
    m = 60
    E, V, Q = qs.lanczos_full(H, v0, m)
    a, b, _ = ora.lanczos_coefficients(mv, v0, m)
    lset = Q._set
    ag, bg, used = lset.coeffs[0]
    assert used == m
    # the early coefficients agree to rounding; later ones drift as the plain
    # recurrence loses orthogonality in both, so compare the extreme Ritz value
    assert np.allclose(ag[:12], a[:12], rtol=1e-11, atol=1e-11)
    assert np.allclose(bg[:12], b[:12], rtol=1e-11, atol=1e-11)
    Eo = np.linalg.eigvalsh(np.diag(a) + np.diag(b, 1) + np.diag(b, -1))
    assert abs(E[0] - Eo[0]) < 1e-10 * abs(Eo[0])


@pytest.mark.parametrize("sym", [dict(kblock=0, pblock=1), dict(kblock=5)])
def test_lin_comb_expm_ftlm_ltlm_match_oracle(qs, ora, sym):
    L = 14
    spec = models.j1j2(L, 1.0, 0.3)
    H, mv, rep = sector(qs, ora, L, sym, spec)
    zz_spec = [("zz", [(1.0, i, i % L + 1) for i in range(1, L + 1)])]
    ZZ = qs.QuantumLinearOperator(H.basis, models.to_terms(qs, zz_spec))
    mzz = lambda x: rep.matvec(zz_spec, np.asarray(x, dtype=np.complex128))  # noqa: E731
    v0 = models.seeded(H.Ns, seed=7, complex_=H.dtype == np.complex128)
    m = 30
    E, V, Q = qs.lanczos_full(H, v0, m, full_ortho=True)
    Qh = np.asarray(Q)
    c = np.random.default_rng(3).standard_normal(m) + 0.5j
    got = qs.lin_comb_Q_T(c, Q)
    assert np.abs(got - Qh.T @ c).max() < 1e-13 * np.abs(c).sum()
    out = np.empty(H.Ns, dtype=np.complex128)
    assert qs.lin_comb_Q_T(c, Q, out=out) is out
    ex = qs.expm_lanczos(E, V, Q, a=-0.7j)
    assert np.abs(ex - ora.expm_lanczos(E, V, Qh, a=-0.7j)).max() < 1e-13
    beta = [0.0, 0.3, 2.5]
    obs_gpu = {"H": H, "ZZ": ZZ}
    obs_ora = {"H": mv, "ZZ": mzz}
    f, fi = qs.ftlm_static_iteration(obs_gpu, E, V, Q, beta=beta)
    fo, fio = ora.ftlm_static_iteration(obs_ora, E, V, Qh, beta=beta)
    lt, li = qs.ltlm_static_iteration(obs_gpu, E, V, Q, beta=beta)
    lo, lio = ora.ltlm_static_iteration(obs_ora, E, V, Qh, beta=beta)
    assert np.allclose(fi, fio, rtol=1e-13, atol=0) and np.allclose(li, lio, rtol=1e-13, atol=0)
    for key in obs_gpu:
        assert np.allclose(f[key], fo[key], rtol=1e-11, atol=1e-12), key
        assert np.allclose(lt[key], lo[key], rtol=1e-11, atol=1e-12), key
    # a scalar temperature gives scalars
    fs, fis = qs.ftlm_static_iteration(obs_gpu, E, V, Q, beta=0.3)
    assert np.ndim(fs["H"]) == 0 and abs(fs["H"] - f["H"][1]) < 1e-12 * abs(f["H"][1])


def test_batch_equals_one_at_a_time(qs, ora):
    """Each start vector's recurrence is the same alone and among others."""
    L = 16
    spec = models.j1j2(L, 1.0, 0.3)
    H, _, _ = sector(qs, ora, L, dict(kblock=2), spec)
    rng = np.random.default_rng(11)
    V0 = rng.standard_normal((H.Ns, 5)) + 1j * rng.standard_normal((H.Ns, 5))
    batch = qs.lanczos_batch(H, V0, 25)
    for r in range(5):
        E, V, Q = qs.lanczos_full(H, V0[:, r], 25)
        Eb, Vb, Qb = batch[r]
        assert np.array_equal(E, Eb)
        assert np.array_equal(np.asarray(Q), np.asarray(Qb))


def test_breakdown_and_errors(qs, kats):
    k = kats["krylov_tools_4x4"]
    A, opA, opB = kat_operators(qs, k)
    # an eigenvector of the diagonal operator: beta = 0 after one step
    E, V, Q = qs.lanczos_full(opB, np.array([1.0, 0, 0, 0]), 3)
    assert len(Q) == 1 and np.allclose(E, [2.0]) and np.allclose(np.asarray(Q), [[1, 0, 0, 0]])
    with pytest.raises(qs.ArgumentError):
        qs.lanczos_full(opA, np.array(k["v0"]), 4)
    with pytest.raises(qs.ArgumentError):
        qs.lanczos_full(opA, np.zeros(4), 2)
    E, V, Q = qs.lanczos_full(opA, np.array(k["v0"]), 3)
    with pytest.raises(qs.DimensionMismatch):
        qs.lin_comb_Q_T([1.0, 2.0], Q)
    with pytest.raises(qs.DimensionMismatch):
        qs.expm_lanczos(E[:2], V, Q)
    with pytest.raises(qs.DimensionMismatch):
        qs.ftlm_static_iteration({"A": opA}, E[:2], V[:2, :2], Q)
    nonherm = qs.QuantumLinearOperator(qs.SpinBasis1D(2, pauli=False), [qs.OperatorTerm("+-", [(1.0, 1, 2)])],
                                       check_herm=False)
    with pytest.raises(qs.ArgumentError):
        qs.lanczos_full(nonherm, np.array(k["v0"]), 2)
