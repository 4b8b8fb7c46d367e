"""Device matvec and Krylov solvers vs the oracle (reference algorithm)."""
import numpy as np
import pytest
import scipy.linalg as sla

import models

pytestmark = pytest.mark.gpu

MV_CASES = [
    # (L, nup, pauli, sym, model)
    (10, 5, False, dict(), "xxz"),
    (10, None, True, dict(), "tfim"),
    (12, 6, False, dict(kblock=0, pblock=1, zblock=1), "j1j2"),
    (12, 6, False, dict(kblock=0, pblock=-1), "j1j2"),
    (12, 6, False, dict(kblock=6, pblock=1, zblock=-1), "xxz"),
    (12, 6, False, dict(kblock=1), "j1j2"),
    (12, 6, False, dict(kblock=5, zblock=1), "j1j2"),
    (12, None, True, dict(kblock=0, pblock=1), "tfim"),
    (12, None, True, dict(kblock=3), "tfim"),
    (10, None, False, dict(kblock=2), "xyz"),
    (12, None, False, dict(kblock=0, pblock=1, zblock=1), "xyz_z"),
    # sublattice-flip sectors (zAblock / zBblock, src/basis.jl:740-741)
    (12, None, True, dict(zBblock=1), "sub"),
    (12, None, True, dict(kblock=0, zBblock=-1, a=2), "sub"),
    (14, None, True, dict(kblock=3, zAblock=1, zBblock=1, a=2), "sub"),
    (12, None, True, dict(zAblock=1, zBblock=-1), "sub"),
]


def spec(model, L):
    if model == "xxz":
        return models.xxz(L, 1.0, 0.5)
    if model == "j1j2":
        return models.j1j2(L, 1.0, 0.5)
    if model == "tfim":
        return models.tfim(L, 1.0, 0.7)
    if model == "xyz":
        return models.xyz_field(L)
    if model == "xyz_z":
        return [t for t in models.xyz_field(L) if t[0] not in ("y", "z")]
    if model == "sub":
        return models.sublattice(L)
    raise ValueError(model)


@pytest.mark.parametrize("L,nup,pauli,sym,model", MV_CASES)
def test_matvec_matches_oracle(qs, ora, L, nup, pauli, sym, model):
    sp = spec(model, L)
    ref = ora.RefBasis(L, nup=nup, pauli=pauli, **sym)
    b = qs.SpinBasis1D(L, nup=nup, pauli=pauli, **sym)
    op = qs.QuantumLinearOperator(b, models.to_terms(qs, sp))
    n = b.Ns
    x = models.seeded(n, complex_=True)
    y0 = models.seeded(n, seed=7, complex_=True)
    cterms = ora.consolidate_terms(sp)
    alpha, beta = 1.25 - 0.5j, -0.5
    for flags, (T, C) in ((0, (False, False)), ("T", (True, False)), ("C", (False, True)), ("H", (True, True))):
        o = {0: op, "T": op.T, "C": op.conj(), "H": op.H}[flags]
        # mul! semantics: alpha * op(A) x + beta * y
        want = alpha * ref.qlo_matvec(cterms, x, transposed=T, conjugated=C) + beta * y0
        if b.symmetric or not C:
            # the reference computes exactly this (symmetric path applies alpha after projecting)
            assert np.allclose(want, ref.qlo_matvec(cterms, x, alpha=alpha, beta=beta, y=y0, transposed=T,
                                                    conjugated=C), atol=1e-12 * max(1, np.abs(want).max()))
        got = o.mul(y0.copy(), x, alpha=alpha, beta=beta)
        scale = max(1.0, np.abs(want).max())
        assert np.max(np.abs(got - want)) <= 1e-13 * scale, flags
    if op.dtype == np.float64:
        xr = models.seeded(n)
        want = ref.qlo_matvec(cterms, xr).real
        got = op.dot(xr)
        assert got.dtype == np.float64
        assert np.max(np.abs(got - want)) <= 1e-13 * max(1.0, np.abs(want).max())
    # repeated calls are bit-identical (fixed per-row summation order)
    assert np.array_equal(op.dot(x), op.dot(x))


def test_qlo_protocol_kat(qs, ora, kats):
    k = kats["qlo_protocol_L3"]
    b = qs.SpinBasis1D(k["L"], nup=k["nup"], pauli=k["pauli"])
    terms = [qs.OperatorTerm(op, [tuple(c) for c in cs]) for op, cs in k["terms"]]
    diag = np.array(k["diagonal"])
    op = qs.QuantumLinearOperator(b, terms, diagonal=diag)
    ref = ora.RefBasis(k["L"], nup=k["nup"], pauli=k["pauli"])
    M = ref.dense(ora.consolidate_terms([(t.op, t.couplings) for t in terms]), diag=diag)
    assert op.Ns == 3 and op.shape == (3, 3) and op.dtype == np.float64
    assert np.array_equal(op.toarray(), M.real)
    assert np.array_equal(op.H.toarray(), M.conj().T.real)
    assert np.array_equal(op.T.toarray(), M.T.real)
    v = np.array([complex(*c) for c in k["vector_unnormalized"]])
    v /= np.linalg.norm(v)
    assert np.allclose(op.dot(v), M @ v, atol=k["atol"])
    dest = np.array([complex(*c) for c in k["destination"]])
    out = op.mul(dest.copy(), v, k["alpha"], k["beta"])
    assert np.allclose(out, k["alpha"] * (M @ v) + k["beta"] * dest, atol=k["atol"])
    vals, vecs = qs.eigsh(op, k=k["eigsh_k"], which="SA")
    assert np.allclose(M.real @ vecs, vecs * vals, atol=k["eigsh_atol"])
    op.set_diagonal(np.zeros(3))
    assert np.allclose(op.toarray(), ref.dense(ora.consolidate_terms([(t.op, t.couplings) for t in terms])).real,
                       atol=0)


def test_unchecked_nonsymmetric_qlo(qs, ora, kats):
    k = kats["unchecked_symmetric_qlo"]
    terms = [(op, [tuple(c) for c in cs]) for op, cs in k["terms"]]
    b = qs.SpinBasis1D(k["L"], nup=k["nup"], pauli=False, kblock=0)
    with pytest.raises(qs.ArgumentError):
        qs.QuantumLinearOperator(b, models.to_terms(qs, terms))
    op = qs.QuantumLinearOperator(b, models.to_terms(qs, terms), check_symm=False)
    ref = ora.RefBasis(k["L"], nup=k["nup"], pauli=False, kblock=0)
    v = models.seeded(b.Ns, complex_=True)
    assert np.allclose(op.dot(v), ref.qlo_matvec(terms, v, extract=False), atol=k["atol"])


def test_operator_errors(qs):
    b = qs.SpinBasis1D(6, nup=3, pauli=False)
    with pytest.raises(qs.ArgumentError, match="not Hermitian"):
        qs.QuantumLinearOperator(b, [qs.OperatorTerm("+-", [(1.0, 1, 2)])])
    with pytest.raises(qs.ArgumentError, match="particle sector"):
        qs.QuantumLinearOperator(b, [qs.OperatorTerm("x", [(1.0, 1)])])
    with pytest.raises(qs.ArgumentError, match="outside"):
        qs.QuantumLinearOperator(b, [qs.OperatorTerm("z", [(1.0, 7)])])
    op = qs.QuantumLinearOperator(b, [qs.OperatorTerm("zz", [(1.0, 1, 2)])])
    with pytest.raises(qs.DimensionMismatch):
        op.dot(np.ones(b.Ns + 1))
    with pytest.raises(qs.ArgumentError, match="k must lie"):
        qs.eigsh(op, k=0)


@pytest.mark.parametrize("sym,model,L,nup,pauli", [
    (dict(), "xxz", 12, 6, False),
    (dict(kblock=0, pblock=1, zblock=1), "j1j2", 16, 8, False),
    (dict(kblock=1), "j1j2", 14, 7, False),
    (dict(kblock=0, pblock=1), "tfim", 14, None, True),
])
def test_eigsh_matches_dense(qs, ora, sym, model, L, nup, pauli):
    sp = spec(model, L)
    b = qs.SpinBasis1D(L, nup=nup, pauli=pauli, **sym)
    op = qs.QuantumLinearOperator(b, models.to_terms(qs, sp))
    rep = ora.RepBasis(L, nup=nup, pauli=pauli, **sym)
    n = b.Ns
    H = np.zeros((n, n), dtype=np.complex128)
    e = np.zeros(n, dtype=np.complex128)
    for j in range(n):
        e[:] = 0
        e[j] = 1
        H[:, j] = rep.matvec(sp, e)
    w = np.linalg.eigvalsh(H)
    info = {}
    vals, vecs = qs.eigsh(op, k=4, which="SA", tol=1e-12, info=info)
    assert np.allclose(vals, w[:4], rtol=1e-10, atol=1e-10 * np.abs(w).max())
    res = op.dot(vecs) - vecs * vals
    assert np.abs(res).max() < 1e-8 * max(1, np.abs(w).max())
    # single-precision Lanczos with FP64 polish reaches the same eigenvalue
    v32 = qs.eigsh(op, k=1, which="SA", tol=1e-10, precision="fp32", return_eigenvectors=False)
    assert abs(v32[0] - w[0]) <= 1e-10 * abs(w[0])
    H = qs.Hamiltonian(b, models.to_terms(qs, sp))
    for prec in ("fp64", "fp32", "fp64df"):
        vh = qs.eigsh(H, k=2, which="SA", tol=1e-12, precision=prec, return_eigenvectors=False)
        assert np.allclose(vh, w[:2], rtol=1e-10, atol=1e-10 * np.abs(w).max()), prec


def test_evolve_and_expm_match_oracle(qs, ora, kats):
    k = kats["matrix_free_krylov_L8"]
    L = k["L"]
    bonds = [(i, i % L + 1) for i in range(1, L + 1)]
    sp = [(op, [(c, a, bb) for a, bb in bonds]) for op, c in k["terms"]]
    b = qs.SpinBasis1D(L, nup=4, pauli=False)
    H = qs.Hamiltonian(b, models.to_terms(qs, sp))
    M = ora.RefBasis(L, nup=4, pauli=False).dense(sp)
    n = b.Ns
    idx = np.arange(1, n + 1)
    v = np.sin(idx) + 1j * np.cos(2 * idx)
    v /= np.linalg.norm(v)
    assert np.allclose(H.dot(v), M @ v, atol=k["matvec_atol"])
    ev = qs.evolve(H, v, 0.0, k["times"])
    assert np.allclose(ev[:, -1], sla.expm(-1j * k["times"][-1] * M) @ v, atol=k["evolve_atol"])
    assert all(abs(np.linalg.norm(ev[:, j]) - 1) < k["norm_atol"] for j in range(ev.shape[1]))
    a = complex(*k["expm_a"])
    E = qs.ExpmMultiplyParallel(H, a)
    assert np.allclose(E.apply(v), sla.expm(a * M) @ v, atol=k["evolve_atol"])
    vals, vecs = qs.eigsh(H, k=2, which="SA")
    assert np.allclose(M @ vecs, vecs * vals, atol=k["eigsh_atol"])


def test_evolve_symmetric_sector_vs_oracle(qs, ora):
    L = 14
    sp = models.tfim(L, 1.0, 0.7)
    sym = dict(kblock=0, pblock=1)
    b = qs.SpinBasis1D(L, pauli=True, **sym)
    H = qs.Hamiltonian(b, models.to_terms(qs, sp))
    rep = ora.RepBasis(L, pauli=True, **sym)
    v = models.seeded(b.Ns, complex_=True)
    v /= np.linalg.norm(v)
    times = np.linspace(0.1, 2.0, 5)
    got = qs.evolve(H, v, 0.0, times, tol=1e-9)
    want = ora.krylov_expmv_times(lambda x: rep.matvec(sp, x), v, [-1j * t for t in times], hermitian=True, tol=1e-9)
    assert np.max(np.linalg.norm(got - want, axis=0)) < 1e-9


@pytest.mark.parametrize("sym,model,L,nup,pauli", [
    (dict(kblock=0, pblock=1, zblock=1), "j1j2", 16, 8, False),
    (dict(kblock=3), "j1j2", 14, 7, False),
    (dict(kblock=2), "tfim", 14, None, True),
])
def test_double_float_krylov_storage(qs, ora, sym, model, L, nup, pauli):
    """Krylov vectors stored as hi+lo floats: eigenpairs and the exponential
    action agree with the FP64 engine and the oracle to FP64-class accuracy."""
    sp = spec(model, L)
    b = qs.SpinBasis1D(L, nup=nup, pauli=pauli, **sym)
    H = qs.Hamiltonian(b, models.to_terms(qs, sp))
    rep = ora.RepBasis(L, nup=nup, pauli=pauli, **sym)
    n = b.Ns
    D = np.zeros((n, n), dtype=np.complex128)
    e = np.zeros(n, dtype=np.complex128)
    for j in range(n):
        e[:] = 0
        e[j] = 1
        D[:, j] = rep.matvec(sp, e)
    w = np.linalg.eigvalsh(D)
    scale = np.abs(w).max()
    vals, vecs = qs.eigsh(H, k=3, which="SA", tol=1e-12, precision="fp64df")
    assert np.allclose(vals, w[:3], rtol=1e-11, atol=1e-11 * scale)
    assert np.abs(D @ vecs - vecs * vals).max() < 1e-9 * scale
    assert np.allclose(np.linalg.norm(vecs, axis=0), 1, atol=1e-12)
    v = models.seeded(n, complex_=True)
    v /= np.linalg.norm(v)
    times = np.linspace(0.2, 1.0, 3)
    got = qs.evolve(H, v, 0.0, times, tol=1e-11, precision="fp64df")
    want = np.stack([sla.expm(-1j * t * D) @ v for t in times], axis=1)
    assert np.max(np.abs(got - want)) < 1e-10
    ref64 = qs.evolve(H, v, 0.0, times, tol=1e-11)
    assert np.max(np.abs(got - ref64)) < 1e-10
    E = qs.ExpmMultiplyParallel(H, -0.3 + 0.2j)
    assert np.max(np.abs(E.apply(v, precision="fp64df") - sla.expm((-0.3 + 0.2j) * D) @ v)) < 1e-10


def test_conjugated_complex_alpha_on_unreduced_basis(qs, ora):
    """The reference conjugates a complex alpha together with the term amplitudes
    when conjugated=true on an unreduced basis (src/operators.jl:2565, 2582) but
    not in its diagonal or symmetric paths.  The engine applies alpha as mul!
    defines it; the oracle records the reference's behaviour."""
    L = 8
    sp = models.xxz(L, 1.0, 0.5)
    ref = ora.RefBasis(L, nup=4, pauli=False)
    b = qs.SpinBasis1D(L, nup=4, pauli=False)
    op = qs.QuantumLinearOperator(b, models.to_terms(qs, sp)).conj()
    cterms = ora.consolidate_terms(sp)
    x = models.seeded(b.Ns, complex_=True)
    alpha = 0.3 + 0.7j
    d = ref.extract_diagonal(cterms)
    offdiag = ref.qlo_matvec(cterms, x, conjugated=True) - np.conj(d) * x
    quirk = ref.qlo_matvec(cterms, x, alpha=alpha, conjugated=True)
    assert np.allclose(quirk, np.conj(alpha) * offdiag + alpha * np.conj(d) * x, atol=1e-13)
    got = op.mul(np.zeros(b.Ns, dtype=complex), x, alpha=alpha)
    assert np.allclose(got, alpha * (offdiag + np.conj(d) * x), atol=1e-13)


@pytest.mark.parametrize("L,nup,pauli,sym,model", MV_CASES)
def test_assembled_matches_matrix_free(qs, ora, L, nup, pauli, sym, model):
    """Hamiltonian (assembled on the device, as the reference assembles H.data)
    against the matrix-free operator and the oracle, FP64 and FP32."""
    sp = spec(model, L)
    b = qs.SpinBasis1D(L, nup=nup, pauli=pauli, **sym)
    terms = models.to_terms(qs, sp)
    op = qs.QuantumLinearOperator(b, terms)
    H = qs.Hamiltonian(b, terms)
    assert H.assembled and H.nnz > 0
    ref = ora.RefBasis(L, nup=nup, pauli=pauli, **sym)
    x = models.seeded(b.Ns, complex_=True)
    want = ref.qlo_matvec(ora.consolidate_terms(sp), x)
    scale = max(1.0, np.abs(want).max())
    for o_h, o_q in ((H, op), (H.H, op.H), (H.conj(), op.conj()), (H.T, op.T)):
        a = o_h.dot(x)
        assert np.max(np.abs(a - o_q.dot(x))) <= 1e-13 * scale
    assert np.max(np.abs(H.dot(x) - want)) <= 1e-13 * scale
    y32 = H.dot(x, precision="fp32")
    assert np.max(np.abs(y32 - want)) <= 2e-5 * scale
    # double-float products: FP64-class accuracy on the FP32 pipe
    ydf = H.dot(x, precision="fp64df")
    assert np.max(np.abs(ydf - want)) <= 1e-13 * scale
    ydf_h = H.H.dot(x, precision="fp64df")
    assert np.max(np.abs(ydf_h - op.H.dot(x))) <= 1e-13 * scale
    if H.dtype == np.float64:
        xr = models.seeded(b.Ns)
        assert np.max(np.abs(H.dot(xr) - op.dot(xr))) <= 1e-13 * scale


@pytest.mark.parametrize("sym", [dict(), dict(kblock=2)])
def test_expm_of_a_non_hermitian_assembled_operator(qs, ora, sym):
    """A non-Hermitian assembled operator takes the Arnoldi (CGS2) path of the
    Krylov exponential (src/operators.jl:1655-1731, non-Hermitian branch):
    compared with dense expm, for one vector and for several times."""
    L, nup = 10, 5
    bonds = [(i, i % L + 1) for i in range(1, L + 1)]
    sp = [("+-", [(1.0, a, b) for a, b in bonds]), ("-+", [(0.35, a, b) for a, b in bonds]),
          ("zz", [(0.4, a, b) for a, b in bonds])]
    b = qs.SpinBasis1D(L, nup=nup, pauli=False, **sym)
    H = qs.Hamiltonian(b, models.to_terms(qs, sp), check_herm=False)
    assert H.assembled
    rep = ora.RepBasis(L, nup=nup, pauli=False, **sym)
    n = b.Ns
    D = np.zeros((n, n), dtype=np.complex128)
    e = np.zeros(n, dtype=np.complex128)
    for j in range(n):
        e[:] = 0
        e[j] = 1
        D[:, j] = rep.matvec(sp, e)
    assert np.abs(D - D.conj().T).max() > 0.1          # really non-Hermitian
    v = models.seeded(n, complex_=True)
    v /= np.linalg.norm(v)
    for a in (-0.7 + 0.4j, 1.3j):
        want = sla.expm(a * D) @ v
        for prec in ("fp64", "fp64df"):
            got = qs.ExpmMultiplyParallel(H, a).apply(v, tol=1e-12, precision=prec)
            assert np.linalg.norm(got - want) < 1e-9 * max(1.0, np.linalg.norm(want)), (a, prec)
    times = np.array([0.3, 1.1, 2.0])
    got = qs.evolve(H, v, 0.0, times, tol=1e-11)
    want = np.stack([sla.expm(-1j * t * D) @ v for t in times], axis=1)
    assert np.max(np.linalg.norm(got - want, axis=0) / np.linalg.norm(want, axis=0)) < 1e-9


def test_krylov_exponential_on_a_matrix(qs, ora):
    """apply(ExpmMultiplyParallel(H, a), V) and evolve(H, V0, t0, times) on a
    matrix of states (src/operators.jl:1895-1949, 2150-2164): every column's
    recursion on one engine, equal to the column-by-column calls."""
    import scipy.linalg as sla
    L = 12
    spec = models.j1j2(L, 1.0, 0.3)
    b = qs.SpinBasis1D(L, nup=6, pauli=False, kblock=2)
    H = qs.Hamiltonian(b, models.to_terms(qs, spec))
    rep = ora.RepBasis(L, nup=6, pauli=False, kblock=2)
    D = np.column_stack([rep.matvec(spec, np.eye(b.Ns, dtype=complex)[:, j]) for j in range(b.Ns)])
    rng = np.random.default_rng(5)
    V = rng.standard_normal((b.Ns, 4)) + 1j * rng.standard_normal((b.Ns, 4))
    E = qs.ExpmMultiplyParallel(H, -0.6j)
    got = E.apply(V)
    assert got.shape == V.shape
    want = sla.expm(-0.6j * D) @ V
    assert np.abs(got - want).max() < 1e-10 * np.abs(V).max()
    for j in range(4):
        assert np.abs(got[:, j] - E.apply(V[:, j])).max() < 1e-12 * np.abs(V).max()
    times = [0.0, 0.4, 1.5]
    st = qs.evolve(H, V, 0.2, times)
    assert st.shape == (b.Ns, 4, 3)
    for i, t in enumerate(times):
        assert np.abs(st[:, :, i] - sla.expm(-1j * (t - 0.2) * D) @ V).max() < 1e-10 * np.abs(V).max()
    im = qs.evolve(H, V, 0.0, 1.0, imag_time=True)
    assert im.shape == (b.Ns, 4)
    ref = sla.expm(-1.0 * D) @ V
    ref /= np.linalg.norm(ref, axis=0)
    assert np.abs(im - ref).max() < 1e-10


def test_stepwise_evolution(qs, ora):
    """evolve(..., stepwise=True) propagates from each time to the next: the
    states of the reference-faithful evolve to the tolerance, for times in any
    order, repeated, and before t0, in real and imaginary time."""
    import scipy.linalg as sla
    L = 12
    spec = models.xxz(L, 1.0, 0.7) + [("z", [(0.2, i) for i in range(1, L + 1)])]
    b = qs.SpinBasis1D(L, nup=6, pauli=False, kblock=3)
    H = qs.Hamiltonian(b, models.to_terms(qs, spec))
    rep = ora.RepBasis(L, nup=6, pauli=False, kblock=3)
    D = np.column_stack([rep.matvec(spec, np.eye(b.Ns, dtype=complex)[:, j]) for j in range(b.Ns)])
    v0 = models.seeded(b.Ns, seed=8, complex_=True)
    v0 /= np.linalg.norm(v0)
    times = [3.0, 0.5, 7.5, 0.5, -1.0, 0.1]
    got = qs.evolve(H, v0, 0.1, times, tol=1e-11, stepwise=True)
    ref = qs.evolve(H, v0, 0.1, times, tol=1e-11)
    for i, t in enumerate(times):
        want = sla.expm(-1j * (t - 0.1) * D) @ v0
        assert np.linalg.norm(got[:, i] - want) < 1e-9, t
        assert np.linalg.norm(got[:, i] - ref[:, i]) < 1e-9, t
    im = qs.evolve(H, v0, 0.0, [0.4, 1.2], imag_time=True, stepwise=True)
    for i, tau in enumerate((0.4, 1.2)):
        want = sla.expm(-tau * D) @ v0
        want /= np.linalg.norm(want)
        assert np.linalg.norm(im[:, i] - want) < 1e-9


def _dense_from_oracle(ora, L, nup, pauli, sym, sp):
    rep = ora.RepBasis(L, nup=nup, pauli=pauli, **sym)
    n = rep.Ns
    D = np.zeros((n, n), dtype=np.complex128)
    e = np.zeros(n, dtype=np.complex128)
    for j in range(n):
        e[:] = 0
        e[j] = 1
        D[:, j] = rep.matvec(sp, e)
    return D


def _expected(w, which, k):
    """The reference's selection and order (src/operators.jl:1587-1596, 3393-3401)."""
    if which == "SA":
        return np.sort(w)[:k]
    if which == "LA":
        return np.sort(w)[::-1][:k]
    if which == "LM":
        return w[np.argsort(-np.abs(w), kind="stable")][:k]
    if which == "SM":
        return w[np.argsort(np.abs(w), kind="stable")][:k]
    ws = np.sort(w)
    return np.sort(np.concatenate([ws[:k // 2], ws[len(ws) - (k - k // 2):]]))[::-1]


def _check_which(vals, w, which, k, tol):
    """Same values as the reference selects (as a set: magnitudes that tie to
    rounding may come in either order) and the reference's order."""
    want = _expected(w, which, k)
    assert np.allclose(np.sort(vals), np.sort(want), rtol=tol, atol=tol * np.abs(w).max()), (which, vals, want)
    key = {"SA": vals, "LA": -vals, "LM": -np.abs(vals), "SM": np.abs(vals), "BE": -vals}[which]
    assert np.all(np.diff(key) >= -tol * np.abs(w).max()), (which, vals)


@pytest.mark.parametrize("which", ["SA", "LA", "LM", "SM", "BE"])
def test_eigsh_which_matches_dense(qs, ora, which):
    """which = SA / LA / LM / SM / BE on the matrix-free, assembled (FP64 and
    double-float engines) and FP32 + polish paths, and on the dense branch."""
    L, nup, sym = 14, 7, dict(kblock=0, pblock=1, zblock=1)
    sp = models.j1j2(L, 1.0, 0.37)   # no exact degeneracies (J2 = 0.5 has some)
    b = qs.SpinBasis1D(L, nup=nup, pauli=False, **sym)
    D = _dense_from_oracle(ora, L, nup, False, sym, sp)
    w = np.linalg.eigvalsh(D)
    k = 4
    scale = float(np.abs(w).max())
    Q = qs.QuantumLinearOperator(b, models.to_terms(qs, sp))
    H = qs.Hamiltonian(b, models.to_terms(qs, sp))
    for op, prec in ((Q, "fp64"), (H, "fp64"), (H, "fp64df"), (H, "fp32")):
        vals, vecs = qs.eigsh(op, k=k, which=which, tol=1e-12, ncv=40, maxiter=3000, precision=prec)
        _check_which(vals, w, which, k, 1e-10)
        assert np.max(np.abs(D @ vecs - vecs * vals)) < 1e-7 * scale, prec
    # k >= Ns - 1 takes the dense branch
    small = qs.SpinBasis1D(8, nup=4, pauli=False, kblock=0, pblock=1)
    sps = models.j1j2(8, 1.0, 0.37)
    Ds = _dense_from_oracle(ora, 8, 4, False, dict(kblock=0, pblock=1), sps)
    ws = np.linalg.eigvalsh(Ds)
    ks = small.Ns - 1
    got = qs.eigsh(qs.QuantumLinearOperator(small, models.to_terms(qs, sps)), k=ks, which=which,
                   return_eigenvectors=False)
    _check_which(got, ws, which, ks, 1e-10)


def test_eigsh_batch_which(qs, ora):
    L = 12
    sp = models.j1j2(L, 1.0, 0.37)
    syms = [dict(kblock=0, pblock=1), dict(kblock=3), dict(kblock=6, pblock=-1)]
    ops = [qs.Hamiltonian(qs.SpinBasis1D(L, nup=6, pauli=False, **sy), models.to_terms(qs, sp)) for sy in syms]
    for which in ("LM", "BE"):
        got = qs.eigsh_batch(ops, k=3, which=which, tol=1e-12, ncv=30, maxiter=3000)
        for i, sy in enumerate(syms):
            w = np.linalg.eigvalsh(_dense_from_oracle(ora, L, 6, False, sy, sp))
            _check_which(got[i], w, which, 3, 1e-10)


def _expected_complex(w, which, k):
    """The reference's ARPACK selection for a non-Hermitian operator (:SR / :LR
    for SA / LA, magnitude for LM / SM) in its output order."""
    key = {"SA": w.real, "LA": -w.real, "LM": -np.abs(w), "SM": np.abs(w)}[which]
    return w[np.argsort(key, kind="stable")][:k]


@pytest.mark.parametrize("which", ["SA", "LA", "LM", "SM"])
@pytest.mark.parametrize("cplx", [True, False])
def test_eigsh_non_hermitian(qs, ora, which, cplx):
    """eigsh of a non-Hermitian operator returns complex eigenvalues and
    vectors (src/operators.jl:3402-3404): Krylov-Schur against the dense
    spectrum, and the dense branch for k >= Ns - 1."""
    L = 12
    bonds = [(i, i % L + 1) for i in range(1, L + 1)]
    a = 0.7 + 0.25j if cplx else 0.7
    sp = [("+-", [(a, i, j) for i, j in bonds]), ("-+", [(0.3, i, j) for i, j in bonds]),
          ("zz", [(0.45, i, j) for i, j in bonds]), ("z", [(0.1 * (i % 3), i) for i in range(1, L + 1)])]
    b = qs.SpinBasis1D(L, nup=6, pauli=False)
    # SM without a shift-invert wants interior eigenvalues (a degenerate
    # cluster near zero here): a diagonal shift makes them the left edge
    shift = np.full(b.Ns, 3.0) if which == "SM" else None
    op = qs.QuantumLinearOperator(b, models.to_terms(qs, sp), diagonal=shift, check_herm=False)
    assert not op.hermitian
    M = ora.RefBasis(L, nup=6, pauli=False).dense(ora.consolidate_terms(sp))
    if shift is not None:
        M = M + np.diag(shift)
    w = np.linalg.eigvals(M)
    k = 4
    vals, vecs = qs.eigsh(op, k=k, which=which, tol=1e-12, ncv=40, maxiter=3000)
    assert vals.dtype == np.complex128 and vecs.dtype == np.complex128
    want = _expected_complex(w, which, k)
    scale = float(np.abs(w).max())
    # the same values (near-ties in the ranking may swap), then each pair's residual
    for v in want:
        assert np.min(np.abs(vals - v)) <= 1e-9 * scale, (which, vals, want)
    assert np.max(np.linalg.norm(M @ vecs - vecs * vals, axis=0)) <= 1e-8 * scale
    assert np.allclose(np.linalg.norm(vecs, axis=0), 1.0, atol=1e-10)
    # dense branch
    bs = qs.SpinBasis1D(6, nup=3, pauli=False)
    bonds6 = [(i, i % 6 + 1) for i in range(1, 7)]
    sp6 = [("+-", [(a, i, j) for i, j in bonds6]), ("-+", [(0.3, i, j) for i, j in bonds6]),
           ("zz", [(0.45, i, j) for i, j in bonds6])]
    ops = qs.QuantumLinearOperator(bs, models.to_terms(qs, sp6), check_herm=False)
    Ms = ora.RefBasis(6, nup=3, pauli=False).dense(ora.consolidate_terms(sp6))
    ws = np.linalg.eigvals(Ms)
    ks = bs.Ns - 1
    got = qs.eigsh(ops, k=ks, which=which, return_eigenvectors=False)
    for v in _expected_complex(ws, which, ks):
        assert np.min(np.abs(got - v)) <= 1e-10 * max(1.0, np.abs(ws).max())


@pytest.mark.parametrize("prec", ["fp64", "fp32", "fp64fx"])
def test_page_locked_output_written_in_place(qs, ora, prec):
    """With a page-locked output and beta = 0 the product writes y through its
    mapped address (no device copy of y): the same values as pageable output."""
    torch = pytest.importorskip("torch")
    import ctypes
    from qsgpu import _lib
    lib = _lib.load()
    L = 16
    b = qs.SpinBasis1D(L, nup=8, pauli=False, kblock=0, pblock=1, zblock=1)
    for op in (qs.Hamiltonian(b, models.to_terms(qs, models.j1j2(L, 1.0, 0.5))),
               qs.QuantumLinearOperator(b, models.to_terms(qs, models.j1j2(L, 1.0, 0.5)))):
        if prec == "fp64fx" and not getattr(op, "fixed_point_classes", 0):
            continue
        dt = torch.float32 if prec == "fp32" else torch.float64
        code = _lib.QS_F32 if prec == "fp32" else _lib.QS_F64
        flags = _lib.QS_FIXED_POINT if prec == "fp64fx" else 0
        x = torch.from_numpy(models.seeded(b.Ns)).to(dt)
        xp = torch.empty(b.Ns, dtype=dt, pin_memory=True)
        xp.copy_(x)
        yp = torch.full((b.Ns,), float("nan"), dtype=dt, pin_memory=True)
        ypage = np.full(b.Ns, np.nan, dtype=np.float32 if prec == "fp32" else np.float64)
        one, zero = np.array([1.0, 0.0]), np.array([0.0, 0.0])
        for y, ptr in ((yp, ctypes.c_void_p(yp.data_ptr())), (ypage, _lib.ptr(ypage))):
            _lib.check(lib.qs_op_matvec(op._h, flags, _lib.ptr(one), ctypes.c_void_p(xp.data_ptr()), code,
                                        _lib.ptr(zero), ptr, code, 1, _lib.QS_MEM_HOST))
        assert np.array_equal(yp.numpy(), ypage)
        want = op.dot(models.seeded(b.Ns))
        tol = 2e-5 if prec == "fp32" else 1e-13
        assert np.max(np.abs(yp.numpy() - want)) <= tol * max(1.0, np.abs(want).max())


def test_transient_assembly_of_matrix_free_solvers(qs, ora, monkeypatch):
    """eigsh / evolve on a matrix-free operator of at least 4,096 states run on an
    assembled form built for the call and dropped after it: the same results
    as the matrix-free solve (QS_TRANSIENT_ASSEMBLY=0) and ARPACK over the
    oracle's product, and the operator left matrix-free (no stored nonzeros)."""
    from qsgpu import _lib
    L = 24
    sym = dict(kblock=0)
    sp = models.j1j2(L, 1.0, 0.37)
    b = qs.SpinBasis1D(L, nup=12, pauli=False, **sym)
    assert b.Ns >= 4096
    Q = qs.QuantumLinearOperator(b, models.to_terms(qs, sp))
    v0 = models.seeded(b.Ns, seed=5)
    v = models.seeded(b.Ns, seed=6, complex_=True)
    v /= np.linalg.norm(v)
    got = {}
    for mode in ("1", "0"):
        monkeypatch.setenv("QS_TRANSIENT_ASSEMBLY", mode)
        e = qs.eigsh(Q, k=2, which="SA", tol=1e-12, v0=v0, return_eigenvectors=False)
        st = qs.evolve(Q, v, 0.0, [0.5, 1.5], tol=1e-10)
        got[mode] = (e, st)
        assert _lib.load().qs_op_nnz(Q._h) < 0   # not assembled after the calls
    rep = ora.RepBasis(L, nup=12, pauli=False, **sym)
    pk = ora.pack_terms(sp)
    d = rep.diagonal(sp)
    want, _ = ora.eigsh_arpack(lambda x: rep.matvec(sp, x, diag=d, packed=pk).real, b.Ns, 2, np.float64, v0=v0,
                               tol=1e-13)
    assert np.max(np.abs(np.sort(got["1"][0]) - np.sort(want))) <= 1e-10 * np.abs(want).max()
    assert np.max(np.abs(got["1"][0] - got["0"][0])) <= 1e-10 * np.abs(got["0"][0]).max()
    assert np.max(np.linalg.norm(got["1"][1] - got["0"][1], axis=0)) <= 1e-9
