"""The oracle against the reference's own known answers (no GPU)."""
import numpy as np
import pytest

import models


def _terms_xxz4(k):
    jxy = np.sqrt(2.0)
    t = k["terms"]
    return [("+-", [(jxy / 2, a, b) for a, b in t[0][2]]), ("-+", [(jxy / 2, a, b) for a, b in t[1][2]]),
            ("zz", [(1.0, a, b) for a, b in t[2][2]]), ("z", [(1 / np.sqrt(3.0), s[0]) for s in t[3][2]])]


def test_spin_basis_states(ora, kats):
    k = kats["spin_basis_1d_L4_nup2_states"]
    b = ora.RefBasis(k["L"], nup=k["nup"], pauli=k["pauli"])
    assert sorted(int(s) for s in b.states) == k["states"]
    for i, s in enumerate(b.states):
        assert b.state_index(s) == i


def test_xxz_spectrum(ora, kats):
    k = kats["xxz_L4_spectrum"]
    b = ora.RefBasis(k["L"], nup=k["nup"], pauli=k["pauli"])
    H = b.dense(ora.consolidate_terms(_terms_xxz4(k)))
    assert np.allclose(H, H.conj().T, atol=1e-15)
    w = np.linalg.eigvalsh(H)
    assert np.allclose(w, k["eigenvalues"], atol=k["atol"], rtol=k["atol"])
    assert abs(np.trace(H).real - k["trace"]) < k["atol"]
    assert abs(np.linalg.norm(H) - k["frobenius"]) < k["atol"]


def test_qlo_protocol(ora, kats):
    k = kats["qlo_protocol_L3"]
    b = ora.RefBasis(k["L"], nup=k["nup"], pauli=k["pauli"])
    terms = [(op, [tuple(c) for c in cs]) for op, cs in k["terms"]]
    diag = np.array(k["diagonal"])
    M = b.dense(ora.consolidate_terms(terms), diag=diag)
    v = np.array([complex(*c) for c in k["vector_unnormalized"]])
    v /= np.linalg.norm(v)
    dest = np.array([complex(*c) for c in k["destination"]])
    out = b.qlo_matvec(ora.consolidate_terms(terms), v, alpha=k["alpha"], beta=k["beta"], y=dest.copy(), diag=diag)
    assert np.allclose(out, k["alpha"] * (M @ v) + k["beta"] * dest, atol=k["atol"])
    # transpose / conj / adjoint flags against the materialised matrix
    for T, C, ref in ((True, False, M.T), (False, True, M.conj()), (True, True, M.conj().T)):
        got = b.qlo_matvec(ora.consolidate_terms(terms), v, diag=diag, transposed=T, conjugated=C)
        assert np.allclose(got, ref @ v, atol=1e-15)


def test_expm_rotation(ora, kats):
    k = kats["expm_rotation_2x2"]
    G = np.array(k["generator"])
    got = ora.krylov_expmv_vector(lambda x: G @ x, np.array([1.0, 0.0]), k["a"], hermitian=False)
    assert np.allclose(got, [np.cos(0.25), np.sin(0.25)], atol=k["atol"])


def test_physical_sectors_union(ora, kats):
    k = kats["physical_sectors_L4"]
    L = k["L"]
    bonds = [(i, i % L + 1) for i in range(1, L + 1)]
    terms = [(op, [(c, a, b) for a, b in bonds]) for op, c in k["terms"]]
    full = np.sort(np.linalg.eigvalsh(ora.RefBasis(L, nup=2, pauli=False).dense(terms)))
    for kw_list in ([dict(kblock=q) for q in range(L)], [dict(pblock=p) for p in (-1, 1)],
                    [dict(zblock=z) for z in (-1, 1)]):
        ev = []
        for kw in kw_list:
            b = ora.RefBasis(L, nup=2, pauli=False, **kw)
            P = b.projector().toarray()
            assert np.allclose(P.conj().T @ P, np.eye(b.Ns), atol=3e-13)
            ev.extend(np.linalg.eigvalsh(b.dense(terms)))
        assert np.allclose(np.sort(ev), full, atol=k["atol"])


def test_translation_sector_projection(ora, kats):
    k = kats["translation_sector_L8"]
    L = k["L"]
    bonds = [(i, i % L + 1) for i in range(1, L + 1)]
    terms = [(op, [(c, a, b) for a, b in bonds]) for op, c in k["terms"]]
    red = ora.RefBasis(L, nup=4, pauli=False, kblock=0)
    par = ora.RefBasis(L, nup=4, pauli=False)
    P = red.projector().toarray()
    assert np.allclose(red.dense(terms), P.conj().T @ par.dense(terms) @ P, atol=k["atol"])


def test_unchecked_symmetric_qlo(ora, kats):
    k = kats["unchecked_symmetric_qlo"]
    red = ora.RefBasis(k["L"], nup=k["nup"], pauli=False, kblock=0)
    par = ora.RefBasis(k["L"], nup=k["nup"], pauli=False)
    terms = [(op, [tuple(c) for c in cs]) for op, cs in k["terms"]]
    P = red.projector().toarray()
    v = models.seeded(red.Ns, complex_=True)
    got = red.qlo_matvec(terms, v, extract=False)
    assert np.allclose(got, P.conj().T @ par.dense(terms) @ P @ v, atol=k["atol"])


def test_matrix_free_krylov(ora, kats):
    k = kats["matrix_free_krylov_L8"]
    L = k["L"]
    bonds = [(i, i % L + 1) for i in range(1, L + 1)]
    terms = [(op, [(c, a, b) for a, b in bonds]) for op, c in k["terms"]]
    b = ora.RefBasis(L, nup=4, pauli=False)
    H = b.dense(terms)
    n = b.Ns
    idx = np.arange(1, n + 1)
    v = np.sin(idx) + 1j * np.cos(2 * idx)
    v /= np.linalg.norm(v)
    import scipy.linalg as sla
    st = ora.krylov_expmv_times(lambda x: H @ x, v, [-1j * t for t in k["times"]], hermitian=True)
    assert np.allclose(st[:, -1], sla.expm(-1j * k["times"][-1] * H) @ v, atol=k["evolve_atol"])
    assert all(abs(np.linalg.norm(st[:, j]) - 1) < k["norm_atol"] for j in range(st.shape[1]))
    a = complex(*k["expm_a"])
    got = ora.krylov_expmv_vector(lambda x: H @ x, v, a, hermitian=True)
    assert np.allclose(got, sla.expm(a * H) @ v, atol=k["evolve_atol"])
    vals, vecs = ora.eigsh_arpack(lambda x: H @ x, n, 2, np.complex128)
    assert np.allclose(H @ vecs, vecs * vals, atol=k["eigsh_atol"])


@pytest.mark.parametrize("L", [8, 10, 12])
def test_two_restatements_agree(ora, L):
    """The reference-algorithm oracle and the representative-space restatement
    build the same sectors and the same reduced matrices."""
    for kw in (dict(kblock=0, pblock=1, zblock=1), dict(kblock=1), dict(kblock=L // 2, pblock=-1),
               dict(kblock=2, zblock=-1), dict(pblock=1), dict(zblock=1)):
        ref = ora.RefBasis(L, nup=L // 2, pauli=False, **kw)
        rep = ora.RepBasis(L, nup=L // 2, pauli=False, **kw)
        assert ref.Ns == rep.Ns
        terms = models.j1j2(L, 1.0, 0.5)
        x = models.seeded(ref.Ns, complex_=True)
        assert np.allclose(ref.qlo_matvec(terms, x), rep.matvec(terms, x), atol=1e-12)


def test_krylov_tools(ora, kats):
    """lanczos_full / lanczos_iter / lin_comb_Q_T / expm_lanczos / FTLM / LTLM
    restatements against test/runtests.jl:130-172."""
    k = kats["krylov_tools_4x4"]
    A = np.array(k["A"])
    B = np.diag(k["B_diagonal"])
    v0 = np.array(k["v0"])
    E, V, Q = ora.lanczos_full(lambda x: A @ x, v0, k["m"])
    assert np.allclose(E, k["E"], atol=k["E_atol"], rtol=0)
    assert np.allclose(Q @ Q.T, np.eye(k["m"]), atol=k["orthonormal_atol"], rtol=0)
    assert np.allclose(ora.lin_comb_Q_T(k["lin_comb_coeff"], Q), k["lin_comb"], atol=k["lin_comb_atol"], rtol=0)
    assert np.allclose(ora.expm_lanczos(E, V, Q, a=k["expm_a"]), k["expm_lanczos"], atol=k["expm_atol"], rtol=0)
    a, b, _ = ora.lanczos_coefficients(lambda x: A @ x, v0, k["m"])
    rows = np.array(list(ora.lanczos_vectors(lambda x: A @ x, v0, a, b)))
    assert np.allclose(rows, Q, atol=k["iter_atol"], rtol=0)
    obs = {"A": lambda x: A @ x, "B": lambda x: B @ x}
    f, fi = ora.ftlm_static_iteration(obs, E, V, Q, beta=k["beta"])
    lt, li = ora.ltlm_static_iteration(obs, E, V, Q, beta=k["beta"])
    assert np.allclose(fi, k["ftlm_identity"], atol=k["ftlm_identity_atol"], rtol=0)
    assert np.allclose(f["B"], k["ftlm_B"], atol=k["ftlm_B_atol"], rtol=0)
    assert np.allclose(li, fi, atol=k["ftlm_identity_atol"], rtol=0)
    assert np.allclose(lt["B"], k["ltlm_B"], atol=k["ltlm_B_atol"], rtol=0)
    with pytest.raises(ora.OracleError):
        ora.lanczos_full(lambda x: A @ x, v0, 4)
    with pytest.raises(ora.OracleError):
        ora.lanczos_full(lambda x: A @ x, np.zeros(4), 2)


def test_general_maps_restate_the_1d_blocks(ora):
    """SpinBasisGeneral's projector algorithm over general maps (translation,
    reflection) gives the 1D SpinBasis1D sectors: the same projector and
    representatives (q = 0 / 1 of an order-2 map is the block +1 / -1)."""
    L = 8
    T = [(i + 1) % L for i in range(L)]
    P = [L - 1 - i for i in range(L)]
    for k in range(L):
        g = ora.general_basis(L, nup=4, pauli=False, blocks=[(T, k)])
        r = ora.RefBasis(L, nup=4, pauli=False, kblock=k)
        assert np.array_equal(g.states, r.states)
        assert np.abs(g.projector().toarray() - r.projector().toarray()).max() == 0
    for qk, qp, kb, pb in ((0, 0, 0, 1), (0, 1, 0, -1), (4, 0, 4, 1), (4, 1, 4, -1)):
        g = ora.general_basis(L, nup=4, pauli=False, blocks=[(T, qk), (P, qp)])
        r = ora.RefBasis(L, nup=4, pauli=False, kblock=kb, pblock=pb)
        assert np.array_equal(g.states, r.states)
        assert np.abs(g.projector().toarray() - r.projector().toarray()).max() < 1e-15


def test_general_columns_are_anchored_orbit_states(ora):
    """On a 4 x 3 torus with (kx, ky, flip) blocks, every column of the
    reference projector is an orbit state: uniform magnitude, real positive
    at its orbit minimum, columns in ascending orbit minimum."""
    import models
    Tx, Ty, Px, Z = models.torus_maps(4, 3)
    for qx, qy, qz in ((0, 0, 0), (1, 0, 1), (2, 1, 0), (3, 2, 1)):
        g = ora.general_basis(12, nup=6, pauli=False, blocks=[(Tx, qx), (Ty, qy), (Z, qz)])
        P = g.projector().tocsc()
        P.sort_indices()
        mins = []
        for j in range(P.shape[1]):
            rows = P.indices[P.indptr[j]:P.indptr[j + 1]]
            vals = P.data[P.indptr[j]:P.indptr[j + 1]]
            assert np.allclose(np.abs(vals), np.abs(vals[0]), rtol=1e-13, atol=0)
            assert abs(vals[0].imag) < 1e-13 and vals[0].real > 0          # rows ascending: first = orbit minimum
            mins.append(int(g.parent_states[rows[0]]))
        assert mins == sorted(mins)
