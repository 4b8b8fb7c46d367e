"""Device results against the oracle at the sizes of the benchmarked workloads.

* J1-J2 chain L=32, nup=16, k=0, p=+1, z=+1 (N = 4,707,969): every orbit
  minimum and orbit size bit-exact against the oracle's representative-space
  restatement; the assembled product (FP64, double-float, fixed-point row sums,
  FP32) and the matrix-free product on three 4096-row ranges spread over the
  sector against the oracle's product of the same rows.
* TFIM L=30, k=0, p=+1, no particle number (N = 17,920,860): the same with a
  complex vector.
* J1-J2 chain L=26, nup=13, J2=0.3: whole-sector products of a complex sector
  (k=3) and of k=13, p=-1.
* The same shapes at L=20-22: reference-algorithm representatives bit-exact,
  whole-sector products against the reference algorithm, eigsh k=1 against
  ARPACK over the oracle's product, evolve against the oracle's Krylov
  restatement.

Tolerances: products 1e-13 of the largest entry (FP32: 2e-5), eigenvalues 1e-10
relative, evolved states 1e-9 in 2-norm.
"""
import numpy as np
import pytest

import models

pytestmark = pytest.mark.gpu

ROWS = 4096


def row_ranges(n):
    return [(0, ROWS), (n // 2, n // 2 + ROWS), (n - ROWS, n)]


def check_rows(got, want, tol, what):
    scale = max(1.0, float(np.abs(want).max()))
    err = float(np.max(np.abs(got - want)))
    assert err <= tol * scale, (what, err, scale)


def orbit_sizes(b):
    return (b.group_order // b.stabilizers().astype(np.int64)).astype(np.int64)


@pytest.fixture(scope="module")
def config2(qs, ora):
    L = 32
    sym = dict(kblock=0, pblock=1, zblock=1)
    b = qs.SpinBasis1D(L, nup=16, pauli=False, **sym)
    rep = ora.RepBasis(L, nup=16, pauli=False, **sym)
    return b, rep, models.j1j2(L, 1.0, 0.5)


def test_config2_representatives_bit_exact(config2):
    b, rep, _ = config2
    assert b.Ns == rep.Ns == 4707969
    assert np.array_equal(b.orbit_minima(), rep.states)
    assert np.array_equal(orbit_sizes(b), rep.orbit.astype(np.int64))
    # state_index of a sample of representatives
    idx = np.arange(0, b.Ns, 997)
    assert np.array_equal(b.index_array(rep.states[idx]), idx)


def test_config2_products_on_row_ranges(qs, ora, config2):
    b, rep, sp = config2
    n = b.Ns
    H = qs.Hamiltonian(b, models.to_terms(qs, sp))
    Q = qs.QuantumLinearOperator(b, models.to_terms(qs, sp))
    x = models.seeded(n)
    pk = ora.pack_terms(sp)
    d = rep.diagonal(sp)
    y64 = H.dot(x)
    ydf = H.dot(x, precision="fp64df")
    yfx = H.dot(x, precision="fp64fx")
    y32 = H.dot(x.astype(np.float32), precision="fp32")
    ymf = Q.dot(x)
    for r0, r1 in row_ranges(n):
        want = rep.matvec(sp, x, diag=d, rows=(r0, r1), packed=pk)[r0:r1]
        assert np.max(np.abs(want.imag)) == 0.0
        want = want.real
        check_rows(y64[r0:r1], want, 1e-13, ("fp64", r0))
        check_rows(ydf[r0:r1], want, 1e-13, ("fp64df", r0))
        check_rows(yfx[r0:r1], want, 1e-13, ("fp64fx", r0))
        check_rows(ymf[r0:r1], want, 1e-13, ("matrix-free", r0))
        check_rows(y32[r0:r1], want, 2e-5, ("fp32", r0))


def test_config3_representatives_and_products(qs, ora):
    L = 30
    sym = dict(kblock=0, pblock=1)
    sp = models.tfim(L, 1.0, 0.7)
    b = qs.SpinBasis1D(L, pauli=True, **sym)
    rep = ora.RepBasis(L, pauli=True, **sym)
    assert b.Ns == rep.Ns == 17920860
    assert np.array_equal(b.orbit_minima(), rep.states)
    assert np.array_equal(orbit_sizes(b), rep.orbit.astype(np.int64))
    n = b.Ns
    H = qs.Hamiltonian(b, models.to_terms(qs, sp))
    Q = qs.QuantumLinearOperator(b, models.to_terms(qs, sp))
    x = models.seeded(n, complex_=True)
    pk = ora.pack_terms(sp)
    d = rep.diagonal(sp)
    y64 = H.dot(x)
    ydf = H.dot(x, precision="fp64df")
    ymf = Q.dot(x)
    for r0, r1 in row_ranges(n):
        want = rep.matvec(sp, x, diag=d, rows=(r0, r1), packed=pk)[r0:r1]
        check_rows(y64[r0:r1], want, 1e-13, ("fp64", r0))
        check_rows(ydf[r0:r1], want, 1e-13, ("fp64df", r0))
        check_rows(ymf[r0:r1], want, 1e-13, ("matrix-free", r0))


@pytest.mark.parametrize("sym", [dict(kblock=3), dict(kblock=13, pblock=-1), dict(kblock=0, pblock=1)])
def test_config4_sectors_whole(qs, ora, sym):
    L = 26
    sp = models.j1j2(L, 1.0, 0.3)
    b = qs.SpinBasis1D(L, nup=13, pauli=False, **sym)
    rep = ora.RepBasis(L, nup=13, pauli=False, **sym)
    assert np.array_equal(b.orbit_minima(), rep.states)
    H = qs.Hamiltonian(b, models.to_terms(qs, sp))
    Q = qs.QuantumLinearOperator(b, models.to_terms(qs, sp))
    x = models.seeded(b.Ns, complex_=True)
    want = rep.matvec(sp, x)
    check_rows(H.dot(x), want, 1e-13, "fp64")
    check_rows(H.dot(x, precision="fp64df"), want, 1e-13, "fp64df")
    check_rows(Q.dot(x), want, 1e-13, "matrix-free")


MID = [
    # config-2 shape, config-4 shape (complex sector), config-3 shape
    (22, 11, False, dict(kblock=0, pblock=1, zblock=1), "j1j2_05"),
    (22, 11, False, dict(kblock=5), "j1j2_03"),
    (20, None, True, dict(kblock=0, pblock=1), "tfim"),
]


def mid_spec(model, L):
    if model == "j1j2_05":
        return models.j1j2(L, 1.0, 0.5)
    if model == "j1j2_03":
        return models.j1j2(L, 1.0, 0.3)
    return models.tfim(L, 1.0, 0.7)


@pytest.mark.parametrize("L,nup,pauli,sym,model", MID)
def test_mid_size_against_reference_algorithm(qs, ora, L, nup, pauli, sym, model):
    sp = mid_spec(model, L)
    ref = ora.RefBasis(L, nup=nup, pauli=pauli, **sym)
    b = qs.SpinBasis1D(L, nup=nup, pauli=pauli, **sym)
    assert np.array_equal(b.states, ref.states)
    ct = ora.consolidate_terms(sp)
    x = models.seeded(b.Ns, complex_=True)
    want = ref.qlo_matvec(ct, x)
    H = qs.Hamiltonian(b, models.to_terms(qs, sp))
    Q = qs.QuantumLinearOperator(b, models.to_terms(qs, sp))
    check_rows(H.dot(x), want, 1e-13, "assembled")
    check_rows(Q.dot(x), want, 1e-13, "matrix-free")


@pytest.mark.parametrize("L,nup,pauli,sym,model", MID)
def test_mid_size_eigsh_and_evolve(qs, ora, L, nup, pauli, sym, model):
    sp = mid_spec(model, L)
    rep = ora.RepBasis(L, nup=nup, pauli=pauli, **sym)
    b = qs.SpinBasis1D(L, nup=nup, pauli=pauli, **sym)
    H = qs.Hamiltonian(b, models.to_terms(qs, sp))
    n = b.Ns
    pk = ora.pack_terms(sp)
    d = rep.diagonal(sp)
    cx = H.dtype == np.complex128

    def mv(v):
        y = rep.matvec(sp, v, diag=d, packed=pk)
        return y if cx else y.real

    v0 = models.seeded(n, seed=11, complex_=cx)
    want, _ = ora.eigsh_arpack(mv, n, 1, np.complex128 if cx else np.float64, v0=v0, tol=1e-13)
    for prec in ("fp64", "fp32", "fp64df"):
        got = qs.eigsh(H, k=1, which="SA", tol=1e-10, v0=v0, precision=prec, return_eigenvectors=False)
        assert abs(got[0] - want[0]) <= 1e-10 * abs(want[0]), (prec, got[0], want[0])
    got = qs.eigsh(qs.QuantumLinearOperator(b, models.to_terms(qs, sp)), k=1, which="SA", tol=1e-10, v0=v0,
                   return_eigenvectors=False)
    assert abs(got[0] - want[0]) <= 1e-10 * abs(want[0])
    v = models.seeded(n, seed=3, complex_=True)
    v /= np.linalg.norm(v)
    times = [0.5, 2.0]
    ref_states = ora.krylov_expmv_times(lambda z: rep.matvec(sp, z, diag=d, packed=pk), v,
                                        [-1j * t for t in times], hermitian=True, tol=1e-9)
    for prec in ("fp64", "fp64df"):
        st = qs.evolve(H, v, 0.0, times, tol=1e-9, precision=prec)
        assert np.max(np.linalg.norm(st - ref_states, axis=0)) < 1e-9, prec
