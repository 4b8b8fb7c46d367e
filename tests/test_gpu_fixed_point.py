"""The fixed-point form of the assembled product (precision="fp64fx",
QS_FIXED_POINT): FP64 vectors, row sums carried exactly in 64-bit integers.
Checked against the oracle's FP64 restatement of the reference product
(src/operators.jl:2554-2636) and against the device's FP64 product, normwise,
with the tolerance written in each assert; non-finite input, extreme scales,
alpha / beta, the adjoint and the row-range host path included."""
import numpy as np
import pytest

import models

pytestmark = pytest.mark.gpu

# (L, nup, pauli, symmetries, model, expected classes: 0 = FP64 fallback)
CASES = [
    (12, 6, False, dict(kblock=0, pblock=1, zblock=1), "j1j2", 2),
    (12, 6, False, dict(kblock=0, pblock=-1), "j1j2", 2),
    (12, 6, False, dict(kblock=6, pblock=1, zblock=-1), "xxz", 1),
    (10, 5, False, dict(), "xxz", 1),
    (12, None, True, dict(kblock=0, pblock=1), "tfim", 1),
    (12, 6, False, dict(kblock=1), "j1j2", 0),          # complex characters
    (10, None, False, dict(kblock=2), "xyz", 0),         # complex operator
]


def spec(model, L):
    return {"xxz": lambda: models.xxz(L, 1.0, 0.5), "j1j2": lambda: models.j1j2(L, 1.0, 0.5),
            "tfim": lambda: models.tfim(L, 1.0, 0.7), "xyz": lambda: models.xyz_field(L)}[model]()


def build(qs, ora, L, nup, pauli, sym, model):
    sp = spec(model, L)
    b = qs.SpinBasis1D(L, nup=nup, pauli=pauli, **sym)
    H = qs.Hamiltonian(b, models.to_terms(qs, sp))
    ref = ora.RefBasis(L, nup=nup, pauli=pauli, **sym)
    return H, ref, ora.consolidate_terms(sp)


@pytest.mark.parametrize("L,nup,pauli,sym,model,ncls", CASES)
def test_fixed_point_matches_reference(qs, ora, L, nup, pauli, sym, model, ncls):
    H, ref, terms = build(qs, ora, L, nup, pauli, sym, model)
    assert H.assembled and H.fixed_point_classes == ncls
    x = models.seeded(H.Ns, complex_=True)
    want = ref.qlo_matvec(terms, x)
    scale = max(1.0, np.abs(want).max())
    y = H.dot(x, precision="fp64fx")
    # normwise FP64 accuracy: every row within 1e-13 of the largest entry
    assert np.max(np.abs(y - want)) <= 1e-13 * scale
    assert np.max(np.abs(y - H.dot(x))) <= 1e-13 * scale
    assert np.max(np.abs(H.H.dot(x, precision="fp64fx") - H.H.dot(x))) <= 1e-13 * scale
    if H.dtype == np.float64:
        xr = models.seeded(H.Ns, seed=7)
        assert np.max(np.abs(H.dot(xr, precision="fp64fx") - ref.qlo_matvec(terms, xr))) <= 1e-13 * scale
    # alpha and beta: y = alpha H x + beta y0
    y0 = models.seeded(H.Ns, seed=11, complex_=True)
    out = y0.copy()
    H.mul(out, x, alpha=0.5 - 0.25j, beta=-1.5 + 0.5j, precision="fp64fx")
    assert np.max(np.abs(out - ((0.5 - 0.25j) * want + (-1.5 + 0.5j) * y0))) <= 1e-13 * scale


def test_fixed_point_scales_zero_and_non_finite(qs, ora):
    """Inputs at 1e-300 and 1e300 (the power-of-two scale leaves the range it
    folds into the row scale), the zero vector, and NaN / inf entries (no
    fixed-point scale exists: the rows are computed as by the FP64 product)."""
    H, ref, terms = build(qs, ora, 18, 9, False, dict(kblock=0, pblock=1, zblock=1), "j1j2")
    assert H.fixed_point_classes == 2
    x = models.seeded(H.Ns)
    want = ref.qlo_matvec(terms, x).real
    for s in (1e-300, 1e-200, 1e200, 1e300):
        y = H.dot(x * s, precision="fp64fx")
        assert np.max(np.abs(y / s - want)) <= 1e-13 * np.abs(want).max(), s
    assert np.array_equal(H.dot(np.zeros(H.Ns), precision="fp64fx"), np.zeros(H.Ns))
    xb = x.copy()
    xb[3] = np.nan
    xb[17] = np.inf
    y = H.dot(xb, precision="fp64fx")
    y64 = H.dot(xb)
    assert np.array_equal(np.isnan(y), np.isnan(y64)) and np.array_equal(np.isinf(y), np.isinf(y64))
    fin = np.isfinite(y64)
    assert fin.sum() > H.Ns // 2
    assert np.max(np.abs(y[fin] - y64[fin])) <= 1e-13 * np.abs(y64[fin]).max()


def test_fixed_point_row_ranges_and_repeat(qs, ora):
    """Large enough for the host path's row ranges (the first range makes the
    integer copy of x for all): repeated calls give identical results, equal
    to the device-buffer product."""
    torch = pytest.importorskip("torch")
    H, ref, terms = build(qs, ora, 20, 10, False, dict(kblock=0, pblock=1, zblock=1), "j1j2")
    assert H.fixed_point_classes == 2 and H.Ns > 2048
    x = models.seeded(H.Ns)
    y1 = H.dot(x, precision="fp64fx")    # first call: variant timing on the full range
    y2 = H.dot(x, precision="fp64fx")    # later calls: four row ranges, copied back while the next computes
    assert np.array_equal(y1, y2)
    y64 = H.dot(x)
    assert np.max(np.abs(y1 - y64)) <= 1e-13 * np.abs(y64).max()
    # device buffers through the C ABI, on the operator's default stream
    import ctypes
    from qsgpu import _lib
    xd = torch.tensor(x, device="cuda")
    yd = torch.empty_like(xd)
    torch.cuda.synchronize()
    one, zero = np.array([1.0, 0.0]), np.array([0.0, 0.0])
    _lib.check(_lib.load().qs_op_matvec(H._h, _lib.QS_FIXED_POINT, _lib.ptr(one), ctypes.c_void_p(xd.data_ptr()),
                                        _lib.QS_F64, _lib.ptr(zero), ctypes.c_void_p(yd.data_ptr()), _lib.QS_F64, 1,
                                        _lib.QS_MEM_DEVICE))
    torch.cuda.synchronize()
    assert np.array_equal(yd.cpu().numpy(), y1)
