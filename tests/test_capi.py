"""The C-ABI library loads, exports every symbol of include/qsgpu.h, and turns
invalid arguments into the reference's errors before touching the device."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    with open(os.path.join(ROOT, "include", "qsgpu.h")) as f:
        src = f.read()
    return sorted(set(re.findall(r"QS_API[^;(]*?\b(qs_\w+)\s*\(", src)))


def test_header_lists_entry_points():
    syms = declared_symbols()
    assert "qs_op_matvec" in syms and "qs_eigsh" in syms and "qs_evolve" in syms
    assert len(syms) >= 20


def test_library_exports_every_declared_symbol(qs):
    from qsgpu import _lib
    lib = _lib.load()
    for name in declared_symbols():
        assert hasattr(lib, name), name
    assert set(declared_symbols()) == set(_lib.EXPORTS)
    assert lib.qs_version().decode().startswith("qsgpu")


def header_constants():
    """name -> value of every QS_* enumerator of include/qsgpu.h."""
    with open(os.path.join(ROOT, "include", "qsgpu.h")) as f:
        src = re.sub(r"/\*.*?\*/", "", f.read(), flags=re.S)
    out = {}
    for body in re.findall(r"enum\s*\{(.*?)\}", src, flags=re.S):
        for name, val in re.findall(r"\b(QS_\w+)\s*=\s*(-?\d+)", body):
            out[name] = int(val)
    return out


def test_binding_constants_match_the_header():
    """The ctypes binding's flag, dtype, memory and status values are the
    header's (a drift would silently select another product form)."""
    import sys
    sys.path.insert(0, os.path.join(ROOT, "quspin.jl_gb300"))
    from qsgpu import _lib
    consts = header_constants()
    for name in ("QS_TRANSPOSE", "QS_CONJUGATE", "QS_DOUBLE_FLOAT", "QS_FIXED_POINT", "QS_MEM_HOST",
                 "QS_MEM_DEVICE", "QS_F64", "QS_C128", "QS_F32", "QS_C64"):
        assert name in consts, name
        assert getattr(_lib, name) == consts[name], name
    flags = [consts[n] for n in ("QS_TRANSPOSE", "QS_CONJUGATE", "QS_DOUBLE_FLOAT", "QS_FIXED_POINT")]
    assert len(set(flags)) == 4 and all(f & (f - 1) == 0 for f in flags)   # distinct single bits


@pytest.mark.parametrize("kwargs,msg", [
    (dict(L=0), "L must be between 1 and 63"),
    (dict(L=64), "L must be between 1 and 63"),
    (dict(L=4, nup=5), "nup must lie between 0 and L"),
    (dict(L=6, nup=3, kblock=1, pblock=1), "pblock can be combined with kblock only at k=0 or pi"),
    (dict(L=6, nup=2, zblock=1), "symmetry transformation leaves the selected particle sector"),
    (dict(L=6, nup=3, zAblock=1), "symmetry transformation leaves the selected particle sector"),
    (dict(L=6, nup=3, a=4, kblock=0), "a must be a positive divisor of L"),
    (dict(L=6, nup=3, pblock=2), "pblock must be +1 or -1"),
    (dict(L=6, nup=3, kblock=0, pblock=1, zblock=1, pzblock=-1), "the requested symmetry sector is empty"),
])
def test_basis_argument_errors(qs, kwargs, msg):
    with pytest.raises(qs.ArgumentError, match=re.escape(msg)):
        qs.SpinBasis1D(**kwargs)


def test_dense_nullspace_guard(qs, ora):
    # zA after a one-site translation needs the reference's dense nullspace
    # intersection, which it refuses above 512 reduced columns with this
    # message (src/symmetry_basis.jl:199-206); the check runs before any device work
    dim = ora.RefBasis(14, kblock=0).Ns
    msg = (f"the requested symmetry intersection requires a dense nullspace of dimension {dim}; "
           "the guarded limit is 512")
    with pytest.raises(qs.ArgumentError, match=re.escape(msg)):
        qs.SpinBasis1D(14, kblock=0, zAblock=1)
