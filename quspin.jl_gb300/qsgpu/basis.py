"""SpinBasis1D on the device (mirror of src/basis.jl:206-213, 622-799, 1016-1057).

Indices follow the reference's Julia convention: ``state_index`` returns and
``state_at`` takes one-based column numbers.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .errors import ArgumentError, DimensionMismatch, UnsupportedError


def basis_spec(L, nup=None, Nup=None, m=None, S="1/2", pauli=True, a=1, kblock=None, pblock=None, zblock=None,
               pzblock=None, zAblock=None, zBblock=None):
    """The C struct of SpinBasis1D(L; ...) keyword arguments, validated."""
    if str(S) not in ("1/2", "0.5"):
        raise ArgumentError("only spin-1/2 bases run on this engine")
    if not (1 <= int(L) <= 63):
        raise ArgumentError("L must be between 1 and 63")
    if nup is not None and Nup is not None:
        raise ArgumentError("specify only one of nup and Nup")
    sel = Nup if nup is None else nup
    if m is not None:
        if sel is not None:
            raise ArgumentError("m cannot be combined with nup or Nup")
        sel = int(round((float(m) + 0.5) * L))
    if sel is not None and not (0 <= int(sel) <= L):
        raise ArgumentError("nup must lie between 0 and L")
    return _lib.BasisSpec(int(L), -1 if sel is None else int(sel), int(bool(pauli)), int(a),
                          int(kblock is not None), int(kblock or 0), int(pblock or 0), int(zblock or 0),
                          int(pzblock or 0), int(zAblock or 0), int(zBblock or 0))


class SpinBasis1D:
    """SpinBasis1D(L; nup, pauli, a, kblock, pblock, zblock, pzblock, zAblock, zBblock)."""

    def __init__(self, L, nup=None, Nup=None, m=None, S="1/2", pauli=True, a=1, kblock=None, pblock=None,
                 zblock=None, pzblock=None, zAblock=None, zBblock=None):
        spec = basis_spec(L, nup=nup, Nup=Nup, m=m, S=S, pauli=pauli, a=a, kblock=kblock, pblock=pblock,
                          zblock=zblock, pzblock=pzblock, zAblock=zAblock, zBblock=zBblock)
        sel = None if spec.nup < 0 else spec.nup
        lib = _lib.load()
        h = ctypes.c_void_p()
        _lib.check(lib.qs_basis_create(ctypes.byref(spec), ctypes.byref(h)))
        self._h = h
        self.L = int(L)
        self.nup = None if sel is None else int(sel)
        self.pauli = bool(pauli)
        self.Ns = int(lib.qs_basis_size(h))
        self.group_order = int(lib.qs_basis_group_order(h))
        self.requires_complex = bool(lib.qs_basis_requires_complex(h))
        blocks = {"nup": self.nup, "pauli": self.pauli}
        order = self.L // int(a) if self.L % int(a) == 0 else None
        if kblock is not None:
            blocks["a"] = int(a)
            blocks["kblock"] = int(kblock) % order
        for name, v in (("pblock", pblock), ("zblock", zblock), ("pzblock", pzblock), ("zAblock", zAblock),
                        ("zBblock", zBblock)):
            if v is not None:
                blocks[name] = int(v)
        self.blocks = blocks
        self.symmetric = any(k in blocks for k in ("kblock", "pblock", "zblock", "pzblock", "zAblock", "zBblock"))
        self._states = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            _lib.load().qs_basis_destroy(h)
            self._h = None

    def __len__(self):
        return self.Ns

    N = property(lambda self: self.L)
    sps = 2
    dtype = np.uint64
    operators = ("I", "z", "+", "-", "x", "y")
    description = "spin-1/2 chain basis"

    @property
    def states(self):
        if self._states is None:
            out = np.zeros(self.Ns, dtype=np.uint64)
            _lib.check(_lib.load().qs_basis_states(self._h, _lib.ptr(out), self.Ns))
            self._states = out
        return self._states.copy()

    def orbit_minima(self):
        out = np.zeros(self.Ns, dtype=np.uint64)
        _lib.check(_lib.load().qs_basis_orbit_minima(self._h, _lib.ptr(out), self.Ns))
        return out

    def stabilizers(self):
        """Stabiliser order of every column's orbit minimum (orbit size = group_order / stab)."""
        out = np.zeros(self.Ns, dtype=np.uint16)
        _lib.check(_lib.load().qs_basis_stabilizers(self._h, _lib.ptr(out), self.Ns))
        return out

    def index_array(self, states):
        """0-based columns of many states at once (-1 where not represented)."""
        q = np.ascontiguousarray(states, dtype=np.uint64)
        out = np.zeros(q.size, dtype=np.int64)
        _lib.check(_lib.load().qs_basis_state_index(self._h, _lib.ptr(q), q.size, _lib.ptr(out)))
        return out

    def representative_array(self, states):
        q = np.ascontiguousarray(states, dtype=np.uint64)
        n = q.size
        reps = np.zeros(n, dtype=np.uint64)
        norms = np.zeros(n)
        amps = np.zeros(n, dtype=np.complex128)
        status = np.zeros(n, dtype=np.int32)
        _lib.check(_lib.load().qs_basis_representative(self._h, _lib.ptr(q), n, _lib.ptr(reps), _lib.ptr(norms),
                                                       _lib.ptr(amps), _lib.ptr(status)))
        return reps, norms, amps, status


def states(basis):
    return basis.states


def state_index(basis, state):
    """One-based column of a representative (src/basis.jl:1016-1022)."""
    if state < 0:
        raise ArgumentError("state must be nonnegative")
    i = int(basis.index_array([state])[0])
    if i < 0:
        raise ArgumentError(f"state {state} is not represented by this basis")
    return i + 1


def state_at(basis, index):
    if not (1 <= index <= basis.Ns):
        raise IndexError(f"index {index} out of bounds for a basis of length {basis.Ns}")
    return basis.states[index - 1]


def _rep_query(basis, state):
    reps, norms, amps, status = basis.representative_array([state])
    if status[0] == 1:
        raise ArgumentError("state is outside the parent particle sector")
    if status[0] == 2:
        raise ArgumentError("state has zero weight in this symmetry sector")
    return int(reps[0]), float(norms[0]), complex(amps[0])


def representative(basis, state):
    if not basis.symmetric:
        return state
    return _rep_query(basis, state)[0]


def normalization(basis, state):
    if not basis.symmetric:
        return 1.0
    return _rep_query(basis, state)[1]


def get_amp(basis, state):
    if not basis.symmetric:
        return 1.0
    return _rep_query(basis, state)[2]


def int_to_state(basis, state, bracket_notation=True):
    if not (0 <= state < (1 << basis.L)):
        raise ArgumentError("state must fit in L bits")
    bits = format(int(state), "b").zfill(basis.L)
    return "|" + " ".join(bits) + ">" if bracket_notation else bits


def state_to_int(basis, state):
    compact = state.strip("|>").replace(" ", "")
    if len(compact) != basis.L:
        raise ArgumentError(f"state must contain exactly {basis.L} binary digits")
    if any(ch not in "01" for ch in compact):
        raise ArgumentError("state must be binary")
    return int(compact, 2)


def _projection(basis, vector, pcon, mode):
    """mode 0: P v (Ns -> rows); mode 1: P^H v (rows -> Ns); columns of a matrix one by one."""
    lib = _lib.load()
    rows = int(lib.qs_basis_projection_rows(basis._h, 1 if pcon else 0))
    if rows < 0:
        raise ArgumentError("the full Hilbert-space dimension exceeds device memory; use pcon=True")
    v = np.asarray(vector)
    nin, nout = (basis.Ns, rows) if mode == 0 else (rows, basis.Ns)
    if v.shape[0] != nin:
        raise DimensionMismatch("the first vector dimension must equal Ns" if mode == 0 else
                                "the first vector dimension does not match the projection space")
    if not np.iscomplexobj(v) and basis.requires_complex:
        raise ArgumentError("this momentum sector requires a complex projection dtype")
    cols = v.reshape(nin, -1)
    out = np.zeros((nout, cols.shape[1]), dtype=np.complex128)
    for c in range(cols.shape[1]):
        x = np.ascontiguousarray(cols[:, c], dtype=np.complex128)
        y = np.zeros(nout, dtype=np.complex128)
        if mode == 0:
            _lib.check(lib.qs_basis_project_from(basis._h, 1 if pcon else 0, _lib.ptr(x), _lib.ptr(y), 0,
                                                 _lib.QS_MEM_HOST))
        else:
            _lib.check(lib.qs_basis_project_to(basis._h, 1 if pcon else 0, _lib.ptr(x), _lib.ptr(y),
                                               _lib.QS_MEM_HOST))
        out[:, c] = y
    if not np.iscomplexobj(v):
        out = out.real.copy()
    return out.reshape((nout,) + v.shape[1:])


def _maybe_sparse(a, sparse):
    if not sparse:
        return a
    import scipy.sparse as sp
    return sp.csc_matrix(a.reshape(a.shape[0], -1))


def project_from(basis, vector, sparse=False, pcon=False):
    """project_from(basis, vector; sparse, pcon) (src/basis.jl:889-908): P v,
    from the sector to the full 2^L space (or the parent particle sector with
    pcon).  Computed on the device; dense unless sparse=True (the reference's
    default output is sparse)."""
    return _maybe_sparse(_projection(basis, vector, pcon, 0), sparse)


def get_vec(basis, vector, sparse=False, pcon=False):
    """get_vec(basis, vector; kwargs...) = project_from (src/basis.jl:910-911)."""
    return project_from(basis, vector, sparse=sparse, pcon=pcon)


def project_to(basis, vector, sparse=False, pcon=False):
    """project_to(basis, vector; sparse, pcon) (src/discrete_basis.jl:2455-2475):
    P^H v, from the full space (or parent sector) to the sector."""
    return _maybe_sparse(_projection(basis, vector, pcon, 1), sparse)


def _normalize_general_map(values, L):
    """_normalize_general_spin_map (src/basis.jl:282-303): a map holding a zero
    or a negative entry is zero-based; a negative entry flips that site's spin.
    Returns 0-based targets and flip flags."""
    values = [int(v) for v in values]
    if len(values) != L:
        raise ArgumentError("a general symmetry map must contain one entry per site")
    zero_based = any(v == 0 for v in values) or any(v < 0 for v in values)
    perm, flips = [], []
    for v in values:
        if zero_based:
            perm.append(v + 1 if v >= 0 else -v)
        else:
            if v == 0:
                raise ArgumentError("one-based symmetry maps cannot contain zero")
            perm.append(abs(v))
        flips.append(1 if v < 0 else 0)
    if sorted(perm) != list(range(1, L + 1)):
        raise ArgumentError("a general symmetry map must be a site permutation")
    return [p - 1 for p in perm], flips


class SpinBasisGeneral(SpinBasis1D):
    """SpinBasisGeneral(L; nup, Nup, m, S, pauli, block_order, blocks...)
    (src/basis.jl:455-600) for spin 1/2 and L <= 63: each block is
    (map, quantum_number) with map a site permutation (negative entries flip
    the spin), intersected in block_order (default: keyword order).  Columns
    are the symmetric orbit states in ascending orbit minimum, labelled by
    the reference's own representatives (its projector is replayed)."""

    def __init__(self, L, nup=None, Nup=None, m=None, S="1/2", pauli=True, block_order=None, make_basis=True,
                 Ns_block_est=None, **blocks):
        if str(S) not in ("1/2", "0.5"):
            raise UnsupportedError("SpinBasisGeneral is implemented for spin 1/2")
        if nup is not None and Nup is not None:
            raise ArgumentError("specify only one of nup and Nup")
        sel = nup if nup is not None else Nup
        if m is not None:
            if sel is not None:
                raise ArgumentError("m cannot be combined with nup or Nup")
            sel = int(round((float(m) + 0.5) * L))
        if sel is not None and not 0 <= int(sel) <= L:
            raise ArgumentError("nup must lie between 0 and L")
        names = list(blocks) if block_order is None else [str(n) for n in block_order]
        for n in blocks:
            if n not in names:
                names.append(n)
        if any(n not in blocks for n in names):
            raise ArgumentError("block_order refers to an unknown symmetry block")
        perms, flips, qnums = [], [], []
        for n in names:
            spec = blocks[n]
            if not isinstance(spec, (tuple, list)) or len(spec) < 2:
                raise ArgumentError("general symmetry blocks must be (map, quantum_number)")
            p, f = _normalize_general_map(spec[0], int(L))
            perms += p
            flips += f
            qnums.append(int(spec[1]))
        k = len(qnums)
        pa = np.ascontiguousarray(perms if k else [0], dtype=np.int32)
        fa = np.ascontiguousarray(flips if k else [0], dtype=np.int32)
        qa = np.ascontiguousarray(qnums if k else [0], dtype=np.int32)
        spec = _lib.GeneralSpec(int(L), -1 if sel is None else int(sel), int(bool(pauli)), k, _lib.ptr(pa),
                                _lib.ptr(fa), _lib.ptr(qa))
        lib = _lib.load()
        h = ctypes.c_void_p()
        _lib.check(lib.qs_basis_create_general(ctypes.byref(spec), ctypes.byref(h)))
        self._h = h
        self.L = int(L)
        self.nup = None if sel is None else int(sel)
        self.pauli = bool(pauli)
        self.Ns = int(lib.qs_basis_size(h))
        self.group_order = int(lib.qs_basis_group_order(h))
        self.requires_complex = bool(lib.qs_basis_requires_complex(h))
        self.blocks = {"nup": self.nup, "pauli": self.pauli}
        self.blocks.update({n: (tuple(blocks[n][0]), int(blocks[n][1])) for n in names})
        self.block_order = names
        self.symmetric = k > 0
        self._states = None
