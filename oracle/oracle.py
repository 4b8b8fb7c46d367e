"""CPU oracle for the QuSpin.jl spin-1/2 hot path.

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py``, to compare against.  The shipped library never
imports it.

Two restatements of the reference, see ``qs_oracle.c``:

* :class:`RefBasis` -- the reference algorithm (explicit projector, argmax
  representatives, lift/scatter/project matvec), IEEE-exact.
* :class:`RepBasis` -- representative-space restatement for large sectors.

The Krylov routines below restate ``src/operators.jl:1655-1893`` in numpy; eigsh
uses SciPy's ARPACK (the reference calls ARPACK through Arpack.jl 0.5,
``src/operators.jl:3367-3408``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def build() -> str:
    """Compile the oracle shared library (gcc, no GPU needed)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return os.path.join(_HERE, "_build", "libqs_oracle.so")


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "_build", "libqs_oracle.so")
        src = os.path.join(_HERE, "qs_oracle.c")
        if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
            build()
        L = ctypes.CDLL(path)
        P = ctypes.c_void_p
        i64 = ctypes.c_int64
        L.ora_basis_create.argtypes = [ctypes.c_int] * 11 + [ctypes.POINTER(P), ctypes.c_char_p, ctypes.c_int]
        L.ora_basis_create.restype = ctypes.c_int
        L.ora_basis_create_general.argtypes = [ctypes.c_int] * 4 + [P, P, P, ctypes.POINTER(P), ctypes.c_char_p,
                                                                     ctypes.c_int]
        L.ora_basis_create_general.restype = ctypes.c_int
        L.ora_basis_free.argtypes = [P]
        for name in ("ora_basis_size", "ora_basis_parent_size", "ora_basis_projector_nnz"):
            getattr(L, name).argtypes = [P]
            getattr(L, name).restype = i64
        L.ora_basis_reduced.argtypes = [P]
        L.ora_basis_states.argtypes = [P, P]
        L.ora_basis_parent_states.argtypes = [P, P]
        L.ora_basis_projector.argtypes = [P, P, P, P]
        L.ora_state_index.argtypes = [P, ctypes.c_uint64]
        L.ora_state_index.restype = i64
        L.ora_representative.argtypes = [P, ctypes.c_uint64, P, P, P]
        L.ora_representative.restype = ctypes.c_int
        L.ora_extract_diagonal.argtypes = [P, ctypes.c_int, P, P, P, P, P, P]
        L.ora_extract_diagonal.restype = ctypes.c_int
        L.ora_qlo_matvec.argtypes = [P, ctypes.c_int, P, P, P, P, P, ctypes.c_int, P, ctypes.c_int,
                                     ctypes.c_int, P, P, P, P]
        L.ora_qlo_matvec.restype = ctypes.c_int
        L.ora_rbasis_create.argtypes = [ctypes.c_int] * 12 + [ctypes.POINTER(P), ctypes.c_char_p, ctypes.c_int]
        L.ora_rbasis_create.restype = ctypes.c_int
        L.ora_rbasis_free.argtypes = [P]
        L.ora_rbasis_size.argtypes = [P]
        L.ora_rbasis_size.restype = i64
        L.ora_rbasis_group_order.argtypes = [P]
        L.ora_rbasis_states.argtypes = [P, P, P]
        L.ora_rbasis_matvec.argtypes = [P, ctypes.c_int, P, P, P, P, P, P, P, P, P, P, i64, i64, ctypes.c_int]
        L.ora_rbasis_matvec.restype = ctypes.c_int
        L.ora_rbasis_diagonal.argtypes = [P, ctypes.c_int, P, P, P, P, P, P]
        L.ora_rbasis_diagonal.restype = ctypes.c_int
        L.ora_num_threads.restype = ctypes.c_int
        _LIB = L
    return _LIB


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _sym_args(L, nup, pauli, a, kblock, pblock, zblock, pzblock, zAblock, zBblock):
    return [int(L), -1 if nup is None else int(nup), int(bool(pauli)), int(a),
            int(kblock is not None), int(kblock or 0), int(pblock or 0), int(zblock or 0),
            int(pzblock or 0), int(zAblock or 0), int(zBblock or 0)]


class OracleError(ValueError):
    pass


# ----------------------------------------------------------------- terms
def consolidate_terms(terms):
    """Restates ``_consolidate_terms`` (src/operators.jl:214-263): sums duplicate
    (op, sites) couplings in first-seen order and drops zero coefficients."""
    coeffs = {}
    order = []
    for op, couplings in terms:
        for c in couplings:
            key = (op, tuple(int(s) for s in c[1:]))
            if key not in coeffs:
                order.append(key)
                coeffs[key] = 0
            coeffs[key] = coeffs[key] + c[0]
    grouped = {}
    op_order = []
    for key in order:
        co = coeffs[key]
        if co == 0:
            continue
        op, sites = key
        if op not in grouped:
            grouped[op] = []
            op_order.append(op)
        grouped[op].append((co,) + sites)
    return [(op, grouped[op]) for op in op_order]


@dataclass
class PackedTerms:
    nterms: int
    ops: np.ndarray
    oplen: np.ndarray
    coup_off: np.ndarray
    coef: np.ndarray
    sites: np.ndarray

    def args(self):
        return [self.nterms, _ptr(self.ops), _ptr(self.oplen), _ptr(self.coup_off), _ptr(self.coef),
                _ptr(self.sites)]


def pack_terms(terms) -> PackedTerms:
    nt = len(terms)
    ops = np.zeros(8 * max(nt, 1), dtype=np.uint8)
    oplen = np.zeros(max(nt, 1), dtype=np.int32)
    off = np.zeros(nt + 1, dtype=np.int64)
    coefs, sites = [], []
    for t, (op, couplings) in enumerate(terms):
        if len(op) > 8:
            raise OracleError("operator strings longer than 8 characters are not supported")
        ops[8 * t:8 * t + len(op)] = np.frombuffer(op.encode(), dtype=np.uint8)
        oplen[t] = len(op)
        off[t + 1] = off[t] + len(couplings)
        for c in couplings:
            if len(c) != len(op) + 1:
                raise OracleError("operator arity and coupling sites differ")
            v = complex(c[0])
            coefs.extend([v.real, v.imag])
            s = [int(x) for x in c[1:]] + [0] * (8 - len(op))
            sites.extend(s)
    coef = np.array(coefs if coefs else [0.0, 0.0], dtype=np.float64)
    site_arr = np.array(sites if sites else [0] * 8, dtype=np.int32)
    return PackedTerms(nt, ops, oplen, off, coef, site_arr)


def is_diag_op(op):
    return all(ch in "Izn|" for ch in op)


# ----------------------------------------------------------------- bases
class RefBasis:
    """SpinBasis1D built with the reference algorithm (explicit projector)."""

    def __init__(self, L, nup=None, pauli=True, a=1, kblock=None, pblock=None, zblock=None,
                 pzblock=None, zAblock=None, zBblock=None, _general=None):
        lb = lib()
        h = ctypes.c_void_p()
        err = ctypes.create_string_buffer(256)
        if _general is not None:
            perms, flips, qnums = _general
            n = len(qnums)
            pa = np.ascontiguousarray(np.asarray(perms, dtype=np.int32).reshape(-1) if n else np.zeros(1, np.int32))
            fa = np.ascontiguousarray(np.asarray(flips, dtype=np.int32).reshape(-1) if n else np.zeros(1, np.int32))
            qa = np.ascontiguousarray(np.asarray(qnums, dtype=np.int32) if n else np.zeros(1, np.int32))
            rc = lb.ora_basis_create_general(int(L), -1 if nup is None else int(nup), int(bool(pauli)), n, _ptr(pa),
                                             _ptr(fa), _ptr(qa), ctypes.byref(h), err, 256)
        else:
            rc = lb.ora_basis_create(*_sym_args(L, nup, pauli, a, kblock, pblock, zblock, pzblock, zAblock,
                                                zBblock), ctypes.byref(h), err, 256)
        if rc != 0:
            raise OracleError(err.value.decode())
        self._h = h
        self.L, self.nup, self.pauli = L, nup, pauli
        self.Ns = int(lb.ora_basis_size(h))
        self.n_parent = int(lb.ora_basis_parent_size(h))
        self.reduced = bool(lb.ora_basis_reduced(h))
        self.states = np.zeros(self.Ns, dtype=np.uint64)
        lb.ora_basis_states(h, _ptr(self.states))
        self.parent_states = np.zeros(self.n_parent, dtype=np.uint64)
        lb.ora_basis_parent_states(h, _ptr(self.parent_states))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().ora_basis_free(self._h)
            self._h = None

    def projector(self):
        import scipy.sparse as sp
        if not self.reduced:
            return sp.identity(self.n_parent, dtype=np.complex128, format="csc")
        lb = lib()
        nnz = int(lb.ora_basis_projector_nnz(self._h))
        colptr = np.zeros(self.Ns + 1, dtype=np.int64)
        rowval = np.zeros(nnz, dtype=np.int64)
        vals = np.zeros(nnz, dtype=np.complex128)
        lb.ora_basis_projector(self._h, _ptr(colptr), _ptr(rowval), _ptr(vals))
        return sp.csc_matrix((vals, rowval, colptr), shape=(self.n_parent, self.Ns))

    def state_index(self, s):
        i = int(lib().ora_state_index(self._h, int(s)))
        if i < 0:
            raise OracleError(f"state {s} is not represented by this basis")
        return i

    def representative(self, s):
        rep = ctypes.c_uint64()
        norm = ctypes.c_double()
        amp = np.zeros(2)
        rc = lib().ora_representative(self._h, int(s), ctypes.byref(rep), ctypes.byref(norm), _ptr(amp))
        if rc == -1:
            raise OracleError("state is outside the parent particle sector")
        if rc == -2:
            raise OracleError("state has zero weight in this symmetry sector")
        return int(rep.value), float(norm.value), complex(amp[0], amp[1])

    def extract_diagonal(self, terms):
        pk = pack_terms(terms)
        out = np.zeros(self.Ns, dtype=np.complex128)
        rc = lib().ora_extract_diagonal(self._h, *pk.args(), _ptr(out))
        if rc:
            raise OracleError("unsupported spin operator")
        return out

    def qlo_matvec(self, terms, x, alpha=1.0, beta=0.0, y=None, diag=None, extract=True,
                   transposed=False, conjugated=False, total_diag=None, packed=None):
        """mul!(y, QuantumLinearOperator(basis, terms; diagonal=diag), x, alpha, beta).
        total_diag: the operator's stored diagonal (user + extracted), as the
        reference keeps it from construction; skips re-extracting it."""
        pk = packed or pack_terms(terms)
        x = np.ascontiguousarray(x, dtype=np.complex128)
        y = np.zeros(self.Ns, dtype=np.complex128) if y is None else np.array(y, dtype=np.complex128)
        if total_diag is not None:
            d = np.ascontiguousarray(total_diag, dtype=np.complex128)
        else:
            d = np.zeros(self.Ns, dtype=np.complex128)
            if extract:
                d += self.extract_diagonal(terms)
            if diag is not None:
                d += np.asarray(diag, dtype=np.complex128)
        a = np.array([complex(alpha).real, complex(alpha).imag])
        b = np.array([complex(beta).real, complex(beta).imag])
        rc = lib().ora_qlo_matvec(self._h, *pk.args(), int(extract), _ptr(d), int(transposed), int(conjugated),
                                  _ptr(a), _ptr(b), _ptr(x), _ptr(y))
        if rc:
            raise OracleError("unsupported spin operator")
        return y

    def dense(self, terms, diag=None, extract=True):
        n = self.Ns
        out = np.zeros((n, n), dtype=np.complex128)
        e = np.zeros(n, dtype=np.complex128)
        for j in range(n):
            e[:] = 0
            e[j] = 1
            out[:, j] = self.qlo_matvec(terms, e, diag=diag, extract=extract)
        return out


def normalize_general_map(values, L):
    """Restates _normalize_general_spin_map (src/basis.jl:282-303): a map is
    zero-based when it holds a zero or a negative entry; a negative entry
    flips that site's spin.  Returns (0-based targets, flip flags)."""
    values = [int(v) for v in values]
    if len(values) != L:
        raise OracleError("a general symmetry map must contain one entry per site")
    zero_based = any(v == 0 for v in values) or any(v < 0 for v in values)
    perm, flips = [], []
    for v in values:
        if zero_based:
            perm.append(v + 1 if v >= 0 else -v)
        else:
            if v == 0:
                raise OracleError("one-based symmetry maps cannot contain zero")
            perm.append(abs(v))
        flips.append(1 if v < 0 else 0)
    if sorted(perm) != list(range(1, L + 1)):
        raise OracleError("a general symmetry map must be a site permutation")
    return [p - 1 for p in perm], flips


def general_basis(L, nup=None, pauli=True, blocks=()):
    """SpinBasisGeneral(L; nup, pauli, blocks...) built with the reference's
    projector algorithm (src/basis.jl:455-600): blocks is a list of
    (map, quantum number) in intersection order."""
    perms, flips, qnums = [], [], []
    for m, q in blocks:
        p, f = normalize_general_map(m, L)
        perms.append(p)
        flips.append(f)
        qnums.append(int(q))
    return RefBasis(L, nup=nup, pauli=pauli, _general=(perms, flips, qnums))


class DenseSector:
    """SpinBasis1D sectors through the reference's level-by-level intersection
    with its dense nullspace branch (src/symmetry_basis.jl:57-213): explicit
    dense projectors, the cyclic projector of the first generator, then per
    generator the represented map P^H S P (entries with abs <= 5e-12 dropped),
    its orbit walk when it is permutation-like, else the nullspace of
    (represented - eigenvalue I) from an SVD with atol = rtol = 2e-10
    (LinearAlgebra.nullspace, the reference's call).  Numpy restatement for
    small parents; the nullspace basis is LAPACK's (as the reference's is
    Julia's LAPACK), so only basis-independent quantities (P P^H, spectra)
    are comparable with another implementation."""

    def __init__(self, L, nup=None, a=1, kblock=None, pblock=None, zblock=None, pzblock=None, zAblock=None,
                 zBblock=None):
        st = _parent_state_list(L, nup)
        self.L, self.nup = L, nup
        self.parent_states = st
        index = {int(s): i for i, s in enumerate(st)}
        full = (1 << L) - 1
        odd = sum(1 << (s - 1) for s in range(1, L + 1, 2))
        even = sum(1 << (s - 1) for s in range(2, L + 1, 2))

        def perm_map(perm):
            def f(s):
                t = 0
                for site in range(1, L + 1):
                    if s >> (site - 1) & 1:
                        t |= 1 << (perm[site - 1] - 1)
                return t
            return f

        order = L // a
        trans = perm_map([(site + a - 1) % L + 1 for site in range(1, L + 1)])
        par = perm_map([L - site + 1 for site in range(1, L + 1)])
        gens = []
        if kblock is not None:
            k = int(kblock) % order
            gens.append((trans, complex(np.cos(2 * np.pi * k / order), np.sin(2 * np.pi * k / order))))
        for v, f in ((pblock, par), (zblock, lambda s: s ^ full), (pzblock, lambda s: par(s) ^ full),
                     (zAblock, lambda s: s ^ odd), (zBblock, lambda s: s ^ even)):
            if v is not None:
                gens.append((f, complex(v)))
        n = len(st)
        self._gens = gens
        self._index = index
        P = self._cyclic(st, index, *gens[0])
        for f, eig in gens[1:]:
            P = self._intersect(P, st, index, f, eig)
        if P.shape[1] == 0:
            raise OracleError("the requested symmetry sector is empty")
        self.P = P
        self.Ns = P.shape[1]
        self.n_parent = n

    @staticmethod
    def _cyclic(st, index, f, eig):
        n = len(st)
        seen = np.zeros(n, bool)
        cols = []
        for start in range(n):
            if seen[start]:
                continue
            orbit = []
            cur = start
            while True:
                orbit.append(cur)
                seen[cur] = True
                nxt = index[f(int(st[cur]))]
                if nxt == start:
                    break
                cur = nxt
            c = np.ones(len(orbit), complex)
            for j in range(1, len(orbit)):
                c[j] = c[j - 1] / eig
            if abs(c[-1] - eig * c[0]) > max(2e-10, 2e-10 * max(abs(c[-1]), abs(eig * c[0]))):
                continue
            col = np.zeros(n, complex)
            col[orbit] = c / np.linalg.norm(c)
            cols.append(col)
        return np.array(cols).T if cols else np.zeros((n, 0), complex)

    @staticmethod
    def _intersect(P, st, index, f, eig):
        n, rd = P.shape
        if rd == 0:
            return P
        perm = np.array([index[f(int(s))] for s in st])
        SP = np.zeros_like(P)
        SP[perm, :] = P              # S P with S[perm[j], j] = 1
        R = P.conj().T @ SP
        R[np.abs(R) <= 5e-12] = 0
        nz = [np.flatnonzero(R[:, c]) for c in range(rd)]
        perm_like = all(len(z) == 1 for z in nz)
        if perm_like:
            mrow = np.array([z[0] for z in nz])
            mph = R[mrow, np.arange(rd)]
            perm_like = np.all(np.abs(np.abs(mph) - 1) <= 2e-10) and len(set(mrow.tolist())) == rd
        if perm_like:
            seen = np.zeros(rd, bool)
            cols = []
            for start in range(rd):
                if seen[start]:
                    continue
                orbit, ph = [], []
                cur = start
                while True:
                    orbit.append(cur)
                    seen[cur] = True
                    ph.append(mph[cur])
                    nxt = mrow[cur]
                    if nxt == start:
                        break
                    cur = nxt
                c = np.ones(len(orbit), complex)
                for j in range(1, len(orbit)):
                    c[j] = c[j - 1] * ph[j - 1] / eig
                closure = c[-1] * ph[-1]
                if abs(closure - eig * c[0]) > max(2e-10, 2e-10 * max(abs(closure), abs(eig * c[0]))):
                    continue
                col = np.zeros(rd, complex)
                col[orbit] = c / np.linalg.norm(c)
                cols.append(col)
            Rp = np.array(cols).T if cols else np.zeros((rd, 0), complex)
        else:
            if rd > 512:
                raise OracleError(f"the requested symmetry intersection requires a dense nullspace of dimension {rd}")
            M = R - eig * np.eye(rd)
            _, sv, vh = np.linalg.svd(M)
            tol = max(2e-10, sv[0] * 2e-10)
            rank = int(np.sum(sv > tol))
            Rp = vh[rank:].conj().T
        out = P @ Rp
        out[np.abs(out) <= 5e-14] = 0
        return out

    def projector_span(self):
        """P P^H over the parent sector (basis independent)."""
        return self.P @ self.P.conj().T

    def generators(self):
        """[(perm, eigenvalue)] of the requested generators in intersection
        order: perm[i] is the parent index of the image of parent state i."""
        st = self.parent_states
        return [(np.array([self._index[f(int(s))] for s in st]), eig) for f, eig in self._gens]


def _parent_state_list(L, nup):
    if nup is None:
        return np.arange(1 << L, dtype=np.uint64)
    from math import comb
    n = comb(L, nup)
    out = np.zeros(n, dtype=np.uint64)
    if nup == 0:
        return out
    s = (1 << nup) - 1
    for i in range(n):
        out[i] = s
        if i == n - 1:
            break
        low = s & -s
        nxt = s + low
        s = nxt | (((nxt ^ s) >> 2) // low)
    return out


class RepBasis:
    """Representative-space restatement (orbit minima, group by closure)."""

    def __init__(self, L, nup=None, pauli=True, a=1, kblock=None, pblock=None, zblock=None,
                 pzblock=None, zAblock=None, zBblock=None, nthreads=0):
        lb = lib()
        h = ctypes.c_void_p()
        err = ctypes.create_string_buffer(256)
        args = _sym_args(L, nup, pauli, a, kblock, pblock, zblock, pzblock, zAblock, zBblock) + [int(nthreads)]
        rc = lb.ora_rbasis_create(*args, ctypes.byref(h), err, 256)
        if rc != 0:
            raise OracleError(err.value.decode())
        self._h = h
        self.L, self.nup, self.pauli = L, nup, pauli
        self.Ns = int(lb.ora_rbasis_size(h))
        self.group_order = int(lb.ora_rbasis_group_order(h))
        self.states = np.zeros(self.Ns, dtype=np.uint64)
        self.orbit = np.zeros(self.Ns, dtype=np.int32)
        lb.ora_rbasis_states(h, _ptr(self.states), _ptr(self.orbit))
        self.nthreads = nthreads

    def __del__(self):
        if getattr(self, "_h", None):
            lib().ora_rbasis_free(self._h)
            self._h = None

    def diagonal(self, terms):
        pk = pack_terms(terms)
        out = np.zeros(self.Ns, dtype=np.complex128)
        if lib().ora_rbasis_diagonal(self._h, *pk.args(), _ptr(out)):
            raise OracleError("unsupported spin operator")
        return out

    def matvec(self, terms, x, alpha=1.0, beta=0.0, y=None, diag=None, rows=None, packed=None):
        pk = packed or pack_terms(terms)
        x = np.ascontiguousarray(x, dtype=np.complex128)
        y = np.zeros(self.Ns, dtype=np.complex128) if y is None else np.ascontiguousarray(y, dtype=np.complex128)
        d = self.diagonal(terms) if diag is None else np.ascontiguousarray(diag, dtype=np.complex128)
        a = np.array([complex(alpha).real, complex(alpha).imag])
        b = np.array([complex(beta).real, complex(beta).imag])
        r0, r1 = (0, self.Ns) if rows is None else rows
        rc = lib().ora_rbasis_matvec(self._h, *pk.args(), _ptr(d), _ptr(a), _ptr(b), _ptr(x), _ptr(y),
                                     int(r0), int(r1), int(self.nthreads))
        if rc:
            raise OracleError("unsupported spin operator")
        return y


# ----------------------------------------------------------------- Krylov
def krylov_factorization(matvec, v, hermitian, krylov_dim=30, dtype=np.complex128):
    """Restates ``_krylov_factorization`` (src/operators.jl:1655-1731)."""
    initial = np.array(v, dtype=dtype)
    beta = np.linalg.norm(initial)
    n = initial.size
    steps = min(int(krylov_dim), n)
    V = np.zeros((n, steps + 1), dtype=dtype)
    Hm = np.zeros((steps + 1, steps), dtype=dtype)
    V[:, 0] = initial / beta
    completed = steps
    terminal = 0.0
    if hermitian:
        prev = 0.0
        for col in range(steps):
            r = np.array(matvec(V[:, col]), dtype=dtype)
            if col > 0:
                r -= prev * V[:, col - 1]
            a = np.vdot(V[:, col], r)
            Hm[col, col] = a
            r -= a * V[:, col]
            terminal = np.linalg.norm(r)
            Hm[col + 1, col] = terminal
            if col < steps - 1:
                Hm[col, col + 1] = terminal
            if terminal <= 100 * np.finfo(float).eps * max(1.0, np.linalg.norm(Hm)):
                completed = col + 1
                break
            elif col < steps - 1:
                V[:, col + 1] = r / terminal
            prev = terminal
    else:
        for col in range(steps):
            r = np.array(matvec(V[:, col]), dtype=dtype)
            for row in range(col + 1):
                c = np.vdot(V[:, row], r)
                Hm[row, col] = c
                r -= c * V[:, row]
            for row in range(col + 1):
                c = np.vdot(V[:, row], r)
                Hm[row, col] += c
                r -= c * V[:, row]
            terminal = np.linalg.norm(r)
            Hm[col + 1, col] = terminal
            if terminal <= 100 * np.finfo(float).eps * max(1.0, np.linalg.norm(Hm)):
                completed = col + 1
                break
            elif col < steps - 1:
                V[:, col + 1] = r / terminal
    return dict(initial=initial, beta=beta, basis=V, hessenberg=Hm, completed=completed, terminal_norm=terminal,
                dimension=n, steps=steps, hermitian=hermitian)


def krylov_project(f, scale):
    """Restates ``_krylov_project`` (src/operators.jl:1733-1756)."""
    import scipy.linalg as sla
    m = f["completed"]
    E = sla.expm(scale * f["hessenberg"][:m, :m])
    result = f["basis"][:, :m] @ E[:, 0] * f["beta"]
    est = (abs(scale) * f["terminal_norm"] * f["beta"] * abs(E[-1, 0])
           if (m == f["steps"] and m < f["dimension"]) else 0.0)
    return result, est


def krylov_expmv_vector(matvec, v, scale, hermitian, tol=1e-12, krylov_dim=30, depth=0):
    """Restates ``_krylov_expmv_vector`` (src/operators.jl:1758-1803)."""
    initial = np.array(v, dtype=np.complex128)
    if scale == 0 or np.linalg.norm(initial) == 0:
        return initial
    f = krylov_factorization(matvec, initial, hermitian, krylov_dim)
    res, est = krylov_project(f, scale)
    if est > tol * max(1.0, np.linalg.norm(res)):
        if depth >= 14:
            raise RuntimeError("Krylov exponential action did not converge; increase krylov_dim")
        mid = krylov_expmv_vector(matvec, initial, scale / 2, hermitian, tol / 2, krylov_dim, depth + 1)
        return krylov_expmv_vector(matvec, mid, scale / 2, hermitian, tol / 2, krylov_dim, depth + 1)
    return res


def krylov_expmv_times(matvec, v, scales, hermitian, tol=1e-12, krylov_dim=30):
    """Restates ``_krylov_expmv_times`` (src/operators.jl:1805-1893)."""
    initial = np.array(v, dtype=np.complex128)
    out = np.zeros((initial.size, len(scales)), dtype=np.complex128)
    if len(scales) == 0:
        return out
    if np.linalg.norm(initial) == 0 or all(s == 0 for s in scales):
        out[:] = initial[:, None]
        return out
    f = krylov_factorization(matvec, initial, hermitian, krylov_dim)
    m = f["completed"]
    if hermitian:
        T = f["hessenberg"][:m, :m]
        Th = np.triu(T) + np.triu(T, 1).conj().T
        Th[np.diag_indices(m)] = np.real(np.diag(T))
        w, U = np.linalg.eigh(Th)
        first = U.conj().T[:, 0]
        for j, s in enumerate(scales):
            if s == 0:
                out[:, j] = initial
                continue
            c = U @ (np.exp(s * w) * first)
            state = f["beta"] * (f["basis"][:, :m] @ c)
            est = (abs(s) * f["terminal_norm"] * f["beta"] * abs(c[-1])
                   if (m == f["steps"] and m < f["dimension"]) else 0.0)
            if est > tol * max(1.0, np.linalg.norm(state)):
                state = krylov_expmv_vector(matvec, initial, s, hermitian, tol, krylov_dim)
            out[:, j] = state
    else:
        for j, s in enumerate(scales):
            if s == 0:
                out[:, j] = initial
                continue
            state, est = krylov_project(f, s)
            if est > tol * max(1.0, np.linalg.norm(state)):
                state = krylov_expmv_vector(matvec, initial, s, hermitian, tol, krylov_dim)
            out[:, j] = state
    return out


def eigsh_arpack(matvec, n, k, dtype, v0=None, tol=0.0, ncv=None, maxiter=None):
    """k smallest-algebraic eigenpairs through SciPy's ARPACK, sorted ascending
    (src/operators.jl:3367-3408 semantics)."""
    import scipy.sparse.linalg as spla
    op = spla.LinearOperator((n, n), matvec=matvec, dtype=dtype)
    vals, vecs = spla.eigsh(op, k=k, which="SA", v0=v0, tol=tol, ncv=ncv, maxiter=maxiter)
    order = np.argsort(vals)
    return vals[order], vecs[:, order]


# ----------------------------------------------------------------- Krylov tools
def lanczos_coefficients(matvec, v0, m, eps=None, full_ortho=False, keep=False):
    """Restates the recurrence of ``lanczos_full`` (src/tools.jl:2742-2805) and
    ``_lanczos_coefficients`` (src/tools.jl:2807-2843): m steps of the
    three-term Lanczos recurrence from v0 / ||v0||, with an optional
    modified Gram-Schmidt pass over every kept vector (``full_ortho``),
    stopping early when beta <= eps.  Returns (alphas, betas, rows) with rows
    the Lanczos vectors (used x n) when ``keep``."""
    v0 = np.asarray(v0)
    n = v0.size
    if not 1 <= m < n:
        raise OracleError("Lanczos dimension m must satisfy 1 <= m < length(v0)")
    nrm = np.linalg.norm(v0)
    if not nrm > 0:
        raise OracleError("initial Lanczos vector must be nonzero")
    first = np.asarray(matvec(v0))
    dt = np.result_type(v0.dtype, first.dtype, np.float64)
    tol = np.finfo(np.float64).eps if eps is None else float(eps)
    q = v0.astype(dt) / nrm
    q_prev = np.zeros(n, dtype=dt)
    r = first.astype(dt) / nrm
    beta_prev = 0.0
    alphas, betas, rows = [], [], []
    for index in range(1, m + 1):
        if keep or full_ortho:
            rows.append(q.copy())
        if index > 1:
            r = np.asarray(matvec(q)).astype(dt)
            r = r - beta_prev * q_prev
        a = float(np.real(np.vdot(q, r)))
        r = r - a * q
        if full_ortho:
            for b in rows:
                r = r - np.vdot(b, r) * b
        alphas.append(a)
        if index == m:
            break
        beta = float(np.linalg.norm(r))
        if beta <= tol:
            break
        betas.append(beta)
        q_prev = q
        q = r / beta
        beta_prev = beta
    return np.array(alphas), np.array(betas), (np.array(rows) if (keep or full_ortho) else None)


def lanczos_full(matvec, v0, m, full_ortho=False, eps=None):
    """Restates ``lanczos_full`` (src/tools.jl:2742-2805): (E, V, Q_T) with Q_T
    the Lanczos vectors in rows and (E, V) the eigenpairs of the tridiagonal."""
    import scipy.linalg as sla
    a, b, rows = lanczos_coefficients(matvec, v0, m, eps, full_ortho, keep=True)
    E, V = sla.eigh_tridiagonal(a, b) if a.size > 1 else (a.copy(), np.ones((1, 1)))
    return E, V, rows


def lanczos_vectors(matvec, v0, alphas, betas):
    """Restates ``_LanczosVectorIterator`` (src/tools.jl:2845-2882): the Lanczos
    vectors regenerated from v0 and the recurrence coefficients."""
    q = np.asarray(v0, dtype=np.result_type(np.asarray(v0).dtype, np.float64))
    q = q / np.linalg.norm(q)
    q_prev = np.zeros_like(q)
    yield q.copy()
    for index in range(1, len(alphas)):
        r = np.asarray(matvec(q)).astype(q.dtype)
        if index > 1:
            r = r - betas[index - 2] * q_prev
        r = r - alphas[index - 1] * q
        q_prev, q = q, r / betas[index - 1]
        yield q.copy()


def lin_comb_Q_T(coeff, rows):
    """Restates ``lin_comb_Q_T`` (src/tools.jl:2909-2945) for rows held as a
    matrix (Lanczos vectors in rows)."""
    coeff = np.asarray(coeff)
    if coeff.size != rows.shape[0]:
        raise OracleError("one coefficient is required per Lanczos vector")
    return rows.T @ coeff


def expm_lanczos(E, V, rows, a=1.0):
    """Restates ``expm_lanczos`` (src/tools.jl:2947-2952)."""
    return lin_comb_Q_T(V @ (np.exp(a * np.asarray(E)) * V[0, :]), rows)


def ftlm_static_iteration(observables, E, V, rows, beta=0.0):
    """Restates ``ftlm_static_iteration`` (src/tools.jl:2966-3013):
    results[key][b] = sum_i <q_i, O q_0> c_i(b) with
    c = V (V[0, :] exp(-E beta)); identity = c[0, :]."""
    scalar = np.isscalar(beta)
    betas = np.atleast_1d(np.asarray(beta, dtype=float))
    E = np.asarray(E)
    c = V @ (V[0, :][:, None] * np.exp(-E[:, None] * betas[None, :]))
    out = {}
    for key, O in observables.items():
        w = O(rows[0])
        ov = np.array([np.vdot(q, w) for q in rows])
        res = ov @ c
        out[key] = res[0] if scalar else res
    ident = c[0, :]
    return out, (ident[0] if scalar else ident)


def ltlm_static_iteration(observables, E, V, rows, beta=0.0):
    """Restates ``ltlm_static_iteration`` (src/tools.jl:3015-3068): Ritz
    vectors up to the Boltzmann cutoff at the smallest beta, weights
    V[0, :nv] exp(-E beta / 2), values w^T (R^* O R) w."""
    scalar = np.isscalar(beta)
    betas = np.atleast_1d(np.asarray(beta, dtype=float))
    E = np.asarray(E)
    m = E.size
    nv = m
    bmin = betas.min()
    if bmin > 0:
        half = np.exp(-(E - E.min()) * bmin / 2)
        idx = np.nonzero(half > np.finfo(float).eps)[0]
        nv = int(idx[-1]) + 1 if idx.size else 1
    En = E[:nv]
    W = V[0, :nv][:, None] * np.exp(-En[:, None] * betas[None, :] / 2)
    R = rows.T @ V[:, :nv]
    out = {}
    for key, O in observables.items():
        OR = np.column_stack([O(R[:, c]) for c in range(nv)])
        P = R.conj().T @ OR
        vals = np.array([np.vdot(W[:, b], P @ W[:, b]) for b in range(betas.size)])
        out[key] = vals[0] if scalar else vals
    ident = np.array([np.sum(np.abs(V[0, :nv]) ** 2 * np.exp(-b * En)) for b in betas])
    return out, (ident[0] if scalar else ident)
