"""Operators and Krylov solvers over libqsgpu (mirror of src/operators.jl).

QuantumLinearOperator (2331-2552, 3133-3365), eigsh (3367-3408), the static
Hamiltonian's matvec (754-766) and evolve (2073-2164); the matvec, Lanczos and
Krylov exponential all run on the device.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .errors import ArgumentError, DimensionMismatch


class OperatorTerm:
    """OperatorTerm(op, couplings): couplings are (coefficient, site, ...) with one-based sites."""

    def __init__(self, op, couplings):
        if not op:
            raise ArgumentError("operator string cannot be empty")
        arity = sum(1 for ch in op if ch != "|")
        norm = []
        for c in couplings:
            c = tuple(c)
            if len(c) != arity + 1:
                raise ArgumentError("operator arity and coupling sites differ")
            if not all(isinstance(s, (int, np.integer)) for s in c[1:]):
                raise ArgumentError("all sites must be integers")
            norm.append(c)
        self.op = str(op)
        self.couplings = norm

    def __eq__(self, other):
        return isinstance(other, OperatorTerm) and self.op == other.op and self.couplings == other.couplings

    def __repr__(self):
        return f"OperatorTerm({self.op!r}, {self.couplings!r})"


def _pack_terms(terms):
    keep = []
    arr = (_lib.Term * max(1, len(terms)))()
    for i, t in enumerate(terms):
        n = len(t.couplings)
        arity = sum(1 for ch in t.op if ch != "|")
        coeffs = np.zeros(2 * max(n, 1))
        sites = np.zeros(max(arity * n, 1), dtype=np.int32)
        cplx = False
        for j, c in enumerate(t.couplings):
            v = c[0]
            if isinstance(v, (complex, np.complexfloating)):
                cplx = True
            v = complex(v)
            coeffs[2 * j], coeffs[2 * j + 1] = v.real, v.imag
            sites[j * arity:(j + 1) * arity] = [int(s) for s in c[1:]]
        opb = t.op.encode()
        keep += [coeffs, sites, opb]
        arr[i] = _lib.Term(opb, n, _lib.ptr(coeffs), _lib.ptr(sites), int(cplx))
    return arr, keep


class QuantumLinearOperator:
    """QuantumLinearOperator(basis, static_list; diagonal, check_symm, check_herm, check_pcon)."""

    def __init__(self, basis, static_list, diagonal=None, check_symm=True, check_herm=True, check_pcon=True,
                 _flags=0, _shared=None):
        self.basis = basis
        self.static_list = list(static_list)
        self._flags = _flags
        if _shared is not None:
            self._h, self._owner = _shared
        else:
            lib = _lib.load()
            arr, keep = _pack_terms(self.static_list)
            checks = (_lib.QS_CHECK_SYMM if check_symm else 0) | (_lib.QS_CHECK_HERM if check_herm else 0) | (
                _lib.QS_CHECK_PCON if check_pcon else 0)
            dptr = None
            d = None
            if diagonal is not None:
                dv = np.asarray(diagonal)
                if dv.shape != (basis.Ns,):
                    raise DimensionMismatch("diagonal must have length Ns")
                if np.iscomplexobj(dv):
                    checks |= _lib.QS_DIAG_COMPLEX
                d = np.ascontiguousarray(dv, dtype=np.complex128)
                dptr = _lib.ptr(d)
            h = ctypes.c_void_p()
            _lib.check(lib.qs_op_create(basis._h, arr, len(self.static_list), dptr, checks, ctypes.byref(h)))
            self._h = h
            self._owner = _Owner(h)
            self._diag = np.zeros(basis.Ns) if d is None else (d if np.iscomplexobj(diagonal) else d.real.copy())
        lib = _lib.load()
        self.dtype = np.complex128 if lib.qs_op_dtype(self._h) == _lib.QS_C128 else np.float64
        self.hermitian = bool(lib.qs_op_hermitian(self._h))
        self.Ns = basis.Ns
        self.shape = (basis.Ns, basis.Ns)
        self.ndim = 2

    @property
    def diagonal(self):
        return self._diag

    @property
    def get_shape(self):
        return self.shape

    def _with_flags(self, toggle):
        op = QuantumLinearOperator(self.basis, self.static_list, _flags=self._flags ^ toggle,
                                   _shared=(self._h, self._owner))
        op._diag = self._diag
        return op

    def transpose(self):
        return self._with_flags(_lib.QS_TRANSPOSE)

    def conj(self):
        return self._with_flags(_lib.QS_CONJUGATE)

    def adjoint(self):
        return self._with_flags(_lib.QS_TRANSPOSE | _lib.QS_CONJUGATE)

    T = property(transpose)
    H = property(adjoint)

    def set_diagonal(self, diagonal):
        d = np.ascontiguousarray(diagonal, dtype=np.complex128)
        if d.shape != (self.Ns,):
            raise DimensionMismatch("diagonal must have length Ns")
        _lib.check(_lib.load().qs_op_set_diagonal(self._h, _lib.ptr(d)))
        self._diag = np.asarray(diagonal).copy()
        return self

    # mul!(out, op, x, alpha, beta)
    def mul(self, out, x, alpha=1.0, beta=0.0, precision="fp64"):
        x = np.asarray(x)
        if out.shape[0] != self.Ns:
            raise DimensionMismatch("output and operator dimensions do not match")
        if x.shape[0] != self.Ns:
            raise DimensionMismatch("operator and value dimensions do not match")
        if x.ndim != out.ndim or (x.ndim == 2 and x.shape[1] != out.shape[1]):
            raise DimensionMismatch("output has the wrong dimensions")
        if precision not in ("fp64", "fp32", "fp64df", "fp64fx"):
            raise ArgumentError("precision must be fp64, fp32, fp64df or fp64fx")
        single = precision == "fp32"
        flags = self._flags | {"fp64df": _lib.QS_DOUBLE_FLOAT, "fp64fx": _lib.QS_FIXED_POINT}.get(precision, 0)
        nrhs = 1 if x.ndim == 1 else x.shape[1]
        ycx = np.iscomplexobj(out)
        if (np.iscomplexobj(x) or self.dtype == np.complex128 or complex(alpha).imag or complex(beta).imag) and not ycx:
            raise ArgumentError("a complex result cannot be stored in a real output")
        if single:
            xdt = np.complex64 if np.iscomplexobj(x) else np.float32
            ydt = np.complex64 if ycx else np.float32
        else:
            xdt = np.complex128 if np.iscomplexobj(x) else np.float64
            ydt = np.complex128 if ycx else np.float64
        xs = np.asfortranarray(x, dtype=xdt)
        ys = np.asfortranarray(out, dtype=ydt) if out.dtype != ydt or not out.flags.f_contiguous else out
        if xs is ys or np.shares_memory(xs, ys):
            xs = xs.copy(order="F")
        code = {np.float64: 0, np.complex128: 1, np.float32: 2, np.complex64: 3}
        a = np.array([complex(alpha).real, complex(alpha).imag])
        b = np.array([complex(beta).real, complex(beta).imag])
        _lib.check(_lib.load().qs_op_matvec(self._h, flags, _lib.ptr(a), _lib.ptr(xs), code[xdt], _lib.ptr(b),
                                            _lib.ptr(ys), code[ydt], nrhs, _lib.QS_MEM_HOST))
        if ys is not out:
            out[...] = ys
        return out

    def dot(self, x, precision="fp64"):
        x = np.asarray(x)
        if x.shape[0] != self.Ns:
            raise DimensionMismatch("operator and value dimensions do not match")
        cpx = np.iscomplexobj(x) or self.dtype == np.complex128
        out = np.zeros(x.shape, dtype=np.complex128 if cpx else np.float64, order="F")
        return self.mul(out, x, precision=precision)

    __matmul__ = dot

    def __mul__(self, x):
        return self.dot(x)

    def toarray(self):
        """Matrix(op): dense materialisation (small Ns only)."""
        return self.dot(np.eye(self.Ns, dtype=self.dtype))


class _Owner:
    def __init__(self, h):
        self.h = h

    def __del__(self):
        if self.h:
            _lib.load().qs_op_destroy(self.h)
            self.h = None


def isquantum_LinearOperator(value):
    return isinstance(value, QuantumLinearOperator)


def apply(op, value, out=None, a=1.0):
    if isinstance(op, ExpmMultiplyParallel):
        return op.apply(value)
    if out is None:
        cpx = np.iscomplexobj(value) or op.dtype == np.complex128 or isinstance(a, complex)
        out = np.zeros(np.shape(value), dtype=np.complex128 if cpx else np.float64, order="F")
    return op.mul(out, value, a, 0.0)


class Hamiltonian(QuantumLinearOperator):
    """Static Hamiltonian(basis, terms): H * v and mul! (src/operators.jl:754-766)
    on the device.  The assembled CSC field H.data is not materialised."""

    def __init__(self, basis, terms, static_fmt=None, check_symm=True, check_herm=True, check_pcon=True,
                 assemble=True):
        super().__init__(basis, terms, check_symm=check_symm, check_herm=check_herm, check_pcon=check_pcon)
        self.assembled = False
        if assemble:
            st = _lib.load().qs_op_assemble(self._h)
            if st == 0:
                self.assembled = True
            elif st != 6:  # 6: not assemblable, stays matrix-free
                _lib.check(st)

    @property
    def nnz(self):
        return int(_lib.load().qs_op_nnz(self._h))

    @property
    def fixed_point_classes(self):
        """Amplitude classes of the precision="fp64fx" product (0: it runs as FP64)."""
        return int(_lib.load().qs_op_fixed_point_classes(self._h))

    def _export(self):
        """The device's assembled matrix as a scipy CSR matrix (duplicates summed)."""
        import scipy.sparse as sp
        if not self.assembled:
            raise ArgumentError("this operator has no assembled form (non-commuting terms stay matrix-free)")
        n, nnz = self.Ns, self.nnz
        rowptr = np.zeros(n + 1, dtype=np.int64)
        cols = np.zeros(max(nnz, 1), dtype=np.int64)
        vals = np.zeros(max(nnz, 1), dtype=np.complex128)
        diag = np.zeros(n, dtype=np.complex128)
        _lib.check(_lib.load().qs_op_export_csr(self._h, _lib.ptr(rowptr), _lib.ptr(cols), _lib.ptr(vals),
                                                _lib.ptr(diag)))
        real = self.dtype == np.float64
        off = sp.csr_matrix(((vals[:nnz].real if real else vals[:nnz]), cols[:nnz], rowptr), shape=(n, n))
        off.sum_duplicates()
        d = diag.real if real else diag
        nz = np.nonzero(d)[0]
        return off + sp.csr_matrix((d[nz], (nz, nz)), shape=(n, n))

    def tocsr(self, time=0):
        """tocsr(H; time) (src/operators.jl:1348): the static matrix H.data, from the device's assembled form."""
        return self._export()

    def tocsc(self, time=0):
        """tocsc(H; time) (src/operators.jl:1347)."""
        return self._export().tocsc()

    def toarray(self, time=0, order=None, out=None):
        """toarray(H; time, out) (src/operators.jl:1343-1344)."""
        a = self._export().toarray()
        if out is None:
            return a
        if out.shape != a.shape:
            raise DimensionMismatch("out must have the same axes as the result")
        out[...] = a
        return out

    todense = toarray


def tocsc(H, time=0):
    """tocsc(H::Hamiltonian; time) (src/operators.jl:1347)."""
    return H.tocsc(time)


def tocsr(H, time=0):
    """tocsr(H::Hamiltonian; time) (src/operators.jl:1348)."""
    return H.tocsr(time)


def toarray(H, time=0, order=None, out=None):
    """toarray(H::Hamiltonian; time, out) (src/operators.jl:1343-1344)."""
    return H.toarray(time, order, out)


def _precision_code(precision):
    """0 = FP64, 1 = FP32 (+ FP64 polish), 2 = double-float on the FP32 pipe."""
    codes = {"fp64": 0, "fp32": 1, "fp64df": 2}
    if precision not in codes:
        raise ArgumentError("precision must be fp64, fp32 or fp64df")
    return codes[precision]


_WHICH = {"SA": 0, "LA": 1, "LM": 2, "SM": 3, "BE": 4}


def _which_code(which):
    """eigsh's `which` (src/operators.jl:3376-3378): SA and LA by algebraic
    value, LM and SM by magnitude, BE half from each end."""
    w = str(which).upper()
    if w not in _WHICH:
        raise ArgumentError("which must be SA, LA, SM, LM, or BE")
    return _WHICH[w]


def eigsh(op, k=None, which="SA", return_eigenvectors=True, v0=None, tol=0.0, ncv=None, maxiter=None,
          precision="fp64", info=None):
    """eigsh(op; k, which=:SA, v0, tol, ncv, maxiter): k extremal eigenpairs."""
    n = op.Ns
    k = min(6, n) if k is None else int(k)
    if not (1 <= k <= n):
        raise ArgumentError("k must lie in 1:Ns")
    code = _which_code(which)
    vv = None
    if v0 is not None:
        vv = np.ascontiguousarray(v0, dtype=op.dtype)
        if vv.shape != (n,):
            raise DimensionMismatch("v0 must have length Ns")
    opts = _lib.EigshOpts(k, code, float(tol), int(ncv or 0), int(maxiter or 0),
                          _precision_code(precision), int(bool(return_eigenvectors)),
                          _lib.ptr(vv) if vv is not None else None, _lib.QS_MEM_HOST)
    if not getattr(op, "hermitian", True):
        # complex eigenvalues and vectors, as the reference returns for a
        # non-Hermitian operator (src/operators.jl:3402-3404)
        if code == 4:
            raise ArgumentError("which must be SA, LA, SM or LM for a non-Hermitian operator")
        cvals = np.zeros(2 * k)
        cvecs = np.zeros((n, k), dtype=np.complex128, order="F") if return_eigenvectors else None
        inf = _lib.EigshInfo()
        _lib.check(_lib.load().qs_eigs(op._h, ctypes.byref(opts), _lib.ptr(cvals),
                                       _lib.ptr(cvecs) if cvecs is not None else None, ctypes.byref(inf)))
        if info is not None:
            info.update(nconv=inf.nconv, restarts=inf.restarts, matvecs=inf.matvecs,
                        max_rel_residual=inf.max_rel_residual, seconds=inf.seconds)
        vals = cvals[0::2] + 1j * cvals[1::2]
        return (vals, cvecs) if return_eigenvectors else vals
    vals = np.zeros(k)
    vecs = np.zeros((n, k), dtype=op.dtype, order="F") if return_eigenvectors else None
    inf = _lib.EigshInfo()
    _lib.check(_lib.load().qs_eigsh(op._h, ctypes.byref(opts), _lib.ptr(vals),
                                    _lib.ptr(vecs) if vecs is not None else None, ctypes.byref(inf)))
    if info is not None:
        info.update(nconv=inf.nconv, restarts=inf.restarts, matvecs=inf.matvecs,
                    max_rel_residual=inf.max_rel_residual, seconds=inf.seconds)
    return (vals, vecs) if return_eigenvectors else vals


def eigsh_batch(ops, k=1, which="SA", tol=0.0, ncv=None, maxiter=None, return_eigenvectors=False, infos=None,
                precision="fp64"):
    """eigsh(op; k, which) on every operator of `ops` at once: each Lanczos
    step is one launch per kernel for all operators, replayed from a CUDA
    graph.  precision "fp64" stores the Krylov vectors in FP64, "fp64df" as
    double-float pairs on the FP32 pipe, "fp32" in FP32 followed by an FP64
    Rayleigh-quotient polish (and a double-float refinement where the polish
    misses the tolerance).  Returns an (len(ops), k) array of eigenvalues and,
    when asked, one Ns_i x k vector block per operator."""
    code = _which_code(which)
    n = len(ops)
    arr = (ctypes.c_void_p * n)(*[o._h for o in ops])
    opts = _lib.EigshOpts(int(k), code, float(tol), int(ncv or 0), int(maxiter or 0),
                          _precision_code(precision), 0, None, _lib.QS_MEM_HOST)
    vals = np.zeros((n, int(k)))
    vecs = None
    vptrs = None
    if return_eigenvectors:
        vecs = [np.zeros((o.Ns, int(k)), dtype=o.dtype, order="F") for o in ops]
        vptrs = (ctypes.c_void_p * n)(*[v.ctypes.data for v in vecs])
    inf = (_lib.EigshInfo * n)()
    _lib.check(_lib.load().qs_eigsh_batch(arr, n, ctypes.byref(opts), _lib.ptr(vals), vptrs, inf))
    if infos is not None:
        infos.extend(dict(nconv=i.nconv, restarts=i.restarts, matvecs=i.matvecs, max_rel_residual=i.max_rel_residual,
                          seconds=i.seconds) for i in inf)
    return (vals, vecs) if return_eigenvectors else vals


def evolve(H, v0, t0, times, eom="SE", iterate=False, imag_time=False, tol=1e-12, krylov_dim=30, precision="fp64",
           stepwise=False):
    """evolve(H, v0, t0, times; eom=:SE) for a static Hamiltonian (src/operators.jl:2073-2164).
    A BlockOps operator evolves block by block (tools.jl:2627-2678).
    stepwise=True (an addition) propagates from each time to the next instead
    of from v0 every time: the same states to tol, far fewer products for
    long time series."""
    from .blocks import BlockOps, evolve_blocks
    if isinstance(H, BlockOps):
        return evolve_blocks(H, v0, t0, times, iterate=iterate, imag_time=imag_time, tol=tol, krylov_dim=krylov_dim,
                             precision=precision)
    if str(eom) not in ("SE", "LvNE"):
        raise ArgumentError("eom must be :SE or :LvNE")
    if str(eom) == "LvNE":
        raise ArgumentError("LvNE evolution is not implemented on this engine")
    scalar = np.isscalar(times)
    ts = np.atleast_1d(np.asarray(times, dtype=np.float64))
    if np.ndim(v0) == 2:
        # a matrix of start states (src/operators.jl:2150-2164): every column's
        # recursion on one engine, states[:, column, time]
        V = np.asfortranarray(v0, dtype=np.complex128)
        if V.shape[0] != H.Ns:
            raise DimensionMismatch("operator and matrix dimensions do not match")
        off = ts - float(t0)
        sc = np.ascontiguousarray(-off + 0j if imag_time else -1j * off)
        out = np.zeros((H.Ns, V.shape[1], ts.size), dtype=np.complex128, order="F")
        _lib.check(_lib.load().qs_expm_columns(H._h, _lib.ptr(V), V.shape[1], _lib.ptr(sc), ts.size, float(tol),
                                               int(krylov_dim), _precision_code(precision), int(bool(imag_time)),
                                               _lib.ptr(out), _lib.QS_MEM_HOST))
        if iterate:
            return (out[:, :, i].copy() for i in range(ts.size))
        return out[:, :, 0].copy() if scalar else out
    v = np.ascontiguousarray(v0, dtype=np.complex128)
    if v.shape != (H.Ns,):
        raise DimensionMismatch("operator and vector dimensions do not match")
    out = np.zeros((H.Ns, ts.size), dtype=np.complex128, order="F")
    call = _lib.load().qs_evolve_stepwise if stepwise else _lib.load().qs_evolve
    _lib.check(call(H._h, _lib.ptr(v), float(t0), _lib.ptr(ts), ts.size, int(bool(imag_time)), float(tol),
                    int(krylov_dim), _precision_code(precision), _lib.ptr(out)))
    if iterate:
        return (out[:, i].copy() for i in range(ts.size))
    if scalar:
        return out[:, 0].copy()
    return out


class ExpmMultiplyParallel:
    """ExpmMultiplyParallel(A, a; dtype) with apply(v; work_array, overwrite_v, tol) (tools.jl:1605-1708)."""

    def __init__(self, A, a=1.0, dtype=None, copy=False):
        if not isinstance(A, QuantumLinearOperator):
            raise ArgumentError("A must be a device operator of this engine")
        if A.shape[0] != A.shape[1]:
            raise ArgumentError("A must be a square matrix")
        self.A = A
        self.a = complex(a)
        self.dtype = np.complex128

    def set_a(self, a, dtype=None):
        if dtype is not None and np.dtype(dtype) not in (np.dtype(np.complex128), np.dtype(np.float64)):
            raise ArgumentError("changing the exponential dtype requires constructing a new operator")
        self.a = complex(a)
        return self

    def apply(self, v, work_array=None, overwrite_v=False, tol=None, precision="fp64"):
        v_in = np.asarray(v)
        if v_in.shape[0] != self.A.shape[1]:
            raise DimensionMismatch("A and v dimensions do not match")
        if work_array is not None:
            if work_array.size != 2 * v_in.size:
                raise DimensionMismatch("work_array must contain twice as many elements as v")
            if work_array.dtype != np.complex128:
                raise ArgumentError("work_array must have element type ComplexF64")
        tol = 1e-12 if tol is None else float(tol)
        cols = v_in.reshape(v_in.shape[0], -1)
        a = np.array([self.a.real, self.a.imag])
        if cols.shape[1] == 1:
            x = np.ascontiguousarray(cols[:, 0], dtype=np.complex128)
            res = np.zeros_like(x)
            _lib.check(_lib.load().qs_expm_multiply(self.A._h, _lib.ptr(a), _lib.ptr(x), _lib.ptr(res), tol, 30,
                                                    _precision_code(precision)))
        else:
            # every column's Krylov recursion on one engine (src/operators.jl:1922-1949)
            X = np.asfortranarray(cols, dtype=np.complex128)
            res = np.zeros(X.shape, dtype=np.complex128, order="F")
            _lib.check(_lib.load().qs_expm_columns(self.A._h, _lib.ptr(X), X.shape[1], _lib.ptr(a), 1, tol, 30,
                                                   _precision_code(precision), 0, _lib.ptr(res), _lib.QS_MEM_HOST))
        res = res.reshape(v_in.shape)
        if work_array is not None:
            work_array[:v_in.size] = v_in.reshape(-1)
            work_array[v_in.size:] = res.reshape(-1)
            res = work_array[v_in.size:].reshape(v_in.shape)
        if overwrite_v:
            if not np.iscomplexobj(v):
                raise ArgumentError("overwrite_v requires an input with the output dtype")
            v[...] = res
            return v
        return res

    def __mul__(self, v):
        return self.apply(v)

    __matmul__ = __mul__


expm_multiply_parallel = ExpmMultiplyParallel


def set_a(op, a, dtype=None):
    return op.set_a(a, dtype)
