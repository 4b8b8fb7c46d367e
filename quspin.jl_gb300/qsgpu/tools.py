"""Krylov tools of QuSpin.jl's ``tools.jl`` (lanczos_full, lanczos_iter,
lin_comb_Q_T, expm_lanczos, ftlm_static_iteration, ltlm_static_iteration) on
the device.

The Lanczos recurrence runs on the batched engine (``qs_lanczos_run``); the
Lanczos vectors stay in device memory and are combined, projected and dotted
there.  ``Q_T`` is a :class:`LanczosRows` (rows = Lanczos vectors, as in the
reference); ``numpy.asarray(Q_T)`` copies it to the host.  The small m x m
tridiagonal eigenproblem (``eigen(SymTridiagonal)`` in the reference) is solved
on the host.  :func:`lanczos_batch` runs the recurrences of many start vectors
(e.g. the random vectors of a finite-temperature estimate) in the same
launches.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .errors import ArgumentError, DimensionMismatch
from .operators import QuantumLinearOperator


def _require_op(A, what="A"):
    if not isinstance(A, QuantumLinearOperator):
        raise TypeError(f"{what} must be a QuantumLinearOperator or Hamiltonian of this package")
    return A


def _tridiagonal_eigen(alphas, betas):
    """eigen(SymTridiagonal(alphas, betas)): ascending values, vectors in columns."""
    m = alphas.size
    T = np.diag(alphas.astype(np.float64))
    if m > 1:
        T += np.diag(betas[: m - 1], 1) + np.diag(betas[: m - 1], -1)
    return np.linalg.eigh(T)


class _LanczosSet:
    """Device-resident Lanczos bases of one operator (qs_lanczos)."""

    def __init__(self, A, V0, m, full_ortho=False, eps=None):
        _require_op(A)
        V0 = np.asarray(V0)
        if V0.ndim == 1:
            V0 = V0[:, None]
        n, R = V0.shape
        if n != A.Ns:
            raise DimensionMismatch("start vectors must have length Ns")
        cplx = np.iscomplexobj(V0) or A.dtype == np.complex128
        buf = np.asfortranarray(V0, dtype=np.complex128 if cplx else np.float64)
        opts = _lib.LanczosOpts(int(m), 1 if full_ortho else 0, float(eps or 0.0),
                                1 if np.iscomplexobj(V0) else 0, _lib.QS_MEM_HOST)
        h = ctypes.c_void_p()
        _lib.check(_lib.load().qs_lanczos_run(A._h, ctypes.byref(opts), int(R), _lib.ptr(buf), ctypes.byref(h)))
        self._h = h
        self.A = A
        self.n, self.R, self.m = n, R, int(m)
        self.complex = bool(_lib.load().qs_lanczos_complex(h))
        self.dtype = np.complex128 if self.complex else np.float64
        self.coeffs = []
        for s in range(R):
            a = np.zeros(self.m)
            b = np.zeros(max(0, self.m - 1))
            used = _lib.i32()
            _lib.check(_lib.load().qs_lanczos_coefficients(h, s, _lib.ptr(a), _lib.ptr(b) if b.size else None,
                                                           ctypes.byref(used)))
            u = int(used.value)
            self.coeffs.append((a[:u].copy(), b[: max(0, u - 1)].copy(), u))
        self._overlaps = {}

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            _lib.load().qs_lanczos_destroy(h)
            self._h = None

    def rows(self, s):
        used = self.coeffs[s][2]
        out = np.empty((used, self.n), dtype=self.dtype)
        _lib.check(_lib.load().qs_lanczos_rows(self._h, s, _lib.ptr(out), _lib.QS_MEM_HOST))
        return out

    def combine(self, s, coeff):
        """sum_i coeff[i, c] q_i (coeff used x nc, any dtype) as complex n x nc."""
        coeff = np.asarray(coeff, dtype=np.complex128)
        if coeff.ndim == 1:
            coeff = coeff[:, None]
        c = np.asfortranarray(coeff)
        out = np.empty((self.n, c.shape[1]), dtype=np.complex128, order="F")
        _lib.check(_lib.load().qs_lanczos_combine(self._h, s, _lib.ptr(c), int(c.shape[1]), _lib.ptr(out),
                                                  _lib.QS_MEM_HOST))
        return out

    def overlaps(self, obs):
        """<q_i, O q_0> of every start (R x m complex), one product per start."""
        _require_op(obs, "observable")
        key = obs._h.value
        if key not in self._overlaps:
            out = np.zeros((self.R, self.m), dtype=np.complex128)
            _lib.check(_lib.load().qs_lanczos_overlaps(self._h, obs._h, _lib.ptr(out)))
            self._overlaps[key] = (obs, out)
        return self._overlaps[key][1]

    def ritz_matrix(self, s, obs, Y):
        """R^* O R with R = Q^T Y (Y used x nv real): nv x nv complex."""
        _require_op(obs, "observable")
        Y = np.asfortranarray(Y, dtype=np.float64)
        nv = Y.shape[1]
        out = np.empty((nv, nv), dtype=np.complex128, order="F")
        _lib.check(_lib.load().qs_lanczos_ritz_matrix(self._h, s, obs._h, _lib.ptr(Y), int(nv), _lib.ptr(out)))
        return out


class LanczosRows:
    """Q_T of one start vector: its Lanczos vectors as rows, held on the
    device.  ``len`` is the number of rows; iteration yields the rows;
    ``numpy.asarray`` copies all of them (used x Ns)."""

    def __init__(self, lset, s):
        self._set = lset
        self._s = s
        self.used = lset.coeffs[s][2]
        self.shape = (self.used, lset.n)
        self.dtype = lset.dtype

    def __len__(self):
        return self.used

    def __array__(self, dtype=None, copy=None):
        a = self._set.rows(self._s)
        return a if dtype is None else a.astype(dtype)

    def __iter__(self):
        return iter(list(np.asarray(self)))

    def __getitem__(self, idx):
        return np.asarray(self)[idx]


def _eig_rows(lset, s):
    a, b, _ = lset.coeffs[s]
    E, V = _tridiagonal_eigen(a, b)
    return E, V, LanczosRows(lset, s)


def lanczos_full(A, v0, m, full_ortho=False, out=None, eps=None):
    """lanczos_full(A, v0, m; full_ortho, out, eps) (src/tools.jl:2742-2805):
    (E, V, Q_T).  The rows stay on the device; when ``out`` (m x Ns) is given
    the rows are also copied into it."""
    v0 = np.asarray(v0)
    if not 1 <= int(m) < v0.size:
        raise ArgumentError("Lanczos dimension m must satisfy 1 <= m < length(v0)")
    if not np.linalg.norm(v0) > 0:
        raise ArgumentError("initial Lanczos vector must be nonzero")
    lset = _LanczosSet(A, v0, m, full_ortho, eps)
    E, V, Q = _eig_rows(lset, 0)
    if out is not None:
        if out.shape != (int(m), v0.size):
            raise DimensionMismatch("out must have shape (m, length(v0))")
        out[: Q.used] = np.asarray(Q)
    return E, V, Q


def lanczos_iter(A, v0, m, return_vec_iter=True, copy_v0=True, copy_A=False, eps=None):
    """lanczos_iter(A, v0, m; return_vec_iter, copy_v0, copy_A, eps)
    (src/tools.jl:2884-2907): (E, V) or (E, V, rows).  The reference
    regenerates the vectors with one product each; here the recurrence keeps
    them on the device and the iterator reads them back (copy_v0 and copy_A
    have nothing to protect)."""
    E, V, Q = lanczos_full(A, v0, m, False, None, eps)
    return (E, V, Q) if return_vec_iter else (E, V)


def lanczos_batch(A, V0, m, full_ortho=False, eps=None):
    """lanczos_full for every column of V0 (Ns x R) at once, the R recurrences
    stepping in the same launches: a list of (E, V, Q_T), one per column.  A
    Fortran-ordered V0 (e.g. the transpose of an R x Ns array) is passed
    without a host copy."""
    V0 = np.asarray(V0)
    if V0.ndim != 2:
        raise ArgumentError("V0 must be Ns x R")
    if not 1 <= int(m) < V0.shape[0]:
        raise ArgumentError("Lanczos dimension m must satisfy 1 <= m < length(v0)")
    lset = _LanczosSet(A, V0, m, full_ortho, eps)
    return [_eig_rows(lset, s) for s in range(lset.R)]


def lin_comb_Q_T(coeff, Q_T, out=None):
    """lin_comb_Q_T(coeff, Q_T; out) (src/tools.jl:2909-2945): sum_i coeff[i] Q_T[i, :]."""
    if not isinstance(Q_T, LanczosRows):
        raise TypeError("Q_T must be the rows returned by lanczos_full / lanczos_iter / lanczos_batch")
    coeff = np.asarray(coeff)
    if coeff.ndim != 1 or coeff.size != Q_T.used:
        raise DimensionMismatch("one coefficient is required per Lanczos vector")
    res = Q_T._set.combine(Q_T._s, coeff)[:, 0]
    if not (np.iscomplexobj(coeff) or Q_T.dtype == np.complex128):
        res = res.real.copy()
    if out is not None:
        if out.shape != (Q_T.shape[1],):
            raise DimensionMismatch("out must match a Lanczos vector")
        out[:] = res
        return out
    return res


def expm_lanczos(E, V, Q_T, a=1, out=None):
    """expm_lanczos(E, V, Q_T; a, out) (src/tools.jl:2947-2952): exp(a A) v0 / ||v0||
    from the Lanczos decomposition."""
    E = np.asarray(E)
    V = np.asarray(V)
    if not (E.size == V.shape[0] == V.shape[1]):
        raise DimensionMismatch("E and V dimensions must agree")
    return lin_comb_Q_T(V @ (np.exp(a * E) * V[0, :]), Q_T, out)


def _temperatures(beta):
    scalar = np.isscalar(beta)
    betas = np.atleast_1d(np.asarray(beta, dtype=np.float64))
    return scalar, betas


def ftlm_static_iteration(observables, E, V, Q_T, beta=0):
    """ftlm_static_iteration(observables, E, V, Q_T; beta) (src/tools.jl:2966-3013):
    one finite-temperature Lanczos iteration; observables maps keys to
    operators of this package.  Returns (results, identity)."""
    E = np.asarray(E)
    V = np.asarray(V)
    m = E.size
    if V.shape != (m, m):
        raise DimensionMismatch("Lanczos inputs must share the same Krylov dimension")
    if not isinstance(Q_T, LanczosRows):
        raise TypeError("Q_T must be the rows returned by lanczos_full / lanczos_iter / lanczos_batch")
    if Q_T.used != m:
        raise DimensionMismatch("too few Lanczos vectors" if Q_T.used < m else "too many Lanczos vectors")
    scalar, betas = _temperatures(beta)
    coefficients = V @ (V[0, :][:, None] * np.exp(-E[:, None] * betas[None, :]))
    results = {}
    for key, obs in observables.items():
        ov = Q_T._set.overlaps(obs)[Q_T._s, :m]
        real = Q_T.dtype == np.float64 and obs.dtype == np.float64
        r = (ov.real if real else ov) @ coefficients
        results[key] = r[0] if scalar else r
    identity = coefficients[0, :]
    return results, (identity[0] if scalar else identity)


def ltlm_static_iteration(observables, E, V, Q_T, beta=0):
    """ltlm_static_iteration(observables, E, V, Q_T; beta) (src/tools.jl:3015-3068):
    one low-temperature Lanczos iteration (Ritz vectors up to the Boltzmann
    cutoff at the smallest beta).  Returns (results, identity)."""
    E = np.asarray(E)
    V = np.asarray(V)
    m = E.size
    if V.shape != (m, m):
        raise DimensionMismatch("Lanczos inputs must share the same Krylov dimension")
    if not isinstance(Q_T, LanczosRows):
        raise TypeError("Q_T must be the rows returned by lanczos_full / lanczos_iter / lanczos_batch")
    scalar, betas = _temperatures(beta)
    if betas.size == 0:
        raise ArgumentError("beta must be nonempty")
    if Q_T.used != m:
        raise DimensionMismatch("too few Lanczos vectors" if Q_T.used < m else "too many Lanczos vectors")
    nv = m
    bmin = betas.min()
    if bmin > 0:
        half = np.exp(-(E - E.min()) * bmin / 2)
        keep = np.nonzero(half > np.finfo(np.float64).eps)[0]
        nv = int(keep[-1]) + 1 if keep.size else 1
    En = E[:nv]
    W = V[0, :nv][:, None] * np.exp(-En[:, None] * betas[None, :] / 2)
    results = {}
    for key, obs in observables.items():
        P = Q_T._set.ritz_matrix(Q_T._s, obs, V[:, :nv])
        vals = np.array([W[:, b] @ (P @ W[:, b]) for b in range(betas.size)])
        if Q_T.dtype == np.float64 and obs.dtype == np.float64:
            vals = vals.real
        results[key] = vals[0] if scalar else vals
    identity = np.array([np.sum(np.abs(V[0, :nv]) ** 2 * np.exp(-b * En)) for b in betas])
    return results, (identity[0] if scalar else identity)
