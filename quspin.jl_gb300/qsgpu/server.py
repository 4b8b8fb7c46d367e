"""Server: a request loop for ground-state and time-evolution solves of mixed
sizes and sectors on one GPU (qs_server_* in include/qsgpu.h).

Requests are admitted in arrival order against a device-memory budget,
operators are cached by sector and terms, and all running solves advance in
the same batched launches; a request that arrives while others run joins them
as soon as its operator is built.  The reference has no counterpart: it runs
one eigsh / evolve per call (src/operators.jl:1558-1640, 2073-2164).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .basis import basis_spec
from .errors import ArgumentError, raise_status
from .operators import _pack_terms, _precision_code


def _result_dict(r):
    return {"status": int(r.status), "Ns": int(r.Ns), "values": [r.values[i] for i in range(r.nvalues)],
            "submit_s": r.submit_s, "admit_s": r.admit_s, "done_s": r.done_s, "matvecs": int(r.matvecs),
            "restarts": int(r.restarts), "error_estimate": r.error_estimate, "vector_len": int(r.vector_len),
            "message": r.message.decode(errors="replace")}


class Server:
    def __init__(self, hbm_budget_gb=150.0, max_slots=64, precision="fp64df", op_cache=True, chunk_steps=8,
                 builders=4, policy="fifo", max_wait_s=10.0):
        """policy "fifo" admits in arrival order; "sjf" admits the smallest
        estimated work first, except a request waiting longer than max_wait_s.
        precision "fp64" or "fp64df" sets the Krylov storage of every solve;
        "fp32" runs eigsh in FP32 with an FP64 polish of each eigenpair (FP64
        eigenvalues, FP32-level eigenvector residuals) and evolve in fp64df."""
        if policy not in ("fifo", "sjf"):
            raise ArgumentError("policy must be fifo or sjf")
        opts = _lib.ServerOpts(float(hbm_budget_gb) * 1e9, int(max_slots), _precision_code(precision),
                               0 if op_cache else 1, int(chunk_steps), int(builders),
                               0 if policy == "fifo" else 1, float(max_wait_s), 0)
        h = ctypes.c_void_p()
        _lib.check(_lib.load().qs_server_create(ctypes.byref(opts), ctypes.byref(h)))
        self._h = h
        self._kind = {}

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().qs_server_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit_eigsh(self, basis, terms, k=1, which="SA", tol=0.0, ncv=None, maxiter=None, v0=None, seed=0,
                     want_vector=False):
        """eigsh(H; k, which, tol, ncv, maxiter) on the sector `basis` (SpinBasis1D keywords)."""
        w = str(which).upper()
        if w not in ("SA", "LA"):
            raise ArgumentError("which must be SA or LA on this engine")
        r = self._prepare(_lib.QS_REQ_EIGSH, basis, terms, v0, dict(
            k=int(k), which=0 if w == "SA" else 1, tol=float(tol), ncv=int(ncv or 0), maxiter=int(maxiter or 0),
            seed=int(seed), want_vector=int(bool(want_vector))))
        self._kind[r] = ("eigsh", int(k))
        return r

    def submit_evolve(self, basis, terms, t, v0=None, imag_time=False, tol=1e-12, krylov_dim=30, seed=0,
                      want_vector=True):
        """evolve(H, v0, 0, [t]; eom=:SE, imag_time, tol, krylov_dim) on the sector `basis`."""
        r = self._prepare(_lib.QS_REQ_EVOLVE, basis, terms, None if v0 is None else np.asarray(v0, np.complex128),
                          dict(t=float(t), imag_time=int(bool(imag_time)), tol=float(tol),
                               krylov_dim=int(krylov_dim), seed=int(seed), want_vector=int(bool(want_vector))))
        self._kind[r] = ("evolve", 1)
        return r

    def _prepare(self, kind, basis, terms, v0, fields):
        spec = basis_spec(**basis)
        arr, keep = _pack_terms(terms)
        r = _lib.Request()
        r.kind = kind
        r.basis = spec
        r.terms = arr
        r.nterms = len(terms)
        for name, v in fields.items():
            setattr(r, name, v)
        if v0 is not None:
            v0 = np.ascontiguousarray(v0)
            r.v0 = _lib.ptr(v0)
            r.v0_len = v0.size * (2 if np.iscomplexobj(v0) else 1)
        t = ctypes.c_int64()
        _lib.check(_lib.load().qs_server_submit(self._h, ctypes.byref(r), ctypes.byref(t)))
        del keep, v0
        return int(t.value)

    def poll(self, ticket):
        res = _lib.Result()
        st = _lib.load().qs_server_poll(self._h, int(ticket), ctypes.byref(res))
        if st not in (0, _lib.QS_PENDING) and res.status == 0:
            _lib.check(st)
        return _result_dict(res)

    def wait(self, ticket, timeout=None):
        """Blocks until the request finishes; raises the request's error if it failed."""
        res = _lib.Result()
        st = _lib.load().qs_server_wait(self._h, int(ticket), float(timeout or 0.0), ctypes.byref(res))
        d = _result_dict(res)
        if st == _lib.QS_PENDING:
            raise TimeoutError(f"request {ticket} still running after {timeout} s")
        if st != 0:
            msg = d["message"] or _lib.load().qs_last_error().decode(errors="replace")
            raise_status(st, msg)
        return d

    def vector(self, ticket):
        """Eigenvectors (Ns x k) or the evolved state (Ns, complex) of a finished request."""
        d = self.poll(ticket)
        if d["status"] != 0:
            raise ArgumentError("request has no result")
        n, ln = d["Ns"], d["vector_len"]
        if ln == 0:
            raise ArgumentError("the request did not keep its vector (want_vector=False)")
        buf = np.zeros(ln)
        _lib.check(_lib.load().qs_server_vector(self._h, int(ticket), _lib.ptr(buf), ln))
        kind, k = self._kind.get(int(ticket), ("eigsh", 1))
        if kind == "evolve":
            return buf.view(np.complex128)
        comps = ln // (n * k)
        if comps == 2:
            return buf.view(np.complex128).reshape(k, n).T
        return buf.reshape(k, n).T

    def release(self, ticket):
        _lib.check(_lib.load().qs_server_release(self._h, int(ticket)))
        self._kind.pop(int(ticket), None)

    def stats(self):
        c = _lib.ServerCounters()
        _lib.check(_lib.load().qs_server_stats(self._h, ctypes.byref(c)))
        return {name: getattr(c, name) for name, _ in c._fields_}
