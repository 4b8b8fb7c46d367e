"""Symmetry-block tools of QuSpin.jl's ``tools.jl`` (block_diag_hamiltonian,
BlockOps, evolve on BlockOps, block_expm) on the device.

Each block is a sector basis with its own assembled Hamiltonian.  The
reference stacks the blocks into sparse matrices (``hcat`` of projectors,
``blockdiag`` of Hamiltonians); here the projector and the block-diagonal
operator are device-backed objects that apply the blocks one by one, and the
block evolution runs every block's Krylov recursions on one batched engine
(``qs_block_expm``): c_b = P_b^H psi, exp(s H_b) c_b, sum_b P_b state_b.
Static Hamiltonians only (dynamic terms are outside this engine).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .basis import SpinBasis1D, project_from, project_to
from .errors import ArgumentError, DimensionMismatch, UnsupportedError
from .operators import Hamiltonian, OperatorTerm, _precision_code


def _block_keywords(values):
    """tools.jl:2170-2178: keyword names as symbols, Nup renamed nup."""
    out = {}
    for k, v in dict(values).items():
        name = str(k)
        out["nup" if name == "Nup" else name] = v
    return out


def _construct_block_basis(basis_con, basis_args, basis_kwargs, block):
    """tools.jl:2180-2186: a basis, or basis_con(basis_args...; basis_kwargs, block...)."""
    if isinstance(block, SpinBasis1D):
        return block
    if not isinstance(block, dict):
        raise ArgumentError("each block must be a basis or dictionary")
    kw = _block_keywords(basis_kwargs)
    kw.update(_block_keywords(block))
    try:
        return basis_con(*basis_args, **kw)
    except ArgumentError as exc:
        if "empty" in str(exc):
            return None     # an empty sector: the reference keeps only length(basis) > 0
        raise


def _normalize_block_terms(static):
    """tools.jl:2090-2097."""
    if all(isinstance(t, OperatorTerm) for t in static):
        return list(static)
    return [OperatorTerm(str(t[0]), list(t[1])) for t in static]


def _require_static(dynamic):
    if dynamic:
        raise UnsupportedError("dynamic (time-dependent) block terms are outside this engine: static Hamiltonians only")


class BlockProjector:
    """hcat(projection_matrix(basis_b)...): rows 2^L, columns the stacked
    block coefficients.  ``P @ c`` and ``P.H @ psi`` run on the device."""

    def __init__(self, bases, pcon=False):
        self.bases = list(bases)
        self.pcon = pcon
        self.sizes = [b.Ns for b in self.bases]
        rows = {int(_lib.load().qs_basis_projection_rows(b._h, 1 if pcon else 0)) for b in self.bases}
        if len(rows) != 1:
            raise DimensionMismatch("the blocks must share one projection space")
        self.shape = (rows.pop(), int(sum(self.sizes)))

    def _split(self, c):
        offs = np.cumsum([0] + self.sizes)
        return [c[offs[i]:offs[i + 1]] for i in range(len(self.bases))]

    def dot(self, c):
        c = np.asarray(c)
        if c.shape[0] != self.shape[1]:
            raise DimensionMismatch("vector length must equal the stacked block dimension")
        out = None
        for b, part in zip(self.bases, self._split(c)):
            y = project_from(b, np.asarray(part, dtype=np.complex128), pcon=self.pcon)
            out = y if out is None else out + y
        return out

    __matmul__ = dot

    def rdot(self, psi):
        """P^H psi: the stacked projections onto every block."""
        psi = np.asarray(psi, dtype=np.complex128)
        return np.concatenate([project_to(b, psi, pcon=self.pcon) for b in self.bases])

    @property
    def H(self):
        proj = self

        class _Adjoint:
            shape = (proj.shape[1], proj.shape[0])

            def dot(self, psi):
                return proj.rdot(psi)

            __matmul__ = dot
        return _Adjoint()

    def toarray(self):
        n = self.shape[1]
        return np.column_stack([self.dot(np.eye(n, dtype=np.complex128)[:, j]) for j in range(n)])


class BlockDiagHamiltonian:
    """blockdiag(H_b.data...): the block Hamiltonians side by side; ``dot``
    applies each block's assembled operator to its slice of the vector."""

    def __init__(self, hamiltonians):
        self.blocks = list(hamiltonians)
        self.sizes = [h.Ns for h in self.blocks]
        n = int(sum(self.sizes))
        self.shape = (n, n)
        self.dtype = np.complex128 if any(h.dtype == np.complex128 for h in self.blocks) else np.float64

    def dot(self, v):
        v = np.asarray(v)
        if v.shape[0] != self.shape[1]:
            raise DimensionMismatch("vector length must equal the stacked block dimension")
        offs = np.cumsum([0] + self.sizes)
        return np.concatenate([h.dot(v[offs[i]:offs[i + 1]]) for i, h in enumerate(self.blocks)])

    __matmul__ = dot

    def toarray(self):
        n = self.shape[1]
        return np.column_stack([self.dot(np.eye(n, dtype=self.dtype)[:, j]) for j in range(n)])


def block_diag_hamiltonian(blocks, static, dynamic, basis_con, basis_args, dtype=np.complex128, basis_kwargs=None,
                           get_proj_kwargs=None, get_proj=True, check_symm=True, check_herm=True, check_pcon=True):
    """block_diag_hamiltonian(blocks, static, dynamic, basis_con, basis_args,
    dtype; basis_kwargs, get_proj_kwargs, get_proj, check_*) (tools.jl:2213-2301):
    (P, H) or H, with P a BlockProjector and H a BlockDiagHamiltonian on the device."""
    _require_static(dynamic)
    terms = _normalize_block_terms(static)
    bases = [b for b in (_construct_block_basis(basis_con, basis_args, basis_kwargs or {}, blk) for blk in blocks)
             if b is not None]
    if not bases:
        raise ArgumentError("at least one block is required")
    hams = [Hamiltonian(b, terms, check_symm=check_symm, check_herm=check_herm, check_pcon=check_pcon)
            for b in bases]
    H = BlockDiagHamiltonian(hams)
    if not get_proj:
        return H
    kw = _block_keywords(get_proj_kwargs or {})
    if set(kw) - {"sparse"}:
        raise ArgumentError(f"unsupported projector keyword(s): {sorted(set(kw) - {'sparse'})}")
    return BlockProjector(bases), H


class BlockOps:
    """BlockOps(blocks, static, dynamic, basis_con, basis_args, dtype;
    basis_kwargs, get_proj_kwargs, save_previous_data, compute_all_blocks,
    check_*) (tools.jl:2303-2443): block bases keyed by repr(block); the
    block Hamiltonians (H_dict) and projectors (P_dict) are built on demand."""

    def __init__(self, blocks, static, dynamic, basis_con, basis_args, dtype=np.complex128, basis_kwargs=None,
                 get_proj_kwargs=None, save_previous_data=True, compute_all_blocks=False, check_symm=True,
                 check_herm=True, check_pcon=True):
        _require_static(dynamic)
        kw = _block_keywords(get_proj_kwargs or {})
        if set(kw) - {"sparse"}:
            raise ArgumentError(f"unsupported projector keyword(s): {sorted(set(kw) - {'sparse'})}")
        self.basis_dict = {}
        self.H_dict = {}
        self.P_dict = {}
        self.dtype = dtype
        self.static = _normalize_block_terms(static)
        self.dynamic = list(dynamic)
        self.save_previous_data = bool(save_previous_data or compute_all_blocks)
        self.sparse_projectors = bool(kw.get("sparse", True))
        self.basis_kwargs = dict(basis_kwargs or {})
        self.check_symm, self.check_herm, self.check_pcon = check_symm, check_herm, check_pcon
        for blk in blocks:
            b = _construct_block_basis(basis_con, basis_args, self.basis_kwargs, blk)
            if b is not None and b.Ns > 0:
                self.basis_dict[repr(blk)] = b
        if compute_all_blocks:
            self.compute_all_blocks()

    def _hamiltonian(self, basis):
        return Hamiltonian(basis, self.static, check_symm=self.check_symm, check_herm=self.check_herm,
                           check_pcon=self.check_pcon)

    def compute_all_blocks(self):
        """compute_all_blocks!(operator) (tools.jl:2356-2377)."""
        for key, b in self.basis_dict.items():
            self.P_dict.setdefault(key, BlockProjector([b]))
            if key not in self.H_dict:
                self.H_dict[key] = self._hamiltonian(b)
        return self

    def update_blocks(self, blocks, basis_con, basis_args, compute_all_blocks=False):
        """update_blocks!(operator, blocks, basis_con, basis_args; compute_all_blocks) (tools.jl:2379-2399)."""
        for blk in blocks:
            key = repr(blk)
            if key in self.basis_dict:
                continue
            b = _construct_block_basis(basis_con, basis_args, self.basis_kwargs, blk)
            if b is not None and b.Ns > 0:
                self.basis_dict[key] = b
        if compute_all_blocks:
            self.compute_all_blocks()
        return self

    def _block_hamiltonians(self):
        """Every block's Hamiltonian, cached when save_previous_data (tools.jl:2401-2443)."""
        out = []
        for key, b in self.basis_dict.items():
            if key in self.H_dict:
                out.append(self.H_dict[key])
                continue
            h = self._hamiltonian(b)
            if self.save_previous_data:
                self.H_dict[key] = h
                self.P_dict.setdefault(key, BlockProjector([b]))
            out.append(h)
        return out


def _block_run(operator, psi_0, scales, tol, krylov_dim, precision):
    hams = operator._block_hamiltonians()
    if not hams:
        raise ArgumentError("initial state has no projection onto the selected blocks")
    psi = np.ascontiguousarray(psi_0, dtype=np.complex128)
    rows = int(_lib.load().qs_basis_projection_rows(hams[0].basis._h, 0))
    if psi.shape != (rows,):
        raise DimensionMismatch("psi_0 must have the length of the full space")
    sc = np.ascontiguousarray(np.asarray(scales, dtype=np.complex128))
    out = np.zeros((rows, sc.size), dtype=np.complex128, order="F")
    handles = (ctypes.c_void_p * len(hams))(*[h._h.value for h in hams])
    _lib.check(_lib.load().qs_block_expm(handles, len(hams), 0, _lib.ptr(psi), _lib.ptr(sc), int(sc.size),
                                         float(tol), int(krylov_dim), _precision_code(precision), _lib.ptr(out),
                                         _lib.QS_MEM_HOST))
    return out


def evolve_blocks(operator, psi_0, t0, times, iterate=False, n_jobs=1, block_diag=False, stack_state=False,
                  imag_time=False, tol=1e-12, krylov_dim=30, precision="fp64"):
    """evolve(operator::BlockOps, psi_0, t0, times; iterate, n_jobs,
    block_diag, stack_state, imag_time, tol, krylov_dim) (tools.jl:2627-2678):
    every block's _krylov_expmv_times on one engine; n_jobs and block_diag
    (the reference's CPU parallelism and its combined-matrix variant) do not
    change the result and have nothing to select here."""
    if int(n_jobs) <= 0:
        raise ArgumentError("n_jobs must be positive")
    scalar = np.isscalar(times)
    ts = np.atleast_1d(np.asarray(times, dtype=np.float64))
    scales = [-(t - t0) if imag_time else -1j * (t - t0) for t in ts]
    out = _block_run(operator, psi_0, scales, tol, krylov_dim, precision)
    if iterate:
        return (out[:, i].copy() for i in range(ts.size))
    return out[:, 0].copy() if scalar else out


def block_expm(operator, psi_0, H_time_eval=0.0, iterate=False, n_jobs=1, block_diag=False, a=-1j, start=None,
               stop=None, endpoint=True, num=50, shift=None, tol=1e-12, krylov_dim=30, precision="fp64"):
    """block_expm(operator::BlockOps, psi_0; H_time_eval, iterate, n_jobs,
    block_diag, a, start, stop, endpoint, num, shift) (tools.jl:2680-2718):
    exp(a s (H + shift)) psi_0 for s = 1 or s on range(start, stop; num).
    A shift multiplies each result by exp(a s shift), which is what adding
    shift * I to every block does."""
    if int(n_jobs) <= 0:
        raise ArgumentError("n_jobs must be positive")
    if start is None and stop is None:
        grid = np.array([1.0])
    else:
        grid = np.linspace(start, stop, int(num) + (0 if endpoint else 1))
        if not endpoint:
            grid = grid[:-1]
    scales = grid * a
    out = _block_run(operator, psi_0, scales, tol, krylov_dim, precision)
    if shift is not None:
        out = out * np.exp(np.asarray(scales) * shift)[None, :]
    if iterate:
        return (out[:, i].copy() for i in range(out.shape[1]))
    return out[:, 0].copy() if out.shape[1] == 1 else out
