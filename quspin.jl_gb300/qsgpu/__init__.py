"""qsgpu -- GB300-native engine for QuSpin.jl's matrix-free Hamiltonian action on
symmetry-reduced spin-1/2 bases and its Krylov solvers.

This package is the host-side mirror of the reference's Julia interface over the
C ABI of libqsgpu (include/qsgpu.h).  Every compute call runs on the GPU; there
is no CPU fallback.
"""
from .basis import (SpinBasis1D, SpinBasisGeneral, get_amp, get_vec, int_to_state, normalization, project_from, project_to,
                    representative, state_at, state_index, state_to_int, states)
from .errors import ArgumentError, DimensionMismatch, ErrorException, UnsupportedError
from .operators import (ExpmMultiplyParallel, Hamiltonian, OperatorTerm, QuantumLinearOperator, apply, eigsh,
                        eigsh_batch, evolve, expm_multiply_parallel, isquantum_LinearOperator, set_a, toarray, tocsc,
                        tocsr)
from .blocks import (BlockDiagHamiltonian, BlockOps, BlockProjector, block_diag_hamiltonian, block_expm,
                     evolve_blocks)
from .server import Server
from .tools import (LanczosRows, expm_lanczos, ftlm_static_iteration, lanczos_batch, lanczos_full, lanczos_iter,
                    lin_comb_Q_T, ltlm_static_iteration)

__all__ = [
    "SpinBasis1D", "SpinBasisGeneral", "states", "state_index", "state_at", "representative", "normalization", "get_amp",
    "int_to_state", "state_to_int", "project_from", "project_to", "get_vec", "OperatorTerm", "QuantumLinearOperator", "Hamiltonian", "eigsh", "eigsh_batch", "evolve",
    "ExpmMultiplyParallel", "expm_multiply_parallel", "apply", "set_a", "isquantum_LinearOperator",
    "ArgumentError", "DimensionMismatch", "ErrorException", "UnsupportedError", "Server",
    "lanczos_full", "lanczos_iter", "lanczos_batch", "lin_comb_Q_T", "expm_lanczos", "ftlm_static_iteration",
    "ltlm_static_iteration", "LanczosRows", "BlockOps", "block_diag_hamiltonian", "block_expm", "evolve_blocks",
    "BlockProjector", "BlockDiagHamiltonian", "tocsc", "tocsr", "toarray",
]
