"""GPU tools of the hot path: expm_multiply_parallel, Lanczos, matvec."""
from .batched import MultiSectorExpm
from .block_tools import block_diag_hamiltonian, block_ops
from .floquet import Floquet
from .expm_multiply_parallel import ExpmMultiplyParallel, expm_multiply_parallel
from .lanczos import (FTLM_static_iteration, LTLM_static_iteration, expm_lanczos, lanczos_full, lanczos_iter,
                      lin_comb_Q_T)
from .matvec import get_matvec_function, matvec

__all__ = ["Floquet", "FTLM_static_iteration", "LTLM_static_iteration", "ExpmMultiplyParallel", "expm_multiply_parallel", "lanczos_full", "lanczos_iter", "lin_comb_Q_T",
           "expm_lanczos", "matvec", "get_matvec_function", "MultiSectorExpm",
           "block_ops", "block_diag_hamiltonian"]
