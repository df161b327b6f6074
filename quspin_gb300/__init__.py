"""quspin_gb300 -- GB300-native (sm_103a) hot path of QuSpin-style exact
diagonalisation: symmetry-reduced bases and Hamiltonians built on the GPU,
the sparse Hamiltonian apply, the truncated-Taylor expm_multiply_parallel and
the Lanczos recurrence, behind QuSpin's own Python signatures."""
from . import tools
from .basis import (spin_basis_1d, spin_basis_general, spinful_fermion_basis_general,
                    spinless_fermion_basis_general)
from .operators import hamiltonian, quantum_LinearOperator
from .sparse import DeviceCSR, DeviceDIA

__all__ = ["spin_basis_1d", "spin_basis_general", "spinless_fermion_basis_general", "spinful_fermion_basis_general",
           "hamiltonian", "quantum_LinearOperator", "DeviceCSR", "DeviceDIA", "tools"]
