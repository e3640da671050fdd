"""GB300-native implementation of mATTOHF's hot path.

The Hartree-Fock Hamiltonian apply h[A(t)]|psi> (kinetic, Hartree, Fock
exchange) inside the RK4 real-time loop and the Krylov ground-state SCF, as
hand-written sm_103a CUDA behind the C ABI in ``include/mattohf.h``.
"""
from .inputs import RunConfig, read_input, define_afield, aave_from_samples, dipole_from_current  # noqa: F401
from .api import Batch, Context, MattohfError  # noqa: F401
from . import _capi  # noqa: F401

__all__ = ["RunConfig", "read_input", "define_afield", "aave_from_samples", "dipole_from_current", "Context",
           "Batch", "MattohfError"]
