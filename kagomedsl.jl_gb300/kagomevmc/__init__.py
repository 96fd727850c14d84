"""kagomevmc -- GB300-native variational Monte Carlo for Gutzwiller-projected
parton states of the kagome Heisenberg model (the hot path of KagomeDSL.jl).

The compute path is libkvmc.so (CUDA, sm_103a) behind the C ABI of
include/kvmc.h; this package is the host-side mirror of the reference's
constructors and Carlo.jl callbacks.
"""
from ._lib import (ArgumentError, BoundsError, DeviceError, KvmcError, SingularException, EXPORTS, LIB_PATH,
                   load)
from .lattice import PI_LINK_IN, PI_LINK_INTER, DoubleKagome, Hamiltonian, Hmat, get_nn, ns, orbitals
from .ansatz import Ansatz, ansatz_hmat, energy_and_gradient, estimate, orbital_derivatives
from .montecarlo import (MC, Engine, Evaluator, Group, MCContext, init_, init_conf_qr, measure_, read_checkpoint_,
                         register_evaluables, sweep_, write_checkpoint)

__all__ = [
    "ArgumentError", "BoundsError", "DeviceError", "KvmcError", "SingularException", "EXPORTS", "LIB_PATH", "load",
    "PI_LINK_IN", "PI_LINK_INTER", "DoubleKagome", "Hamiltonian", "Hmat", "get_nn", "ns", "orbitals",
    "MC", "Engine", "Evaluator", "Group", "MCContext", "init_", "init_conf_qr", "measure_", "read_checkpoint_",
    "register_evaluables", "sweep_", "write_checkpoint",
    "Ansatz", "ansatz_hmat", "energy_and_gradient", "estimate", "orbital_derivatives",
]
