"""polyq_gb300 -- GB300-native amplitude evaluation for Clifford+T path sums.

The per-branch enumeration of polyq's cached engine runs as hand-written sm_103a CUDA
behind a C-ABI (include/polyq_gb300.h); this package is its Python front-end.
"""
from .circuit import Circuit, phase_from_pi_fraction, phase_from_radians  # noqa: F401
from .rng import Rng, random_clifford_t, random_layered  # noqa: F401
from .sim import Batch, Simulator, get_tuning, pack_bits, set_tuning  # noqa: F401

__all__ = ["Circuit", "Simulator", "Batch", "Rng", "random_clifford_t", "random_layered", "pack_bits",
           "phase_from_pi_fraction", "phase_from_radians", "set_tuning", "get_tuning"]
