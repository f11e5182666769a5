"""GB300-native pseudo-spectral 3D lattice evolution (the PSpectCosmo hot path).

The compute path is libpsc.so (hand-written sm_103a CUDA behind the C ABI declared in
include/psc.h); this package is its Python mirror of the reference's interface.
"""
from .params import MODEL_PHI2, MODEL_PHI2CHI2, Params
from .lattice import Ensemble, Lattice, PscError, generate_ic, load_library

__all__ = ["Params", "Lattice", "Ensemble", "PscError", "generate_ic", "load_library", "MODEL_PHI2",
           "MODEL_PHI2CHI2"]
