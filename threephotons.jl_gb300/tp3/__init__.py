"""GB300 c3 + Bayes scorer for ThreePhotons.jl's structure-determination hot path.

Import with ``threephotons.jl_gb300`` on sys.path (the directory name holds a dot,
so it is a source directory, not an importable package name)::

    sys.path.insert(0, "<repo>/threephotons.jl_gb300")
    import tp3
"""
from ._lib import TP3Error, load, LIB_PATH, SIGNATURES  # noqa: F401
from ._lib import (TP3_ANGULAR_PERSISTENT, TP3_ANGULAR_TILE, TP3_HOST_INPUT_DIRECT, TP3_HOST_INPUT_STAGED,  # noqa: F401
                   TP3_MODE_AUTO, TP3_MODE_PLAIN_FP32,
                   TP3_MODE_TC_BF16X3, TP3_MODE_TC_TF32X3, TP3_MOVE_DRIFT, TP3_MOVE_LEARNED, TP3_MOVE_REFERENCE,
                   TP3_MOVE_SHELL_SO3)
from .api import (BasisTypeGB300, CUDA_init, FullCorrelation_parallized, SphericalHarmonicsVolume,  # noqa: F401
                  Umat, calculate_basis, complexBasis_choice, dq, energy, rotateStructure, rotationMatrix)
from . import structure  # noqa: F401
