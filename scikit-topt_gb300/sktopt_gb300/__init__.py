"""GB300-native engine for scikit-topt's density-method hot path.

Host-side classes mirror the reference's plugin surface (FEM, filters,
optimizers); every numerical kernel runs in ``libtopt_gb300.so`` (CUDA,
sm_103a).  There is no CPU fallback: when the library is missing the first
call raises.
"""
from ._build import build, library_path

__version__ = "0.1.0"

__all__ = ["build", "library_path", "__version__"]
