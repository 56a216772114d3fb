"""GB300-native multigroup Monte Carlo transport for Abeille.

The compute path is a CUDA library for sm_103a behind the C-ABI declared in
include/abeille_gb300.h; this package builds it in-tree, binds it with ctypes,
and provides the problem builder, synthetic decks and the reference-shaped
Transporter / driver classes.
"""
from . import abi, decks  # noqa: F401
from .engine import (BatchEngine, Engine, FixedSource, GpuDeltaTracker, GpuSurfaceTracker, PowerIterator, Server,  # noqa: F401
                     PARTICLE_DTYPE, SITE_DTYPE, TRACE_DTYPE)
from .problem import ProblemBuilder, infix_to_rpn, tokenize_region  # noqa: F401

__version__ = "0.4.0"
