"""GB300-native (sm_103a) drop-in engine for ROOTPWA's extended-likelihood hot path.

pwaLikelihood (DoEval / Gradient / FdF / Hessian, rank-reflectivity parameter
layout) and ampIntegralMatrix run as hand-written CUDA kernels in
libpwa_gb300.so behind the C ABI of include/pwa_gb300.h.
"""
from ._native import PwaError, lib  # noqa: F401
from .likelihood import ampIntegralMatrix, pwaLikelihood  # noqa: F401
from .multibin import pwaMultibin  # noqa: F401
from .warmstart import pwaMLP  # noqa: F401
from .ampfile import ampFileInfo, readAmplitudeFile, writeAmplitudeFile  # noqa: F401
from . import autotune  # noqa: F401
