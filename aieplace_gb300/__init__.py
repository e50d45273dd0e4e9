"""GB300-native ePlace global placement (a drop-in for the AIEplace placer loop).

All compute runs in libaieplace_gb300.so (hand-written sm_103a CUDA behind a
C ABI, include/aieplace.h).  Build it with aieplace_gb300.build.build().
"""
from ._lib import APError, lib  # noqa: F401
from .placer import BatchPlacer, Placer  # noqa: F401
from . import synth  # noqa: F401
from .design import Design  # noqa: F401
from .surrogate import Surrogate  # noqa: F401
