"""wavetorch_gb300: the time-stepping path of fancompute/wavetorch on GB300.

Drop-in modules with the reference's names and constructor signatures; the
time loop, its adjoint and the rho -> c map run as hand-written sm_103a CUDA
kernels behind the C ABI in ``include/wavetorch_gb300.h``.
"""
from . import cell, geom, probe, rnn, source, utils, io, functional, losses, ragged  # noqa: F401
from .cell import WaveCell, TimeStep
from .geom import WaveGeometry, WaveGeometryHoley, WaveGeometryFreeForm
from .probe import WaveProbe, WaveIntensityProbe
from .rnn import WaveRNN
from .source import WaveSource, WaveLineSource
from .functional import WaveStepFn, WaveSeqFn, RhoToCFn
from ._lib import WaveKernelError

__all__ = ["WaveCell", "WaveGeometryHoley", "WaveGeometryFreeForm", "WaveProbe",
           "WaveIntensityProbe", "WaveRNN", "WaveSource", "WaveLineSource", "TimeStep",
           "WaveStepFn", "WaveSeqFn", "RhoToCFn", "WaveKernelError"]

__version__ = "0.1.0"
