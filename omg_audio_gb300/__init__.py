"""GB300-native stochastic energy path tracer for omg-audio's late field and
ambient dome. The compute runs in libomg_cuda.so (hand-written sm_103a CUDA
behind the C ABI in include/omg_cuda.h); this package is its Python face.
"""
from . import _lib
from ._lib import OmgError
from .engine import Batch, Context, DomeProbe, Job, MeshBuilder, Scene, TraceConfig
from .materials import Material
from .tracer import Echogram, ReverbParams

__all__ = ["Batch", "Context", "DomeProbe", "Echogram", "Job", "Material", "MeshBuilder", "OmgError",
           "ReverbParams", "Scene", "TraceConfig"]
