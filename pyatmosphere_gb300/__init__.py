"""GB300-native engine for pyAtmosphere's split-step beam-propagation Monte
Carlo, behind the reference's Python API.

    import pyatmosphere_gb300 as pyatmosphere

The classes and functions below mirror the reference package; fields are
complex64 torch tensors on the GPU and all propagation, screen synthesis and
measures run in the engine's CUDA kernels (libatm.so)."""
from pyatmosphere_gb300 import gpu
from pyatmosphere_gb300 import measures
from pyatmosphere_gb300 import simulations

from pyatmosphere_gb300.channels import Channel, QuickChannel
from pyatmosphere_gb300.grids import *
from pyatmosphere_gb300.pathes import *
from pyatmosphere_gb300.phase_screens import *
from pyatmosphere_gb300.pupils import *
from pyatmosphere_gb300.sources import *

from pyatmosphere_gb300.theory.models import *

__all__ = [
    "Channel",
    "QuickChannel",
]
