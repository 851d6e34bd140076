"""The GB300 engine: ctypes binding of libatm.so and host-side inputs."""
from ._lib import EngineError, load  # noqa: F401
from .plan import EnginePlan  # noqa: F401
from .spectra import annulus_psd, draw_spectra  # noqa: F401
