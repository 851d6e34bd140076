"""Analytic PDT models (the reference's theory/pdt package)."""
from .pdt import *  # noqa: F401,F403
from .elliptic_beam import EllipticBeamAnalyticalPDT  # noqa: F401
