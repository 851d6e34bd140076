"""PDT surrogate trained by the engine's own MLP kernels."""
from .model import Box, SimConfig, Surrogate, features, ks_binned, ks_hist, targets_from_measures  # noqa: F401
