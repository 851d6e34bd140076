"""Empirical phase structure function of the first screen
(simulations/structure_function.py, theory/phase_screens/sf.py)."""
from __future__ import annotations

import numpy as np

from .. import gpu
from .measure import Measure
from .result import Result


def calculate_sf(screen):
    """mean over rows of (phi[:, :-r] - phi[:, r:])^2, r = 1..N-1, per row."""
    import torch
    s = screen.to(torch.float64)
    n = s.shape[1]
    return torch.stack([((s[:, :-r] - s[:, r:]) ** 2).sum(dim=1) / (n - r) for r in range(1, n)])


def calculate_structure_function(channel, output):
    """Row mean of calculate_sf; CUDA screens go through the engine's
    atm_structure_function kernel."""
    import torch
    if isinstance(output, torch.Tensor) and output.is_cuda and output.dim() == 2 and not output.is_complex():
        from ..engine.plan import structure_function
        return structure_function(output[None])[0].cpu().numpy()
    if not isinstance(output, torch.Tensor):
        output = torch.from_numpy(np.asarray(output))
    return gpu.get_array(calculate_sf(output.real if output.is_complex() else output).mean(dim=1))


class StructureFunctionResult(Result):
    def __init__(self, channel, *args, **kwargs):
        measures = [Measure(channel, "phase_screen", calculate_structure_function)]
        super().__init__(*args, channel=channel, measures=measures, **kwargs)

    @property
    def structure_function(self):
        return np.asarray(self.measures[0]).mean(axis=0)

    @property
    def r(self):
        return np.arange(1, self.channel.grid.resolution[0]) * self.channel.grid.delta

    def theoretical(self):
        ps = self.channel.path.phase_screen
        return ps.model.sf_phi(self.r, 2 * np.pi / ps.wvl, ps.thickness)
