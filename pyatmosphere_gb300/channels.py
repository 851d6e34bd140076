"""Channel (the reference's channels.py:17-80) on the GB300 engine.

``Channel.run`` drives the fused engine (``atm_run``): the source, every
vacuum step and every screen of one realisation in one call; the returned
field is a complex64 torch tensor [N, N] on the engine device.
"""
from __future__ import annotations

import numpy as np

from . import gpu
from .grids import RandLogPolarGrid, RectGrid
from .measures import I
from .pathes import IdenticalPhaseScreensPath, PhaseScreensPath, VacuumPath
from .phase_screens import SSPhaseScreen
from .pupils import CirclePupil
from .sources import GaussianSource, PlaneSource
from .theory.atmosphere import get_rytov2
from .theory.models import MVKModel
from .utils import CrossRef

__all__ = ["Channel", "QuickChannel"]


class Channel:
    grid = CrossRef("channel")
    source = CrossRef("channel")
    path = CrossRef("channel")
    pupil = CrossRef("channel")

    def __init__(self, grid, source, path, pupil=None, name=""):
        self.grid = grid
        self.source = source
        self.path = path
        self.pupil = pupil
        self.output = None
        self.name = name

    # ------------------------------------------------------------------
    def _fused_ok(self):
        return (type(self.source) in (GaussianSource, PlaneSource)
                and (isinstance(self.path, VacuumPath) or
                     (isinstance(self.path, PhaseScreensPath) and
                      all(type(s) is SSPhaseScreen for s in self.path.phase_screens))))

    def _run_fused(self, shift=(0, 0), wind=False, length=None, path_output_loss=True):
        import torch
        from .engine.runner import draw_channel_spectra, get_plan, to_device
        plan = get_plan(self, batch=1, shift=shift, path_output_loss=path_output_loss, length=length)
        field = torch.empty((1, plan.N, plan.N), dtype=torch.complex64, device=plan.device)
        if plan.n_screens:
            self.path.init_phase_screens()
            spectra = draw_channel_spectra(self, 1, wind=wind, clear=False)
            plan.run(*to_device(*spectra), field_out=field)
        else:
            plan.run(None, None, None, field_out=field)
        return field[0]

    def run(self, pupil=True, *args, **kwargs):
        if self._fused_ok() and not args and set(kwargs) <= {"shift", "wind", "length"}:
            if "length" in kwargs and not isinstance(self.path, VacuumPath):
                raise TypeError("length= applies to VacuumPath channels only")
            out = self._run_fused(shift=kwargs.get("shift", (0, 0)), wind=kwargs.get("wind", False),
                                  length=kwargs.get("length"))
        else:
            out = self.path.output(self.source.output(), *args, **kwargs)
        if pupil:
            return self.pupil.output(out)
        return out

    def generator(self, pupil=True, store_output=True, *args, **kwargs):
        self.output = None
        if store_output:
            path_output = yield from self.path.generator(self.source.output(), *args, **kwargs)
            self.output = self.pupil.output(path_output) if pupil else path_output
        else:
            yield from self.path.generator(self.source.output(), *args, **kwargs)

    def get_rythov2(self):
        return get_rytov2(self.path.phase_screen.model.Cn2, self.source.k, self.path.length)

    def plot(self, *args, **kwargs):
        try:
            from matplotlib import pyplot as plt
        except ImportError as e:  # plotting is outside the engine
            raise RuntimeError("Channel.plot needs matplotlib") from e
        plt.imshow(gpu.get_array(I(self, *args, **kwargs)), extent=self.grid.extent)


def QuickChannel(Cn2=1e-15, length=1e3, count_ps=5, beam_w0=0.09, beam_wvl=808e-9, aperture_radius=0.02,
                 grid_resolution=1024, grid_delta=0.001):
    return Channel(
        grid=RectGrid(resolution=grid_resolution, delta=grid_delta),
        source=GaussianSource(wvl=beam_wvl, w0=beam_w0, F0=np.inf),
        path=IdenticalPhaseScreensPath(
            phase_screen=SSPhaseScreen(
                model=MVKModel(Cn2=Cn2, l0=3e-3, L0=1e3),
                f_grid=RandLogPolarGrid(points=2 ** 10, f_min=1 / 1e3 / 15, f_max=1 / 3e-3 * 2)),
            length=length, count=count_ps),
        pupil=CirclePupil(radius=aperture_radius))
