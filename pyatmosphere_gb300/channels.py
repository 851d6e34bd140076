"""Channel: a grid, a source, a path and a pupil on the GB300 engine (the
reference's channels.py:17-80 offers the same class and factory).

A channel whose source is Gaussian or plane and whose path is a vacuum path or
a path of sparse-spectrum screens runs as one fused engine call
(``atm_run``: the source, every vacuum segment and every screen of the
realisation); any other channel runs its path segment by segment.  Fields are
complex64 torch tensors [N, N] on the engine device.
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

# keyword arguments Channel.run passes on to the fused engine call
_FUSED_KWARGS = {"shift", "wind", "length"}


class Channel:
    grid = CrossRef("channel")
    source = CrossRef("channel")
    path = CrossRef("channel")
    pupil = CrossRef("channel")

    def __init__(self, grid, source, path, pupil=None, name=""):
        self.name = name
        self.output = None
        self.grid, self.source, self.path, self.pupil = grid, source, path, pupil

    # ---- which runs the fused engine call serves --------------------------
    def _fused_ok(self):
        if type(self.source) not in (GaussianSource, PlaneSource):
            return False
        if isinstance(self.path, VacuumPath):
            return True
        from .engine.runner import screen_kind
        return isinstance(self.path, PhaseScreensPath) and (
            all(type(s) is SSPhaseScreen for s in self.path.phase_screens) or screen_kind(self.path) == "fft")

    def _run_fused(self, shift=(0, 0), wind=False, length=None, path_output_loss=True):
        import torch
        from .engine.runner import get_plan, run_single, screen_kind
        if screen_kind(self.path) == "fft" and (tuple(shift) != (0, 0) or wind):
            raise TypeError("FFT phase screens take no shift / wind")
        plan = get_plan(self, batch=1, shift=shift, path_output_loss=path_output_loss, length=length)
        field = torch.empty((1, plan.N, plan.N), dtype=torch.complex64, device=plan.device)
        run_single(self, plan, field, wind=wind)
        return field[0]

    def run(self, pupil=True, *args, **kwargs):
        """The field at the receiver of one realisation (behind the pupil
        unless pupil=False)."""
        fused = self._fused_ok() and not args and set(kwargs) <= _FUSED_KWARGS
        if fused:
            if "length" in kwargs and not isinstance(self.path, VacuumPath):
                raise TypeError("length= applies to channels with a VacuumPath only")
            field = self._run_fused(**kwargs)
        else:
            field = self.path.output(self.source.output(), *args, **kwargs)
        return self.pupil.output(field) if pupil else field

    def generator(self, pupil=True, store_output=True, *args, **kwargs):
        """Yields what the path yields after each screen; with store_output the
        receiver field (behind the pupil unless pupil=False) is left in
        self.output."""
        self.output = None
        path_output = yield from self.path.generator(self.source.output(), *args, **kwargs)
        if store_output:
            self.output = self.pupil.output(path_output) if pupil else path_output

    def get_rythov2(self):
        """Plane-wave Rytov variance of the path's turbulence."""
        return get_rytov2(self.path.phase_screen.model.Cn2, self.source.k, self.path.length)

    def plot(self, *args, **kwargs):
        try:
            from matplotlib import pyplot as plt
        except ImportError as e:  # plotting is outside the engine
            raise RuntimeError("Channel.plot needs matplotlib") from e
        plt.imshow(gpu.get_array(I(self, *args, **kwargs)), extent=self.grid.extent)


def QuickChannel(Cn2=1e-15, length=1e3, count_ps=5, beam_w0=0.09, beam_wvl=808e-9, aperture_radius=0.02,
                 grid_resolution=1024, grid_delta=0.001):
    """A ready channel: collimated Gaussian beam, `count_ps` sparse-spectrum
    screens of MVK turbulence (inner scale 3 mm, outer scale 1 km) on 1024
    log-polar annuli from 1/(15 L0) to 2/l0, and a circular aperture."""
    l0, L0 = 3e-3, 1e3
    spectrum = RandLogPolarGrid(points=2 ** 10, f_min=1 / L0 / 15, f_max=1 / l0 * 2)
    screen = SSPhaseScreen(model=MVKModel(Cn2=Cn2, l0=l0, L0=L0), f_grid=spectrum)
    return Channel(grid=RectGrid(resolution=grid_resolution, delta=grid_delta),
                   source=GaussianSource(wvl=beam_wvl, w0=beam_w0, F0=np.inf),
                   path=IdenticalPhaseScreensPath(phase_screen=screen, length=length, count=count_ps),
                   pupil=CirclePupil(radius=aperture_radius))
