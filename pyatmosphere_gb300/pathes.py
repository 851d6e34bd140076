"""Propagation paths on the GB300 engine (the reference's pathes.py:10-95
offers the same classes).

A path of length L with screens at z_0 < ... < z_{n-1} is the chain of
segments

    vacuum z_0, screen 0, vacuum z_1 - z_0, screen 1, ..., vacuum L - z_{n-1}

where a screen multiplies the field by exp(-i phi) and by the attenuation of
the path's share of its losses over the vacuum step before it.  Whole
channels of Gaussian / plane sources and sparse-spectrum screens go to the
fused engine (``Channel.run`` -> ``atm_run``); these classes also run the
chain segment by segment on any field: a vacuum segment is ``atm_vacuum``
and each screen's phasor comes from ``atm_screen``.
"""
from __future__ import annotations

import copy
from abc import ABC, abstractmethod

import numpy as np

from . import gpu

__all__ = ["AbstractPath", "VacuumPath", "PhaseScreensPath", "IdenticalPhaseScreensPath"]

# where each screen of IdenticalPhaseScreensPath sits in its slab, as a
# fraction of the slab thickness
_SLAB_OFFSET = {"before": 0.0, "middle": 0.5, "after": 1.0}


def attenuate(field, losses_db):
    """The field after a loss of `losses_db` decibels (unchanged at 0)."""
    if not losses_db:
        return field
    return field * 10 ** (-losses_db / 20)


def _vacuum_plan(channel):
    """A plan (cached on the channel) that only runs atm_vacuum steps."""
    from .engine.plan import EnginePlan
    N, delta, wvl = channel.grid.N, float(channel.grid.delta), float(channel.source.wvl)
    plans = channel.__dict__.setdefault("_atm_plans", {})
    key = ("vacuum-steps", N, delta, wvl, str(gpu.device()))
    if key not in plans:
        plans[key] = EnginePlan(N, delta, wvl, 1.0, float("inf"), [], 1.0, batch=1, device=gpu.device())
    return plans[key]


def _as_field(channel, value):
    """A fresh complex64 [N, N] engine tensor holding `value` (a field, or a
    scalar such as PlaneSource's output broadcast over the grid)."""
    import torch
    N = channel.grid.N
    t = value if isinstance(value, torch.Tensor) else torch.as_tensor(np.asarray(value))
    t = t.to(gpu.device(), torch.complex64)
    return t.expand(N, N).clone() if t.shape != (N, N) else t.clone()


def _finish(generator):
    """Exhausts a segment generator and returns its return value."""
    box = []

    def keep():
        box.append((yield from generator))

    for _ in keep():
        pass
    return box[0]


class AbstractPath(ABC):
    def __init__(self, length, losses_db=0):
        self.length = length
        self.losses_db = losses_db

    @abstractmethod
    def lossless_output(self, input, *args, **kwargs):
        """The field at the end of the path, before the path's losses."""

    def append_losses(self, input, losses_db=None):
        """A segment's own loss; a segment without one (None or 0) takes the
        whole path's."""
        return attenuate(input, losses_db if losses_db else self.losses_db)

    def output(self, input, *args, **kwargs):
        return self.append_losses(self.lossless_output(input, *args, **kwargs))


class VacuumPath(AbstractPath):
    def lossless_output(self, input, length=None):
        step = self.length if length is None else length
        if not step > 0:
            return input  # a zero-length segment leaves the field as it is
        return _vacuum_plan(self.channel).vacuum(_as_field(self.channel, input), float(step))


class PhaseScreensPath(AbstractPath):
    def __init__(self, length, phase_screens, positions, losses_db=0):
        super().__init__(length, losses_db)
        self.phase_screens = phase_screens
        self.positions = positions

    def init_phase_screens(self):
        for screen in self.phase_screens:
            screen.channel = self.channel

    def segments(self):
        """[(vacuum length before screen i, screen i)], then the length of the
        last vacuum segment."""
        z = [0.0] + [float(p) for p in self.positions]
        steps = [(z[i + 1] - z[i], screen) for i, screen in enumerate(self.phase_screens)]
        return steps, self.length - z[-1]

    def lossless_output(self, input, *args, **kwargs):
        return _finish(self.generator(input, *args, **kwargs))

    def generator(self, input, *args, **kwargs):
        """Yields (field just after screen i, screen i) for every screen and
        returns the field at the end of the path."""
        import torch
        self.init_phase_screens()
        vacuum = VacuumPath(length=None)
        vacuum.channel = self.channel
        steps, last = self.segments()
        field = input
        for dz, screen in steps:
            if hasattr(screen, "generate_with_phasor"):
                phi, phasor = screen.generate_with_phasor(*args, **kwargs)
            else:
                phi = screen.generate(*args, **kwargs)
                phasor = torch.polar(torch.ones_like(phi), -phi)
            arrived = _as_field(self.channel, vacuum.output(field, length=dz))
            field = self.append_losses(phasor * arrived, losses_db=self.losses_db * dz / self.length)
            yield field, phi
        return vacuum.output(field, length=last)


class IdenticalPhaseScreensPath(PhaseScreensPath):
    def __init__(self, length, count, phase_screen, position_in_slab="middle", losses_db=0):
        if position_in_slab not in _SLAB_OFFSET:
            raise ValueError(f"position_in_slab must be one of {', '.join(_SLAB_OFFSET)}; got {position_in_slab!r}")
        slab = length / count
        phase_screen.thickness = slab
        # one shallow copy per slab: the copies share the model and spectral grid
        screens = [copy.copy(phase_screen) for _ in range(count)]
        self.phase_screen = screens[0]
        super().__init__(length=length, phase_screens=screens,
                         positions=(np.arange(count) + _SLAB_OFFSET[position_in_slab]) * slab, losses_db=losses_db)
