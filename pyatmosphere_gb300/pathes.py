"""Propagation paths (the reference's pathes.py:10-95) on the GB300 engine.

``Channel.run`` sends whole channels to the fused engine (``atm_run``).  The
path objects themselves also work step by step on any input field
(``output`` / ``generator``): each vacuum step is ``atm_vacuum`` and each
screen's phasor comes from ``atm_screen``.
"""
from __future__ import annotations

import copy
from abc import ABC, abstractmethod

import numpy as np

from . import gpu

__all__ = ["AbstractPath", "VacuumPath", "PhaseScreensPath", "IdenticalPhaseScreensPath"]


def _vacuum_plan(channel):
    from .engine.plan import EnginePlan
    N, delta = channel.grid.N, float(channel.grid.delta)
    key = ("vacuum", N, delta, float(channel.source.wvl), str(gpu.device()))
    cache = channel.__dict__.setdefault("_atm_plans", {})
    if key not in cache:
        cache[key] = EnginePlan(N, delta, float(channel.source.wvl), 1.0, float("inf"), [], 1.0, batch=1,
                                device=gpu.device())
    return cache[key]


def _as_field(channel, input):
    import torch
    N = channel.grid.N
    if not isinstance(input, torch.Tensor):
        input = torch.as_tensor(np.broadcast_to(np.asarray(input), (N, N)).copy())
    if input.dim() == 0 or input.shape != (N, N):
        input = input.expand(N, N)
    return input.to(gpu.device(), torch.complex64).contiguous().clone()


class AbstractPath(ABC):
    def __init__(self, length, losses_db=0):
        self.length = length
        self.losses_db = losses_db

    @abstractmethod
    def lossless_output(self, input, *args, **kwargs):
        pass

    def append_losses(self, input, losses_db=None):
        losses_db = losses_db or self.losses_db
        return input * 10 ** (-losses_db / 20) if losses_db else input

    def output(self, input, *args, **kwargs):
        return self.append_losses(self.lossless_output(input, *args, **kwargs))


class VacuumPath(AbstractPath):
    def lossless_output(self, input, length=None):
        length = length if length is not None else self.length
        if length > 0:
            field = _as_field(self.channel, input)
            return _vacuum_plan(self.channel).vacuum(field, float(length))
        return input


class PhaseScreensPath(AbstractPath):
    def __init__(self, length, phase_screens, positions, losses_db=0):
        self.positions = positions
        self.phase_screens = phase_screens
        super().__init__(length, losses_db)

    def init_phase_screens(self):
        for phase_screen in self.phase_screens:
            phase_screen.channel = self.channel

    def lossless_output(self, input, *args, **kwargs):
        generator = self.generator(input, *args, **kwargs)
        try:
            while True:
                next(generator)
        except StopIteration as e:
            return e.value

    def generator(self, input, *args, **kwargs):
        vacuum_path = VacuumPath(length=None)
        vacuum_path.channel = self.channel
        self.init_phase_screens()
        for i, phase_screen in enumerate(self.phase_screens):
            vacuum_path.length = self.positions[i] - self.positions[i - 1] if i > 0 else self.positions[0]
            import torch
            if hasattr(phase_screen, "generate_with_phasor"):
                screen, phasor = phase_screen.generate_with_phasor(*args, **kwargs)
            else:
                screen = phase_screen.generate(*args, **kwargs)
                phasor = torch.polar(torch.ones_like(screen), -screen)  # exp(-i phi), complex64
            part_losses_db = self.losses_db * vacuum_path.length / self.length
            field = _as_field(self.channel, vacuum_path.output(input))
            input = self.append_losses(phasor * field, losses_db=part_losses_db)
            yield input, screen
        return vacuum_path.output(input, length=self.length - self.positions[-1])


class IdenticalPhaseScreensPath(PhaseScreensPath):
    def __init__(self, length, count, phase_screen, position_in_slab="middle", losses_db=0):
        thickness = length / count
        if position_in_slab == "before":
            positions = np.arange(count) * thickness
        elif position_in_slab == "middle":
            positions = (np.arange(count) + 1 / 2) * thickness
        elif position_in_slab == "after":
            positions = (np.arange(count) + 1) * thickness
        else:
            raise ValueError("Available values for position_in_slab: 'before', 'middle' and 'after'")
        phase_screen.thickness = thickness
        phase_screens = [copy.copy(phase_screen) for _ in range(count)]
        self.phase_screen = phase_screens[0]
        super().__init__(length=length, phase_screens=phase_screens, positions=positions, losses_db=losses_db)
