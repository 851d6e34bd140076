"""Measures (the reference's measures.py:1-38) through the engine's fused
reduction (``atm_measures``: FP64 accumulation of I, I x, -I y, I x^2,
-I x y, I y^2 over the field in one pass).  Scalars are Python floats."""
from __future__ import annotations

from . import gpu


def _moments(channel, output):
    import torch
    from .engine.plan import EnginePlan
    N = channel.grid.N
    key = ("measures", N, float(channel.grid.delta), str(gpu.device()))
    cache = channel.__dict__.setdefault("_atm_plans", {})
    if key not in cache:
        cache[key] = EnginePlan(N, float(channel.grid.delta), 1e-6, 1.0, float("inf"), [], 1.0, batch=1,
                                device=gpu.device())
    field = output.to(gpu.device(), torch.complex64).reshape(1, N, N).contiguous()
    return cache[key].measures(field)[0].cpu().numpy()


def _field(channel, output, args, kwargs):
    if output is not None:
        return output
    return channel.run(*args, **kwargs)


def I(channel, output=None, *args, **kwargs):
    if output is not None:
        return abs(output) ** 2
    return abs(channel.run(*args, **kwargs)) ** 2


def eta(channel, output=None, *args, **kwargs):
    return float(_moments(channel, _field(channel, output, args, kwargs))[0])


def mean_x(channel, output=None, *args, **kwargs):
    kwargs["pupil"] = False
    return float(_moments(channel, _field(channel, output, args, kwargs))[1])


def mean_y(channel, output=None, *args, **kwargs):
    kwargs["pupil"] = False
    return float(_moments(channel, _field(channel, output, args, kwargs))[2])


def mean_x2(channel, output=None, *args, **kwargs):
    kwargs["pupil"] = False
    return float(_moments(channel, _field(channel, output, args, kwargs))[3])


def mean_xy(channel, output=None, *args, **kwargs):
    kwargs["pupil"] = False
    return float(_moments(channel, _field(channel, output, args, kwargs))[4])


def mean_y2(channel, output=None, *args, **kwargs):
    kwargs["pupil"] = False
    return float(_moments(channel, _field(channel, output, args, kwargs))[5])


def mean_r(channel, output=None, *args, **kwargs):
    """|centroid| (commented out in the reference, measures.py:20-23; restored
    because BeamPropagationResult uses it)."""
    kwargs["pupil"] = False
    m = _moments(channel, _field(channel, output, args, kwargs))
    return float((m[1] ** 2 + m[2] ** 2) ** 0.5)


def mean_r2(channel, output=None, *args, **kwargs):
    """Sum of I r^2 delta^2 (measures.py:40-42, restored)."""
    kwargs["pupil"] = False
    m = _moments(channel, _field(channel, output, args, kwargs))
    return float(m[3] + m[5])
