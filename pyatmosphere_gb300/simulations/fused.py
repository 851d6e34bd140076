"""Which measure chains the engine's fused reduction can serve, and where
each one's value sits in ``atm_run``'s per-realisation output."""
from __future__ import annotations

import functools

from .. import measures as M
from ..engine import _lib

_MOMENT = {M.mean_x: _lib.OUT_MEAN_X, M.mean_y: _lib.OUT_MEAN_Y, M.mean_x2: _lib.OUT_MEAN_X2,
           M.mean_xy: _lib.OUT_MEAN_XY, M.mean_y2: _lib.OUT_MEAN_Y2}


def classify(channel, mtype, ops):
    """Returns a key describing the value, or None if not fusable."""
    from .beam import BeamResult
    from .pdt import PDTResult, TrackedPDTResult
    if mtype == "atmosphere":
        if len(ops) == 1:
            op = ops[0]
            if op in _MOMENT:
                return ("slot", _MOMENT[op])
            if op is M.eta:
                return ("slot", _lib.OUT_ETA_TOTAL)
            if op is M.mean_r:
                return ("mean_r",)
            if op is M.mean_r2:
                return ("mean_r2",)
            if getattr(op, "__func__", None) is BeamResult.mean_x2_r:
                return ("slot", _lib.OUT_MEAN_X2_R)
            return None
        if len(ops) == 2 and ops[1] is M.eta and isinstance(ops[0], functools.partial):
            owner = getattr(ops[0].func, "__self__", None)
            if isinstance(owner, PDTResult) and getattr(ops[0].func, "__func__", None) is PDTResult.append_pupil \
                    and not isinstance(owner, TrackedPDTResult):
                sx, sy = owner.pupil_shift
                return ("pupil", (float(ops[0].args[0].radius), float(sx), float(sy)))
            return None
        if len(ops) == 3 and ops[2] is M.eta and isinstance(ops[1], functools.partial):
            owner = getattr(ops[0], "__self__", None)
            if isinstance(owner, TrackedPDTResult) and \
                    getattr(ops[0], "__func__", None) is TrackedPDTResult.set_pupil_position:
                return ("tracked", (float(ops[1].args[0].radius),))
        return None
    if mtype == "pupil" and len(ops) == 1 and ops[0] is M.eta and channel.pupil is not None:
        return ("pupil", (float(channel.pupil.radius), 0.0, 0.0))
    if mtype == "phase_screen" and len(ops) == 1 and len(getattr(channel.path, "phase_screens", ())) > 0:
        from .structure_function import calculate_structure_function
        if ops[0] is calculate_structure_function:
            return ("screen_sf",)  # of the first screen, from atm_screen + atm_structure_function
        return None
    if mtype == "propagation" and len(ops) == 1 and len(getattr(channel.path, "phase_screens", ())) > 0:
        # after every screen and at the receiver (the engine's per-step measures)
        from .si import intensity_at_center
        op = ops[0]
        if op is intensity_at_center:
            return ("step", _lib.OUT_I_CENTER)
        if op in _MOMENT:
            return ("step", _MOMENT[op])
        if op is M.eta:
            return ("step", _lib.OUT_ETA_TOTAL)
        if op is M.mean_r:
            return ("step_mean_r",)
        if op is M.mean_r2:
            return ("step_mean_r2",)
    return None


def _steps(out, base, n, slots):
    """[R][n + 1] values of the given slots: after each screen, then at the receiver."""
    import numpy as np
    cols = [out[:, [base + i * _lib.STEP_SLOTS + s for s in slots]] for i in range(n)] + [out[:, slots]]
    return np.stack(cols, axis=1)


def resolve(kind, out, pupils, tracked, n_screens=0):
    """Per-realisation values of one measure: [R] (or [R][n + 1] for the
    per-step kinds) from atm_run's output rows."""
    base = _lib.OUT_PUPIL0 + len(pupils) + len(tracked)
    if kind[0] == "step":
        return _steps(out, base, n_screens, [kind[1]])[:, :, 0]
    if kind[0] == "step_mean_r":
        v = _steps(out, base, n_screens, [_lib.OUT_MEAN_X, _lib.OUT_MEAN_Y])
        return (v[:, :, 0] ** 2 + v[:, :, 1] ** 2) ** 0.5
    if kind[0] == "step_mean_r2":
        v = _steps(out, base, n_screens, [_lib.OUT_MEAN_X2, _lib.OUT_MEAN_Y2])
        return v[:, :, 0] + v[:, :, 1]
    if kind[0] == "slot":
        return out[:, kind[1]]
    if kind[0] == "mean_r":
        return (out[:, _lib.OUT_MEAN_X] ** 2 + out[:, _lib.OUT_MEAN_Y] ** 2) ** 0.5
    if kind[0] == "mean_r2":
        return out[:, _lib.OUT_MEAN_X2] + out[:, _lib.OUT_MEAN_Y2]
    if kind[0] == "pupil":
        return out[:, _lib.OUT_PUPIL0 + pupils.index(kind[1])]
    if kind[0] == "tracked":
        return out[:, _lib.OUT_PUPIL0 + len(pupils) + tracked.index(kind[1][0])]
    raise KeyError(kind)
