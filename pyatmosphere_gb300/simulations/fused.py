"""Which measure chains the engine's fused reduction can serve, and where
each one's value sits in ``atm_run``'s per-realisation output."""
from __future__ import annotations

from .. import measures as M
from ..engine import _lib

_MOMENT = {M.mean_x: _lib.OUT_MEAN_X, M.mean_y: _lib.OUT_MEAN_Y, M.mean_x2: _lib.OUT_MEAN_X2,
           M.mean_xy: _lib.OUT_MEAN_XY, M.mean_y2: _lib.OUT_MEAN_Y2}


def classify(channel, mtype, ops):
    """Returns a key describing the value, or None if not fusable."""
    from .beam import BeamResult
    from .pdt import PDTResult, PupilStop, TrackedPDTResult
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
        if len(ops) == 2 and ops[1] is M.eta and isinstance(ops[0], PupilStop):
            owner = ops[0].result
            if isinstance(owner, PDTResult) and not isinstance(owner, TrackedPDTResult):
                sx, sy = owner.pupil_shift
                return ("pupil", (float(ops[0].pupil.radius), float(sx), float(sy)))
            return None
        if len(ops) == 3 and ops[2] is M.eta and isinstance(ops[1], PupilStop):
            owner = getattr(ops[0], "__self__", None)
            if isinstance(owner, TrackedPDTResult) and owner is ops[1].result and \
                    getattr(ops[0], "__func__", None) is TrackedPDTResult.set_pupil_position:
                return ("tracked", (float(ops[1].pupil.radius),))
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


def run_batched(plans, batch: int) -> int:
    """One batch of realisations of every channel through the fused engine.

    plans: {channel: [(measure, kind from classify, time tuple or None)]}.
    Spectra are drawn realisation by realisation, channel by channel, screen
    by screen (the per-realisation loop's order); one draw serves every time
    value of a realisation (the wind cache), and the screens move by (0, t)
    for time value t.  Appends each measure's values and returns the number
    of realisations run."""
    import numpy as np
    from ..engine.runner import draw_channel_fft, draw_channel_spectra, get_plan, screen_kind, to_device
    live = [m for ms in plans.values() for m, _, _ in ms if not m.is_done]
    wanted = [m.max_size - len(m) for m in live if m.max_size is not None]
    R = max(1, min(batch, max(wanted) if wanted else batch))
    chans = list(plans)
    for c in chans:
        c.path.init_phase_screens()
    draws = {c: [] for c in chans}
    fft = {c: screen_kind(c.path) == "fft" for c in chans}
    for _ in range(R):
        for c in chans:
            draws[c].append(draw_channel_fft(c, 1) if fft[c] else draw_channel_spectra(c, 1, wind=True, clear=True))
    for c, entries in plans.items():
        if fft[c]:
            # normals, sub_x, sub_y, sub_mean per realisation; the amplitude grids and n_sub are shared
            cat = {k: np.concatenate([d[k] for d in draws[c]]) for k in (0, 2, 3, 4)}
            spectra = (cat[0], draws[c][0][1], cat[2], cat[3], cat[4])
            n_sub = draws[c][0][5]
        else:
            spectra = [np.concatenate([d[k] for d in draws[c]]) for k in range(3)]
        pupils = sorted({k[1] for _, k, _ in entries if k[0] == "pupil"})
        tracked = sorted({k[1][0] for _, k, _ in entries if k[0] == "tracked"})
        steps = any(k[0].startswith("step") for _, k, _ in entries)
        plan = get_plan(c, batch=batch, pupils=pupils, tracked=tracked, path_output_loss=False,
                        step_measures=steps)
        dev = to_device(*spectra)
        shifts = sorted({float(t or 0) for _, _, T in entries for t in (T or (0,))})
        want_sf = any(k[0] == "screen_sf" for _, k, _ in entries)
        outs, sfs = {}, {}
        try:
            for t in shifts:
                if fft[c]:
                    outs[t] = plan.run_fft(*dev, n_sub).cpu().numpy()  # one time value (no shift)
                    continue
                plan.set_shift((0.0, t))
                outs[t] = plan.run(*dev).cpu().numpy()
                if want_sf:
                    import torch
                    from ..engine.plan import structure_function
                    phi = torch.empty((R, plan.N, plan.N), dtype=torch.float32, device=plan.device)
                    plan.screen(*dev, 0, phi_out=phi)
                    sfs[t] = structure_function(phi).cpu().numpy()
            plan.check()
        finally:
            plan.set_shift((0.0, 0.0))

        def values(kind, t):
            return sfs[t] if kind[0] == "screen_sf" else resolve(kind, outs[t], pupils, tracked, plan.n_screens)

        for m, kind, T in entries:
            per_t = [values(kind, float(t or 0)) for t in (T or (0,))]
            for r in range(R):
                if m.is_done:
                    break
                row = per_t[0][r] if T is None else [v[r] for v in per_t]
                val = np.asarray(row, dtype=float).tolist()
                m.data.append(val)
                m.iteration_data = val
    return R
