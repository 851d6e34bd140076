"""Monte-Carlo driver (simulations/simulation.py:7-152).

``Simulation.iter`` keeps the reference's per-realisation semantics
(channel -> time -> measure type -> operation chain).  ``Simulation.run``
first tries the batched engine path: when every measure of every channel is
one the engine computes in its fused reductions (Beam moments, mean_x2_r,
eta through fixed or centroid-tracked CirclePupils, total eta, and the same
quantities after every screen for "propagation" measures such as SIResult
and BeamPropagationResult), it runs ``gpu.config['batch']`` realisations per
engine call, once per time shift of the wind measures, and appends their
scalars; otherwise it falls back to ``iter`` (engine propagation, one
realisation at a time).  Spectra are drawn from numpy's global RNG in the
same order as the reference (realisation by realisation, channel by
channel, screen by screen), so a seeded run reproduces the reference's
realisations.
"""
from __future__ import annotations

from typing import Sequence

from .. import gpu
from .measure import Measure
from .result import Result


class Simulation:
    def __init__(self, results_list: Sequence[Result] = None, measures_list: Sequence[Measure] = None):
        self.measures = {}
        if measures_list:
            for measures in measures_list:
                self.add_measures(measures)
        self.results_list = results_list or []
        for result in self.results_list:
            for measures in result.measures:
                self.add_measures(measures)

    def add_measures(self, measures):
        """channel - time - measure_type - operations"""
        d = self.measures.setdefault(measures.channel, {})
        d = d.setdefault(measures.time, {})
        d = d.setdefault(measures.measure_type, {})
        d.setdefault(measures.operations, []).append(measures)

    def init_measures_iteration_data(self):
        for measures in self.flattened_measures():
            empty = None
            if measures.time:
                if measures.measure_type == "propagation":
                    empty = [[None for _ in range(len(measures.channel.path.positions) + 1)] for _ in measures.time]
                else:
                    empty = [None for _ in measures.time]
            elif measures.measure_type == "propagation":
                empty = [None for _ in range(len(measures.channel.path.positions) + 1)]
            measures.iteration_data = empty

    def process_operations(self, output, operations_measures, time_id, propagation_id=None):
        for operations, measures_list in operations_measures.items():
            if self.is_measures_done(measures_list):
                continue
            measures = measures_list[0]
            out = output.clone() if hasattr(output, "clone") else output.copy()
            for operation in operations:
                out = operation(measures.channel, output=out)
            for measures in measures_list:
                if measures.is_done:
                    continue
                if measures.time is not None:
                    if propagation_id is not None:
                        measures.iteration_data[time_id][propagation_id] = out
                    else:
                        measures.iteration_data[time_id] = out
                else:
                    if propagation_id is not None:
                        measures.iteration_data[propagation_id] = out
                    else:
                        measures.iteration_data = out

    def iter(self):
        self.init_measures_iteration_data()
        for channel, channel_measures in self.measures.items():
            for ps in channel.path.phase_screens:
                ps.cache_clear()
            for time, time_measures in channel_measures.items():
                time = time or [None]
                for time_id, time_value in enumerate(time):
                    for propagation_id, (propagation_result, phase_screen) in enumerate(
                            channel.generator(pupil=False, shift=(0, time_value or 0), store_output=True, wind=True)):
                        self.process_operations(propagation_result, time_measures.get("propagation", {}), time_id,
                                                propagation_id)
                        if propagation_id == 0:
                            self.process_operations(phase_screen, time_measures.get("phase_screen", {}), time_id)
                    self.process_operations(channel.output, time_measures.get("atmosphere", {}), time_id)
                    self.process_operations(channel.output, time_measures.get("propagation", {}), time_id, -1)
                    if channel.pupil:
                        self.process_operations(channel.pupil.output(channel.output), time_measures.get("pupil", {}),
                                                time_id)
        for measures in self.flattened_measures():
            if not measures.is_done:
                measures.data.append(measures.iteration_data)

    def flattened_measures(self, measures=None):
        measures = measures if measures is not None else self.measures
        if isinstance(measures, dict):
            for values in measures.values():
                yield from self.flattened_measures(values)
        else:
            yield from measures

    def is_measures_done(self, measures=None):
        return all(m.is_done for m in self.flattened_measures(measures))

    # ------------------------------------------------------------------
    # batched engine path
    # ------------------------------------------------------------------
    def _batch_plan(self):
        """Per channel: [(measure, fused kind, time tuple or None)], or None if
        some measure is outside what the engine fuses."""
        from .fused import classify
        plans = {}
        for channel, by_time in self.measures.items():
            if not getattr(channel, "_fused_ok", lambda: False)():
                return None
            entries = []
            for time, by_type in by_time.items():
                for mtype, by_ops in by_type.items():
                    for ops, ms in by_ops.items():
                        kind = classify(channel, mtype, ops)
                        if kind is None:
                            return None
                        entries += [(m, kind, time) for m in ms]
            plans[channel] = entries
        return plans

    def _batched_iter(self, plans):
        import numpy as np
        from ..engine.runner import draw_channel_spectra, get_plan, to_device
        from .fused import resolve
        batch = int(gpu.config.get("batch", 256))
        live = [m for ms in plans.values() for m, _, _ in ms if not m.is_done]
        sized = [m.max_size - len(m) for m in live if m.max_size is not None]
        R = max(1, min(batch, max(sized) if sized else batch))
        chans = list(plans)
        for c in chans:
            c.path.init_phase_screens()
        # reference RNG order: realisation, then channel, then screen; one
        # spectrum per realisation serves every time shift (wind cache)
        per = {c: [] for c in chans}
        for _ in range(R):
            for c in chans:
                per[c].append(draw_channel_spectra(c, 1, wind=True, clear=True))
        for c, entries in plans.items():
            spectra = [np.concatenate([p[k] for p in per[c]]) for k in range(3)]
            pupils = sorted({k[1] for _, k, _ in entries if k[0] == "pupil"})
            tracked = sorted({k[1][0] for _, k, _ in entries if k[0] == "tracked"})
            steps = any(k[0].startswith("step") for _, k, _ in entries)
            plan = get_plan(c, batch=batch, pupils=pupils, tracked=tracked, path_output_loss=False,
                            step_measures=steps)
            dev = to_device(*spectra)
            # screens move by (0, t) for each time value (Simulation.iter's shift=(0, time))
            shifts = sorted({float(t or 0) for _, _, T in entries for t in (T or (0,))})
            outs, sfs = {}, {}
            want_sf = any(k[0] == "screen_sf" for _, k, _ in entries)
            try:
                for t in shifts:
                    plan.set_shift((0.0, t))
                    outs[t] = plan.run(*dev).cpu().numpy()
                    if want_sf:
                        import torch
                        from ..engine.plan import structure_function
                        phi = torch.empty((R, plan.N, plan.N), dtype=torch.float32, device=plan.device)
                        plan.screen(*dev, 0, phi_out=phi)
                        sfs[t] = structure_function(phi).cpu().numpy()
            finally:
                plan.set_shift((0.0, 0.0))
            n = plan.n_screens
            def values(kind, t):
                if kind[0] == "screen_sf":
                    return sfs[t]
                return resolve(kind, outs[t], pupils, tracked, n)

            for m, kind, T in entries:
                if T is None:
                    vals = values(kind, 0.0)
                    rows = [vals[r] for r in range(R)]
                else:
                    vs = [values(kind, float(t or 0)) for t in T]
                    rows = [[v[r] for v in vs] for r in range(R)]
                for r in range(R):
                    if m.is_done:
                        break
                    val = np.asarray(rows[r], dtype=float).tolist()
                    m.data.append(val)
                    m.iteration_data = val
        return R

    def run(self, *args, plot_step: int = None, save_step: int = None, **kwargs):
        try:
            iteration = 0
            plans = self._batch_plan()
            while not self.is_measures_done():
                if plans is not None:
                    n = self._batched_iter(plans)
                else:
                    self.iter()
                    n = 1
                for it in range(iteration + 1, iteration + n + 1):
                    self.process_output(it, plot_step=plot_step, save_step=save_step)
                iteration += n
        except KeyboardInterrupt:
            pass
        finally:
            self.process_output(0, plot_step=plot_step, save_step=save_step)

    def process_output(self, iteration, plot_step, save_step):
        if plot_step and iteration % plot_step == 0:
            for result in self.results_list:
                result.plot_output()
            try:
                from IPython import display
                display.clear_output(wait=True)
            except ModuleNotFoundError:
                pass
        if save_step and iteration % save_step == 0:
            for result in self.results_list:
                result.save_output()
