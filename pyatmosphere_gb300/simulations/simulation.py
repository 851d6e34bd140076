"""Monte-Carlo driver on the GB300 engine (the reference's
simulations/simulation.py:7-152 offers the same class and methods).

Measures are grouped by (channel, time list, measure type, operation
chain); a group's chain runs once per value it is offered and its result
goes to every measure of the group.  Per realisation, a channel offers, in
this order and once per time value t of the group (screens shifted by
(0, t), one spectrum draw serving every t):

    "propagation" i   the field just after screen i   (and "phase_screen":
                      the first screen, when i = 0)
    "atmosphere"      the receiver field
    "propagation" -1  the receiver field
    "pupil"           the receiver field behind the channel's pupil

Groups see the values in the order they were added, so a chain that reads
another measure's value of this realisation (BeamResult.mean_x2_r,
TrackedPDTResult.set_pupil_position) finds it.

``run`` first tries the batched engine path: when every measure is one the
engine's fused reductions produce (beam moments, mean_x2_r, eta through fixed
or centroid-tracked circular pupils, total eta, the per-screen values of
"propagation" measures, the first screen's structure function), it runs
``gpu.config['batch']`` realisations per engine call, once per time value,
with spectra drawn from numpy's global generator in the per-realisation
order (realisation, channel, screen).  Otherwise it runs ``iter`` (engine
propagation, one realisation at a time).  Either way a seeded run gives the
reference's realisations.
"""
from __future__ import annotations

from typing import Sequence

from .. import gpu
from .measure import Measure
from .result import Result


def _blank(measure):
    """Empty per-realisation value of a measure: one slot per time value and,
    for "propagation" measures, one per screen plus the receiver."""
    steps = len(measure.channel.path.positions) + 1 if measure.measure_type == "propagation" else None

    def one():
        return [None] * steps if steps else None

    return [one() for _ in measure.time] if measure.time else one()


def _store(measure, value, time_id, step):
    if measure.time is None and step is None:
        measure.iteration_data = value
        return
    slot = measure.iteration_data
    if measure.time is not None:
        if step is None:
            slot[time_id] = value
            return
        slot = slot[time_id]
    slot[step] = value


def _copy(value):
    return value.clone() if hasattr(value, "clone") else value.copy() if hasattr(value, "copy") else value


class Simulation:
    def __init__(self, results_list: Sequence[Result] = None, measures_list: Sequence[Measure] = None):
        self._groups: dict = {}  # (channel, time, measure_type, operations) -> [Measure]
        for m in measures_list or ():
            self.add_measures(m)
        self.results_list = list(results_list or ())
        for result in self.results_list:
            for m in result.measures:
                self.add_measures(m)

    def add_measures(self, measures):
        key = (measures.channel, measures.time, measures.measure_type, measures.operations)
        self._groups.setdefault(key, []).append(measures)

    @property
    def measures(self):
        """The groups as nested dicts: channel -> time -> measure type -> operations -> [Measure]."""
        tree = {}
        for (channel, time, mtype, ops), ms in self._groups.items():
            tree.setdefault(channel, {}).setdefault(time, {}).setdefault(mtype, {})[ops] = ms
        return tree

    def flattened_measures(self, measures=None):
        if measures is None:
            for ms in self._groups.values():
                yield from ms
        elif isinstance(measures, dict):
            for v in measures.values():
                yield from self.flattened_measures(v)
        else:
            yield from measures

    def is_measures_done(self, measures=None):
        return all(m.is_done for m in self.flattened_measures(measures))

    # ------------------------------------------------------------------
    # one realisation at a time
    # ------------------------------------------------------------------
    @staticmethod
    def _offers(channel, time_value):
        """(measure type, step, value) in the order one realisation offers them."""
        walk = channel.generator(pupil=False, shift=(0, time_value or 0), store_output=True, wind=True)
        for i, (field, screen) in enumerate(walk):
            yield "propagation", i, field
            if i == 0:
                yield "phase_screen", None, screen
        yield "atmosphere", None, channel.output
        yield "propagation", -1, channel.output
        if channel.pupil:
            yield "pupil", None, channel.pupil.output(channel.output)

    def process_operations(self, output, operations_measures, time_id, propagation_id=None):
        """Runs each group's chain on `output` and stores the result in its
        measures (operations_measures: {operations: [Measure]})."""
        for ops, group in operations_measures.items():
            if self.is_measures_done(group):
                continue
            value = _copy(output)
            for op in ops:
                value = op(group[0].channel, output=value)
            for m in group:
                if not m.is_done:
                    _store(m, value, time_id, propagation_id)

    def iter(self):
        for m in self.flattened_measures():
            m.iteration_data = _blank(m)
        channels = list(dict.fromkeys(key[0] for key in self._groups))
        for channel in channels:
            for screen in getattr(channel.path, "phase_screens", ()):
                screen.cache_clear()  # a new spectrum per realisation
            times = list(dict.fromkeys(key[1] for key in self._groups if key[0] is channel))
            for time in times:
                by_type = {}
                for (c, t, mtype, ops), group in self._groups.items():
                    if c is channel and t == time:
                        by_type.setdefault(mtype, {})[ops] = group
                for time_id, t in enumerate(time or [None]):
                    for mtype, step, value in self._offers(channel, t):
                        if mtype in by_type:
                            self.process_operations(value, by_type[mtype], time_id, step)
        for m in self.flattened_measures():
            if not m.is_done:
                m.data.append(m.iteration_data)

    # ------------------------------------------------------------------
    # batched engine path
    # ------------------------------------------------------------------
    def _batch_plan(self):
        """Per channel: [(measure, fused kind, time tuple or None)], or None if
        some measure is outside what the engine fuses."""
        from ..engine.runner import screen_kind
        from .fused import classify
        plans = {}
        for (channel, time, mtype, ops), group in self._groups.items():
            if not getattr(channel, "_fused_ok", lambda: False)():
                return None
            if screen_kind(channel.path) == "fft" and (time is not None or mtype == "phase_screen"):
                return None  # FFT screens do not move with time; the screen measures use atm_screen
            kind = classify(channel, mtype, ops)
            if kind is None:
                return None
            plans.setdefault(channel, []).extend((m, kind, time) for m in group)
        return plans

    def _batched_iter(self, plans):
        from .fused import run_batched
        return run_batched(plans, int(gpu.config.get("batch", 256)))

    # ------------------------------------------------------------------
    def run(self, *args, plot_step: int = None, save_step: int = None, **kwargs):
        """Realisations until every measure has max_size values; an interrupt
        (Ctrl-C) stops early, keeping what was measured, and the final
        process_output saves it."""
        done = 0
        try:
            batched = self._batch_plan()
            while not self.is_measures_done():
                if batched is not None:
                    n = self._batched_iter(batched)
                else:
                    self.iter()
                    n = 1
                for it in range(done + 1, done + n + 1):
                    self.process_output(it, plot_step=plot_step, save_step=save_step)
                done += n
        except KeyboardInterrupt:
            pass
        finally:
            self.process_output(0, plot_step=plot_step, save_step=save_step)

    def process_output(self, iteration, plot_step, save_step):
        """Plots every plot_step-th and saves every save_step-th iteration
        (iteration 0: the end of the run)."""
        if plot_step and not iteration % plot_step:
            for result in self.results_list:
                result.plot_output()
            try:
                from IPython.display import clear_output
            except ImportError:
                clear_output = None
            if clear_output is not None:
                clear_output(wait=True)
        if save_step and not iteration % save_step:
            for result in self.results_list:
                result.save_output()
