"""The GB300 engine behind the reference package's own backend switch.

    import pyatmosphere                          # the reference, unmodified
    from pyatmosphere_gb300 import reference_hook
    reference_hook.install(pyatmosphere)
    pyatmosphere.gpu.config["engine"] = "gb300"

The reference picks its array module with ``gpu.config["use_gpu"]``
(pyatmosphere/gpu.py:4-20: numpy, or cupy when True).  ``install`` adds the
``"engine"`` key to that same dict; while it is "gb300" the reference's hot
path runs in libatm and its arrays stay numpy:

    Channel.run                          (channels.py:31-35)
        one fused atm_run per realisation for a Gaussian / plane source and a
        vacuum path or a path of SSPhaseScreen screens; other channels run the
        reference's own path, whose steps below go to the engine
    VacuumPath.lossless_output           (pathes.py:27-40)    atm_vacuum
    SSPhaseScreen.generate_phase_screen  (phase_screens.py:108-136)
        atm_screen of the spectrum the reference's own _get_spectrum draws;
        the engine forms the real screen (the imaginary part, which only
        PhaseScreen.generator reads, is returned as zero)
    Simulation.run                       (simulations/simulation.py:127-138)
        the batched engine path when every measure is one the fused
        reductions produce (beam moments, eta, BeamResult.mean_x2_r, PDT and
        tracked-PDT transmittances); otherwise the reference's loop, whose
        propagation runs on the engine through the methods above

Spectra always come from the reference's ``_get_spectrum`` (numpy's global
generator, scipy's annulus quadratures), so a seeded run gives the
realisations the reference gives.  Any other value of the switch leaves
every method the reference's own.  ``uninstall`` restores the originals.
"""
from __future__ import annotations

import functools

import numpy as np

from . import gpu

SWITCH_KEY = "engine"
SWITCH_VALUE = "gb300"

_PATCHES = (
    ("channels", "Channel", "run"),
    ("pathes", "VacuumPath", "lossless_output"),
    ("phase_screens", "SSPhaseScreen", "generate_phase_screen"),
    ("simulations.simulation", "Simulation", "run"),
)


def _module(ref, dotted):
    mod = ref
    for part in dotted.split("."):
        mod = getattr(mod, part)
    return mod


def enabled(ref) -> bool:
    return ref.gpu.config.get(SWITCH_KEY) == SWITCH_VALUE


def _to_numpy(t):
    return t.detach().cpu().numpy()


# ---------------------------------------------------------------------------
# replacements
# ---------------------------------------------------------------------------
def _channel_run(ref, original):
    @functools.wraps(original)
    def run(self, pupil=True, *args, **kwargs):
        from .engine.runner import fusable, get_plan, run_single, screen_kind
        if not enabled(ref) or args or not set(kwargs) <= {"shift", "wind"} or not fusable(self):
            return original(self, pupil, *args, **kwargs)
        if screen_kind(self.path) == "fft" and kwargs:
            return original(self, pupil, *args, **kwargs)  # FFT screens take no shift / wind
        import torch
        plan = get_plan(self, batch=1, shift=kwargs.get("shift", (0, 0)), path_output_loss=True)
        field = torch.empty((1, plan.N, plan.N), dtype=torch.complex64, device=plan.device)
        run_single(self, plan, field, wind=kwargs.get("wind", False))
        plan.check()
        out = _to_numpy(field[0])
        return self.pupil.output(out) if pupil else out

    return run


def _vacuum_step(ref, original):
    @functools.wraps(original)
    def lossless_output(self, input, length=None):
        step = self.length if length is None else length
        if not enabled(ref) or not step > 0:
            return original(self, input, length)
        import torch
        from .engine.plan import EnginePlan
        from .engine.runner import grid_size
        ch = self.channel
        N, delta, wvl = grid_size(ch.grid), float(ch.grid.delta), float(ch.source.wvl)
        plans = ch.__dict__.setdefault("_atm_plans", {})
        key = ("vacuum-steps", N, delta, wvl, str(gpu.device()))
        if key not in plans:
            plans[key] = EnginePlan(N, delta, wvl, 1.0, float("inf"), [], 1.0, batch=1, device=gpu.device())
        a = np.array(np.broadcast_to(np.asarray(input, dtype=np.complex64), (N, N)))  # a writable copy
        field = torch.from_numpy(a).to(gpu.device())
        plans[key].vacuum(field, float(step))
        return _to_numpy(field)

    return lossless_output


def _ss_screen(ref, original):
    @functools.wraps(original)
    def generate_phase_screen(self, shift=(0, 0), wind=False):
        if not enabled(ref):
            return original(self, shift=shift, wind=wind)
        import torch
        from .engine.plan import EnginePlan
        from .engine.runner import grid_size, to_device
        sp = self._get_spectrum(use_cached_spectrum=wind)
        N, delta = grid_size(self.grid), float(self.grid.delta)
        base = np.asarray(self.f_grid.base, np.float32)
        key = (N, delta, float(shift[0]), float(shift[1]), base.tobytes(), str(gpu.device()))
        if getattr(self, "_atm_screen_key", None) != key:
            self._atm_screen_plan = EnginePlan(N, delta, float(self.wvl), 1.0, float("inf"), [0.0], 1.0,
                                               f_base=base, shift=shift, batch=1, device=gpu.device())
            self._atm_screen_key = key
        plan = self._atm_screen_plan
        rho, theta, value = to_device(np.asarray(sp.rho, np.float32).reshape(1, 1, -1),
                                      np.asarray(sp.theta, np.float32).reshape(1, 1, -1),
                                      np.asarray(sp.value, np.complex64).reshape(1, 1, -1))
        phi = torch.empty((1, N, N), dtype=torch.float32, device=plan.device)
        plan.screen(rho, theta, value, 0, phi_out=phi)
        plan.check()
        return _to_numpy(phi[0]).astype(np.complex64)

    return generate_phase_screen


def classify_reference(ref, channel, mtype, ops):
    """The fused-output kind (see simulations.fused.resolve) of a measure
    chain built from the reference's own measures and result classes, or None."""
    M = ref.measures
    moments = {M.mean_x: 1, M.mean_y: 2, M.mean_x2: 3, M.mean_xy: 4, M.mean_y2: 5}
    PDT = ref.simulations.pdt.PDTResult
    Tracked = ref.simulations.pdt.TrackedPDTResult
    Beam = ref.simulations.beam.BeamResult

    def pupil_partial(op):
        return isinstance(op, functools.partial) and getattr(op.func, "__func__", None) is PDT.append_pupil

    if mtype == "atmosphere":
        if len(ops) == 1:
            if ops[0] in moments:
                return ("slot", moments[ops[0]])
            if ops[0] is M.eta:
                return ("slot", 0)
            if getattr(ops[0], "__func__", None) is Beam.mean_x2_r:
                return ("slot", 6)
            return None
        if len(ops) == 2 and ops[1] is M.eta and pupil_partial(ops[0]):
            owner = ops[0].func.__self__
            if type(owner) is PDT:
                sx, sy = owner.pupil_shift
                return ("pupil", (float(ops[0].args[0].radius), float(sx), float(sy)))
            return None
        if len(ops) == 3 and ops[2] is M.eta and pupil_partial(ops[1]):
            owner = getattr(ops[0], "__self__", None)
            if isinstance(owner, Tracked) and getattr(ops[0], "__func__", None) is Tracked.set_pupil_position:
                return ("tracked", (float(ops[1].args[0].radius),))
        return None
    if mtype == "pupil" and len(ops) == 1 and ops[0] is M.eta and getattr(channel, "pupil", None) is not None:
        return ("pupil", (float(channel.pupil.radius), 0.0, 0.0))
    return None


def _batch_plan_reference(ref, sim):
    from .engine.runner import fusable, screen_kind
    plans = {}
    for channel, by_time in sim.measures.items():
        if not fusable(channel):
            return None
        fft = screen_kind(channel.path) == "fft"
        for time, by_type in by_time.items():
            if fft and time is not None:
                return None  # FFT screens do not move with time
            if fft and "phase_screen" in by_type:
                return None
            for mtype, by_ops in by_type.items():
                for ops, ms in by_ops.items():
                    kind = classify_reference(ref, channel, mtype, ops)
                    if kind is None:
                        return None
                    plans.setdefault(channel, []).extend((m, kind, time) for m in ms)
    return plans or None


def _simulation_run(ref, original):
    @functools.wraps(original)
    def run(self, *args, plot_step=None, save_step=None, **kwargs):
        plans = _batch_plan_reference(ref, self) if enabled(ref) else None
        if plans is None:
            return original(self, *args, plot_step=plot_step, save_step=save_step, **kwargs)
        from .simulations.fused import run_batched
        done = 0
        try:
            while not self.is_measures_done():
                n = run_batched(plans, int(gpu.config.get("batch", 256)))
                for it in range(done + 1, done + n + 1):
                    self.process_output(it, plot_step=plot_step, save_step=save_step)
                done += n
        except KeyboardInterrupt:
            pass  # what was measured is kept and saved below, as the reference does
        finally:
            self.process_output(0, plot_step=plot_step, save_step=save_step)

    return run


def install(ref) -> None:
    """Wraps the reference's hot-path methods (idempotent) and adds the
    engine switch to its gpu.config (default off)."""
    makers = {("channels", "Channel", "run"): _channel_run,
              ("pathes", "VacuumPath", "lossless_output"): _vacuum_step,
              ("phase_screens", "SSPhaseScreen", "generate_phase_screen"): _ss_screen,
              ("simulations.simulation", "Simulation", "run"): _simulation_run}
    ref.gpu.config.setdefault(SWITCH_KEY, None)
    for (mod, cls_name, meth), make in makers.items():
        cls = getattr(_module(ref, mod), cls_name)
        if getattr(cls, f"_gb300_original_{meth}", None) is not None:
            continue
        original = cls.__dict__[meth]
        setattr(cls, f"_gb300_original_{meth}", original)
        setattr(cls, meth, make(ref, original))


def uninstall(ref) -> None:
    """Restores the reference's own methods."""
    for mod, cls_name, meth in _PATCHES:
        cls = getattr(_module(ref, mod), cls_name)
        original = cls.__dict__.get(f"_gb300_original_{meth}")
        if original is not None:
            setattr(cls, meth, original)
            delattr(cls, f"_gb300_original_{meth}")


def installed(ref) -> bool:
    return all(getattr(getattr(_module(ref, m), c), f"_gb300_original_{f}", None) is not None for m, c, f in _PATCHES)
