"""Generates the golden vectors in this folder by running the reference
pyAtmosphere itself (pure Python) on injected, seeded inputs.

Usage (from the repository root, in a container where the reference tree is
available)::

    python tests/golden/make_golden.py /path/to/pyAtmosphere

matplotlib and pandas are only needed by the reference's plotting and CSV
code; they are replaced by empty stub modules so that the propagation path
imports.  Spectra are injected by replacing ``SSPhaseScreen._get_spectrum`` on
every screen of the path (phase_screens.py:93-106); FFT-screen normals by
replacing ``numpy.random.normal`` during the call (phase_screens.py:46).

The output is ``golden.npz`` (a few hundred KB).  Tests only read that file;
nothing at test time imports the reference.
"""
from __future__ import annotations

import os
import sys
import time
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import atm_oracle as orc  # noqa: E402  (for the seeded draws only)


def import_reference(path):
    for m in ["matplotlib", "matplotlib.pyplot", "pandas"]:
        sys.modules.setdefault(m, types.ModuleType(m))
    sys.modules["matplotlib"].pyplot = sys.modules["matplotlib.pyplot"]
    sys.modules["matplotlib.pyplot"].plt = None
    sys.path.insert(0, path)
    import pyatmosphere  # noqa: F401
    from pyatmosphere import gpu
    gpu.config["use_gpu"] = False
    return pyatmosphere


def make_channel(pa, N, delta, wvl, w0, F0, length, count, Cn2, l0, L0, points,
                 f_min, f_max, radius, position="middle"):
    from pyatmosphere.channels import Channel
    from pyatmosphere.grids import RectGrid, RandLogPolarGrid
    from pyatmosphere.sources import GaussianSource
    from pyatmosphere.pathes import IdenticalPhaseScreensPath
    from pyatmosphere.phase_screens import SSPhaseScreen
    from pyatmosphere.theory.models import MVKModel
    from pyatmosphere.pupils import CirclePupil
    return Channel(
        grid=RectGrid(resolution=N, delta=delta),
        source=GaussianSource(wvl=wvl, w0=w0, F0=F0),
        path=IdenticalPhaseScreensPath(
            phase_screen=SSPhaseScreen(
                model=MVKModel(Cn2=Cn2, l0=l0, L0=L0),
                f_grid=RandLogPolarGrid(points=points, f_min=f_min, f_max=f_max)),
            length=length, count=count, position_in_slab=position),
        pupil=CirclePupil(radius=radius))


class Injector:
    """Serves the injected spectrum of (current realisation, screen i)."""

    def __init__(self, channel, rho, theta, value):
        from pyatmosphere.utils import PolarDiscreteFunction
        self.r = 0
        self.rho, self.theta, self.value = rho, theta, value
        channel.path.init_phase_screens()
        for i, ps in enumerate(channel.path.phase_screens):
            def getter(use_cached_spectrum, i=i):
                return PolarDiscreteFunction(rho=self.rho[self.r, i].copy(),
                                             theta=self.theta[self.r, i].copy(),
                                             value=self.value[self.r, i].copy())
            ps._get_spectrum = getter


def spec_kwargs(spec: orc.ChannelSpec):
    return dict(N=spec.N, delta=spec.delta, wvl=spec.wvl, w0=spec.w0, F0=spec.F0,
                length=spec.length, count=spec.count, Cn2=spec.Cn2, l0=spec.l0,
                L0=spec.L0, points=spec.points, f_min=spec.f_min, f_max=spec.f_max,
                radius=spec.pupil_radius, position=spec.position)


def channel_psd(pa, spec):
    ch = make_channel(pa, **spec_kwargs(spec))
    ch.path.init_phase_screens()
    return np.asarray(ch.path.phase_screens[0]._get_psd()), np.asarray(ch.path.phase_screens[0].f_grid.base)


def run_realisations(pa, spec, seed, R, tracked=True):
    """Runs R realisations through the reference Simulation with BeamResult,
    PDTResult and TrackedPDTResult and returns the per-realisation scalars."""
    from pyatmosphere import simulations
    ch = make_channel(pa, **spec_kwargs(spec))
    psd, base = channel_psd(pa, spec)
    rho, theta, value = orc.draw_spectra(seed, range(R), spec.count, base, psd)
    inj = Injector(ch, rho, theta, value)
    beam = simulations.BeamResult(ch, max_size=R)
    pdt = simulations.PDTResult(ch, max_size=R)
    results = [beam, pdt]
    if tracked:
        tpdt = simulations.TrackedPDTResult(ch, max_size=R)
        results.append(tpdt)
    sim = simulations.Simulation(results)
    for r in range(R):
        inj.r = r
        sim.iter()
    out = {
        "mean_x": np.array(beam.measures[0].data), "mean_y": np.array(beam.measures[1].data),
        "mean_x2": np.array(beam.measures[2].data), "mean_xy": np.array(beam.measures[3].data),
        "mean_y2": np.array(beam.measures[4].data), "mean_x2_r": np.array(beam.measures[5].data),
        "eta_0": np.array(pdt.measures[0].data),
    }
    if tracked:
        out["tracked_eta_0"] = np.array(tpdt.measures[2].data)
    return out, (rho, theta, value), ch


def main(ref_path):
    pa = import_reference(ref_path)
    from pyatmosphere import measures
    from pyatmosphere.channels import Channel
    from pyatmosphere.grids import RectGrid
    from pyatmosphere.sources import GaussianSource
    from pyatmosphere.pathes import VacuumPath
    from pyatmosphere.phase_screens import SSPhaseScreen, FFTPhaseScreen
    from pyatmosphere.theory.models import MVKModel
    from pyatmosphere.grids import RandLogPolarGrid
    from pyatmosphere.pupils import CirclePupil
    from pyatmosphere.utils import PolarDiscreteFunction
    g = {}

    # 1. vacuum propagation of Gaussian beams (itest_vacuum_propagation / itest_sources geometry, N=128)
    for tag, F0 in [("inf", np.inf), ("f20000", 20000.0), ("fm6000", -6000.0)]:
        ch = Channel(grid=RectGrid(128, 4e-3), source=GaussianSource(wvl=809e-9, w0=0.05, F0=F0),
                     path=VacuumPath(length=4e3), pupil=CirclePupil(radius=0.05))
        u = ch.run(pupil=False)
        g[f"vac_{tag}_field"] = np.asarray(u, np.complex64)
        g[f"vac_{tag}_mean_x2"] = measures.mean_x2(ch, output=u)
        g[f"vac_{tag}_mean_y2"] = measures.mean_y2(ch, output=u)
        g[f"vac_{tag}_eta"] = measures.eta(ch, output=u)

    # 2. sparse-spectrum screen, N=64, P=64, with and without shift
    spec = orc.ChannelSpec(N=64, delta=2e-3, points=64, length=1e3, count=1, Cn2=1e-14)
    ch = make_channel(pa, **spec_kwargs(spec))
    ch.path.init_phase_screens()
    ps = ch.path.phase_screens[0]
    psd = np.asarray(ps._get_psd())
    rho, theta, value = orc.draw_spectra(11, [0], 1, np.asarray(ps.f_grid.base), psd)
    ps._get_spectrum = lambda use_cached_spectrum: PolarDiscreteFunction(rho[0, 0], theta[0, 0], value[0, 0])
    g["ss_rho"], g["ss_theta"], g["ss_value"] = rho[0, 0], theta[0, 0], value[0, 0]
    g["ss_screen"] = np.asarray(ps.generate(), np.float32)
    g["ss_screen_shift"] = np.asarray(ps.generate(shift=(0.05, -0.1)), np.float32)

    # 3. full small channel (N=128, 3 screens, P=256) through Channel.run
    spec = orc.ChannelSpec(N=128, delta=3e-3, w0=0.06, length=5e3, count=3, points=256,
                           Cn2=2e-15, pupil_radius=0.08)
    ch = make_channel(pa, **spec_kwargs(spec))
    psd, base = channel_psd(pa, spec)
    rho, theta, value = orc.draw_spectra(7, [0], spec.count, base, psd)
    Injector(ch, rho, theta, value)
    u = ch.run(pupil=False)
    g["small_field"] = np.asarray(u, np.complex64)
    g["small_rho"], g["small_theta"], g["small_value"] = rho[0], theta[0], value[0]
    g["small_eta_pupil"] = measures.eta(ch, output=ch.pupil.output(u))
    for m in ["mean_x", "mean_y", "mean_x2", "mean_xy", "mean_y2"]:
        g[f"small_{m}"] = getattr(measures, m)(ch, output=u)

    # 4. the same small channel with screens placed "before" (first step of length 0)
    spec_b = orc.ChannelSpec(**{**spec.__dict__, "position": "before"})
    ch = make_channel(pa, **spec_kwargs(spec_b))
    Injector(ch, rho, theta, value)
    g["small_before_field"] = np.asarray(ch.run(pupil=False), np.complex64)

    # 5. PSD annulus weights at the two headline geometries
    c1 = orc.ChannelSpec()
    c2 = orc.ChannelSpec(N=2048, delta=1.5e-3, w0=0.12, length=50e3, Cn2=5e-16, pupil_radius=0.2)
    g["c1_psd"], g["c1_base"] = channel_psd(pa, c1)
    g["c2_psd"], g["c2_base"] = channel_psd(pa, c2)

    # 6. Monte-Carlo measures through Simulation (Beam, PDT, TrackedPDT)
    t = time.time()
    res, _, _ = run_realisations(pa, c1, seed=1234, R=4)
    for k, v in res.items():
        g[f"c1_{k}"] = v
    print(f"512^2 channel realisations: {time.time() - t:.1f}s")
    t = time.time()
    res, _, _ = run_realisations(pa, c2, seed=99, R=2, tracked=False)
    for k, v in res.items():
        g[f"c2_{k}"] = v
    print(f"2048^2 channel realisations: {time.time() - t:.1f}s")

    # 7. FFT screen with 3 subharmonic levels, normals injected
    rng = np.random.default_rng(5)
    N = 64
    draws = [rng.standard_normal((N, N)), rng.standard_normal((N, N))]
    for _ in range(3):
        draws += [rng.standard_normal((3, 3)), rng.standard_normal((3, 3))]
    queue = list(draws)
    orig = np.random.normal
    np.random.normal = lambda size=None: queue.pop(0)
    try:
        fps = FFTPhaseScreen(3, model=MVKModel(Cn2=1e-14, l0=6e-3, L0=1e3), thickness=1e3,
                             wvl=808e-9, grid=RectGrid(N, 2e-3))
        g["fft_screen"] = np.asarray(fps.generate(complex=True))
    finally:
        np.random.normal = orig
    g["fft_normals"] = np.stack([np.stack(draws[0:2])], 0)
    g["fft_sub_normals"] = np.stack([np.stack(draws[2 + 2 * i:4 + 2 * i]) for i in range(3)], 0)

    # 8. seeded runs through the public API (numpy global RNG, no injection):
    #    Channel.run and a Simulation with Beam / PDT / TrackedPDT results
    spec = orc.ChannelSpec(N=128, delta=3e-3, w0=0.06, length=5e3, count=3, points=256, Cn2=2e-15,
                           pupil_radius=0.08)
    np.random.seed(123)
    ch = make_channel(pa, **spec_kwargs(spec))
    u = ch.run(pupil=False)
    g["seeded_run_field"] = np.asarray(u, np.complex64)
    from pyatmosphere import simulations
    np.random.seed(321)
    ch = make_channel(pa, **spec_kwargs(spec))
    beam = simulations.BeamResult(ch, max_size=3)
    pdt = simulations.PDTResult(ch, max_size=5)
    tpdt = simulations.TrackedPDTResult(ch, max_size=5)
    sim = simulations.Simulation([beam, pdt, tpdt])
    sim.run()
    for i, nm in enumerate(["mean_x", "mean_y", "mean_x2", "mean_xy", "mean_y2", "mean_x2_r"]):
        g[f"seeded_sim_{nm}"] = np.array(beam.measures[i].data)
    g["seeded_sim_eta"] = np.array(pdt.measures[0].data)
    g["seeded_sim_tracked_eta"] = np.array(tpdt.measures[2].data)

    # 9. seeded wind (time-shifted screens) and per-step ("propagation") results
    np.random.seed(555)
    ch = make_channel(pa, **spec_kwargs(spec))
    times = [0.0, 0.02, 0.05]
    tc = simulations.TimeCoherenceResult(ch, times, max_size=4)
    bwc = simulations.TimeBWcorrSimulation(ch, times, max_size=4)
    simulations.Simulation([tc, bwc]).run()
    g["wind_times"] = np.array(times)
    g["wind_eta"] = np.array(tc.measures[0].data)
    g["wind_mean_x"] = np.array(bwc.measures[0].data)
    g["wind_mean_y"] = np.array(bwc.measures[1].data)
    np.random.seed(777)
    ch = make_channel(pa, **spec_kwargs(spec))
    si = simulations.SIResult(ch, max_size=4)
    simulations.Simulation([si]).run()
    g["si_center"] = np.array(si.measures[0].data, dtype=float)
    np.random.seed(888)
    ch = make_channel(pa, **spec_kwargs(spec))
    ch.path.init_phase_screens()  # the result reads phase_screen.wvl through the channel
    sfr = simulations.StructureFunctionResult(ch, max_size=2)
    simulations.Simulation([sfr]).run()
    g["sf_seeded"] = np.array(sfr.measures[0].data, dtype=float)

    out = os.path.join(HERE, "golden.npz")
    np.savez_compressed(out, **{k: np.asarray(v) for k, v in g.items()})
    print("wrote", out, os.path.getsize(out), "bytes")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PYATMOSPHERE_REF", "../pyAtmosphere"))
