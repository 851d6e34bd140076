"""Python handle on an engine plan (one channel geometry, one batch size).

All tensors handed to the engine are CUDA tensors on the plan's device;
calls are ordered on the current torch stream of that device.
"""
from __future__ import annotations

import ctypes
import math
from typing import Optional, Sequence

import numpy as np
import torch

from . import _lib
from ._lib import check, load


def _dptr(arr: Optional[np.ndarray], ctype):
    if arr is None:
        return None
    return arr.ctypes.data_as(ctypes.POINTER(ctype))


def _tptr(t: Optional[torch.Tensor]):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _stream(device) -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


class EnginePlan:
    """Owns an ``AtmPlan`` (include/atm.h)."""

    def __init__(self, N: int, delta: float, wvl: float, w0: float, F0: float,
                 positions: Sequence[float], length: float, f_base: Optional[np.ndarray] = None,
                 losses_db: float = 0.0, path_output_loss: bool = False,
                 shift: Sequence[float] = (0.0, 0.0), pupils: Sequence[tuple] = (),
                 tracked: Sequence[float] = (), batch: int = 1, source: str = "gaussian",
                 cheb_cut: float = 0.0, col_tile: int = 0, device=None, flags: int = 0):
        if not torch.cuda.is_available():
            raise _lib.EngineError("the GB300 engine needs a CUDA device; none is available")
        self.lib = load()
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None
                                   else torch.device(device).index or 0)
        self.N = int(N)
        self.n_screens = len(positions)
        self.batch = int(batch)
        self.P = 0 if f_base is None else int(len(f_base))
        self._base = None if f_base is None else np.ascontiguousarray(f_base, dtype=np.float32)
        self._kw = dict(N=self.N, delta=float(delta), source=source, cheb_cut=float(cheb_cut),
                        col_tile=int(col_tile), batch=self.batch, shift=(float(shift[0]), float(shift[1])),
                        losses_db=float(losses_db or 0.0), path_output_loss=bool(path_output_loss),
                        tracked=list(tracked), flags=int(flags))
        self.n_pupils = len(list(pupils))
        self.n_tracked = len(tracked)
        d = self._desc(wvl, w0, F0, positions, length, pupils)
        self._handle = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            check(self.lib.atm_plan_create(ctypes.byref(d), ctypes.byref(self._handle)))
        self._geometry = (wvl, w0, F0, list(positions), length, list(pupils))
        self._refresh_info()
        self.n_out = self.info["n_out"]

    def _refresh_info(self):
        info = _lib.AtmPlanInfo()
        check(self.lib.atm_plan_info(self._handle, ctypes.byref(info)))
        self.info = {f: getattr(info, f) for f, _ in _lib.AtmPlanInfo._fields_}

    def _desc(self, wvl, w0, F0, positions, length, pupils):
        k = self._kw
        pupils = list(pupils)
        # keep the arrays alive while the descriptor is in use
        self._pos = np.ascontiguousarray(positions, dtype=np.float64)
        self._pr = np.ascontiguousarray([p[0] for p in pupils] or [0.0], dtype=np.float64)
        self._psx = np.ascontiguousarray([p[1] if len(p) > 1 else 0.0 for p in pupils] or [0.0], dtype=np.float64)
        self._psy = np.ascontiguousarray([p[2] if len(p) > 2 else 0.0 for p in pupils] or [0.0], dtype=np.float64)
        self._tr = np.ascontiguousarray(k["tracked"] or [0.0], dtype=np.float64)
        d = _lib.AtmChannelDesc()
        d.abi_version = _lib.ABI_VERSION
        d.resolution = k["N"]
        d.delta = k["delta"]
        d.source_kind = _lib.SOURCE_PLANE if k["source"] == "plane" else _lib.SOURCE_GAUSSIAN
        d.wvl = float(wvl)
        d.w0 = float(w0) if w0 else 0.0
        d.F0 = float(F0)
        d.n_screens = len(self._pos)
        d.positions = _dptr(self._pos, ctypes.c_double)
        d.length = float(length)
        d.losses_db = k["losses_db"]
        d.path_output_loss = 1 if k["path_output_loss"] else 0
        d.points = self.P
        d.f_base = _dptr(self._base, ctypes.c_float)
        d.shift_x, d.shift_y = k["shift"]
        d.n_pupils = len(pupils)
        d.pupil_radius = _dptr(self._pr, ctypes.c_double)
        d.pupil_shift_x = _dptr(self._psx, ctypes.c_double)
        d.pupil_shift_y = _dptr(self._psy, ctypes.c_double)
        d.n_tracked = len(k["tracked"])
        d.tracked_radius = _dptr(self._tr, ctypes.c_double)
        d.batch = k["batch"]
        d.cheb_cut = k["cheb_cut"]
        d.col_tile = k["col_tile"]
        d.flags = k["flags"]
        return d

    def update(self, wvl, w0, F0, positions, length, pupils=()):
        """Re-targets the plan (atm_plan_update): same grid, spectral grid,
        pupil count and batch, at most the creating screen count; new source /
        path / pupil radii."""
        d = self._desc(wvl, w0, F0, positions, length, pupils)
        with torch.cuda.device(self.device):
            check(self.lib.atm_plan_update(self._handle, ctypes.byref(d)))
        self.n_screens = len(positions)
        self._geometry = (wvl, w0, F0, list(positions), length, list(pupils))

    def channel(self, wvl, w0, F0, positions, length, pupils=()) -> "EngineChannel":
        """A channel table set for this plan (atm_channel_create): the state
        `update` would set, built once; run it with `run_channel`."""
        d = self._desc(wvl, w0, F0, positions, length, pupils)
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            check(self.lib.atm_channel_create(self._handle, ctypes.byref(d), ctypes.byref(h)))
        return EngineChannel(self, h, len(positions))

    def run_channel(self, ch: "EngineChannel", rho, theta, value, out: Optional[torch.Tensor] = None,
                    field_out=None) -> torch.Tensor:
        """atm_run with the channel's state in place of the plan's (atm_run_channel)."""
        batch = int(rho.shape[0])
        r, t, v = self._spectra(rho, theta, value, batch, ch.n_screens)
        if out is None:
            out = torch.empty((batch, self.n_out), dtype=torch.float64, device=self.device)
        with torch.cuda.device(self.device):
            check(self.lib.atm_run_channel(self._handle, ch.handle, r, t, v, batch, _tptr(out), _tptr(field_out),
                                           None, _stream(self.device)))
        return out

    def set_shift(self, shift):
        """Moves every screen by `shift` (x, y) metres (atm_plan_update with the
        plan's geometry), as generate_phase_screen(shift=...) does."""
        shift = (float(shift[0]), float(shift[1]))
        if shift == self._kw["shift"]:
            return
        self._kw["shift"] = shift
        wvl, w0, F0, positions, length, pupils = self._geometry
        self.update(wvl, w0, F0, positions, length, pupils)

    def autotune(self, batch: Optional[int] = None, repeats: int = 3) -> dict:
        """Times the FFT-pass launch variants on the plan's workspace
        (atm_autotune) and keeps the fastest; returns the choice."""
        with torch.cuda.device(self.device):
            check(self.lib.atm_autotune(self._handle, int(batch or self.batch), int(repeats), _stream(self.device)))
        self._refresh_info()
        return {k: self.info[k] for k in ("col_tile", "row_variant", "col_variant", "tuned")}

    def set_variants(self, row_variant: int, col_tile: int, col_variant: int):
        """Launch choices by hand (atm_plan_set_variants); results do not change."""
        check(self.lib.atm_plan_set_variants(self._handle, int(row_variant), int(col_tile), int(col_variant)))
        self._refresh_info()

    def draw_spectra(self, seed, first, sqrt_psd, rho, theta, value, channel: Optional["EngineChannel"] = None):
        """Seeded spectra on the device into the given tensors: atm_draw_spectra
        for the plan's own screens, atm_channel_draw_spectra for a channel
        table set's (sqrt_psd [n][P], rho / theta / value [batch][n][P] with n
        the channel's screen count)."""
        batch = int(rho.shape[0])
        n = self.n_screens if channel is None else channel.n_screens
        self._spectra(rho, theta, value, batch, n)
        if sqrt_psd.device != self.device or sqrt_psd.dtype != torch.float32 or not sqrt_psd.is_contiguous() or \
                tuple(sqrt_psd.shape) != (n, self.P):
            raise ValueError(f"sqrt_psd must be a contiguous float32 [{n}, {self.P}] tensor on {self.device}")
        with torch.cuda.device(self.device):
            if channel is None:
                check(self.lib.atm_draw_spectra(self._handle, int(seed), int(first), _tptr(sqrt_psd), batch,
                                                _tptr(rho), _tptr(theta), _tptr(value), _stream(self.device)))
            else:
                check(self.lib.atm_channel_draw_spectra(self._handle, channel.handle, int(seed), int(first),
                                                        _tptr(sqrt_psd), batch, _tptr(rho), _tptr(theta),
                                                        _tptr(value), _stream(self.device)))

    def check(self):
        """Waits for the plan's work on the current stream and raises
        EngineError (code ERR_TIMEOUT or ERR_NONFINITE) if its kernels recorded
        a wait that ran out or non-finite spectra since the last check
        (atm_plan_check); the measures of those runs are NaN."""
        with torch.cuda.device(self.device):
            check(self.lib.atm_plan_check(self._handle, _stream(self.device)))

    # ------------------------------------------------------------------
    def close(self):
        h = getattr(self, "_handle", None)
        if h is not None and h.value:
            with torch.cuda.device(self.device):
                self.lib.atm_plan_destroy(h)
            self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------------
    def _spectra(self, rho, theta, value, batch, n_screens=None):
        n_screens = self.n_screens if n_screens is None else n_screens
        if n_screens == 0:
            return None, None, None
        for t, dt in ((rho, torch.float32), (theta, torch.float32), (value, torch.complex64)):
            if t.device != self.device or t.dtype != dt or not t.is_contiguous():
                raise ValueError("spectra must be contiguous CUDA tensors (float32, float32, complex64) "
                                 f"on {self.device}")
            if tuple(t.shape) != (batch, n_screens, self.P):
                raise ValueError(f"spectra shape {tuple(t.shape)} != {(batch, n_screens, self.P)}")
        return _tptr(rho), _tptr(theta), _tptr(value)

    def run(self, rho, theta, value, out: Optional[torch.Tensor] = None, field_out=None,
            mean_intensity=None) -> torch.Tensor:
        batch = self.batch if rho is None else int(rho.shape[0])
        r, t, v = self._spectra(rho, theta, value, batch)
        if out is None:
            out = torch.empty((batch, self.n_out), dtype=torch.float64, device=self.device)
        with torch.cuda.device(self.device):
            check(self.lib.atm_run(self._handle, r, t, v, batch, _tptr(out), _tptr(field_out),
                                   _tptr(mean_intensity), _stream(self.device)))
        return out

    def run_fft(self, normals, amp, sub_x, sub_y, sub_mean, n_sub: int, out: Optional[torch.Tensor] = None,
                field_out=None) -> torch.Tensor:
        """atm_run with FFT screens (atm_run_fft; the plan needs FLAG_FFT_SCREENS)."""
        batch = int(normals.shape[0])
        if out is None:
            out = torch.empty((batch, self.n_out), dtype=torch.float64, device=self.device)
        with torch.cuda.device(self.device):
            check(self.lib.atm_run_fft(self._handle, _tptr(normals), _tptr(amp), _tptr(sub_x), _tptr(sub_y),
                                       _tptr(sub_mean), int(n_sub), batch, _tptr(out), _tptr(field_out),
                                       _stream(self.device)))
        return out

    def screen(self, rho, theta, value, screen: int, phi_out=None, phasor_out=None):
        batch = int(rho.shape[0])
        r, t, v = self._spectra(rho, theta, value, batch)
        with torch.cuda.device(self.device):
            check(self.lib.atm_screen(self._handle, r, t, v, batch, int(screen), _tptr(phi_out),
                                      _tptr(phasor_out), _stream(self.device)))
        return phi_out, phasor_out

    def vacuum(self, field: torch.Tensor, dz: float) -> torch.Tensor:
        if field.dtype != torch.complex64 or not field.is_contiguous() or field.device != self.device:
            raise ValueError("field must be a contiguous complex64 tensor on the plan's device")
        batch = field.numel() // (self.N * self.N)
        with torch.cuda.device(self.device):
            check(self.lib.atm_vacuum(self._handle, _tptr(field), batch, float(dz), _stream(self.device)))
        return field

    def measures(self, field: torch.Tensor, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        if field.dtype != torch.complex64 or not field.is_contiguous() or field.device != self.device:
            raise ValueError("field must be a contiguous complex64 tensor on the plan's device")
        batch = field.numel() // (self.N * self.N)
        if out is None:
            out = torch.empty((batch, self.n_out), dtype=torch.float64, device=self.device)
        with torch.cuda.device(self.device):
            check(self.lib.atm_measures(self._handle, _tptr(field), batch, _tptr(out), _stream(self.device)))
        return out

    def capture(self, rho, theta, value, out=None):
        """Captures one atm_run on these (fixed) tensors into a CUDA graph and
        returns (graph, out): graph.replay() re-runs the whole launch
        sequence with one launch call.  Refill rho / theta / value in place
        between replays.  A warm-up run outside the capture comes first so
        that the engine's per-device launch settings are already cached."""
        batch = int(rho.shape[0]) if rho is not None else self.batch
        if out is None:
            out = torch.empty((batch, self.n_out), dtype=torch.float64, device=self.device)
        s = torch.cuda.Stream(device=self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            self.run(rho, theta, value, out=out)
        torch.cuda.current_stream(self.device).wait_stream(s)
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            self.run(rho, theta, value, out=out)
        return g, out

    # ------------------------------------------------------------------
    def profile_begin(self, max_launches: int):
        check(self.lib.atm_profile_begin(self._handle, int(max_launches)))

    def profile_end(self) -> dict:
        n = len(_lib.KIND_NAMES)
        ms = (ctypes.c_double * n)()
        cnt = (ctypes.c_int32 * n)()
        with torch.cuda.device(self.device):
            check(self.lib.atm_profile_end(self._handle, ms, cnt, n))
        return {k: {"ms": ms[i], "launches": cnt[i]} for i, k in enumerate(_lib.KIND_NAMES)}


def set_wait_budget(ns: int, device=None):
    """Budget (ns) of the engine's device waits for work on `device`
    (atm_set_wait_budget; default 2e9)."""
    lib = load()
    dev = torch.device("cuda", torch.cuda.current_device() if device is None else torch.device(device).index or 0)
    with torch.cuda.device(dev):
        check(lib.atm_set_wait_budget(int(ns)))


def structure_function(phi: torch.Tensor) -> torch.Tensor:
    """Phase structure function along x averaged over rows
    (atm_structure_function): phi [B][N][N] float32 CUDA -> [B][N-1] float64."""
    if phi.dim() != 3 or phi.shape[1] != phi.shape[2] or not phi.is_cuda:
        raise ValueError("phi must be a [B][N][N] CUDA tensor")
    phi = phi.to(torch.float32).contiguous()
    B, N = int(phi.shape[0]), int(phi.shape[1])
    out = torch.empty((B, N - 1), dtype=torch.float64, device=phi.device)
    with torch.cuda.device(phi.device):
        check(load().atm_structure_function(_tptr(phi), B, N, _tptr(out), _stream(phi.device)))
    return out


def fma_peak_tflops(device=None, blocks: int = 0, iters: int = 4096) -> float:
    """Measured FP32 FMA throughput of the device (TFLOP/s), from the
    engine's probe kernel; best of three launches after a warm-up."""
    lib = load()
    dev = torch.device("cuda", torch.cuda.current_device() if device is None else torch.device(device).index or 0)
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    blocks = blocks or sms * 8
    best = None
    with torch.cuda.device(dev):
        for i in range(4):
            ms = ctypes.c_double()
            check(lib.atm_fma_probe(blocks, iters, ctypes.byref(ms), _stream(dev)))
            if i > 0:
                best = ms.value if best is None else min(best, ms.value)
    flops = blocks * 256.0 * iters * 16.0
    return flops / (best * 1e-3) / 1e12


class EngineChannel:
    """Handle of a channel table set (atm_channel_create) of one plan."""

    def __init__(self, plan: EnginePlan, handle, n_screens: int):
        self.plan = plan
        self.handle = handle
        self.n_screens = int(n_screens)

    def close(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            with torch.cuda.device(self.plan.device):
                self.plan.lib.atm_channel_destroy(h)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
