"""Engine switch (the reference's pyatmosphere/gpu.py:4-20).

``config["use_gpu"]`` selects the array backend in the reference (numpy or
cupy).  Here the only backend is the GB300 engine: fields are torch CUDA
tensors and every propagation, screen and measure runs in libatm.so.
Setting ``use_gpu`` to False makes engine calls raise instead of falling
back to a CPU path.  ``batch`` is the number of realisations the batched
Monte-Carlo path runs per engine call.
"""
from __future__ import annotations

config = {
    "use_gpu": True,
    "engine": "gb300",
    "device": None,      # torch device; None = current CUDA device
    "batch": 256,        # realisations per engine call in Simulation
    "cheb_cut": 0.0,     # low-frequency block cut (0 = engine default)
}


def get_xp():
    """Array module of engine outputs (torch)."""
    require_engine()
    import torch
    return torch


def get_array(xp_array):
    """Host numpy copy of an engine array (cupy's ``.get()`` in the reference)."""
    try:
        import torch
        if isinstance(xp_array, torch.Tensor):
            return xp_array.detach().cpu().numpy()
    except ImportError:  # pragma: no cover
        pass
    return xp_array


def require_engine():
    if not config.get("use_gpu", True):
        raise RuntimeError("pyatmosphere_gb300 runs on the GB300 engine only (gpu.config['use_gpu'] is False); "
                           "use the reference pyatmosphere package for its numpy path")


def device():
    import torch
    require_engine()
    if not torch.cuda.is_available():
        raise RuntimeError("the GB300 engine needs a CUDA device; none is available")
    d = config.get("device")
    return torch.device(d) if d is not None else torch.device("cuda", torch.cuda.current_device())
