"""Launch-shape autotuner for the photon engine.

Times short trial launches of a simulation on its resident mesh over a grid of
(threads per block, persistent blocks per SM, fluence accumulation policy) and
keeps the fastest.  Trials reuse one session per candidate, so each timing is
a device-only kernel measurement (CUDA events on the session's stream) after a
warm-up launch.  Results are cached per (mesh, workload signature).

The accumulation policy is the atomic-staging choice: float64 atomics into one
buffer, or float32 atomics with the overflow buffer of the reference.
"""
from __future__ import annotations

import dataclasses
import itertools
from typing import Dict, Iterable, Optional, Tuple

from .core import Mesh, Session, SimConfig

_cache: Dict[Tuple, dict] = {}


def _sm_count(device: int) -> int:
    import torch
    return torch.cuda.get_device_properties(device).multi_processor_count


def _signature(mesh: Mesh, cfg: SimConfig):
    return (id(mesh), mesh.ne, cfg.maxgate, cfg.issavedet, int(cfg.fast_math),
            tuple(map(tuple, __import__("numpy").asarray(cfg.media).round(6).tolist())))


def autotune(mesh: Mesh, cfg: SimConfig, photons_per_lane: int = 32,
             threads: Iterable[int] = (64, 128), blocks_per_sm: Iterable[int] = (6, 8),
             accum: Iterable[int] = (1, 0), repeats: int = 2, use_cache: bool = True) -> dict:
    """Returns {'threads', 'blocks', 'accum_f64', 'photons_per_ms', 'trials'} and
    leaves `cfg` unchanged; apply with dataclasses.replace(cfg, **choice).

    Each trial launch gives every lane of the candidate grid the same number
    of photons (`photons_per_lane`): a launch ends with the drain of its last
    photons in flight, and a fixed photon count would favour small grids,
    whose lanes each run more photons past that drain.  The persistent grid
    hands photons out dynamically, so the grid size also sets the photons per
    thread (launch photons / lanes)."""
    key = (_signature(mesh, cfg), photons_per_lane, tuple(threads), tuple(blocks_per_sm), tuple(accum))
    if use_cache and key in _cache:
        return _cache[key]
    sms = _sm_count(mesh.device)
    trials = []
    best = None
    for th, bps, acc in itertools.product(threads, blocks_per_sm, accum):
        # same resident warps per SM for each thread count
        blocks = sms * bps * (128 // th)
        trial_photons = blocks * th * photons_per_lane
        c = dataclasses.replace(cfg, nphoton=trial_photons, threads=th, blocks=blocks, accum_f64=acc,
                                save_field=False)
        s = Session(mesh, c)
        s.launch(0, trial_photons)
        s.sync()
        ms = []
        for r in range(repeats):
            s.launch((r + 1) * trial_photons, trial_photons)
            ms.append(s.sync())
        s.end(collect=False)
        rate = trial_photons / min(ms)
        trials.append(dict(threads=th, blocks=blocks, accum_f64=acc, photons_per_ms=rate,
                           photons_per_thread=photons_per_lane))
        if best is None or rate > best["photons_per_ms"]:
            best = trials[-1]
    out = dict(best, trials=trials)
    _cache[key] = out
    return out


def tuned(mesh: Mesh, cfg: SimConfig, **kw) -> SimConfig:
    """`cfg` with the autotuned launch shape and accumulation policy."""
    b = autotune(mesh, cfg, **kw)
    return dataclasses.replace(cfg, threads=b["threads"], blocks=b["blocks"], accum_f64=b["accum_f64"])
