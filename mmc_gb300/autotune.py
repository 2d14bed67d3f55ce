"""Launch-shape autotuner for the photon engine.

Times short trial launches of a simulation on its resident mesh over a grid of
(threads per block, persistent blocks per SM, fluence accumulation policy) and
keeps the fastest.  Trials reuse one session per candidate, so each timing is
a device-only kernel measurement (CUDA events on the session's stream) after a
warm-up launch.  Results are cached per (mesh, workload signature).

The accumulation policy is the atomic-staging choice: float64 atomics into one
buffer, or float32 atomics with the overflow buffer of the reference.

A batch is tuned as a batch (autotune_batch): the batched kernel stages every
simulation's media table in each block's shared memory, so the block shape
that is best for one simulation can starve a large batch of resident blocks
(256 simulations: 20 KB per block; 16 blocks of 64 threads per SM do not fit,
and a shape tuned on one simulation ran the 256-simulation batch 1.4x slower
than 8 blocks of 128 threads).
"""
from __future__ import annotations

import dataclasses
import itertools
from typing import Dict, Iterable, Optional, Tuple

import numpy as np

from .core import Mesh, Session, SimConfig, launch_batch

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


def autotune_batch(meshes, cfgs, photons_per_lane: int = 32, threads: Iterable[int] = (64, 128),
                   blocks_per_sm: Iterable[int] = (6, 8), accum: Iterable[int] = (1, 0), repeats: int = 2,
                   use_cache: bool = True) -> dict:
    """As autotune, for one batched launch over all of `cfgs` (each on its
    mesh): every candidate shape runs trial batched launches of the whole
    batch, the trial photons of a launch split over the simulations in
    proportion to their photon counts (at least one each).  Each candidate
    holds a session -- a fluence buffer -- per simulation while it runs, as
    the batched run itself does."""
    key = ("batch", tuple(_signature(m, c) for m, c in zip(meshes, cfgs)), photons_per_lane, tuple(threads),
           tuple(blocks_per_sm), tuple(accum))
    if use_cache and key in _cache:
        return _cache[key]
    sms = _sm_count(meshes[0].device)
    w = np.array([max(int(c.nphoton), 1) for c in cfgs], np.float64)
    trials = []
    best = None
    for th, bps, acc in itertools.product(threads, blocks_per_sm, accum):
        blocks = sms * bps * (128 // th)
        trial = blocks * th * photons_per_lane
        counts = np.maximum(1, np.floor(trial * w / w.sum())).astype(np.int64)
        sess = [Session(m, dataclasses.replace(c, nphoton=int(k) * (repeats + 1), threads=th, blocks=blocks,
                                               accum_f64=acc, save_field=False, issaveseed=0))
                for m, c, k in zip(meshes, cfgs, counts)]
        try:
            launch_batch(sess, [0] * len(sess), counts.tolist())
            sess[0].sync()
            ms = []
            for r in range(repeats):
                launch_batch(sess, [int(k) * (r + 1) for k in counts], counts.tolist())
                ms.append(sess[0].sync())  # the batch is timed on the first session's events
        finally:
            for s_ in sess:
                s_.end(collect=False)
        rate = float(counts.sum()) / min(ms)
        trials.append(dict(threads=th, blocks=blocks, accum_f64=acc, photons_per_ms=rate,
                           photons_per_thread=photons_per_lane))
        if best is None or rate > best["photons_per_ms"]:
            best = trials[-1]
    out = dict(best, trials=trials)
    _cache[key] = out
    return out
