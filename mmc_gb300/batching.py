"""Size-aware scheduling of many simulations on one GPU.

One persistent batched launch over every simulation (simulate_batch) removes
the start-up and drain of each small simulation's own launch, but it keeps
every simulation's fluence buffer live and stages every media table in each
block's shared memory for the whole run.  simulate_many sorts the simulations
by photon count and runs them as a sequence of batched launches of about
`group_photons` photons each, so a launch holds simulations of similar size
and only their buffers; the sequence is captured as one CUDA graph
(mmcgb_session_launch_batches), instantiated once and updated in place by
later calls of the same shape.  On the 256-simulation shell workload (photons
log-uniform 1e5-1e7) groups of 6e7 photons ran the whole set in 14.0 s
against 17.1 s for one launch and 20.5 s for one plain launch per simulation;
groups of 3e7, 1e8 and 2e8 photons took 14.5, 14.0 and 14.6 s.  Two options
measured no better and are off by default: running the largest simulations
on their own, gate-phased, on a stream of their own (solo_photons; 14.5-15.6 s
with 4e6-8e6 photon thresholds) and spreading the groups over several
overlapping streams (streams; 14.9-15.0 s with 2 or 3), which makes
concurrent launches compete for the L2.  Each result equals the simulation
run alone: photon streams depend only on (seed, photon index).
"""
from __future__ import annotations

from typing import Optional, Sequence

from .core import Mesh, Session, SimConfig, SimResult, launch_batch, launch_batches


def simulate_many(meshes: Sequence[Mesh], cfgs: Sequence[SimConfig], group_photons: Optional[int] = 60_000_000,
                  solo_photons: Optional[int] = None, streams: int = 1) -> list:
    """Runs every (mesh, cfg) pair and returns their SimResults in order.
    The simulations, in increasing photon count, run as batched launches of
    at most `group_photons` photons each (a larger simulation alone; None:
    one launch for all) on a stream of their own; with `streams` > 1 the
    launches alternate over that many streams.  With `solo_photons`, the
    simulations of at least that many photons run instead as their own
    session launches (gate-phased where the automatic mode engages), chained
    on another stream that overlaps the batched launches."""
    import torch
    n = len(cfgs)
    if len(meshes) != n or n == 0:
        raise ValueError("need one mesh per config")
    dev = meshes[0].device
    if any(m.device != dev for m in meshes):
        raise ValueError("all meshes must live on one device")
    sessions = []
    try:
        for m, c in zip(meshes, cfgs):
            sessions.append(Session(m, c))
        big = solo_photons if solo_photons is not None else float("inf")
        solo = [i for i, c in enumerate(cfgs) if int(c.nphoton) >= big]
        small = [i for i, c in enumerate(cfgs) if 0 < int(c.nphoton) < big]
        # batched launches of simulations of similar size, on their own stream(s)
        sides = [torch.cuda.Stream(device=dev) for _ in range(max(1, int(streams)))]
        groups, cur, tot = [], [], 0
        for i in sorted(small, key=lambda k: int(cfgs[k].nphoton)):
            if cur and group_photons is not None and tot + int(cfgs[i].nphoton) > group_photons:
                groups.append(cur)
                cur, tot = [], 0
            cur.append(i)
            tot += int(cfgs[i].nphoton)
        if cur:
            groups.append(cur)
        if len(sides) == 1 and groups:  # the groups in sequence, as one CUDA graph
            launch_batches([[sessions[i] for i in g] for g in groups], [[0] * len(g) for g in groups],
                           [[int(cfgs[i].nphoton) for i in g] for g in groups], sides[0].cuda_stream)
        else:
            for k, g in enumerate(groups):  # consecutive groups alternate over the side streams
                launch_batch([sessions[i] for i in g], [0] * len(g), [int(cfgs[i].nphoton) for i in g],
                             stream=sides[k % len(sides)].cuda_stream)
        # the large ones: each on its session's stream, each waiting for the one before
        prev = None
        for i in solo:
            st = torch.cuda.ExternalStream(sessions[i].stream, device=dev)
            if prev is not None:
                st.wait_event(prev)
            sessions[i].launch(0, int(cfgs[i].nphoton))
            prev = torch.cuda.Event()
            prev.record(st)
        # every session's end waits for the launches that wrote its buffers
        results = []
        for s in sessions:
            results.append(s.end())
        for st in sides:
            st.synchronize()
        return results
    finally:
        for s in sessions:
            if getattr(s, "_h", None) is not None:
                s.end(collect=False)
