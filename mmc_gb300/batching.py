"""Size-aware scheduling of many simulations on one GPU.

One persistent batched launch over every simulation (simulate_batch) removes
the start-up and drain of each small simulation's own launch, but it also
traces the large simulations unphased, with every simulation's fluence
buffer live at once.  A simulation of a few million photons fills the GPU by
itself and gains from gate-phased tracing (only a window of its gate planes
live in L2), so simulate_many runs those on their own, one after another on
one stream, and the small ones together in batched launches on a second
stream; the two streams overlap, so one side's launch drain is filled by the
other side's blocks.  Each result equals the simulation run alone: photon
streams depend only on (seed, photon index).
"""
from __future__ import annotations

from typing import Optional, Sequence

from .core import Mesh, Session, SimConfig, SimResult, launch_batch


def simulate_many(meshes: Sequence[Mesh], cfgs: Sequence[SimConfig], solo_photons: int = 4_000_000,
                  group_photons: Optional[int] = None) -> list:
    """Runs every (mesh, cfg) pair and returns their SimResults in order.
    Simulations of at least `solo_photons` photons run as their own session
    launches (gate-phased where the automatic mode engages), chained on one
    stream; the others run as batched launches of at most `group_photons`
    photons each (None: one launch) on another stream."""
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
        solo = [i for i, c in enumerate(cfgs) if int(c.nphoton) >= solo_photons]
        small = [i for i, c in enumerate(cfgs) if int(c.nphoton) < solo_photons and int(c.nphoton) > 0]
        # the small simulations: batched launches on their own stream
        side = torch.cuda.Stream(device=dev)
        groups, cur, tot = [], [], 0
        for i in sorted(small, key=lambda k: int(cfgs[k].nphoton)):
            if cur and group_photons is not None and tot + int(cfgs[i].nphoton) > group_photons:
                groups.append(cur)
                cur, tot = [], 0
            cur.append(i)
            tot += int(cfgs[i].nphoton)
        if cur:
            groups.append(cur)
        for g in groups:
            launch_batch([sessions[i] for i in g], [0] * len(g), [int(cfgs[i].nphoton) for i in g],
                         stream=side.cuda_stream)
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
        side.synchronize()
        return results
    finally:
        for s in sessions:
            if getattr(s, "_h", None) is not None:
                s.end(collect=False)
