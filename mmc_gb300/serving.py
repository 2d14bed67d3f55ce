"""Continuous-batching simulation server.

Requests (a resident mesh, optical properties, source, detectors, photon
count) arrive at any time.  The server runs the GPU in waves: every wave is
one persistent launch over admitted requests, composed shortest remaining
work first within a per-wave photon budget.  Waves are pipelined: up
to `depth` of them are in flight on separate CUDA streams
(mmcgb_session_launch_batch_on), so the next wave's blocks take over the SMs
while the current wave's last photons drain, and the host plans the next wave
while the device works.  When a wave completes the server admits waiting
requests while the free device memory, less a reserve, covers their fluence
and detector buffers, and hands requests whose photons are all traced to a
background thread (output stage + readback).  A request that arrives while
others are on the GPU therefore joins within a wave or two and shares the
device with them; the engine's per-photon random streams make each result
identical to running the request alone (tests/test_gpu_serving.py).

The meshes stay resident (one upload each); nothing about a request is
uploaded except its small parameter block and tables.
"""
from __future__ import annotations

import dataclasses
import threading
import time
from collections import deque
from typing import Dict, List, Optional

import numpy as np

from .core import Mesh, Session, SimConfig, SimResult, launch_batch


@dataclasses.dataclass
class Request:
    mesh: str
    cfg: SimConfig
    arrival: float = 0.0            # perf_counter time the request entered the system
    rid: int = -1
    admitted: float = 0.0
    finished: float = 0.0
    result: Optional[SimResult] = None
    error: Optional[str] = None

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


def device_bytes(mesh: Mesh, cfg: SimConfig) -> int:
    """Device memory a request holds while admitted (fluence + detector buffers)."""
    flen = mesh.ne * cfg.maxgate * max(1, int(cfg.srcnum))
    per = 8 if cfg.accum_f64 else 8  # float64, or two float32 halves
    nmed = np.asarray(cfg.media).reshape(-1, 4).shape[0]
    reclen = 2 + (2 + (1 if cfg.ismomentum else 0)) * (nmed - 1) + (6 if cfg.issaveexit else 0)
    det = cfg.maxdetphoton * (reclen * 4 + (16 if cfg.issaveseed else 0)) if cfg.issavedet else 0
    nodal = 4 * mesh.nn * ((cfg.nodemua is not None) + (cfg.nodemua is not None and cfg.nodemusp is not None))
    return flen * per + det + nodal + (1 << 16)


class Server:
    def __init__(self, meshes: Dict[str, Mesh], wave_photons: int = 4_000_000, min_share: int = 50_000,
                 max_active: int = 128, memory_budget: Optional[int] = None, reserve: int = 2 << 30,
                 depth: int = 2, max_wave_requests: int = 16):
        import torch
        self.meshes = meshes
        self.wave_photons = int(wave_photons)
        self.min_share = int(min_share)
        self.max_active = int(max_active)
        self.depth = max(1, int(depth))
        self.max_wave_requests = max(1, int(max_wave_requests))
        dev = next(iter(meshes.values())).device
        free, _ = torch.cuda.mem_get_info(dev)
        self.budget = int(memory_budget) if memory_budget else max(0, free - reserve)
        self.in_use = 0
        self.pending: deque = deque()
        # active entries: [request, session, photons assigned to waves, device bytes, waves in flight]
        self.active: List[list] = []
        self.completed: List[Request] = []
        self.waves = 0
        self.wave_ms: List[float] = []
        self.enqueue_ms: List[float] = []  # host time to enqueue one wave (setup copies + launch)
        self._streams = [torch.cuda.Stream(device=dev) for _ in range(self.depth)]
        self._inflight: deque = deque()  # (event, [(entry, count)], launch time)
        self._last_done: Optional[float] = None
        self._lock = threading.Lock()
        self._next_id = 0
        # readback + normalization of finished requests overlaps the next wave
        from concurrent.futures import ThreadPoolExecutor
        self._finisher = ThreadPoolExecutor(max_workers=4)
        self._finishing: List = []

    def submit(self, req: Request) -> Request:
        with self._lock:
            req.rid = self._next_id
            self._next_id += 1
            if not req.arrival:
                req.arrival = time.perf_counter()
            self.pending.append(req)
        return req

    def _admit(self):
        while self.pending and len(self.active) < self.max_active:
            req = self.pending[0]
            mesh = self.meshes[req.mesh]
            need = device_bytes(mesh, req.cfg)
            if self.active and self.in_use + need > self.budget:
                break  # wait for memory to free up (FIFO: no overtaking)
            self.pending.popleft()
            try:
                sess = Session(mesh, req.cfg)
            except Exception as e:  # reported per request; the server keeps going
                req.error, req.finished = str(e), time.perf_counter()
                self.completed.append(req)
                continue
            req.admitted = time.perf_counter()
            self.in_use += need
            self.active.append([req, sess, 0, need, 0])

    def _launch_wave(self) -> bool:
        """Composes the next wave shortest-remaining-first: requests in order
        of untraced photons take their remainder (at least `min_share`) until
        the wave's photon budget or `max_wave_requests` is reached.  Small
        requests thus finish in one wave, and a wave mixes few requests, so
        their fluence buffers and meshes compete less for the L2."""
        import torch
        live = [a for a in self.active if a[2] < a[0].cfg.nphoton]
        if not live:
            return False
        live.sort(key=lambda a: (a[0].cfg.nphoton - a[2], a[0].rid))
        budget = self.wave_photons
        picked, counts = [], []
        for a in live:
            if len(picked) >= self.max_wave_requests or budget <= 0:
                break
            k = min(a[0].cfg.nphoton - a[2], max(budget, self.min_share))
            picked.append(a)
            counts.append(k)
            budget -= k
        live = picked
        st = self._streams[self.waves % self.depth]
        t0 = time.perf_counter()
        launch_batch([a[1] for a in live], [a[2] for a in live], counts, stream=st.cuda_stream)
        self.enqueue_ms.append((time.perf_counter() - t0) * 1e3)
        ev = torch.cuda.Event()
        ev.record(st)
        for a, k in zip(live, counts):
            a[2] += k
            a[4] += 1
        self._inflight.append((ev, list(zip(live, counts)), time.perf_counter()))
        self.waves += 1
        return True

    def _complete_wave(self):
        ev, members, t_launch = self._inflight.popleft()
        ev.synchronize()
        now = time.perf_counter()
        # device time per wave, seen from the host: the gap between consecutive completions
        self.wave_ms.append((now - max(t_launch, self._last_done or t_launch)) * 1e3)
        self._last_done = now
        for a, _ in members:
            a[4] -= 1
            if a[2] >= a[0].cfg.nphoton and a[4] == 0:
                self.active = [x for x in self.active if x is not a]
                self._finishing.append(self._finisher.submit(self._finish, a))

    def step(self) -> bool:
        """Admits, keeps up to `depth` waves in flight, completes the oldest
        one and finishes requests whose photons are all traced.  Returns
        False when there is nothing to do."""
        with self._lock:
            self._admit()
        while len(self._inflight) < self.depth and self._launch_wave():
            pass
        if not self._inflight:
            return False
        self._complete_wave()
        self._reap(block=False)
        return True

    def _finish(self, a):
        req, sess = a[0], a[1]
        try:
            req.result = sess.end()
        except Exception as e:
            req.error = str(e)
        req.finished = time.perf_counter()
        return a

    def _reap(self, block: bool):
        keep = []
        for f in self._finishing:
            if block or f.done():
                a = f.result()
                with self._lock:
                    self.in_use -= a[3]
                    self.completed.append(a[0])
            else:
                keep.append(f)
        self._finishing = keep

    def run(self, arrivals: Optional[List[Request]] = None, deadline: float = float("inf")):
        """Serves until all submitted (and scheduled) requests are done.
        `arrivals`: requests with `arrival` times in the future (perf_counter
        clock) that are submitted when their time comes."""
        sched = sorted(arrivals or [], key=lambda r: r.arrival)
        try:
            self._serve(sched, deadline)
        finally:
            for st in self._streams:  # no wave outlives the loop, whatever ended it
                st.synchronize()
        return self.completed

    def _serve(self, sched, deadline):
        i = 0
        while True:
            now = time.perf_counter()
            while i < len(sched) and sched[i].arrival <= now:
                self.submit(sched[i])
                i += 1
            busy = self.step()
            if not busy:
                if self._finishing:
                    self._reap(block=True)
                    continue
                if i >= len(sched) and not self.pending:
                    break
                if i < len(sched):
                    time.sleep(max(0.0, min(0.005, sched[i].arrival - time.perf_counter())))
            if time.perf_counter() > deadline:
                raise TimeoutError("serving deadline exceeded")
        return self.completed

    def stats(self) -> dict:
        done = [r for r in self.completed if r.error is None]
        lat = np.array([r.latency for r in done]) * 1e3
        photons = sum(r.cfg.nphoton for r in done)
        t0 = min((r.arrival for r in done), default=0.0)
        t1 = max((r.finished for r in done), default=0.0)
        return dict(requests=len(done), errors=len(self.completed) - len(done), photons=photons,
                    p50_ms=float(np.percentile(lat, 50)) if len(lat) else None,
                    p99_ms=float(np.percentile(lat, 99)) if len(lat) else None,
                    span_s=t1 - t0, photons_per_ms=photons / max((t1 - t0) * 1e3, 1e-9),
                    waves=self.waves, mean_wave_ms=float(np.mean(self.wave_ms)) if self.wave_ms else None,
                    mean_enqueue_ms=float(np.mean(self.enqueue_ms)) if self.enqueue_ms else None)
