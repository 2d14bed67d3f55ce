"""The batched, serving and differentiation benchmark workloads
(``python bench.py --workload batched|serving|replay``).  Each prints one JSON
line.  Meshes are the seeded synthetic recipes of mmc_gb300.meshgen.

batched  256 simulations on the 4-layer shell mesh (1.296M tets): random
         per-layer mua (log-uniform 1e-3..1e-1), mus' (0.5..3), g (0.8..0.95),
         a source 0.5 mm inside the r=25 mm surface at a random angle pointing
         inward, photons log-uniform 1e5..1e7, element fluence, 10 gates of
         0.5 ns.  One persistent launch for all (simulate_batch) against one
         simulate() each, wall clock with host buffers, plus the device-only
         ratio and the drop-in ratio (mesh set up per simulation); the
         autotuner picks the launch shape.
serving  Poisson arrivals (200/s) over three resident meshes (162k-tet cube,
         1.3M-tet inclusion cube, 0.6 mm shell mesh with 6.0M tets): photons
         log-uniform 1e5..1e8, per-layer properties as above, a random surface
         pencil source, 1-8 detectors, 10 gates, float32 fluence.  p50/p99
         latency and photons/ms, against the same requests run one at a time.
replay   shell mesh, pencil (30,30,5.5) +z, 8 detectors R=1.5 mm on the shell
         surface at polar angles 10..80 deg, 1e7 photons with seeds; L =
         sum_d c_d log W_d; forward and replay (backward) throughput.
"""
from __future__ import annotations

import dataclasses
import json
import time

import numpy as np

from mmc_gb300 import meshgen
from mmc_gb300.autotune import autotune_batch
from mmc_gb300.clocks import ClockSampler
from mmc_gb300.core import Mesh, SimConfig, simulate, simulate_batch

CENTER = np.array([30.0, 30.0, 30.0])


def _random_media(rng, base):
    media = base.copy()
    k = media.shape[0] - 1
    g = rng.uniform(0.8, 0.95, k)
    musp = rng.uniform(0.5, 3.0, k)
    media[1:, 0] = 10 ** rng.uniform(-3, -1, k)
    media[1:, 1] = musp / (1 - g)
    media[1:, 2] = g
    return media.astype(np.float32)


def _surface_source(rng, radius=24.5):
    u = rng.normal(size=3)
    u /= np.linalg.norm(u)
    return tuple(CENTER + radius * u), tuple(-u)


def run_batched(args):
    m = meshgen.shell_mesh(n=60, jitter=0.25, seed=4321)
    mesh = Mesh(m.node, m.elem, m.label)
    t0 = time.perf_counter()
    Mesh(m.node, m.elem, m.label).close()
    mesh_s = time.perf_counter() - t0  # host preparation + upload of the 1.296M-tet mesh (warm context)
    rng = np.random.default_rng(2026)
    cfgs = []
    for i in range(256):
        pos, d = _surface_source(rng)
        cfgs.append(SimConfig(media=_random_media(rng, m.media), nphoton=int(10 ** rng.uniform(5, 7)), seed=i + 1,
                              srcpos=pos, srcdir=d, tend=5e-9, tstep=0.5e-9, basisorder=0, isnormalized=1))
    tune = autotune_batch([mesh] * len(cfgs), cfgs)  # the batch is tuned as the batch it runs
    cfgs = [dataclasses.replace(c, threads=tune["threads"], blocks=tune["blocks"], accum_f64=tune["accum_f64"])
            for c in cfgs]
    total = sum(c.nphoton for c in cfgs)
    clocks = ClockSampler(0)
    clocks.start()
    # serial plain launches through the public API, mesh resident: one simulate() per simulation
    serial_ms, serial_wall = 0.0, 0.0
    for c in cfgs:
        t0 = time.perf_counter()
        r = simulate(mesh, c)
        serial_wall += time.perf_counter() - t0
        serial_ms += r.kernel_ms
        del r
    # all simulations in one persistent launch (simulate_batch: setup, launch, output stage, readback)
    t0 = time.perf_counter()
    results = simulate_batch([mesh] * len(cfgs), cfgs)
    batched_wall = time.perf_counter() - t0
    batched_ms = results[0].kernel_ms
    absorbed = float(np.mean([r.absorbed_fraction for r in results]))
    del results
    # size-aware scheduling (batching.simulate_many): the simulations grouped by photon count into
    # batched launches of about 6e7 photons
    from mmc_gb300.batching import simulate_many
    t0 = time.perf_counter()
    results = simulate_many([mesh] * len(cfgs), cfgs)
    scheduled_wall = time.perf_counter() - t0
    del results
    clk = clocks.stop()
    # the drop-in path as the reference runs it: every simulation prepares and uploads its mesh
    # (mmcgb_run, the counterpart of mmc_run_cu) -- serial wall time plus the measured mesh setup
    dropin_wall = serial_wall + len(cfgs) * mesh_s
    line = {"metric": "aggregate photons/ms, 256 batched simulations", "value": total / (batched_wall * 1e3),
            "unit": "photons/ms", "n_gpus": 1, "higher_is_better": True, "workload": "batched-256-shells",
            "speedup_vs_serial_plain": serial_wall / batched_wall,
            "serial_plain_photons_per_ms": total / (serial_wall * 1e3),
            "speedup_vs_serial_plain_kernel_only": serial_ms / batched_ms,
            "speedup_vs_serial_dropin_with_mesh_setup": dropin_wall / batched_wall,
            "scheduled_photons_per_ms": total / (scheduled_wall * 1e3),
            "scheduled_speedup_vs_serial_plain": serial_wall / scheduled_wall,
            "scheduled_wall_s": scheduled_wall,
            "batched_wall_s": batched_wall, "batched_kernel_ms": batched_ms,
            "serial_wall_s": serial_wall, "serial_kernel_ms": serial_ms, "mesh_setup_s": mesh_s,
            "photons": total, "mean_absorbed_fraction": absorbed,
            "autotune": {k: v for k, v in tune.items() if k != "trials"}, "data": "synthetic", "clocks": clk,
            "config": {"mesh": "4-layer shells 1.296M tets", "sims": 256, "gates": 10,
                       "timing": "wall clock through simulate()/simulate_batch(), host buffers included"}}
    return line


def serving_requests(nreq: int):
    """The serving workload's three resident meshes and its `nreq` requests
    (arrival times relative to 0)."""
    from mmc_gb300.serving import Request
    rng = np.random.default_rng(7)
    meshes = {}
    recipes = {"cube162k": meshgen.homogeneous_cube(n=30),
               "incl1.3M": meshgen.inclusion_cube(n=60, jitter=0.25, seed=12345),
               "shell6M": meshgen.shell_mesh(n=100, jitter=0.15, seed=99)}
    for k, mm in recipes.items():
        meshes[k] = (Mesh(mm.node, mm.elem, mm.label), mm)
    keys = list(meshes)
    reqs = []
    t = 0.0
    for i in range(nreq):
        key = keys[rng.integers(len(keys))]
        mm = meshes[key][1]
        t += rng.exponential(1.0 / 200.0)
        if key == "shell6M":
            pos, d = _surface_source(rng)
            media = _random_media(rng, mm.media)
        else:  # surface pencil on the z=0 face pointing into the cube
            pos, d = (float(rng.uniform(10, 50)), float(rng.uniform(10, 50)), 0.0), (0.0, 0.0, 1.0)
            media = mm.media.copy()
            media[1:, 0] = 10 ** rng.uniform(-3, -1, len(media) - 1)
        ndet = int(rng.integers(1, 9))
        det = []
        for j in range(ndet):
            if key == "shell6M":
                p, _ = _surface_source(rng, 25.0)
            else:
                p = (float(rng.uniform(5, 55)), float(rng.uniform(5, 55)), 0.0)
            det.append([*p, 2.0])
        cfg = SimConfig(media=media, nphoton=int(10 ** rng.uniform(5, 8)), seed=1000 + i, srcpos=pos, srcdir=d,
                        tend=5e-9, tstep=0.5e-9, issavedet=1, detpos=np.array(det, np.float32),
                        maxdetphoton=200_000, basisorder=0, isnormalized=1, accum_f64=0)
        reqs.append(Request(mesh=key, cfg=cfg, arrival=t))
    return meshes, reqs


def run_serving(args):
    from mmc_gb300.serving import Server
    meshes, reqs = serving_requests(args.requests)
    # continuous batching
    srv = Server({k: v[0] for k, v in meshes.items()}, wave_photons=8_000_000, min_share=100_000)
    clocks = ClockSampler(0)
    clocks.start()
    t0 = time.perf_counter()
    for r in reqs:
        r.arrival += t0
    srv.run(arrivals=reqs, deadline=t0 + 1800)
    st = srv.stats()
    # the same requests one at a time, in arrival order (plain launches)
    service = []
    for r in reqs:
        s0 = time.perf_counter()
        simulate(meshes[r.mesh][0], r.cfg)
        service.append(time.perf_counter() - s0)
    clk = clocks.stop()
    fin, lat = 0.0, []
    arr = [r.arrival - t0 for r in reqs]
    for a, s in zip(arr, service):
        fin = max(fin, a) + s
        lat.append(fin - a)
    photons = sum(r.cfg.nphoton for r in reqs)
    serial_rate = photons / (max(fin - arr[0], 1e-9) * 1e3)
    line = {"metric": "served photons/ms (continuous batching)", "value": st["photons_per_ms"], "unit": "photons/ms",
            "n_gpus": 1, "higher_is_better": True, "workload": "serving-3-meshes",
            "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "requests": st["requests"], "waves": st["waves"],
            "mean_wave_ms": st["mean_wave_ms"], "mean_wave_enqueue_ms": st["mean_enqueue_ms"],
            "serial_plain_photons_per_ms": serial_rate,
            "speedup_vs_serial_plain": st["photons_per_ms"] / serial_rate,
            "serial_p50_ms": float(np.percentile(np.array(lat) * 1e3, 50)),
            "serial_p99_ms": float(np.percentile(np.array(lat) * 1e3, 99)), "photons": photons, "data": "synthetic",
            "clocks": clk,
            "config": {"arrival_rate_hz": 200, "photons": "log-uniform 1e5-1e8", "gates": 10, "fluence": "float32"}}
    return line


def run_replay(args):
    from mmc_gb300 import replay as rp
    m = meshgen.shell_mesh(n=60, jitter=0.25, seed=4321)
    mesh = Mesh(m.node, m.elem, m.label)
    th = np.deg2rad(np.arange(10, 90, 10))
    det = np.array([[*(CENTER + 25.0 * np.array([np.sin(a), 0.0, -np.cos(a)])), 1.5] for a in th], np.float32)
    cfg = SimConfig(media=m.media, nphoton=10_000_000, seed=31, srcpos=(30.0, 30.0, 5.5), tend=5e-9, tstep=5e-9,
                    issavedet=1, issaveseed=1, detpos=det, maxdetphoton=5_000_000, basisorder=0, isnormalized=0)
    c = np.random.default_rng(3).normal(size=len(det))
    clocks = ClockSampler(0)
    clocks.start()
    t0 = time.perf_counter()
    fwd = simulate(mesh, cfg)
    t1 = time.perf_counter()
    L, W, gmua, gmus = rp.loss_and_grads(mesh, cfg, fwd.detp, fwd.seeds, c)
    t2 = time.perf_counter()
    clk = clocks.stop()
    nrep = len(fwd.detp)
    line = {"metric": "replay (backward) photons/ms", "value": 2 * nrep / ((t2 - t1) * 1e3), "unit": "photons/ms",
            "n_gpus": 1, "higher_is_better": True, "workload": "replay-8-detectors",
            "forward_photons_per_ms": cfg.nphoton / ((t1 - t0) * 1e3), "forward_kernel_ms": fwd.kernel_ms,
            "detected": int(fwd.detected), "replayed": nrep, "loss": L,
            "detector_weights": [float(x) for x in W], "backward_s": t2 - t1,
            "grad_mua_norm": float(np.linalg.norm(gmua)), "grad_mus_norm": float(np.linalg.norm(gmus)),
            "data": "synthetic", "clocks": clk,
            "config": {"mesh": "4-layer shells 1.296M tets", "photons": 10_000_000}}
    return line


def run(args):
    line = {"batched": run_batched, "serving": run_serving, "replay": run_replay}[args.workload](args)
    print(json.dumps(line), flush=True)


def summaries(args) -> dict:
    """The three forms in brief, for the default benchmark line: each runs
    its full workload and keeps the figures that compare it with serial
    plain launches (a failure is reported in place of its figures)."""
    keep = {"batched": ("value", "unit", "speedup_vs_serial_plain", "speedup_vs_serial_plain_kernel_only",
                        "serial_plain_photons_per_ms", "scheduled_photons_per_ms", "scheduled_speedup_vs_serial_plain",
                        "photons", "autotune", "clocks"),
            "serving": ("value", "unit", "speedup_vs_serial_plain", "serial_plain_photons_per_ms", "p50_ms", "p99_ms",
                        "serial_p50_ms", "serial_p99_ms", "requests", "waves", "photons", "clocks"),
            "replay": ("value", "unit", "forward_photons_per_ms", "detected", "replayed", "backward_s", "clocks")}
    out = {}
    for name, fn in (("batched", run_batched), ("serving", run_serving), ("replay", run_replay)):
        try:
            line = fn(args)
            out[name] = {"metric": line["metric"], **{k: line[k] for k in keep[name] if k in line}}
        except Exception as e:  # reported, so the benchmark line is still printed
            out[name] = {"error": f"{type(e).__name__}: {e}"}
    return out
