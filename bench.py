"""Benchmark: photons/ms of per-photon tetrahedral tracing on the 1.296M-tet
heterogeneous cube (60^3 voxels at 1 mm, 6 tets/voxel, orientation-safe
+/-0.25 mm node jitter, r=10 mm inclusion; pencil source (30,30,0) +z; 50 gates
of 0.1 ns; 4 detectors R=2 mm saving per-medium partial paths and scatter
counts; 1e8 photons per job).

A step is the whole 1e8-photon job with the mesh and all buffers resident on
the GPU (each step traces a new photon range of the same seed), traced
gate-phased: one persistent launch per window of time gates, photons parked
between windows.  L2 is flushed (256 MB write) before every timed step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

BYTES_PER_STEP = 92  # 64 B face planes + 16 B neighbour ids + 4 B label + 8 B fluence RMW per ray-tet test
PHOTONS_PER_STEP = 100_000_000
JOB_PHOTONS = 100_000_000
WORKLOAD = "inclusion-cube-1.3M-tets"


def workload_config(nphoton):
    from mmc_gb300 import meshgen
    from mmc_gb300.core import SimConfig
    m = meshgen.inclusion_cube(n=60, jitter=0.25, seed=12345)
    cfg = SimConfig(media=m.media, nphoton=nphoton, seed=1648335518, srcpos=(30.0, 30.0, 0.0),
                    srcdir=(0.0, 0.0, 1.0), tstart=0.0, tend=5e-9, tstep=1e-10, issavedet=1,
                    detpos=meshgen.c1_detectors(), maxdetphoton=2_000_000, basisorder=0, isnormalized=1)
    return m, cfg


# Port-to-reference speed factor of the CPU baseline: the oracle's photon loop
# ran at 0.821x the reference CPU engine's own printed speed (the reference's
# sources built as its `make sse` target does, oracle/build_ref.sh) on the same
# 1.296M-tet workload, 8 threads of an x86 Xeon @ 2.70 GHz, 1e6 and 2e6 photons
# (88.9/86.7 vs 73.0/71.2 photons/ms); 0.731x on one thread (12.45 vs 9.10).
# The reference engine is SSE4 code and does not build on the Arm host of the
# GPU, so the factor is measured on the x86 build host and reported beside the
# port's speed: ratio against the reference engine = ratio against the port x 0.821.
PORT_VS_REFERENCE = {"factor": 0.821, "threads": 8, "host": "x86 Xeon @ 2.70 GHz",
                     "measured": "oracle photon loop 73.0/71.2 vs reference mmc -G -1 -M s -C 0 88.9/86.7 photons/ms, "
                                 "1e6/2e6 photons of this workload"}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic(key="dram_bytes_per_photon"):
    """Bytes per photon of the engine's launches (all gate windows of a step)
    from the committed ncu summary, measured on a 5e6-photon step: DRAM
    (dram_bytes_per_photon) or L2 (l2_bytes_per_photon, lts__t_bytes)."""
    path = os.path.join(ROOT, "profiles", "photon_engine_phased_inclusion_cube.md")
    try:
        for line in open(path):
            if line.startswith(key + ":"):
                return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


def l2_peak(device):
    """This GPU's L2 read bandwidth, measured now (mmcgb_l2_read_bandwidth:
    64 MiB resident buffer, 20 sweeps of 16-byte L1-bypassing loads)."""
    import ctypes as C
    from mmc_gb300 import _native
    g = C.c_double()
    rc = _native.load().mmcgb_l2_read_bandwidth(int(device), 64 << 20, 20, C.byref(g))
    return g.value if rc == 0 else None


def cpu_baseline(m, cfg, target_s=12.0):
    """The CPU oracle (C restatement of the path) on all host cores, on a
    bounded sample of the same workload."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    import dataclasses
    cores = os.cpu_count() or 1
    n = 20000
    while True:
        c = dataclasses.replace(cfg, nphoton=n, maxdetphoton=max(1000, n))
        dt = oracle.run(m.node, m.elem, m.label, c, nthreads=cores, normalize=False)["sim_seconds"]
        if dt >= target_s * 0.5 or n >= 5_000_000:
            return {"value": n / (dt * 1e3), "unit": "photons/ms", "cores": cores, "kind": "port",
                    "sample": f"{n} photons of the {JOB_PHOTONS:.0e}-photon job, {dt:.1f} s of photon loop "
                              f"on {cores} threads (mesh preparation excluded, as the reference times "
                              f"its speed)",
                    "port_vs_reference": PORT_VS_REFERENCE}
        n = int(n * min(10.0, max(1.5, target_s / max(dt, 1e-3))))


def run_reference(args, rank, world):
    if rank != 0:
        return
    m, cfg = workload_config(PHOTONS_PER_STEP)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    import dataclasses
    cores = os.cpu_count() or 1
    # size one step to a few seconds of photon loop; each step times the photon loop alone, as the
    # reference times the speed it reports (mesh preparation and output stage excluded)
    n = 20000
    c = dataclasses.replace(cfg, nphoton=n, maxdetphoton=n)
    dt = oracle.run(m.node, m.elem, m.label, c, nthreads=cores, normalize=False)["sim_seconds"]
    n = max(20000, int(n * 4.0 / max(dt, 1e-3)))
    c = dataclasses.replace(cfg, nphoton=n, maxdetphoton=n)
    for _ in range(args.warmup):
        oracle.run(m.node, m.elem, m.label, dataclasses.replace(c, nphoton=2000, maxdetphoton=2000),
                   nthreads=cores, normalize=False)
    times = []
    for k in range(args.steps):
        ck = dataclasses.replace(c, photon_offset=k * n)
        times.append(oracle.run(m.node, m.elem, m.label, ck, nthreads=cores, normalize=False)["sim_seconds"])
    total = sum(times)
    value = n * args.steps / (total * 1e3)
    line = {"impl": "reference", "metric": "photons/ms", "value": value, "unit": "photons/ms", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "photons_per_step": n, "gates": 50, "detectors": 4,
                       "note": "CPU restatement of the reference algorithm (reference C sources are not on the box); "
                               "photon loop timed, as the reference times its reported speed"},
            "cpu_baseline": {"value": value, "unit": "photons/ms", "cores": cores, "kind": "port",
                             "sample": f"{n} photons per step x {args.steps} steps on {cores} threads, "
                                       f"photon loop only", "port_vs_reference": PORT_VS_REFERENCE},
            "e2e": {"value": value, "unit": "photons/ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--photons-per-step", type=int, default=PHOTONS_PER_STEP)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--exact", action="store_true",
                    help="IEEE arithmetic (photon-for-photon reproducible on the CPU) instead of fast math")
    ap.add_argument("--workload", default="plain", choices=["plain", "batched", "serving", "replay"],
                    help="plain: the 1.3M-tet benchmark (default); batched / serving / replay: the batched, "
                         "continuous-batching and differentiation workloads (one JSON line each)")
    ap.add_argument("--requests", type=int, default=64, help="serving: number of requests")
    ap.add_argument("--no-forms", action="store_true",
                    help="plain runs: leave out the batched / serving / replay summaries (run at N=1 after the "
                         "timed steps, under 'forms')")
    args = ap.parse_args()
    if args.workload != "plain":
        from mmc_gb300 import workloads
        return workloads.run(args)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        import torch
        backend = "nccl" if args.impl == "ours" else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local_rank)
        dist.init_process_group(backend=backend)

    if args.impl == "reference":
        run_reference(args, rank, world)
        if dist is not None:
            dist.destroy_process_group()
        return

    import torch
    from mmc_gb300.core import Mesh, Session, simulate
    import dataclasses

    torch.cuda.set_device(local_rank)
    nps = args.photons_per_step
    m, cfg = workload_config(nps)
    cfg = dataclasses.replace(cfg, fast_math=0 if args.exact else 1)
    mesh = Mesh(m.node, m.elem, m.label, device=local_rank)
    ne, nn = mesh.ne, mesh.nn
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{local_rank}")

    def barrier():
        if dist is not None:
            dist.barrier()

    # ---- device-resident throughput (value) ----
    # rank r simulates photons [r*K*nps, (r+1)*K*nps) of the job: no data-path collective
    sess = Session(mesh, dataclasses.replace(cfg, photon_offset=rank * (args.steps + args.warmup) * nps))
    window = sess.phase_window(nps)
    # every step saves its own detected photons, as a fresh job would: the record count is reset
    # before each launch (outside the timed region), so no step finds the record buffer full
    detcount = sess.device_buffers()["detcount"]
    if detcount is None:
        detcount = torch.zeros(1, device=f"cuda:{local_rank}")  # no records saved: nothing to reset
    for w in range(args.warmup):
        detcount.zero_()
        torch.cuda.synchronize()
        sess.launch(w * nps, nps)
        sess.sync()
    from mmc_gb300.clocks import ClockSampler
    sampler = ClockSampler(local_rank)
    barrier()
    torch.cuda.synchronize()
    sampler.start()
    kernel_ms = []
    raytet0 = None
    t_wall = time.perf_counter()
    for k in range(args.steps):
        flush.zero_()
        detcount.zero_()
        torch.cuda.synchronize()
        sess.launch((args.warmup + k) * nps, nps)
        kernel_ms.append(sess.sync())
    torch.cuda.synchronize()
    barrier()
    wall = time.perf_counter() - t_wall
    clocks = sampler.stop()
    res = sess.end(collect=True)
    total_ms = float(sum(kernel_ms))
    if dist is not None:
        t = torch.tensor([total_ms], dtype=torch.float64, device=f"cuda:{local_rank}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    photons_all = nps * args.steps * world
    value = photons_all / total_ms
    steps_per_photon = res.raytet / ((args.warmup + args.steps) * nps)
    raytet_per_launch = steps_per_photon * nps
    avg_ms = float(np.mean(kernel_ms))
    # engine launches per step: one per window of gates (the library's automatic window)
    span = window
    launches_per_step = -(-cfg.maxgate // span) if span > 0 else 1
    # all of the library's kernels in a step: the engine launches, the two kernels that order the
    # parked photons between windows, and the fold of the replicated near-source cells
    kernels_per_step = launches_per_step + 2 * (launches_per_step - 1) + 1
    achieved = raytet_per_launch * BYTES_PER_STEP / (avg_ms * 1e-3) / 1e9
    peak, peak_kind = peaks()
    tpp = profiled_traffic()

    # ---- end to end through the public API with host buffers ----
    # N = 1: simulate() on the resident mesh.  N > 1: simulate_sharded(), the call a sharded job
    # makes: each rank traces its shard, the raw device buffers are summed and the records
    # gathered with NCCL, then one output stage and one copy of the final field to the host.
    e2e = None
    e2e_dropin = None
    if not args.no_e2e:
        from mmc_gb300.core import pinned_empty
        ecfg = dataclasses.replace(cfg, photon_offset=10 ** 12)
        out = pinned_empty((ecfg.maxgate, mesh.ne))  # the application's host buffer, reused every step
        # one untimed full-size call: the device pool grows to the run's buffers (the gate-phasing
        # queues of 1e8 photons) once per process, as in any application that calls repeatedly
        simulate(mesh, dataclasses.replace(ecfg, photon_offset=ecfg.photon_offset - nps), out=out)
        esteps = max(1, min(args.steps, 3))
        if dist is not None:
            from mmc_gb300.distributed import simulate_sharded
            job = dataclasses.replace(ecfg, nphoton=nps * world)  # per-rank work fixed: weak scaling
            simulate_sharded(mesh, dataclasses.replace(job, photon_offset=job.photon_offset - nps * world))
        barrier()
        t0 = time.perf_counter()
        d2h = 0
        for k in range(esteps):
            if dist is None:
                r = simulate(mesh, dataclasses.replace(ecfg, photon_offset=ecfg.photon_offset + k * nps), out=out)
            else:
                r = simulate_sharded(mesh, dataclasses.replace(job, photon_offset=job.photon_offset + k * nps * world))
            d2h = r.field.nbytes + (r.detp.nbytes if r.detp is not None else 0) + 64
        barrier()
        et = time.perf_counter() - t0
        if dist is not None:
            t = torch.tensor([et], dtype=torch.float64, device=f"cuda:{local_rank}")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            et = float(t.item())
        h2d = cfg.media.nbytes + cfg.detpos.nbytes + 200
        e2e = {"value": nps * esteps * world / (et * 1e3), "unit": "photons/ms", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "steps": esteps,
               "path": "simulate() on the resident mesh" if dist is None else
                       "simulate_sharded(): per-rank shard, NCCL sum of deposits and gather of records, "
                       "one output stage"}
        if dist is None:
            # the drop-in path as the reference runs it: mmcgb_run (mmc_run_cu's counterpart)
            # prepares and uploads the mesh, simulates, normalizes and frees, every call
            from mmc_gb300 import core
            dsteps = 2
            core.run(m.node, m.elem, m.label, dataclasses.replace(ecfg, photon_offset=ecfg.photon_offset - nps),
                     out=out)
            t0 = time.perf_counter()
            for k in range(dsteps):
                core.run(m.node, m.elem, m.label,
                         dataclasses.replace(ecfg, photon_offset=ecfg.photon_offset + (esteps + k) * nps), out=out)
            dt = time.perf_counter() - t0
            mesh_bytes = m.node.nbytes + m.elem.nbytes + m.label.nbytes
            e2e_dropin = {"value": nps * dsteps / (dt * 1e3), "unit": "photons/ms",
                          "h2d_bytes_per_step": int(h2d + mesh_bytes), "d2h_bytes_per_step": int(d2h),
                          "steps": dsteps,
                          "path": "mmcgb_run through the C ABI: host mesh prepared, uploaded and freed per call"}

    # ---- the level the gathers are served from: L2 traffic against the measured L2 bandwidth ----
    l2 = None
    l2pp = profiled_traffic("l2_bytes_per_photon")
    l2bw = l2_peak(local_rank)
    if l2bw and not l2pp:
        l2 = {"peak": l2bw, "unit": "GB/s", "peak_kind": "measured now (mmcgb_l2_read_bandwidth)"}
    if l2pp and l2bw:
        l2_ach = l2pp * nps / (avg_ms * 1e-3) / 1e9
        l2 = {"achieved": l2_ach, "peak": l2bw, "unit": "GB/s", "frac": l2_ach / l2bw,
              "peak_kind": "measured now (mmcgb_l2_read_bandwidth)",
              "traffic_bytes_per_photon": l2pp,
              "note": "lts__t_bytes of the engine's launches per photon (ncu, 5e6-photon step) x photons / step time"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(m, cfg)

    # ---- the batched, serving and differentiation forms (N = 1, after everything timed above) ----
    forms = None
    if world == 1 and not args.no_forms:
        mesh = flush = out = None  # free the benchmark's device memory first
        torch.cuda.empty_cache()
        from mmc_gb300 import workloads
        forms = workloads.summaries(args)

    if rank == 0:
        line = {
            "metric": "photons/ms", "value": value, "unit": "photons/ms", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (f64 fluence accumulation, %s)" % ("IEEE" if args.exact else "fast math"),
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "ne": ne, "nn": nn, "photons_per_step": nps,
                       "job_photons": JOB_PHOTONS, "gates": 50, "detectors": 4, "savedet": True,
                       "l2": "flushed (256 MB write) before each timed step",
                       "tracing": f"gate-phased, automatic window of {window} gates (the live gate planes "
                                  "fill ~70% of L2; parked photons resumed in spatial order)" if window else
                                  "one launch per step",
                       "steps_per_photon": steps_per_photon, "detected_per_step": res.detected,
                       "absorbed_fraction": res.absorbed_fraction, "wall_s": wall},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind,
                         "traffic": (tpp * nps) if tpp else None,
                         "bytes_per_test": BYTES_PER_STEP, "tests_per_launch": raytet_per_launch,
                         "avg_launch_ms": avg_ms, "launches_per_step": launches_per_step,
                         "note": "per step: the step's phased launches together"},
            "l2_roofline": l2,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "e2e_dropin": e2e_dropin,
            "gpu_launches": args.steps * kernels_per_step,
            "clocks": clocks,
            "forms": forms,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
