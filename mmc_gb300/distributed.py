"""Multi-GPU runs: photon sharding with one reduction at the end.

Photons are independent and each photon's random stream depends only on
(seed, photon index), so rank r of N simply simulates its contiguous photon
range with its own resident copy of the mesh -- no communication while
tracing.  The one exchange step follows the reference's multi-device host
code (src/mmc_cu_host.cu:403-429 splits photons by workload, :772-783 and
:916-921 sum the fields and append the detected records): a sum all-reduce of
the raw element deposits (float64), the escaped/launched weights and the
counters, and an all-gather of the detected-photon records and seeds.  The
normalization runs once on the global totals (it is not linear in the
per-rank results).

With the NCCL backend and the default runner the exchange stays on the GPUs:
each rank traces its shard in a session, the session's raw device buffers
(deposits, energies, counters) are summed in place with NCCL and the detected
records gathered with NCCL, and only then does the session's output stage run
on the device and copy the final field to the host once.  A custom runner (the
CPU oracle in the gloo tests) goes through the host: its result is summed and
gathered with the group's backend, then normalized on the host.
"""
from __future__ import annotations

import dataclasses
from typing import Callable, Optional

import numpy as np

from .core import Mesh, Session, SimConfig, SimResult, normalize_host, simulate


def shard(nphoton: int, rank: int, world: int):
    """(offset, count) of rank's contiguous photon range."""
    base, extra = divmod(int(nphoton), int(world))
    count = base + (1 if rank < extra else 0)
    offset = rank * base + min(rank, extra)
    return offset, count


def _dist():
    import torch.distributed as dist
    return dist


def _device(group):
    import torch
    dist = _dist()
    backend = dist.get_backend(group)
    if backend == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def reduce_results(local: SimResult, group=None) -> SimResult:
    """Sums raw deposits, energies and counters over the ranks and gathers the
    detected records (in rank order).  Every rank receives the totals."""
    import torch
    dist = _dist()
    dev = _device(group)
    world = dist.get_world_size(group)
    field = torch.from_numpy(np.ascontiguousarray(local.field)).to(dev)
    dist.all_reduce(field, op=dist.ReduceOp.SUM, group=group)
    scal = torch.tensor([local.energytot, local.energyesc], dtype=torch.float64, device=dev)
    dist.all_reduce(scal, op=dist.ReduceOp.SUM, group=group)
    cnt = torch.tensor([local.raytet, local.aborted, local.detected], dtype=torch.int64, device=dev)
    dist.all_reduce(cnt, op=dist.ReduceOp.SUM, group=group)
    detp, seeds = local.detp, local.seeds
    if detp is not None:
        n = torch.tensor([detp.shape[0]], dtype=torch.int64, device=dev)
        sizes = [torch.zeros_like(n) for _ in range(world)]
        dist.all_gather(sizes, n, group=group)
        sizes = [int(x.item()) for x in sizes]
        width = detp.shape[1] * 4 + (16 if seeds is not None else 0)
        rows = np.zeros((max(sizes) if sizes else 0, width), np.uint8)
        local_rows = detp.view(np.uint8).reshape(detp.shape[0], -1)
        if seeds is not None:
            local_rows = np.concatenate([local_rows, seeds], axis=1)
        rows[:detp.shape[0]] = local_rows
        t = torch.from_numpy(rows).to(dev)
        parts = [torch.zeros_like(t) for _ in range(world)]
        dist.all_gather(parts, t, group=group)
        allrows = np.concatenate([p.cpu().numpy()[:s] for p, s in zip(parts, sizes)], axis=0)
        ncol = detp.shape[1]
        detp = np.ascontiguousarray(allrows[:, :ncol * 4]).view(np.float32).reshape(-1, ncol)
        seeds = np.ascontiguousarray(allrows[:, ncol * 4:]) if seeds is not None else None
    sc = scal.cpu().numpy()
    cn = cnt.cpu().numpy()
    return dataclasses.replace(local, field=field.cpu().numpy(), energytot=float(sc[0]), energyesc=float(sc[1]),
                               raytet=int(cn[0]), aborted=int(cn[1]), detected=int(cn[2]), detp=detp, seeds=seeds)


def _gather_rows(t, nrows, width, group):
    """All-gathers the first nrows rows (width elements each) of the flat
    device tensor t from every rank; returns (rows of all ranks in rank
    order, as a host array)."""
    import torch
    dist = _dist()
    world = dist.get_world_size(group)
    n = torch.tensor([nrows], dtype=torch.int64, device=t.device)
    sizes = [torch.zeros_like(n) for _ in range(world)]
    dist.all_gather(sizes, n, group=group)
    sizes = [int(x.item()) for x in sizes]
    pad = torch.zeros((max(max(sizes), 1), width), dtype=t.dtype, device=t.device)
    if nrows:
        pad[:nrows] = t[:nrows * width].view(nrows, width)
    parts = [torch.empty_like(pad) for _ in range(world)]
    dist.all_gather(parts, pad, group=group)
    return torch.cat([p[:k] for p, k in zip(parts, sizes)]).cpu().numpy()


def _simulate_sharded_on_device(mesh: Mesh, cfg: SimConfig, off: int, n: int, group) -> SimResult:
    """The rank's shard in a session; the raw device buffers are combined with
    NCCL before the output stage (src/mmc_cu_host.cu:772-783, :916-921)."""
    import torch
    dist = _dist()
    local_cfg = dataclasses.replace(cfg, photon_offset=cfg.photon_offset + off, nphoton=n, accum_f64=1)
    sess = Session(mesh, local_cfg)
    try:
        if n:
            sess.launch(0, n)
        sess.sync()
        b = sess.device_buffers()
        saved = 0
        if b["detcount"] is not None:
            saved = min(int(b["detcount"].item()), int(cfg.maxdetphoton))
        for key in ("field", "energy", "energy_src", "counters", "detcount"):
            if b[key] is not None:
                dist.all_reduce(b[key], op=dist.ReduceOp.SUM, group=group)
        detp = seeds = None
        if b["detp"] is not None:
            reclen = b["reclen"]
            detp = _gather_rows(b["detp"], saved, reclen, group).reshape(-1, reclen)
            if b["seeds"] is not None:
                seeds = _gather_rows(b["seeds"], saved, 16, group).reshape(-1, 16)
        torch.cuda.synchronize(mesh.device)  # the collectives ran on NCCL's stream
        res = sess.end(collect=True, records=False)
    finally:
        if getattr(sess, "_h", None) is not None:
            sess.end(collect=False)
    return dataclasses.replace(res, detp=detp, seeds=seeds)


def simulate_sharded(mesh: Mesh, cfg: SimConfig, group=None,
                     runner: Optional[Callable[[SimConfig], SimResult]] = None) -> SimResult:
    """One simulation split over the ranks of `group`.  Default: the rank's GPU
    traces its shard and, with NCCL, the ranks combine their device buffers
    before the output stage (`mesh` a resident Mesh; the shards accumulate in
    float64 there whatever cfg.accum_f64 says, since the float32 scheme's
    two buffers are not summed across ranks).  `runner` replaces the
    rank's simulation (it returns raw element deposits, e.g. the CPU oracle);
    its result is combined on the host (`mesh` needs node/elem/label)."""
    dist = _dist()
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    off, n = shard(cfg.nphoton, rank, world)
    if runner is None and dist.get_backend(group) == "nccl":
        return _simulate_sharded_on_device(mesh, cfg, off, n, group)
    if int(cfg.srcnum) > 1:
        raise ValueError("a simulation whose patterns share photons (srcnum > 1) is combined on the GPUs (NCCL) only")
    local_cfg = dataclasses.replace(cfg, photon_offset=cfg.photon_offset + off, nphoton=n, isnormalized=0,
                                    basisorder=0, save_field=True)
    run = runner or (lambda c: simulate(mesh, c))
    total = reduce_results(run(local_cfg), group)
    field, norm = normalize_host(mesh.node, mesh.elem, mesh.label, cfg, total.field, total.energytot,
                                 total.energyesc)
    return dataclasses.replace(total, field=field, normalizer=norm)
