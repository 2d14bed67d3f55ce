"""Multi-rank path on CPU: two gloo ranks each simulate their photon shard
(the CPU oracle stands in for the rank's GPU), then reduce.  The result must
equal one single-process run of all photons: photon streams depend only on
(seed, photon index), so sharding changes nothing but summation order."""
import dataclasses
import os
import socket
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _case():
    from mmc_gb300 import meshgen
    from mmc_gb300.core import SimConfig
    m = meshgen.inclusion_cube(n=8, jitter=0.5, seed=2)
    cfg = SimConfig(media=m.media, nphoton=6001, seed=99, srcpos=(30.0, 30.0, 0.0), tend=5e-9, tstep=1e-9,
                    issavedet=1, issaveseed=1, detpos=np.array([[40, 30, 0, 4], [50, 30, 0, 4]], np.float32),
                    maxdetphoton=10000, basisorder=1, fast_math=0)
    return m, cfg


def _oracle_runner(m):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from mmc_gb300.core import SimResult

    def run(c):
        r = oracle.run(m.node, m.elem, m.label, c, nthreads=2, normalize=False)
        return SimResult(field=r["raw"], detp=r["detp"], seeds=r["seeds"], detected=r["detected"],
                         energytot=float(c.nphoton), energyesc=r["energyesc"], normalizer=1.0, raytet=r["raytet"],
                         aborted=r["aborted"], kernel_ms=0.0, maxgate=c.maxgate, reclen=r["reclen"])
    return run


def _worker(rank, world, port, out):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import torch.distributed as dist
    from mmc_gb300 import distributed as D
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    m, cfg = _case()
    res = D.simulate_sharded(m, cfg, runner=_oracle_runner(m))
    if rank == 0:
        np.savez(out, field=res.field, detp=res.detp, seeds=res.seeds, eesc=res.energyesc, etot=res.energytot,
                 raytet=res.raytet, detected=res.detected, norm=res.normalizer)
    dist.barrier()
    dist.destroy_process_group()


def test_shard_ranges_cover_all_photons():
    from mmc_gb300.distributed import shard
    for n, w in [(10, 3), (7, 8), (1000003, 4)]:
        parts = [shard(n, r, w) for r in range(w)]
        assert sum(c for _, c in parts) == n
        assert all(parts[i][0] + parts[i][1] == parts[i + 1][0] for i in range(w - 1))


def test_two_gloo_ranks_equal_one_run(tmp_path):
    port = _free_port()
    out = str(tmp_path / "r.npz")
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = np.load(out)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    m, cfg = _case()
    ref = oracle.run(m.node, m.elem, m.label, cfg, nthreads=2, normalize=True)
    np.testing.assert_allclose(got["field"], ref["field"], rtol=1e-10)
    assert float(got["norm"]) == pytest.approx(ref["normalizer"], rel=1e-10)
    assert int(got["raytet"]) == ref["raytet"] and int(got["detected"]) == ref["detected"]
    rows = lambda d, s: sorted(map(bytes, np.concatenate([d.view(np.uint8).reshape(len(d), -1), s], 1)))
    assert rows(got["detp"], got["seeds"]) == rows(ref["detp"], ref["seeds"])
