"""The sharded run's GPU path with the default runner: a one-rank NCCL group
on this GPU.  The rank traces its shard in a session, its raw device buffers
are summed and its records gathered with NCCL, and the session's output stage
runs on the combined buffers -- the code a multi-GPU job runs, with one rank.
The result must equal simulate() of the same photons.  (The two-rank
exchange itself is tested with gloo ranks on the CPU, tests/test_distributed.py.)"""
import dataclasses
import socket

import numpy as np
import pytest

from mmc_gb300 import distributed as D
from mmc_gb300 import meshgen
from mmc_gb300.core import Mesh, SimConfig, simulate

pytestmark = pytest.mark.gpu


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


@pytest.fixture(scope="module")
def nccl_group(gpu_ready):
    import torch
    import torch.distributed as dist
    torch.cuda.set_device(0)
    dist.init_process_group("nccl", init_method=f"tcp://127.0.0.1:{_free_port()}", rank=0, world_size=1)
    yield None
    dist.destroy_process_group()


@pytest.mark.parametrize("basisorder,isnormalized", [(0, 0), (1, 1)])
def test_sharded_default_runner_equals_one_simulation(nccl_group, small_inclusion, basisorder, isnormalized):
    m = small_inclusion
    mesh = Mesh(m.node, m.elem, m.label)
    cfg = SimConfig(media=m.media, nphoton=60000, seed=515, srcpos=(30.0, 30.0, 0.0), srcdir=(0.0, 0.0, 1.0),
                    tend=5e-9, tstep=1e-9, issavedet=1, issaveseed=1, detpos=meshgen.c1_detectors(),
                    maxdetphoton=60000, basisorder=basisorder, isnormalized=isnormalized)
    got = D.simulate_sharded(mesh, cfg)
    ref = simulate(mesh, cfg)
    np.testing.assert_allclose(got.field, ref.field, rtol=1e-10, atol=1e-14)
    assert got.normalizer == pytest.approx(ref.normalizer, rel=1e-10)
    assert got.raytet == ref.raytet and got.detected == ref.detected > 0
    assert got.energytot == ref.energytot
    rows = lambda d, s: sorted(map(bytes, np.concatenate([d.view(np.uint8).reshape(len(d), -1), s], 1)))  # noqa: E731
    assert rows(got.detp, got.seeds) == rows(ref.detp, ref.seeds)


def test_sharded_shared_patterns_equal_one_simulation(nccl_group, small_inclusion):
    """Patterns sharing each photon: the per-pattern energy slots are summed with
    the deposits, so every pattern is normalized as in one simulation."""
    m = small_inclusion
    mesh = Mesh(m.node, m.elem, m.label)
    pat = np.random.default_rng(3).uniform(0.1, 1.0, 4 * 3 * 2).astype(np.float32)
    cfg = SimConfig(media=m.media, nphoton=40000, seed=77, srctype="pattern", srcpos=(20.0, 20.0, 0.5),
                    srcdir=(0.0, 0.0, 1.0), srcparam1=(20.0, 0, 0, 4), srcparam2=(0, 20.0, 0, 3), srcpattern=pat,
                    srcnum=2, tend=5e-9, tstep=1e-9, basisorder=1, isnormalized=1)
    got = D.simulate_sharded(mesh, cfg)
    ref = simulate(mesh, cfg)
    assert got.field.shape == ref.field.shape == (5, m.nn, 2)
    np.testing.assert_allclose(got.field, ref.field, rtol=1e-10, atol=1e-14)
    assert got.normalizer == pytest.approx(ref.normalizer, rel=1e-10)
    np.testing.assert_allclose(got.energy_src, ref.energy_src, rtol=1e-12)
