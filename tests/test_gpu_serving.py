"""The continuous-batching server: requests over several resident meshes
arrive while others run, share waves, and each result equals the same request
run alone."""
import dataclasses
import time

import numpy as np
import pytest

from mmc_gb300 import meshgen
from mmc_gb300.core import Mesh, SimConfig, simulate
from mmc_gb300.serving import Request, Server, device_bytes

pytestmark = pytest.mark.gpu


def _requests(meshes, n, seed=0):
    rng = np.random.default_rng(seed)
    reqs = []
    keys = list(meshes)
    for i in range(n):
        key = keys[i % len(keys)]
        base = meshes[key][1]
        media = base.media.copy()
        media[1:, 0] *= np.exp(rng.uniform(-0.5, 0.5, len(media) - 1))
        media[1:, 1] *= rng.uniform(0.7, 1.3, len(media) - 1)
        nph = int(10 ** rng.uniform(3.5, 5.0))
        cfg = SimConfig(media=media, nphoton=nph, seed=1000 + i, srcpos=(30.0, 30.0, 0.0) if key != "shell"
                        else (30.0, 30.0, 5.6), tend=5e-9, tstep=0.5e-9, issavedet=1, issaveseed=1,
                        detpos=np.array([[40, 30, 0, 3], [30, 30, 5, 4]], np.float32), maxdetphoton=20000,
                        basisorder=0, isnormalized=1)
        reqs.append(Request(mesh=key, cfg=cfg))
    return reqs


@pytest.fixture(scope="module")
def meshes(gpu_ready):
    a = meshgen.homogeneous_cube(n=12)
    b = meshgen.inclusion_cube(n=16, jitter=0.5, seed=4)
    c = meshgen.shell_mesh(n=20, jitter=0.5, seed=5)
    return {k: (Mesh(m.node, m.elem, m.label), m) for k, m in (("cube", a), ("incl", b), ("shell", c))}


def _check(reqs, meshes):
    for r in reqs:
        assert r.error is None, r.error
        alone = simulate(meshes[r.mesh][0], r.cfg)
        np.testing.assert_allclose(r.result.field, alone.field, rtol=1e-9, atol=1e-12)
        assert r.result.raytet == alone.raytet and r.result.detected == alone.detected


def test_requests_arriving_during_service_match_solo_runs(meshes):
    srv = Server({k: v[0] for k, v in meshes.items()}, wave_photons=60000, min_share=5000)
    reqs = _requests(meshes, 12)
    t0 = time.perf_counter()
    for i, r in enumerate(reqs):  # staggered arrivals: later ones join while earlier ones run
        r.arrival = t0 + 0.01 * i
    done = srv.run(arrivals=reqs, deadline=t0 + 300)
    assert len(done) == len(reqs)
    assert srv.waves > 3
    _check(reqs, meshes)
    st = srv.stats()
    assert st["p99_ms"] >= st["p50_ms"] > 0


def test_memory_admission_queues_requests(meshes):
    reqs = _requests(meshes, 6, seed=1)
    need = max(device_bytes(meshes[r.mesh][0], r.cfg) for r in reqs)
    srv = Server({k: v[0] for k, v in meshes.items()}, wave_photons=30000, memory_budget=int(need * 2.5))
    for r in reqs:
        srv.submit(r)
    seen = 0
    while srv.step() or srv._finishing:
        seen = max(seen, len(srv.active))
        assert srv.in_use <= srv.budget
        srv._reap(block=not srv.active)
    assert seen <= 2
    assert len(srv.completed) == len(reqs)
    _check(reqs, meshes)
