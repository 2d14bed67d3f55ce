"""Size-independent properties of the CUDA engine on the full 1.296M-tet
inclusion cube (the benchmark mesh), where the oracle would take too long,
plus edge cases of the interface."""
import dataclasses

import numpy as np
import pytest

from mmc_gb300 import _native, meshgen
from mmc_gb300.core import Mesh, Session, SimConfig, simulate

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def full_mesh(gpu_ready):
    m = meshgen.inclusion_cube(n=60, jitter=0.25, seed=12345)
    return m, Mesh(m.node, m.elem, m.label)


def _cfg(m, **kw):
    base = dict(media=m.media, nphoton=1_000_000, seed=1648335518, srcpos=(30.0, 30.0, 0.0),
                srcdir=(0.0, 0.0, 1.0), tend=5e-9, tstep=1e-10, issavedet=1, issaveseed=1,
                detpos=meshgen.c1_detectors(), maxdetphoton=200000, basisorder=0, isnormalized=0)
    base.update(kw)
    return SimConfig(**base)


def test_energy_conservation_full_size(full_mesh):
    """Deposited (sum of (w0-w1) over elements) + escaped weight = launched
    weight; roulette is off with 50 gates, so the balance is exact up to
    rounding."""
    m, mesh = full_mesh
    r = simulate(mesh, _cfg(m))
    mua = m.media[m.label, 0].astype(np.float64)
    deposited = float((r.field.sum(0) * mua).sum())
    assert r.aborted == 0
    assert abs(deposited + r.energyesc - r.energytot) < 1e-5 * r.energytot
    assert 600 < r.raytet / 1e6 < 660  # ray-tet tests per photon on this mesh


def test_sharded_launches_add_up_to_one_launch(full_mesh):
    """Photon streams depend only on (seed, photon index): two half launches
    accumulate exactly the deposits and records of one full launch."""
    m, mesh = full_mesh
    cfg = _cfg(m, nphoton=400_000)
    full = simulate(mesh, cfg)
    s = Session(mesh, cfg)
    s.launch(0, 200_000)
    s.launch(200_000, 200_000)
    s.sync()
    split = s.end()
    np.testing.assert_allclose(split.field, full.field, rtol=1e-9, atol=1e-12)
    assert split.raytet == full.raytet and split.detected == full.detected
    rows = lambda d, sd: sorted(map(bytes, np.concatenate([d.view(np.uint8).reshape(len(d), -1), sd], 1)))
    assert rows(split.detp, split.seeds) == rows(full.detp, full.seeds)
    # escaped weight is summed per lane in float32 before the float64 total: grouping-dependent at ~1e-10
    assert split.energyesc == pytest.approx(full.energyesc, rel=1e-9)


def test_detector_saturation_reports_all_detections(full_mesh):
    m, mesh = full_mesh
    r = simulate(mesh, _cfg(m, nphoton=200_000, maxdetphoton=100))
    assert r.detected > 100 and r.detp.shape[0] == 100


def test_zero_photons(full_mesh):
    m, mesh = full_mesh
    r = simulate(mesh, _cfg(m, nphoton=0))
    assert r.raytet == 0 and r.detected == 0 and not r.field.any()


def test_bad_meshes_are_rejected(gpu_ready):
    m = meshgen.homogeneous_cube(n=2)
    elem = m.elem.copy()
    elem[0, 0] = m.nn + 5
    with pytest.raises(_native.MmcgbError) as e:
        Mesh(m.node, elem, m.label)
    assert e.value.code == 3
    lab = m.label.copy()
    lab[0] = 300
    with pytest.raises(_native.MmcgbError) as e:
        Mesh(m.node, m.elem, lab)
    assert e.value.code == 3


def test_phased_launch_split_by_queue_memory(full_mesh):
    """A gate-phased launch whose parked-photon queues would not fit is traced as
    several phased launches over consecutive photon ranges (mmcgb_config.phase_chunk
    forces the split here): the same photons, the same results."""
    m, mesh = full_mesh
    cfg = _cfg(m, nphoton=3_000_000, phased=8, issaveseed=1)
    s = Session(mesh, cfg)
    try:
        assert s.phase_plan(cfg.nphoton) == (8, 3_000_000)
    finally:
        s.end(collect=False)
    one = simulate(mesh, cfg)
    split_cfg = dataclasses.replace(cfg, phase_chunk=1_100_000)
    s = Session(mesh, split_cfg)
    try:
        assert s.phase_plan(cfg.nphoton) == (8, 1_000_000)  # three equal launches
    finally:
        s.end(collect=False)
    split = simulate(mesh, split_cfg)
    np.testing.assert_allclose(split.field, one.field, rtol=1e-9, atol=1e-12)
    assert split.raytet == one.raytet and split.detected == one.detected
    rows = lambda d, sd: sorted(map(bytes, np.concatenate([d.view(np.uint8).reshape(len(d), -1), sd], 1)))  # noqa: E731
    assert rows(split.detp, split.seeds) == rows(one.detp, one.seeds)


def test_automatic_phasing_plan_of_the_benchmark_job(full_mesh):
    """The benchmark job (1e8 photons, 50 gates, float64) is traced gate-phased
    in one set of window launches when its queues fit; automatic phasing keeps
    at least 4e6 photons per launch and otherwise runs unphased."""
    m, mesh = full_mesh
    cfg = _cfg(m, nphoton=100_000_000, issaveseed=0, maxdetphoton=2_000_000)
    s = Session(mesh, cfg)
    try:
        w, chunk = s.phase_plan(100_000_000)
        assert 1 <= w < 50 and chunk == 100_000_000
        assert s.phase_plan(3_000_000) == (0, 0)  # too few photons to phase
        s2 = Session(mesh, dataclasses.replace(cfg, phase_chunk=30_000_000))
        try:
            assert s2.phase_plan(100_000_000) == (w, 25_000_000)
            assert s2.phase_plan(10_000_000) == (w, 10_000_000)
        finally:
            s2.end(collect=False)
        s3 = Session(mesh, dataclasses.replace(cfg, phase_chunk=3_000_000))
        try:
            assert s3.phase_plan(100_000_000) == (0, 0)  # launches below 4e6 photons run unphased
        finally:
            s3.end(collect=False)
    finally:
        s.end(collect=False)
