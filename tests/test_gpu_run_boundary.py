"""mmcgb_run, the one-shot counterpart of the reference's mmc_run_cu
(src/mmc_cu_host.h:56), through the C ABI: it equals mmcgb_simulate on a
resident mesh, and with `accumulate` it adds into the caller's field and
exiting-weight arrays and normalizes the sum in place, as mmc_run_cu does to
cfg->exportfield and mesh->dref (src/mmc_cu_host.cu:916-982, :984-1061)."""
import dataclasses

import numpy as np
import pytest

from mmc_gb300 import core, meshgen
from mmc_gb300.core import Mesh, SimConfig, simulate

pytestmark = pytest.mark.gpu


def _rows(r):
    return sorted(map(bytes, np.concatenate([r.detp.view(np.uint8).reshape(len(r.detp), -1), r.seeds], 1)))


@pytest.fixture(scope="module")
def case(gpu_ready, small_inclusion):
    m = small_inclusion
    cfg = SimConfig(media=m.media, nphoton=40000, seed=4711, srcpos=(30.0, 30.0, 0.0), srcdir=(0.0, 0.0, 1.0),
                    tend=5e-9, tstep=1e-9, issavedet=1, issaveseed=1, detpos=meshgen.c1_detectors(),
                    maxdetphoton=40000, basisorder=0, isnormalized=0, fast_math=0)
    return m, Mesh(m.node, m.elem, m.label), cfg


def test_run_equals_simulate_on_a_resident_mesh(case):
    m, mesh, cfg = case
    for bo, norm in ((0, 0), (1, 1)):
        c = dataclasses.replace(cfg, basisorder=bo, isnormalized=norm)
        a = core.run(m.node, m.elem, m.label, c)
        b = simulate(mesh, c)
        assert a.raytet == b.raytet and a.detected == b.detected > 0
        assert _rows(a) == _rows(b)
        # float64 atomics: only the summation order differs
        np.testing.assert_allclose(a.field, b.field, rtol=1e-12, atol=0)
        assert a.energyesc == pytest.approx(b.energyesc, rel=1e-12)
        assert a.normalizer == pytest.approx(b.normalizer, rel=1e-12)


def test_run_accumulates_into_the_callers_field(case):
    m, mesh, cfg = case
    rng = np.random.default_rng(3)
    G = cfg.maxgate
    # element output, raw: field = previous + this run
    prev = rng.random((G, m.ne)) * 10.0
    out = prev.copy()
    core.run(m.node, m.elem, m.label, dataclasses.replace(cfg, accumulate=1), out=out)
    raw = simulate(mesh, cfg).field
    np.testing.assert_allclose(out, prev + raw, rtol=1e-12, atol=1e-12)
    # node output, raw: the run's deposits are scattered to the nodes and added
    c1 = dataclasses.replace(cfg, basisorder=1)
    prevn = rng.random((G, m.nn))
    outn = prevn.copy()
    core.run(m.node, m.elem, m.label, dataclasses.replace(c1, accumulate=1), out=outn)
    np.testing.assert_allclose(outn, prevn + simulate(mesh, c1).field, rtol=1e-12, atol=1e-12)
    # normalized: the sum is normalized in place with this run's energies
    cn = dataclasses.replace(cfg, isnormalized=1)
    out = prev.copy()
    r = core.run(m.node, m.elem, m.label, dataclasses.replace(cn, accumulate=1), out=out)
    want, norm = core.normalize_host(m.node, m.elem, m.label, cn, prev + raw, r.energytot, r.energyesc)
    np.testing.assert_allclose(out, want, rtol=1e-10)
    assert r.normalizer == pytest.approx(norm, rel=1e-10)


def test_two_accumulating_runs_equal_one_run(case):
    """The respin pattern of mmc_run_cu: runs over consecutive photon ranges
    accumulating into one field give the field of a single run."""
    m, mesh, cfg = case
    out = np.zeros((cfg.maxgate, m.ne))
    half = cfg.nphoton // 2
    for k in range(2):
        core.run(m.node, m.elem, m.label,
                 dataclasses.replace(cfg, accumulate=1, nphoton=half, photon_offset=k * half), out=out)
    np.testing.assert_allclose(out, simulate(mesh, cfg).field, rtol=1e-10, atol=1e-12)


def test_run_accumulates_exiting_weight(case):
    m, mesh, cfg = case
    c = dataclasses.replace(cfg, issaveref=1, issavedet=0, issaveseed=0)
    nf = core.prepare_host(m.node, m.elem, m.label)["nf"]
    prev = np.random.default_rng(5).random((c.maxgate, nf))
    dref = prev.copy()
    core.run(m.node, m.elem, m.label, dataclasses.replace(c, accumulate=1), dref=dref)
    np.testing.assert_allclose(dref, prev + simulate(mesh, c).dref, rtol=1e-12, atol=1e-12)
