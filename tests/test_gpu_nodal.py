"""Per-node absorption and scattering on the GPU (the reference's
DOT-reconstruction mode, src/mmc_core.cl:785-793).

* photon by photon against the CPU oracle (IEEE arithmetic), for element and
  dual-grid output and a wp replay;
* with the benchmark's fast arithmetic, a nodal run equals the run labelled
  by its element means (the identity the oracle is pinned through), and its
  plain, gate-phased and batched launches agree;
* through pmmc's nodemua/nodemusp keys.
"""
import dataclasses

import numpy as np
import pytest

from mmc_gb300 import pmmc
from mmc_gb300.core import Mesh, SimConfig, simulate, simulate_batch
from test_oracle_nodal import _cfg, labelled_by_means, nodal_fields, prepared_cube

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cube(gpu_ready):
    m = prepared_cube(n=12)
    rng = np.random.default_rng(5)
    mua = rng.uniform(0.002, 0.05, len(m.node)).astype(np.float32)
    mus = rng.uniform(0.5, 2.0, len(m.node)).astype(np.float32)
    return m, Mesh(m.node, m.elem, m.label), mua, mus


def _rows(detp):
    return sorted(map(bytes, detp.view(np.uint8).reshape(len(detp), -1)))


@pytest.mark.parametrize("method", ["elem", "grid"])
def test_nodal_run_matches_oracle_photon_by_photon(oracle_mod, cube, method):
    m, mesh, mua, mus = cube
    cfg = _cfg(m.media, nphoton=4000, nodemua=mua, nodemusp=mus, method=method, gridstep=2.0, issaveseed=1)
    g = simulate(mesh, cfg, trace=True)
    o = oracle_mod.run(m.node, m.elem, m.label, cfg, nthreads=4, trace=True, normalize=False)
    assert np.array_equal(g.photon_weight.view(np.uint32), o["photon_weight"].view(np.uint32))
    assert np.array_equal(g.photon_steps, o["photon_steps"])
    assert g.raytet == o["raytet"] and g.detected == o["detected"] > 0
    np.testing.assert_allclose(g.field, o["raw"], rtol=1e-8, atol=1e-12)
    assert _rows(g.detp) == _rows(o["detp"])
    # nodemua alone: mus from the media table
    cfg1 = dataclasses.replace(cfg, nodemusp=None, issaveseed=0)
    g1 = simulate(mesh, cfg1, trace=True)
    o1 = oracle_mod.run(m.node, m.elem, m.label, cfg1, nthreads=4, trace=True, normalize=False)
    assert np.array_equal(g1.photon_weight.view(np.uint32), o1["photon_weight"].view(np.uint32))


def test_nodal_wp_replay_matches_oracle(oracle_mod, cube):
    m, mesh, mua, mus = cube
    fwd = simulate(mesh, _cfg(m.media, nphoton=6000, nodemua=mua, nodemusp=mus, issaveseed=1))
    assert fwd.detected > 0
    n = len(fwd.detp)
    rcfg = _cfg(m.media, nphoton=n, nodemua=mua, nodemusp=mus, outputtype="wp", issavedet=0,
                replayseed=fwd.seeds.view(np.uint64).reshape(n, 2),
                replayweight=fwd.detp[:, -1].copy(), replaytime=np.zeros(n, np.float32))
    g = simulate(mesh, rcfg)
    o = oracle_mod.run(m.node, m.elem, m.label, rcfg, nthreads=4, normalize=False)
    np.testing.assert_allclose(g.field, o["raw"], rtol=1e-7, atol=1e-12)
    assert g.field.sum() > 0


def test_fast_nodal_run_equals_the_run_labelled_by_element_means(gpu_ready):
    m = prepared_cube(n=12)
    mua, mus = nodal_fields(m.node)
    label, media = labelled_by_means(m, mua, mus)
    base = dict(nphoton=200_000, fast_math=1, issaveseed=1, maxdetphoton=200_000)  # every record kept
    nodal = simulate(Mesh(m.node, m.elem, m.label), _cfg(m.media, nodemua=mua, nodemusp=mus, **base), trace=True)
    lab = simulate(Mesh(m.node, m.elem, label), _cfg(media, **base), trace=True)
    assert np.array_equal(nodal.photon_weight.view(np.uint32), lab.photon_weight.view(np.uint32))
    assert nodal.raytet == lab.raytet and nodal.detected == lab.detected > 0
    np.testing.assert_allclose(nodal.field, lab.field, rtol=1e-9, atol=1e-15)
    # the same photons reach the same detectors with the same scatter counts; the per-medium columns
    # follow the labels, so their totals are compared
    def key(r, M):
        return sorted(zip(r.seeds.view(np.uint64)[:, 0].tolist(), r.detp[:, 0].tolist(),
                          r.detp[:, 1:1 + M].sum(1).tolist()))
    assert key(nodal, len(m.media) - 1) == key(lab, len(media) - 1)


def test_nodal_launch_forms_agree(cube):
    m, mesh, mua, mus = cube
    cfg = _cfg(m.media, nphoton=60_000, fast_math=1, issaveseed=1, nodemua=mua, nodemusp=mus,
               tend=2e-9, tstep=0.1e-9)
    plain = simulate(mesh, dataclasses.replace(cfg, phased=-1))
    phased = simulate(mesh, dataclasses.replace(cfg, phased=3))
    batch = simulate_batch([mesh, mesh], [cfg, dataclasses.replace(cfg, nodemua=None, nodemusp=None)])
    for r in (phased, batch[0]):
        np.testing.assert_allclose(r.field, plain.field, rtol=1e-9, atol=1e-15)
        assert r.raytet == plain.raytet and _rows(r.detp) == _rows(plain.detp)
    solo = simulate(mesh, dataclasses.replace(cfg, nodemua=None, nodemusp=None, phased=-1))
    np.testing.assert_allclose(batch[1].field, solo.field, rtol=1e-9, atol=1e-15)
    assert batch[1].raytet != plain.raytet


def test_pmmc_nodal_keys_run_the_nodal_path(cube):
    m, mesh, mua, mus = cube
    out = pmmc.run(dict(nphoton=20000, node=m.node, elem=m.elem, elemprop=m.label, prop=m.media,
                        srcpos=[30, 30, 0], srcdir=[0, 0, 1], tstart=0, tend=5e-9, tstep=5e-9, seed=3,
                        isnormalized=0, basisorder=0, nodemua=mua, nodemusp=mus))
    r = simulate(mesh, SimConfig(media=m.media, nphoton=20000, seed=3, srcpos=(30, 30, 0), tend=5e-9, tstep=5e-9,
                                 isnormalized=0, basisorder=0, nodemua=mua, nodemusp=mus))
    np.testing.assert_allclose(out["flux"][:, 0], r.field[0], rtol=1e-9, atol=1e-15)

