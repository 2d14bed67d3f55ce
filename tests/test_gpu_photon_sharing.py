"""Several patterns sharing each photon (a pattern source with srcnum > 1, the
reference's photon sharing, src/mmc_core.cl:929-942, :1907-1911).

* photon by photon against the CPU oracle (IEEE arithmetic): final weights,
  ray-tet counts, per-pattern deposits and energies, detected records whose
  last column is the launch pixel;
* against the reference's own multi-pattern runs (tests/golden/src_pattern3.npz),
  statistically, with both arithmetic policies;
* each pattern normalized with its own energies, for element, node and
  dual-grid output; gate-phased and batched runs equal the plain one.
"""
import dataclasses

import numpy as np
import pytest

import golden_checks as gc
from mmc_gb300 import meshgen
from mmc_gb300.core import Mesh, SimConfig, normalize_host, simulate, simulate_batch

pytestmark = pytest.mark.gpu

K, NX, NY = 3, 4, 3
PATTERN = np.random.default_rng(11).uniform(0.1, 1.0, NX * NY * K).astype(np.float32)  # pixel-major


@pytest.fixture(scope="module")
def void_cube(gpu_ready):
    m = meshgen.homogeneous_cube(n=12)
    label = m.label.copy()
    label[meshgen.centroids(m.node, m.elem)[:, 2] < 5.0] = 0
    m = meshgen.Mesh(m.node, m.elem, label, m.media, "cube-void")
    return m, Mesh(m.node, m.elem, m.label)


def _cfg(m, **kw):
    base = dict(media=m.media, nphoton=4000, seed=29, srctype="pattern", srcpos=(20.0, 20.0, 0.0),
                srcdir=(0.0, 0.0, 1.0), srcparam1=(20.0, 0, 0, NX), srcparam2=(0, 20.0, 0, NY), srcpattern=PATTERN,
                srcnum=K, tend=5e-9, tstep=1e-9, basisorder=0, isnormalized=0, fast_math=0, issavedet=1,
                detpos=np.array([[30.0, 30.0, 60.0, 8.0], [30.0, 30.0, 0.0, 15.0]], np.float32),
                maxdetphoton=20000)
    base.update(kw)
    return SimConfig(**base)


def _rows(detp):
    return sorted(map(bytes, detp.view(np.uint8).reshape(len(detp), -1)))


def test_shared_patterns_match_oracle_photon_by_photon(oracle_mod, void_cube):
    m, mesh = void_cube
    cfg = _cfg(m)
    g = simulate(mesh, cfg, trace=True)
    o = oracle_mod.run(m.node, m.elem, m.label, cfg, nthreads=4, trace=True, normalize=False)
    assert g.field.shape == o["raw"].shape == (cfg.maxgate, m.ne, K)
    assert np.array_equal(g.photon_weight.view(np.uint32), o["photon_weight"].view(np.uint32))
    assert np.array_equal(g.photon_steps, o["photon_steps"])
    assert g.raytet == o["raytet"] and g.detected == o["detected"] > 0
    np.testing.assert_allclose(g.field, o["raw"], rtol=1e-8, atol=1e-12)
    np.testing.assert_allclose(g.energy_src, o["energy_src"], rtol=1e-6)
    assert g.energytot == pytest.approx(o["energy_src"][0].sum(), rel=1e-6)
    # the detected records are the oracle's; their last column holds the launch pixel
    assert _rows(g.detp) == _rows(o["detp"])
    pix = g.detp[:, -1].view(np.int32)
    assert pix.min() >= 0 and pix.max() < NX * NY


def test_one_shared_pattern_of_ones_is_the_single_pattern_run(void_cube):
    """A photon shared by patterns starts with weight 1: with one pattern of all
    ones next to another, the first pattern's deposits are those of the single
    pattern of ones (roulette is off with several gates, so paths do not depend
    on the weight)."""
    m, mesh = void_cube
    two = np.stack([np.ones(NX * NY, np.float32), PATTERN[::K]], axis=1).ravel()
    shared = simulate(mesh, _cfg(m, srcnum=2, srcpattern=two, issavedet=0))
    single = simulate(mesh, _cfg(m, srcnum=1, srcpattern=np.ones(NX * NY, np.float32), issavedet=0))
    np.testing.assert_allclose(shared.field[..., 0], single.field, rtol=1e-9, atol=1e-12)
    assert shared.energy_src[0, 0] == pytest.approx(single.energytot, rel=1e-9)


@pytest.mark.parametrize("fast_math", [0, 1])
def test_shared_patterns_match_reference_runs(gpu_ready, fast_math):
    m, cfg, fx = gc.case_mesh_and_config("src_pattern3")
    r = simulate(Mesh(m.node, m.elem, m.label), dataclasses.replace(cfg, fast_math=fast_math))
    msgs = gc.check_patterns(r.field[0], fx)
    assert not msgs, "\n".join(msgs)


@pytest.mark.parametrize("basisorder", [0, 1])
def test_each_pattern_normalized_with_its_own_energies(void_cube, basisorder):
    m, mesh = void_cube
    raw = simulate(mesh, _cfg(m, fast_math=1, issavedet=0))
    out = simulate(mesh, _cfg(m, fast_math=1, issavedet=0, isnormalized=1, basisorder=basisorder,
                              outputtype="fluence"))
    norms = []
    for p in range(K):
        one = _cfg(m, srcnum=1, srcpattern=None, srctype="pencil", isnormalized=1, basisorder=basisorder,
                   outputtype="fluence")
        f, n = normalize_host(m.node, m.elem, m.label, one, raw.field[..., p], raw.energy_src[0, p],
                              raw.energy_src[1, p])
        # the same photons, so the same energies; deposits summed in another order
        np.testing.assert_allclose(out.field[..., p], f, rtol=1e-9, atol=1e-15)
        norms.append(n)
    assert out.normalizer == pytest.approx(np.mean(norms), rel=1e-9)


def test_shared_patterns_on_the_dual_grid(oracle_mod, void_cube):
    m, mesh = void_cube
    cfg = _cfg(m, method="grid", gridstep=2.0, issavedet=0)
    g = simulate(mesh, cfg)
    o = oracle_mod.run(m.node, m.elem, m.label, cfg, nthreads=4, normalize=False)
    assert g.field.shape == o["raw"].shape and g.field.shape[-1] == K
    np.testing.assert_allclose(g.field, o["raw"], rtol=1e-8, atol=1e-12)
    n = simulate(mesh, dataclasses.replace(cfg, isnormalized=1))
    # one scale factor per pattern, from that pattern's launched weight
    for p in range(K):
        mask = g.field[..., p] > 0
        ratio = n.field[..., p][mask] / g.field[..., p][mask]
        assert np.ptp(ratio) <= 1e-9 * ratio.max()


def test_phased_and_batched_runs_equal_the_plain_run(void_cube):
    m, mesh = void_cube
    cfg = _cfg(m, nphoton=20000, fast_math=1, issaveseed=1)
    plain = simulate(mesh, dataclasses.replace(cfg, phased=-1))
    phased = simulate(mesh, dataclasses.replace(cfg, phased=2))
    np.testing.assert_allclose(phased.field, plain.field, rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(phased.energy_src, plain.energy_src, rtol=1e-9)
    assert phased.raytet == plain.raytet and _rows(phased.detp) == _rows(plain.detp)
    pencil = SimConfig(media=m.media, nphoton=5000, seed=3, srcpos=(30.0, 30.0, 30.0), tend=5e-9, tstep=1e-9,
                       basisorder=0, isnormalized=0)
    batch = simulate_batch([mesh, mesh], [cfg, pencil])
    np.testing.assert_allclose(batch[0].field, plain.field, rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(batch[0].energy_src, plain.energy_src, rtol=1e-9)
    assert _rows(batch[0].detp) == _rows(plain.detp)
    np.testing.assert_allclose(batch[1].field, simulate(mesh, pencil).field, rtol=1e-9, atol=1e-12)
