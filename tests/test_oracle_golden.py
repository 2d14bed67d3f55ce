"""The CPU oracle against the reference golden fixtures (statistical parity),
at the fixtures' own photon counts: this pins the oracle, which in turn checks
the CUDA engine photon by photon."""
import dataclasses
import os

import pytest

import golden_checks as gc

NTHREADS = os.cpu_count() or 4


SOURCE_CASES = ["src_isotropic", "src_cone", "src_disk", "src_gaussian", "src_planar"]


@pytest.mark.parametrize("name", ["cube6k", "incl48k"] + SOURCE_CASES)
def test_oracle_matches_reference_runs(oracle_mod, name):
    m, cfg, fx = gc.case_mesh_and_config(name)
    r = oracle_mod.run(m.node, m.elem, m.label, cfg, nthreads=NTHREADS, normalize=False)
    msgs = gc.check_field(r["raw"], fx, m.media, m.label, cfg.nphoton)
    msgs += gc.check_tests_per_photon(r["raytet"] / cfg.nphoton, fx)
    if cfg.issavedet:
        msgs += gc.check_detectors(r["detp"], m.media, fx)
    assert r["aborted"] == 0
    assert not msgs, "\n".join(msgs)


def test_oracle_exiting_weight_matches_reference_runs(oracle_mod):
    """Exiting weight per exterior face and gate (-X) against the reference."""
    m, cfg, fx = gc.case_mesh_and_config("dref_cube6k")
    r = oracle_mod.run(m.node, m.elem, m.label, cfg, nthreads=NTHREADS, normalize=False)
    assert r["nf"] == int(fx["nf"])
    msgs = gc.check_dref(r["dref"], fx)
    assert not msgs, "\n".join(msgs)
    # escaped weight = weight out through exterior faces + weight of photons stopped at the time limit
    assert 0.99 * r["energyesc"] < r["dref"].sum() <= r["energyesc"]


def test_oracle_dual_grid_matches_reference_runs(oracle_mod):
    """Dual-grid (DMMC, -M G) fluence on 2 mm voxels against the reference."""
    m, cfg, fx = gc.case_mesh_and_config("grid_cube6k")
    assert oracle_mod.grid_dims(m.node, cfg.gridstep) == tuple(int(x) for x in fx["dim"])
    r = oracle_mod.run(m.node, m.elem, m.label, cfg, nthreads=NTHREADS, normalize=False)
    msgs = gc.check_grid(r["raw"], fx)
    assert not msgs, "\n".join(msgs)
    # every deposit is the lost weight divided by mua: the grid holds the absorbed energy
    assert r["raw"].sum() * m.media[1, 0] == pytest.approx(r["energytot"] - r["energyesc"], rel=1e-5)


@pytest.mark.parametrize("name", ["bench_dmmc-cube60", "bench_dmmc-cube60b"])
def test_oracle_builtin_benchmarks_match_reference_runs(oracle_mod, name):
    """The reference's built-in benchmarks (-Q dmmc-cube60, dmmc-cube60b: a
    6-tet cube, so photons cross few, large elements) with dual-grid output."""
    m, cfg, fx = gc.case_mesh_and_config(name)
    r = oracle_mod.run(m.node, m.elem, m.label, cfg, nthreads=NTHREADS, normalize=False)
    msgs = gc.check_bench(r["raw"], fx) + gc.check_tests_per_photon(r["raytet"] / cfg.nphoton, fx)
    assert not msgs, "\n".join(msgs)


def test_oracle_trajectories_match_reference_runs(oracle_mod):
    """Trajectory records (-D M: launch, every scattering event, photon end)
    against the reference's records: records per photon and their histogram,
    end weights, escaped fraction, mean record position and weight."""
    import numpy as np
    m, cfg, fx = gc.case_mesh_and_config("traj_cube6k")
    r = oracle_mod.run(m.node, m.elem, m.label, cfg, nthreads=NTHREADS, normalize=False, trace=True)
    assert r["ntraj"] == len(r["traj"]) < cfg.maxjumpdebug
    msgs = gc.check_traj(r["traj"], cfg.nphoton, fx)
    assert not msgs, "\n".join(msgs)
    # each photon's last record carries its final weight; a small buffer keeps the first records
    t = r["traj"]
    ids = t[:, 0].view(np.uint32)
    order = np.argsort(ids, kind="stable")
    last = np.r_[np.nonzero(np.diff(ids[order]))[0], len(ids) - 1]
    assert np.array_equal(t[order][last, 4], r["photon_weight"])
    small = oracle_mod.run(m.node, m.elem, m.label, dataclasses.replace(cfg, nphoton=200, maxjumpdebug=500),
                           nthreads=1, normalize=False)
    assert small["ntraj"] > 500 and len(small["traj"]) == 500


def test_oracle_detects_a_planted_error(oracle_mod):
    """The statistical check has power: a 5% change of the absorption
    coefficient, planted in the oracle's input, must fail it."""
    import dataclasses
    import numpy as np
    m, cfg, fx = gc.case_mesh_and_config("cube6k")
    media = m.media.copy()
    media[1, 0] *= 1.05
    r = oracle_mod.run(m.node, m.elem, m.label, dataclasses.replace(cfg, media=media), nthreads=NTHREADS,
                       normalize=False)
    assert gc.check_field(r["raw"], fx, m.media, m.label, cfg.nphoton)


@pytest.mark.parametrize("name", ["c0_cube162k", "c1_incl1296k"])
def test_oracle_matches_reference_runs_on_the_benchmark_workloads(oracle_mod, name):
    """The two benchmark workloads themselves (162k-tet cube; 1.296M-tet
    inclusion cube with 50 gates and 4 detectors), 1e6 photons, against 10
    reference runs each; on the cube also the node output (the CUDA host's
    scatter and the reference's mesh_normalize, pinned by the fixture)."""
    import numpy as np
    m, cfg, fx = gc.case_mesh_and_config(name)
    r = oracle_mod.run(m.node, m.elem, m.label, cfg, nthreads=NTHREADS, normalize=False)
    msgs = gc.check_field(r["raw"], fx, m.media, m.label, cfg.nphoton)
    msgs += gc.check_tests_per_photon(r["raytet"] / cfg.nphoton, fx)
    if cfg.issavedet:
        msgs += gc.check_detectors(r["detp"], m.media, fx)
    if "node_mean" in fx:
        # node output with the absorbed weight the reference CPU engine tallies (its deposits x mua)
        ncfg = dataclasses.replace(cfg, basisorder=1, isnormalized=1)
        e_dep = float((r["raw"].sum(0) * m.media[m.label, 0].astype(np.float64)).sum())
        node, _ = oracle_mod.normalize(m.node, m.elem, m.label, ncfg, r["raw"], float(cfg.nphoton),
                                       float(cfg.nphoton) - e_dep)
        msgs += gc.check_nodes(node[0], fx)
    assert r["aborted"] == 0
    assert not msgs, "\n".join(msgs)


def test_oracle_shared_patterns_match_reference_runs(oracle_mod):
    """Three patterns sharing each photon (srcnum 3): every (element, pattern)
    cell and each pattern's total against the reference runs; each pattern's
    launched weight is the sum of its values at the photons' launch pixels."""
    m, cfg, fx = gc.case_mesh_and_config("src_pattern3")
    r = oracle_mod.run(m.node, m.elem, m.label, cfg, nthreads=NTHREADS, normalize=False)
    assert r["raw"].shape == (1, m.ne, 3)
    msgs = gc.check_patterns(r["raw"][0], fx)
    assert not msgs, "\n".join(msgs)
    # the reference's seed-SEED0 run printed each pattern's launched weight: the same mean per photon
    # within sampling noise of the pixel draws (12 pixels, values 0.1-1)
    et = fx["energies_seed0"][:, 0]
    assert r["energy_src"][0] == pytest.approx(et, rel=0.03)
    assert r["energytot"] == pytest.approx(r["energy_src"][0].sum(), rel=1e-12)


def test_per_pattern_normalization_matches_reference(oracle_mod):
    """The reference's normalized output of a multi-pattern run equals each
    pattern's raw deposits put through the single-pattern output stage with that
    pattern's own energies (the values its log printed)."""
    import numpy as np
    from mmc_gb300 import core
    m, cfg, fx = gc.case_mesh_and_config("src_pattern3")
    raw, normed, en = fx["raw_seed0"], fx["norm_seed0"], fx["energies_seed0"]
    one = dataclasses.replace(cfg, srcnum=1, isnormalized=1, srcpattern=None, srctype="pencil")
    for p in range(raw.shape[1]):
        etot = float(en[p, 0])
        eesc = etot * (1.0 - float(en[p, 1]) / 100.0)
        field, norm = core.normalize_host(m.node, m.elem, m.label, one, raw[:, p][None, :], etot, eesc)
        np.testing.assert_allclose(field[0], normed[:, p], rtol=2e-5)
        assert norm == pytest.approx(float(en[p, 2]), rel=1e-5)
