"""Dual-grid (DMMC, the reference's -M G) output on the GPU: the same voxel
deposits as the oracle photon by photon (IEEE arithmetic, sums to summation
order), statistical parity with the reference runs (tests/golden/
grid_cube6k.npz), the normalization of src/mmc_mesh.c:2204-2206, and the same
result when a run is traced gate-phased."""
import dataclasses

import numpy as np
import pytest

import golden_checks as gc
from mmc_gb300.core import Mesh, simulate

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def grid_case(gpu_ready):
    m, cfg, fx = gc.case_mesh_and_config("grid_cube6k")
    return m, Mesh(m.node, m.elem, m.label), cfg, fx


def test_grid_matches_oracle(oracle_mod, grid_case):
    m, mesh, cfg, fx = grid_case
    assert mesh.grid_dims(cfg.gridstep) == tuple(int(x) for x in fx["dim"])
    small = dataclasses.replace(cfg, nphoton=20000, fast_math=0, tend=5e-9, tstep=1e-9)
    g = simulate(mesh, small, trace=True)
    o = oracle_mod.run(m.node, m.elem, m.label, small, nthreads=4, trace=True, normalize=False)
    assert np.array_equal(g.photon_weight.view(np.uint32), o["photon_weight"].view(np.uint32))
    assert np.array_equal(g.photon_steps, o["photon_steps"])
    np.testing.assert_allclose(g.field, o["raw"], rtol=1e-8, atol=1e-12)
    # gate-phased tracing deposits the same
    p = simulate(mesh, dataclasses.replace(small, phased=2))
    np.testing.assert_allclose(p.field, g.field, rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("fast_math", [0, 1])
def test_grid_matches_reference_runs(grid_case, fast_math):
    m, mesh, cfg, fx = grid_case
    r = simulate(mesh, dataclasses.replace(cfg, fast_math=fast_math))
    msgs = gc.check_grid(r.field, fx)
    assert not msgs, "\n".join(msgs)


@pytest.mark.parametrize("outputtype", ["flux", "fluence", "energy"])
def test_grid_normalization(grid_case, outputtype):
    m, mesh, cfg, fx = grid_case
    c = dataclasses.replace(cfg, nphoton=20000, outputtype=outputtype)
    raw = simulate(mesh, c)
    n = simulate(mesh, dataclasses.replace(c, isnormalized=1))
    et = np.float32(n.energytot)
    want = 1.0 / float(et) if outputtype != "energy" else float(np.float32(1.0) / et)
    if outputtype == "flux":
        want /= float(np.float32(c.tstep))
    assert n.normalizer == pytest.approx(want, rel=1e-12)
    np.testing.assert_allclose(n.field, raw.field * want, rtol=1e-9, atol=1e-15)
