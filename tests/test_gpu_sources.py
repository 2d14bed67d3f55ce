"""Photon sources on the GPU.

* Every source type of the reference (src/mmc_raytrace.c:2346-2671), with the
  beam-focus variants, against the CPU oracle photon by photon (IEEE
  arithmetic): final weights, ray-tet counts, detectors, launched weight and
  fluence.  Sources on the z=0 face sit over a void voxel layer (z < 5 mm),
  where each photon is located per launch.
* The sources with reference golden data (tests/golden/src_*.npz) against the
  reference runs, statistically, with both arithmetic policies.
* A source that launches photons outside the mesh is reported as an error.
"""
import dataclasses

import numpy as np
import pytest

import golden_checks as gc
from mmc_gb300 import _native, meshgen
from mmc_gb300.core import Mesh, SimConfig, simulate

pytestmark = pytest.mark.gpu

CENTRE = dict(srcpos=(30.0, 30.0, 30.0), srcdir=(0.0, 0.0, 1.0))
FACE = dict(srcpos=(30.0, 30.0, 0.0), srcdir=(0.0, 0.0, 1.0))
AREA = dict(srcpos=(20.0, 20.0, 0.0), srcdir=(0.0, 0.0, 1.0), srcparam1=(20.0, 0, 0, 0), srcparam2=(0, 20.0, 0, 0))

CASES = {
    "isotropic": dict(srctype="isotropic", **CENTRE),
    "cone": dict(srctype="cone", srcpos=(30.0, 30.0, 30.0), srcdir=(0.6, 0.0, 0.8), srcparam1=(0.6, 0, 0, 0)),
    "cone_uniform_angle": dict(srctype="cone", srcparam1=(0.4, 1, 0, 0), **CENTRE),
    "arcsine": dict(srctype="arcsine", **CENTRE),
    "zgaussian": dict(srctype="zgaussian", srcparam1=(0.3, 0, 0, 0), **CENTRE),
    "disk": dict(srctype="disk", srcparam1=(10.0, 0, 0, 0), **FACE),
    "ring": dict(srctype="ring", srcparam1=(12.0, 6.0, 0.5, 2.5), **FACE),
    "gaussian": dict(srctype="gaussian", srcparam1=(5.0, 0, 0, 0), **FACE),
    "gaussian_focused": dict(srctype="gaussian", srcparam1=(5.0, 0.0008, 0, 0), focus=20.0, **FACE),
    "planar": dict(srctype="planar", **AREA),
    "planar_converging": dict(srctype="planar", focus=30.0, **AREA),
    "planar_diverging": dict(srctype="planar", focus=-30.0, **AREA),
    "planar_diffuse": dict(srctype="planar", focus=float("nan"), **AREA),
    "planar_lambertian": dict(srctype="planar", focus=float("-inf"), **AREA),
    "pattern": dict(srctype="pattern", srcpos=(20.0, 20.0, 0.0), srcdir=(0.0, 0.0, 1.0), srcparam1=(20.0, 0, 0, 4),
                    srcparam2=(0, 20.0, 0, 3), srcpattern=np.linspace(0.1, 1.0, 12).astype(np.float32)),
    "pattern3d": dict(srctype="pattern3d", srcpos=(25.0, 25.0, 1.0), srcdir=(0.0, 0.0, 1.0), srcparam1=(4, 4, 2, 0),
                      srcpattern=np.linspace(0.2, 1.0, 32).astype(np.float32)),
    "fourier": dict(srctype="fourier", srcpos=(20.0, 20.0, 0.0), srcdir=(0.0, 0.0, 1.0),
                    srcparam1=(20.0, 0, 0, 2.5), srcparam2=(0, 20.0, 0, 1.3)),
    "fourierx": dict(srctype="fourierx", srcpos=(20.0, 20.0, 0.0), srcdir=(0.0, 0.0, 1.0),
                     srcparam1=(20.0, 0, 0, 20.0), srcparam2=(2.0, 1.0, 0.25, 0.5)),
    "fourierx2d": dict(srctype="fourierx2d", srcpos=(20.0, 20.0, 0.0), srcdir=(0.0, 0.0, 1.0),
                       srcparam1=(20.0, 0, 0, 20.0), srcparam2=(2.0, 3.0, 0.1, 0.2)),
    "line": dict(srctype="line", srcpos=(20.0, 30.0, 30.0), srcdir=(1.0, 0.0, 0.0), srcparam1=(20.0, 0, 0, 0)),
    "slit": dict(srctype="slit", srcpos=(20.0, 30.0, 0.0), srcdir=(0.0, 0.0, 1.0), srcparam1=(20.0, 0, 0, 0)),
    "pencilarray": dict(srctype="pencilarray", srcpos=(20.0, 20.0, 0.0), srcdir=(0.0, 0.0, 1.0),
                        srcparam1=(20.0, 0, 0, 5), srcparam2=(0, 20.0, 0, 4)),
    "hyperboloid": dict(srctype="hyperboloid", srcparam1=(3.0, 2.0, 10.0, 0), **FACE),
}


@pytest.fixture(scope="module")
def void_layer_cube(gpu_ready):
    """The 12^3-voxel cube (5 mm voxels) with its bottom voxel layer (z < 5 mm) void."""
    m = meshgen.homogeneous_cube(n=12)
    label = m.label.copy()
    label[meshgen.centroids(m.node, m.elem)[:, 2] < 5.0] = 0
    m = meshgen.Mesh(m.node, m.elem, label, m.media, "cube-void")
    return m, Mesh(m.node, m.elem, m.label)


@pytest.mark.parametrize("name", sorted(CASES))
def test_source_matches_oracle_photon_by_photon(oracle_mod, void_layer_cube, name):
    m, mesh = void_layer_cube
    cfg = SimConfig(media=m.media, nphoton=3000, seed=17, tend=5e-9, tstep=1e-9, basisorder=0, isnormalized=0,
                    fast_math=0, **CASES[name])
    g = simulate(mesh, cfg, trace=True)
    o = oracle_mod.run(m.node, m.elem, m.label, cfg, nthreads=4, trace=True)
    assert o["outside"] == 0
    assert np.array_equal(g.photon_weight.view(np.uint32), o["photon_weight"].view(np.uint32)), name
    assert np.array_equal(g.photon_steps, o["photon_steps"]), name
    assert g.raytet == o["raytet"]
    assert g.energytot == pytest.approx(o["energytot"], rel=1e-6)
    np.testing.assert_allclose(g.field, o["raw"], rtol=1e-8, atol=1e-12)


@pytest.mark.parametrize("name", ["src_isotropic", "src_cone", "src_disk", "src_gaussian", "src_planar"])
@pytest.mark.parametrize("fast_math", [0, 1])
def test_source_matches_reference_runs(gpu_ready, name, fast_math):
    m, cfg, fx = gc.case_mesh_and_config(name)
    cfg = dataclasses.replace(cfg, fast_math=fast_math)
    r = simulate(Mesh(m.node, m.elem, m.label), cfg)
    msgs = gc.check_field(r.field, fx, m.media, m.label, cfg.nphoton)
    msgs += gc.check_tests_per_photon(r.raytet / cfg.nphoton, fx)
    assert not msgs, "\n".join(msgs)


def test_launch_outside_the_mesh_is_an_error(oracle_mod, void_layer_cube):
    m, mesh = void_layer_cube
    cfg = SimConfig(media=m.media, nphoton=2000, seed=3, tend=5e-9, tstep=5e-9, basisorder=0, srctype="disk",
                    srcparam1=(50.0, 0, 0, 0), **FACE)  # most of the disk lies beyond the 60 mm cube
    with pytest.raises(_native.MmcgbError) as e:
        simulate(mesh, cfg)
    assert e.value.code == 4
    assert oracle_mod.run(m.node, m.elem, m.label, cfg, nthreads=4)["outside"] > 0


def test_exiting_weight_per_face(oracle_mod, gpu_ready):
    """issaveref (-X): the exiting weight per exterior face and gate equals the
    oracle's (IEEE arithmetic, to summation order) and matches the reference
    runs statistically (fast arithmetic); normalized output divides by the
    launched weight (src/mmc_mesh.c:2160-2167)."""
    m, cfg, fx = gc.case_mesh_and_config("dref_cube6k")
    mesh = Mesh(m.node, m.elem, m.label)
    assert mesh.nf == int(fx["nf"])
    small = dataclasses.replace(cfg, nphoton=20000, fast_math=0)
    g = simulate(mesh, small)
    o = oracle_mod.run(m.node, m.elem, m.label, small, nthreads=4, normalize=False)
    np.testing.assert_allclose(g.dref, o["dref"], rtol=1e-9, atol=1e-12)
    r = simulate(mesh, dataclasses.replace(cfg, fast_math=1))
    msgs = gc.check_dref(r.dref, fx)
    assert not msgs, "\n".join(msgs)
    n = simulate(mesh, dataclasses.replace(small, isnormalized=1))
    np.testing.assert_allclose(n.dref, g.dref / np.float32(g.energytot), rtol=1e-6)


def test_host_locate_before_and_after_the_locator_grid(oracle_mod, void_layer_cube):
    """The initial-element search scans every element until a simulation needs
    the locator grid (any source but the pencil beam); with the grid built it
    gives the same elements (the lowest-index enclosing one, 0 outside)."""
    m, _ = void_layer_cube
    mesh = Mesh(m.node, m.elem, m.label)
    rng = np.random.default_rng(9)
    pts = np.concatenate([rng.uniform(-5, 65, (200, 3)), m.node[rng.integers(0, m.nn, 50)],  # nodes: shared corners
                          rng.uniform(0, 60, (50, 3)).round(0)]).astype(np.float32)      # faces and edges
    before = [mesh.locate(p) for p in pts]
    simulate(mesh, SimConfig(media=m.media, nphoton=100, seed=1, tend=5e-9, tstep=5e-9, basisorder=0,
                             **CASES["disk"]))
    after = [mesh.locate(p) for p in pts]
    assert before == after
    assert before == [oracle_mod.initelem(m.node, m.elem, m.label, p) for p in pts]
