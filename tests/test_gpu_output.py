"""The output stage on the device (element -> node scatter, surface nodal
volume fix, normalization) against the same stage on the host
(mmcgb_normalize_host, itself pinned bit-exactly to the reference's
mesh_normalize, src/mmc_mesh.c:2154-2279).  Both stages read the raw element
deposits of one run; the device version sums with float64 atomics, so the two
agree to summation order."""
import dataclasses

import numpy as np
import pytest

from mmc_gb300 import meshgen
from mmc_gb300.core import Mesh, SimConfig, normalize_host, simulate

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cube(gpu_ready):
    m = meshgen.inclusion_cube(n=16, jitter=0.4, seed=9)
    return m, Mesh(m.node, m.elem, m.label)


@pytest.mark.parametrize("basisorder", [0, 1])
@pytest.mark.parametrize("outputtype", ["flux", "fluence", "energy"])
@pytest.mark.parametrize("isreflect", [0, 1])
def test_device_output_matches_host(cube, basisorder, outputtype, isreflect):
    m, mesh = cube
    base = SimConfig(media=m.media, nphoton=40000, seed=21, srcpos=(30.0, 30.0, 0.0), tend=3e-9, tstep=1e-9,
                     isreflect=isreflect, outputtype=outputtype, basisorder=basisorder, isnormalized=1)
    res = simulate(mesh, base)
    raw = simulate(mesh, dataclasses.replace(base, basisorder=0, isnormalized=0))
    # the raw run repeats the same photons; its deposits differ from res's only in atomic order
    assert raw.energyesc == pytest.approx(res.energyesc, rel=1e-5)  # float per-lane tallies
    field, norm = normalize_host(m.node, m.elem, m.label, base, raw.field, res.energytot, res.energyesc)
    assert res.normalizer == pytest.approx(norm, rel=1e-9)
    np.testing.assert_allclose(res.field, field, rtol=1e-9, atol=1e-12 * np.abs(field).max())


def test_device_output_float32_accumulation(cube):
    m, mesh = cube
    base = SimConfig(media=m.media, nphoton=40000, seed=22, srcpos=(30.0, 30.0, 0.0), tend=3e-9, tstep=1e-9,
                     basisorder=1, isnormalized=1, accum_f64=0)
    res = simulate(mesh, base)
    raw = simulate(mesh, dataclasses.replace(base, basisorder=0, isnormalized=0, accum_f64=1))
    field, norm = normalize_host(m.node, m.elem, m.label, base, raw.field, res.energytot, res.energyesc)
    # float32 partial sums carry about 1e-7 relative rounding per element
    assert res.normalizer == pytest.approx(norm, rel=1e-5)
    np.testing.assert_allclose(res.field, field, rtol=1e-4, atol=1e-6 * np.abs(field).max())
