"""Element ids beyond 25 bits.

The packed face word of a tet record holds the neighbour id in 32 - b bits and
the neighbour's medium label in b bits, b being the fewest bits that hold the
mesh's largest label.  Here a 162,000-tet inclusion cube (labels 1 and 2, so
b = 2 and 30 bits of element ids) is appended to a disjoint 33.8M-tet block
that no photon reaches, so every element the photons visit has an id above
2^25: each photon must follow exactly the path it follows in the cube alone.
"""
import numpy as np
import pytest

from mmc_gb300 import meshgen
from mmc_gb300.core import Mesh, SimConfig, simulate

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def meshes(gpu_ready):
    small = meshgen.inclusion_cube(n=30, size=60.0, jitter=0.25, seed=7)
    pad_node, pad_elem = meshgen.kuhn_cube(178, 1.0, origin=(100.0, 0.0, 0.0))  # x in [100, 278]
    pad_ne = pad_elem.shape[0]
    node = np.concatenate([pad_node.astype(np.float32), small.node])
    elem = np.concatenate([pad_elem, small.elem + np.int32(pad_node.shape[0])])
    label = np.concatenate([np.ones(pad_ne, np.int32), small.label])
    assert pad_ne > 2**25
    del pad_node, pad_elem
    big = Mesh(node, elem, label)
    return small, Mesh(small.node, small.elem, small.label), big, pad_ne


@pytest.mark.parametrize("phased", [-1, 2])
def test_photons_follow_the_same_paths_with_element_ids_above_2_25(meshes, phased):
    small, small_mesh, big_mesh, pad_ne = meshes
    cfg = SimConfig(media=small.media, nphoton=300_000, seed=99, srcpos=(30.0, 30.0, 0.0),
                    srcdir=(0.0, 0.0, 1.0), tend=5e-9, tstep=1e-9, issavedet=1, issaveseed=1,
                    detpos=np.array([[40.0, 30.0, 0.0, 2.0], [45.0, 30.0, 0.0, 2.0]], np.float32),
                    maxdetphoton=100_000, basisorder=0, isnormalized=0, phased=phased)
    a = simulate(small_mesh, cfg)
    b = simulate(big_mesh, cfg)
    assert a.aborted == 0 and b.aborted == 0
    assert b.raytet == a.raytet and b.detected == a.detected > 0
    assert not b.field[:, :pad_ne].any()
    # the same deposits per element, summed by float64 atomics in another order
    np.testing.assert_allclose(b.field[:, pad_ne:], a.field, rtol=1e-9, atol=1e-12)
    rows = lambda r: sorted(map(bytes, np.concatenate([r.detp.view(np.uint8).reshape(len(r.detp), -1), r.seeds], 1)))
    assert rows(b) == rows(a)
    assert b.energytot == a.energytot
    assert b.energyesc == pytest.approx(a.energyesc, rel=1e-9)
