"""Replicated near-source cells: the gate-0 deposits of each photon's first
ray-tet tests go to one of several copies of the gate-0 plane and are folded
into the fluence after every launch.  The sums equal those of the batched
launch, which deposits into the cells themselves, for one launch, several
launches of a session and the respin graph.
"""
import numpy as np
import pytest

from mmc_gb300 import meshgen
from mmc_gb300.core import Mesh, Session, SimConfig, simulate, simulate_batch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case(gpu_ready):
    m = meshgen.inclusion_cube(n=24, size=60.0, jitter=0.25, seed=3)
    cfg = SimConfig(media=m.media, nphoton=200_000, seed=5, srcpos=(30.0, 30.0, 0.0), srcdir=(0.0, 0.0, 1.0),
                    tend=5e-9, tstep=1e-9, basisorder=0, isnormalized=0, fast_math=1)
    return Mesh(m.node, m.elem, m.label), cfg


def test_replicated_cells_sum_to_the_cells_themselves(case):
    mesh, cfg = case
    solo = simulate(mesh, cfg)
    (batch,) = simulate_batch([mesh], [cfg])
    assert solo.raytet == batch.raytet
    assert solo.field[0].max() > 100 * np.median(solo.field[0][solo.field[0] > 0])  # a hot spot to spread
    np.testing.assert_allclose(solo.field, batch.field, rtol=1e-9, atol=1e-15)


def test_every_launch_folds_its_copies(case):
    mesh, cfg = case
    solo = simulate(mesh, cfg)
    s = Session(mesh, cfg)
    s.launch(0, 100_000)
    s.launch(100_000, 100_000)
    two = s.end()
    np.testing.assert_allclose(two.field, solo.field, rtol=1e-9, atol=1e-15)
    s = Session(mesh, cfg)
    s.launch_repeat(0, 50_000, 4)
    graph = s.end()
    np.testing.assert_allclose(graph.field, solo.field, rtol=1e-9, atol=1e-15)
