"""The CUDA engine against the reference golden fixtures (statistical parity
with 10 runs of the reference CPU engine)."""
import pytest

import golden_checks as gc
from mmc_gb300.core import Mesh, simulate

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["cube6k", "incl48k"])
@pytest.mark.parametrize("accum_f64,fast_math", [(1, 0), (0, 0), (1, 1), (0, 1)])
def test_engine_matches_reference_runs(gpu_ready, name, accum_f64, fast_math):
    import dataclasses
    m, cfg, fx = gc.case_mesh_and_config(name, seed=9001)
    cfg = dataclasses.replace(cfg, accum_f64=accum_f64, fast_math=fast_math)
    mesh = Mesh(m.node, m.elem, m.label)
    r = simulate(mesh, cfg)
    msgs = gc.check_field(r.field, fx, m.media, m.label, cfg.nphoton)
    msgs += gc.check_tests_per_photon(r.raytet / cfg.nphoton, fx)
    if cfg.issavedet:
        msgs += gc.check_detectors(r.detp, m.media, fx)
    assert r.aborted == 0
    assert not msgs, "\n".join(msgs)
