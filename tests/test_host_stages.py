"""The product's host stages (libmmcgb.so, no GPU) against the CPU oracle and
the reference pins: mesh preparation bit for bit, normalization to float
rounding of the reference's float32 staging."""
import dataclasses

import numpy as np
import pytest

import golden_checks as gc
from mmc_gb300 import core, meshgen


@pytest.mark.parametrize("name", ["cube6k", "incl48k"])
def test_prepare_host_matches_reference_and_oracle(oracle_mod, name):
    m, cfg, fx = gc.case_mesh_and_config(name)
    pin = gc.load(name + "_pins")
    p = core.prepare_host(m.node, m.elem, m.label)
    o = oracle_mod.prep_mesh(m.node, m.elem, m.label)
    for k in ("elem", "facenb", "normals", "evol", "nvol"):
        np.testing.assert_array_equal(p[k], o[k], err_msg=k)
    sub = pin["sub"]
    np.testing.assert_array_equal(p["normals"][sub], pin["normals"])
    np.testing.assert_array_equal(p["evol"][sub], pin["evol"])
    assert p["nf"] == int(pin["nf"])


@pytest.mark.parametrize("name", ["cube6k", "incl48k"])
@pytest.mark.parametrize("basisorder", [0, 1])
def test_normalize_host_matches_reference(name, basisorder):
    m, cfg, fx = gc.case_mesh_and_config(name)
    pin = gc.load(name + "_pins")
    raw = np.random.default_rng(123).random((cfg.maxgate, m.ne)) * 100.0
    etot, eabs = float(pin["norm_etot"]), float(pin["norm_eabs"])
    c = dataclasses.replace(cfg, basisorder=basisorder, isnormalized=1, outputtype="flux")
    field, norm = core.normalize_host(m.node, m.elem, m.label, c, raw, etot, etot - eabs)
    idx = pin["sub"] if basisorder == 0 else pin["nsub"]
    np.testing.assert_allclose(field[:, idx], pin[f"norm{basisorder}_field"], rtol=2e-6)
    assert norm == pytest.approx(float(pin[f"norm{basisorder}_normalizer"]), rel=2e-6)


def test_normalize_host_matches_oracle_exactly(oracle_mod):
    m = meshgen.inclusion_cube(n=8, jitter=0.5, seed=1)
    from mmc_gb300.core import SimConfig
    raw = np.random.default_rng(5).random((4, m.ne))
    for bo in (0, 1):
        for ot in ("flux", "fluence", "energy"):
            cfg = SimConfig(media=m.media, basisorder=bo, tend=4e-9, tstep=1e-9, outputtype=ot)
            f1, n1 = core.normalize_host(m.node, m.elem, m.label, cfg, raw, 1000.0, 700.0)
            f2, n2 = oracle_mod.normalize(m.node, m.elem, m.label, cfg, raw, 1000.0, 700.0)
            np.testing.assert_allclose(f1, f2, rtol=1e-13)
            assert n1 == pytest.approx(n2, rel=1e-13)


def test_oversized_mesh_rejected_before_any_gpu_work():
    from mmc_gb300 import _native
    node = np.zeros((4, 3), np.float32)
    elem = np.ones((4, 4), np.int32)
    lab = np.ones(4, np.int32)
    d, keep = core._desc(node, elem, lab)
    d.ne = 9_000_000  # beyond the 24-bit neighbour field of the packed records
    rc = _native.load().mmcgb_prepare_host(d, None, None, None, None, None, None)
    assert rc == 3
