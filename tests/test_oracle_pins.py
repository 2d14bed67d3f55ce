"""Host stages of the oracle pinned against the reference's own code, run on
the same inputs (fixtures from tests/golden/make_golden.py, produced by the
reference's mmc_prep and mesh_normalize through oracle/ref_driver.c)."""
import numpy as np
import pytest

import golden_checks as gc


@pytest.mark.parametrize("name", ["cube6k", "incl48k"])
def test_mesh_preparation_matches_reference(oracle_mod, name):
    m, cfg, fx = gc.case_mesh_and_config(name)
    pin = gc.load(name + "_pins")
    o = oracle_mod.prep_mesh(m.node, m.elem, m.label)
    sub = pin["sub"]
    assert o["nf"] == int(pin["nf"])
    np.testing.assert_array_equal(o["elem"][sub], pin["elem"])      # orientation fix
    np.testing.assert_array_equal(o["facenb"][sub], pin["facenb"])  # neighbours + exterior numbering
    np.testing.assert_array_equal(o["evol"][sub], pin["evol"])
    np.testing.assert_array_equal(o["nvol"], pin["nvol"])
    np.testing.assert_array_equal(o["normals"][sub], pin["normals"])


@pytest.mark.parametrize("name", ["cube6k", "incl48k"])
@pytest.mark.parametrize("basisorder", [0, 1])
def test_normalization_matches_reference(oracle_mod, name, basisorder):
    import dataclasses
    m, cfg, fx = gc.case_mesh_and_config(name)
    pin = gc.load(name + "_pins")
    G = cfg.maxgate
    raw = np.random.default_rng(123).random((G, m.ne)) * 100.0
    etot, eabs = float(pin["norm_etot"]), float(pin["norm_eabs"])
    c = dataclasses.replace(cfg, basisorder=basisorder, isnormalized=1, outputtype="flux")
    field, norm = oracle_mod.normalize(m.node, m.elem, m.label, c, raw, etot, etot - eabs)
    idx = pin["sub"] if basisorder == 0 else pin["nsub"]
    # the reference stages the raw field through float32 (src/mmc_cu_host.cu:430)
    np.testing.assert_allclose(field[:, idx], pin[f"norm{basisorder}_field"], rtol=2e-6)
    assert norm == pytest.approx(float(pin[f"norm{basisorder}_normalizer"]), rel=2e-6)
