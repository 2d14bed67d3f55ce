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


def test_exit_image_matches_reference():
    """The exit image of an area detector (-x 2): the reference's own records
    binned by io.detector_image equal the <session>.img the reference wrote
    from them (tests/golden/detimage_cube6k.npz)."""
    from mmc_gb300 import io, meshgen
    from mmc_gb300.core import SimConfig
    fx = gc.load("detimage_cube6k")
    m = meshgen.homogeneous_cube(n=10)
    cfg = SimConfig(media=m.media, tend=5e-9, tstep=float(fx["tstep"]), detpos=fx["detpos"], issavedet=1,
                    issaveexit=2)
    img = io.detector_image(fx["detp"], cfg, fx["detparam1"], fx["detparam2"])
    assert img.shape == fx["img"].shape == (5, 8, 8) and fx["img"].sum() > 0
    np.testing.assert_allclose(img, fx["img"], rtol=2e-6, atol=1e-6)
