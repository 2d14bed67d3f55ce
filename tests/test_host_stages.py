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
    """A packed face word keeps 32 - b bits for the neighbour id, b being the bits of
    the mesh's largest label: with labels up to 63 (b = 6) a mesh holds at most
    2^25 - 1 elements.  The check reads only the labels, before any other array."""
    from mmc_gb300 import _native
    lib = _native.load()
    node = np.zeros((4, 3), np.float32)
    elem = np.ones((4, 4), np.int32)
    lab = np.ones(2**25, np.int32)
    lab[7] = 63
    d, keep = core._desc(node, elem, lab)
    d.ne = 2**25  # one element more than 25 neighbour bits hold
    rc = lib.mmcgb_prepare_host(d, None, None, None, None, None, None)
    assert rc == 3
    assert "33554431" in lib.mmcgb_last_error().decode()
    lab[7] = 64  # labels are limited to 0..63 whatever the mesh size
    d.ne = 16
    assert lib.mmcgb_prepare_host(d, None, None, None, None, None, None) == 3


def test_fluence_beyond_the_32bit_cell_index_rejected_before_any_gpu_work():
    """Gates x elements must stay below 2^31-1 cells (the engine's deposit index is
    32-bit); such a run fails with MMCGB_E_ARG at the host check, before any
    allocation, for element and dual-grid output alike."""
    import ctypes as C
    from mmc_gb300 import _native
    from mmc_gb300.core import SimConfig
    lib = _native.load()
    m = meshgen.homogeneous_cube(n=4)  # 384 tets
    d, keep = core._desc(m.node, m.elem, m.label)
    ok = SimConfig(media=m.media, srcpos=(30.0, 30.0, 0.0), tend=5e-9, tstep=1e-9)
    c, k1 = ok.to_c()
    e0 = C.c_int32(-1)
    assert lib.mmcgb_check_config(d, C.byref(c), C.byref(e0)) == 0, lib.mmcgb_last_error()
    assert 1 <= e0.value <= m.ne
    gates = (2**31 - 1) // m.ne + 1  # one gate more than the index reaches
    big = SimConfig(media=m.media, srcpos=(30.0, 30.0, 0.0), tstart=0.0, tstep=1e-12, tend=gates * 1e-12)
    assert big.maxgate * m.ne >= 2**31 - 1
    c2, k2 = big.to_c()
    assert lib.mmcgb_check_config(d, C.byref(c2), None) == 1
    assert "2^31-1" in lib.mmcgb_last_error().decode()
    fits = SimConfig(media=m.media, srcpos=(30.0, 30.0, 0.0), tstart=0.0, tstep=1e-12, tend=(gates - 2) * 1e-12)
    assert fits.maxgate * m.ne < 2**31 - 1
    c3, k3 = fits.to_c()
    assert lib.mmcgb_check_config(d, C.byref(c3), None) == 0, lib.mmcgb_last_error()
    grid = SimConfig(media=m.media, srcpos=(30.0, 30.0, 0.0), tstep=1e-9, tend=40e-9, method="grid", gridstep=0.05)
    c4, k4 = grid.to_c()  # 1201^3 voxels x 40 gates
    assert lib.mmcgb_check_config(d, C.byref(c4), None) == 1
    assert "gridstep" in lib.mmcgb_last_error().decode()


def test_host_check_reports_the_initial_element():
    """A given e0 is kept only when it encloses the source; otherwise the source
    is located (src/mmc_mesh.c:1325-1329)."""
    import ctypes as C
    from mmc_gb300 import _native
    from mmc_gb300.core import SimConfig
    lib = _native.load()
    m = meshgen.homogeneous_cube(n=4)
    d, keep = core._desc(m.node, m.elem, m.label)
    cfg = SimConfig(media=m.media, srcpos=(30.0, 30.0, 0.0), tend=5e-9, tstep=1e-9)
    c, k1 = cfg.to_c()
    e = C.c_int32(0)
    assert lib.mmcgb_check_config(d, C.byref(c), C.byref(e)) == 0
    located = e.value
    assert located >= 1
    c.e0 = m.ne if located != m.ne else 1  # an element that does not hold the source
    assert lib.mmcgb_check_config(d, C.byref(c), C.byref(e)) == 0
    assert e.value == located
    c.srcpos = (C.c_float * 3)(100.0, 30.0, 0.0)  # outside the mesh: a pencil cannot start
    assert lib.mmcgb_check_config(d, C.byref(c), C.byref(e)) == 4


def test_shared_pattern_options_checked_before_any_gpu_work():
    """srcnum > 1 needs a pattern source, does not replay, and multiplies the
    fluence cells that the 32-bit index must hold."""
    import ctypes as C
    from mmc_gb300 import _native
    from mmc_gb300.core import SimConfig
    lib = _native.load()
    m = meshgen.homogeneous_cube(n=4)  # 384 tets
    d, keep = core._desc(m.node, m.elem, m.label)
    pat = np.ones(4 * 3 * 2, np.float32)
    base = dict(media=m.media, srcpos=(10.0, 10.0, 0.0), tend=5e-9, tstep=1e-9, srctype="pattern",
                srcparam1=(20.0, 0, 0, 4), srcparam2=(0, 20.0, 0, 3), srcpattern=pat, srcnum=2)
    e0 = C.c_int32(-1)

    def rc(**kw):
        c, k = SimConfig(**{**base, **kw}).to_c()
        return lib.mmcgb_check_config(d, C.byref(c), C.byref(e0))

    assert rc() == 0, lib.mmcgb_last_error()
    assert rc(srctype="planar") == 1
    assert rc(srcnum=-1) == 1
    seeds = np.zeros((5, 2), np.uint64)
    assert rc(nphoton=5, replayseed=seeds, replayweight=np.ones(5, np.float32),
              replaytime=np.ones(5, np.float32)) == 1
    gates = (2**31 - 1) // m.ne // 8 + 1  # fits alone, not with 8 patterns
    assert rc(srcnum=1, srcpattern=pat[:12], tend=gates * 1e-9) == 0
    assert rc(srcnum=8, srcpattern=np.ones(12 * 8, np.float32), tend=gates * 1e-9) == 1
    assert "patterns" in lib.mmcgb_last_error().decode()
