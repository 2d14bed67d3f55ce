"""Per-node absorption and scattering (the reference's DOT-reconstruction mode,
src/mmc_core.cl:785-793; pmmc keys nodemua/nodemusp, src/pmmc.cpp:630-672):
each step takes its element's mua (and mus) as the mean of the element's four
nodal values, summed in node order, in place of the media row of its label.

The reference's CPU engine has no such mode, so the oracle's restatement is
pinned through two identities with its pinned media-table path:

* nodal values equal to a medium's (powers of two, so the mean is exact)
  give the media-table run bit for bit;
* a nodal run equals the run in which every element carries a label of its
  own mean (mua, mus) pair, same g and n: the photons take the same paths,
  weights and deposits.

Also the host-side checks: one value per node, finite values, and pmmc's
flags without their arrays refused.
"""
import ctypes as C

import numpy as np
import pytest

from mmc_gb300 import core, meshgen, pmmc
from mmc_gb300.core import SimConfig


def element_means(elem, v):
    """float32 mean of each element's four nodal values, summed in node order."""
    v = np.asarray(v, np.float32)
    e = np.asarray(elem) - 1
    s = (v[e[:, 0]] + v[e[:, 1]]) + v[e[:, 2]]
    return np.float32(0.25) * (s + v[e[:, 3]])


def prepared_cube(n=10):
    """A cube mesh whose element node order is already the prepared one (the
    orientation fix leaves it alone), so nodal means are taken in that order."""
    m = meshgen.homogeneous_cube(n=n)
    elem = core.prepare_host(m.node, m.elem, m.label)["elem"]
    return meshgen.Mesh(m.node, elem, m.label, m.media, "cube")


def nodal_fields(node):
    """Nodal mua and mus varying across the cube: two values each, split by z and x."""
    mua = np.where(node[:, 2] < 30.0, 0.01, 0.03).astype(np.float32)
    mus = np.where(node[:, 0] < 30.0, 1.1, 0.7).astype(np.float32)
    return mua, mus


def _cfg(media, **kw):
    base = dict(media=media, nphoton=3000, seed=17, srcpos=(30.0, 30.0, 0.0), srcdir=(0.0, 0.0, 1.0),
                tend=5e-9, tstep=1e-9, basisorder=0, isnormalized=0, fast_math=0, issavedet=1,
                detpos=np.array([[36.0, 30.0, 0.0, 3.0], [30.0, 30.0, 60.0, 10.0]], np.float32),
                maxdetphoton=10000)
    base.update(kw)
    return SimConfig(**base)


def labelled_by_means(m, mua, mus):
    """The mesh relabelled by each element's distinct (mean mua, mean mus) pair,
    with a media table holding those pairs (g and n of the original medium 1)."""
    pairs = np.stack([element_means(m.elem, mua), element_means(m.elem, mus)], 1)
    uniq, label = np.unique(pairs, axis=0, return_inverse=True)
    assert len(uniq) <= 63
    g, n = m.media[1, 2], m.media[1, 3]
    media = np.vstack([m.media[:1], np.column_stack([uniq, np.full(len(uniq), g), np.full(len(uniq), n)])])
    return label.astype(np.int32).ravel() + 1, media.astype(np.float32)


def test_uniform_nodal_values_give_the_media_table_run(oracle_mod):
    m = prepared_cube()
    media = m.media.copy()
    media[1, :2] = (0.0625, 2.0)
    ones = np.ones(len(m.node), np.float32)
    plain = oracle_mod.run(m.node, m.elem, m.label, _cfg(media), trace=True, normalize=False)
    nodal = oracle_mod.run(m.node, m.elem, m.label, _cfg(media, nodemua=0.0625 * ones, nodemusp=2.0 * ones),
                           trace=True, normalize=False)
    assert np.array_equal(nodal["photon_weight"].view(np.uint32), plain["photon_weight"].view(np.uint32))
    assert np.array_equal(nodal["photon_steps"], plain["photon_steps"])
    assert np.array_equal(nodal["raw"], plain["raw"])
    assert nodal["detected"] == plain["detected"] > 0


def test_nodal_run_is_the_run_labelled_by_element_means(oracle_mod):
    m = prepared_cube()
    mua, mus = nodal_fields(m.node)
    label, media = labelled_by_means(m, mua, mus)
    assert len(media) > 6  # elements straddling the splits take mixed means
    nodal = oracle_mod.run(m.node, m.elem, m.label, _cfg(m.media, nodemua=mua, nodemusp=mus),
                           trace=True, normalize=False)
    lab = oracle_mod.run(m.node, m.elem, label, _cfg(media), trace=True, normalize=False)
    assert np.array_equal(nodal["photon_weight"].view(np.uint32), lab["photon_weight"].view(np.uint32))
    assert np.array_equal(nodal["photon_steps"], lab["photon_steps"])
    assert np.array_equal(nodal["raw"], lab["raw"])
    # the records agree in everything but the per-medium columns, which follow the labels
    assert nodal["detected"] == lab["detected"] > 0
    assert np.array_equal(nodal["detp"][:, 0], lab["detp"][:, 0])
    assert np.array_equal(nodal["detp"][:, -1], lab["detp"][:, -1])
    # mus alone from the table: nodemusp is read only with nodemua
    only_mus = oracle_mod.run(m.node, m.elem, m.label, _cfg(m.media, nodemusp=mus), trace=True, normalize=False)
    plain = oracle_mod.run(m.node, m.elem, m.label, _cfg(m.media), trace=True, normalize=False)
    assert np.array_equal(only_mus["photon_weight"], plain["photon_weight"])


def test_nodal_arrays_checked_before_any_gpu_work():
    from mmc_gb300 import _native
    lib = _native.load()
    m = meshgen.homogeneous_cube(n=4)
    d, keep = core._desc(m.node, m.elem, m.label)
    nn = len(m.node)
    e0 = C.c_int32(-1)

    def rc(**kw):
        c, k = SimConfig(media=m.media, srcpos=(30.0, 30.0, 0.0), tend=5e-9, tstep=1e-9, **kw).to_c(nn)
        return lib.mmcgb_check_config(d, C.byref(c), C.byref(e0))

    ok = np.full(nn, 0.01, np.float32)
    assert rc(nodemua=ok) == 0, lib.mmcgb_last_error()
    assert rc(nodemua=ok, nodemusp=ok) == 0
    bad = ok.copy()
    bad[5] = np.nan
    assert rc(nodemua=bad) == 1 and b"finite" in lib.mmcgb_last_error()
    assert rc(nodemua=ok, nodemusp=bad) == 1
    assert rc(nodemusp=bad) == 0  # nodemusp alone is not read
    with pytest.raises(ValueError, match="one value per node"):
        rc(nodemua=ok[:-1])


def test_pmmc_nodal_keys():
    m = meshgen.homogeneous_cube(n=4)
    nn = len(m.node)
    base = dict(node=m.node, elem=m.elem, prop=m.media, srcpos=[30, 30, 0])
    *_, sc, _ = pmmc._parse(dict(base, nodemua=np.full(nn, 0.02), nodemusp=np.full(nn, 1.5)))
    assert sc.nodemua.dtype == np.float32 and sc.nodemua.shape == (nn,) and sc.nodemusp[0] == np.float32(1.5)
    # the array switches the mode on, whatever the flag says (src/pmmc.cpp:651)
    *_, sc, _ = pmmc._parse(dict(base, isnodalmua=0, nodemua=np.full(nn, 0.02)))
    assert sc.nodemua is not None
    for flag in ("isnodalmua", "isnodalmusp"):
        with pytest.raises(ValueError, match=flag):
            pmmc._parse(dict(base, **{flag: 1}))
