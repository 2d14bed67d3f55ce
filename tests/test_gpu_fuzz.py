"""Randomized differential test of the CUDA engine against the CPU oracle.

Seeded random configurations cross the options the dedicated tests cover one
at a time: meshes with void layers and inclusions, media (zero absorption,
index mismatches), boundary conditions, gate counts (one gate: roulette on),
sources, patterns sharing photons, detectors with exit/momentum columns and
seeds, float32 or float64 accumulation, element or dual-grid output, the
exiting weight per face, per-node mua/mus and gate-phased tracing.  With IEEE arithmetic every
photon must end as the oracle's (weight bits, ray-tet tests, detector), and the
deposits, records and tallies must agree, through the general kernels (per-photon
tracing on) and through the kernels the configuration selects otherwise.
"""

import dataclasses

import numpy as np
import pytest

from mmc_gb300 import _native, meshgen
from mmc_gb300.core import Mesh, SimConfig, simulate

pytestmark = pytest.mark.gpu

NCASES = 64


def _meshes():
    cube = meshgen.homogeneous_cube(n=10)
    void = cube.label.copy()
    void[meshgen.centroids(cube.node, cube.elem)[:, 2] < 6.0] = 0
    incl = meshgen.inclusion_cube(n=10, jitter=1.0, seed=3)
    shell = meshgen.shell_mesh(n=10, jitter=1.0, seed=5)
    return {"cube": cube, "void": meshgen.Mesh(cube.node, cube.elem, void, cube.media, "void"),
            "incl": incl, "shell": shell}


@pytest.fixture(scope="module")
def fuzz_meshes(gpu_ready):
    return {k: (m, Mesh(m.node, m.elem, m.label)) for k, m in _meshes().items()}


def _case(k):
    rng = np.random.default_rng(1000 + k)
    name = ["cube", "void", "incl", "shell"][k % 4]
    kw = dict(nphoton=1500, seed=int(rng.integers(1, 2**31)), fast_math=0, basisorder=0, isnormalized=0)
    kw["nout"] = float(rng.choice([1.0, 1.37]))
    kw["isreflect"] = int(rng.integers(0, 4))
    kw["isspecular"] = int(rng.integers(0, 2))
    kw["voidtime"] = int(rng.integers(0, 2))
    kw["tstep"] = float(rng.choice([5e-9, 1e-9, 0.5e-9]))
    kw["tend"] = 5e-9
    kw["accum_f64"] = int(rng.integers(0, 2))
    kw["outputtype"] = str(rng.choice(["flux", "fluence", "energy"]))
    # the source: on the z=0 face (void layer: over it) or inside
    if name == "void":
        st = str(rng.choice(["pencil", "disk", "planar", "gaussian", "pattern"]))
        kw.update(srctype=st, srcpos=(20.0 + rng.uniform(0, 5), 20.0, 0.0), srcdir=(0.0, 0.0, 1.0))
        if st == "disk":
            kw["srcparam1"] = (float(rng.uniform(2, 10)), 0, 0, 0)
        elif st == "gaussian":
            kw["srcparam1"] = (float(rng.uniform(2, 6)), 0, 0, 0)
        elif st == "planar":
            kw.update(srcparam1=(15.0, 0, 0, 0), srcparam2=(0, 15.0, 0, 0))
        elif st == "pattern":
            K = int(rng.integers(1, 4))
            kw.update(srcparam1=(15.0, 0, 0, 3), srcparam2=(0, 15.0, 0, 2), srcnum=K,
                      srcpattern=rng.uniform(0.1, 1.0, 6 * K).astype(np.float32))
    elif rng.random() < 0.5:
        kw.update(srctype="pencil", srcpos=(30.0, 30.0, 0.0), srcdir=(0.0, 0.0, 1.0))
    else:
        st = str(rng.choice(["isotropic", "cone", "pencil"]))
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        kw.update(srctype=st, srcpos=tuple(float(x) for x in rng.uniform(22, 38, 3)), srcdir=tuple(float(x) for x in d))
        if st == "cone":
            kw["srcparam1"] = (float(rng.uniform(0.1, 1.0)), 0, 0, 0)
    # detectors on the z=0 face, with the record options
    ndet = int(rng.integers(0, 4))
    if ndet:
        kw["detpos"] = np.array([[rng.uniform(10, 50), rng.uniform(10, 50), 0.0, rng.uniform(3, 8)]
                                 for _ in range(ndet)], np.float32)
        kw.update(issavedet=1, maxdetphoton=5000, issaveseed=int(rng.integers(0, 2)),
                  issaveexit=int(rng.integers(0, 2)), ismomentum=int(rng.integers(0, 2)))
    kw["issaveref"] = int(rng.random() < 0.3)
    if rng.random() < 0.25:
        kw.update(method="grid", gridstep=float(rng.choice([2.0, 3.0])))
    gates = int(round(kw["tend"] / kw["tstep"]))
    kw["phased"] = int(rng.choice([-1, 2])) if gates > 2 else -1
    return name, kw, rng


def _nodal(k, m):
    """Per-node mua (and mus) for a fifth of the cases, from a stream of their own
    so that the other draws of a case stay as they are."""
    rng = np.random.default_rng(5000 + k)
    if rng.random() >= 0.2:
        return {}
    nn = len(m.node)
    out = dict(nodemua=rng.uniform(0.0, 0.05, nn).astype(np.float32))
    if rng.random() < 0.5:
        out["nodemusp"] = rng.uniform(0.2, 5.0, nn).astype(np.float32)
    return out


def _media(m, rng):
    media = np.array(m.media, np.float32).copy()
    for r in range(1, media.shape[0]):
        media[r] = (rng.choice([0.0, rng.uniform(0.001, 0.05)]), rng.uniform(0.2, 5.0), rng.uniform(0.0, 0.95),
                    rng.choice([1.0, 1.37, 1.45]))
    return media


def _rows(detp, seeds):
    if detp is None or len(detp) == 0:
        return []
    a = detp.view(np.uint8).reshape(len(detp), -1)
    if seeds is not None:
        a = np.concatenate([a, seeds], 1)
    return sorted(map(bytes, a))


@pytest.mark.parametrize("k", range(NCASES))
def test_random_configuration_matches_oracle(oracle_mod, fuzz_meshes, k):
    name, kw, rng = _case(k)
    m, mesh = fuzz_meshes[name]
    cfg = SimConfig(media=_media(m, rng), **kw, **_nodal(k, m))
    # float32 sums depend on the order of the additions; float64 ones hardly
    tol = dict(rtol=1e-7, atol=1e-9) if cfg.accum_f64 else dict(rtol=3e-5, atol=1e-6)
    try:
        o = oracle_mod.run(m.node, m.elem, m.label, cfg, nthreads=4, trace=True, normalize=False)
    except ValueError:
        o = None
    if o is None or o["outside"]:
        # a source the oracle cannot place (outside the mesh): the engine reports it as an error
        with pytest.raises(_native.MmcgbError):
            simulate(mesh, cfg, trace=True)
        return
    g = simulate(mesh, cfg, trace=True)
    assert np.array_equal(g.photon_weight.view(np.uint32), o["photon_weight"].view(np.uint32)), kw
    assert np.array_equal(g.photon_steps, o["photon_steps"])
    assert np.array_equal(g.photon_det, o["photon_det"])
    assert g.raytet == o["raytet"] and g.aborted == o["aborted"] == 0
    np.testing.assert_allclose(g.field, o["raw"], **tol)
    assert g.energytot == pytest.approx(o["energytot"], rel=1e-6)
    assert g.energyesc == pytest.approx(o["energyesc"], rel=1e-6, abs=1e-6)
    if cfg.issavedet:
        assert g.detected == o["detected"]
        assert _rows(g.detp, g.seeds) == _rows(o["detp"], o["seeds"])
    if cfg.issaveref:
        np.testing.assert_allclose(g.dref, o["dref"], rtol=1e-7, atol=1e-9)
    # the kernels the configuration selects without per-photon tracing give the same deposits
    f = simulate(mesh, cfg)
    np.testing.assert_allclose(f.field, o["raw"], **tol)
    assert f.raytet == o["raytet"]
    if cfg.issavedet:
        assert _rows(f.detp, f.seeds) == _rows(o["detp"], o["seeds"])


def test_random_configurations_batched_equal_solo_runs(fuzz_meshes):
    """Sixteen of the random configurations (four meshes, mixed options) in one
    batched launch: each result equals its solo run."""
    from mmc_gb300.core import simulate_batch
    meshes, cfgs, solo = [], [], []
    for k in range(16):
        name, kw, rng = _case(k)
        m, mesh = fuzz_meshes[name]
        cfg = SimConfig(media=_media(m, rng), **kw)
        try:
            solo.append(simulate(mesh, cfg))
        except _native.MmcgbError:  # a source outside the mesh: not batched
            continue
        cfgs.append(cfg)
        meshes.append(mesh)
    assert len(cfgs) >= 12
    batch = simulate_batch(meshes, cfgs)
    for k, (cfg, b, s) in enumerate(zip(cfgs, batch, solo)):
        tol = dict(rtol=1e-7, atol=1e-9) if cfg.accum_f64 else dict(rtol=3e-5, atol=1e-6)
        np.testing.assert_allclose(b.field, s.field, **tol, err_msg=f"case {k}")
        assert b.raytet == s.raytet and b.detected == s.detected, k
        if cfg.issavedet:
            assert _rows(b.detp, b.seeds) == _rows(s.detp, s.seeds), k
        if cfg.issaveref:
            np.testing.assert_allclose(b.dref, s.dref, rtol=1e-7, atol=1e-9)


@pytest.mark.parametrize("k", range(0, NCASES, 4))
def test_fast_policy_launch_forms_agree(fuzz_meshes, k):
    """With the fast arithmetic policy the plain, gate-phased and batched kernels,
    and a simulation split into two launches, compute the same photons: equal
    ray-tet counts and records, deposits equal up to summation order."""
    from mmc_gb300.core import Session, simulate_batch
    name, kw, rng = _case(k)
    m, mesh = fuzz_meshes[name]
    cfg = SimConfig(media=_media(m, rng), **dict(kw, fast_math=1, nphoton=4000))
    tol = dict(rtol=1e-7, atol=1e-9) if cfg.accum_f64 else dict(rtol=3e-5, atol=1e-6)
    try:
        ref = simulate(mesh, dataclasses.replace(cfg, phased=-1))
    except _native.MmcgbError:
        return  # a source outside the mesh
    runs = [simulate_batch([mesh], [cfg])[0]]
    if cfg.maxgate > 2:
        runs.append(simulate(mesh, dataclasses.replace(cfg, phased=1)))
    s = Session(mesh, cfg)
    s.launch(0, 1500)
    s.launch(1500, 2500)
    s.sync()
    runs.append(s.end())
    for r in runs:
        assert r.raytet == ref.raytet and r.detected == ref.detected
        np.testing.assert_allclose(r.field, ref.field, **tol)
        if cfg.issavedet:
            assert _rows(r.detp, r.seeds) == _rows(ref.detp, ref.seeds)


@pytest.mark.parametrize("k", range(0, NCASES, 3))
@pytest.mark.parametrize("outputtype", ["wl", "wp", "jacobian", "wn"])
def test_random_replays_match_oracle(oracle_mod, fuzz_meshes, k, outputtype):
    """The replay of a random configuration's detected photons (their seeds,
    weights and times) deposits what the oracle's replay does (IEEE arithmetic)."""
    from mmc_gb300 import replay as rp
    name, kw, rng = _case(k)
    m, mesh = fuzz_meshes[name]
    det = np.array([[30.0, 30.0, 0.0, 25.0], [30.0, 30.0, 60.0, 25.0]], np.float32)
    kw = dict(kw, issavedet=1, issaveseed=1, detpos=det, maxdetphoton=20000, issaveexit=0, ismomentum=0,
              method="elem", issaveref=0, phased=-1, accum_f64=1, nphoton=4000, srcnum=1)
    if kw.get("srctype") == "pattern":
        kw.update(srcpattern=np.asarray(kw["srcpattern"])[:6])
    cfg = SimConfig(media=_media(m, rng), **kw)
    try:
        fwd = simulate(mesh, cfg)
    except _native.MmcgbError:
        return  # a source outside the mesh
    if fwd.detected < 5:
        return
    s, w, t, idx = rp.replay_inputs(fwd.detp, fwd.seeds, np.asarray(cfg.media), 0, cfg.tstart, cfg.tend)
    rcfg = dataclasses.replace(cfg, nphoton=len(idx), replayseed=s, replayweight=w, replaytime=t,
                               outputtype=outputtype, photon_offset=0)
    g = simulate(mesh, rcfg)
    o = oracle_mod.run(m.node, m.elem, m.label, rcfg, nthreads=4, normalize=False)
    assert g.raytet == o["raytet"]
    np.testing.assert_allclose(g.field, o["raw"], rtol=1e-7, atol=1e-12 * max(1.0, np.abs(o["raw"]).max()))
