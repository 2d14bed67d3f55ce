"""Replay and the replay Jacobians.

* Replay identity (the reference's own check, matlab/mmcjmua.m:55-60): the
  detected photons, re-traced from their saved seeds, are detected again with
  identical records.
* dL/dmua and dL/dmus of L = sum_d c_d log W_d from one replay pair, on
  element groups (each group relabelled as its own copy of its layer's
  medium).  Changing mua does not change photon paths, so the mua gradient
  must match central finite differences (+-1%, common random numbers) closely.
  The summed mus Jacobian of a group must equal the medium derivative built
  from the saved per-medium scattering counts and path lengths; that
  derivative is checked against finite differences statistically.
"""
import dataclasses

import numpy as np
import pytest

from mmc_gb300 import io, meshgen
from mmc_gb300 import replay as rp
from mmc_gb300.core import Mesh, SimConfig, simulate

pytestmark = pytest.mark.gpu

CENTER = np.array([30.0, 30.0, 30.0])


def _det():
    th = np.deg2rad([10.0, 20.0, 30.0, 40.0])
    return np.array([[*(CENTER + 25.0 * np.array([np.sin(a), 0.0, -np.cos(a)])), 3.0] for a in th], np.float32)


def _make_groups(m, ngroups, radius, layers, seed):
    cen = meshgen.centroids(m.node, m.elem)
    rng = np.random.default_rng(seed)
    label = m.label.copy()
    media = [row for row in m.media]
    groups = []
    for g in range(ngroups):
        a = np.deg2rad(rng.uniform(5, 40))
        p = CENTER + rng.uniform(21.0, 24.0) * np.array([np.sin(a), 0.0, -np.cos(a)])
        near = np.nonzero((np.linalg.norm(cen - p, axis=1) < radius) & np.isin(label, layers))[0]
        lay = np.bincount(label[near]).argmax()
        sel = near[label[near] == lay]
        new = len(media)
        media.append(m.media[lay].copy())
        label[sel] = new
        groups.append(new)
    return label, np.array(media, np.float32), groups


@pytest.fixture(scope="module")
def grouped(gpu_ready):
    """Shell mesh (2 mm voxels) with 8 element groups near the surface under the
    detectors, each relabelled 5..12 with a copy of its layer's medium."""
    m = meshgen.shell_mesh(n=30, jitter=0.3, seed=6)
    label, media, groups = _make_groups(m, 8, 3.0, [1, 2, 3, 4], 11)
    return m, Mesh(m.node, m.elem, label), label, media, groups


def _cfg(media, n, **kw):
    base = dict(media=media, nphoton=n, seed=5, srcpos=(30.0, 30.0, 5.5), tend=5e-9, tstep=5e-9, issavedet=1,
                issaveseed=1, detpos=_det(), maxdetphoton=2_000_000, basisorder=0, isnormalized=0, minenergy=0.0)
    base.update(kw)
    return SimConfig(**base)


def _loss(res, media, c):
    w = rp.detected_weight(res.detp, media).astype(np.float64)
    ids = res.detp[:, 0].astype(int)
    W = np.array([w[ids == d + 1].sum() for d in range(len(c))])
    return float(np.sum(c * np.log(W)))


def test_replay_reproduces_detected_photons(grouped, tmp_path):
    m, mesh, label, media, groups = grouped
    cfg = _cfg(media, 200_000)
    fwd = simulate(mesh, cfg)
    assert fwd.detected > 100
    # through the .mch file, as a reference user would
    path = str(tmp_path / "run.mch")
    io.write_mch(path, fwd.detp, fwd.seeds, maxmedia=len(media) - 1, detnum=4, totalphoton=cfg.nphoton,
                 detected=fwd.detected)
    detp, hdr, seeds = io.read_mch(path)
    assert hdr["savedphoton"] == fwd.detected and seeds.shape == (fwd.detected, 16)
    s, w, t, idx = rp.replay_inputs(detp, seeds, media, 0, cfg.tstart, cfg.tend)
    rcfg = dataclasses.replace(cfg, nphoton=len(idx), replayseed=s, replayweight=w, replaytime=t, outputtype="wl")
    rep = simulate(mesh, rcfg)
    rows = lambda d: sorted(map(bytes, d.view(np.uint8).reshape(len(d), -1)))
    assert rep.detected == len(idx)
    assert rows(rep.detp) == rows(detp[idx])
    # wl = replay weight x path length: summed over elements it equals sum_p w_p * (total path of p)
    M = len(media) - 1
    total_path = detp[idx][:, 1 + M:1 + 2 * M].astype(np.float64).sum(1)
    assert rep.field.sum() == pytest.approx(float((w.astype(np.float64) * total_path).sum()), rel=1e-4)


def test_mua_gradient_matches_central_differences(grouped):
    m, mesh, label, media, groups = grouped
    c = np.array([0.7, -1.2, 0.4, 1.1])
    cfg = _cfg(media, 300_000)
    fwd = simulate(mesh, cfg)
    L, W, gmua, gmus = rp.loss_and_grads(mesh, cfg, fwd.detp, fwd.seeds, c)
    for g in groups:
        dm = 0.01 * media[g, 0]
        mp, mm = media.copy(), media.copy()
        mp[g, 0] += dm
        mm[g, 0] -= dm
        fd = (_loss(simulate(mesh, dataclasses.replace(cfg, media=mp)), mp, c)
              - _loss(simulate(mesh, dataclasses.replace(cfg, media=mm)), mm, c)) / (2 * dm)
        an = float(gmua[label == g].sum())
        assert an == pytest.approx(fd, rel=2e-3, abs=1e-6 * max(1.0, abs(L))), (g, an, fd)


def _medium_mus_lr(detp, media, c, g):
    """dL/dmus of medium g from the detected records alone: each record holds
    the photon's scattering count and path length per medium, so
    dW_d/dmus_g = sum_p w_p (nscat_pg / mus_g - ppath_pg)."""
    M = len(media) - 1
    w = rp.detected_weight(detp, media).astype(np.float64)
    ids = detp[:, 0].astype(int)
    a = detp[:, g].astype(np.float64) / float(media[g, 1]) - detp[:, M + g].astype(np.float64)
    return float(sum(c[d] * (w[ids == d + 1] * a[ids == d + 1]).sum() / w[ids == d + 1].sum() for d in range(len(c))))


@pytest.fixture(scope="module")
def scattering_groups(gpu_ready):
    """Six large element groups (6 mm spheres) in the two strongly scattering
    layers (mus 8.6 and 7.8 /mm) under the detectors."""
    m = meshgen.shell_mesh(n=30, jitter=0.3, seed=6)
    label, media, groups = _make_groups(m, 6, 6.0, [3, 4], 12)
    return Mesh(m.node, m.elem, label), label, media, groups


def test_mus_jacobian_sums_to_medium_derivative(scattering_groups):
    """Summed over a group, the replayed scatter-count deposits (wn) equal the
    saved per-medium scattering counts of the same detected photons and the
    path deposits (wl) equal their saved partial path lengths, each weighted by
    the replay weight.  J_mus = wn/mus - wl is a small difference of two large
    sums, so the composed gradient is checked against a tolerance scaled by
    the sums themselves."""
    mesh, label, media, groups = scattering_groups
    c = np.array([0.7, -1.2, 0.4, 1.1])
    cfg = _cfg(media, 500_000)
    fwd = simulate(mesh, cfg)
    M = len(media) - 1
    w = rp.detected_weight(fwd.detp, media).astype(np.float32)
    wl, idx = rp.replay(mesh, cfg, fwd.detp, fwd.seeds, "wl", weight=w)
    wn, _ = rp.replay(mesh, cfg, fwd.detp, fwd.seeds, "wn", weight=w)
    d = fwd.detp[idx].astype(np.float64)
    wr = w[idx].astype(np.float64)
    for g in groups:
        assert wn.field[:, label == g].sum() == pytest.approx((wr * d[:, g]).sum(), rel=1e-6), g
        assert wl.field[:, label == g].sum() == pytest.approx((wr * d[:, M + g]).sum(), rel=1e-3), g
    L, W, gmua, gmus = rp.loss_and_grads(mesh, cfg, fwd.detp, fwd.seeds, c)
    ids = fwd.detp[:, 0].astype(int)
    coef = np.abs(np.array([c[i - 1] / W[i - 1] for i in ids])) * w.astype(np.float64)
    for g in groups:
        scale = (coef * (fwd.detp[:, g] / media[g, 1] + fwd.detp[:, M + g])).sum()
        lr = _medium_mus_lr(fwd.detp, media, c, g)
        assert abs(float(gmus[label == g].sum()) - lr) < 1e-3 * scale, g


def test_mus_gradient_agrees_with_central_differences(scattering_groups):
    """Changing mus moves the scattering points, so paths past the first
    changed segment are re-randomized even with common random numbers and the
    difference quotient is noisy; the likelihood-ratio estimate is noisy too.
    Both are averaged over independent seeds and compared within four
    combined standard errors, with the errors required to be small against
    the signal so that the comparison has power."""
    mesh, label, media, groups = scattering_groups
    c = np.array([0.7, -1.2, 0.4, 1.1])
    K = 4
    an = np.zeros((K, len(groups)))
    fd = np.zeros((K, len(groups)))
    for k in range(K):
        cfg = _cfg(media, 1_000_000, seed=100 + k, issaveseed=0)
        fwd = simulate(mesh, cfg)
        for j, g in enumerate(groups):
            an[k, j] = _medium_mus_lr(fwd.detp, media, c, g)
            ds = 0.05 * media[g, 1]
            mp, mm = media.copy(), media.copy()
            mp[g, 1] += ds
            mm[g, 1] -= ds
            fd[k, j] = (_loss(simulate(mesh, dataclasses.replace(cfg, media=mp)), mp, c)
                        - _loss(simulate(mesh, dataclasses.replace(cfg, media=mm)), mm, c)) / (2 * ds)
    se = np.sqrt(an.var(0, ddof=1) / K + fd.var(0, ddof=1) / K)
    print("dL/dmus likelihood ratio:", an.mean(0), "central differences:", fd.mean(0), "se:", se)
    assert np.all(np.abs(an.mean(0) - fd.mean(0)) < 4 * se + 1e-3 * np.abs(fd.mean(0)))
    assert np.median(se) < 0.5 * np.abs(fd.mean(0)).max()
    assert np.corrcoef(an.mean(0), fd.mean(0))[0, 1] > 0.8


@pytest.mark.parametrize("outputtype", ["wl", "wp", "jacobian", "wn"])
def test_replay_outputs_match_oracle(oracle_mod, gpu_ready, outputtype):
    """The replay deposits (the reference's -O L / P / J and the scatter-count
    replay) against the oracle's replay of the same seeds, weights and times
    (IEEE arithmetic): equal up to the order of the atomic additions."""
    m = meshgen.inclusion_cube(n=12, jitter=0.4, seed=3)
    mesh = Mesh(m.node, m.elem, m.label)
    det = np.array([[40, 30, 0, 3], [45, 30, 0, 3]], np.float32)
    cfg = SimConfig(media=m.media, nphoton=40000, seed=8, srcpos=(30.0, 30.0, 0.0), tend=5e-9, tstep=1e-9,
                    issavedet=1, issaveseed=1, detpos=det, maxdetphoton=100000, basisorder=0, isnormalized=0,
                    fast_math=0)
    fwd = simulate(mesh, cfg)
    assert fwd.detected > 50
    s, w, t, idx = rp.replay_inputs(fwd.detp, fwd.seeds, np.asarray(cfg.media), 1, cfg.tstart, cfg.tend)
    rcfg = dataclasses.replace(cfg, nphoton=len(idx), replayseed=s, replayweight=w, replaytime=t,
                               outputtype=outputtype, photon_offset=0)
    g = simulate(mesh, rcfg)
    o = oracle_mod.run(m.node, m.elem, m.label, rcfg, nthreads=4, normalize=False)
    assert g.field.sum() > 0
    np.testing.assert_allclose(g.field, o["raw"], rtol=1e-8, atol=1e-12 * np.abs(o["raw"]).max())
    assert g.raytet == o["raytet"]


# ---- against the reference's own replay --------------------------------------------------

def test_replay_jacobian_outputs_match_reference_replays(gpu_ready):
    """The differentiation workload (4-layer shell mesh, 1.296M tets, pencil
    (30,30,5.5) +z, 8 detectors R=1.5 mm, 1e6 photons, one 5 ns gate, no
    roulette): a forward run and the replay of its detected photons give the
    raw wl (replay weight x path length) and wp (x mus / slen0) deposits.  The
    reference engine did the same 10 times (forward, then -E run.mch -O L / -O P,
    tests/golden/replay_shell.npz); this run must score like a fresh reference
    run on the per-element deposits, and the totals and detected counts must lie
    within the reference's run-to-run spread."""
    import golden_checks as gc
    fx = gc.load("replay_shell")
    m = meshgen.shell_mesh(n=60, jitter=0.25, seed=4321)
    mesh = Mesh(m.node, m.elem, m.label)
    cfg = SimConfig(media=m.media, nphoton=int(fx["photons"]), seed=20261204, srcpos=(30.0, 30.0, 5.5),
                    srcdir=(0.0, 0.0, 1.0), tend=5e-9, tstep=5e-9, issavedet=1, issaveseed=1,
                    detpos=fx["detectors"], maxdetphoton=2_000_000, basisorder=0, isnormalized=0, minenergy=0.0)
    fwd = simulate(mesh, cfg)
    msgs = []
    n, nm, ns = fwd.detected, fx["ndet"].mean(), fx["ndet"].std(ddof=1)
    if abs(n - nm) > 3.5 * ns * gc.INFLATE:
        msgs.append(f"detected {n} vs reference {nm:.0f} +- {ns:.0f}")
    for key in ("wl", "wp"):
        rep, idx = rp.replay(mesh, cfg, fwd.detp, fwd.seeds, outputtype=key)
        assert len(idx) == fwd.detected and rep.detected == len(idx)  # every photon retraced to its detector
        x = rep.field.sum(0)
        msgs += gc._zcheck(f"{key} per element", x[fx[key + "_sub"]], fx[key + "_mean"], fx[key + "_std"], 100,
                           fx["null_" + key + "_frac"], fx["null_" + key + "_meanz"])
        t, tm, ts = x.sum(), fx[key + "_total"].mean(), fx[key + "_total"].std(ddof=1)
        if abs(t - tm) > 3.5 * ts * gc.INFLATE:
            msgs.append(f"{key} total {t:.5g} vs reference {tm:.5g} +- {ts:.3g}")
    assert not msgs, "\n".join(msgs)


def test_replay_loss_autograd_function(gpu_ready):
    """ReplayLoss, the torch.autograd.Function of L = sum_d c_d log W_d, on the
    differentiation workload's mesh (4-layer shells, 1.296M tets, 8 detectors):
    its value and backward() gradients per medium equal loss_and_grads summed
    over each medium's elements, and dL/dmua per medium agrees with central
    differences (+-1%, common random numbers: absorption does not move any
    photon, so the difference quotient is smooth)."""
    import torch
    fx_det = np.array([[*(CENTER + 25.0 * np.array([np.sin(a), 0.0, -np.cos(a)])), 1.5]
                       for a in np.deg2rad(np.arange(10, 90, 10))], np.float32)
    m = meshgen.shell_mesh(n=60, jitter=0.25, seed=4321)
    mesh = Mesh(m.node, m.elem, m.label)
    cfg = SimConfig(media=m.media, nphoton=1_000_000, seed=77, srcpos=(30.0, 30.0, 5.5), srcdir=(0.0, 0.0, 1.0),
                    tend=5e-9, tstep=5e-9, issavedet=1, issaveseed=1, detpos=fx_det, maxdetphoton=2_000_000,
                    basisorder=0, isnormalized=0, minenergy=0.0)
    c = np.random.default_rng(3).normal(size=len(fx_det))
    mua = torch.tensor(m.media[:, 0].astype(np.float64), requires_grad=True)
    mus = torch.tensor(m.media[:, 1].astype(np.float64), requires_grad=True)
    L = rp.ReplayLoss.apply(mesh, cfg, c, mua, mus)
    L.backward()
    # the same forward and replays through the plain API
    fwd = simulate(mesh, cfg)
    L2, W, gmua, gmus = rp.loss_and_grads(mesh, cfg, fwd.detp, fwd.seeds, c)
    nmed = m.media.shape[0]
    assert float(L.detach()) == pytest.approx(L2, rel=1e-9)
    np.testing.assert_allclose(mua.grad.numpy(), np.bincount(m.label, gmua, nmed), rtol=1e-6, atol=1e-9)
    np.testing.assert_allclose(mus.grad.numpy(), np.bincount(m.label, gmus, nmed), rtol=1e-6, atol=1e-9)
    assert mua.grad[0] == 0 and np.all(mua.grad.numpy()[1:] != 0)
    # dL/dmua per layer against central differences of the loss itself
    for k in range(1, nmed):
        d = 0.01 * float(m.media[k, 0])
        vals = []
        for sgn in (1.0, -1.0):
            t = mua.detach().clone()
            t[k] += sgn * d
            vals.append(float(rp.ReplayLoss.apply(mesh, cfg, c, t, mus.detach())))
        fd = (vals[0] - vals[1]) / (2 * d)
        g = float(mua.grad[k])
        assert g == pytest.approx(fd, rel=5e-3, abs=1e-4 * abs(float(L.detach())) + 1e-6), (k, g, fd)


def test_mua_gradient_on_50_element_groups_of_the_differentiation_workload(gpu_ready):
    """The differentiation workload as specified: the 4-layer shell mesh (1 mm
    grid, 1.296M tets), pencil (30,30,5.5) +z, 8 detectors R=1.5 mm at polar
    angles 10..80 degrees, 1e7 photons with saved seeds, L = sum_d c_d log W_d
    with c_d ~ N(0,1).  50 element groups (2 mm spheres at random places between
    the source and the detectors, each relabelled as its own copy of its
    layer's medium): dL/dmua of each group from one replay pair equals the
    central difference (+-1%, common random numbers) of two forward runs."""
    m = meshgen.shell_mesh(n=60, jitter=0.25, seed=4321)
    cen = meshgen.centroids(m.node, m.elem)
    rng = np.random.default_rng(50)
    label = m.label.copy()
    media = [row for row in m.media]
    groups = []
    while len(groups) < 50:
        a = np.deg2rad(rng.uniform(2.0, 80.0))
        p = CENTER + rng.uniform(18.5, 24.5) * np.array([np.sin(a), rng.uniform(-0.1, 0.1), -np.cos(a)])
        near = np.nonzero((np.linalg.norm(cen - p, axis=1) < 2.0) & np.isin(label, [1, 2, 3, 4]))[0]
        if near.size < 4:
            continue
        lay = np.bincount(label[near]).argmax()
        label[near[label[near] == lay]] = len(media)
        groups.append(len(media))
        media.append(m.media[lay].copy())
    media = np.array(media, np.float32)
    mesh = Mesh(m.node, m.elem, label)
    det = np.array([[*(CENTER + 25.0 * np.array([np.sin(a), 0.0, -np.cos(a)])), 1.5]
                    for a in np.deg2rad(np.arange(10, 90, 10))], np.float32)
    cfg = _cfg(media, 10_000_000, seed=31, detpos=det, maxdetphoton=5_000_000)
    c = np.random.default_rng(3).normal(size=len(det))
    fwd = simulate(mesh, cfg)
    L, W, gmua, gmus = rp.loss_and_grads(mesh, cfg, fwd.detp, fwd.seeds, c)
    assert np.all(W > 0)
    an, fd = [], []
    for g in groups:
        dm = 0.01 * media[g, 0]
        mp, mm = media.copy(), media.copy()
        mp[g, 0] += dm
        mm[g, 0] -= dm
        lp = _loss(simulate(mesh, dataclasses.replace(cfg, media=mp, issaveseed=0)), mp, c)
        lm = _loss(simulate(mesh, dataclasses.replace(cfg, media=mm, issaveseed=0)), mm, c)
        fd.append((lp - lm) / (2 * dm))
        an.append(float(gmua[label == g].sum()))
    an, fd = np.array(an), np.array(fd)
    scale = np.abs(fd).max()
    print(f"dL/dmua on 50 groups: max |grad| {scale:.3e}, max |analytic - central| {np.abs(an - fd).max():.3e}")
    assert scale > 0 and np.count_nonzero(np.abs(fd) > 1e-3 * scale) >= 10  # the groups see light
    np.testing.assert_allclose(an, fd, rtol=2e-3, atol=1e-4 * scale)
