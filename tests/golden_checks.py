"""Statistical parity checks against the reference golden fixtures
(tests/golden/*.npz, made by tests/golden/make_golden.py from 10 runs of the
reference CPU engine).  Shared by the oracle tests (CPU) and the engine tests
(GPU).

A single run with the fixture's photon count is an independent sample; its
difference from the 10-run mean has variance sigma^2 (1 + 1/10), sigma being
the run-to-run spread of the reference.  With sigma estimated from 10 runs,
z = diff / (s sqrt(1.1)) follows Student's t with 9 degrees of freedom, so a
Gaussian run would put 98.5% of the well-sampled cells inside 3 sigma (not the
99.7% of a known sigma), and sparsely visited cells have heavier tails still.
So the thresholds are calibrated on the reference itself: the fixtures hold
the coverage and mean z of six fresh reference runs scored the same way, and a
candidate run passes when it scores like them (see _zcheck); aggregate
quantities must lie within 3 sigma.
"""
import dataclasses
import os

import numpy as np

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
INFLATE = np.sqrt(1.0 + 1.0 / 10.0)


def load(name):
    return dict(np.load(os.path.join(HERE, name + ".npz")))


def case_mesh_and_config(name, nphoton=None, seed=4242):
    from mmc_gb300 import meshgen
    from mmc_gb300.core import SimConfig
    fx = load(name)
    if name == "cube6k":
        m = meshgen.homogeneous_cube(n=10)
        cfg = SimConfig(media=m.media, nphoton=nphoton or int(fx["photons"]), seed=seed, srcpos=(30.0, 30.0, 0.0),
                        srcdir=(0.0, 0.0, 1.0), tend=5e-9, tstep=5e-9, basisorder=0, isnormalized=0)
    elif name == "incl48k":
        m = meshgen.inclusion_cube(n=20, jitter=0.6, seed=7)
        cfg = SimConfig(media=m.media, nphoton=nphoton or int(fx["photons"]), seed=seed, srcpos=(30.0, 30.0, 0.0),
                        srcdir=(0.0, 0.0, 1.0), tend=5e-9, tstep=0.5e-9, basisorder=0, isnormalized=0, issavedet=1,
                        detpos=meshgen.c1_detectors(), maxdetphoton=200000)
    elif name == "c0_cube162k":
        # the 162k-tet benchmark cube: 30^3 voxels at 2 mm, one 5 ns gate
        m = meshgen.homogeneous_cube(n=30)
        cfg = SimConfig(media=m.media, nphoton=nphoton or int(fx["photons"]), seed=seed, srcpos=(30.0, 30.0, 0.0),
                        srcdir=(0.0, 0.0, 1.0), tend=5e-9, tstep=5e-9, basisorder=0, isnormalized=0)
    elif name == "c1_incl1296k":
        # the 1.296M-tet benchmark workload: 50 gates of 0.1 ns, 4 detectors
        m = meshgen.inclusion_cube(n=60, jitter=0.25, seed=12345)
        cfg = SimConfig(media=m.media, nphoton=nphoton or int(fx["photons"]), seed=seed, srcpos=(30.0, 30.0, 0.0),
                        srcdir=(0.0, 0.0, 1.0), tend=5e-9, tstep=1e-10, basisorder=0, isnormalized=0, issavedet=1,
                        detpos=meshgen.c1_detectors(), maxdetphoton=2_000_000)
    elif name == "grid_cube6k":
        m = meshgen.homogeneous_cube(n=10)
        cfg = SimConfig(media=m.media, nphoton=nphoton or int(fx["photons"]), seed=seed, srcpos=(30.0, 30.0, 0.0),
                        srcdir=(0.0, 0.0, 1.0), tend=5e-9, tstep=5e-9, basisorder=0, isnormalized=0, method="grid",
                        gridstep=float(fx["step"]))
    elif name == "dref_cube6k":
        m = meshgen.homogeneous_cube(n=10)
        cfg = SimConfig(media=m.media, nphoton=nphoton or int(fx["photons"]), seed=seed, srcpos=(30.0, 30.0, 0.0),
                        srcdir=(0.0, 0.0, 1.0), tend=5e-9, tstep=1e-9, basisorder=0, isnormalized=0, issaveref=1)
    elif name == "traj_cube6k":
        m = meshgen.homogeneous_cube(n=10)
        cfg = SimConfig(media=m.media, nphoton=nphoton or int(fx["photons"]), seed=seed, srcpos=(30.0, 30.0, 0.0),
                        srcdir=(0.0, 0.0, 1.0), tend=5e-9, tstep=1e-9, basisorder=0, isnormalized=0,
                        maxjumpdebug=int(fx["maxjumpdebug"]))
    elif name.startswith("bench_"):
        # the reference's built-in benchmarks (-Q), dual-grid output on 1 mm voxels
        from mmc_gb300 import io
        d, cfg, _ = io.load_input(io.builtin_benchmark(name[len("bench_"):]))
        m = meshgen.Mesh(d["node"], d["elem"], d["label"], cfg.media, name)
        cfg = dataclasses.replace(cfg, nphoton=nphoton or int(fx["photons"]), seed=seed, isnormalized=0,
                                  method="grid", gridstep=1.0, basisorder=0, issavedet=0)
    elif name == "src_pattern3":
        # three patterns sharing each photon over the void-layer cube6k face; the fixture holds them
        # as [pattern, x, y], the engine takes them pixel-major (pixel y*nx+x, patterns adjacent)
        m = meshgen.homogeneous_cube(n=10)
        label = m.label.copy()
        label[meshgen.centroids(m.node, m.elem)[:, 2] < 6.0] = 0
        m = meshgen.Mesh(m.node, m.elem, label, m.media, "cube6k-void")
        pat = fx["pattern"]
        K, nx, ny = pat.shape
        cfg = SimConfig(media=m.media, nphoton=nphoton or int(fx["photons"]), seed=seed, tend=5e-9, tstep=5e-9,
                        basisorder=0, isnormalized=0, srctype="pattern", srcpos=(20.0, 20.0, 0.0),
                        srcdir=(0.0, 0.0, 1.0), srcparam1=(20.0, 0, 0, nx), srcparam2=(0, 20.0, 0, ny),
                        srcpattern=np.ascontiguousarray(pat.transpose(2, 1, 0)).ravel(), srcnum=K)
    elif name.startswith("src_"):
        # source types (tests/golden/make_golden.py SOURCE_CASES): the cube6k mesh, with the
        # voxel layer z < 6 mm void for the sources on the z=0 face
        m = meshgen.homogeneous_cube(n=10)
        src = {
            "src_isotropic": dict(srctype="isotropic", srcpos=(30.0, 30.0, 30.0), srcdir=(0.0, 0.0, 1.0)),
            "src_cone": dict(srctype="cone", srcpos=(30.0, 30.0, 30.0), srcdir=(0.6, 0.0, 0.8),
                             srcparam1=(0.6, 0, 0, 0)),
            "src_disk": dict(srctype="disk", srcpos=(30.0, 30.0, 0.0), srcdir=(0.0, 0.0, 1.0),
                             srcparam1=(10.0, 0, 0, 0)),
            "src_gaussian": dict(srctype="gaussian", srcpos=(30.0, 30.0, 0.0), srcdir=(0.0, 0.0, 1.0),
                                 srcparam1=(5.0, 0, 0, 0)),
            "src_planar": dict(srctype="planar", srcpos=(20.0, 20.0, 0.0), srcdir=(0.0, 0.0, 1.0),
                               srcparam1=(20.0, 0, 0, 0), srcparam2=(0, 20.0, 0, 0)),
        }[name]
        if src["srcpos"][2] == 0.0:
            label = m.label.copy()
            label[meshgen.centroids(m.node, m.elem)[:, 2] < 6.0] = 0
            m = meshgen.Mesh(m.node, m.elem, label, m.media, "cube6k-void")
        cfg = SimConfig(media=m.media, nphoton=nphoton or int(fx["photons"]), seed=seed, tend=5e-9, tstep=5e-9,
                        basisorder=0, isnormalized=0, **src)
    else:
        raise KeyError(name)
    return m, cfg, fx


def zstats(x, mean, std, rel_noise_max=0.25):
    """(fraction of well-sampled cells with |z| < 3, mean z, cell count)."""
    ok = (mean > 0) & (std > 0) & (std < rel_noise_max * mean)
    z = (x[ok] - mean[ok]) / (std[ok] * INFLATE)
    return float(np.mean(np.abs(z) < 3.0)), float(np.mean(z)) if z.size else 0.0, int(ok.sum())


def _zcheck(what, x, mean, std, nmin, null_frac, null_meanz):
    """Coverage and bias of one run against the thresholds set by fresh
    reference runs (the null): coverage no lower than the worst fresh run
    minus 0.5%, |mean z| no larger than the largest fresh-run value + 0.1."""
    f, mz, n = zstats(x, mean, std)
    need = float(np.min(null_frac)) - 0.005
    mz_max = float(np.max(np.abs(null_meanz))) + 0.1
    if n < nmin or f < need or abs(mz) > mz_max:
        return [f"{what}: {f:.4f} of {n} cells within 3 sigma (need {need:.4f}), mean z {mz:+.3f} "
                f"(limit {mz_max:.3f})"]
    return []


def check_field(raw, fx, media, label, photons):
    """raw: (gates, ne) element deposits of one run.  Fixtures of large meshes
    keep the per-element statistics of a subset of the elements (`esub`)."""
    msgs = []
    per_elem = raw.sum(0)
    if "esub" in fx:
        per_elem = per_elem[fx["esub"]]
    msgs += _zcheck("per-element", per_elem, fx["elem_mean"], fx["elem_std"], 100,
                    fx["null_elem_frac"], fx["null_elem_meanz"])
    msgs += _zcheck("(element,gate) cells", raw.reshape(-1)[fx["cells"]], fx["cell_mean"], fx["cell_std"], 50,
                    fx["null_cell_frac"], fx["null_cell_meanz"])
    gm, gs = fx["gate_mean"], fx["gate_std"]
    gz = np.abs(raw.sum(1) - gm) / (gs * INFLATE)
    if np.any(gz[gm > 0] > 4.0):
        msgs.append(f"per-gate totals z = {np.round(gz, 2)}")
    absorbed = float((raw.sum(0) * media[label, 0].astype(np.float64)).sum() / photons)
    a = fx["absorbed"]
    if abs(absorbed - a.mean()) > 3 * a.std(ddof=1) * INFLATE:
        msgs.append(f"absorbed fraction {absorbed:.5f} vs reference {a.mean():.5f} +- {a.std(ddof=1):.5f}")
    return msgs


def check_patterns(raw, fx):
    """raw: (ne, srcnum) element deposits of one single-gate run whose patterns
    share photons: every (element, pattern) cell and each pattern's total."""
    msgs = _zcheck("(element,pattern) cells", raw.reshape(-1), fx["cell_mean"], fx["cell_std"], 100,
                   fx["null_cell_frac"], fx["null_cell_meanz"])
    tz = np.abs(raw.sum(0) - fx["total_mean"]) / (fx["total_std"] * INFLATE)
    if np.any(tz > 4.0):
        msgs.append(f"per-pattern totals z = {np.round(tz, 2)}")
    return msgs


def check_nodes(node, fx):
    """node: (datalen,) normalized node output of one single-gate run."""
    return _zcheck("per-node", node, fx["node_mean"], fx["node_std"], 100, fx["null_node_frac"],
                   fx["null_node_meanz"])


def check_dref(dref, fx):
    """dref: (gates, nf) raw exiting weight per exterior face of one run."""
    msgs = _zcheck("per-face exiting weight", dref.sum(0), fx["face_mean"], fx["face_std"], 100,
                   fx["null_face_frac"], fx["null_face_meanz"])
    gm, gs = fx["gate_mean"], fx["gate_std"]
    gz = np.abs(dref.sum(1) - gm) / (gs * INFLATE)
    if np.any(gz[gm > 0] > 4.0):
        msgs.append(f"per-gate exiting totals z = {np.round(gz, 2)}")
    return msgs


def check_grid(raw, fx):
    """raw: (gates, voxels) dual-grid deposits of one run."""
    msgs = _zcheck("per-voxel", raw.sum(0), fx["vox_mean"], fx["vox_std"], 100,
                   fx["null_vox_frac"], fx["null_vox_meanz"])
    t = fx["total"]
    if abs(raw.sum() - t.mean()) > 3 * t.std(ddof=1) * INFLATE:
        msgs.append(f"grid total {raw.sum():.1f} vs reference {t.mean():.1f} +- {t.std(ddof=1):.1f}")
    return msgs


# records-per-photon histogram edges of the trajectory statistics
TRAJ_EDGES = np.array([0, 3, 4, 6, 10, 20, 50, 100, 200, 400, 800, 1 << 30])


def traj_stats(traj, nphoton):
    """Statistics of one run's trajectory records (id bits, x, y, z, w, eid
    bits), with every record of the run kept.  A photon's records are in
    order in the buffer (one thread writes them), so a stable sort by photon
    id gives each photon's launch record first and its end record last."""
    ids = traj[:, 0].view(np.uint32)
    order = np.argsort(ids, kind="stable")
    t, ids = traj[order], ids[order]
    cnt = np.bincount(ids, minlength=nphoton).astype(np.float64)
    first = np.r_[0, np.nonzero(np.diff(ids))[0] + 1]
    last = np.r_[first[1:] - 1, len(ids) - 1]
    return dict(
        records_per_photon=cnt.mean(),
        hist=np.histogram(cnt, TRAJ_EDGES)[0] / float(nphoton),
        final_weight=float(t[last, 4].astype(np.float64).mean()),
        escaped=float((t[last, 5].view(np.int32) <= 0).mean()),
        mean_pos=t[:, 1:4].astype(np.float64).mean(0),
        mean_weight=float(t[:, 4].astype(np.float64).mean()),
        launch_pos=t[first, 1:4].astype(np.float64).mean(0),
        launch_weight=float(t[first, 4].astype(np.float64).mean()),
    )


TRAJ_KEYS = ("records_per_photon", "hist", "final_weight", "escaped", "mean_pos", "mean_weight")


def check_traj(traj, nphoton, fx, nsigma=4.0):
    """Trajectory statistics of one run against the reference runs: each
    within nsigma run-to-run deviations, the launch records exact."""
    st = traj_stats(traj, nphoton)
    msgs = []
    for k in TRAJ_KEYS:
        x = np.atleast_1d(st[k])
        runs = fx["traj_" + k].reshape(len(fx["traj_" + k]), -1)   # (runs, values)
        m, s = runs.mean(0), runs.std(0, ddof=1)
        if k == "hist":  # multinomial bin fractions: the binomial sigma, steadier than 10 runs' spread
            s = np.sqrt(m * (1.0 - m) / nphoton)
        ok = s > 0
        z = np.abs(x[ok] - m[ok]) / (s[ok] * INFLATE)
        if np.any(z > nsigma):
            msgs.append(f"trajectory {k}: {np.round(x, 4)} vs reference {np.round(m, 4)} +- {np.round(s, 4)}")
        if np.any(~ok & (x != m)):
            msgs.append(f"trajectory {k}: {np.round(x, 4)} vs constant reference {np.round(m, 4)}")
    if not np.allclose(st["launch_pos"], fx["traj_launch_pos"][0]) or st["launch_weight"] != 1.0:
        msgs.append(f"launch records at {st['launch_pos']} w {st['launch_weight']}")
    return msgs


def check_bench(raw, fx):
    """raw: (gates, voxels) dual-grid deposits of one run of a built-in benchmark."""
    x = raw.sum(0)
    msgs = [] if x.size == int(fx["nvox"]) else [f"grid of {x.size} voxels vs the reference's {int(fx['nvox'])}"]
    if msgs:
        return msgs
    msgs = _zcheck("per-voxel", x[fx["sub"]], fx["vox_mean"], fx["vox_std"], 100,
                   fx["null_vox_frac"], fx["null_vox_meanz"])
    t = fx["total"]
    if abs(x.sum() - t.mean()) > 3 * t.std(ddof=1) * INFLATE:
        msgs.append(f"grid total {x.sum():.1f} vs reference {t.mean():.1f} +- {t.std(ddof=1):.1f}")
    return msgs


def check_tests_per_photon(tpp, fx, rel=0.01, nsigma=4.0):
    """Within `rel` of the reference mean, or nsigma run-to-run deviations
    where the reference's own spread is wider (few, large elements)."""
    t = fx["tests_per_photon"]
    ref = float(t.mean())
    tol = max(rel * ref, nsigma * float(t.std(ddof=1)) * INFLATE)
    return [] if abs(tpp - ref) <= tol else [f"ray-tet tests/photon {tpp:.2f} vs reference {ref:.2f} (tolerance {tol:.2f})"]


def check_detectors(detp, media, fx):
    msgs = []
    M = media.shape[0] - 1
    mua = media[1:, 0].astype(np.float64)
    ids = detp[:, 0].astype(int)
    pp = detp[:, 1 + M:1 + 2 * M].astype(np.float64)
    w = detp[:, -1] * np.exp(-(pp * mua).sum(1))
    ndet = fx["det_count"].shape[1]
    for k in range(ndet):
        cnt = np.count_nonzero(ids == k + 1)
        cm, cs = fx["det_count"][:, k].mean(), fx["det_count"][:, k].std(ddof=1)
        if abs(cnt - cm) > 3.5 * max(cs, 1.0) * INFLATE:
            msgs.append(f"detector {k + 1}: {cnt} photons vs reference {cm:.1f} +- {cs:.1f}")
        ws = w[ids == k + 1].sum()
        wm, wsd = fx["det_wsum"][:, k].mean(), fx["det_wsum"][:, k].std(ddof=1)
        if abs(ws - wm) > 3.5 * max(wsd, 1e-12) * INFLATE:
            msgs.append(f"detector {k + 1}: weight {ws:.4g} vs reference {wm:.4g} +- {wsd:.3g}")
    plen = pp.mean(0)
    pm, ps = fx["det_plen"].mean(0), fx["det_plen"].std(0, ddof=1)
    if np.any(np.abs(plen - pm) > 3.5 * ps * INFLATE + 1e-9):
        msgs.append(f"mean partial path {plen} vs reference {pm} +- {ps}")
    ns = detp[:, 1:1 + M].astype(np.float64).mean(0)
    nm, nsd = fx["det_nscat"].mean(0), fx["det_nscat"].std(0, ddof=1)
    if np.any(np.abs(ns - nm) > 3.5 * nsd * INFLATE + 1e-9):
        msgs.append(f"mean scatter count {ns} vs reference {nm} +- {nsd}")
    return msgs
