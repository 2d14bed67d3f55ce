"""Generates the golden fixtures of the two benchmark workloads from runs of
the reference MMC CPU engine (oracle/_ref, built from the reference sources by
oracle/build_ref.sh).  Needs the reference build, so it runs in the development
container only; the fixtures are committed and used on every machine.

  c1_incl1296k  the 1.3M-tet workload: cube [0,60]^3 mm, 1 mm grid, 6 tets per
                voxel (1,296,000 tets, 226,981 nodes), interior nodes jittered
                by +/-0.25 mm (orientation-safe re-draw, seed 12345), tets with
                centroid within 10 mm of (30,30,30) labelled 2 (mua 0.05,
                mus 5, g 0.9, n 1.37), the rest 1 (mua 0.005, mus 1, g 0.01,
                n 1.37); pencil (30,30,0) +z; 50 gates of 0.1 ns; 4 detectors
                R=2 mm on z=0 at x=40,45,50,55; detected photons saved;
                1e6 photons per run
  c0_cube162k   the 162k-tet workload: homogeneous cube [0,60]^3 mm, 2 mm grid
                (162,000 tets, 29,791 nodes), mua 0.005, mus 1, g 0.01,
                n 1.37; pencil (30,30,0) +z; one gate 0-5 ns; 1e6 photons per
                run; element deposits plus the node output of each run
                (0.25 of each element's deposit on its 4 nodes, as the
                reference's CUDA host scatters, src/mmc_cu_host.cu:916-976,
                then the reference's own mesh_normalize, src/mmc_mesh.c:2154-2279,
                run by oracle/ref_driver.c)

Each case: 10 runs with seeds SEED0..SEED0+9 (one OpenMP thread each: the
reference's results depend on the thread count), branchless Badouel tracer,
element deposits, unnormalized (-M s -C 0 -U 0, -b 1), and 6 runs with fresh
seeds that calibrate the null (a fresh reference run scored against the 10-run
statistics, as tests/golden_checks.py scores a candidate).

Stored per case: per-gate totals, per-element sums over the gates (all
elements of c0; a random subset of the visited elements of c1, to keep the
fixture small), a random subset of the well-sampled (element, gate) cells, the
absorbed weight per launched photon (deposits x mua), ray-tet tests per
photon; for c1 the detector statistics; for c0 the normalized node output.

  python tests/golden/make_baseline_golden.py [c1_incl1296k] [c0_cube162k]
"""
from __future__ import annotations

import os
import struct
import subprocess
import sys
import tempfile
import zlib
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import golden_checks as gc  # noqa: E402
import make_golden as mg  # noqa: E402
import oracle  # noqa: E402  (test infrastructure: initial element, as the reference's InitElem)
from mmc_gb300 import meshgen  # noqa: E402

NRUNS, NNULL, SEED0 = mg.NRUNS, mg.NNULL, mg.SEED0
PHOTONS = 1000000
WORKERS = os.cpu_count() or 4


def run_one(wd, name, seed, photons, gates, ne, savedet):
    """One reference run (ref_driver around the reference lifecycle): its raw
    element deposits as float32 (gates, ne), ray-tet tests and, with
    detectors, the detected-photon table -- all from the same run."""
    sess = f"{name}_{seed}"
    detp_out = os.path.join(wd, sess + ".detp")
    cmd = [mg.REF + "_detp", "-f", os.path.join(wd, name + ".json"), "-c", "sse", "-M", "s", "-C", "0", "-b", "1",
           "-U", "0", "-F", "bin", "-s", sess, "-E", str(seed), "-n", str(photons), "-D", "T",
           "-d", "1" if savedet else "0"]
    env = dict(os.environ, OMP_NUM_THREADS="1", MMCGB_DETP_OUT=detp_out)
    p = subprocess.run(cmd, cwd=wd, env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError(p.stdout[-2000:])
    tests = None
    for line in p.stdout.splitlines():
        if "ray-tetrahedron tests" in line:
            tests = float(line.split("photon/ms")[1].split()[1].strip(","))
    binf = os.path.join(wd, sess + ".bin")
    raw = np.fromfile(binf, np.float64).reshape(gates, ne).astype(np.float32)
    os.remove(binf)
    out = dict(raw=raw, tests=tests)
    if savedet:
        buf = open(detp_out, "rb").read()
        count, cols = struct.unpack("<ii", buf[:8])
        out["det"] = np.frombuffer(buf, np.float32, count=count * cols, offset=8).reshape(count, cols).copy()
        os.remove(detp_out)
    return out


def field_stats(name, m, runs, nulls, photons, esub_size=None, ncells=30000):
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    G, ne = runs[0]["raw"].shape
    fields = np.stack([r["raw"] for r in runs]).astype(np.float64)  # (runs, G, ne)
    per_elem = fields.sum(axis=1)
    per_gate = fields.sum(axis=2)
    mean_e = per_elem.mean(0)
    if esub_size is None:
        esub = np.arange(ne, dtype=np.int32)
    else:
        visited = np.flatnonzero(mean_e > 0)
        esub = np.sort(rng.choice(visited, size=min(esub_size, visited.size), replace=False)).astype(np.int32)
    flat = fields.reshape(len(runs), -1)
    # (element, gate) cells: drawn among the well-sampled ones (run-to-run spread below a
    # quarter of the mean, the cells the z-test scores), most cells of 50 gates being sparse
    fm, fs = flat.mean(0), flat.std(0, ddof=1)
    cand = np.flatnonzero((fm > 0) & (fs > 0) & (fs < 0.25 * fm))
    cells = np.sort(rng.choice(cand, size=min(ncells, cand.size), replace=False))
    mua = m.media[m.label, 0].astype(np.float64)
    fx = dict(
        ne=ne, nn=m.nn, gates=G, photons=photons, seeds=np.arange(len(runs)) + SEED0,
        esub=esub, elem_mean=mean_e[esub].astype(np.float32), elem_std=per_elem[:, esub].std(0, ddof=1).astype(np.float32),
        gate_mean=per_gate.mean(0), gate_std=per_gate.std(0, ddof=1),
        cells=cells.astype(np.int64), cell_mean=flat[:, cells].mean(0).astype(np.float32),
        cell_std=flat[:, cells].std(0, ddof=1).astype(np.float32),
        absorbed=(per_elem * mua[None, :]).sum(1) / photons,
        tests_per_photon=np.array([r["tests"] / photons for r in runs]),
    )
    st_e = [gc.zstats(r["raw"].astype(np.float64).sum(0)[esub], fx["elem_mean"], fx["elem_std"]) for r in nulls]
    st_c = [gc.zstats(r["raw"].reshape(-1)[cells].astype(np.float64), fx["cell_mean"], fx["cell_std"]) for r in nulls]
    fx.update(null_elem_frac=np.array([t[0] for t in st_e]), null_elem_meanz=np.array([t[1] for t in st_e]),
              null_cell_frac=np.array([t[0] for t in st_c]), null_cell_meanz=np.array([t[1] for t in st_c]))
    return fx


def det_stats(m, runs, ndet):
    M = m.media.shape[0] - 1
    mua = m.media[1:, 0].astype(np.float64)
    counts, wsum, plen, nscat = [], [], [], []
    for r in runs:
        d = r["det"]
        ids = d[:, 0].astype(int)
        pp = d[:, 1 + M:1 + 2 * M].astype(np.float64)
        w = d[:, -1] * np.exp(-(pp * mua).sum(1))
        counts.append([np.count_nonzero(ids == k + 1) for k in range(ndet)])
        wsum.append([w[ids == k + 1].sum() for k in range(ndet)])
        plen.append(pp.mean(0))
        nscat.append(d[:, 1:1 + M].astype(np.float64).mean(0))
    return dict(det_count=np.array(counts, np.float64), det_wsum=np.array(wsum), det_plen=np.array(plen),
                det_nscat=np.array(nscat))


def make_c1(wd):
    name = "c1_incl1296k"
    m = meshgen.inclusion_cube()
    c = dict(mesh=m, photons=PHOTONS, t1=5e-9, dt=1e-10, det=meshgen.c1_detectors())
    c["e0"] = oracle.initelem(m.node, m.elem, m.label, (30.0, 30.0, 0.0))
    mg.write_json(os.path.join(wd, name + ".json"), name, c)
    G = 50
    seeds = [SEED0 + k for k in range(NRUNS)] + [SEED0 + 1000 + k for k in range(NNULL)]
    with ThreadPoolExecutor(max_workers=WORKERS) as ex:
        res = list(ex.map(lambda s: run_one(wd, name, s, PHOTONS, G, m.ne, True), seeds))
    runs, nulls = res[:NRUNS], res[NRUNS:]
    fx = field_stats(name, m, runs, nulls, PHOTONS, esub_size=150000)
    fx.update(det_stats(m, runs, 4))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **fx)
    print(name, "absorbed", fx["absorbed"].mean(), "+-", fx["absorbed"].std(ddof=1),
          "tests/photon", fx["tests_per_photon"].mean(), "detected", fx["det_count"].sum(1).mean(),
          "null elem", fx["null_elem_frac"], "null cell", fx["null_cell_frac"])


def normalize_nodes(wd_, name_, seed, raw, eabs):
    """Node output of one run's raw element deposits through the reference's own
    output stage (oracle/ref_driver.c: 0.25 scatter to the nodes, mesh_normalize)."""
    fin = os.path.join(wd_, f"{name_}_{seed}.nin")
    fout = os.path.join(wd_, f"{name_}_{seed}.nout")
    with open(fin, "wb") as f:
        f.write(np.array([eabs, float(PHOTONS)], np.float64).tobytes())
        f.write(np.ascontiguousarray(raw, np.float64).tobytes())
    cmd = [mg.REF + "_detp", "-f", os.path.join(wd_, name_ + ".json"), "-c", "sse", "-M", "s", "-C", "1",
           "-b", "1", "-U", "1", "-n", "1"]
    env = dict(os.environ, OMP_NUM_THREADS="1", MMCGB_NORM_IN=fin, MMCGB_NORM_OUT=fout)
    p = subprocess.run(cmd, cwd=wd_, env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError(p.stdout[-2000:])
    data = np.fromfile(fout, np.float64)
    os.remove(fin)
    os.remove(fout)
    return data[:-1], data[-1]


def make_c0(wd):
    name = "c0_cube162k"
    m = meshgen.homogeneous_cube(n=30)
    c = dict(mesh=m, photons=PHOTONS, t1=5e-9, dt=5e-9, det=None)
    c["e0"] = oracle.initelem(m.node, m.elem, m.label, (30.0, 30.0, 0.0))
    mg.write_json(os.path.join(wd, name + ".json"), name, c)
    seeds = [SEED0 + k for k in range(NRUNS)] + [SEED0 + 1000 + k for k in range(NNULL)]
    mua = m.media[m.label, 0].astype(np.float64)

    def one(seed):
        r = run_one(wd, name, seed, PHOTONS, 1, m.ne, False)
        # node output of this run: the CUDA host's 0.25 scatter and the reference's own
        # mesh_normalize, with the absorbed weight the CPU engine tallies (its deposits x mua)
        raw = r["raw"].astype(np.float64)
        eabs = float((raw[0] * mua).sum())
        w, _ = normalize_nodes(wd, name, seed, raw, eabs)
        r["node"] = w.astype(np.float64)
        return r

    with ThreadPoolExecutor(max_workers=WORKERS) as ex:
        res = list(ex.map(one, seeds))
    runs, nulls = res[:NRUNS], res[NRUNS:]
    fx = field_stats(name, m, runs, nulls, PHOTONS)
    nodes = np.stack([r["node"] for r in runs])
    fx.update(node_mean=nodes.mean(0), node_std=nodes.std(0, ddof=1))
    st = [gc.zstats(r["node"], fx["node_mean"], fx["node_std"]) for r in nulls]
    fx.update(null_node_frac=np.array([t[0] for t in st]), null_node_meanz=np.array([t[1] for t in st]))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **fx)
    print(name, "absorbed", fx["absorbed"].mean(), "+-", fx["absorbed"].std(ddof=1),
          "tests/photon", fx["tests_per_photon"].mean(), "null elem", fx["null_elem_frac"],
          "null node", fx["null_node_frac"])


def main(only=()):
    if not os.path.exists(mg.REF + "_detp"):
        subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    with tempfile.TemporaryDirectory() as wd:
        if not only or "c0_cube162k" in only:
            make_c0(wd)
        if not only or "c1_incl1296k" in only:
            make_c1(wd)


if __name__ == "__main__":
    main(tuple(sys.argv[1:]))
