"""Generates the golden fixtures in tests/golden/ by running the reference MMC
CPU engine (built from the reference sources by oracle/build_ref.sh into
oracle/_ref/mmc).  Needs the reference tree, so it runs in the development
container only; the fixtures it writes are committed and used everywhere.

For each case the reference runs 10 times (seeds SEED0..SEED0+9), one OpenMP
thread each (its results depend on the thread count), with the branchless
Badouel tracer and element-based output (-M s -C 0), unnormalized (-U 0):

  cube6k   homogeneous 60 mm cube, 10^3 voxels x 6 tets, mua=0.005 mus=1 g=0.01
           n=1.37, pencil (30,30,0) +z, one 5 ns gate, 1e5 photons
  incl48k  20^3 voxels x 6 tets at 3 mm, +/-0.6 mm jitter, r=10 mm inclusion
           (mua=0.05 mus=5 g=0.9), 10 gates of 0.5 ns, 4 detectors R=2 mm on
           z=0 at x=40..55, detected photons saved, 1e5 photons
  src_*    source types on the cube6k mesh, one 5 ns gate, 1e5 photons:
           isotropic and cone (half angle 0.6 rad about (0.6,0,0.8)) at the
           centre; disk (R=10 mm), gaussian (waist 5 mm) and planar (20x20 mm)
           on the z=0 face over a 6 mm void layer (voxel layer z<6 mm; the
           reference needs the layer's tets labelled -1, its source-element
           candidates, which it then treats as void, label 0)
  dref_cube6k / grid_cube6k / traj_cube6k
           the cube6k mesh with exiting weight per face (-X 1, 5 gates of
           1 ns), dual-grid output on 2 mm voxels (-M G), trajectory records
           (-D M, 5 gates of 1 ns, 2e4 photons: statistics per run)
  bench_dmmc-cube60, bench_dmmc-cube60b
           the reference's built-in benchmarks (-Q), dual-grid output on
           1 mm voxels, 1e5 photons
  detimage_cube6k
           the exit image of an area detector (-x 2): the cube6k pencil run
           with one 30 mm detector at (10,10,0), 5 gates of 1 ns, 2e4 photons;
           the reference's detected records (with exit columns) and the
           <session>.img it bins from them, 8 x 8 pixels over 40 x 40 mm given
           as the Source's Param1/Param2, where the reference's JSON reader
           takes them
  src_pattern3
           three patterns sharing each photon (srcnum 3, photon sharing): a
           4 x 3 pixel pattern source over 20 x 20 mm of the void-layer cube6k
           face, the patterns given as a JData array [3, 4, 3]; statistics per
           (element, pattern), and the seed-SEED0 run's raw and normalized
           output with the per-pattern energies the reference prints

Six more runs with fresh seeds calibrate the null: their coverage of the
10-run statistics (fraction of cells within 3 sigma, mean z) is stored, and a
candidate must score like a fresh reference run does.

Stored per case: mean and standard deviation over the 10 runs of the
per-element fluence summed over gates and of the per-gate totals, a random
subset of (element, gate) cells, detector statistics, absorbed fraction and
ray-tet tests per photon; plus, for seed SEED0, the normalized element output
(-U 1) next to the raw one, which pins the normalization.

  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
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
from mmc_gb300 import meshgen  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref", "mmc")
NRUNS = 10
NNULL = 6
SEED0 = 20260101


SOURCE_CASES = {
    "src_isotropic": dict(Type="isotropic", Pos=[30.0, 30.0, 30.0], Dir=[0.0, 0.0, 1.0], void=False),
    "src_cone": dict(Type="cone", Pos=[30.0, 30.0, 30.0], Dir=[0.6, 0.0, 0.8], Param1=[0.6, 0, 0, 0], void=False),
    "src_disk": dict(Type="disk", Pos=[30.0, 30.0, 0.0], Dir=[0.0, 0.0, 1.0], Param1=[10.0, 0, 0, 0], void=True),
    "src_gaussian": dict(Type="gaussian", Pos=[30.0, 30.0, 0.0], Dir=[0.0, 0.0, 1.0], Param1=[5.0, 0, 0, 0],
                         void=True),
    "src_planar": dict(Type="planar", Pos=[20.0, 20.0, 0.0], Dir=[0.0, 0.0, 1.0], Param1=[20.0, 0, 0, 0],
                       Param2=[0, 20.0, 0, 0], void=True),
}


def void_layer_labels(m):
    """Labels of the cube6k mesh with the voxel layer z < 6 mm made void (0)."""
    label = m.label.copy()
    label[meshgen.centroids(m.node, m.elem)[:, 2] < 6.0] = 0
    return label


def case_defs():
    cube = meshgen.homogeneous_cube(n=10)
    incl = meshgen.inclusion_cube(n=20, jitter=0.6, seed=7)
    cases = {
        "cube6k": dict(mesh=cube, photons=100000, t1=5e-9, dt=5e-9, det=None),
        "incl48k": dict(mesh=incl, photons=100000, t1=5e-9, dt=0.5e-9, det=meshgen.c1_detectors()),
    }
    for name, src in SOURCE_CASES.items():
        c = dict(mesh=cube, photons=100000, t1=5e-9, dt=5e-9, det=None, src=src)
        if src["void"]:
            lab = void_layer_labels(cube)
            c["mesh"] = meshgen.Mesh(cube.node, cube.elem, lab, cube.media, "cube6k-void")
            c["reflabel"] = np.where(lab == 0, -1, lab)  # the reference's source candidates
        cases[name] = c
    return cases


def write_json(path, name, c):
    m = c["mesh"]
    elem = np.c_[m.elem, c.get("reflabel", m.label)].tolist()
    src = c.get("src") or dict(Pos=[30.0, 30.0, 0.0], Dir=[0.0, 0.0, 1.0])
    source = {k: v for k, v in src.items() if k in ("Type", "Pos", "Dir", "Param1", "Param2")}
    cfg = {
        "Session": {"ID": name, "Photons": c["photons"], "RNGSeed": SEED0, "OutputFormat": "bin",
                    "DoMismatch": 1},
        "Domain": {"Media": [dict(mua=float(r[0]), mus=float(r[1]), g=float(r[2]), n=float(r[3]))
                             for r in m.media]},
        "Mesh": {"MeshNode": m.node.astype(np.float64).tolist(), "MeshElem": elem, "InitElem": int(c["e0"])},
        "Forward": {"T0": 0.0, "T1": c["t1"], "Dt": c["dt"]},
        "Optode": {"Source": source},
    }
    if c["det"] is not None:
        cfg["Optode"]["Detector"] = [{"Pos": [float(d[0]), float(d[1]), float(d[2])], "R": float(d[3])}
                                     for d in c["det"]]
    with open(path, "w") as f:
        json.dump(cfg, f)


def read_mch(path):
    with open(path, "rb") as f:
        buf = f.read()
    hdr = struct.unpack("<4sIIIIIIIfIfIiI2i", buf[:64])
    colcount, saved = hdr[4], hdr[7]
    data = np.frombuffer(buf, np.float32, count=saved * colcount, offset=64).reshape(saved, colcount)
    return data, dict(maxmedia=hdr[2], detnum=hdr[3], colcount=colcount, total=hdr[5], detected=hdr[6])


def read_jdata(obj):
    """Decodes one JData array (base64 + zlib) of the reference's JSON output."""
    import base64
    import zlib
    dt = {"uint32": np.uint32, "single": np.float32, "double": np.float64, "int32": np.int32}[obj["_ArrayType_"]]
    raw = zlib.decompress(base64.b64decode(obj["_ArrayZipData_"]))
    return np.frombuffer(raw, dt).reshape(obj["_ArraySize_"])


def run_ref_detp(workdir, name, seed, photons):
    """Detected photons of one run: the reference lifecycle run by
    oracle/ref_driver.c, which dumps cfg.exportdetected (the reference's own
    .mch/.jdt writers take their column count from cfg.his, which the CPU path
    leaves at 0).  Columns: detid, nscat[M], ppath[M], w0."""
    sess = f"{name}_{seed}_det"
    out = os.path.join(workdir, sess + ".detp")
    cmd = [REF + "_detp", "-f", os.path.join(workdir, name + ".json"), "-c", "sse", "-M", "s", "-C", "0", "-b", "1",
           "-U", "0", "-F", "bin", "-s", sess, "-E", str(seed), "-n", str(photons), "-d", "1"]
    env = dict(os.environ, OMP_NUM_THREADS="1", MMCGB_DETP_OUT=out)
    p = subprocess.run(cmd, cwd=workdir, env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError(p.stdout[-2000:])
    buf = open(out, "rb").read()
    count, cols = struct.unpack("<ii", buf[:8])
    return np.frombuffer(buf, np.float32, count=count * cols, offset=8).reshape(count, cols)


def run_ref_mesh(workdir, name):
    """The reference's prepared mesh (after mmc_prep) dumped by oracle/ref_driver.c."""
    out = os.path.join(workdir, name + ".meshdump")
    norm_in = os.path.join(workdir, name + ".nin")
    with open(norm_in, "wb") as f:  # a normalize-only run so no photons are simulated
        f.write(np.zeros(2, np.float64).tobytes())
    cmd = [REF + "_detp", "-f", os.path.join(workdir, name + ".json"), "-c", "sse", "-M", "s", "-C", "0", "-b", "1",
           "-n", "1"]
    env = dict(os.environ, OMP_NUM_THREADS="1", MMCGB_MESH_OUT=out)
    p = subprocess.run(cmd, cwd=workdir, env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError(p.stdout[-2000:])
    buf = open(out, "rb").read()
    nn, ne, nf = struct.unpack("<iii", buf[:12])
    o = 12
    def take(dt, n):
        nonlocal o
        a = np.frombuffer(buf, dt, count=n, offset=o)
        o += a.nbytes
        return a
    elem = take(np.int32, ne * 4).reshape(ne, 4)
    facenb = take(np.int32, ne * 4).reshape(ne, 4)
    evol = take(np.float32, ne)
    nvol = take(np.float32, nn)
    normals = take(np.float32, ne * 16).reshape(ne, 16)
    return dict(nn=nn, ne=ne, nf=nf, elem=elem, facenb=facenb, evol=evol, nvol=nvol, normals=normals)


def run_ref_normalize(workdir, name, raw, eabs, etot, basisorder):
    """The reference's output stage (elem->node scatter + mesh_normalize) applied
    to a given raw element field, through oracle/ref_driver.c."""
    fin = os.path.join(workdir, f"{name}_{basisorder}.nin")
    fout = os.path.join(workdir, f"{name}_{basisorder}.nout")
    with open(fin, "wb") as f:
        f.write(np.array([eabs, etot], np.float64).tobytes())
        f.write(np.ascontiguousarray(raw, np.float64).tobytes())
    cmd = [REF + "_detp", "-f", os.path.join(workdir, name + ".json"), "-c", "sse", "-M", "s", "-C", str(basisorder),
           "-b", "1", "-U", "1", "-n", "1"]
    env = dict(os.environ, OMP_NUM_THREADS="1", MMCGB_NORM_IN=fin, MMCGB_NORM_OUT=fout)
    p = subprocess.run(cmd, cwd=workdir, env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError(p.stdout[-2000:])
    data = np.fromfile(fout, np.float64)
    return data[:-1], data[-1]


def run_ref(workdir, name, seed, photons, normalized=False, savedet=False):
    sess = f"{name}_{seed}_{int(normalized)}"
    cmd = [REF, "-f", os.path.join(workdir, name + ".json"), "-c", "sse", "-M", "s", "-C", "0", "-b", "1",
           "-U", "1" if normalized else "0", "-F", "bin", "-s", sess, "-E", str(seed), "-n", str(photons),
           "-D", "T", "-d", "1" if savedet else "0"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    p = subprocess.run(cmd, cwd=workdir, env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError(p.stdout[-2000:])
    log = p.stdout
    raw = np.fromfile(os.path.join(workdir, sess + ".bin"), np.float64)
    tests = None
    absorbed = None
    for line in log.splitlines():
        if "ray-tetrahedron tests" in line:
            tests = float(line.split("photon/ms")[1].split()[1].strip(","))
        if "absorbed:" in line:
            absorbed = float(line.split("absorbed:")[1].strip().split("%")[0].split("m")[-1]) / 100.0
    out = dict(raw=raw, tests=tests, absorbed=absorbed)
    if savedet:
        out["det"] = run_ref_detp(workdir, name, seed, photons)
    return out


def run_ref_dref(workdir, name, seed, photons, nf, gates):
    """Exiting weight per exterior face and gate of one reference run (-X 1),
    read from its text output <session>_dref.dat (the binary writer of the
    reference stores the fluence array under that name instead)."""
    sess = f"{name}_{seed}_ref"
    cmd = [REF, "-f", os.path.join(workdir, name + ".json"), "-c", "sse", "-M", "s", "-C", "0", "-b", "1",
           "-U", "0", "-F", "ascii", "-s", sess, "-E", str(seed), "-n", str(photons), "-X", "1", "-D", "T"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    p = subprocess.run(cmd, cwd=workdir, env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError(p.stdout[-2000:])
    vals = np.loadtxt(os.path.join(workdir, sess + "_dref.dat"))[:, 1]
    return vals.reshape(gates, nf)


def make_dref_case(wd):
    """dref_cube6k: exiting weight per exterior face of the cube6k mesh, pencil
    (30,30,0) +z, 5 gates of 1 ns, 1e5 photons; 10 runs + 6 null runs."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    name = "dref_cube6k"
    m = meshgen.homogeneous_cube(n=10)
    c = dict(mesh=m, photons=100000, t1=5e-9, dt=1e-9, det=None)
    c["e0"] = oracle.initelem(m.node, m.elem, m.label, (30.0, 30.0, 0.0))
    write_json(os.path.join(wd, name + ".json"), name, c)
    nf = oracle.prep_mesh(m.node, m.elem, m.label)["nf"]
    G = 5
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        runs = list(ex.map(lambda s: run_ref_dref(wd, name, s, c["photons"], nf, G), [SEED0 + k for k in range(NRUNS)]))
        nulls = list(ex.map(lambda s: run_ref_dref(wd, name, s, c["photons"], nf, G),
                            [SEED0 + 1000 + k for k in range(NNULL)]))
    runs = np.stack(runs)              # (runs, G, nf)
    per_face = runs.sum(1)
    per_gate = runs.sum(2)
    sys.path.insert(0, os.path.dirname(HERE))
    import golden_checks as gc
    fx = dict(nf=nf, gates=G, photons=c["photons"], face_mean=per_face.mean(0), face_std=per_face.std(0, ddof=1),
              gate_mean=per_gate.mean(0), gate_std=per_gate.std(0, ddof=1))
    st = [gc.zstats(x.sum(0), fx["face_mean"], fx["face_std"]) for x in nulls]
    fx.update(null_face_frac=np.array([t[0] for t in st]), null_face_meanz=np.array([t[1] for t in st]))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **fx)
    print(name, "nf", nf, "escaped per photon", per_gate.sum(1).mean() / c["photons"])


PATTERN3 = np.random.default_rng(77).uniform(0.1, 1.0, (3, 4, 3)).astype(np.float32)  # [pattern, x, y]


def jdata_array(a):
    """A float32 array as a zlib-compressed JData object, row-major as JData stores it."""
    import base64
    b = np.ascontiguousarray(a, np.float32).tobytes()
    return {"_ArrayType_": "single", "_ArraySize_": list(a.shape), "_ArrayZipType_": "zlib",
            "_ArrayZipSize_": [1, int(a.size)], "_ArrayZipData_": base64.b64encode(zlib.compress(b)).decode()}


def run_ref_patterns(workdir, name, seed, photons, ne, K, normalized=False):
    """Raw (or normalized) element output of one multi-pattern run, (ne, K), and the
    per-pattern launched energy / absorbed percentage / normalizer lines of its log."""
    sess = f"{name}_{seed}_{int(normalized)}"
    cmd = [REF, "-f", os.path.join(workdir, name + ".json"), "-c", "sse", "-M", "s", "-C", "0", "-b", "1",
           "-U", "1" if normalized else "0", "-F", "bin", "-s", sess, "-E", str(seed), "-n", str(photons), "-D", "T"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    p = subprocess.run(cmd, cwd=workdir, env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError(p.stdout[-2000:])
    raw = np.fromfile(os.path.join(workdir, sess + ".bin"), np.float64).reshape(ne, K)
    energies = []
    for line in p.stdout.splitlines():
        if "total simulated energy:" in line:
            import re
            clean = re.sub(r"\x1b\[[0-9;]*m", "", line)
            etot = float(clean.split("total simulated energy:")[1].split()[0])
            absp = float(clean.split("absorbed:")[1].split("%")[0])
            norm = float(clean.split("normalizor=")[1].split()[0])
            energies.append((etot, absp, norm))
    return raw, np.array(energies)


def make_pattern_case(wd):
    """src_pattern3: three patterns sharing each photon; 10 runs + 6 null runs."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    name = "src_pattern3"
    cube = meshgen.homogeneous_cube(n=10)
    lab = void_layer_labels(cube)
    m = meshgen.Mesh(cube.node, cube.elem, lab, cube.media, "cube6k-void")
    K, nx, ny = PATTERN3.shape
    src = dict(Type="pattern", Pos=[20.0, 20.0, 0.0], Dir=[0.0, 0.0, 1.0], Param1=[20.0, 0, 0, nx],
               Param2=[0, 20.0, 0, ny])
    c = dict(mesh=m, photons=100000, t1=5e-9, dt=5e-9, det=None, src=src, reflabel=np.where(lab == 0, -1, lab))
    c["e0"] = oracle.initelem(m.node, m.elem, m.label, (20.0, 20.0, 0.0))
    path = os.path.join(wd, name + ".json")
    write_json(path, name, c)
    cfgj = json.load(open(path))
    cfgj["Optode"]["Source"]["Pattern"] = jdata_array(PATTERN3)
    json.dump(cfgj, open(path, "w"))
    ne = m.ne
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        runs = list(ex.map(lambda s: run_ref_patterns(wd, name, s, c["photons"], ne, K)[0],
                           [SEED0 + k for k in range(NRUNS)]))
        nulls = list(ex.map(lambda s: run_ref_patterns(wd, name, s, c["photons"], ne, K)[0],
                            [SEED0 + 1000 + k for k in range(NNULL)]))
        normed, energies = ex.submit(run_ref_patterns, wd, name, SEED0, c["photons"], ne, K, True).result()
    runs = np.stack(runs)  # (runs, ne, K)
    flat = runs.reshape(NRUNS, -1)
    tot = runs.sum(1)      # (runs, K)
    sys.path.insert(0, os.path.dirname(HERE))
    import golden_checks as gc
    fx = dict(ne=ne, srcnum=K, photons=c["photons"], pattern=PATTERN3,
              cell_mean=flat.mean(0), cell_std=flat.std(0, ddof=1), total_mean=tot.mean(0), total_std=tot.std(0, ddof=1),
              raw_seed0=runs[0], norm_seed0=normed, energies_seed0=energies)
    st = [gc.zstats(x.reshape(-1), fx["cell_mean"], fx["cell_std"]) for x in nulls]
    fx.update(null_cell_frac=np.array([t[0] for t in st]), null_cell_meanz=np.array([t[1] for t in st]))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **fx)
    print(name, "per-pattern totals", tot.mean(0), "energies", energies)


def make_detimage_case(wd):
    """detimage_cube6k: the reference's records and its exit image of one run."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    name = "detimage_cube6k"
    m = meshgen.homogeneous_cube(n=10)
    det = np.array([[10.0, 10.0, 0.0, 30.0]])
    src = dict(Pos=[30.0, 30.0, 0.0], Dir=[0.0, 0.0, 1.0], Param1=[40.0, 0, 0, 8], Param2=[0, 40.0, 0, 8])
    c = dict(mesh=m, photons=20000, t1=5e-9, dt=1e-9, det=det, src=src)
    c["e0"] = oracle.initelem(m.node, m.elem, m.label, (30.0, 30.0, 0.0))
    write_json(os.path.join(wd, name + ".json"), name, c)
    sess = f"{name}_{SEED0}"
    out = os.path.join(wd, sess + ".detp")
    cmd = [REF + "_detp", "-f", os.path.join(wd, name + ".json"), "-c", "sse", "-M", "s", "-C", "0", "-b", "1",
           "-U", "0", "-F", "bin", "-s", sess, "-E", str(SEED0), "-n", str(c["photons"]), "-d", "1", "-x", "2"]
    env = dict(os.environ, OMP_NUM_THREADS="1", MMCGB_DETP_OUT=out)
    p = subprocess.run(cmd, cwd=wd, env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError(p.stdout[-2000:])
    buf = open(out, "rb").read()
    count, cols = struct.unpack("<ii", buf[:8])
    detp = np.frombuffer(buf, np.float32, count=count * cols, offset=8).reshape(count, cols)
    img = np.fromfile(os.path.join(wd, sess + ".img"), np.float32).reshape(5, 8, 8)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), detp=detp, img=img, detpos=det.astype(np.float32),
                        detparam1=np.array(src["Param1"], np.float32), detparam2=np.array(src["Param2"], np.float32),
                        tstep=np.float32(c["dt"]), gates=5)
    print(name, "records", detp.shape, "image sum", img.sum())


def run_ref_grid(workdir, name, seed, photons, nvox):
    """Dual-grid (DMMC, -M G) fluence of one reference run, unnormalized."""
    sess = f"{name}_{seed}_grid"
    cmd = [REF, "-f", os.path.join(workdir, name + ".json"), "-c", "sse", "-M", "G", "-C", "0", "-b", "1",
           "-U", "0", "-F", "bin", "-s", sess, "-E", str(seed), "-n", str(photons), "-D", "T"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    p = subprocess.run(cmd, cwd=workdir, env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError(p.stdout[-2000:])
    raw = np.fromfile(os.path.join(workdir, sess + ".bin"), np.float64)
    return raw.reshape(-1, nvox)


def make_grid_case(wd):
    """grid_cube6k: the cube6k run (pencil (30,30,0) +z, one 5 ns gate, 1e5
    photons) with dual-grid output on 2 mm voxels; 10 runs + 6 null runs."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    name = "grid_cube6k"
    m = meshgen.homogeneous_cube(n=10)
    c = dict(mesh=m, photons=100000, t1=5e-9, dt=5e-9, det=None)
    c["e0"] = oracle.initelem(m.node, m.elem, m.label, (30.0, 30.0, 0.0))
    path = os.path.join(wd, name + ".json")
    write_json(path, name, c)
    cfgj = json.load(open(path))
    cfgj["Domain"]["Step"] = [2.0, 2.0, 2.0]
    json.dump(cfgj, open(path, "w"))
    dim = oracle.grid_dims(m.node, 2.0)
    nvox = int(np.prod(dim))
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        runs = list(ex.map(lambda s: run_ref_grid(wd, name, s, c["photons"], nvox), [SEED0 + k for k in range(NRUNS)]))
        nulls = list(ex.map(lambda s: run_ref_grid(wd, name, s, c["photons"], nvox),
                            [SEED0 + 1000 + k for k in range(NNULL)]))
    vox = np.stack([r.sum(0) for r in runs])
    sys.path.insert(0, os.path.dirname(HERE))
    import golden_checks as gc
    fx = dict(dim=np.array(dim), photons=c["photons"], step=2.0, vox_mean=vox.mean(0), vox_std=vox.std(0, ddof=1),
              total=np.array([r.sum() for r in runs]))
    st = [gc.zstats(x.sum(0), fx["vox_mean"], fx["vox_std"]) for x in nulls]
    fx.update(null_vox_frac=np.array([t[0] for t in st]), null_vox_meanz=np.array([t[1] for t in st]))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **fx)
    print(name, "dim", dim, "absorbed per photon", fx["total"].mean() * 0.005 / c["photons"])


def run_ref_traj(workdir, name, seed, photons, maxjump):
    """Trajectory records of one reference run (-D M): <session>.mch with six
    columns (src/mmc_host.c:452-459)."""
    sess = f"{name}_{seed}_traj"
    cmd = [REF, "-f", os.path.join(workdir, name + ".json"), "-c", "sse", "-M", "s", "-C", "0", "-b", "1",
           "-U", "0", "-F", "bin", "-s", sess, "-E", str(seed), "-n", str(photons), "-D", "M",
           "--maxjumpdebug", str(maxjump)]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    p = subprocess.run(cmd, cwd=workdir, env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError(p.stdout[-2000:])
    data, hdr = read_mch(os.path.join(workdir, sess + ".mch"))
    assert hdr["colcount"] == 6 and hdr["detected"] == 0 and len(data) < maxjump
    return data


def make_traj_case(wd):
    """traj_cube6k: trajectory records (-D M) of the cube6k mesh, pencil
    (30,30,0) +z, 5 gates of 1 ns, 2e4 photons; statistics of 10 runs."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    name = "traj_cube6k"
    m = meshgen.homogeneous_cube(n=10)
    c = dict(mesh=m, photons=20000, t1=5e-9, dt=1e-9, det=None)
    c["e0"] = oracle.initelem(m.node, m.elem, m.label, (30.0, 30.0, 0.0))
    write_json(os.path.join(wd, name + ".json"), name, c)
    maxjump = 6000000
    sys.path.insert(0, os.path.dirname(HERE))
    import golden_checks as gc
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        stats = list(ex.map(lambda s: gc.traj_stats(run_ref_traj(wd, name, s, c["photons"], maxjump), c["photons"]),
                            [SEED0 + k for k in range(NRUNS)]))
    fx = dict(photons=c["photons"], maxjumpdebug=maxjump, edges=gc.TRAJ_EDGES)
    for k in gc.TRAJ_KEYS + ("launch_pos", "launch_weight"):
        fx["traj_" + k] = np.array([s[k] for s in stats], np.float64)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **fx)
    print(name, "records/photon", fx["traj_records_per_photon"].mean(), "+-", fx["traj_records_per_photon"].std())


def run_ref_bench(workdir, name, seed, photons):
    """One run of a built-in benchmark of the reference (-Q name, src/mmc_bench.c)
    with dual-grid output, unnormalized: (grid deposits, absorbed fraction,
    ray-tet tests per photon).  With -Q the reference prints no energy line
    (its debug flags come from the benchmark's JSON), so the absorbed fraction
    is taken from the deposits."""
    sess = f"{name}_{seed}_bench"
    cmd = [REF, "-Q", name, "-c", "sse", "-M", "g", "-U", "0", "-F", "bin", "-s", sess, "-E", str(seed),
           "-n", str(photons), "-D", "T"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    p = subprocess.run(cmd, cwd=workdir, env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError(p.stdout[-2000:])
    tests = None
    for line in p.stdout.splitlines():
        if "ray-tetrahedron tests" in line:
            tests = float(line.split("photon/ms")[1].split()[1].strip(","))
    raw = np.fromfile(os.path.join(workdir, sess + ".bin"), np.float64)
    # grid deposits are the lost weight over mua (0.005 throughout): absorbed fraction from their sum
    return raw, raw.sum() * 0.005 / photons, tests / photons


def make_bench_cases(wd):
    """bench_dmmc-cube60(b): the reference's built-in benchmarks (6-tet 60 mm
    cube, pencil (30.1,30.2,0) +z, one 5 ns gate) with dual-grid output on
    1 mm voxels, 1e5 photons per run; 10 runs + 6 null runs each."""
    sys.path.insert(0, os.path.dirname(HERE))
    import golden_checks as gc
    for bench in ("dmmc-cube60", "dmmc-cube60b"):
        photons = 100000
        with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
            runs = list(ex.map(lambda s: run_ref_bench(wd, bench, s, photons), [SEED0 + k for k in range(NRUNS)]))
            nulls = list(ex.map(lambda s: run_ref_bench(wd, bench, s, photons),
                                [SEED0 + 1000 + k for k in range(NNULL)]))
        vox = np.stack([r[0] for r in runs])
        # a random subset of the visited voxels keeps the fixture small
        rng = np.random.default_rng(zlib.crc32(bench.encode()))
        sub = np.sort(rng.choice(np.flatnonzero(vox.mean(0) > 0), size=20000, replace=False)).astype(np.int32)
        fx = dict(photons=photons, nvox=vox.shape[1], sub=sub, vox_mean=vox[:, sub].mean(0).astype(np.float32),
                  vox_std=vox[:, sub].std(0, ddof=1).astype(np.float32), total=vox.sum(1), absorbed=np.array([r[1] for r in runs]),
                  tests_per_photon=np.array([r[2] for r in runs]))
        st = [gc.zstats(x[0][sub], fx["vox_mean"], fx["vox_std"]) for x in nulls]
        fx.update(null_vox_frac=np.array([t[0] for t in st]), null_vox_meanz=np.array([t[1] for t in st]))
        np.savez_compressed(os.path.join(HERE, f"bench_{bench}.npz"), **fx)
        print(bench, "absorbed", fx["absorbed"].mean(), "tests/photon", fx["tests_per_photon"].mean())


def main(only=()):
    """Regenerates every case, or only the named ones (each case draws its
    random cell subset from its own generator, so cases are independent)."""
    if not os.path.exists(REF):
        subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    with tempfile.TemporaryDirectory() as wd:
        if not only or "dref_cube6k" in only:
            make_dref_case(wd)
        if not only or "grid_cube6k" in only:
            make_grid_case(wd)
        if not only or "traj_cube6k" in only:
            make_traj_case(wd)
        if not only or "bench" in only:
            make_bench_cases(wd)
        if not only or "src_pattern3" in only:
            make_pattern_case(wd)
        if not only or "detimage_cube6k" in only:
            make_detimage_case(wd)
        for name, c in case_defs().items():
            if only and name not in only:
                continue
            rng = np.random.default_rng(zlib.crc32(name.encode()))
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import oracle
            srcpos = tuple((c.get("src") or {}).get("Pos", (30.0, 30.0, 0.0)))
            c["e0"] = oracle.initelem(c["mesh"].node, c["mesh"].elem, c["mesh"].label, srcpos)
            write_json(os.path.join(wd, name + ".json"), name, c)
            m = c["mesh"]
            ne = m.ne
            G = int(round(c["t1"] / c["dt"]))
            savedet = c["det"] is not None
            with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
                runs = list(ex.map(lambda s: run_ref(wd, name, s, c["photons"], savedet=savedet),
                                   [SEED0 + k for k in range(NRUNS)]))
                norm = ex.submit(run_ref, wd, name, SEED0, c["photons"], True, False).result()
                # null calibration: fresh reference runs scored against the 10-run statistics
                nulls = list(ex.map(lambda s: run_ref(wd, name, s, c["photons"]),
                                    [SEED0 + 1000 + k for k in range(NNULL)]))
            fields = np.stack([r["raw"].reshape(G, ne) for r in runs])  # (runs, G, ne)
            per_elem = fields.sum(axis=1)
            per_gate = fields.sum(axis=2)
            cells = rng.choice(G * ne, size=min(4000, G * ne), replace=False)
            flat = fields.reshape(NRUNS, -1)[:, cells]
            fx = dict(
                ne=ne, nn=m.nn, gates=G, photons=c["photons"], seeds=np.arange(NRUNS) + SEED0,
                elem_mean=per_elem.mean(0).astype(np.float32), elem_std=per_elem.std(0, ddof=1).astype(np.float32),
                gate_mean=per_gate.mean(0), gate_std=per_gate.std(0, ddof=1),
                cells=cells.astype(np.int32), cell_mean=flat.mean(0).astype(np.float32),
                cell_std=flat.std(0, ddof=1).astype(np.float32),
                # absorbed weight per launched photon: element deposits are (w0-w1)/mua
                absorbed=(fields.sum(axis=1) * m.media[m.label, 0][None, :].astype(np.float64)).sum(1) / c["photons"],
                tests_per_photon=np.array([r["tests"] / c["photons"] for r in runs]),
                raw_seed0=runs[0]["raw"].astype(np.float32) if G == 1 else np.zeros(0, np.float32),
                norm_seed0=norm["raw"].astype(np.float32) if G == 1 else np.zeros(0, np.float32),
            )
            sys.path.insert(0, os.path.dirname(HERE))
            import golden_checks as gc
            nf = [np.array([r["raw"].reshape(G, ne).sum(0) for r in nulls]),
                  np.array([r["raw"].reshape(-1)[cells] for r in nulls])]
            st = [[gc.zstats(x, fx["elem_mean"], fx["elem_std"]) for x in nf[0]],
                  [gc.zstats(x, fx["cell_mean"], fx["cell_std"]) for x in nf[1]]]
            fx.update(null_elem_frac=np.array([t[0] for t in st[0]]), null_elem_meanz=np.array([t[1] for t in st[0]]),
                      null_cell_frac=np.array([t[0] for t in st[1]]), null_cell_meanz=np.array([t[1] for t in st[1]]))
            if savedet:
                M = m.media.shape[0] - 1
                mua = m.media[1:, 0].astype(np.float64)
                ndet = len(c["det"])
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
                fx.update(det_count=np.array(counts, np.float64), det_wsum=np.array(wsum),
                          det_plen=np.array(plen), det_nscat=np.array(nscat))
            np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **fx)
            if name.startswith("src_"):  # the source cases reuse the cube6k mesh: no pins of their own
                print(name, "absorbed", fx["absorbed"].mean(), "tests/photon", fx["tests_per_photon"].mean())
                continue
            # pins of the host stages: prepared mesh and output normalization
            md = run_ref_mesh(wd, name)
            sub = np.sort(rng.choice(ne, size=min(ne, 3000), replace=False)).astype(np.int32)
            pin = dict(nn=md["nn"], ne=md["ne"], nf=md["nf"], sub=sub, elem=md["elem"][sub], facenb=md["facenb"][sub],
                       evol=md["evol"][sub], normals=md["normals"][sub], nvol=md["nvol"])
            raw = np.random.default_rng(123).random((G, ne)) * 100.0
            eabs, etot = 0.27 * c["photons"], float(c["photons"])
            nsub = np.sort(rng.choice(m.nn, size=min(m.nn, 2000), replace=False)).astype(np.int32)
            pin["nsub"] = nsub
            for bo in (0, 1):
                w, norm = run_ref_normalize(wd, name, raw, eabs, etot, bo)
                w = w.reshape(G, -1)[:, sub if bo == 0 else nsub]
                pin[f"norm{bo}_field"] = w.astype(np.float64)
                pin[f"norm{bo}_normalizer"] = norm
            pin["norm_eabs"], pin["norm_etot"] = eabs, etot
            np.savez_compressed(os.path.join(HERE, f"{name}_pins.npz"), **pin)
            print(name, "ne", ne, "absorbed", fx["absorbed"].mean(), "tests/photon", fx["tests_per_photon"].mean())


if __name__ == "__main__":
    main(tuple(sys.argv[1:]))
