"""Generates tests/golden/replay_shell.npz: statistics of the reference MMC CPU
engine's replay outputs (oracle/_ref, built from the reference sources by
oracle/build_ref.sh).  Development container only; the fixture is committed.

Workload (the differentiation workload): the 4-layer spherical-shell mesh
(cube [0,60]^3 mm, 1 mm grid, 6 tets per voxel, +/-0.25 mm orientation-safe
jitter with seed 4321; layers by centroid radius r<18, 18-20, 20-23, 23-25 mm,
void beyond 25 mm), pencil source at (30,30,5.5) mm pointing +z (0.5 mm inside
the outer surface), one gate 0-5 ns, 8 detectors of radius 1.5 mm on the
r = 25 mm surface in the y = 30 plane at polar angles 10..80 degrees,
1e6 photons per forward run, no roulette (minenergy 0: the reference's seed-file
replay turns roulette off, src/mmc_mesh.c:895, so a forward photon that had
drawn a roulette number would not retrace its path).

Each of the 10 runs (plus 6 null runs):
  1. a forward run with seed SEED0+k, one OpenMP thread, saving the detected
     photons and the RNG state each started from (oracle/ref_driver.c dumps
     cfg.exportdetected and cfg.exportseed, src/mmc_host.c:405-409);
  2. an .mch file holding those photons' seeds and path lengths, written in the
     column layout the reference's seed-file reader takes its replay weights
     and times from (src/mmc_mesh.c:815-898: detector id in column 0, path
     lengths of media 1..M in columns 2..M+1, launch weight last);
  3. two replays of all detected photons by the reference engine
     (-E run.mch -O L and -O P, unnormalized): the raw per-element
     "wl" (replay weight x path length, src/mmc_raytrace.c:1527-1530) and "wp"
     (replay weight x path length x mus / slen0, :1535-1543) deposits.
Stored: per-element means/sds of wl and wp over a random subset of the visited
elements, the totals per run, the detected counts, and the null calibration.

  python tests/golden/make_replay_golden.py
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
NAME = "replay_shell"
SRCPOS = (30.0, 30.0, 5.5)


def detectors():
    c = np.array([30.0, 30.0, 30.0])
    th = np.deg2rad(np.arange(10, 90, 10))
    return np.array([[*(c + 25.0 * np.array([np.sin(a), 0.0, -np.cos(a)])), 1.5] for a in th], np.float32)


def forward(wd, seed):
    sess = f"{NAME}_{seed}_fwd"
    detp_out, seed_out = os.path.join(wd, sess + ".detp"), os.path.join(wd, sess + ".seed")
    cmd = [mg.REF + "_detp", "-f", os.path.join(wd, NAME + ".json"), "-c", "sse", "-M", "s", "-C", "0", "-b", "1",
           "-U", "0", "-F", "bin", "-s", sess, "-E", str(seed), "-n", str(PHOTONS), "-d", "1", "-q", "1", "-e", "0"]
    env = dict(os.environ, OMP_NUM_THREADS="1", MMCGB_DETP_OUT=detp_out, MMCGB_SEED_OUT=seed_out)
    p = subprocess.run(cmd, cwd=wd, env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError(p.stdout[-2000:])
    os.remove(os.path.join(wd, sess + ".bin"))
    buf = open(detp_out, "rb").read()
    count, cols = struct.unpack("<ii", buf[:8])
    detp = np.frombuffer(buf, np.float32, count=count * cols, offset=8).reshape(count, cols).copy()
    buf = open(seed_out, "rb").read()
    n, seedbyte = struct.unpack("<ii", buf[:8])
    assert n == count and seedbyte == 16
    seeds = np.frombuffer(buf, np.uint8, count=n * 16, offset=8).reshape(n, 16).copy()
    return detp, seeds


def write_replay_mch(path, detp, seeds, M):
    """The reference's seed-file reader (src/mmc_mesh.c:815-898) takes the
    detector id from column 0, path lengths of media 1..M from columns
    2..M+1 and the launch weight from the last column: records are written
    as [detid, total scatter count, ppath_1..ppath_M, w0]."""
    n = len(detp)
    rec = np.zeros((n, M + 3), np.float32)
    rec[:, 0] = detp[:, 0]
    rec[:, 1] = detp[:, 1:1 + M].sum(1)
    rec[:, 2:2 + M] = detp[:, 1 + M:1 + 2 * M]
    rec[:, -1] = detp[:, -1]
    # 64-byte history header (src/mmc_utils.h:168-184)
    hdr = struct.pack("<4sIIIIIIIfIfIiI2i", b"MCXH", 1, M, 8, M + 3, PHOTONS, n, n, 1.0, 16, 1.0, 1, 1, 0, 0, 0)
    with open(path, "wb") as f:
        f.write(hdr)
        f.write(rec.tobytes())
        f.write(np.ascontiguousarray(seeds, np.uint8).tobytes())


def replay(wd, seed, out):
    sess = f"{NAME}_{seed}_{out}"
    cmd = [mg.REF + "_detp", "-f", os.path.join(wd, NAME + ".json"), "-c", "sse", "-M", "s", "-C", "0", "-b", "1",
           "-U", "0", "-F", "bin", "-s", sess, "-E", os.path.join(wd, f"{NAME}_{seed}.mch"), "-O", out, "-P", "0"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    p = subprocess.run(cmd, cwd=wd, env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError(p.stdout[-2000:])
    f = os.path.join(wd, sess + ".bin")
    raw = np.fromfile(f, np.float64)
    os.remove(f)
    return raw


def one(wd, seed, M):
    detp, seeds = forward(wd, seed)
    write_replay_mch(os.path.join(wd, f"{NAME}_{seed}.mch"), detp, seeds, M)
    return dict(ndet=len(detp), det_ids=np.bincount(detp[:, 0].astype(int), minlength=9)[1:],
                wl=replay(wd, seed, "L"), wp=replay(wd, seed, "P"))


def main():
    if not os.path.exists(mg.REF + "_detp"):
        subprocess.run(["bash", os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    m = meshgen.shell_mesh(n=60, jitter=0.25, seed=4321)
    M = m.media.shape[0] - 1
    seeds = [SEED0 + k for k in range(NRUNS)] + [SEED0 + 1000 + k for k in range(NNULL)]
    with tempfile.TemporaryDirectory() as wd:
        c = dict(mesh=m, photons=PHOTONS, t1=5e-9, dt=5e-9, det=detectors(), src=dict(Pos=list(SRCPOS), Dir=[0, 0, 1.0]))
        c["e0"] = oracle.initelem(m.node, m.elem, m.label, SRCPOS)
        mg.write_json(os.path.join(wd, NAME + ".json"), NAME, c)
        with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
            res = list(ex.map(lambda s: one(wd, s, M), seeds))
    runs, nulls = res[:NRUNS], res[NRUNS:]
    rng = np.random.default_rng(zlib.crc32(NAME.encode()))
    fx = dict(ne=m.ne, photons=PHOTONS, seeds=np.array(seeds[:NRUNS]), detectors=detectors(),
              ndet=np.array([r["ndet"] for r in runs], np.float64),
              det_ids=np.array([r["det_ids"] for r in runs], np.float64))
    for key in ("wl", "wp"):
        f = np.stack([r[key] for r in runs])
        mean, sd = f.mean(0), f.std(0, ddof=1)
        visited = np.flatnonzero(mean > 0)
        sub = np.sort(rng.choice(visited, size=min(150000, visited.size), replace=False)).astype(np.int32)
        fx[key + "_sub"] = sub
        fx[key + "_mean"] = mean[sub].astype(np.float32)
        fx[key + "_std"] = sd[sub].astype(np.float32)
        fx[key + "_total"] = f.sum(1)
        st = [gc.zstats(r[key][sub], fx[key + "_mean"], fx[key + "_std"]) for r in nulls]
        fx["null_" + key + "_frac"] = np.array([t[0] for t in st])
        fx["null_" + key + "_meanz"] = np.array([t[1] for t in st])
        print(key, "total", f.sum(1).mean(), "+-", f.sum(1).std(ddof=1), "well-sampled",
              gc.zstats(fx[key + "_mean"], fx[key + "_mean"], fx[key + "_std"])[2], "null", fx["null_" + key + "_frac"])
    print("detected per run", fx["ndet"].mean(), "per detector", fx["det_ids"].mean(0))
    np.savez_compressed(os.path.join(HERE, NAME + ".npz"), **fx)


if __name__ == "__main__":
    main()
