"""Front ends on the GPU: the command line (JSON in, .bin/.mch out, .mch
replay) and the pmmc-style run(dict)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from mmc_gb300 import io, meshgen, pmmc
from mmc_gb300.core import Mesh, SimConfig, simulate

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cli_run_and_replay(gpu_ready, tmp_path):
    m = meshgen.inclusion_cube(n=12, jitter=0.4, seed=3)
    cfg = {"Session": {"ID": "cli", "Photons": 20000, "RNGSeed": 5, "BasisOrder": 0, "DoSaveSeed": 1},
           "Domain": {"Media": m.media.tolist()},
           "Mesh": {"MeshNode": m.node.tolist(), "MeshElem": np.c_[m.elem, m.label].tolist()},
           "Forward": {"T0": 0.0, "T1": 5e-9, "Dt": 1e-9},
           "Optode": {"Source": {"Pos": [30, 30, 0], "Dir": [0, 0, 1]},
                      "Detector": [{"Pos": [40, 30, 0], "R": 3}, {"Pos": [45, 30, 0], "R": 3}]}}
    (tmp_path / "in.json").write_text(json.dumps(cfg))
    env = dict(os.environ, PYTHONPATH=ROOT)
    r = subprocess.run([sys.executable, "-m", "mmc_gb300", "-f", "in.json", "-s", "base", "-d", "1", "-q", "1",
                        "-F", "bin"], cwd=tmp_path, env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    field = io.read_bin(str(tmp_path / "base.bin"), 5)
    detp, hdr, seeds = io.read_mch(str(tmp_path / "base.mch"))
    assert field.shape == (5, m.ne) and hdr["savedphoton"] > 0 and seeds is not None
    # same run through the Python API
    mesh = Mesh(m.node, m.elem, m.label)
    ref = simulate(mesh, SimConfig(media=m.media, nphoton=20000, seed=5, srcpos=(30, 30, 0), tend=5e-9, tstep=1e-9,
                                   basisorder=0, issavedet=1, issaveseed=1,
                                   detpos=np.array([[40, 30, 0, 3], [45, 30, 0, 3]], np.float32)))
    np.testing.assert_allclose(field, ref.field, rtol=1e-9)
    # replay of detector 1 from the .mch file (-E file.mch -P 1 -O l)
    r = subprocess.run([sys.executable, "-m", "mmc_gb300", "-f", "in.json", "-s", "rep", "-E", "base.mch", "-P", "1",
                        "-O", "l", "-d", "1", "-U", "0", "-F", "bin"], cwd=tmp_path, env=env, capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    rep = io.read_bin(str(tmp_path / "rep.bin"), 5)
    assert rep.sum() > 0
    d2, h2, _ = io.read_mch(str(tmp_path / "rep.mch"))
    assert h2["savedphoton"] == int((detp[:, 0] == 1).sum())
    # the reference's default output format is text: <session>.dat, `index value` per gate
    r = subprocess.run([sys.executable, "-m", "mmc_gb300", "-f", "in.json", "-s", "txt"], cwd=tmp_path, env=env,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    txt = np.loadtxt(tmp_path / "txt.dat")
    assert txt.shape == (5 * m.ne, 2) and np.array_equal(txt[:m.ne, 0], np.arange(1, m.ne + 1))
    np.testing.assert_allclose(txt[:, 1].reshape(5, m.ne), field, rtol=1e-5, atol=1e-30)
    r = subprocess.run([sys.executable, "-m", "mmc_gb300", "-f", "in.json", "-F", "jnii"], cwd=tmp_path, env=env,
                       capture_output=True, text=True)
    assert r.returncode != 0 and "not supported" in r.stderr


def test_pmmc_run_matches_api(gpu_ready):
    m = meshgen.inclusion_cube(n=10, jitter=0.4, seed=2)
    cfg = dict(node=m.node, elem=m.elem, elemprop=m.label, prop=m.media, srcpos=[30, 30, 0], srcdir=[0, 0, 1],
               nphoton=30000, seed=11, tstart=0.0, tend=5e-9, tstep=1e-9, issavedet=1, issaveseed=1,
               detpos=[[40, 30, 0, 3]], basisorder=1, outputtype="flux")
    out = pmmc.run(cfg)
    assert out["flux"].shape == (m.nn, 5)                       # [datalen, maxgate], as pmmc
    assert out["detp"].shape[0] == 1 + 2 * 2 + 1               # [columns, ndetected]
    assert out["seeds"].shape[0] == 16
    mesh = Mesh(m.node, m.elem, m.label)
    ref = simulate(mesh, SimConfig(media=m.media, nphoton=30000, seed=11, srcpos=(30, 30, 0), tend=5e-9, tstep=1e-9,
                                   basisorder=1, issavedet=1, issaveseed=1, detpos=np.array([[40, 30, 0, 3]], np.float32)))
    np.testing.assert_allclose(out["flux"], ref.field.T, rtol=1e-9)
    # replay through pmmc with the seed matrix
    rep = pmmc.run(dict(cfg, seed=out["seeds"], detphotons=out["detp"], outputtype="wl", isnormalized=0))
    assert rep["flux"].sum() > 0
    with pytest.raises(ValueError):
        pmmc.run(dict(cfg, prop=m.media[:1]))
    # issave2pt=0: records only, no fluence output (src/pmmc.cpp:1154)
    rec = pmmc.run(dict(cfg, issave2pt=0))
    assert "flux" not in rec and rec["detp"].shape == out["detp"].shape
    # patterns sharing each photon: a leading srcnum axis, [srcnum, datalen, maxgate]
    pat = np.random.default_rng(1).uniform(0.1, 1, (2, 4, 3)).astype(np.float32)
    sh = pmmc.run(dict(cfg, srctype="pattern", srcpos=[20, 20, 0.5], srcparam1=[20, 0, 0, 4], srcparam2=[0, 20, 0, 3],
                       srcpattern=pat, issavedet=0, basisorder=0))
    assert sh["flux"].shape == (2, m.ne, 5)


def test_cli_sources_grid_and_exiting_weight(gpu_ready, tmp_path):
    """The command line with a wide-field source (Optode.Source Type/Param1), the
    dual-grid method (-M G, Domain.Step) and the exiting weight (-X 1)."""
    m = meshgen.homogeneous_cube(n=10)
    label = m.label.copy()
    label[meshgen.centroids(m.node, m.elem)[:, 2] < 6.0] = -1  # the reference's source candidates
    cfg = {"Session": {"ID": "g", "Photons": 20000, "RNGSeed": 5, "DoSaveRef": 1},
           "Domain": {"Media": m.media.tolist(), "Step": [2.0, 2.0, 2.0]},
           "Mesh": {"MeshNode": m.node.tolist(), "MeshElem": np.c_[m.elem, label].tolist()},
           "Forward": {"T0": 0.0, "T1": 5e-9, "Dt": 5e-9},
           "Optode": {"Source": {"Type": "disk", "Pos": [30, 30, 0], "Dir": [0, 0, 1], "Param1": [10, 0, 0, 0]}}}
    (tmp_path / "in.json").write_text(json.dumps(cfg))
    env = dict(os.environ, PYTHONPATH=ROOT)
    r = subprocess.run([sys.executable, "-m", "mmc_gb300", "-f", "in.json", "-M", "G", "-U", "0", "-F", "bin"],
                       cwd=tmp_path, env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    grid = io.read_bin(str(tmp_path / "g.bin"), 1)
    assert grid.shape == (1, 31 * 31 * 31) and grid.sum() > 0
    dref = np.loadtxt(tmp_path / "g_dref.dat")
    assert dref.shape[0] > 0 and dref[:, 1].sum() > 0


def test_pmmc_sources_grid_and_exiting_weight(gpu_ready):
    m = meshgen.homogeneous_cube(n=10)
    label = m.label.copy()
    label[meshgen.centroids(m.node, m.elem)[:, 2] < 6.0] = 0
    out = pmmc.run(dict(node=m.node, elem=m.elem, elemprop=label, prop=m.media, srcpos=[20, 20, 0],
                        srcdir=[0, 0, 1], srctype="planar", srcparam1=[20, 0, 0, 0], srcparam2=[0, 20, 0, 0],
                        nphoton=20000, seed=3, tstart=0.0, tend=5e-9, tstep=1e-9, method="grid", steps=[3, 3, 3],
                        issaveref=1, isnormalized=1))
    assert out["flux"].shape == (21, 21, 21, 5)   # [dim.x, dim.y, dim.z, maxgate]
    assert out["dref"].shape[1] == 5 and out["dref"].sum() > 0


def test_exit_image_through_pmmc_and_cli(gpu_ready, tmp_path):
    """issaveexit=2: pmmc returns the exit image [nx, ny, maxgate] as 'detp'
    and the command line writes <session>.img; the image per launched photon
    agrees with the reference's run of the same configuration
    (tests/golden/detimage_cube6k.npz) within sampling noise."""
    import golden_checks as gc
    fx = gc.load("detimage_cube6k")
    m = meshgen.homogeneous_cube(n=10)
    n = 200000
    out = pmmc.run(dict(node=m.node, elem=m.elem, elemprop=m.label, prop=m.media, srcpos=[30, 30, 0], srcdir=[0, 0, 1],
                        nphoton=n, seed=5, tstart=0.0, tend=5e-9, tstep=1e-9, issavedet=1, issaveexit=2,
                        detpos=fx["detpos"], detparam1=fx["detparam1"], detparam2=fx["detparam2"], basisorder=0))
    img = out["detp"]
    assert img.shape == (8, 8, 5)
    ref = fx["img"].transpose(2, 1, 0) / 20000.0
    assert img.sum() / n == pytest.approx(ref.sum(), rel=0.05)
    hot = ref.sum(2) > 0.02 * ref.sum(2).max()  # well-populated pixels: within 20%
    np.testing.assert_allclose(img.sum(2)[hot] / n, ref.sum(2)[hot], rtol=0.2)
    # the command line writes the same image from its own run
    cfgj = {"Session": {"ID": "img", "Photons": 50000, "RNGSeed": 5, "DoSaveExit": 2, "DoPartialPath": 1,
                        "BasisOrder": 0},
            "Domain": {"Media": [dict(mua=float(r[0]), mus=float(r[1]), g=float(r[2]), n=float(r[3])) for r in m.media]},
            "Mesh": {"MeshNode": m.node.tolist(), "MeshElem": np.c_[m.elem, m.label].tolist()},
            "Forward": {"T0": 0.0, "T1": 5e-9, "Dt": 1e-9},
            "Optode": {"Source": {"Pos": [30, 30, 0], "Dir": [0, 0, 1], "Param1": [40, 0, 0, 8], "Param2": [0, 40, 0, 8]},
                       "Detector": [{"Pos": [10, 10, 0], "R": 30}]}}
    (tmp_path / "in.json").write_text(json.dumps(cfgj))
    r = subprocess.run([sys.executable, "-m", "mmc_gb300", "-f", "in.json"], cwd=tmp_path,
                       env=dict(os.environ, PYTHONPATH=ROOT), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    cli = np.fromfile(tmp_path / "img.img", np.float32).reshape(5, 8, 8)
    assert cli.sum() / 50000 == pytest.approx(ref.sum(), rel=0.08)
