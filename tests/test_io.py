"""File formats and front-end parsing (no GPU): .mch round trip, JSON input
(inline mesh and MeshID .dat files), pmmc dict parsing, .bin/.dat writers."""
import json
import os

import numpy as np
import pytest

from mmc_gb300 import io, meshgen, pmmc


def test_mch_roundtrip(tmp_path):
    rng = np.random.default_rng(0)
    detp = rng.random((37, 6)).astype(np.float32)
    seeds = rng.integers(0, 255, (37, 16), dtype=np.uint8)
    p = str(tmp_path / "a.mch")
    io.write_mch(p, detp, seeds, maxmedia=2, detnum=4, totalphoton=1000, detected=40, unitinmm=1.0)
    d, h, s = io.read_mch(p)
    assert h["magic"] == b"MCXH" and h["version"] == 1 and h["colcount"] == 6 and h["savedphoton"] == 37
    assert h["detected"] == 40 and h["seedbyte"] == 16 and os.path.getsize(p) == 64 + 37 * 6 * 4 + 37 * 16
    assert np.array_equal(d, detp) and np.array_equal(s, seeds)


def _write_case(tmp_path, inline=True):
    m = meshgen.inclusion_cube(n=4, jitter=0.3, seed=1)
    cfg = {"Session": {"ID": "t", "Photons": 1234, "RNGSeed": 77, "DoMismatch": 1, "BasisOrder": 0},
           "Domain": {"Media": [{"mua": 0, "mus": 0, "g": 1, "n": 1}, {"mua": 0.005, "mus": 1, "g": 0.01, "n": 1.37},
                                {"mua": 0.05, "mus": 5, "g": 0.9, "n": 1.37}]},
           "Forward": {"T0": 0.0, "T1": 5e-9, "Dt": 1e-9},
           "Optode": {"Source": {"Pos": [30, 30, 0], "Dir": [0, 0, 1]},
                      "Detector": [{"Pos": [40, 30, 0], "R": 2}]}}
    if inline:
        cfg["Mesh"] = {"MeshNode": m.node.tolist(), "MeshElem": np.c_[m.elem, m.label].tolist(), "InitElem": 0}
    else:
        cfg["Mesh"] = {"MeshID": "x"}
        with open(tmp_path / "node_x.dat", "w") as f:
            f.write(f"1\t{m.nn}\n")
            for i, p in enumerate(m.node):
                f.write(f"{i + 1}\t{p[0]:.8e}\t{p[1]:.8e}\t{p[2]:.8e}\n")
        with open(tmp_path / "elem_x.dat", "w") as f:
            f.write(f"1\t{m.ne}\n")
            for i, (e, lab) in enumerate(zip(m.elem, m.label)):
                f.write(f"{i + 1}\t{e[0]}\t{e[1]}\t{e[2]}\t{e[3]}\t{lab}\n")
    p = tmp_path / "in.json"
    p.write_text(json.dumps(cfg))
    return str(p), m


def test_json_input_with_jdata_mesh(tmp_path):
    """MeshNode / MeshElem as zlib-compressed JData arrays, as the reference's
    tools write large meshes, read like the inline lists."""
    import base64
    import zlib
    path, m = _write_case(tmp_path)
    cfg = json.loads(open(path).read())

    def jd(a, t):
        return {"_ArrayType_": t, "_ArraySize_": list(a.shape), "_ArrayZipType_": "zlib",
                "_ArrayZipSize_": [1, int(a.size)], "_ArrayZipData_": base64.b64encode(zlib.compress(a.tobytes())).decode()}
    cfg["Mesh"]["MeshNode"] = jd(np.ascontiguousarray(m.node, np.float32), "single")
    cfg["Mesh"]["MeshElem"] = jd(np.ascontiguousarray(np.c_[m.elem, m.label], np.int32), "int32")
    p = tmp_path / "jd.json"
    p.write_text(json.dumps(cfg))
    mesh, _, _ = io.load_input(str(p))
    assert np.array_equal(mesh["node"], m.node) and np.array_equal(mesh["elem"], m.elem)
    assert np.array_equal(mesh["label"], m.label)


@pytest.mark.parametrize("inline", [True, False])
def test_json_input(tmp_path, inline):
    path, m = _write_case(tmp_path, inline)
    mesh, cfg, meta = io.load_input(path)
    np.testing.assert_allclose(mesh["node"], m.node, rtol=1e-6)
    assert np.array_equal(mesh["elem"], m.elem) and np.array_equal(mesh["label"], m.label)
    assert cfg.nphoton == 1234 and cfg.seed == 77 and cfg.maxgate == 5 and cfg.basisorder == 0
    assert cfg.issavedet == 1 and cfg.detpos.shape == (1, 4) and meta["session"] == "t"
    assert cfg.media.shape == (3, 4) and cfg.ismomentum == 0
    c = json.loads(open(path).read())
    c["Session"]["DoDCS"] = 1  # the reference's key for momentum transfer (src/mmc_utils.c:2269)
    open(path, "w").write(json.dumps(c))
    assert io.load_input(path)[1].ismomentum == 1


def test_pmmc_dict_parsing():
    m = meshgen.homogeneous_cube(n=3)
    node, elem, label, fnb, sc, seeds = pmmc._parse(dict(
        node=m.node, elem=m.elem, elemprop=m.label, prop=m.media, srcpos=[30, 30, 0], srcdir=[0, 0, 2],
        nphoton=1e4, tstart=0, tend=5e-9, tstep=1e-9, issavedet=1, detpos=[[40, 30, 0, 2]], outputtype="fluence",
        method="elem", seed=99))
    assert sc.nphoton == 10000 and sc.seed == 99 and sc.outputtype == "fluence" and sc.maxgate == 5
    assert np.allclose(sc.srcdir, (0, 0, 1)) and seeds is None
    with pytest.raises(ValueError):
        pmmc._parse(dict(node=m.node, elem=m.elem, prop=m.media, srcpos=[1, 1, 1], method="plucker"))
    with pytest.raises(ValueError):
        pmmc._parse(dict(node=m.node, elem=m.elem, prop=m.media, srcpos=[1, 1, 1], srctype="laser"))
    # source types, parameters, focus (the 4th srcdir entry) and patterns (Fortran order, x fastest)
    pat = np.arange(6, dtype=np.float32).reshape(3, 2, order="F")
    *_, sc, _ = pmmc._parse(dict(node=m.node, elem=m.elem, prop=m.media, srcpos=[1, 1, 1], srctype="pattern",
                                srcdir=[0, 0, 1, -5], srcparam1=[10, 0, 0, 3], srcparam2=[0, 10, 0, 2],
                                srcpattern=pat))
    assert sc.srctype == "pattern" and sc.focus == -5 and sc.srcparam1 == (10, 0, 0, 3)
    assert sc.srcpattern.tolist() == [0, 1, 2, 3, 4, 5]
    # a uint8 [16, N] seed matrix selects replay
    *_, s2 = pmmc._parse(dict(node=m.node, elem=m.elem, prop=m.media, srcpos=[30, 30, 0],
                              seed=np.zeros((16, 5), np.uint8)))
    assert s2.shape == (16, 5)


def test_bin_and_dat_writers(tmp_path):
    f = np.arange(12, dtype=np.float64).reshape(3, 4)
    io.write_bin(str(tmp_path / "a.bin"), f)
    assert np.array_equal(io.read_bin(str(tmp_path / "a.bin"), 3), f)
    io.write_dat(str(tmp_path / "a.dat"), f)
    lines = open(tmp_path / "a.dat").read().split("\n")
    assert lines[0].split("\t")[0] == "1" and len([x for x in lines if x]) == 12


def test_builtin_benchmarks_and_session_flags():
    """-Q inputs (src/mmc_bench.c:44-190): the 6-tet 60 mm cube with the benchmark's
    source, detectors and mismatch flag; Session.DebugFlag letters or bit mask
    and Session.RayTracer reach the front end."""
    for name, mismatch in (("dmmc-cube60", 0), ("dmmc-cube60b", 1)):
        mesh, cfg, meta = io.load_input(io.builtin_benchmark(name))
        assert mesh["elem"].shape == (6, 4) and mesh["node"].shape == (8, 3)
        assert cfg.isreflect == mismatch and cfg.e0 == 2 and cfg.nphoton == 1_000_000
        assert cfg.srcpos == (30.1, 30.2, 0.0) and cfg.detpos.shape == (4, 4)
        assert meta["session"] == name
    with pytest.raises(ValueError):
        io.builtin_benchmark("edgeimmc")
    d = io.builtin_benchmark("dmmc-cube60")
    d["Session"].update(DebugFlag="TM", RayTracer="g")
    _, _, meta = io.load_input(d)
    assert meta["debugflag"] == "TM" and meta["raytracer"] == "g"
    d["Session"]["DebugFlag"] = (1 << 9) | (1 << 13)   # T and M as a bit mask (src/mmc_utils.c:139)
    assert io.load_input(d)[2]["debugflag"] == "TM"


def test_cli_lists_builtin_benchmarks():
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-m", "mmc_gb300", "-Q"], env=dict(os.environ, PYTHONPATH=root),
                       capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.split() == ["Built-in", "benchmarks:", "dmmc-cube60", "dmmc-cube60b"]
    # the reference's flags: -v prints the version; -m is its MC method (1, MCML, is refused), not momentum
    r = subprocess.run([sys.executable, "-m", "mmc_gb300", "-v"], env=dict(os.environ, PYTHONPATH=root),
                       capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.startswith("mmc_gb300")
    r = subprocess.run([sys.executable, "-m", "mmc_gb300", "-Q", "dmmc-cube60", "-m", "1"],
                       env=dict(os.environ, PYTHONPATH=root), capture_output=True, text=True)
    assert r.returncode != 0 and "MCML" in r.stderr


def test_pmmc_debuglevel_parsing():
    """debuglevel letters of pmmc (src/pmmc.cpp:692-710): M asks for trajectories."""
    m = meshgen.homogeneous_cube(n=2)
    base = dict(node=m.node, elem=m.elem, prop=m.media, srcpos=[30, 30, 0])
    sc = pmmc._parse(dict(base, debuglevel="M", maxjumpdebug=500))[4]
    assert sc.maxjumpdebug == 500
    assert pmmc._parse(dict(base, debuglevel="m"))[4].maxjumpdebug == 10_000_000
    assert pmmc._parse(dict(base, debuglevel="R"))[4].maxjumpdebug == 0
    for bad in ("", "Q"):
        with pytest.raises(ValueError):
            pmmc._parse(dict(base, debuglevel=bad))


def test_shared_patterns_from_json_and_pmmc(tmp_path):
    """A 3-D pattern [srcnum, Nx, Ny] (srcnum, Ny > 1) of a pattern source holds
    patterns sharing each photon: from a JData array in JSON (zlib-compressed,
    as the reference reads it, or plain) and from a pmmc array; both give the
    engine's pixel-major layout (pixel y*Nx + x, patterns adjacent)."""
    import base64
    import zlib
    K, nx, ny = 3, 4, 2
    A = np.arange(K * nx * ny, dtype=np.float32).reshape(K, nx, ny)  # [pattern, x, y]
    want = np.ascontiguousarray(A.transpose(2, 1, 0)).ravel()
    path, m = _write_case(tmp_path)
    cfg = json.loads(open(path).read())
    src = dict(Type="pattern", Pos=[10, 10, 0], Dir=[0, 0, 1], Param1=[20, 0, 0, nx], Param2=[0, 20, 0, ny])
    for enc in ("zlib", "gzip", "plain"):
        if enc == "plain":
            src["Pattern"] = {"_ArrayType_": "single", "_ArraySize_": [K, nx, ny], "_ArrayData_": A.ravel().tolist()}
        else:
            co = zlib.compressobj(wbits=31 if enc == "gzip" else 15)
            z = co.compress(A.tobytes()) + co.flush()
            src["Pattern"] = {"_ArrayType_": "single", "_ArraySize_": [K, nx, ny], "_ArrayZipType_": enc,
                              "_ArrayZipSize_": [1, A.size], "_ArrayZipData_": base64.b64encode(z).decode()}
        cfg["Optode"]["Source"] = src
        p = tmp_path / f"pat_{enc}.json"
        p.write_text(json.dumps(cfg))
        _, sc, _ = io.load_input(str(p))
        assert sc.srcnum == K and np.array_equal(sc.srcpattern, want), enc
    *_, sc, _ = pmmc._parse(dict(node=m.node, elem=m.elem, prop=m.media, srcpos=[10, 10, 0], srctype="pattern",
                                srcparam1=[20, 0, 0, nx], srcparam2=[0, 20, 0, ny], srcpattern=np.asfortranarray(A)))
    assert sc.srcnum == K and np.array_equal(sc.srcpattern, want)
    # a 2-D pattern stays one pattern; so does a 3-D array for the 3-D pattern source
    *_, sc, _ = pmmc._parse(dict(node=m.node, elem=m.elem, prop=m.media, srcpos=[10, 10, 0], srctype="pattern3d",
                                srcparam1=[K, nx, ny, 0], srcpattern=A))
    assert sc.srcnum == 1


def test_unsupported_outputs_are_errors(tmp_path):
    """The reference's RF (frequency-domain) and adjoint outputs are refused by
    name rather than replaced by another output."""
    path, m = _write_case(tmp_path)
    cfg = json.loads(open(path).read())
    for key, val in (("OutputType", "R"), ("OutputType", "A"), ("OutputType", "q")):
        c = json.loads(json.dumps(cfg))
        c["Session"][key] = val
        p = tmp_path / f"o_{val}.json"
        p.write_text(json.dumps(c))
        with pytest.raises(ValueError):
            io.load_input(str(p))
    c = json.loads(json.dumps(cfg))
    c["Forward"]["Omega"] = 6.28e8
    p = tmp_path / "omega.json"
    p.write_text(json.dumps(c))
    with pytest.raises(ValueError, match="RF"):
        io.load_input(str(p))
    with pytest.raises(ValueError, match="RF"):
        pmmc._parse(dict(node=m.node, elem=m.elem, prop=m.media, srcpos=[30, 30, 0], omega=1e8))
    assert io.output_type("F") == "fluence" and io.output_type("wl") == "wl"
    for k in ("mcmethod", "isextdet", "isnodalmua", "isnodalmusp", "adjointmode"):
        with pytest.raises(ValueError, match=k):
            pmmc._parse(dict(node=m.node, elem=m.elem, prop=m.media, srcpos=[30, 30, 0], **{k: 1}))
    pmmc._parse(dict(node=m.node, elem=m.elem, prop=m.media, srcpos=[30, 30, 0], mcmethod=0, isextdet=0))
