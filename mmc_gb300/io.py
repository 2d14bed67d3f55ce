"""File formats of the reference's front ends.

* JSON input (``mmc -f input.json``; the subset the photon path reads,
  src/mmc_utils.c:1566-2392): Session, Domain.Media, Mesh (MeshNode/MeshElem
  inline, or MeshID naming node_/elem_/prop_/facenb_<ID>.dat files),
  Forward (T0/T1/Dt/N0), Optode.Source (Pos/Dir), Optode.Detector[{Pos, R}].
* ``.mch`` detected-photon history: 64-byte header (magic "MCXH", version 1,
  src/mmc_utils.h:168-184), float32 records, then 16-byte RNG seeds
  (src/mmc_mesh.c:1978-2010).
* ``.bin`` output: raw float64 [gate][datalen] (src/mmc_utils.c:966-990).
* ``.dat`` output: text "index value" per line (src/mmc_mesh.c:1759-1813).
"""
from __future__ import annotations

import json
import os
import struct
from typing import Optional

import numpy as np

from .core import SOURCE_TYPES, SimConfig

MCH_HEADER = struct.Struct("<4sIIIIIIIfIfIiI2i")  # 64 bytes
OUTPUT_LETTERS = {"x": "flux", "f": "fluence", "e": "energy", "j": "jacobian", "l": "wl", "p": "wp", "n": "wn"}
OUTPUT_NAMES = {"flux": "flux", "fluence": "fluence", "energy": "energy", "jacobian": "jacobian", "wl": "wl",
                "wp": "wp", "wn": "wn"}
# the reference's frequency-domain (RF) and adjoint outputs, which this library does not provide
UNSUPPORTED_OUTPUTS = {"r": "RF (frequency-domain) fluence", "a": "adjoint mua Jacobian",
                       "d": "adjoint D Jacobian", "u": "adjoint mus Jacobian", "v": "adjoint musp Jacobian",
                       "w": "dual adjoint Jacobian"}


def output_type(code) -> str:
    """The output type named by a -O letter or a name; unsupported ones are an error."""
    k = str(code).lower()
    if k in OUTPUT_LETTERS:
        return OUTPUT_LETTERS[k]
    if k in OUTPUT_NAMES:
        return OUTPUT_NAMES[k]
    if k in UNSUPPORTED_OUTPUTS:
        raise ValueError(f"output type '{code}' ({UNSUPPORTED_OUTPUTS[k]}) is not supported")
    raise ValueError(f"unknown output type '{code}'")


# ---------------------------------------------------------------------------
# .dat meshes (src/mmc_mesh.c:563-780): a "1 count" header line, then rows
# ---------------------------------------------------------------------------
def _read_table(path, ncols, skip_index=True):
    with open(path) as f:
        head = f.readline().split()
        n = int(head[1])
        rows = np.loadtxt(f, max_rows=n, ndmin=2)
    return rows[:, 1:1 + ncols] if skip_index else rows[:, :ncols]


def read_dat_mesh(mesh_id: str, root: str):
    node = _read_table(os.path.join(root, f"node_{mesh_id}.dat"), 3).astype(np.float32)
    el = _read_table(os.path.join(root, f"elem_{mesh_id}.dat"), 5)
    elem = el[:, :4].astype(np.int32)
    label = el[:, 4].astype(np.int32) if el.shape[1] > 4 else np.ones(len(el), np.int32)
    out = dict(node=node, elem=elem, label=label)
    fnb = os.path.join(root, f"facenb_{mesh_id}.dat")
    if os.path.exists(fnb):
        out["facenb"] = _read_table(fnb, 4, skip_index=False).astype(np.int32)
    prop = os.path.join(root, f"prop_{mesh_id}.dat")
    if os.path.exists(prop):
        p = _read_table(prop, 4).astype(np.float32)
        out["media"] = np.vstack([[0.0, 0.0, 1.0, 1.0], p]).astype(np.float32)
    return out


_JDATA_TYPES = {"single": np.float32, "double": np.float64, "int32": np.int32, "uint32": np.uint32,
                "int8": np.int8, "uint8": np.uint8, "int16": np.int16, "uint16": np.uint16}


def _jdata_array(obj) -> np.ndarray:
    """A JData array object: _ArrayData_ (a list) or _ArrayZipData_ (base64 of zlib or
    gzip bytes), row-major, of _ArrayType_ and _ArraySize_."""
    import base64
    import zlib
    dt = _JDATA_TYPES[str(obj.get("_ArrayType_", "double"))]
    shape = [int(x) for x in np.ravel(obj["_ArraySize_"])]
    if "_ArrayZipData_" in obj:
        ztype = str(obj.get("_ArrayZipType_", "zlib")).lower()
        if ztype not in ("zlib", "gzip"):
            raise ValueError(f"JData compression '{ztype}' is not supported (zlib, gzip)")
        raw = zlib.decompress(base64.b64decode(obj["_ArrayZipData_"]), 31 if ztype == "gzip" else 15)
        return np.frombuffer(raw, dt).reshape(shape)
    return np.asarray(obj["_ArrayData_"], dt).reshape(shape)


def _media_from_json(media):
    rows = []
    for m in media:
        if isinstance(m, dict):
            rows.append([m.get("mua", 0.0), m.get("mus", 0.0), m.get("g", 1.0), m.get("n", 1.0)])
        else:
            rows.append(list(m)[:4])
    return np.asarray(rows, np.float32)


def builtin_benchmark(name: str) -> dict:
    """The reference's built-in benchmark inputs (src/mmc_bench.c:44-190) in
    the photon path's scope, as JSON dicts: dmmc-cube60 (no refractive
    mismatch) and dmmc-cube60b (mismatch on), a 60 mm cube of 6 tets (the
    Kuhn split along the main diagonal), mua 0.005 mus 1 g 0.01 n 1.37, 1e6
    photons, pencil at (30.1, 30.2, 0) +z, one 5 ns gate, 4 detectors R=1 mm
    on z=0 at 10 mm from the axis.  The implicit-MMC benchmarks (edgeimmc,
    nodeimmc, faceimmc) need the iMMC tracer, which is not built."""
    if name not in BENCHMARKS:
        raise ValueError(f"unsupported benchmark '{name}' (built in: {', '.join(BENCHMARKS)})")
    from . import meshgen
    m = meshgen.homogeneous_cube(n=1)
    return {
        "Session": {"ID": name, "Photons": 1e6, "RNGSeed": 1648335518, "OutputFormat": "bin",
                    "DoMismatch": BENCHMARKS[name]},
        "Domain": {"Media": [dict(mua=float(r[0]), mus=float(r[1]), g=float(r[2]), n=float(r[3])) for r in m.media]},
        "Mesh": {"MeshNode": m.node.tolist(), "MeshElem": np.c_[m.elem, m.label].tolist(), "InitElem": 2},
        "Forward": {"T0": 0.0, "T1": 5e-9, "Dt": 5e-9},
        "Optode": {"Source": {"Pos": [30.1, 30.2, 0.0], "Dir": [0.0, 0.0, 1.0]},
                   "Detector": [{"Pos": p, "R": 1.0} for p in
                                ([30.0, 20.0, 0.0], [30.0, 40.0, 0.0], [20.0, 30.0, 0.0], [40.0, 30.0, 0.0])]},
    }


# built-in benchmarks of the photon path -> Session.DoMismatch
BENCHMARKS = {"dmmc-cube60": 0, "dmmc-cube60b": 1}


def load_input(path):
    """Reads a reference JSON input (a path, or the parsed dict); returns
    (mesh dict, SimConfig, meta)."""
    if isinstance(path, dict):
        cfgj, root = path, os.getcwd()
    else:
        with open(path) as f:
            cfgj = json.load(f)
        root = os.path.dirname(os.path.abspath(path))
    ses = cfgj.get("Session", {})
    dom = cfgj.get("Domain", {})
    msh = cfgj.get("Mesh", {})
    fwd = cfgj.get("Forward", {})
    opt = cfgj.get("Optode", {})
    if "MeshNode" in msh:
        # plain nested lists, or JData arrays (N x 3 'single', N x 5 'int32', row-major as stored;
        # src/mmc_utils.c:1594-1675)
        def arr(v, dt):
            return _jdata_array(v).astype(dt) if isinstance(v, dict) else np.asarray(v, dt)
        node = arr(msh["MeshNode"], np.float32).reshape(-1, 3)
        el = arr(msh["MeshElem"], np.int64)
        elem = el[:, :4].astype(np.int32)
        label = el[:, 4].astype(np.int32) if el.shape[1] > 4 else np.ones(len(el), np.int32)
        mesh = dict(node=node, elem=elem, label=label)
    elif "MeshID" in msh:
        mesh = read_dat_mesh(str(msh["MeshID"]), root)
    else:
        raise ValueError("input has neither Mesh.MeshNode/MeshElem nor Mesh.MeshID")
    if "Media" in dom:
        media = _media_from_json(dom["Media"])
    elif "media" in mesh:
        media = mesh["media"]
    else:
        raise ValueError("input has no Domain.Media and no prop_<ID>.dat")
    unit = float(msh.get("LengthUnit", dom.get("LengthUnit", 1.0)))
    if unit != 1.0:
        mesh["node"] = (mesh["node"] * unit).astype(np.float32)
    src = opt.get("Source", {})
    dets = opt.get("Detector", [])
    detpos = None
    if dets:
        detpos = np.array([[*d["Pos"][:3], d.get("R", 1.0)] for d in dets], np.float32)
    # a 4th Dir entry is the focal length; the reference writes NaN/+-inf as strings
    special = {"_NaN_": float("nan"), "_Inf_": float("inf"), "-_Inf_": float("-inf")}
    dir4 = [special[x] if isinstance(x, str) else float(x) for x in src.get("Dir", [0.0, 0.0, 1.0])]
    srcdir = np.asarray(dir4[:3], np.float64)
    srcdir = srcdir / np.linalg.norm(srcdir)
    focus = dir4[3] if len(dir4) > 3 else 0.0
    stype = str(src.get("Type", "pencil")).lower() or "pencil"
    if stype not in SOURCE_TYPES:
        raise ValueError(f"unknown source type '{stype}'")
    pattern = src.get("Pattern")
    srcnum = 1
    if isinstance(pattern, dict) and ("_ArrayZipData_" in pattern or "_ArrayData_" in pattern):
        # a JData array, row-major as stored, turned column-major as the reference does
        # (mcx_convertrow2col); [srcnum, Nx, Ny] holds patterns sharing each photon
        # (src/mmc_utils.c:2086-2104)
        arr = _jdata_array(pattern)
        if arr.ndim == 3 and arr.shape[0] > 1 and arr.shape[2] > 1 and stype == "pattern":
            srcnum = int(arr.shape[0])
        pattern = arr.ravel(order="F")
    elif isinstance(pattern, dict):
        pattern = pattern.get("Data")
    pattern = None if pattern is None else np.asarray(pattern, np.float32).ravel()
    t0 = float(fwd.get("T0", 0.0))
    t1 = float(fwd.get("T1", 5e-9))
    dt = float(fwd.get("Dt", t1 - t0))
    otype = output_type(ses.get("OutputType", "x"))
    if float(fwd.get("Omega", 0.0)) > 0.0:
        raise ValueError("Forward.Omega > 0 asks for RF (frequency-domain) output, which is not supported")
    cfg = SimConfig(
        media=media, nphoton=int(float(ses.get("Photons", 1e6))), seed=int(ses.get("RNGSeed", 0x623F9A9E)),
        srcpos=tuple(float(x) for x in src.get("Pos", [0, 0, 0])[:3]), srcdir=tuple(float(x) for x in srcdir),
        srctype=stype, srcparam1=tuple(float(x) for x in (list(src.get("Param1", [])) + [0.0] * 4)[:4]),
        srcparam2=tuple(float(x) for x in (list(src.get("Param2", [])) + [0.0] * 4)[:4]), focus=focus,
        srcpattern=pattern, srcnum=srcnum,
        e0=int(msh.get("InitElem", 0)), tstart=t0, tend=t1, tstep=dt,
        isreflect=int(ses.get("DoMismatch", 1)), issaveref=int(ses.get("DoSaveRef", 0)),
        gridstep=float(np.ravel(dom.get("Step", [1.0]))[0]), isspecular=int(ses.get("DoSpecular", 0)),
        issavedet=int(ses.get("DoPartialPath", 1 if dets else 0)), issaveseed=int(ses.get("DoSaveSeed", 0)),
        issaveexit=int(ses.get("DoSaveExit", 0)), isnormalized=int(ses.get("DoNormalize", 1)),
        ismomentum=int(ses.get("DoDCS", 0)),
        basisorder=int(ses.get("BasisOrder", 1)), outputtype=otype, nout=float(fwd.get("N0", 1.0)),
        detpos=detpos, unitinmm=unit)
    # the area detector of the exit image (issaveexit = 2): the reference's JSON reader takes its
    # Param1/Param2 from the Source object (src/mmc_utils.c:1811, :2194-2226)
    def vec4(v):
        v = list(np.ravel(v)) if v is not None else []
        return tuple(float(x) for x in v) if len(v) == 4 else (0.0, 0.0, 0.0, 0.0)
    meta_det = dict(detparam1=vec4(src.get("Param1")), detparam2=vec4(src.get("Param2")))
    meta = dict(session=str(ses.get("ID", "default")), outputformat=str(ses.get("OutputFormat", "ascii")),
                **meta_det,
                saveweight=int(ses.get("DoSaveVolume", 1)), root=root,
                raytracer=str(ses.get("RayTracer", "")).lower()[:1],
                debugflag=str(ses.get("DebugFlag", "")) if not isinstance(ses.get("DebugFlag"), int) else
                _debug_letters(ses["DebugFlag"]))
    return mesh, cfg, meta


# debug flag letters by bit, src/mmc_utils.c:139 (T = detected count, M = trajectories)
DEBUG_LETTERS = "SCBWDIOXATRPEM"


def _debug_letters(level: int) -> str:
    return "".join(c for i, c in enumerate(DEBUG_LETTERS) if int(level) >> i & 1)


# ---------------------------------------------------------------------------
# .mch
# ---------------------------------------------------------------------------
def write_mch(path: str, detp: np.ndarray, seeds: Optional[np.ndarray], maxmedia: int, detnum: int,
              totalphoton: int, detected: int, unitinmm: float = 1.0, normalizer: float = 1.0,
              savedetflag: int = 0, srcnum: int = 1):
    detp = np.ascontiguousarray(detp, np.float32)
    n, cols = detp.shape if detp.ndim == 2 else (0, 0)
    seedbyte = 16 if seeds is not None else 0
    hdr = MCH_HEADER.pack(b"MCXH", 1, maxmedia, detnum, cols, int(totalphoton) & 0xFFFFFFFF, int(detected), n,
                          float(unitinmm), seedbyte, float(normalizer), max(1, int(srcnum)), 1, savedetflag, 0, 0)
    with open(path, "wb") as f:
        f.write(hdr)
        f.write(detp.tobytes())
        if seeds is not None:
            f.write(np.ascontiguousarray(seeds, np.uint8).reshape(n, 16).tobytes())


def read_mch(path: str):
    """Returns (records (n, cols) float32, header dict, seeds (n, 16) uint8 or None)."""
    with open(path, "rb") as f:
        buf = f.read()
    h = MCH_HEADER.unpack(buf[:64])
    if h[0] != b"MCXH":
        raise ValueError(f"{path}: not an mch file")
    keys = ["magic", "version", "maxmedia", "detnum", "colcount", "totalphoton", "detected", "savedphoton",
            "unitinmm", "seedbyte", "normalizer", "srcnum", "respin", "savedetflag"]
    hd = dict(zip(keys, h[:14]))
    n, cols = hd["savedphoton"], hd["colcount"]
    detp = np.frombuffer(buf, np.float32, count=n * cols, offset=64).reshape(n, cols).copy()
    seeds = None
    if hd["seedbyte"]:
        off = 64 + n * cols * 4
        seeds = np.frombuffer(buf, np.uint8, count=n * hd["seedbyte"], offset=off).reshape(n, hd["seedbyte"]).copy()
    return detp, hd, seeds


# ---------------------------------------------------------------------------
# fluence outputs
# ---------------------------------------------------------------------------
def write_bin(path: str, field: np.ndarray):
    np.ascontiguousarray(field, np.float64).tofile(path)


def read_bin(path: str, gates: int):
    d = np.fromfile(path, np.float64)
    return d.reshape(gates, -1)


def write_dat(path: str, field: np.ndarray):
    """Text output (mesh_saveweight, src/mmc_mesh.c:1759-1797): per gate and element (or
    node), `index value`; with patterns sharing photons (a trailing srcnum axis)
    `index pattern value` for each pattern."""
    field = np.asarray(field, np.float64)
    with open(path, "w") as f:
        for g in range(field.shape[0]):
            if field.ndim == 3:
                for j in range(field.shape[1]):
                    for k in range(field.shape[2]):
                        f.write(f"{j + 1}\t{k + 1}\t{field[g, j, k]:e}\n")
            else:
                for j, v in enumerate(field[g]):
                    f.write(f"{j + 1}\t{v:e}\n")


# ---------------------------------------------------------------------------
# detector image (issaveexit = 2)
# ---------------------------------------------------------------------------
R_C0 = np.float32(3.335640951981520e-12)  # 1 / speed of light, s/mm


def detector_image(detp: np.ndarray, cfg: SimConfig, detparam1, detparam2) -> np.ndarray:
    """Time-resolved image of the detected photons' exit positions over an area
    detector (mesh_getdetimage, src/mmc_mesh.c:2028-2074): records with exit
    columns (issaveexit) are binned by exit (x, y) into detparam1.w x
    detparam2.w pixels spanning detparam1.x + detparam2.x by detparam1.y +
    detparam2.y from the first detector's (x, y), and by time of flight into the
    gates, each adding its detected weight w0 * exp(-sum mua * L).  Returns
    (maxgate, ny, nx) float32, the layout of the reference's <session>.img.
    As in the reference, the time bin takes the optical path truncated to whole
    millimetres and a photon whose exit lies outside the image is left out."""
    media = np.asarray(cfg.media, np.float32).reshape(-1, 4)
    M = media.shape[0] - 1
    nx, ny = int(detparam1[3]), int(detparam2[3])
    G = cfg.maxgate
    img = np.zeros((G, ny, nx), np.float32)
    detp = np.asarray(detp, np.float32)
    if len(detp) == 0 or nx <= 0 or ny <= 0 or cfg.detpos is None or len(cfg.detpos) == 0:
        return img
    unit = np.float32(cfg.unitinmm)
    path = np.zeros(len(detp), np.float32)
    weight = detp[:, -1].copy()
    for j in range(1, M + 1):
        pp = detp[:, M + j]
        path = (path + pp * media[j, 3]).astype(np.float32)
        weight = (weight * np.exp(-(pp * media[j, 0] * unit)).astype(np.float32)).astype(np.float32)
    ntg = (path.astype(np.int32).astype(np.float32) * R_C0 / np.float32(cfg.tstep)).astype(np.int32)
    ntg = np.minimum(ntg, G - 1)
    x0, y0 = np.float32(cfg.detpos[0][0]), np.float32(cfg.detpos[0][1])
    xr = np.float32(detparam1[0]) + np.float32(detparam2[0])
    yr = np.float32(detparam1[1]) + np.float32(detparam2[1])
    xi = ((detp[:, -7] - x0) / xr * np.float32(nx)).astype(np.int32)  # truncation toward zero, as C
    yi = ((detp[:, -6] - y0) / yr * np.float32(ny)).astype(np.int32)
    ok = (xi >= 0) & (xi <= nx - 1) & (yi >= 0) & (yi <= ny - 1)
    np.add.at(img, (ntg[ok], yi[ok], xi[ok]), weight[ok])
    return img
