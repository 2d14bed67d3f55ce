"""ctypes wrapper of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker.  The product never imports it.
The oracle restates the reference's GPU photon path in plain C; see
oracle/mmc_oracle.h for what it follows and how it differs.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
OUTPUT_TYPES = {"flux": 0, "fluence": 1, "energy": 2, "jacobian": 3, "wl": 4, "wp": 5, "wn": 16}
SOURCE_TYPES = {"pencil": 0, "isotropic": 1, "cone": 2, "gaussian": 3, "planar": 4, "pattern": 5, "fourier": 6,
                "arcsine": 7, "disk": 8, "fourierx": 9, "fourierx2d": 10, "zgaussian": 11, "line": 12, "slit": 13,
                "pencilarray": 14, "pattern3d": 15, "hyperboloid": 16, "ring": 17}
_lib = None


class OCfg(C.Structure):
    _fields_ = [
        ("nphoton", C.c_uint64), ("photon_offset", C.c_uint64), ("seed", C.c_uint64),
        ("srcpos", C.c_float * 3), ("srcdir", C.c_float * 3), ("e0", C.c_int),
        ("tstart", C.c_float), ("tend", C.c_float), ("tstep", C.c_float), ("maxgate", C.c_int),
        ("isreflect", C.c_int), ("isspecular", C.c_int), ("voidtime", C.c_int),
        ("issavedet", C.c_int), ("issaveexit", C.c_int), ("ismomentum", C.c_int),
        ("minenergy", C.c_float), ("roulettesize", C.c_float), ("nout", C.c_float),
        ("outputtype", C.c_int), ("basisorder", C.c_int), ("isnormalized", C.c_int),
        ("maxdetphoton", C.c_uint32), ("nmedia", C.c_int), ("media", C.c_void_p),
        ("detnum", C.c_int), ("detpos", C.c_void_p),
        ("replayseed", C.c_void_p), ("replayweight", C.c_void_p), ("replaytime", C.c_void_p),
        ("accum_f64", C.c_int), ("step_budget", C.c_uint64),
        ("srctype", C.c_int), ("srcparam1", C.c_float * 4), ("srcparam2", C.c_float * 4), ("focus", C.c_float),
        ("srcpattern", C.c_void_p), ("issaveref", C.c_int), ("method", C.c_int), ("gridstep", C.c_float),
        ("srcnum", C.c_int), ("nodemua", C.c_void_p), ("nodemusp", C.c_void_p),
    ]


class OOut(C.Structure):
    _fields_ = [
        ("field_raw", C.c_void_p), ("detp", C.c_void_p), ("seeds", C.c_void_p),
        ("photon_weight", C.c_void_p), ("photon_steps", C.c_void_p), ("photon_det", C.c_void_p),
        ("detected", C.c_uint32), ("reclen", C.c_int), ("energytot", C.c_double),
        ("energyesc", C.c_double), ("raytet", C.c_uint64), ("aborted", C.c_uint64), ("outside", C.c_uint64),
        ("dref", C.c_void_p), ("nf", C.c_int),
        ("traj", C.c_void_p), ("maxtraj", C.c_uint32), ("ntraj", C.c_uint32),
        ("sim_seconds", C.c_double), ("energy_src", C.c_void_p),
    ]


def build(force=False):
    src = os.path.join(HERE, "mmc_oracle.c")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "mmc_oracle.h"))):
        subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-o", LIB + ".tmp",
                        src, "-lm"], check=True)
        os.replace(LIB + ".tmp", LIB)
    return LIB


def load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(LIB)
        lib.oracle_run.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.POINTER(OCfg),
                                   C.POINTER(OOut), C.c_int]
        lib.oracle_run.restype = C.c_int
        lib.oracle_normalize.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.POINTER(OCfg),
                                         C.c_void_p, C.c_double, C.c_double, C.c_void_p]
        lib.oracle_normalize.restype = C.c_double
        lib.oracle_prep_mesh.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.POINTER(C.c_int)]
        lib.oracle_initelem.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        lib.oracle_expf.argtypes = [C.c_float]
        lib.oracle_expf.restype = C.c_float
        lib.oracle_logf.argtypes = [C.c_float]
        lib.oracle_logf.restype = C.c_float
        lib.oracle_sincos2pi.argtypes = [C.c_float, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        lib.oracle_rng_seed.argtypes = [C.c_uint64, C.c_uint64, C.POINTER(C.c_uint64 * 2)]
        lib.oracle_rng_next.argtypes = [C.POINTER(C.c_uint64 * 2)]
        lib.oracle_rng_next.restype = C.c_float
        _lib = lib
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def _arr(node, elem, label):
    node = np.ascontiguousarray(node, np.float32).reshape(-1, 3)
    elem = np.ascontiguousarray(elem, np.int32).reshape(-1, 4)
    label = np.ascontiguousarray(label, np.int32).reshape(-1)
    return node, elem, label


def prep_mesh(node, elem, label):
    lib = load()
    node, elem, label = _arr(node, elem, label)
    nn, ne = node.shape[0], elem.shape[0]
    ee = np.empty((ne, 4), np.int32)
    fnb = np.empty((ne, 4), np.int32)
    nrm = np.empty((ne, 16), np.float32)
    evol = np.empty(ne, np.float32)
    nvol = np.empty(nn, np.float32)
    nf = C.c_int()
    rc = lib.oracle_prep_mesh(nn, _p(node), ne, _p(elem), _p(label), None, _p(ee), _p(fnb), _p(nrm),
                              _p(evol), _p(nvol), C.byref(nf))
    if rc:
        raise ValueError("oracle: bad mesh")
    return dict(elem=ee, facenb=fnb, normals=nrm, evol=evol, nvol=nvol, nf=nf.value)


def grid_dims(node, step):
    """(dim.x, dim.y, dim.z) of the dual-grid output (oracle_grid_dims)."""
    lib = load()
    node = np.ascontiguousarray(node, np.float32).reshape(-1, 3)
    dim = (C.c_int * 3)()
    org = (C.c_float * 3)()
    lib.oracle_grid_dims(node.shape[0], _p(node), C.c_float(float(step)), dim, org)
    return tuple(int(x) for x in dim)


def initelem(node, elem, label, p):
    lib = load()
    node, elem, label = _arr(node, elem, label)
    ee = prep_mesh(node, elem, label)["elem"]
    pp = np.asarray(p, np.float32)
    return int(lib.oracle_initelem(node.shape[0], _p(node), ee.shape[0], _p(ee), _p(pp)))


def _ocfg(cfg, maxgate, e0, keep):
    c = OCfg()
    c.nphoton = int(cfg.nphoton)
    c.photon_offset = int(cfg.photon_offset)
    c.seed = int(cfg.seed) & 0xFFFFFFFFFFFFFFFF
    c.srcpos = (C.c_float * 3)(*[float(x) for x in cfg.srcpos])
    c.srcdir = (C.c_float * 3)(*[float(x) for x in cfg.srcdir])
    c.e0 = int(e0)
    c.tstart = float(cfg.tstart)
    c.tstep = float(cfg.tstep)
    c.maxgate = int(maxgate)
    # the per-launch window end the engine uses: tstart + tstep*maxgate (float)
    c.tend = float(np.float32(cfg.tstart) + np.float32(cfg.tstep) * np.float32(maxgate))
    c.isreflect, c.isspecular, c.voidtime = int(cfg.isreflect), int(cfg.isspecular), int(cfg.voidtime)
    c.issavedet, c.issaveexit, c.ismomentum = int(cfg.issavedet), int(cfg.issaveexit), int(cfg.ismomentum)
    c.minenergy, c.roulettesize, c.nout = float(cfg.minenergy), float(cfg.roulettesize), float(cfg.nout)
    ot = cfg.outputtype
    c.outputtype = OUTPUT_TYPES[ot] if isinstance(ot, str) else int(ot)
    c.basisorder, c.isnormalized = int(cfg.basisorder), int(cfg.isnormalized)
    c.maxdetphoton = int(cfg.maxdetphoton)
    med = np.ascontiguousarray(cfg.media, np.float32).reshape(-1, 4)
    keep.append(med)
    c.nmedia, c.media = med.shape[0], _p(med)
    if cfg.detpos is not None and len(cfg.detpos):
        det = np.ascontiguousarray(cfg.detpos, np.float32).reshape(-1, 4)
        keep.append(det)
        c.detnum, c.detpos = det.shape[0], _p(det)
    if cfg.replayseed is not None:
        rs = np.ascontiguousarray(cfg.replayseed, np.uint64).reshape(-1, 2)
        rw = np.ascontiguousarray(cfg.replayweight, np.float32)
        rt = np.ascontiguousarray(cfg.replaytime, np.float32)
        keep += [rs, rw, rt]
        c.replayseed, c.replayweight, c.replaytime = _p(rs), _p(rw), _p(rt)
    c.accum_f64 = int(cfg.accum_f64)
    c.step_budget = int(cfg.step_budget) if cfg.step_budget else 100000000
    st = getattr(cfg, "srctype", 0)
    c.srctype = SOURCE_TYPES[st] if isinstance(st, str) else int(st)
    c.srcparam1 = (C.c_float * 4)(*[float(x) for x in getattr(cfg, "srcparam1", (0, 0, 0, 0))])
    c.srcparam2 = (C.c_float * 4)(*[float(x) for x in getattr(cfg, "srcparam2", (0, 0, 0, 0))])
    c.focus = float(getattr(cfg, "focus", 0.0))
    c.issaveref = int(getattr(cfg, "issaveref", 0))
    m = getattr(cfg, "method", 0)
    c.method = {"elem": 0, "grid": 1}[m] if isinstance(m, str) else int(m)
    c.gridstep = float(getattr(cfg, "gridstep", 1.0))
    c.srcnum = int(getattr(cfg, "srcnum", 1))
    pat = getattr(cfg, "srcpattern", None)
    if pat is not None:
        pat = np.ascontiguousarray(pat, np.float32).ravel()
        keep.append(pat)
        c.srcpattern = _p(pat)
    for k in ("nodemua", "nodemusp"):
        v = getattr(cfg, k, None)
        if v is not None:
            v = np.ascontiguousarray(v, np.float32).ravel()
            keep.append(v)
            setattr(c, k, _p(v))
    return c


def run(node, elem, label, cfg, nthreads=1, trace=False, normalize=True):
    """Runs the oracle on the mesh arrays with a SimConfig; returns a dict."""
    lib = load()
    node, elem, label = _arr(node, elem, label)
    nn, ne = node.shape[0], elem.shape[0]
    maxgate = cfg.maxgate
    e0 = cfg.e0 if cfg.e0 else initelem(node, elem, label, cfg.srcpos)
    st = getattr(cfg, "srctype", 0)
    st = SOURCE_TYPES[st] if isinstance(st, str) else int(st)
    if e0 <= 0 and st in (0, 1, 2, 7):  # point sources start in the initial element
        raise ValueError("oracle: source outside the mesh")
    e0 = max(int(e0), 0)
    keep = []
    c = _ocfg(cfg, maxgate, e0, keep)
    for k in ("nodemua", "nodemusp"):
        v = getattr(cfg, k, None)
        if v is not None and np.size(v) != nn:
            raise ValueError(f"oracle: {k} needs one value per node ({nn})")
    framelen = ne
    if c.method == 1:
        framelen = int(np.prod(grid_dims(node, cfg.gridstep if cfg.gridstep > 0 else 1.0)))
    K = max(1, c.srcnum) if c.srctype == 5 else 1
    raw = np.zeros((maxgate, framelen) if K == 1 else (maxgate, framelen, K), np.float64)
    esrc = np.zeros((2, K), np.float64) if K > 1 else None
    nmed = c.nmedia
    reclen = 1 + (2 + (1 if cfg.ismomentum else 0)) * (nmed - 1) + (6 if cfg.issaveexit else 0) + 1
    out = OOut()
    detp = np.zeros((int(cfg.maxdetphoton), reclen), np.float32) if cfg.issavedet else None
    seeds = np.zeros((int(cfg.maxdetphoton), 16), np.uint8) if cfg.issavedet and cfg.issaveseed else None
    pw = np.zeros(int(cfg.nphoton), np.float32) if trace else None
    ps = np.zeros(int(cfg.nphoton), np.uint32) if trace else None
    pd = np.zeros(int(cfg.nphoton), np.int32) if trace else None
    out.field_raw, out.detp, out.seeds = _p(raw), _p(detp), _p(seeds)
    out.photon_weight, out.photon_steps, out.photon_det = _p(pw), _p(ps), _p(pd)
    dref = np.zeros(maxgate * 4 * ne, np.float64) if getattr(cfg, "issaveref", 0) else None  # nf <= 4 ne
    out.dref = _p(dref)
    maxtraj = int(getattr(cfg, "maxjumpdebug", 0))
    traj = np.zeros((maxtraj, 6), np.float32) if maxtraj else None
    out.traj, out.maxtraj = _p(traj), maxtraj
    out.energy_src = _p(esrc)
    rc = lib.oracle_run(nn, _p(node), ne, _p(elem), _p(label), C.byref(c), C.byref(out), int(nthreads))
    if rc:
        raise ValueError("oracle run failed")
    res = dict(raw=raw, detected=int(out.detected), energytot=out.energytot, energyesc=out.energyesc,
               raytet=int(out.raytet), aborted=int(out.aborted), outside=int(out.outside), reclen=int(out.reclen), e0=e0,
               photon_weight=pw, photon_steps=ps, photon_det=pd)
    saved = min(int(out.detected), int(cfg.maxdetphoton)) if cfg.issavedet else 0
    res["detp"] = detp[:saved] if detp is not None else None
    res["seeds"] = seeds[:saved] if seeds is not None else None
    res["nf"] = int(out.nf)
    res["dref"] = dref[:maxgate * out.nf].reshape(maxgate, out.nf) if dref is not None else None
    res["ntraj"] = int(out.ntraj)
    res["sim_seconds"] = float(out.sim_seconds)
    res["traj"] = traj[:min(int(out.ntraj), maxtraj)] if traj is not None else None
    res["energy_src"] = esrc
    if not normalize:
        return res
    # each pattern is normalized with its own energies (src/mmc_cu_host.cu:984-995); the
    # normalizer reported is their mean
    tot = esrc[0] if K > 1 else [out.energytot]
    esc = esrc[1] if K > 1 else [out.energyesc]
    fields, norms = [], []
    for p in range(K):
        raw_p = np.ascontiguousarray(raw[..., p] if K > 1 else raw)
        if c.method == 1:  # dual grid: one scale factor (src/mmc_mesh.c:2204-2206)
            norm = 1.0
            if cfg.isnormalized:
                et = float(np.float32(tot[p]))
                if c.outputtype == OUTPUT_TYPES["energy"]:
                    norm = float(np.float32(1.0) / np.float32(et))
                else:
                    norm = 1.0 / (et * cfg.unitinmm ** 3)
                    if c.outputtype == OUTPUT_TYPES["flux"]:
                        norm /= float(np.float32(cfg.tstep))
            fields.append(raw_p * norm)
        else:
            datalen = nn if cfg.basisorder else ne
            field = np.zeros((maxgate, datalen), np.float64)
            norm = lib.oracle_normalize(nn, _p(node), ne, _p(elem), _p(label), C.byref(c), _p(raw_p),
                                        float(tot[p]), float(esc[p]), _p(field))
            fields.append(field)
        norms.append(norm)
    res["field"] = fields[0] if K == 1 else np.stack(fields, axis=-1)
    res["normalizer"] = norms[0] if K == 1 else sum(norms) / K
    return res


def normalize(node, elem, label, cfg, raw, energytot, energyesc):
    lib = load()
    node, elem, label = _arr(node, elem, label)
    nn, ne = node.shape[0], elem.shape[0]
    keep = []
    c = _ocfg(cfg, cfg.maxgate, 1, keep)
    raw = np.ascontiguousarray(raw, np.float64)
    datalen = nn if cfg.basisorder else ne
    field = np.zeros((cfg.maxgate, datalen), np.float64)
    norm = lib.oracle_normalize(nn, _p(node), ne, _p(elem), _p(label), C.byref(c), _p(raw), energytot,
                                energyesc, _p(field))
    return field, norm
