"""pmmc-compatible Python interface: ``run(cfg: dict) -> dict``.

Mirrors the reference binding ``pmmc.run`` (src/pmmc.cpp:903-1351, key
parsing :117-890) for the photon path: the same input keys and the same
output keys and array layouts (``flux`` as [datalen, maxgate], ``detp`` as
[columns, ndetected], ``seeds`` as [16, ndetected]; these are transposed views
of the row-major arrays the engine returns).  Errors raise ``ValueError`` for
bad inputs and ``RuntimeError`` for engine failures, as pmmc does.
"""
from __future__ import annotations

import dataclasses
import time

import numpy as np

from . import _native
from .core import SOURCE_TYPES, Mesh, SimConfig, simulate

_SCALARS_INT = ["nphoton", "isreflect", "isspecular", "ismomentum", "issaveexit", "issavedet", "issaveseed",
                "basisorder", "isnormalized", "maxdetphoton", "voidtime", "e0", "issaveref"]
_SCALARS_FLOAT = ["tstart", "tstep", "tend", "roulettesize", "minenergy", "unitinmm", "nout"]
_METHODS = {"plucker": None, "havel": None, "badouel": None, "elem": "elem", "grid": "grid"}
_OUTPUTS = {"flux", "fluence", "energy", "jacobian", "wl", "wp", "wn"}
# keys of the reference's binding for options this library does not provide: refused when set,
# rather than ignored
_UNSUPPORTED = {"mcmethod": "MCML-style albedo weighting (an option of the reference's CPU engine)",
                "isextdet": "wide-field detector elements", "adjointmode": "adjoint outputs"}


def version() -> str:
    from . import __version__
    return f"mmc_gb300 {__version__}"


def gpuinfo():
    import torch
    return [dict(name=torch.cuda.get_device_name(i), id=i + 1) for i in range(torch.cuda.device_count())]


def _parse(cfg: dict):
    for req in ("node", "elem", "prop", "srcpos"):
        if req not in cfg:
            raise ValueError(f"cfg.{req} is required")
    for k, what in _UNSUPPORTED.items():
        if k in cfg and np.any(np.asarray(cfg[k]) != 0):
            raise ValueError(f"cfg.{k} ({what}) is not supported")
    node = np.asarray(cfg["node"], np.float32)
    elem = np.asarray(cfg["elem"])
    if elem.ndim != 2 or elem.shape[1] not in (4, 5):
        raise ValueError("the 'elem' field must have 4 columns (labels in 'elemprop') or 5")
    if elem.shape[1] == 5 and "elemprop" not in cfg:
        label = elem[:, 4].astype(np.int32)
    else:
        label = np.asarray(cfg.get("elemprop", np.ones(len(elem))), np.int32).reshape(-1)
    elem = elem[:, :4].astype(np.int32)
    prop = np.asarray(cfg["prop"], np.float32).reshape(-1, 4)
    method = str(cfg.get("method", "elem")).lower()
    if method not in _METHODS:
        raise ValueError(f"unknown method '{method}'")
    if _METHODS[method] is None:
        raise ValueError(f"method '{method}' is not implemented (use 'elem': branchless Badouel, element deposit)")
    srctype = str(cfg.get("srctype", "pencil")).lower()
    if srctype not in SOURCE_TYPES:
        raise ValueError(f"unknown srctype '{srctype}'")
    kw = dict(media=prop, srcpos=tuple(np.asarray(cfg["srcpos"], np.float64).ravel()[:3]), srctype=srctype,
              method=_METHODS[method])
    if "steps" in cfg:  # dual-grid voxel edge (the reference takes steps[0] for all axes)
        kw["gridstep"] = float(np.asarray(cfg["steps"], np.float64).ravel()[0])
    if "srcdir" in cfg:
        d4 = np.asarray(cfg["srcdir"], np.float64).ravel()
        d = d4[:3]
        kw["srcdir"] = tuple(d / np.linalg.norm(d))
        if d4.size > 3:
            kw["focus"] = float(d4[3])
    for k in ("srcparam1", "srcparam2"):
        if k in cfg:
            v = list(np.asarray(cfg[k], np.float64).ravel()) + [0.0] * 4
            kw[k] = tuple(float(x) for x in v[:4])
    if "srcpattern" in cfg:
        # pmmc passes patterns as [Nx, Ny(, Nz)] arrays in Fortran order: x runs fastest.  A pattern
        # source given [srcnum, Nx, Ny] (srcnum > 1, Ny > 1) holds patterns that share each photon,
        # as the reference reads a 3-D JSON pattern (src/mmc_utils.c:2100-2102)
        pat = np.asarray(cfg["srcpattern"], np.float32)
        if (pat.ndim == 3 and pat.shape[0] > 1 and pat.shape[2] > 1
                and srctype == "pattern"):
            kw["srcnum"] = int(pat.shape[0])
        kw["srcpattern"] = pat.ravel(order="F")
    for k in _SCALARS_INT:
        if k in cfg:
            kw[k] = int(cfg[k])
    for k in _SCALARS_FLOAT:
        if k in cfg:
            kw[k] = float(cfg[k])
    if float(cfg.get("omega", 0.0) or 0.0) > 0.0:
        raise ValueError("omega > 0 asks for RF (frequency-domain) output, which is not supported")
    if "outputtype" in cfg:
        ot = str(cfg["outputtype"]).lower()
        if ot not in _OUTPUTS:
            raise ValueError("the specified output type is not supported")
        kw["outputtype"] = ot
    if "detpos" in cfg:
        kw["detpos"] = np.asarray(cfg["detpos"], np.float32).reshape(-1, 4)
    # per-node mua/musp (src/pmmc.cpp:630-672): giving the array switches the mode on; the flags
    # alone would have the reference's kernel read an array it never uploaded, so they are refused
    for arr, flag in (("nodemua", "isnodalmua"), ("nodemusp", "isnodalmusp")):
        if arr in cfg:
            kw[arr] = np.asarray(cfg[arr], np.float32).ravel(order="F")
        elif int(cfg.get(flag, 0) or 0):
            raise ValueError(f"cfg.{flag} needs cfg.{arr}, one value per node")
    for k in ("detparam1", "detparam2"):  # the area detector of the exit image (issaveexit = 2)
        if k in cfg:
            v = list(np.asarray(cfg[k], np.float64).ravel()) + [0.0] * 4
            kw[k] = tuple(float(x) for x in v[:4])
    if "debuglevel" in cfg:  # letters R, M, P (src/pmmc.cpp:692-710); M saves photon trajectories
        dl = str(cfg["debuglevel"]).upper()
        if not dl:
            raise ValueError("the 'debuglevel' field must be a non-empty string")
        if not any(c in "RMP" for c in dl):
            raise ValueError("the specified debuglevel is not supported")
        if "M" in dl:
            kw["maxjumpdebug"] = int(cfg.get("maxjumpdebug", 10000000))
    seeds = None
    if "seed" in cfg:
        s = cfg["seed"]
        if np.isscalar(s):
            kw["seed"] = int(s)
        else:
            seeds = np.asarray(s, np.uint8)
            if seeds.shape[0] != 16:
                raise ValueError("the row number of cfg.seed does not match RNG seed byte-length")
    if "tend" in kw and "tstep" not in kw:
        kw["tstep"] = kw["tend"] - kw.get("tstart", 0.0)
    if "issave2pt" in cfg and not int(cfg["issave2pt"]):  # no fluence output (src/pmmc.cpp:1154)
        kw["save_field"] = False
    return node, elem, label, cfg.get("facenb"), SimConfig(**kw), seeds


def run(cfg: dict) -> dict:
    node, elem, label, facenb, sc, seeds = _parse(cfg)
    device = max(0, int(cfg.get("gpuid", 1)) - 1) if np.isscalar(cfg.get("gpuid", 1)) else 0
    t0 = time.perf_counter()
    try:
        mesh = Mesh(node, elem, label, facenb, device=device)
        if seeds is not None:
            from . import replay as rp
            detp = np.asarray(cfg.get("detphotons"), np.float32)
            if detp is None or detp.ndim != 2:
                raise ValueError("you give cfg.seed for replay, but did not specify cfg.detphotons")
            res, idx = rp.replay(mesh, sc, detp.T.copy(), seeds.T.copy(),
                                 sc.outputtype if sc.outputtype in ("wl", "wp", "wn", "jacobian") else "wl",
                                 int(cfg.get("replaydet", 0)), normalize=bool(sc.isnormalized))
            nph = len(idx)
        else:
            res = simulate(mesh, sc)
            nph = sc.nphoton
        mesh_dims = mesh.grid_dims(sc.gridstep) if sc.method == "grid" else None
        mesh.close()
    except _native.MmcgbError as e:
        if e.code == 1:
            raise ValueError(str(e)) from e
        raise RuntimeError(str(e)) from e
    # [datalen, maxgate]; with patterns sharing photons [srcnum, datalen, maxgate] (src/pmmc.cpp:1196-1207)
    field = None if res.field is None else res.field.T
    if field is not None and sc.method == "grid":  # [dim.x, dim.y, dim.z, maxgate] (+ a leading srcnum), x fastest
        dx, dy, dz = mesh_dims
        if res.field.ndim == 3:
            field = res.field.reshape(-1, dz, dy, dx, res.field.shape[-1]).transpose(4, 3, 2, 1, 0)
        else:
            field = res.field.reshape(-1, dz, dy, dx).transpose(3, 2, 1, 0)
    out = {"stat": dict(runtime=(time.perf_counter() - t0) * 1e3, nphoton=nph,
                                             energytot=res.energytot, energyabs=res.energytot - res.energyesc,
                                             normalizer=res.normalizer, raytet=res.raytet,
                                             kernel_ms=res.kernel_ms)}
    if field is not None:
        out["flux"] = field
    if sc.issaveref and res.dref is not None:
        out["dref"] = res.dref.T  # [nf, maxgate], as pmmc (src/pmmc.cpp:1226-1234)
    if res.traj is not None:
        out["traj"] = res.traj.T  # [6, records]: id, x, y, z, weight, element (src/pmmc.cpp:1092-1108)
    if sc.issavedet and res.detp is not None and sc.issaveexit == 2:
        # the exit image [nx, ny, maxgate] instead of the records (src/pmmc.cpp:1135-1146)
        from .io import detector_image
        out["detp"] = detector_image(res.detp, sc, sc.detparam1, sc.detparam2).transpose(2, 1, 0)
    elif sc.issavedet and res.detp is not None and len(res.detp):
        out["detp"] = res.detp.T
        if sc.issaveseed and res.seeds is not None:
            out["seeds"] = res.seeds.T
    return out
