"""Command line front end mirroring the reference's ``mmc`` binary for the
photon path (src/mmc.c:58-112 and the option table of src/mmc_utils.c:103-128):

    python -m mmc_gb300 -f input.json [-n photons] [-E seed|file.mch] [-s session]
        [-C basisorder] [-U normalize] [-O x|f|e|j|l|p] [-d savedet] [-x saveexit]
        [-q saveseed] [-m momentum] [-b reflect] [-e minenergy] [-P replaydet]
        [-H maxdetphoton] [-F bin|dat|mch] [-G gpu] [-D T|M] [--maxjumpdebug n] [-M s|G] [-X 0|1]
        [-S 0|1]
    python -m mmc_gb300 -Q [dmmc-cube60|dmmc-cube60b] [options]   (built-in benchmarks)

Writes <session>.bin (or .dat) with the normalized output and, when detected
photons are saved, <session>.mch -- as the reference does in standalone mode
(src/mmc_cu_host.cu:1397-1440).  `-E file.mch` replays the photons saved in a
previous run (src/mmc_mesh.c:815-898).  `-D M` saves photon trajectories (a
record per launch, scattering event and photon end, at most --maxjumpdebug of
them) into <session>.mch with 6 columns and `detected` 0, written after (and so
in place of) the detected photons, as src/mmc_host.c:434-459 does.
"""
from __future__ import annotations

import argparse
import dataclasses
import os
import sys
import time

import numpy as np


def _intflag(v):
    return int(float(v))


def main(argv=None):
    ap = argparse.ArgumentParser(prog="mmc_gb300", description=__doc__, formatter_class=argparse.RawTextHelpFormatter)
    ap.add_argument("-f", "--input")
    ap.add_argument("-Q", "--bench", nargs="?", const="")   # built-in benchmark; alone: list them
    ap.add_argument("-n", "--photon", type=_intflag)
    ap.add_argument("-E", "--seed")
    ap.add_argument("-s", "--session")
    ap.add_argument("-C", "--basisorder", type=int)
    ap.add_argument("-U", "--normalize", type=int)
    ap.add_argument("-O", "--outputtype")
    ap.add_argument("-d", "--savedet", type=int)
    ap.add_argument("-x", "--saveexit", type=int)
    ap.add_argument("-q", "--saveseed", type=int)
    ap.add_argument("-m", "--mc", type=int)        # 0 MCX-style photon weights; 1 (MCML) is a CPU-engine option
    ap.add_argument("--momentum", type=int)        # save momentum transfer (implies -d 1, src/mmc_utils.c:4185-4190)
    ap.add_argument("-u", "--unitinmm", type=float)
    ap.add_argument("-V", "--specular", type=int)
    ap.add_argument("-k", "--voidtime", type=int)
    # launch and back-end choices of the reference with no counterpart here: accepted, ignored
    ap.add_argument("-A", "--autopilot")
    ap.add_argument("-c", "--compute")
    ap.add_argument("-W", "--workload")
    ap.add_argument("--atomic")
    ap.add_argument("-v", "--version", action="store_true")
    ap.add_argument("-b", "--reflect", type=int)
    ap.add_argument("-e", "--minenergy", type=float)
    ap.add_argument("-P", "--replaydet", type=int, default=0)
    ap.add_argument("-H", "--maxdetphoton", type=_intflag)
    ap.add_argument("-F", "--outputformat")
    ap.add_argument("-G", "--gpu", type=int, default=1)
    ap.add_argument("-D", "--debug", default="")
    ap.add_argument("--maxjumpdebug", type=_intflag, default=10000000)  # src/mmc_utils.c:342
    ap.add_argument("-M", "--method")
    ap.add_argument("-S", "--save2pt", type=int)
    ap.add_argument("-X", "--saveref", type=int)
    ap.add_argument("-r", "--root", default="")
    args = ap.parse_args(argv)
    if args.version:
        from . import __version__
        print(f"mmc_gb300 {__version__}")
        return 0
    if args.mc:
        ap.error("-m 1 (MCML-style albedo weighting) is an option of the reference's CPU engine, not provided here")

    from . import io
    from .core import Mesh, simulate

    if args.bench == "":
        print("Built-in benchmarks:\n" + "".join(f"\t{n}\n" for n in io.BENCHMARKS), end="")
        return 0
    if args.bench is not None:
        try:
            source = io.builtin_benchmark(args.bench)
        except ValueError as e:
            ap.error(str(e))
    elif args.input:
        source = args.input
    else:
        ap.error("an input file (-f) or a built-in benchmark (-Q) is required")
    mesh_d, cfg, meta = io.load_input(source)
    method = (args.method or meta.get("raytracer") or "s").lower()
    if method not in ("s", "elem", "b", "g", "grid"):
        ap.error("only the branchless Badouel tracer is implemented: -M s (element output) or -M G (dual grid)")
    upd = {}
    if args.photon is not None:
        upd["nphoton"] = args.photon
    if args.basisorder is not None:
        upd["basisorder"] = args.basisorder
    if args.normalize is not None:
        upd["isnormalized"] = args.normalize
    if args.outputtype:
        upd["outputtype"] = io.output_type(args.outputtype)
    for k, a in (("issavedet", args.savedet), ("issaveexit", args.saveexit), ("issaveseed", args.saveseed),
                 ("ismomentum", args.momentum), ("isreflect", args.reflect), ("minenergy", args.minenergy),
                 ("maxdetphoton", args.maxdetphoton), ("issaveref", args.saveref), ("unitinmm", args.unitinmm),
                 ("isspecular", args.specular), ("voidtime", args.voidtime)):
        if a is not None:
            upd[k] = a
    if args.momentum:
        upd["issavedet"] = 1
    replay_file = None
    if args.seed is not None:
        if args.seed.endswith(".mch"):
            replay_file = args.seed
        else:
            upd["seed"] = int(args.seed)
    if method in ("g", "grid"):
        upd["method"] = "grid"
        upd["basisorder"] = 0  # the dual grid has no nodal form (src/mmc_utils.c:2300-2302)
    debug = (args.debug + meta.get("debugflag", "")).upper()
    if "M" in debug:
        upd["maxjumpdebug"] = args.maxjumpdebug
    cfg = dataclasses.replace(cfg, **upd)
    session = args.session or meta["session"]
    fmt = (args.outputformat or meta["outputformat"]).lower()
    # the reference's formats (src/mmc_utils.c:171): text (its default) or raw float64; the NIfTI,
    # JNIfTI, mc2 and tx3 containers are not written here
    if fmt not in ("ascii", "dat", "bin"):
        ap.error(f"output format '{fmt}' is not supported (ascii, bin)")
    outdir = args.root or os.getcwd()
    device = max(0, args.gpu - 1)
    mesh = Mesh(mesh_d["node"], mesh_d["elem"], mesh_d["label"], mesh_d.get("facenb"), device=device)

    t0 = time.perf_counter()
    if replay_file:
        from . import replay as rp
        detp, hdr, seeds = io.read_mch(replay_file)
        if seeds is None:
            raise SystemExit(f"{replay_file} holds no seeds (rerun the baseline with -q 1)")
        res, idx = rp.replay(mesh, cfg, detp, seeds, cfg.outputtype if cfg.outputtype in ("wl", "wp", "wn", "jacobian")
                             else "wl", args.replaydet, normalize=bool(cfg.isnormalized))
        nphoton = len(idx)
    else:
        res = simulate(mesh, cfg)
        nphoton = cfg.nphoton
    dt = time.perf_counter() - t0
    print(f"simulated {nphoton} photons in {dt * 1e3:.1f} ms ({nphoton / max(dt * 1e3, 1e-9):.2f} photon/ms), "
          f"{res.raytet} ray-tetrahedron tests, kernel {res.kernel_ms:.1f} ms")
    if res.energytot > 0 and not replay_file:
        print(f"total simulated energy: {res.energytot:.0f}\tabsorbed: {100 * res.absorbed_fraction:.5f}%\t"
              f"normalizor={res.normalizer:g}")
    if "T" in debug:
        print(f"detected {res.detected} photons")
    base = os.path.join(outdir, session)
    save2pt = args.save2pt if args.save2pt is not None else meta.get("saveweight", 1)
    if res.field is not None and save2pt:
        if fmt in ("ascii", "dat"):
            io.write_dat(base + ".dat", res.field)
        else:
            io.write_bin(base + ".bin", res.field)
    if res.dref is not None:  # exiting weight per exterior face: <session>_dref.dat (src/mmc_mesh.c:1726-1800)
        io.write_dat(base + "_dref.dat", res.dref)
    if res.detp is not None and cfg.issavedet and cfg.issaveexit == 2:  # <session>.img (src/mmc_host.c:424-430)
        io.detector_image(res.detp, cfg, meta.get("detparam1", (0, 0, 0, 0)), meta.get("detparam2", (0, 0, 0, 0))).tofile(base + ".img")
    if res.detp is not None and cfg.issavedet:
        io.write_mch(base + ".mch", res.detp, res.seeds if cfg.issaveseed else None,
                     maxmedia=np.asarray(cfg.media).shape[0] - 1,
                     detnum=0 if cfg.detpos is None else len(cfg.detpos), totalphoton=nphoton,
                     detected=res.detected, unitinmm=cfg.unitinmm, normalizer=res.normalizer, srcnum=cfg.srcnum)
    if res.traj is not None:
        if res.ntraj > len(res.traj):
            print(f"WARNING: the saved trajectory positions ({res.ntraj}) are more than what you have specified "
                  f"({len(res.traj)}), please use the --maxjumpdebug option to specify a greater number")
        io.write_mch(base + ".mch", res.traj, None, maxmedia=np.asarray(cfg.media).shape[0] - 1,
                     detnum=0 if cfg.detpos is None else len(cfg.detpos), totalphoton=nphoton, detected=0,
                     unitinmm=cfg.unitinmm, normalizer=res.normalizer)
    mesh.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
