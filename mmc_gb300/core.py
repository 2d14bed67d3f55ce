"""Python front of the photon engine: resident meshes, simulation settings and
results as numpy arrays, over the C ABI of libmmcgb.so.

    mesh = Mesh(node, elem, label)            # uploads + ray-tracer precompute
    res = simulate(mesh, SimConfig(nphoton=1e6, media=..., srcpos=..., ...))
    res.field   # (maxgate, datalen) float64, normalized like the reference

Field layout follows the reference's exported weight array
(src/mmc_cu_host.cu:916-976): gate-major, element (basisorder 0) or node
(basisorder 1) fastest.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
from typing import Optional, Sequence

import numpy as np

from . import _native as N

OUTPUT_TYPES = {"flux": 0, "fluence": 1, "energy": 2, "jacobian": 3, "wl": 4, "wp": 5, "wn": 16}
# the reference's source type names and numbers (src/mmc_utils.h:101-105)
SOURCE_TYPES = {"pencil": 0, "isotropic": 1, "cone": 2, "gaussian": 3, "planar": 4, "pattern": 5, "fourier": 6,
                "arcsine": 7, "disk": 8, "fourierx": 9, "fourierx2d": 10, "zgaussian": 11, "line": 12, "slit": 13,
                "pencilarray": 14, "pattern3d": 15, "hyperboloid": 16, "ring": 17}


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data


def _desc(node, elem, label, facenb=None):
    node = np.ascontiguousarray(node, dtype=np.float32).reshape(-1, 3)
    elem = np.ascontiguousarray(elem, dtype=np.int32).reshape(-1, 4)
    label = np.ascontiguousarray(label, dtype=np.int32).reshape(-1)
    fnb = None if facenb is None else np.ascontiguousarray(facenb, dtype=np.int32).reshape(-1, 4)
    d = N.MeshDesc(node.shape[0], elem.shape[0], _ptr(node), _ptr(elem), _ptr(label), _ptr(fnb))
    return d, (node, elem, label, fnb)


def prepare_host(node, elem, label, facenb=None):
    """Host mesh preparation (mmcgb_prepare_host): dict of elem, facenb,
    normals, evol, nvol, nf.  Needs no GPU."""
    d, keep = _desc(node, elem, label, facenb)
    ne, nn = d.ne, d.nn
    out = dict(elem=np.empty((ne, 4), np.int32), facenb=np.empty((ne, 4), np.int32),
               normals=np.empty((ne, 16), np.float32), evol=np.empty(ne, np.float32), nvol=np.empty(nn, np.float32))
    nf = C.c_int32()
    N.check(N.load().mmcgb_prepare_host(C.byref(d), _ptr(out["elem"]), _ptr(out["facenb"]), _ptr(out["normals"]),
                                        _ptr(out["evol"]), _ptr(out["nvol"]), C.byref(nf)))
    out["nf"] = nf.value
    return out


def normalize_host(node, elem, label, cfg: "SimConfig", raw, energytot: float, energyesc: float):
    """Output stage on the host (mmcgb_normalize_host): returns (field, normalizer)."""
    d, keep = _desc(node, elem, label)
    c, ckeep = cfg.to_c(d.nn)
    raw = np.ascontiguousarray(raw, np.float64)
    datalen = d.nn if cfg.basisorder else d.ne
    field = np.zeros((cfg.maxgate, datalen), np.float64)
    norm = C.c_double()
    N.check(N.load().mmcgb_normalize_host(C.byref(d), C.byref(c), _ptr(raw), float(energytot), float(energyesc),
                                          _ptr(field), C.byref(norm)))
    return field, norm.value


class Mesh:
    """A tetrahedral mesh resident on one GPU (mmcgb_mesh_create)."""

    def __init__(self, node, elem, label, facenb=None, device: int = 0):
        lib = N.load()
        self._node = np.ascontiguousarray(node, dtype=np.float32).reshape(-1, 3)
        self._elem = np.ascontiguousarray(elem, dtype=np.int32).reshape(-1, 4)
        self._label = np.ascontiguousarray(label, dtype=np.int32).reshape(-1)
        if self._label.shape[0] != self._elem.shape[0]:
            raise ValueError("label must have one entry per element")
        fnb = None if facenb is None else np.ascontiguousarray(facenb, dtype=np.int32).reshape(-1, 4)
        desc = N.MeshDesc(self._node.shape[0], self._elem.shape[0], _ptr(self._node), _ptr(self._elem),
                          _ptr(self._label), _ptr(fnb))
        h = C.c_void_p()
        N.check(lib.mmcgb_mesh_create(C.byref(desc), int(device), C.byref(h)))
        self._h = h
        self.device = int(device)
        nn, ne, nf = C.c_int32(), C.c_int32(), C.c_int32()
        N.check(lib.mmcgb_mesh_info(h, C.byref(nn), C.byref(ne), C.byref(nf)))
        self.nn, self.ne, self.nf = nn.value, ne.value, nf.value

    @property
    def handle(self):
        if self._h is None:
            raise ValueError("mesh was closed")
        return self._h

    @property
    def node(self):
        return self._node

    @property
    def elem(self):
        """Element node ids as given (before the orientation fix)."""
        return self._elem

    @property
    def label(self):
        return self._label

    def export(self):
        """(elem after orientation fix, facenb, evol, nvol) host copies."""
        lib = N.load()
        elem = np.empty((self.ne, 4), np.int32)
        fnb = np.empty((self.ne, 4), np.int32)
        evol = np.empty(self.ne, np.float32)
        nvol = np.empty(self.nn, np.float32)
        N.check(lib.mmcgb_mesh_export(self.handle, _ptr(elem), _ptr(fnb), _ptr(evol), _ptr(nvol)))
        return elem, fnb, evol, nvol

    def locate(self, p) -> int:
        arr = (C.c_float * 3)(*[float(x) for x in p])
        return int(N.load().mmcgb_mesh_locate(self.handle, C.byref(arr)))

    def grid_dims(self, step: float = 1.0):
        """(dim.x, dim.y, dim.z) of the dual-grid output for voxel edge `step`
        (mmcgb_grid_info); the grid field is (maxgate, dim.z, dim.y, dim.x)."""
        dim = (C.c_int32 * 3)()
        org = (C.c_float * 3)()
        N.check(N.load().mmcgb_grid_info(self._h, float(step), dim, org))
        return tuple(int(x) for x in dim)

    def close(self):
        if getattr(self, "_h", None) is not None:
            N.load().mmcgb_mesh_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclasses.dataclass
class SimConfig:
    """Settings of one simulation (defaults: src/mmc_utils.c:207-363)."""
    media: np.ndarray                         # (nmedia, 4) mua mus g n, row 0 = background
    nphoton: int = 1000000
    seed: int = 0x623F9A9E
    srcpos: Sequence[float] = (0.0, 0.0, 0.0)
    srcdir: Sequence[float] = (0.0, 0.0, 1.0)
    e0: int = 0
    tstart: float = 0.0
    tend: float = 5e-9
    tstep: float = 5e-9
    isreflect: int = 1
    isspecular: int = 0
    voidtime: int = 1
    issavedet: int = 0
    issaveseed: int = 0
    issaveexit: int = 0
    ismomentum: int = 0
    minenergy: float = 1e-6
    roulettesize: float = 10.0
    nout: float = 1.0
    unitinmm: float = 1.0
    outputtype: str = "flux"
    basisorder: int = 1
    isnormalized: int = 1
    maxdetphoton: int = 1000000
    detpos: Optional[np.ndarray] = None       # (ndet, 4) x y z r
    replayseed: Optional[np.ndarray] = None   # (N, 2) uint64 initial RNG states
    replayweight: Optional[np.ndarray] = None
    replaytime: Optional[np.ndarray] = None
    accum_f64: int = 1
    photon_offset: int = 0
    step_budget: int = 0
    threads: int = 0
    blocks: int = 0
    fast_math: int = 1
    phased: int = 0
    srctype: object = "pencil"                  # name or the reference's number (SOURCE_TYPES)
    srcparam1: Sequence[float] = (0.0, 0.0, 0.0, 0.0)
    srcparam2: Sequence[float] = (0.0, 0.0, 0.0, 0.0)
    focus: float = 0.0                          # the reference's srcdir.w
    srcpattern: Optional[np.ndarray] = None     # pattern / pattern3d weights
    issaveref: int = 0                          # exiting weight per exterior face (result.dref)
    maxjumpdebug: int = 0                       # > 0: save up to this many trajectory records
    method: object = "elem"                     # "elem" (element output) or "grid" (dual-grid, DMMC)
    gridstep: float = 1.0                       # voxel edge of the grid output (mm)
    phase_chunk: int = 0                        # max photons per gate-phased launch (0: what memory holds)
    accumulate: int = 0                         # 1: add into the caller's field/dref (mmc_run_cu's +=)
    detparam1: Sequence[float] = (0.0, 0.0, 0.0, 0.0)  # area detector of the exit image (issaveexit = 2,
    detparam2: Sequence[float] = (0.0, 0.0, 0.0, 0.0)  # io.detector_image): edge vectors, pixels in w
    srcnum: int = 1                             # patterns sharing each photon (pattern source; the field
                                                # gains a last axis of srcnum, srcpattern is pixel-major)
    nodemua: Optional[np.ndarray] = None        # per-node mua (nn): element mua = mean of its nodes'
    nodemusp: Optional[np.ndarray] = None       # per-node mus (nn), used only with nodemua
    save_field: bool = True

    @property
    def maxgate(self) -> int:
        return int((np.float32(self.tend) - np.float32(self.tstart)) / np.float32(self.tstep) + np.float32(0.5))

    def to_c(self, nn: Optional[int] = None):
        """The C configuration and the arrays it points into.  `nn`: the mesh's
        node count, against which per-node arrays are checked."""
        keep = {}
        c = N.Config()
        c.nphoton = int(self.nphoton)
        c.photon_offset = int(self.photon_offset)
        c.seed = int(self.seed) & 0xFFFFFFFFFFFFFFFF
        c.srcpos = (C.c_float * 3)(*[float(x) for x in self.srcpos])
        c.srcdir = (C.c_float * 3)(*[float(x) for x in self.srcdir])
        st = self.srctype
        c.srctype = SOURCE_TYPES[st] if isinstance(st, str) else int(st)
        c.srcparam1 = (C.c_float * 4)(*[float(x) for x in self.srcparam1])
        c.srcparam2 = (C.c_float * 4)(*[float(x) for x in self.srcparam2])
        c.focus = float(self.focus)
        if self.srcpattern is not None:
            pat = np.ascontiguousarray(self.srcpattern, dtype=np.float32).reshape(-1)
            keep["pattern"] = pat
            c.srcpattern = _ptr(pat)
        c.issaveref = int(self.issaveref)
        c.maxjumpdebug = int(self.maxjumpdebug)
        c.phase_chunk = int(self.phase_chunk)
        c.accumulate = int(self.accumulate)
        c.srcnum = int(self.srcnum)
        for k in ("nodemua", "nodemusp"):
            v = getattr(self, k)
            if v is not None:
                v = np.ascontiguousarray(v, dtype=np.float32).reshape(-1)
                if nn is not None and v.shape[0] != nn:
                    raise ValueError(f"{k} needs one value per node ({nn}), got {v.shape[0]}")
                keep[k] = v
                setattr(c, k, _ptr(v))
        m = self.method
        c.method = {"elem": 0, "grid": 1}[m] if isinstance(m, str) else int(m)
        c.gridstep = float(self.gridstep)
        c.e0 = int(self.e0)
        c.tstart, c.tend, c.tstep = float(self.tstart), float(self.tend), float(self.tstep)
        c.isreflect, c.isspecular, c.voidtime = int(self.isreflect), int(self.isspecular), int(self.voidtime)
        c.issavedet, c.issaveseed = int(self.issavedet), int(self.issaveseed)
        c.issaveexit, c.ismomentum = int(self.issaveexit), int(self.ismomentum)
        c.minenergy, c.roulettesize = float(self.minenergy), float(self.roulettesize)
        c.nout, c.unitinmm = float(self.nout), float(self.unitinmm)
        ot = self.outputtype
        c.outputtype = OUTPUT_TYPES[ot] if isinstance(ot, str) else int(ot)
        c.basisorder, c.isnormalized = int(self.basisorder), int(self.isnormalized)
        c.maxdetphoton = int(self.maxdetphoton)
        med = np.ascontiguousarray(self.media, dtype=np.float32).reshape(-1, 4)
        keep["media"] = med
        c.nmedia, c.media = med.shape[0], _ptr(med)
        if self.detpos is not None and len(self.detpos):
            det = np.ascontiguousarray(self.detpos, dtype=np.float32).reshape(-1, 4)
            keep["det"] = det
            c.detnum, c.detpos = det.shape[0], _ptr(det)
        if self.replayseed is not None:
            rs = np.ascontiguousarray(self.replayseed, dtype=np.uint64).reshape(-1, 2)
            rw = np.ascontiguousarray(self.replayweight, dtype=np.float32).reshape(-1)
            rt = np.ascontiguousarray(self.replaytime, dtype=np.float32).reshape(-1)
            if not (rs.shape[0] == rw.shape[0] == rt.shape[0] == c.nphoton):
                raise ValueError("replay arrays must have nphoton entries")
            keep.update(rs=rs, rw=rw, rt=rt)
            c.replayseed, c.replayweight, c.replaytime = _ptr(rs), _ptr(rw), _ptr(rt)
        c.accum_f64 = int(self.accum_f64)
        c.step_budget = int(self.step_budget)
        c.threads, c.blocks = int(self.threads), int(self.blocks)
        c.fast_math = int(self.fast_math)
        c.phased = int(self.phased)
        return c, keep


@dataclasses.dataclass
class SimResult:
    field: Optional[np.ndarray]      # (maxgate, datalen) float64
    detp: Optional[np.ndarray]       # (saved, reclen) float32
    seeds: Optional[np.ndarray]      # (saved, 16) uint8
    detected: int
    energytot: float
    energyesc: float
    normalizer: float
    raytet: int
    aborted: int
    kernel_ms: float
    maxgate: int
    reclen: int
    photon_weight: Optional[np.ndarray] = None
    photon_steps: Optional[np.ndarray] = None
    photon_det: Optional[np.ndarray] = None
    dref: Optional[np.ndarray] = None   # (maxgate, nf) exiting weight per exterior face (issaveref)
    traj: Optional[np.ndarray] = None   # (records, 6) trajectory: id bits, x, y, z, weight, eid bits
    ntraj: int = 0                      # trajectory records produced (more than kept when truncated)
    energy_src: Optional[np.ndarray] = None  # srcnum > 1: (2, srcnum) launched / escaped weight per pattern

    @property
    def absorbed_fraction(self) -> float:
        return (self.energytot - self.energyesc) / self.energytot if self.energytot else 0.0


def _alloc_result(mesh: Mesh, cfg: SimConfig, trace: bool, out: Optional[np.ndarray] = None):
    G = cfg.maxgate
    if cfg.method in ("grid", 1):
        datalen = int(np.prod(mesh.grid_dims(cfg.gridstep)))
    else:
        datalen = mesh.nn if cfg.basisorder else mesh.ne
    nmed = np.asarray(cfg.media).reshape(-1, 4).shape[0]
    reclen = 1 + (2 + (1 if cfg.ismomentum else 0)) * (nmed - 1) + (6 if cfg.issaveexit else 0) + 1
    K = max(1, int(cfg.srcnum))
    shape = (G, datalen) if K == 1 else (G, datalen, K)
    arrs = {}
    if out is not None:
        if out.dtype != np.float64 or out.shape != shape or not out.flags.c_contiguous:
            raise ValueError(f"out must be a C-contiguous float64 array of shape {shape}")
        arrs["field"] = out
    else:
        arrs["field"] = np.empty(shape, np.float64) if cfg.save_field else None
    arrs["energy_src"] = np.zeros((2, K), np.float64) if K > 1 else None
    if cfg.issavedet:
        arrs["detp"] = np.empty((int(cfg.maxdetphoton), reclen), np.float32)
        arrs["seeds"] = np.empty((int(cfg.maxdetphoton), 16), np.uint8) if cfg.issaveseed else None
    else:
        arrs["detp"] = arrs["seeds"] = None
    if trace:
        n = int(cfg.nphoton)
        arrs["photon_weight"] = np.zeros(n, np.float32)
        arrs["photon_steps"] = np.zeros(n, np.uint32)
        arrs["photon_det"] = np.zeros(n, np.int32)
    else:
        arrs["photon_weight"] = arrs["photon_steps"] = arrs["photon_det"] = None
    arrs["dref"] = np.zeros((G, mesh.nf), np.float64) if cfg.issaveref else None
    arrs["traj"] = np.zeros((int(cfg.maxjumpdebug), 6), np.float32) if cfg.maxjumpdebug else None
    r = N.Result()
    for k in ("field", "detp", "seeds", "photon_weight", "photon_steps", "photon_det", "dref", "traj", "energy_src"):
        setattr(r, k, _ptr(arrs[k]))
    return r, arrs


def _make_result(r: N.Result, arrs) -> SimResult:
    saved = int(r.saved)

    def rows(a):  # the saved rows; a copy only when it frees most of the buffer
        if a is None:
            return None
        return a[:saved].copy() if 4 * saved < len(a) else a[:saved]
    detp, seeds = rows(arrs["detp"]), rows(arrs["seeds"])
    return SimResult(field=arrs["field"], detp=detp, seeds=seeds, detected=int(r.detected),
                     energytot=r.energytot, energyesc=r.energyesc, normalizer=r.normalizer,
                     raytet=int(r.raytet), aborted=int(r.aborted), kernel_ms=float(r.kernel_ms),
                     maxgate=int(r.maxgate), reclen=int(r.reclen), photon_weight=arrs["photon_weight"],
                     photon_steps=arrs["photon_steps"], photon_det=arrs["photon_det"], dref=arrs["dref"],
                     traj=None if arrs["traj"] is None else arrs["traj"][:min(int(r.ntraj), len(arrs["traj"]))].copy(),
                     ntraj=int(r.ntraj), energy_src=arrs.get("energy_src"))


def simulate(mesh: Mesh, cfg: SimConfig, trace: bool = False, out: Optional[np.ndarray] = None) -> SimResult:
    """Runs one simulation on a resident mesh (mmcgb_simulate).  `out`: an
    optional preallocated (maxgate, datalen) float64 array for the field (for
    example pinned host memory reused across calls).  `trace`: also return
    each photon's final weight, ray-tet test count and detector; such runs
    take the general kernels (the same results, a few percent slower)."""
    lib = N.load()
    c, keep = cfg.to_c(mesh.nn)
    r, arrs = _alloc_result(mesh, cfg, trace, out)
    N.check(lib.mmcgb_simulate(mesh.handle, C.byref(c), C.byref(r)))
    del keep
    return _make_result(r, arrs)


class _HostMesh:
    """Sizes of a host mesh, for laying out the outputs of a one-shot run."""

    def __init__(self, node, elem, nf=0):
        self.nn, self.ne, self.nf = int(len(node)), int(len(elem)), int(nf)
        self._node = node

    def grid_dims(self, step):
        lo = self._node.min(0).astype(np.float32) - np.float32(1e-6)
        hi = self._node.max(0).astype(np.float32) + np.float32(1e-6)
        return tuple(int((hi[k] - lo[k]) / np.float32(step)) + 1 for k in range(3))


def run(node, elem, label, cfg: SimConfig, device: int = 0, out: Optional[np.ndarray] = None,
        dref: Optional[np.ndarray] = None) -> SimResult:
    """One-shot simulation through mmcgb_run, the counterpart of the reference's
    mmc_run_cu (src/mmc_cu_host.h:56): the mesh is prepared, uploaded, simulated
    and released in one call, with host arrays in and out.  `out` (maxgate x
    datalen float64) and `dref` (maxgate x nf) are the caller's arrays; with
    cfg.accumulate the run adds into them as mmc_run_cu adds into
    cfg->exportfield and mesh->dref."""
    lib = N.load()
    node = np.ascontiguousarray(node, np.float32)
    elem = np.ascontiguousarray(elem, np.int32)
    label = np.ascontiguousarray(label, np.int32)
    d, dkeep = _desc(node, elem, label)
    nf = dref.shape[1] if dref is not None else 0
    if cfg.issaveref and dref is None:
        nfo = C.c_int32()
        N.check(lib.mmcgb_prepare_host(C.byref(d), None, None, None, None, None, C.byref(nfo)))
        nf = nfo.value
    c, keep = cfg.to_c(d.nn)
    r, arrs = _alloc_result(_HostMesh(node, elem, nf), cfg, False, out)
    if dref is not None:
        if dref.dtype != np.float64 or dref.shape != (cfg.maxgate, nf) or not dref.flags.c_contiguous:
            raise ValueError("dref must be a C-contiguous float64 (maxgate, nf) array")
        arrs["dref"] = dref
        r.dref = _ptr(dref)
    N.check(lib.mmcgb_run(C.byref(d), C.byref(c), int(device), C.byref(r)))
    del keep, dkeep
    return _make_result(r, arrs)


def simulate_batch(meshes: Sequence[Mesh], cfgs: Sequence[SimConfig]) -> list:
    """Runs many simulations in one persistent launch (mmcgb_simulate_batch)."""
    lib = N.load()
    n = len(cfgs)
    if len(meshes) != n or n == 0:
        raise ValueError("need one mesh per config")
    carr = (N.Config * n)()
    rarr = (N.Result * n)()
    harr = (C.c_void_p * n)()
    keeps, allarrs = [], []
    for i in range(n):
        c, keep = cfgs[i].to_c(meshes[i].nn)
        carr[i] = c
        keeps.append(keep)
        r, arrs = _alloc_result(meshes[i], cfgs[i], False)
        rarr[i] = r
        allarrs.append(arrs)
        harr[i] = meshes[i].handle
    N.check(lib.mmcgb_simulate_batch(n, harr, carr, rarr))
    return [_make_result(rarr[i], allarrs[i]) for i in range(n)]


class Session:
    """A simulation run as several launches accumulating into the same device
    buffers (mmcgb_session_*): the reference's respin loop, and the way the
    benchmark times device-resident work."""

    def __init__(self, mesh: Mesh, cfg: SimConfig):
        lib = N.load()
        self.mesh, self.cfg = mesh, cfg
        self._c, self._keep = cfg.to_c(mesh.nn)
        h = C.c_void_p()
        N.check(lib.mmcgb_session_begin(mesh.handle, C.byref(self._c), None, C.byref(h)))
        self._h = h

    def launch(self, photon_offset: int, nphoton: int):
        N.check(N.load().mmcgb_session_launch(self._h, int(photon_offset), int(nphoton)))

    def launch_repeat(self, photon_offset: int, nphoton: int, repeats: int):
        """`repeats` launches of `nphoton` photons as one CUDA graph
        (mmcgb_session_launch_repeat); sync() then times the whole graph."""
        N.check(N.load().mmcgb_session_launch_repeat(self._h, int(photon_offset), int(nphoton), int(repeats)))

    def phase_window(self, nphoton: int) -> int:
        """The gate window a launch of `nphoton` photons runs with (0 = one
        launch; mmcgb_session_phase_window)."""
        return self.phase_plan(nphoton)[0]

    def phase_plan(self, nphoton: int):
        """(gate window, photons per phased launch) of a launch of `nphoton`
        photons (mmcgb_session_phase_window)."""
        w, ch = C.c_int32(), C.c_uint64()
        N.check(N.load().mmcgb_session_phase_window(self._h, int(nphoton), C.byref(w), C.byref(ch)))
        return int(w.value), int(ch.value)

    @property
    def stream(self) -> int:
        """The session's cudaStream_t as an integer handle."""
        return int(N.load().mmcgb_session_stream(self._h) or 0)

    def sync(self) -> float:
        ms = C.c_float()
        N.check(N.load().mmcgb_session_sync(self._h, C.byref(ms)))
        return float(ms.value)

    def device_buffers(self) -> dict:
        """Torch tensors aliasing the session's raw device buffers
        (mmcgb_session_device_buffers): ``field`` (maxgate*datalen float64, None
        with float32 accumulation), ``energy`` (2 float64), ``counters`` (3 int64),
        ``detcount`` (1 int32), ``detp`` (maxdetphoton*reclen float32),
        ``seeds`` (maxdetphoton*16 uint8) where the run saves them, and with
        srcnum > 1 patterns ``energy_src`` (64 slots x 2 x srcnum float64) and a
        field of maxgate*datalen*srcnum.  What they
        hold when the session ends is what end() reads back and normalizes.
        Synchronize the session before using them."""
        import torch
        o = N.DeviceOut()
        N.check(N.load().mmcgb_session_device_buffers(self._h, C.byref(o)))
        cfg, G = self.cfg, self.cfg.maxgate
        if cfg.method in ("grid", 1):
            datalen = int(np.prod(self.mesh.grid_dims(cfg.gridstep)))
        else:
            datalen = self.mesh.ne
        nmed = np.asarray(cfg.media).reshape(-1, 4).shape[0]
        reclen = 1 + (2 + (1 if cfg.ismomentum else 0)) * (nmed - 1) + (6 if cfg.issaveexit else 0) + 1
        maxdet = int(cfg.maxdetphoton) if cfg.issavedet else 0
        dev = torch.device("cuda", self.mesh.device)

        def wrap(ptr, n, typestr):
            if not ptr or n == 0:
                return None
            iface = {"shape": (int(n),), "typestr": typestr, "data": (int(ptr), False), "version": 3,
                     "strides": None}
            return torch.as_tensor(type("DevArray", (), {"__cuda_array_interface__": iface})(), device=dev)

        K = max(1, int(cfg.srcnum))
        return dict(field=wrap(o.field_raw, G * datalen * K, "<f8"), energy=wrap(o.energy, 2, "<f8"),
                    energy_src=wrap(o.energy_src, 64 * 2 * K, "<f8") if K > 1 else None,
                    counters=wrap(o.counters, 3, "<i8"), detcount=wrap(o.detcount, 1, "<i4"),
                    detp=wrap(o.detp, maxdet * reclen, "<f4"),
                    seeds=wrap(o.seeds, maxdet * 16, "|u1") if cfg.issaveseed else None, reclen=reclen)

    def end(self, collect: bool = True, records: bool = True) -> Optional[SimResult]:
        """Reads back, runs the output stage and releases the session.
        `records=False` leaves the detected records (and seeds) out."""
        lib = N.load()
        h, self._h = self._h, None
        if h is None:
            return None
        if not collect:
            N.check(lib.mmcgb_session_end(h, None))
            return None
        r, arrs = _alloc_result(self.mesh, self.cfg, False)
        if not records:
            r.detp = r.seeds = None
            arrs["detp"] = arrs["seeds"] = None
        N.check(lib.mmcgb_session_end(h, C.byref(r)))
        return _make_result(r, arrs)

    def __del__(self):
        if getattr(self, "_h", None) is not None:
            try:
                N.load().mmcgb_session_end(self._h, None)
            except Exception:
                pass


def launch_batch(sessions, offsets, counts, stream: Optional[int] = None):
    """One persistent launch over several sessions (mmcgb_session_launch_batch).
    With `stream` (a cudaStream_t handle, e.g. torch.cuda.Stream().cuda_stream)
    the launch is enqueued there with no ordering against the sessions' own
    streams (mmcgb_session_launch_batch_on): the caller waits for that stream
    before syncing or ending the sessions."""
    n = len(sessions)
    h = (C.c_void_p * n)(*[s._h for s in sessions])
    o = (C.c_uint64 * n)(*[int(x) for x in offsets])
    k = (C.c_uint64 * n)(*[int(x) for x in counts])
    if stream is None:
        N.check(N.load().mmcgb_session_launch_batch(n, h, o, k))
    else:
        N.check(N.load().mmcgb_session_launch_batch_on(n, h, o, k, C.c_void_p(int(stream))))


def launch_batches(groups, offsets, counts, stream: int):
    """A sequence of batched launches captured as one CUDA graph
    (mmcgb_session_launch_batches): groups[g] is a list of sessions run in one
    persistent launch, the groups one after another on `stream` (a
    cudaStream_t handle); offsets/counts hold each group's photon ranges as
    lists parallel to the groups."""
    sizes = [len(g) for g in groups]
    flat = [s._h for g in groups for s in g]
    off = [int(x) for o in offsets for x in o]
    cnt = [int(x) for c in counts for x in c]
    n = len(flat)
    N.check(N.load().mmcgb_session_launch_batches(len(groups), (C.c_int32 * len(sizes))(*sizes), (C.c_void_p * n)(*flat),
                                                   (C.c_uint64 * n)(*off), (C.c_uint64 * n)(*cnt),
                                                   C.c_void_p(int(stream))))


def pinned_empty(shape, dtype=np.float64) -> np.ndarray:
    """A page-locked host array (through torch's pinned allocator): device to
    host copies into it run at the interconnect's full rate."""
    import torch
    t = torch.empty(int(np.prod(shape)), dtype=getattr(torch, np.dtype(dtype).name), pin_memory=True)
    return t.numpy().reshape(shape)  # the array's base holds the tensor, keeping the allocation alive
