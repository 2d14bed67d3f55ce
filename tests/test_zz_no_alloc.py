"""The no-allocation entry point, mmcgb_simulate_noalloc, through the C ABI.

It serves callers that cannot let a library allocate device memory (a program
whose own pool already owns the GPU's free memory, or a serving loop that must
not take the device-wide synchronization of cudaMalloc/cudaFree).  Here the
test plays that caller: it owns the output buffers (torch tensors) and checks
two calls in a row against mmcgb_simulate on the same inputs -- each call
starts from its cleared scratch, so both must agree with the allocating entry.
This file is collected last so that a stop-at-first-failure run has already
run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from mmc_gb300 import _native, meshgen
from mmc_gb300.core import Mesh, SimConfig, simulate

pytestmark = pytest.mark.gpu


class DeviceOut(C.Structure):
    _fields_ = [("field_raw", C.c_void_p), ("detp", C.c_void_p), ("seeds", C.c_void_p),
                ("detcount", C.c_void_p), ("energy", C.c_void_p), ("counters", C.c_void_p)]


def _bind():
    lib = _native.load()
    fn = lib.mmcgb_simulate_noalloc
    fn.argtypes = [C.c_void_p, C.POINTER(_native.Config), C.POINTER(DeviceOut), C.c_void_p]
    fn.restype = C.c_int32
    return lib, fn


def _device_memory_state(dev):
    """(free bytes, default-pool reserved bytes, default-pool used bytes) of `dev`
    through the driver API: the library's other entries allocate with
    cudaMallocAsync from the default pool, plain cudaMalloc shows in the free
    bytes."""
    import torch
    cu = C.CDLL("libcuda.so.1")
    free, total = C.c_size_t(), C.c_size_t()
    assert cu.cuMemGetInfo_v2(C.byref(free), C.byref(total)) == 0
    pool = C.c_void_p()
    assert cu.cuDeviceGetDefaultMemPool(C.byref(pool), C.c_int(dev.index)) == 0
    reserved, used = C.c_uint64(), C.c_uint64()
    assert cu.cuMemPoolGetAttribute(pool, C.c_int(5), C.byref(reserved)) == 0  # RESERVED_MEM_CURRENT
    assert cu.cuMemPoolGetAttribute(pool, C.c_int(7), C.byref(used)) == 0      # USED_MEM_CURRENT
    torch.cuda.synchronize(dev)
    return free.value, reserved.value, used.value


def _rows(detp, seeds):
    return sorted(map(bytes, np.concatenate([detp.view(np.uint8).reshape(len(detp), -1), seeds], 1)))


def _outputs(cfg, ne, reclen, dev):
    import torch
    return dict(field=torch.empty(cfg.maxgate * ne, dtype=torch.float64, device=dev),
                energy=torch.empty(2, dtype=torch.float64, device=dev),
                counters=torch.empty(2, dtype=torch.int64, device=dev),
                detp=torch.empty(cfg.maxdetphoton * reclen, dtype=torch.float32, device=dev),
                seeds=torch.empty(cfg.maxdetphoton * 16, dtype=torch.uint8, device=dev),
                detcount=torch.empty(1, dtype=torch.int32, device=dev))


def _check_against(ref, o, cfg, ne, what):
    G, reclen = cfg.maxgate, ref.reclen
    np.testing.assert_allclose(o["field"].cpu().numpy().reshape(G, ne), ref.field, rtol=1e-9, atol=1e-12,
                               err_msg=what)
    e = o["energy"].cpu().numpy()
    assert e[1] == pytest.approx(ref.energyesc, rel=1e-9), what
    k = o["counters"].cpu().numpy()
    assert int(k[0]) == ref.raytet and int(k[1]) == 0, what
    n = int(o["detcount"].cpu().item())
    assert n == ref.detected > 0, what
    n = min(n, cfg.maxdetphoton)  # detcount counts every detection; only maxdetphoton rows are stored
    got_p = o["detp"].cpu().numpy()[: n * reclen].reshape(n, reclen)
    got_s = o["seeds"].cpu().numpy()[: n * 16].reshape(n, 16)
    assert _rows(got_p, got_s) == _rows(ref.detp, ref.seeds), what


def test_noalloc_matches_simulate_on_two_calls(gpu_ready, small_inclusion):
    import torch
    lib, fn = _bind()
    m = small_inclusion
    mesh = Mesh(m.node, m.elem, m.label)
    cfg = SimConfig(media=m.media, nphoton=50000, seed=77, srcpos=(30.0, 30.0, 0.0), srcdir=(0.0, 0.0, 1.0),
                    tend=5e-9, tstep=0.5e-9, basisorder=0, isnormalized=0, issavedet=1, issaveseed=1,
                    detpos=meshgen.c1_detectors(), maxdetphoton=20000)
    ref = simulate(mesh, cfg)
    c, keep = cfg.to_c()
    dev = torch.device("cuda", 0)
    o = _outputs(cfg, mesh.ne, ref.reclen, dev)
    out = DeviceOut(o["field"].data_ptr(), o["detp"].data_ptr(), o["seeds"].data_ptr(), o["detcount"].data_ptr(),
                    o["energy"].data_ptr(), o["counters"].data_ptr())
    stream = torch.cuda.current_stream(dev)
    states = []
    for call in range(2):
        rc = fn(mesh.handle, C.byref(c), C.byref(out), C.c_void_p(stream.cuda_stream))
        assert rc == 0, lib.mmcgb_last_error().decode()
        torch.cuda.synchronize(dev)
        states.append(_device_memory_state(dev))
        _check_against(ref, o, cfg, mesh.ne, f"call {call}")
    # The first call on a device may load the library's device code and its fixed array;
    # from then on a call takes no device memory: neither cudaMalloc (free bytes) nor the
    # stream-ordered pool the other entries allocate from.
    assert states[1] == states[0], f"device memory changed across a call: {states}"
    del keep


def test_noalloc_checks_a_given_initial_element(gpu_ready, small_inclusion):
    """A caller-supplied e0 that does not enclose the source is replaced by the
    located element, as mmcgb_simulate does; the results agree."""
    import torch
    lib, fn = _bind()
    m = small_inclusion
    mesh = Mesh(m.node, m.elem, m.label)
    cfg = SimConfig(media=m.media, nphoton=20000, seed=91, srcpos=(30.0, 30.0, 0.0), srcdir=(0.0, 0.0, 1.0),
                    tend=5e-9, tstep=1e-9, basisorder=0, isnormalized=0, issavedet=1, issaveseed=1,
                    detpos=meshgen.c1_detectors(), maxdetphoton=20000)
    ref = simulate(mesh, cfg)
    e_true = mesh.locate((30.0, 30.0, 0.0))
    wrong = mesh.ne if e_true != mesh.ne else 1
    c, keep = cfg.to_c()
    c.e0 = wrong
    dev = torch.device("cuda", 0)
    o = _outputs(cfg, mesh.ne, ref.reclen, dev)
    out = DeviceOut(o["field"].data_ptr(), o["detp"].data_ptr(), o["seeds"].data_ptr(), o["detcount"].data_ptr(),
                    o["energy"].data_ptr(), o["counters"].data_ptr())
    rc = fn(mesh.handle, C.byref(c), C.byref(out), C.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
    assert rc == 0, lib.mmcgb_last_error().decode()
    torch.cuda.synchronize(dev)
    _check_against(ref, o, cfg, mesh.ne, f"e0 {wrong} given, source in {e_true}")
    del keep


def test_noalloc_rejects_sizes_beyond_its_maximum(gpu_ready, small_cube):
    import torch
    lib, fn = _bind()
    m = small_cube
    mesh = Mesh(m.node, m.elem, m.label)
    dev = torch.device("cuda", 0)
    field = torch.empty(mesh.ne, dtype=torch.float64, device=dev)
    energy = torch.empty(2, dtype=torch.float64, device=dev)
    counters = torch.empty(2, dtype=torch.int64, device=dev)
    detp = torch.empty(1000 * 8, dtype=torch.float32, device=dev)
    detcount = torch.empty(1, dtype=torch.int32, device=dev)
    out = DeviceOut(field.data_ptr(), detp.data_ptr(), None, detcount.data_ptr(), energy.data_ptr(),
                    counters.data_ptr())
    # 65 media rows > MMCGB_NOALLOC_MAX_MEDIA (64)
    media = np.tile(m.media[1], (65, 1))
    media[0] = m.media[0]
    cfg = SimConfig(media=media, nphoton=1000, srcpos=(30.0, 30.0, 0.0), basisorder=0, isnormalized=0)
    c, keep = cfg.to_c()
    assert fn(mesh.handle, C.byref(c), C.byref(out), None) == 1
    assert "64" in lib.mmcgb_last_error().decode()
    # 257 detectors > MMCGB_NOALLOC_MAX_DET (256)
    dets = np.zeros((257, 4), np.float32)
    dets[:, 0] = np.linspace(1.0, 59.0, 257)
    dets[:, 3] = 0.5
    cfg = SimConfig(media=m.media, nphoton=1000, srcpos=(30.0, 30.0, 0.0), basisorder=0, isnormalized=0,
                    issavedet=1, detpos=dets, maxdetphoton=1000)
    c2, keep2 = cfg.to_c()
    assert fn(mesh.handle, C.byref(c2), C.byref(out), None) == 1
    msg = lib.mmcgb_last_error().decode()
    assert "maximum" in msg and "256" in msg, msg
    # per-node properties would need device copies of the nodal arrays
    cfg = SimConfig(media=m.media, nphoton=1000, srcpos=(30.0, 30.0, 0.0), basisorder=0, isnormalized=0,
                    nodemua=np.full(mesh.nn, 0.01, np.float32))
    c3, keep3 = cfg.to_c(mesh.nn)
    assert fn(mesh.handle, C.byref(c3), C.byref(out), None) == 1
    assert "per-node" in lib.mmcgb_last_error().decode()
    torch.cuda.synchronize(dev)
    del keep, keep2, keep3
