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


def _rows(detp, seeds):
    return sorted(map(bytes, np.concatenate([detp.view(np.uint8).reshape(len(detp), -1), seeds], 1)))


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
    G, ne = cfg.maxgate, mesh.ne
    reclen = ref.reclen
    field = torch.empty(G * ne, dtype=torch.float64, device=dev)
    energy = torch.empty(2, dtype=torch.float64, device=dev)
    counters = torch.empty(2, dtype=torch.int64, device=dev)
    detp = torch.empty(cfg.maxdetphoton * reclen, dtype=torch.float32, device=dev)
    seeds = torch.empty(cfg.maxdetphoton * 16, dtype=torch.uint8, device=dev)
    detcount = torch.empty(1, dtype=torch.int32, device=dev)
    out = DeviceOut(field.data_ptr(), detp.data_ptr(), seeds.data_ptr(), detcount.data_ptr(),
                    energy.data_ptr(), counters.data_ptr())
    stream = torch.cuda.current_stream(dev)
    for call in range(2):
        rc = fn(mesh.handle, C.byref(c), C.byref(out), C.c_void_p(stream.cuda_stream))
        assert rc == 0, lib.mmcgb_last_error().decode()
        torch.cuda.synchronize(dev)
        np.testing.assert_allclose(field.cpu().numpy().reshape(G, ne), ref.field, rtol=1e-9, atol=1e-12,
                                   err_msg=f"call {call}")
        e = energy.cpu().numpy()
        assert e[1] == pytest.approx(ref.energyesc, rel=1e-9)
        k = counters.cpu().numpy()
        assert int(k[0]) == ref.raytet and int(k[1]) == 0
        n = int(detcount.cpu().item())
        assert n == ref.detected > 0
        got_p = detp.cpu().numpy()[: n * reclen].reshape(n, reclen)
        got_s = seeds.cpu().numpy()[: n * 16].reshape(n, 16)
        assert _rows(got_p, got_s) == _rows(ref.detp, ref.seeds)
    del keep


def test_noalloc_rejects_sizes_beyond_its_maximum(gpu_ready, small_cube):
    import torch
    lib, fn = _bind()
    m = small_cube
    mesh = Mesh(m.node, m.elem, m.label)
    media = np.tile(m.media[1], (65, 1))  # 65 rows > MMCGB_NOALLOC_MAX_MEDIA (64)
    media[0] = m.media[0]
    cfg = SimConfig(media=media, nphoton=1000, srcpos=(30.0, 30.0, 0.0), basisorder=0, isnormalized=0)
    c, keep = cfg.to_c()
    dev = torch.device("cuda", 0)
    field = torch.empty(mesh.ne, dtype=torch.float64, device=dev)
    energy = torch.empty(2, dtype=torch.float64, device=dev)
    counters = torch.empty(2, dtype=torch.int64, device=dev)
    out = DeviceOut(field.data_ptr(), None, None, None, energy.data_ptr(), counters.data_ptr())
    rc = fn(mesh.handle, C.byref(c), C.byref(out), None)
    assert rc == 1
    assert "maximum" in lib.mmcgb_last_error().decode()
    del keep
