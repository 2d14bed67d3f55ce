"""The oracle's math kernels and RNG recipe (the CUDA engine runs the same
operation sequence; the GPU tests check that the two agree bit for bit)."""
import ctypes as C

import numpy as np
import pytest


def _ulp_err(got, ref):
    got = np.asarray(got, np.float32).astype(np.float64)
    ulp = np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)
    return np.abs(got - ref) / ulp


def test_expf_accuracy(oracle_mod):
    lib = oracle_mod.load()
    x = np.concatenate([np.linspace(-87.0, 0.0, 20001), np.linspace(-2.0, 2.0, 4001)]).astype(np.float32)
    got = np.array([lib.oracle_expf(float(v)) for v in x], np.float32)
    assert _ulp_err(got, np.exp(x.astype(np.float64))).max() <= 2.0
    assert lib.oracle_expf(-200.0) == 0.0


def test_logf_accuracy(oracle_mod):
    lib = oracle_mod.load()
    u = np.concatenate([np.float32(1e-6) + np.linspace(0, 1, 20001, dtype=np.float32),
                        np.geomspace(1e-6, 1.0, 5001).astype(np.float32)])
    got = np.array([lib.oracle_logf(float(v)) for v in u], np.float32)
    ref = np.log(u.astype(np.float64))
    err = np.abs(got.astype(np.float64) - ref)
    # near log(x)=0 compare absolutely, elsewhere in ulps
    big = np.abs(ref) > 1e-3
    assert _ulp_err(got[big], ref[big]).max() <= 3.0
    assert err[~big].max() < 1e-9


def test_sincos2pi_accuracy(oracle_mod):
    lib = oracle_mod.load()
    s, c = C.c_float(), C.c_float()
    u = np.linspace(0, 1, 40001, endpoint=False, dtype=np.float32)
    ss, cc = [], []
    for v in u:
        lib.oracle_sincos2pi(float(v), C.byref(s), C.byref(c))
        ss.append(s.value)
        cc.append(c.value)
    ref = 2 * np.pi * u.astype(np.float64)
    assert np.abs(np.array(ss) - np.sin(ref)).max() < 3e-7
    assert np.abs(np.array(cc) - np.cos(ref)).max() < 3e-7


def _xorshift_py(t0, t1, n):
    """xorshift128+ with the float extraction of src/mmc_core.cl:517-531,
    restated with Python integers."""
    M = (1 << 64) - 1
    out = []
    for _ in range(n):
        s1, s0 = t0, t1
        t0 = s0
        s1 ^= (s1 << 23) & M
        t1 = s1 ^ s0 ^ (s1 >> 18) ^ (s0 >> 5)
        r = (t1 + s0) & M
        lo = r & 0xFFFFFFFF
        bits = 0x3F800000 | (lo >> 9)
        out.append(np.frombuffer(np.uint32(bits).tobytes(), np.float32)[0] - np.float32(1.0))
    return out, (t0, t1)


def test_xorshift128p_recipe(oracle_mod):
    lib = oracle_mod.load()
    st = (C.c_uint64 * 2)()
    lib.oracle_rng_seed(1648335518, 12345, C.byref(st))
    t0, t1 = st[0], st[1]
    ref, _ = _xorshift_py(t0, t1, 1000)
    got = [lib.oracle_rng_next(C.byref(st)) for _ in range(1000)]
    assert np.array_equal(np.array(got, np.float32), np.array(ref, np.float32))
    assert all(0.0 <= v < 1.0 for v in got)


def test_per_photon_seeds_are_distinct(oracle_mod):
    lib = oracle_mod.load()
    seen = set()
    st = (C.c_uint64 * 2)()
    for pid in range(5000):
        lib.oracle_rng_seed(7, pid, C.byref(st))
        seen.add((st[0], st[1]))
    assert len(seen) == 5000
