"""The two benchmark workloads against the reference, through the benchmark's
own path: fast math, float64 accumulation, and for the 1.296M-tet case the
gate-phased engine with the window the automatic mode picks on this GPU.
Each run is scored against 10 runs of the reference CPU engine with the same
photon count (tests/golden/c1_incl1296k.npz, c0_cube162k.npz, made by
tests/golden/make_baseline_golden.py) the way a fresh reference run scores:
per-element and per-(element, gate) coverage within 3 sigma, per-gate
totals, absorbed fraction, ray-tet tests per photon and, on the 1.296M-tet
case, detected counts, weights, mean partial paths and scatter counts per
detector."""
import dataclasses

import numpy as np
import pytest

import golden_checks as gc
from mmc_gb300 import meshgen
from mmc_gb300.core import Mesh, Session, SimConfig, simulate

pytestmark = pytest.mark.gpu


def auto_window(mesh, cfg, nphoton=100_000_000):
    """The gate window the automatic phased mode picks for a launch of the
    benchmark's size (1e8 photons)."""
    s = Session(mesh, dataclasses.replace(cfg, phased=0))
    try:
        return s.phase_window(nphoton)
    finally:
        s.end(collect=False)


@pytest.fixture(scope="module")
def c1(gpu_ready):
    m = meshgen.inclusion_cube(n=60, jitter=0.25, seed=12345)
    fx = gc.load("c1_incl1296k")
    cfg = SimConfig(media=m.media, nphoton=int(fx["photons"]), seed=9001, srcpos=(30.0, 30.0, 0.0),
                    srcdir=(0.0, 0.0, 1.0), tend=5e-9, tstep=1e-10, issavedet=1, detpos=meshgen.c1_detectors(),
                    maxdetphoton=2_000_000, basisorder=0, isnormalized=0, fast_math=1, accum_f64=1)
    mesh = Mesh(m.node, m.elem, m.label)
    window = auto_window(mesh, cfg)
    assert 1 <= window < 50
    return m, mesh, dataclasses.replace(cfg, phased=window), fx


def test_inclusion_cube_1296k_matches_reference_runs(c1):
    m, mesh, cfg, fx = c1
    assert cfg.maxgate == int(fx["gates"]) == 50 and mesh.ne == int(fx["ne"])
    r = simulate(mesh, cfg)
    assert r.aborted == 0
    msgs = gc.check_field(r.field, fx, m.media, m.label, cfg.nphoton)
    msgs += gc.check_tests_per_photon(r.raytet / cfg.nphoton, fx)
    msgs += gc.check_detectors(r.detp, m.media, fx)
    assert r.detected == len(r.detp)
    assert not msgs, "\n".join(msgs)


def test_inclusion_cube_1296k_float32_vs_float64_accumulation(c1):
    """The reference's float32 accumulation (with its overflow buffer) against
    float64 on the same photons of the benchmark workload: the per-cell error."""
    m, mesh, cfg, fx = c1
    a = simulate(mesh, cfg).field
    c32 = dataclasses.replace(cfg, accum_f64=0)
    b = simulate(mesh, dataclasses.replace(c32, phased=auto_window(mesh, c32))).field
    nz = a > 1e-6 * a.max()
    rel = np.abs(b[nz] - a[nz]) / a[nz]
    tot = abs(b.sum() - a.sum()) / a.sum()
    print(f"float32 vs float64 accumulation, {nz.sum()} cells: median {np.median(rel):.2e}, "
          f"99.9th percentile {np.quantile(rel, 0.999):.2e}, max {rel.max():.2e}, total {tot:.2e}")
    assert np.median(rel) < 1e-6 and rel.max() < 1e-3 and tot < 1e-6


@pytest.fixture(scope="module")
def c0(gpu_ready):
    m = meshgen.homogeneous_cube(n=30)
    fx = gc.load("c0_cube162k")
    cfg = SimConfig(media=m.media, nphoton=int(fx["photons"]), seed=9002, srcpos=(30.0, 30.0, 0.0),
                    srcdir=(0.0, 0.0, 1.0), tend=5e-9, tstep=5e-9, basisorder=0, isnormalized=0, fast_math=1,
                    accum_f64=1)
    return m, Mesh(m.node, m.elem, m.label), cfg, fx


def test_cube_162k_elements_and_nodes_match_reference_runs(c0):
    """Element deposits, and the node output of the same photons (the GPU
    output stage: 0.25 scatter, nodal volumes, energy balance) against the
    reference's own output stage applied to each reference run."""
    m, mesh, cfg, fx = c0
    assert mesh.ne == int(fx["ne"]) == 162000 and mesh.nn == 29791
    raw = simulate(mesh, cfg)
    msgs = gc.check_field(raw.field, fx, m.media, m.label, cfg.nphoton)
    msgs += gc.check_tests_per_photon(raw.raytet / cfg.nphoton, fx)
    node = simulate(mesh, dataclasses.replace(cfg, basisorder=1, isnormalized=1))
    assert node.raytet == raw.raytet  # the same photons
    # The reference CPU engine normalizes with the weight its deposits absorbed; the
    # CUDA host (and this library) with launched minus escaped weight
    # (src/mmc_host.c:372 vs src/mmc_cu_host.cu:987).  The fixture uses the former:
    # convert, with both figures taken from this run (they differ by the weight still
    # in flight at the end of the window, ~1e-3 here).
    mua = m.media[m.label, 0].astype(np.float64)
    e_dep = float((raw.field.sum(0) * mua).sum())
    e_cuda = node.energytot - node.energyesc
    assert abs(e_dep / e_cuda - 1.0) < 0.01
    msgs += gc.check_nodes(node.field[0] * (e_dep / e_cuda), fx)
    assert not msgs, "\n".join(msgs)
