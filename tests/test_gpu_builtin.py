"""The reference's built-in benchmarks (-Q dmmc-cube60 / dmmc-cube60b,
src/mmc_bench.c:44-190) on the GPU: a 60 mm cube of 6 tets, so each photon
scatters many times inside one large element before it crosses a face.

* Through the command line (-Q name -M G), against 10 reference runs
  (tests/golden/bench_*.npz): per-voxel dual-grid fluence, total, ray-tet
  tests per photon.
* IEEE arithmetic against the oracle photon by photon.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

import golden_checks as gc
from mmc_gb300 import io
from mmc_gb300.core import Mesh, simulate

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("bench", ["dmmc-cube60", "dmmc-cube60b"])
def test_cli_builtin_benchmark_matches_reference_runs(gpu_ready, tmp_path, bench):
    fx = gc.load("bench_" + bench)
    env = dict(os.environ, PYTHONPATH=ROOT)
    r = subprocess.run([sys.executable, "-m", "mmc_gb300", "-Q", bench, "-M", "G", "-U", "0", "-E", "4242",
                        "-n", str(int(fx["photons"]))], cwd=tmp_path, env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    raw = io.read_bin(str(tmp_path / (bench + ".bin")), 1)
    msgs = gc.check_bench(raw, fx)
    tests = float(r.stdout.split("photon/ms), ")[1].split()[0])
    msgs += gc.check_tests_per_photon(tests / int(fx["photons"]), fx)
    assert not msgs, "\n".join(msgs)


def test_cli_lists_builtin_benchmarks(gpu_ready):
    r = subprocess.run([sys.executable, "-m", "mmc_gb300", "-Q"], env=dict(os.environ, PYTHONPATH=ROOT),
                       capture_output=True, text=True)
    assert r.returncode == 0 and "dmmc-cube60b" in r.stdout
    r = subprocess.run([sys.executable, "-m", "mmc_gb300", "-Q", "edgeimmc"], env=dict(os.environ, PYTHONPATH=ROOT),
                       capture_output=True, text=True)
    assert r.returncode != 0 and "unsupported benchmark" in r.stderr


@pytest.mark.parametrize("bench", ["dmmc-cube60", "dmmc-cube60b"])
def test_builtin_benchmark_matches_oracle_photon_by_photon(oracle_mod, gpu_ready, bench):
    import dataclasses
    m, cfg, _ = gc.case_mesh_and_config("bench_" + bench, nphoton=5000)
    cfg = dataclasses.replace(cfg, fast_math=0)
    g = simulate(Mesh(m.node, m.elem, m.label), cfg, trace=True)
    o = oracle_mod.run(m.node, m.elem, m.label, cfg, nthreads=8, trace=True, normalize=False)
    assert np.array_equal(g.photon_weight.view(np.uint32), o["photon_weight"].view(np.uint32))
    assert np.array_equal(g.photon_steps, o["photon_steps"])
    np.testing.assert_allclose(g.field, o["raw"], rtol=1e-8, atol=1e-12)
