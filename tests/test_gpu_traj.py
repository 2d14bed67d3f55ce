"""Photon trajectory records (the reference's -D M, savedebugdata in
src/mmc_raytrace.c:1739-1756 and src/mmc_core.cl:692-704) on the GPU.

* IEEE arithmetic: the record set (photon id, position, weight, element at
  launch, every scattering event and photon end) equals the oracle's bit for
  bit, through one launch, the gate-phased launches (photons parked and
  resumed between windows) and a session of several launches.
* Fast arithmetic: the record statistics match the reference's runs
  (tests/golden/traj_cube6k.npz).
* A full buffer keeps maxjumpdebug records and reports how many there were.
* The command line (-D M) and pmmc (debuglevel 'M') write them as the
  reference does.
"""
import dataclasses
import json
import os
import subprocess
import sys

import numpy as np
import pytest

import golden_checks as gc
from mmc_gb300 import io, meshgen, pmmc
from mmc_gb300.core import Mesh, Session, SimConfig, simulate

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def by_photon(traj):
    """Records grouped by photon id, each photon's in the order written."""
    order = np.argsort(traj[:, 0].view(np.uint32), kind="stable")
    return traj[order]


@pytest.fixture(scope="module")
def incl(gpu_ready):
    m = meshgen.inclusion_cube(n=12, jitter=0.4, seed=3)
    return m, Mesh(m.node, m.elem, m.label)


def test_records_match_oracle_bit_for_bit(oracle_mod, incl):
    m, mesh = incl
    cfg = SimConfig(media=m.media, nphoton=4000, seed=21, srcpos=(30.0, 30.0, 0.0), srcdir=(0.0, 0.0, 1.0),
                    tend=5e-9, tstep=0.5e-9, basisorder=0, isnormalized=0, fast_math=0, maxjumpdebug=2000000)
    o = oracle_mod.run(m.node, m.elem, m.label, cfg, nthreads=8, trace=True)
    assert o["ntraj"] == len(o["traj"]) < cfg.maxjumpdebug
    want = by_photon(o["traj"]).view(np.uint32)
    for phased in (0, 3):  # one launch; windows of 3 gates with parked photons
        g = simulate(mesh, dataclasses.replace(cfg, phased=phased), trace=True)
        assert g.ntraj == o["ntraj"], phased
        assert np.array_equal(by_photon(g.traj).view(np.uint32), want), phased
        assert np.array_equal(g.photon_weight.view(np.uint32), o["photon_weight"].view(np.uint32))


def test_session_records_carry_global_photon_ids(oracle_mod, incl):
    """Launches at photon offsets write the photon's index in the whole
    simulation, so a session's records equal one run's."""
    m, mesh = incl
    cfg = SimConfig(media=m.media, nphoton=3000, seed=5, srcpos=(30.0, 30.0, 0.0), srcdir=(0.0, 0.0, 1.0),
                    tend=5e-9, tstep=1e-9, basisorder=0, isnormalized=0, fast_math=0, maxjumpdebug=2000000)
    s = Session(mesh, cfg)
    for off in range(0, 3000, 1000):
        s.launch(off, 1000)
    r = s.end()
    o = oracle_mod.run(m.node, m.elem, m.label, cfg, nthreads=8)
    assert r.ntraj == o["ntraj"]
    assert np.array_equal(by_photon(r.traj).view(np.uint32), by_photon(o["traj"]).view(np.uint32))
    assert set(np.unique(r.traj[:, 0].view(np.uint32))) == set(range(3000))


def test_records_match_reference_runs(gpu_ready):
    m, cfg, fx = gc.case_mesh_and_config("traj_cube6k")
    r = simulate(Mesh(m.node, m.elem, m.label), dataclasses.replace(cfg, fast_math=1))
    assert r.ntraj == len(r.traj) < cfg.maxjumpdebug
    msgs = gc.check_traj(r.traj, cfg.nphoton, fx)
    assert not msgs, "\n".join(msgs)


def test_full_buffer_keeps_the_first_records(incl):
    m, mesh = incl
    cfg = SimConfig(media=m.media, nphoton=2000, seed=1, srcpos=(30.0, 30.0, 0.0), srcdir=(0.0, 0.0, 1.0),
                    tend=5e-9, tstep=5e-9, basisorder=0, maxjumpdebug=1000)
    r = simulate(mesh, cfg)
    assert r.ntraj > 1000 and r.traj.shape == (1000, 6)
    assert np.all(r.traj[:, 4] > 0) and np.all(r.traj[:, 4] <= 1)


def test_cli_and_pmmc_write_trajectories(gpu_ready, tmp_path):
    m = meshgen.homogeneous_cube(n=8)
    cfg = {"Session": {"ID": "t", "Photons": 500, "RNGSeed": 2, "DebugFlag": "M"},
           "Domain": {"Media": m.media.tolist()},
           "Mesh": {"MeshNode": m.node.tolist(), "MeshElem": np.c_[m.elem, m.label].tolist()},
           "Forward": {"T0": 0.0, "T1": 5e-9, "Dt": 5e-9},
           "Optode": {"Source": {"Pos": [30, 30, 0], "Dir": [0, 0, 1]}}}
    (tmp_path / "in.json").write_text(json.dumps(cfg))
    env = dict(os.environ, PYTHONPATH=ROOT)
    r = subprocess.run([sys.executable, "-m", "mmc_gb300", "-f", "in.json", "--maxjumpdebug", "1000000"],
                       cwd=tmp_path, env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    traj, hdr, seeds = io.read_mch(str(tmp_path / "t.mch"))
    assert hdr["colcount"] == 6 and hdr["detected"] == 0 and seeds is None
    assert set(np.unique(traj[:, 0].view(np.uint32))) == set(range(500))
    out = pmmc.run(dict(node=m.node, elem=m.elem, elemprop=m.label, prop=m.media, srcpos=[30, 30, 0],
                        srcdir=[0, 0, 1], nphoton=500, seed=2, tstart=0.0, tend=5e-9, tstep=5e-9, debuglevel="M",
                        maxjumpdebug=1000000))
    assert out["traj"].shape[0] == 6 and out["traj"].shape[1] == len(traj)
    with pytest.raises(ValueError):
        pmmc.run(dict(node=m.node, elem=m.elem, prop=m.media, srcpos=[30, 30, 0], debuglevel="Q"))
