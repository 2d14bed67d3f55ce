"""Batched launches: several simulations (different meshes, optical
properties, sources, photon counts) share one persistent launch.  Each photon
stream depends only on its simulation's seed and photon index, so every
simulation must give the same deposits and detected records alone and in the
mix (float64 accumulation: equal up to the order of the additions)."""
import dataclasses

import numpy as np
import pytest

from mmc_gb300 import meshgen
from mmc_gb300.core import Mesh, Session, SimConfig, launch_batch, simulate, simulate_batch

pytestmark = pytest.mark.gpu


def _rows(r):
    return sorted(map(bytes, np.concatenate([r.detp.view(np.uint8).reshape(len(r.detp), -1), r.seeds], 1)))


def _cases():
    a = meshgen.inclusion_cube(n=16, jitter=0.5, seed=4)
    b = meshgen.shell_mesh(n=20, jitter=0.5, seed=5)
    ma, mb = Mesh(a.node, a.elem, a.label), Mesh(b.node, b.elem, b.label)
    det = np.array([[40, 30, 0, 3], [45, 30, 0, 3]], np.float32)
    sh_media = b.media.copy()
    sh_media[1:, 0] *= 1.7
    cfgs = [
        SimConfig(media=a.media, nphoton=30000, seed=1, srcpos=(30, 30, 0), tend=5e-9, tstep=0.5e-9,
                  issavedet=1, issaveseed=1, detpos=det, maxdetphoton=50000, basisorder=0, isnormalized=0),
        SimConfig(media=sh_media, nphoton=7000, seed=2, srcpos=(30, 30, 5.6), srcdir=(0, 0, 1), tend=5e-9,
                  tstep=0.5e-9, issavedet=1, issaveseed=1, detpos=np.array([[30, 30, 5, 4]], np.float32),
                  maxdetphoton=50000, basisorder=0, isnormalized=0),
        SimConfig(media=a.media, nphoton=120000, seed=3, srcpos=(30, 30, 0), tend=5e-9, tstep=1e-9,
                  issavedet=1, issaveseed=1, detpos=det, maxdetphoton=50000, basisorder=0, isnormalized=0),
    ]
    return [ma, mb, ma], cfgs


def test_batch_equals_individual_runs(gpu_ready):
    meshes, cfgs = _cases()
    alone = [simulate(m, c) for m, c in zip(meshes, cfgs)]
    mixed = simulate_batch(meshes, cfgs)
    for a, b in zip(alone, mixed):
        np.testing.assert_allclose(b.field, a.field, rtol=1e-9, atol=1e-12)
        assert a.raytet == b.raytet and a.detected == b.detected
        assert _rows(a) == _rows(b)
        assert b.energyesc == pytest.approx(a.energyesc, rel=1e-9)


def test_session_waves_equal_individual_runs(gpu_ready):
    """Sessions advanced in several shared waves (the serving loop's launch
    pattern) reproduce their one-shot results."""
    meshes, cfgs = _cases()
    alone = [simulate(m, c) for m, c in zip(meshes, cfgs)]
    sess = [Session(m, c) for m, c in zip(meshes, cfgs)]
    done = [0] * len(cfgs)
    quantum = 20000
    while any(d < c.nphoton for d, c in zip(done, cfgs)):
        live = [i for i, c in enumerate(cfgs) if done[i] < c.nphoton]
        counts = [min(quantum, cfgs[i].nphoton - done[i]) for i in live]
        launch_batch([sess[i] for i in live], [done[i] for i in live], counts)
        for i, k in zip(live, counts):
            done[i] += k
    res = [s.end() for s in sess]
    for a, b in zip(alone, res):
        np.testing.assert_allclose(b.field, a.field, rtol=1e-9, atol=1e-12)
        assert a.raytet == b.raytet and _rows(a) == _rows(b)


def test_overlapping_waves_on_two_streams(gpu_ready):
    """Waves enqueued on two caller streams with no ordering between them
    (mmcgb_session_launch_batch_on) run concurrently into the same sessions;
    once both streams are synchronized every session equals its solo run."""
    import torch
    meshes, cfgs = _cases()
    alone = [simulate(m, c) for m, c in zip(meshes, cfgs)]
    sess = [Session(m, c) for m, c in zip(meshes, cfgs)]
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    half = [c.nphoton // 2 for c in cfgs]
    launch_batch(sess, [0] * len(cfgs), half, stream=streams[0].cuda_stream)
    launch_batch(sess, half, [c.nphoton - h for c, h in zip(cfgs, half)], stream=streams[1].cuda_stream)
    for st in streams:
        st.synchronize()
    res = [s.end() for s in sess]
    for a, b in zip(alone, res):
        np.testing.assert_allclose(b.field, a.field, rtol=1e-9, atol=1e-12)
        assert a.raytet == b.raytet and _rows(a) == _rows(b)


def test_respin_graph_equals_one_launch(gpu_ready):
    """The respin loop as a CUDA graph (mmcgb_session_launch_repeat), also
    after an in-place update of the graph for a new photon range, equals one
    launch of all the photons."""
    meshes, cfgs = _cases()
    m, c = meshes[2], cfgs[2]
    n = c.nphoton // 4
    alone = simulate(m, dataclasses.replace(c, nphoton=4 * n))
    s = Session(m, dataclasses.replace(c, nphoton=4 * n))
    s.launch_repeat(0, n, 2)
    assert s.sync() > 0
    s.launch_repeat(2 * n, n, 2)  # same shape: the instantiated graph is updated in place
    r = s.end()
    np.testing.assert_allclose(r.field, alone.field, rtol=1e-9, atol=1e-12)
    assert r.raytet == alone.raytet and _rows(r) == _rows(alone)


def test_batch_mixing_grid_output_and_trajectories(gpu_ready):
    """A pencil-beam simulation with dual-grid output or trajectory records
    runs in the general kernels; a batch holding one next to a plain element
    simulation must run them there too, each equal to its solo run."""
    a = meshgen.inclusion_cube(n=16, jitter=0.5, seed=4)
    m = Mesh(a.node, a.elem, a.label)
    base = SimConfig(media=a.media, nphoton=20000, seed=9, srcpos=(30, 30, 0), tend=5e-9, tstep=1e-9,
                     basisorder=0, isnormalized=0)
    cfgs = [base, dataclasses.replace(base, seed=10, method="grid", gridstep=2.0),
            dataclasses.replace(base, seed=11, maxjumpdebug=4_000_000)]
    alone = [simulate(m, c) for c in cfgs]
    mixed = simulate_batch([m, m, m], cfgs)
    for a_, b_ in zip(alone, mixed):
        assert b_.field.shape == a_.field.shape
        np.testing.assert_allclose(b_.field, a_.field, rtol=1e-9, atol=1e-12)
        assert a_.raytet == b_.raytet
    t_a, t_b = alone[2].traj, mixed[2].traj
    assert alone[2].ntraj == mixed[2].ntraj == len(t_b)
    order = lambda t: t[np.argsort(t[:, 0].view(np.uint32), kind="stable")].view(np.uint32)  # noqa: E731
    assert np.array_equal(order(t_a), order(t_b))


def test_simulate_many_equals_solo_runs(gpu_ready, small_inclusion):
    """Size-aware scheduling (batching.simulate_many): simulations grouped by
    photon count into batched launches, optionally the largest run on their own
    on a second stream, optionally the groups over two streams; every result
    equals the simulation run alone."""
    import dataclasses
    from mmc_gb300.batching import simulate_many
    m = small_inclusion
    mesh = Mesh(m.node, m.elem, m.label)
    rng = np.random.default_rng(21)
    cfgs = []
    for i, n in enumerate([3000, 120000, 8000, 90000, 500, 20000]):
        media = m.media.copy()
        media[1:, 0] *= rng.uniform(0.5, 2.0, len(media) - 1)
        cfgs.append(SimConfig(media=media, nphoton=n, seed=300 + i, srcpos=(30.0, 30.0, 0.0),
                              srcdir=(0.0, 0.0, 1.0), tend=5e-9, tstep=1e-9, basisorder=0, isnormalized=0,
                              issavedet=1, issaveseed=1, detpos=meshgen.c1_detectors(), maxdetphoton=50000))
    for solo, group, streams in ((50000, None, 1), (50000, 25000, 2), (None, 100000, 1)):
        got = simulate_many([mesh] * len(cfgs), cfgs, group_photons=group, solo_photons=solo, streams=streams)
        for c, r in zip(cfgs, got):
            ref = simulate(mesh, c)
            assert r.raytet == ref.raytet and r.detected == ref.detected
            # raw deposits (float64 atomics): equal up to summation order; the escaped weight is
            # summed per lane in float32 first, so it agrees to float32 rounding across launch shapes
            assert r.energyesc == pytest.approx(ref.energyesc, rel=1e-6)
            np.testing.assert_allclose(r.field, ref.field, rtol=1e-10, atol=1e-14)
            rows = lambda x: sorted(map(bytes, np.concatenate([x.detp.view(np.uint8).reshape(len(x.detp), -1), x.seeds], 1)))  # noqa: E731
            assert rows(r) == rows(ref)


def test_batched_launches_as_one_graph(gpu_ready, small_inclusion):
    """mmcgb_session_launch_batches: a sequence of batched launches captured as
    one CUDA graph.  Two calls of the same shape (the second updates the
    instantiated graph in place) over consecutive photon ranges, then a call
    of another shape: every simulation equals its solo run of all its photons."""
    import torch
    from mmc_gb300.core import launch_batches
    m = small_inclusion
    mesh = Mesh(m.node, m.elem, m.label)
    cfgs = [SimConfig(media=m.media, nphoton=n, seed=700 + i, srcpos=(30.0, 30.0, 0.0), srcdir=(0.0, 0.0, 1.0),
                      tend=5e-9, tstep=1e-9, basisorder=0, isnormalized=0, issavedet=1, issaveseed=1,
                      detpos=meshgen.c1_detectors(), maxdetphoton=50000)
            for i, n in enumerate([6000, 9000, 30000, 12000, 4000])]
    st = torch.cuda.Stream()
    sess = [Session(mesh, c) for c in cfgs]
    groups = [[sess[0], sess[1]], [sess[2]], [sess[3], sess[4]]]
    idx = [[0, 1], [2], [3, 4]]
    half = [[cfgs[i].nphoton // 2 for i in g] for g in idx]
    rest = [[cfgs[i].nphoton - cfgs[i].nphoton // 2 for i in g] for g in idx]
    launch_batches(groups, [[0] * len(g) for g in idx], half, st.cuda_stream)
    launch_batches(groups, half, rest, st.cuda_stream)  # same shape: the graph is updated in place
    got = [s.end() for s in sess]
    sess2 = [Session(mesh, c) for c in cfgs]
    launch_batches([sess2], [[0] * 5], [[c.nphoton for c in cfgs]], st.cuda_stream)  # another shape
    got2 = [s.end() for s in sess2]
    st.synchronize()
    for c, a, b in zip(cfgs, got, got2):
        ref = simulate(mesh, c)
        for r in (a, b):
            assert r.raytet == ref.raytet and r.detected == ref.detected
            np.testing.assert_allclose(r.field, ref.field, rtol=1e-10, atol=1e-14)
