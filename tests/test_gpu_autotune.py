"""The launch-shape autotuner (mmc_gb300/autotune.py): it times every
candidate (threads per block x persistent blocks per SM x accumulation
policy), returns the fastest as a valid launch shape, and a simulation run
with the tuned shape gives the results of the default shape -- photon streams
depend only on (seed, photon index), so the shape moves no photon."""
import dataclasses

import numpy as np
import pytest

from mmc_gb300 import meshgen
from mmc_gb300.autotune import autotune, tuned
from mmc_gb300.core import Mesh, SimConfig, simulate

pytestmark = pytest.mark.gpu


def _rows(r):
    return sorted(map(bytes, np.concatenate([r.detp.view(np.uint8).reshape(len(r.detp), -1), r.seeds], 1)))


def test_autotune_picks_a_valid_shape_that_changes_no_result(gpu_ready, small_inclusion):
    import torch
    m = small_inclusion
    mesh = Mesh(m.node, m.elem, m.label)
    cfg = SimConfig(media=m.media, nphoton=200000, seed=2718, srcpos=(30.0, 30.0, 0.0), srcdir=(0.0, 0.0, 1.0),
                    tend=5e-9, tstep=0.5e-9, issavedet=1, issaveseed=1, detpos=meshgen.c1_detectors(),
                    maxdetphoton=200000, basisorder=0, isnormalized=0)
    t = autotune(mesh, cfg, threads=(64, 128), blocks_per_sm=(6, 8), accum=(1, 0), repeats=1, use_cache=False)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    assert len(t["trials"]) == 8
    assert all(tr["photons_per_ms"] > 0 for tr in t["trials"])
    assert t["photons_per_ms"] == max(tr["photons_per_ms"] for tr in t["trials"])
    assert t["threads"] in (64, 128) and t["accum_f64"] in (0, 1)
    assert t["blocks"] % sms == 0 and t["blocks"] // sms * t["threads"] in (6 * 128, 8 * 128)
    # every float64 candidate shape gives the default shape's results
    ref = simulate(mesh, cfg)
    for tr in t["trials"]:
        c = dataclasses.replace(cfg, threads=tr["threads"], blocks=tr["blocks"], accum_f64=tr["accum_f64"])
        r = simulate(mesh, c)
        assert r.raytet == ref.raytet and r.detected == ref.detected and _rows(r) == _rows(ref)
        if tr["accum_f64"]:
            np.testing.assert_allclose(r.field, ref.field, rtol=1e-10, atol=1e-14)
        else:  # the reference's float32 accumulation: rounding only
            nz = ref.field > 1e-6 * ref.field.max()
            assert np.median(np.abs(r.field[nz] / ref.field[nz] - 1)) < 1e-6
    # tuned() applies the choice; the cached result is returned for the same workload
    c = tuned(mesh, cfg, threads=(64, 128), blocks_per_sm=(6, 8), accum=(1,), repeats=1)
    assert (c.threads, c.accum_f64) in {(64, 1), (128, 1)} and c.blocks % sms == 0
    assert autotune(mesh, cfg, threads=(64, 128), blocks_per_sm=(6, 8), accum=(1,), repeats=1) is \
        autotune(mesh, cfg, threads=(64, 128), blocks_per_sm=(6, 8), accum=(1,), repeats=1)


def test_autotune_batch_tunes_the_batched_launch(gpu_ready, small_inclusion):
    """A batch is tuned with batched trial launches of the whole batch; the
    chosen shape gives every simulation of the batch its default-shape result."""
    from mmc_gb300.autotune import autotune_batch
    from mmc_gb300.core import simulate_batch
    import torch
    m = small_inclusion
    mesh = Mesh(m.node, m.elem, m.label)
    rng = np.random.default_rng(9)
    cfgs = []
    for i in range(6):
        media = m.media.copy()
        media[1:, 0] *= rng.uniform(0.5, 2.0, len(media) - 1)
        cfgs.append(SimConfig(media=media, nphoton=int(rng.integers(20000, 80000)), seed=100 + i,
                              srcpos=(30.0, 30.0, 0.0), srcdir=(0.0, 0.0, 1.0), tend=5e-9, tstep=1e-9,
                              basisorder=0, isnormalized=0))
    t = autotune_batch([mesh] * 6, cfgs, accum=(1,), repeats=1, use_cache=False)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    assert len(t["trials"]) == 4 and t["accum_f64"] == 1 and t["blocks"] % sms == 0
    assert t["photons_per_ms"] == max(tr["photons_per_ms"] for tr in t["trials"])
    ref = simulate_batch([mesh] * 6, cfgs)
    got = simulate_batch([mesh] * 6, [dataclasses.replace(c, threads=t["threads"], blocks=t["blocks"]) for c in cfgs])
    for a, b in zip(got, ref):
        assert a.raytet == b.raytet
        np.testing.assert_allclose(a.field, b.field, rtol=1e-10, atol=1e-14)
