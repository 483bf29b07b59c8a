"""Host logic of the batched subsystem step (serenity_gb300/batch.py) on the CPU: the
log-uniform cluster sizes of the subsystem workload, and the block-size autotuner's choice
and cache (timings faked; the batched builds are covered by tests/test_gpu_batch.py)."""
import json
import types

import numpy as np

from serenity_gb300 import batch


def test_cluster_sizes_are_seeded_log_uniform_in_range():
    s = batch.cluster_sizes(4000, 3, 40, seed=0)
    assert s == batch.cluster_sizes(4000, 3, 40, seed=0)
    assert s != batch.cluster_sizes(4000, 3, 40, seed=1)
    assert min(s) >= 3 and max(s) <= 40
    # log-uniform: about as many clusters in [3, 11) as in [11, 40]
    lo = sum(1 for m in s if m < 11)
    assert abs(lo / len(s) - 0.5) < 0.06


def test_autotuner_picks_fastest_and_caches(tmp_path, monkeypatch):
    timings = {64: 3.0, 96: 1.5, 128: 2.0}
    built = []

    class FakeBatch:
        def __init__(self, ctx, workloads, precision, mb, grids=None):
            self.mb = mb
            built.append(mb)

        def capture(self):
            pass

        def replay(self):
            pass

        def close(self):
            pass

    monkeypatch.setattr(batch, "SubsystemBatch", FakeBatch)
    monkeypatch.setattr(batch, "_time", lambda fn, ctx, reps=3: timings[fn.__self__.mb])
    monkeypatch.setattr(batch, "xcgpu", types.SimpleNamespace(
        Grid=types.SimpleNamespace(build=lambda *a, **k: object()), PREC_MIXED=1))
    w = types.SimpleNamespace(basis_name="DEF2-SVP", func="PBE", Z=np.zeros(300), coords=None, n_rad=75, n_ang=302)
    cache = str(tmp_path / "tune.json")
    best, t = batch.autotune_block(object(), [w, w], precision=1, cache_path=cache)
    assert best == 96 and t == timings and built == [64, 96, 128]
    stored = json.load(open(cache))
    assert list(stored.values()) == [96]
    assert list(stored)[0].startswith("DEF2-SVP/PBE/1/")  # basis, functional, precision, size bucket
    built.clear()
    best2, t2 = batch.autotune_block(object(), [w, w], precision=1, cache_path=cache)
    assert best2 == 96 and t2 == {} and built == []  # answered from the cache
