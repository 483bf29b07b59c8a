"""Host logic of the serving loop (serenity_gb300/serve.py) on the CPU: admission of waiting
requests into batches under the HBM budget, the batch cap and the work cap, continuous
batching over two streams, LRU eviction that never drops a geometry with requests in
flight (and whose evicted geometries still serve later requests; a grid goes with the last
resident that uses it), rejection beyond a
latency budget, and the bookkeeping of reserved bytes and latencies.  The GPU pieces (streams, events, the library's
batched build, the request's density matrix) are replaced by fakes that record what the loop
asks of them; the builds themselves are covered by tests/test_gpu_batch.py."""
import sys
import types

import numpy as np
import pytest

from serenity_gb300 import serve


class FakeEvent:
    def __init__(self, polls):
        self.polls = polls  # queries answered "not yet" before the work counts as done

    def record(self, stream):
        pass

    def query(self):
        self.polls -= 1
        return self.polls < 0


class FakeStream:
    n = 0

    def __init__(self):
        FakeStream.n += 1
        self.cuda_stream = FakeStream.n

    def wait_event(self, ev):
        pass


class FakeCtxManager:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


def fake_torch(polls):
    cuda = types.SimpleNamespace(Stream=FakeStream, Event=lambda: FakeEvent(polls),
                                 stream=lambda s: FakeCtxManager())
    return types.SimpleNamespace(cuda=cuda, float64="float64", empty_like=lambda x: object(),
                                 empty=lambda *a, **k: object())


class FakePlan:
    def __init__(self, npoints, nblocks):
        self.st = {"npoints": npoints, "nblocks": nblocks, "flops_per_spin": 1000.0}

    def stats(self):
        return dict(self.st)


class FakeCtx:
    def __init__(self):
        self.bytes_in_use = 0
        self.batches = []
        self.stream = None

    def set_stream(self, s):
        self.stream = s

    def vxc_batch(self, items, precision):
        self.batches.append((self.stream, [it[0] for it in items]))

    def check_async(self):
        pass


def fake_xcgpu(npoints, nblocks):
    class Grid:
        @staticmethod
        def build(ctx, Z, coords, n_rad=0, n_ang=0):
            ctx.bytes_in_use += 1000
            return object()

    def Basis(ctx, shells):
        return object()

    def Plan(ctx, grid, basis, block, thr):
        ctx.bytes_in_use += 500
        return FakePlan(npoints, nblocks)

    return types.SimpleNamespace(Grid=Grid, Basis=Basis, Plan=Plan, PREC_MIXED=1, PREC_FP64=0)


def workload(nbf=24):
    return types.SimpleNamespace(nbf=nbf, nspin=1, nocc=5, Z=[8, 1, 1], coords=np.zeros((3, 3)), n_rad=10, n_ang=14,
                                 shells=None)


@pytest.fixture
def make_server(monkeypatch):
    def make(budget, max_batch=64, polls=1, npoints=1000, nblocks=8, **kw):
        monkeypatch.setitem(sys.modules, "torch", fake_torch(polls))
        monkeypatch.setattr(serve, "xcgpu", fake_xcgpu(npoints, nblocks))
        def density(S, nocc, seed):
            assert S is not None  # every arriving request finds its geometry's overlap
            return object()
        monkeypatch.setattr(serve, "density_on_gpu", density)
        monkeypatch.setattr(serve, "overlap_on_gpu", lambda ctx, r: ("S", id(r)))
        ctx = FakeCtx()
        return serve.Server(ctx, budget, precision=1, max_batch=max_batch, nstreams=2, **kw), ctx
    return make


def _requests(n, ngeom):
    return [serve.Request(i, 0.0, (i % ngeom, "SVP"), workload(), "PBE", i) for i in range(n)]


def _work(npoints=1000, nblocks=8, nbf=24):
    return serve._work_bytes(npoints, nbf, 1, True, nblocks)


def test_all_requests_served_and_reservations_returned(make_server):
    srv, ctx = make_server(budget=10 ** 9)
    reqs = _requests(20, 4)
    stats = srv.run(reqs)
    assert stats["requests"] == 20
    assert all(r.latency is not None and r.latency >= 0 for r in reqs)
    assert srv.reserved == 0 and not srv.inflight
    assert sum(len(p) for _, p in ctx.batches) == 20
    assert len(ctx.batches[0][1]) == 20  # all waiting requests fit the first batch
    assert stats["resident_geometries"] == 4  # one resident per (geometry, basis), reused
    assert all(r.busy == 0 for r in srv.cache.values())


def test_batch_cap_and_alternating_streams(make_server):
    srv, ctx = make_server(budget=10 ** 9, max_batch=3, polls=2)
    srv.run(_requests(10, 2))
    sizes = [len(p) for _, p in ctx.batches]
    assert max(sizes) <= 3 and sum(sizes) == 10
    streams = [s for s, _ in ctx.batches]
    assert all(a != b for a, b in zip(streams, streams[1:]))  # batches alternate over the two streams


def test_budget_limits_batch_size(make_server):
    one = _work()
    # room for the residents plus the work of two requests at a time
    srv, ctx = make_server(budget=2 * 1000 + 2 * 500 + 2 * one + one // 2)
    srv.run(_requests(9, 2))
    sizes = [len(p) for _, p in ctx.batches]
    assert sum(sizes) == 9
    assert sizes[0] == 2 and max(sizes) <= 2  # the third request of a batch would exceed the budget
    assert srv.reserved == 0


def test_a_request_larger_than_the_budget_still_runs_alone(make_server):
    srv, ctx = make_server(budget=10)  # smaller than any request: admitted one at a time
    srv.run(_requests(3, 1))
    assert [len(p) for _, p in ctx.batches] == [1, 1, 1]


def test_eviction_spares_geometries_with_requests_in_flight(make_server):
    srv, ctx = make_server(budget=10 ** 9)
    w = workload()
    a = srv.resident((0, "SVP"), w)
    b = srv.resident((1, "SVP"), w)
    a.plan()  # a request on geometry 0 is in flight
    srv.budget = 0  # everything must go that can
    srv._evict()
    assert (0, "SVP") in srv.cache and (1, "SVP") not in srv.cache
    a.release(0)
    srv._evict()
    assert not srv.cache


def test_eviction_drops_a_grid_with_its_last_resident(make_server):
    srv, ctx = make_server(budget=10 ** 9)
    w = workload()
    srv.resident((0, "SVP"), w)
    srv.resident((0, "TZVP"), w)  # the same geometry in a second basis shares the grid
    srv.resident((1, "SVP"), w).plan()  # in flight: stays, and so does its grid
    assert srv.cache[(0, "SVP")].grid is srv.cache[(0, "TZVP")].grid
    srv.budget = 0
    srv._evict()
    assert list(srv.cache) == [(1, "SVP")]
    assert 0 not in srv.grids and 1 in srv.grids
    r = srv.resident((0, "SVP"), w)  # a later request rebuilds the geometry's grid
    assert 0 in srv.grids and r.grid is srv.grids[0]


def test_work_bytes_grow_with_points_functions_and_spins():
    base = serve._work_bytes(1000, 24, 1, True, 8)
    assert serve._work_bytes(2000, 24, 1, True, 8) > base
    assert serve._work_bytes(1000, 48, 1, True, 8) > base
    assert serve._work_bytes(1000, 24, 2, True, 8) > base
    assert serve._work_bytes(1000, 24, 1, False, 8) < base


def test_evicted_geometry_serves_later_requests(make_server):
    srv, ctx = make_server(budget=10 ** 9)
    srv.run(_requests(2, 1))
    srv.budget = 0
    srv._evict()  # the geometry's resident data goes, its overlap stays
    assert not srv.cache and (0, "SVP") in srv.overlaps
    srv.budget = 10 ** 9
    later = [serve.Request(5, 0.0, (0, "SVP"), workload(), "PBE", 5)]
    stats = srv.run(later)
    assert stats["served"] == 1 and later[0].latency is not None


def test_work_cap_splits_batches(make_server):
    srv, ctx = make_server(budget=10 ** 9, max_batch_flops=2500.0)  # each request: 1000 flops
    srv.run(_requests(7, 2))
    sizes = [len(p) for _, p in ctx.batches]
    assert sum(sizes) == 7 and max(sizes) <= 2


def test_latency_budget_rejects_beyond_the_predicted_wait(make_server):
    srv, ctx = make_server(budget=10 ** 9, latency_budget_s=2.5e-3)
    srv.rate_flops = 1e6  # measured service rate: each request (1000 flops) takes 1 ms
    reqs = _requests(6, 2)
    stats = srv.run(reqs)
    # arriving together, the first two fit the 2.5 ms budget and the rest would wait longer
    assert stats["served"] == 2 and stats["rejected"] == 4
    assert all((r.latency is None) == r.rejected for r in reqs)
    assert srv.queued_flops == 0 and srv.reserved == 0
