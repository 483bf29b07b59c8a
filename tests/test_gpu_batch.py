"""Batched builds (one persistent launch per stage for many subsystems), CUDA-graph
replay, and the serving loop: every result is the same as the build run alone
(FP64 atomics reorder the Vxc sums only, so 1e-12 relative / 1e-13 Eh)."""
import numpy as np
import pytest

from serenity_gb300 import workload as wl

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from serenity_gb300 import xcgpu
    return xcgpu.Context()


def _workloads(func="PBE"):
    out = []
    for i, m in enumerate([2, 5, 3, 4, 1]):
        sym, xyz = wl.water_cluster(m, seed=50 + i, jitter=0.2)
        out.append(wl.Workload(sym, xyz, "DEF2-SVP", func if i % 2 == 0 else "LDA", 5 * m, 30, 110, 50 + i))
    return out


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_equals_single_builds(ctx, precision):
    from serenity_gb300.batch import SubsystemBatch
    ws = _workloads()
    b = SubsystemBatch(ctx, ws, precision=precision)
    b.run()
    res = b.results()
    for (plan, func, P, V, en), w, (Vb, eb, nb) in zip(b.items, ws, res):
        Vs, es, ns = plan.vxc(func, np.asarray(w.density()), precision=precision)
        assert abs(eb - es) <= 1e-13 * max(1, abs(es))
        assert abs(nb - ns) <= 1e-13 * ns
        np.testing.assert_allclose(Vb, Vs, rtol=0, atol=1e-12 * max(1.0, np.abs(Vs).max()))


def test_graph_replay_and_loop(ctx):
    from serenity_gb300.batch import SubsystemBatch
    ws = _workloads()
    b = SubsystemBatch(ctx, ws)
    b.loop()
    ref = b.results()
    b.capture()
    for _ in range(2):
        b.replay()
    res = b.results()
    for (V0, e0, n0), (V1, e1, n1) in zip(ref, res):
        assert abs(e0 - e1) <= 1e-13 * max(1, abs(e0))
        np.testing.assert_allclose(V1, V0, rtol=0, atol=1e-12 * max(1.0, np.abs(V0).max()))
    b.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_requests_sharing_one_plan_in_a_batch(ctx, precision):
    """Several density matrices of one geometry in one batch (plans are read-only; each
    request's work buffers are its own slice of the stream's arena)."""
    import torch
    from serenity_gb300 import xcgpu
    sym, xyz = wl.water_cluster(3, seed=7, jitter=0.2)
    ws = [wl.Workload(sym, xyz, "DEF2-SVP", "PBE", 15, 30, 110, seed) for seed in (1, 2, 3)]
    grid = xcgpu.Grid.build(ctx, ws[0].Z, ws[0].coords, n_rad=30, n_ang=110)
    plan = xcgpu.Plan(ctx, grid, xcgpu.Basis(ctx, ws[0].shells), 128, 1e-9)
    items = []
    for w, func in zip(ws, ["PBE", "LDA", "PBE"]):
        P = torch.from_numpy(np.ascontiguousarray(np.asarray(w.density()).reshape(1, w.nbf, w.nbf))).cuda()
        items.append((plan, func, P, torch.empty_like(P), torch.empty(2, dtype=torch.float64, device="cuda")))
    ctx.vxc_batch(items, precision, sync=True)
    for (_, func, P, V, en), w in zip(items, ws):
        Vs, es, ns = plan.vxc(func, np.asarray(w.density()), precision=precision)
        e = en.cpu().numpy()
        assert abs(e[0] - es) <= 1e-13 * max(1, abs(es))
        assert abs(e[1] - ns) <= 1e-13 * ns
        np.testing.assert_allclose(V.cpu().numpy().reshape(Vs.shape), Vs, rtol=0, atol=1e-12 * max(1.0, np.abs(Vs).max()))


@pytest.mark.parametrize("precision", [0, 1])
def test_serving_results_same_alone_and_in_the_mix(ctx, precision):
    from serenity_gb300 import serve
    server = serve.Server(ctx, hbm_budget=8 << 30, precision=precision, max_batch=4, nstreams=2)
    reqs, _ = serve.make_requests(server, n=14, rate=2000.0, seed=3, max_waters=6, n_rad=30, n_ang=110)
    stats = server.run(reqs)
    assert stats["requests"] == 14 and stats["batches"] >= 2
    assert stats["residents_built_while_serving"] == 0
    for rq in reqs:
        rq_plan = server.cache[rq.key].plans[0]
        V_mix = rq.V_dev.cpu().numpy()
        e_mix = rq.en_dev.cpu().numpy()
        V_alone, e_alone, n_alone = rq_plan.vxc(rq.func, rq.P_dev, precision=precision,
                                                out=rq.V_dev.clone())
        assert abs(e_mix[0] - e_alone) <= 1e-12 * max(1, abs(e_alone))
        assert abs(e_mix[1] - n_alone) <= 1e-12 * n_alone
        np.testing.assert_allclose(V_mix, V_alone.cpu().numpy(), rtol=0, atol=1e-12 * max(1.0, np.abs(V_mix).max()))
