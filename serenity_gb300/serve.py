"""Request loop for Vxc builds with continuous batching under an HBM budget.

Requests (geometry, basis, functional, density matrix) arrive over time.  The loop
keeps grids, bases and plans resident across repeat geometries (an LRU cache counted
against the budget), admits waiting requests into the next batch as in-flight
batches retire and memory frees up, and runs each batch as one persistent launch per
heavy stage (``xcgpu_vxc_batch``).  Batches alternate between compute streams so the
next batch's kernels start on SMs the previous batch's tail leaves idle, and the
setup of new geometries (grid, screening) runs on its own stream while batches
compute.  Latency is measured from a request's arrival to the completion of its batch.

Under load two bounds keep latency from growing with the queue: a batch takes waiting
requests only up to a cap on its estimated work (the plans' contraction flops), so a
large build does not hold many small ones until it ends; and with a latency budget a
request whose predicted completion (the work queued ahead of it at the measured service
rate) lies beyond the budget is rejected on arrival instead of joining the queue.
"""
import collections
import math
import time

import numpy as np

from . import workload as wl
from . import xcgpu


class Request:
    """One Vxc request.  Its density matrix is the request payload: it is formed on the
    GPU when the request arrives (seeded), so that only requests in the system hold one."""
    __slots__ = ("rid", "arrival", "key", "workload", "P_dev", "V_dev", "en_dev", "func", "done", "latency",
                 "nbytes", "plan_slot", "exc", "nel", "seed", "ready", "flops", "rejected")

    def __init__(self, rid, arrival, key, workload, func, seed):
        self.rid, self.arrival, self.key, self.workload = rid, arrival, key, workload
        self.func, self.seed = func, seed
        self.P_dev = self.V_dev = self.en_dev = self.ready = None
        self.done = None
        self.latency = None
        self.exc = self.nel = None
        self.flops = 0.0
        self.rejected = False

    def fresh(self):
        """The same request, not yet served."""
        return Request(self.rid, self.arrival, self.key, self.workload, self.func, self.seed)


def _work_bytes(npts, nbf, nspin, gga, nblocks):
    per_point = 8 * (nspin * (1 + (3 if gga else 0)) * 2 + 1) + 32
    return npts * per_point + nspin * nbf * nbf * (8 + 8) + nblocks * 64


class Resident:
    """Grid, basis and plan of one geometry.  A build only reads its plan (its work
    buffers come from the stream's arena), so every request on the geometry, in one
    batch or in batches in flight together, shares the one plan."""

    def __init__(self, ctx, w, grid=None):
        self.grid = grid if grid is not None else xcgpu.Grid.build(ctx, w.Z, w.coords, n_rad=w.n_rad, n_ang=w.n_ang)
        self.basis = xcgpu.Basis(ctx, w.shells)
        self.plans = [xcgpu.Plan(ctx, self.grid, self.basis, 128, 1e-9)]
        self.busy = 0  # requests admitted and not yet retired
        self.ctx = ctx

    def plan(self):
        self.busy += 1
        return 0, self.plans[0]

    def release(self, i):
        self.busy -= 1


class Server:
    def __init__(self, ctx, hbm_budget, precision=xcgpu.PREC_MIXED, max_batch=64, nstreams=2, max_batch_flops=None,
                 latency_budget_s=None):
        import torch
        self.torch = torch
        self.ctx = ctx
        self.budget = hbm_budget
        self.precision = precision
        self.max_batch = max_batch
        self.streams = [torch.cuda.Stream() for _ in range(nstreams)]
        self.setup_stream = torch.cuda.Stream()
        self.cache = collections.OrderedDict()
        self.grids = {}  # geometry -> grid, shared by the bases of that geometry
        self.inflight = []
        self.reserved = 0
        self.residents_built = 0
        # overlap matrices (the request generator's metric) by geometry key: kept apart from
        # the evictable cache, so a request that arrives after its geometry was evicted still
        # finds it
        self.overlaps = {}
        self.max_batch_flops = max_batch_flops
        self.latency_budget_s = latency_budget_s
        self.queued_flops = 0.0  # estimated work admitted and not yet retired
        self.rate_flops = None  # measured service rate (flops/s), a running average

    # -- resident data --------------------------------------------------------------------
    def resident(self, key, w):
        r = self.cache.get(key)
        if r is None:
            self.ctx.set_stream(self.setup_stream.cuda_stream)
            gkey = key[0]
            if gkey not in self.grids:
                self.grids[gkey] = xcgpu.Grid.build(self.ctx, w.Z, w.coords, n_rad=w.n_rad, n_ang=w.n_ang)
            r = Resident(self.ctx, w, self.grids[gkey])
            self.cache[key] = r
            self.residents_built += 1
        self.cache.move_to_end(key)
        return r

    def overlap(self, key, w):
        """The geometry's overlap matrix on the GPU, from its resident plan on first use."""
        S = self.overlaps.get(key)
        if S is None:
            S = overlap_on_gpu(self.ctx, self.resident(key, w))
            self.overlaps[key] = S
        return S

    def _evict(self):
        """Drop least recently used residents that have no request in flight until the
        budget holds; a geometry's grid goes with the last resident that shares it."""
        while self.ctx.bytes_in_use + self.reserved > self.budget and self.cache:
            key, r = next(iter(self.cache.items()))
            if r.busy:
                self.cache.move_to_end(key)
                if all(x.busy for x in self.cache.values()):
                    return
                continue
            self.cache.pop(key)
            if not any(k[0] == key[0] for k in self.cache):
                self.grids.pop(key[0], None)

    # -- batches --------------------------------------------------------------------------
    def _arrive(self, rq):
        """Admit the request (or reject it if its predicted completion exceeds the latency
        budget) and form its density matrix on the setup stream (no host synchronisation).
        Returns False for a rejected request."""
        torch = self.torch
        r = self.resident(rq.key, rq.workload)
        rq.flops = _plan_flops(r.plans[0], rq.workload.nspin)
        if self.latency_budget_s is not None and self.rate_flops:
            if (self.queued_flops + rq.flops) / self.rate_flops > self.latency_budget_s:
                rq.rejected = True
                return False
        self.queued_flops += rq.flops
        S = self.overlap(rq.key, rq.workload)
        with torch.cuda.stream(self.setup_stream):
            rq.P_dev = density_on_gpu(S, rq.workload.nocc, rq.seed)
            rq.ready = torch.cuda.Event()
            rq.ready.record(self.setup_stream)
        return True

    def _launch(self, batch, stream):
        torch = self.torch
        items = []
        with torch.cuda.stream(stream):
            for rq in batch:
                stream.wait_event(rq.ready)
                w = rq.workload
                rq.V_dev = torch.empty_like(rq.P_dev)
                rq.en_dev = torch.empty(2, dtype=torch.float64, device="cuda")
                items.append((rq.plan_slot[1], rq.func, rq.P_dev, rq.V_dev, rq.en_dev))
        self.ctx.set_stream(stream.cuda_stream)
        self.ctx.vxc_batch(items, self.precision)
        ev = torch.cuda.Event()
        ev.record(stream)
        self.inflight.append((batch, ev, stream, time.perf_counter()))

    def _retire(self, now_fn, keep_results):
        keep = []
        for batch, ev, stream, t_launch in self.inflight:
            if ev.query():
                self.ctx.set_stream(stream.cuda_stream)
                self.ctx.check_async()
                t = now_fn()
                work = sum(rq.flops for rq in batch)
                self.queued_flops -= work
                dt = time.perf_counter() - t_launch
                if dt > 0 and work > 0:  # service rate, averaged over recent batches
                    r_ = work / dt
                    self.rate_flops = r_ if self.rate_flops is None else 0.8 * self.rate_flops + 0.2 * r_
                for rq in batch:
                    rq.done = t
                    rq.latency = t - rq.arrival
                    r, (i, _) = self.cache.get(rq.key), rq.plan_slot
                    if r is not None:
                        r.release(i)
                    self.reserved -= rq.nbytes
                    if not keep_results:
                        rq.P_dev = rq.V_dev = None
                yield batch
            else:
                keep.append((batch, ev, stream, t_launch))
        self.inflight = keep

    def run(self, requests, on_complete=None, keep_results=True):
        """Serve requests (sorted by arrival, seconds from start).  Returns stats.  With
        keep_results False a request's P and V are dropped when it completes (E_xc and
        N_el stay in en_dev)."""
        pending = collections.deque()
        todo = collections.deque(sorted(requests, key=lambda r: r.arrival))
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0  # noqa: E731
        built0 = self.residents_built
        sidx = 0
        completed = 0
        rejected = []
        while todo or pending or self.inflight:
            t = now()
            while todo and todo[0].arrival <= t:
                rq = todo.popleft()
                if self._arrive(rq):
                    pending.append(rq)
                else:
                    rejected.append(rq)
            for batch in self._retire(now, keep_results):
                completed += len(batch)
                if on_complete:
                    on_complete(batch)
            if pending and len(self.inflight) < len(self.streams):
                batch = []
                bflops = 0.0
                while pending and len(batch) < self.max_batch:
                    rq = pending[0]
                    if batch and self.max_batch_flops is not None and bflops + rq.flops > self.max_batch_flops:
                        break
                    w = rq.workload
                    r = self.resident(rq.key, w)
                    slot = r.plan()
                    st = slot[1].stats()
                    rq.nbytes = _work_bytes(st["npoints"], w.nbf, w.nspin, True, st["nblocks"])
                    self._evict()
                    if batch and self.ctx.bytes_in_use + self.reserved + rq.nbytes > self.budget:
                        r.release(slot[0])
                        break
                    rq.plan_slot = slot
                    self.reserved += rq.nbytes
                    bflops += rq.flops
                    batch.append(pending.popleft())
                if batch:
                    self._launch(batch, self.streams[sidx % len(self.streams)])
                    sidx += 1
                    continue
            if not self.inflight and todo and not pending:
                time.sleep(max(0.0, min(0.001, todo[0].arrival - now())))
            else:
                time.sleep(0.0002)
        total = now()
        served = [r for r in requests if r.latency is not None]
        lat = np.array([r.latency for r in served]) if served else np.zeros(1)
        return {"requests": len(requests), "served": len(served), "rejected": len(rejected), "wall_s": total,
                "throughput_req_s": len(served) / total,
                "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
                "mean_ms": float(lat.mean() * 1e3), "batches": sidx, "resident_geometries": len(self.cache),
                "residents_built_while_serving": self.residents_built - built0}


def density_on_gpu(S_dev, nocc, seed):
    """Random orthonormalised density on the GPU: P = 2 C (C^T S C)^-1 C^T for a seeded
    Gaussian C (the projector onto span C, the same P as Loewdin-orthonormalising C),
    symmetrised, returned in FP64 as [1, n, n].  This is synthetic request input, formed
    with FP32 GEMMs (the FP64 form cost a third of the serving run's GPU time); Cholesky
    without an info check keeps the host unsynchronised."""
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    n = S_dev.shape[0]
    S = S_dev.to(torch.float32)
    C = torch.randn(n, nocc, generator=g, device="cuda", dtype=torch.float32)
    L, _ = torch.linalg.cholesky_ex(C.T @ (S @ C))
    P = 2.0 * C @ torch.cholesky_solve(C.T.contiguous(), L)
    P = (0.5 * (P + P.T)).to(torch.float64)
    return P.contiguous().reshape(1, n, n)


def overlap_on_gpu(ctx, resident):
    """Overlap matrix of a resident geometry by grid integration (adder with v = 1)."""
    import torch
    S = resident.plans[0].add_scalar(np.ones(resident.grid.n), block_ave_threshold=0.0, precision=xcgpu.PREC_MIXED)[0]
    return torch.from_numpy(np.ascontiguousarray(S)).cuda()


def _plan_flops(plan, nspin):
    """Estimated work of a build on this plan: the contractions' flops (4 npts n_b^2 per
    block and spin)."""
    return float(plan.stats().get("flops_per_spin", 0.0)) * nspin


def make_requests(server, n=2000, rate=200.0, seed=0, max_waters=128, n_rad=50, n_ang=110, geometries=32):
    """Poisson stream: cluster sizes 1..max_waters log-uniform, def2-SVP / def2-TZVP 70/30,
    LDA / PBE 50/50, each request with its own random orthonormalised P (seeded; formed on
    arrival).  Requests draw their cluster from a pool of `geometries` clusters whose sizes
    are themselves drawn log-uniform, so geometries repeat and stay resident.  The pool is
    made resident here (grid, basis, plan, overlap for the P generator); returns
    (requests, setup seconds)."""
    rng = np.random.default_rng(seed)
    pool = [int(round(math.exp(rng.uniform(0.0, math.log(max_waters))))) for _ in range(geometries)]
    t = 0.0
    reqs = []
    t0 = time.perf_counter()
    for i in range(n):
        t += rng.exponential(1.0 / rate)
        m = pool[int(rng.integers(len(pool)))]
        basis = "DEF2-SVP" if rng.uniform() < 0.7 else "DEF2-TZVP"
        func = "LDA" if rng.uniform() < 0.5 else "PBE"
        key = (m, basis)
        sym, xyz = wl.water_cluster(m, seed=1000 + m, jitter=0.2)
        w = wl.Workload(sym, xyz, basis, func, 5 * m, n_rad, n_ang, seed)
        server.overlap(key, w)
        reqs.append(Request(i, t, key, w, func, seed * 100000 + i))
    server.ctx.set_stream(server.streams[0].cuda_stream)
    return reqs, time.perf_counter() - t0
