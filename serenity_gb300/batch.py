"""Many independent XC builds in one batched launch: the subsystem step of a
freeze-and-thaw / FDE cycle (FreezeAndThawTask.cpp:151-411 runs the subsystem Fock
builds one after another; here all of them run in one persistent launch per heavy
stage, captured once into a CUDA graph and replayed).

The block size of the plans (points per block: the M extent of the density tiles and
the K extent of the adder tiles) is chosen by ``autotune_block`` and cached on disk.
"""
import json
import math
import os
import time

import numpy as np

from . import workload as wl
from . import xcgpu


def cluster_sizes(n, lo, hi, seed):
    """n cluster sizes drawn log-uniformly from [lo, hi] (integers)."""
    rng = np.random.default_rng(seed)
    return [int(round(math.exp(x))) for x in rng.uniform(math.log(lo), math.log(hi), size=n)]


def subsystem_workloads(n=64, lo=3, hi=40, seed=0, basis="DEF2-SVP", func="PBE", n_rad=75, n_ang=302):
    """The batched subsystem workload: n water clusters of log-uniform size, each with
    its own Becke grid and random orthonormalised density matrix."""
    out = []
    for i, m in enumerate(cluster_sizes(n, lo, hi, seed)):
        sym, xyz = wl.water_cluster(m, seed=seed * 1000 + i, jitter=0.2)
        out.append(wl.Workload(sym, xyz, basis, func, 5 * m, n_rad, n_ang, seed * 1000 + i))
    return out


class SubsystemBatch:
    """Resident grids, bases, plans and density matrices for a list of workloads."""

    def __init__(self, ctx, workloads, precision=xcgpu.PREC_MIXED, max_block=128, grids=None):
        import torch
        self.ctx, self.precision, self.max_block = ctx, precision, max_block
        self.items = []
        self.grids = grids or [xcgpu.Grid.build(ctx, w.Z, w.coords, n_rad=w.n_rad, n_ang=w.n_ang) for w in workloads]
        for w, g in zip(workloads, self.grids):
            b = xcgpu.Basis(ctx, w.shells)
            plan = xcgpu.Plan(ctx, g, b, max_block, 1e-9)
            P = np.asarray(w.density())
            Pc = np.ascontiguousarray(np.stack([m.T for m in P.reshape(w.nspin, w.nbf, w.nbf)]))
            P_dev = torch.from_numpy(Pc).cuda()
            V_dev = torch.zeros_like(P_dev)
            en = torch.zeros(2, dtype=torch.float64, device="cuda")
            self.items.append((plan, w.func, P_dev, V_dev, en))
        self.workloads = workloads
        self.graph = None
        self.npoints = sum(g.n for g in self.grids)

    def run(self):
        self.ctx.vxc_batch(self.items, self.precision)

    def capture(self):
        """Warm up (allocates the work buffers), then capture one batched build."""
        self.run()
        self.ctx.check_async()
        self.ctx.graph_begin()
        self.run()
        self.graph = self.ctx.graph_end()
        return self.graph

    def replay(self):
        self.ctx.graph_launch(self.graph)

    def loop(self):
        """The per-cluster loop: one build call per subsystem."""
        for plan, func, P, V, en in self.items:
            self.ctx.vxc_batch([(plan, func, P, V, en)], self.precision)

    def results(self):
        self.ctx.check_async()
        out = []
        for (plan, func, P, V, en), w in zip(self.items, self.workloads):
            Vh = V.cpu().numpy().reshape(w.nspin, w.nbf, w.nbf).transpose(0, 2, 1)
            e = en.cpu().numpy()
            out.append((Vh, float(e[0]), float(e[1])))
        return out

    def close(self):
        if self.graph is not None:
            self.ctx.graph_destroy(self.graph)
            self.graph = None


def _time(fn, ctx, reps=3):
    import torch
    fn()
    ctx.check_async()
    best = 1e30
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fn()
        ctx.check_async()
        best = min(best, time.perf_counter() - t0)
    return best


CACHE = os.path.join(os.path.expanduser("~"), ".cache", "serenity_gb300_autotune.json")


def autotune_block(ctx, workloads, precision=xcgpu.PREC_MIXED, candidates=(64, 96, 128), cache_path=None):
    """Pick the plan block size (points per block) with the fastest graph replay for
    this batch; the choice is cached per (basis, functional, precision, size bucket)."""
    cache_path = cache_path or CACHE
    key = "%s/%s/%d/%d" % (workloads[0].basis_name, workloads[0].func, precision,
                           int(math.log2(max(1, sum(len(w.Z) for w in workloads)))))
    try:
        with open(cache_path) as f:
            cache = json.load(f)
    except (OSError, ValueError):
        cache = {}
    if key in cache:
        return cache[key], {}
    grids = [xcgpu.Grid.build(ctx, w.Z, w.coords, n_rad=w.n_rad, n_ang=w.n_ang) for w in workloads]
    timings = {}
    for mb in candidates:
        b = SubsystemBatch(ctx, workloads, precision, mb, grids=grids)
        b.capture()
        timings[mb] = _time(b.replay, ctx)
        b.close()
    best = min(timings, key=timings.get)
    cache[key] = best
    try:  # written whole and renamed, so a concurrent reader never sees a partial file
        os.makedirs(os.path.dirname(cache_path), exist_ok=True)
        tmp = "%s.%d.tmp" % (cache_path, os.getpid())
        with open(tmp, "w") as f:
            json.dump(cache, f)
        os.replace(tmp, cache_path)
    except OSError:
        pass
    return best, timings
