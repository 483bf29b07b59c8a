"""Python binding of the xcgpu C ABI (``include/xcgpu.h``) through ctypes.

The GPU library is the only implementation: if ``libxcgpu.so`` cannot be loaded,
or no CUDA device is present, every constructor raises.  There is no CPU
fallback.  Array arguments are numpy arrays (host memory, ``XCGPU_MEM_HOST``) or
any object exposing ``data_ptr()`` on the GPU (``XCGPU_MEM_DEVICE``, e.g. a torch
CUDA tensor).
"""
import ctypes
import os

import numpy as np

from . import build as _build

MEM_HOST, MEM_DEVICE = 0, 1
PREC_FP64, PREC_MIXED = 0, 1
FUNC = {"LDA": 1, "PBE": 2, "BLYP": 3, "BP86": 4, "SLATER": 16, "VWN5": 17, "PBEX": 18, "PBEC": 19, "B88": 20,
        "LYP": 21, "PW92": 22, "P86": 23, "PZ81": 24}
STATUS = {0: "OK", 1: "INVALID", 2: "CUDA", 3: "NO_MEMORY", 4: "BUDGET", 5: "UNSUPPORTED", 6: "TIMEOUT", 7: "IO"}


class XcgpuError(RuntimeError):
    """Raised for a non-OK status (the reference throws SerenityError at this boundary)."""

    def __init__(self, status, message):
        super().__init__("xcgpu %s: %s" % (STATUS.get(status, status), message))
        self.status = status


class Config(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("hbm_budget", ctypes.c_uint64), ("scratch_bytes", ctypes.c_uint64)]


class Shell(ctypes.Structure):
    _fields_ = [("l", ctypes.c_int32), ("pure", ctypes.c_int32), ("nprim", ctypes.c_int32),
                ("center", ctypes.c_double * 3), ("alpha", ctypes.POINTER(ctypes.c_double)),
                ("coef", ctypes.POINTER(ctypes.c_double))]


class Request(ctypes.Structure):
    _fields_ = [("plan", ctypes.c_void_p), ("func", ctypes.c_int), ("nspin", ctypes.c_int),
                ("block_ave_threshold", ctypes.c_double), ("P", ctypes.c_void_p), ("V", ctypes.c_void_p),
                ("exc_nel", ctypes.c_void_p)]


class PlanStats(ctypes.Structure):
    _fields_ = [("nblocks", ctypes.c_uint32), ("max_block", ctypes.c_uint32), ("nbf", ctypes.c_uint32),
                ("max_active", ctypes.c_uint32), ("npoints", ctypes.c_uint64), ("sum_active", ctypes.c_uint64),
                ("flops_per_spin", ctypes.c_double)]


_lib = None
vp = ctypes.c_void_p
dp = ctypes.POINTER(ctypes.c_double)


def library(build_if_needed=True):
    """Load libxcgpu.so (building it first if it is missing or stale)."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_needed:
        _build.build()
    if not os.path.exists(_build.LIB):
        raise XcgpuError(2, "libxcgpu.so not built (%s)" % _build.LIB)
    L = ctypes.CDLL(_build.LIB)
    S = ctypes.c_int
    L.xcgpu_ctx_create.argtypes = [ctypes.POINTER(Config), ctypes.POINTER(vp)]
    L.xcgpu_ctx_destroy.argtypes = [vp]
    L.xcgpu_last_error.argtypes = [vp]
    L.xcgpu_last_error.restype = ctypes.c_char_p
    L.xcgpu_set_stream.argtypes = [vp, vp]
    L.xcgpu_synchronize.argtypes = [vp]
    L.xcgpu_bytes_in_use.argtypes = [vp]
    L.xcgpu_bytes_in_use.restype = ctypes.c_uint64
    L.xcgpu_kernel_launches.argtypes = [vp]
    L.xcgpu_kernel_launches.restype = ctypes.c_uint64
    L.xcgpu_grid_create.argtypes = [vp, vp, vp, ctypes.c_uint64, ctypes.POINTER(vp)]
    L.xcgpu_grid_build.argtypes = [vp, S, vp, vp, S, S, S, ctypes.c_double, S, S, ctypes.c_char_p, ctypes.POINTER(vp)]
    L.xcgpu_grid_build_partition.argtypes = [vp, S, vp, vp, S, S, S, ctypes.c_double, S, S, S, ctypes.c_char_p,
                                             ctypes.POINTER(vp)]
    L.xcgpu_grid_npoints.argtypes = [vp]
    L.xcgpu_grid_npoints.restype = ctypes.c_uint64
    L.xcgpu_grid_copy.argtypes = [vp, vp, vp]
    L.xcgpu_grid_destroy.argtypes = [vp]
    L.xcgpu_basis_create.argtypes = [vp, ctypes.POINTER(Shell), ctypes.c_uint32, ctypes.POINTER(vp)]
    L.xcgpu_basis_nbf.argtypes = [vp]
    L.xcgpu_basis_nbf.restype = ctypes.c_uint32
    L.xcgpu_basis_coefs.argtypes = [vp, ctypes.c_uint32, vp]
    L.xcgpu_basis_destroy.argtypes = [vp]
    L.xcgpu_plan_create.argtypes = [vp, vp, vp, ctypes.c_uint32, ctypes.c_double, ctypes.POINTER(vp)]
    L.xcgpu_plan_get_stats.argtypes = [vp, ctypes.POINTER(PlanStats)]
    L.xcgpu_block_on_grid.argtypes = [vp, ctypes.c_uint32, S, vp, vp, vp, vp]
    L.xcgpu_block_active.argtypes = [vp, ctypes.c_uint32, vp]
    L.xcgpu_block_active.restype = ctypes.c_int32
    L.xcgpu_plan_destroy.argtypes = [vp]
    L.xcgpu_density.argtypes = [vp, S, vp, vp, vp, S, S]
    L.xcgpu_functional.argtypes = [vp, S, S, ctypes.c_uint64, ctypes.c_uint32, vp, vp, vp, vp, vp, S]
    L.xcgpu_functional_prec.argtypes = [vp, S, S, ctypes.c_uint64, ctypes.c_uint32, vp, vp, vp, vp, vp, S, S]
    L.xcgpu_functional_is_gga.argtypes = [S]
    L.xcgpu_add_scalar.argtypes = [vp, ctypes.c_double, S, vp, vp, vp, S, S]
    L.xcgpu_vxc.argtypes = [vp, S, S, S, ctypes.c_double, vp, vp, dp, dp, S]
    L.xcgpu_vxc_batch.argtypes = [vp, ctypes.POINTER(Request), ctypes.c_uint32, S, S]
    L.xcgpu_nadd_vxc.argtypes = [vp, ctypes.POINTER(vp), ctypes.c_uint32, S, S, S, ctypes.c_double, vp,
                                 ctypes.POINTER(vp), vp, dp, S]
    L.xcgpu_xc_gradient.argtypes = [vp, S, S, vp, vp, S, vp, S]
    L.xcgpu_lr_kernel.argtypes = [vp, S, vp, ctypes.c_uint32, ctypes.POINTER(vp), ctypes.POINTER(vp), S,
                                  ctypes.c_double, S]
    L.xcgpu_lr_kernel_spin.argtypes = [vp, S, S, vp, ctypes.c_uint32, ctypes.POINTER(vp), ctypes.POINTER(vp), S,
                                       ctypes.c_double, S]
    L.xcgpu_nadd_vxc_all.argtypes = [ctypes.POINTER(vp), ctypes.c_uint32, S, S, S, ctypes.c_double,
                                     ctypes.POINTER(vp), ctypes.POINTER(vp), dp, S]
    L.xcgpu_check_async.argtypes = [vp]
    L.xcgpu_graph_begin.argtypes = [vp]
    L.xcgpu_graph_end.argtypes = [vp, ctypes.POINTER(vp)]
    L.xcgpu_graph_launch.argtypes = [vp, vp]
    L.xcgpu_graph_destroy.argtypes = [vp]
    L.xcgpu_set_timing.argtypes = [vp, S]
    L.xcgpu_get_timing.argtypes = [vp, vp, vp]
    for name in ["xcgpu_vxc_batch", "xcgpu_nadd_vxc", "xcgpu_nadd_vxc_all", "xcgpu_xc_gradient", "xcgpu_lr_kernel", "xcgpu_lr_kernel_spin", "xcgpu_check_async", "xcgpu_graph_begin", "xcgpu_graph_end",
                 "xcgpu_graph_launch", "xcgpu_set_timing", "xcgpu_get_timing"]:
        getattr(L, name).restype = S
    for name in ["xcgpu_ctx_create", "xcgpu_set_stream", "xcgpu_synchronize", "xcgpu_grid_create", "xcgpu_grid_build",
                 "xcgpu_grid_build_partition", "xcgpu_grid_copy", "xcgpu_basis_create", "xcgpu_basis_coefs", "xcgpu_plan_create",
                 "xcgpu_plan_get_stats", "xcgpu_block_on_grid", "xcgpu_density", "xcgpu_functional", "xcgpu_functional_prec",
                 "xcgpu_add_scalar", "xcgpu_vxc"]:
        getattr(L, name).restype = S
    _lib = L
    return L


def _ptr(a):
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return ctypes.c_void_p(a.data_ptr())
    return a.ctypes.data_as(ctypes.c_void_p)


def _mem(a):
    return MEM_DEVICE if hasattr(a, "data_ptr") else MEM_HOST


def _f64(a):
    if hasattr(a, "data_ptr"):
        return a
    return np.ascontiguousarray(a, dtype=np.float64)


class Context:
    """One GPU, one stream, an HBM budget (bytes; 0 = 90% of free memory)."""

    def __init__(self, device=0, hbm_budget=0, scratch_bytes=0):
        L = library()
        h = vp()
        cfg = Config(device, hbm_budget, scratch_bytes)
        st = L.xcgpu_ctx_create(ctypes.byref(cfg), ctypes.byref(h))
        if st != 0:
            raise XcgpuError(st, "cannot create a context on CUDA device %d (is a GPU present?)" % device)
        self.h = h
        self.L = L

    def check(self, st):
        if st != 0:
            raise XcgpuError(st, self.L.xcgpu_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.L.xcgpu_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_ptr):
        self.check(self.L.xcgpu_set_stream(self.h, ctypes.c_void_p(stream_ptr)))

    def synchronize(self):
        self.check(self.L.xcgpu_synchronize(self.h))

    @property
    def bytes_in_use(self):
        return int(self.L.xcgpu_bytes_in_use(self.h))

    @property
    def kernel_launches(self):
        return int(self.L.xcgpu_kernel_launches(self.h))

    def vxc_batch(self, items, precision=PREC_MIXED, sync=False):
        """items: list of (plan, func, P_dev, V_dev, exc_nel_dev) with device tensors
        (P, V column-major per spin); all builds run in one persistent launch per stage."""
        arr = (Request * len(items))()
        for i, (plan, func, P, V, en) in enumerate(items):
            nspin = P.numel() // (plan.nbf * plan.nbf)
            arr[i] = Request(plan.h.value if isinstance(plan.h, ctypes.c_void_p) else plan.h,
                             FUNC[func] if isinstance(func, str) else int(func), nspin, 1e-11,
                             P.data_ptr(), V.data_ptr(), en.data_ptr())
        self.check(self.L.xcgpu_vxc_batch(self.h, arr, len(items), precision, 1 if sync else 0))

    def check_async(self):
        self.check(self.L.xcgpu_check_async(self.h))

    def graph_begin(self):
        self.check(self.L.xcgpu_graph_begin(self.h))

    def graph_end(self):
        g = vp()
        self.check(self.L.xcgpu_graph_end(self.h, ctypes.byref(g)))
        return g

    def graph_launch(self, g):
        self.check(self.L.xcgpu_graph_launch(self.h, g))

    def graph_destroy(self, g):
        self.L.xcgpu_graph_destroy(g)

    def functional(self, func, rho, grad=None, skip_block=128, precision=PREC_FP64):
        """FunctionalLibrary::calcData(GRADIENTS, ., order 1) on host arrays
        rho [nspin, n], grad [nspin, 3, n] -> (epuv, dfdrho, dfdgrad); precision
        PREC_MIXED evaluates as the mixed build does (restricted PBE in FP32 pairs)."""
        fid = FUNC[func] if isinstance(func, str) else int(func)
        rho = _f64(rho)
        nspin, n = rho.shape
        gga = bool(self.L.xcgpu_functional_is_gga(fid))
        g = _f64(grad) if gga else None
        epuv = np.zeros(n)
        dr = np.zeros((nspin, n))
        dg = np.zeros((nspin, 3, n)) if gga else None
        self.check(self.L.xcgpu_functional_prec(self.h, fid, nspin, n, skip_block, _ptr(rho), _ptr(g), _ptr(epuv),
                                                _ptr(dr), _ptr(dg), precision, MEM_HOST))
        return epuv, dr, dg


def nadd_vxc_all(subsystems, func, precision=PREC_FP64, block_ave_threshold=1e-11):
    """Every subsystem's non-additive XC potential from one set of densities on a shared
    (supersystem) grid: subsystems = [(plan, P), ...] with host P [nbf,nbf] or
    [nspin,nbf,nbf].  Returns ([V_i [nspin, nbf_i, nbf_i]], E_nadd)."""
    if not subsystems:
        raise ValueError("nadd_vxc_all: no subsystems")
    ctx = subsystems[0][0].ctx
    fid = FUNC[func] if isinstance(func, str) else int(func)
    P0 = np.asarray(subsystems[0][1], dtype=np.float64)
    nspin = 1 if P0.ndim == 2 else P0.shape[0]
    Ps, Vs = [], []
    for plan, P in subsystems:
        M = np.asarray(P, dtype=np.float64).reshape(nspin, plan.nbf, plan.nbf)
        Ps.append(np.ascontiguousarray(np.stack([m.T for m in M])))
        Vs.append(np.zeros((nspin, plan.nbf, plan.nbf)))
    k = len(subsystems)
    plans = (vp * k)(*[pl.h for pl, _ in subsystems])
    pp = (vp * k)(*[x.ctypes.data for x in Ps])
    vv = (vp * k)(*[x.ctypes.data for x in Vs])
    e = ctypes.c_double()
    ctx.check(ctx.L.xcgpu_nadd_vxc_all(plans, k, fid, nspin, precision, block_ave_threshold, pp, vv, ctypes.byref(e),
                                       MEM_HOST))
    return [V.transpose(0, 2, 1) for V in Vs], e.value


PARTITION = {"becke": 0, "ssf": 1}


class Grid:
    def __init__(self, ctx, xyz=None, w=None, handle=None):
        self.ctx = ctx
        if handle is None:
            xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1)
            w = np.ascontiguousarray(w, dtype=np.float64)
            h = vp()
            ctx.check(ctx.L.xcgpu_grid_create(ctx.h, _ptr(xyz), _ptr(w), w.size, ctypes.byref(h)))
            handle = h
        self.h = handle
        self.n = int(ctx.L.xcgpu_grid_npoints(self.h))

    @staticmethod
    def build(ctx, Z, xyz_bohr, n_rad=0, n_ang=0, accuracy=0, weight_threshold=1e-14, smoothing=3, sort=True,
              lebedev_table=None, partition="becke"):
        """Atom-centred grid; partition "becke" or "ssf" (the reference's GRIDTYPE)."""
        from .basis import LEBEDEV_TABLE
        Z = np.ascontiguousarray(Z, dtype=np.int32)
        xyz = np.ascontiguousarray(xyz_bohr, dtype=np.float64).reshape(-1)
        h = vp()
        ctx.check(ctx.L.xcgpu_grid_build_partition(ctx.h, len(Z), _ptr(Z), _ptr(xyz), n_rad, n_ang, accuracy,
                                                   weight_threshold, PARTITION[partition], smoothing, int(sort),
                                                   (lebedev_table or LEBEDEV_TABLE).encode(), ctypes.byref(h)))
        return Grid(ctx, handle=h)

    def points(self):
        xyz = np.zeros(3 * self.n)
        w = np.zeros(self.n)
        self.ctx.check(self.ctx.L.xcgpu_grid_copy(self.h, _ptr(xyz), _ptr(w)))
        return xyz.reshape(-1, 3), w

    def __del__(self):
        if getattr(self, "h", None) and self.ctx.h:
            self.ctx.L.xcgpu_grid_destroy(self.h)
            self.h = None


class Basis:
    def __init__(self, ctx, shells):
        self.ctx = ctx
        self.shells = shells
        arr = (Shell * shells.nshell)()
        self._keep = []
        off = 0
        for i in range(shells.nshell):
            n = int(shells.nprim[i])
            a = np.ascontiguousarray(shells.alpha[off:off + n])
            c = np.ascontiguousarray(shells.coef[off:off + n])
            self._keep += [a, c]
            arr[i].l = int(shells.l[i])
            arr[i].pure = int(shells.pure[i])
            arr[i].nprim = n
            for k in range(3):
                arr[i].center[k] = float(shells.centers[3 * i + k])
            arr[i].alpha = a.ctypes.data_as(dp)
            arr[i].coef = c.ctypes.data_as(dp)
            off += n
        h = vp()
        ctx.check(ctx.L.xcgpu_basis_create(ctx.h, arr, shells.nshell, ctypes.byref(h)))
        self.h = h
        self.nbf = int(ctx.L.xcgpu_basis_nbf(h))

    def coefs(self, s):
        out = np.zeros(int(self.shells.nprim[s]))
        self.ctx.check(self.ctx.L.xcgpu_basis_coefs(self.h, s, _ptr(out)))
        return out

    def __del__(self):
        if getattr(self, "h", None) and self.ctx.h:
            self.ctx.L.xcgpu_basis_destroy(self.h)
            self.h = None


class Plan:
    """BasisFunctionOnGridController: blocks of max_block points, per-block screening."""

    def __init__(self, ctx, grid, basis, max_block=128, radial_threshold=1e-9):
        self.ctx, self.grid, self.basis = ctx, grid, basis
        h = vp()
        ctx.check(ctx.L.xcgpu_plan_create(ctx.h, grid.h, basis.h, max_block, radial_threshold, ctypes.byref(h)))
        self.h = h
        self.max_block = max_block
        self.nbf = basis.nbf

    def stats(self):
        s = PlanStats()
        self.ctx.check(self.ctx.L.xcgpu_plan_get_stats(self.h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in PlanStats._fields_}

    def block_on_grid(self, block, deriv=1):
        n = min(self.max_block, self.grid.n - block * self.max_block)
        v = np.zeros(n * self.nbf)
        g = np.zeros(3 * n * self.nbf) if deriv >= 1 else None
        hh = np.zeros(6 * n * self.nbf) if deriv >= 2 else None
        neg = np.zeros(self.nbf, dtype=np.int32)
        self.ctx.check(self.ctx.L.xcgpu_block_on_grid(self.h, block, deriv, _ptr(v), _ptr(g), _ptr(hh), _ptr(neg)))
        out = {"values": v.reshape(self.nbf, n).T, "negligible": neg}
        if deriv >= 1:
            out["grad"] = g.reshape(3, self.nbf, n).transpose(0, 2, 1)
        if deriv >= 2:
            out["hess"] = hh.reshape(6, self.nbf, n).transpose(0, 2, 1)
        return out

    def active(self, block):
        n = self.ctx.L.xcgpu_block_active(self.h, block, None)
        idx = np.zeros(max(n, 1), dtype=np.int32)
        self.ctx.L.xcgpu_block_active(self.h, block, _ptr(idx))
        return idx[:n]

    def density(self, P, grad=True, precision=PREC_FP64):
        """rho [nspin, n], grad [nspin, 3, n] for P [nbf, nbf] or [nspin, nbf, nbf] (symmetric)."""
        P = np.asarray(P, dtype=np.float64)
        nspin = 1 if P.ndim == 2 else P.shape[0]
        Pc = np.ascontiguousarray(np.stack([m.T for m in P.reshape(nspin, self.nbf, self.nbf)]))
        rho = np.zeros((nspin, self.grid.n))
        g = np.zeros((nspin, 3, self.grid.n)) if grad else None
        self.ctx.check(self.ctx.L.xcgpu_density(self.h, nspin, _ptr(Pc), _ptr(rho), _ptr(g), precision, MEM_HOST))
        return rho, g

    def add_scalar(self, v, g=None, F=None, block_ave_threshold=1e-11, precision=PREC_FP64):
        v = np.ascontiguousarray(v, dtype=np.float64).reshape(-1)
        nspin = v.size // self.grid.n
        gg = None if g is None else np.ascontiguousarray(g, dtype=np.float64).reshape(-1)
        Fc = np.zeros((nspin, self.nbf, self.nbf)) if F is None else np.ascontiguousarray(
            np.stack([m.T for m in np.asarray(F, dtype=np.float64).reshape(nspin, self.nbf, self.nbf)]))
        self.ctx.check(self.ctx.L.xcgpu_add_scalar(self.h, block_ave_threshold, nspin, _ptr(v), _ptr(gg), _ptr(Fc),
                                                   precision, MEM_HOST))
        return Fc.transpose(0, 2, 1)

    def vxc(self, func, P, precision=PREC_FP64, block_ave_threshold=1e-11, out=None):
        """Whole build; P host array [nbf,nbf] / [nspin,nbf,nbf] or a device tensor
        (column-major per spin).  Returns (V, Exc, Nel)."""
        fid = FUNC[func] if isinstance(func, str) else int(func)
        exc, nel = ctypes.c_double(), ctypes.c_double()
        if hasattr(P, "data_ptr"):
            nspin = P.numel() // (self.nbf * self.nbf)
            V = out
            self.ctx.check(self.ctx.L.xcgpu_vxc(self.h, fid, nspin, precision, block_ave_threshold, _ptr(P), _ptr(V),
                                                ctypes.byref(exc), ctypes.byref(nel), MEM_DEVICE))
            return V, exc.value, nel.value
        P = np.asarray(P, dtype=np.float64)
        nspin = 1 if P.ndim == 2 else P.shape[0]
        Pc = np.ascontiguousarray(np.stack([m.T for m in P.reshape(nspin, self.nbf, self.nbf)]))
        V = np.zeros((nspin, self.nbf, self.nbf))
        self.ctx.check(self.ctx.L.xcgpu_vxc(self.h, fid, nspin, precision, block_ave_threshold, _ptr(Pc), _ptr(V),
                                            ctypes.byref(exc), ctypes.byref(nel), MEM_HOST))
        return V.transpose(0, 2, 1), exc.value, nel.value

    def lr_kernel(self, func, P0, trials, precision=PREC_FP64, block_ave_threshold=1e-11, kind="singlet"):
        """XC kernel part of linear-response sigma vectors (KernelSigmavector::calcF): for
        each trial matrix the matrix F.  kind "singlet" or "triplet": P0 the restricted
        ground-state total density, trials and results [nbf, nbf]; "unrestricted": P0 and
        each trial [2, nbf, nbf] (alpha, beta), results [2, nbf, nbf]."""
        fid = FUNC[func] if isinstance(func, str) else int(func)
        ns = 2 if kind == "unrestricted" else 1
        colmajor = lambda M: np.ascontiguousarray(np.stack(  # noqa: E731
            [m.T for m in np.asarray(M, dtype=np.float64).reshape(ns, self.nbf, self.nbf)]))
        P0c = colmajor(P0)
        Ds = [colmajor(D) for D in trials]
        Fs = [np.zeros((ns, self.nbf, self.nbf)) for _ in trials]
        k = len(trials)
        dp = (vp * max(1, k))(*[x.ctypes.data for x in Ds])
        fp = (vp * max(1, k))(*[x.ctypes.data for x in Fs])
        if kind == "singlet":
            self.ctx.check(self.ctx.L.xcgpu_lr_kernel(self.h, fid, _ptr(P0c), k, dp, fp, precision,
                                                      block_ave_threshold, MEM_HOST))
        else:
            code = {"triplet": 1, "unrestricted": 2}[kind]
            self.ctx.check(self.ctx.L.xcgpu_lr_kernel_spin(self.h, fid, code, _ptr(P0c), k, dp, fp, precision,
                                                           block_ave_threshold, MEM_HOST))
        out = [np.swapaxes(F, 1, 2) for F in Fs]
        return out if ns == 2 else [F[0] for F in out]

    def xc_gradient(self, func, P, shell_atom, natoms):
        """XC part of the nuclear gradient (FuncPotential<M>::getGeomGradients), FP64:
        natoms x 3.  shell_atom[s] = atom of shell s; P host [nbf,nbf] or [nspin,nbf,nbf]."""
        fid = FUNC[func] if isinstance(func, str) else int(func)
        P = np.asarray(P, dtype=np.float64)
        nspin = 1 if P.ndim == 2 else P.shape[0]
        Pc = np.ascontiguousarray(np.stack([m.T for m in P.reshape(nspin, self.nbf, self.nbf)]))
        sa = np.ascontiguousarray(shell_atom, dtype=np.int32)
        G = np.zeros(3 * natoms)
        self.ctx.check(self.ctx.L.xcgpu_xc_gradient(self.h, fid, nspin, _ptr(Pc), _ptr(sa), natoms, _ptr(G), MEM_HOST))
        return G.reshape(3, natoms).T

    def nadd_vxc(self, func, P, env, precision=PREC_FP64, block_ave_threshold=1e-11):
        """Non-additive XC potential of this (active) subsystem in the field of the
        environment subsystems env = [(plan, P_env), ...] on the same grid
        (NAddFuncPotential<M>::getMatrix).  P host arrays [nbf,nbf] / [nspin,nbf,nbf].
        Returns (V [nspin, nbf, nbf] of this plan's basis, E_nadd)."""
        fid = FUNC[func] if isinstance(func, str) else int(func)
        P = np.asarray(P, dtype=np.float64)
        nspin = 1 if P.ndim == 2 else P.shape[0]

        def colmajor(M, nbf):
            return np.ascontiguousarray(np.stack([m.T for m in np.asarray(M, dtype=np.float64).reshape(nspin, nbf, nbf)]))
        Pc = colmajor(P, self.nbf)
        envc = [colmajor(Pe, pl.nbf) for pl, Pe in env]
        plans = (vp * max(1, len(env)))(*[pl.h for pl, _ in env])
        ptrs = (vp * max(1, len(env)))(*[e.ctypes.data for e in envc])
        V = np.zeros((nspin, self.nbf, self.nbf))
        e = ctypes.c_double()
        self.ctx.check(self.ctx.L.xcgpu_nadd_vxc(self.h, plans, len(env), fid, nspin, precision, block_ave_threshold,
                                                 _ptr(Pc), ptrs, _ptr(V), ctypes.byref(e), MEM_HOST))
        return V.transpose(0, 2, 1), e.value

    def __del__(self):
        if getattr(self, "h", None) and self.ctx.h:
            self.ctx.L.xcgpu_plan_destroy(self.h)
            self.h = None
