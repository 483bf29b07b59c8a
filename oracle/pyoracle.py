"""ORACLE -- test infrastructure only.

ctypes binding of ``oracle/_build/liboracle.so`` (the CPU FP64 restatement of the
reference's XC grid path, see ``oracle/oracle.h``).  Only ``tests/``, the smoke
check and ``bench.py``'s CPU-baseline leg import this module.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

FUNC = {"LDA": 1, "PBE": 2, "BLYP": 3, "BP86": 4, "SLATER": 16, "VWN5": 17, "PBEX": 18, "PBEC": 19, "B88": 20,
        "LYP": 21, "PW92": 22, "P86": 23, "PZ81": 24}

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_basis_create.restype = ctypes.c_void_p
        L.orc_basis_create.argtypes = [ctypes.c_int, _ip, _ip, _ip, _dp, _dp, _dp]
        L.orc_basis_free.argtypes = [ctypes.c_void_p]
        L.orc_basis_nbf.argtypes = [ctypes.c_void_p]
        L.orc_basis_shell_coefs.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp]
        L.orc_block_on_grid.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int, ctypes.c_double, ctypes.c_int, _dp,
                                        ctypes.c_void_p, ctypes.c_void_p, _ip]
        L.orc_density.argtypes = [ctypes.c_void_p, _dp, ctypes.c_long, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                  _dp, _dp, ctypes.c_void_p]
        L.orc_functional.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_long, ctypes.c_int, _dp, ctypes.c_void_p,
                                     _dp, _dp, ctypes.c_void_p]
        L.orc_functional_is_gga.argtypes = [ctypes.c_int]
        L.orc_active_functions.restype = ctypes.c_long
        L.orc_active_functions.argtypes = [ctypes.c_void_p, _dp, ctypes.c_long, ctypes.c_int, ctypes.c_double]
        L.orc_add_scalar.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_long, ctypes.c_int, ctypes.c_double,
                                     ctypes.c_double, ctypes.c_int, _dp, ctypes.c_void_p, _dp]
        L.orc_vxc.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_long, ctypes.c_int, ctypes.c_double,
                              ctypes.c_double, ctypes.c_int, ctypes.c_int, _dp, _dp,
                              ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double), ctypes.c_int]
        L.orc_becke_grid.restype = ctypes.c_long
        L.orc_becke_grid.argtypes = [ctypes.c_int, _ip, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_char_p, _dp, _dp,
                                     ctypes.c_long, ctypes.c_int]
        L.orc_ahlrichs_radial.argtypes = [ctypes.c_double, ctypes.c_int, _dp, _dp]
        L.orc_solid_harmonics.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, _dp]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class Basis:
    def __init__(self, shells):
        L = lib()
        self.shells = shells
        self.h = L.orc_basis_create(shells.nshell, shells.l, shells.pure, shells.nprim, shells.centers, shells.alpha,
                                    shells.coef)
        self.nbf = L.orc_basis_nbf(self.h)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_basis_free(self.h)
            self.h = None

    def shell_coefs(self, s):
        out = np.zeros(int(self.shells.nprim[s]))
        lib().orc_basis_shell_coefs(self.h, s, out)
        return out

    def block(self, xyz, thr, deriv=1):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        n = xyz.shape[0]
        v = np.zeros(n * self.nbf)
        g = np.zeros(3 * n * self.nbf) if deriv >= 1 else None
        h = np.zeros(6 * n * self.nbf) if deriv >= 2 else None
        neg = np.zeros(self.nbf, dtype=np.int32)
        lib().orc_block_on_grid(self.h, xyz.reshape(-1), n, thr, deriv, v, _ptr(g), _ptr(h), neg)
        out = {"values": v.reshape(self.nbf, n).T, "negligible": neg}
        if deriv >= 1:
            out["grad"] = g.reshape(3, self.nbf, n).transpose(0, 2, 1)
        if deriv >= 2:
            out["hess"] = h.reshape(6, self.nbf, n).transpose(0, 2, 1)
        return out

    def density(self, xyz, P, max_block=128, thr=1e-9, grad=True):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1)
        n = xyz.size // 3
        P = np.asarray(P, dtype=np.float64)
        nspin = 1 if P.ndim == 2 else P.shape[0]
        Pc = np.ascontiguousarray(np.stack([m.T for m in P.reshape(nspin, self.nbf, self.nbf)]).reshape(-1))
        rho = np.zeros(nspin * n)
        g = np.zeros(nspin * 3 * n) if grad else None
        lib().orc_density(self.h, xyz, n, max_block, thr, nspin, Pc, rho, _ptr(g))
        return rho.reshape(nspin, n), (g.reshape(nspin, 3, n) if grad else None)

    def add_scalar(self, xyz, w, v, g=None, max_block=128, thr=1e-9, ave_thr=1e-11):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1)
        n = xyz.size // 3
        v = np.ascontiguousarray(v, dtype=np.float64).reshape(-1)
        nspin = v.size // n
        gg = None if g is None else np.ascontiguousarray(g, dtype=np.float64).reshape(-1)
        F = np.zeros(nspin * self.nbf * self.nbf)
        lib().orc_add_scalar(self.h, xyz, np.ascontiguousarray(w, dtype=np.float64), n, max_block, thr, ave_thr,
                             nspin, v, _ptr(gg), F)
        F = F.reshape(nspin, self.nbf, self.nbf).transpose(0, 2, 1)
        return F

    def active_functions(self, xyz, max_block=128, thr=1e-9):
        """Sum over blocks of the non-negligible function count."""
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        return int(lib().orc_active_functions(self.h, xyz, len(xyz), max_block, thr))

    def vxc(self, xyz, w, func, P, max_block=128, thr=1e-9, ave_thr=1e-11, threads=0):
        """Whole build: returns (V [nspin,nbf,nbf], Exc, Nel)."""
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1)
        n = xyz.size // 3
        P = np.asarray(P, dtype=np.float64)
        nspin = 1 if P.ndim == 2 else P.shape[0]
        Pc = np.ascontiguousarray(np.stack([m.T for m in P.reshape(nspin, self.nbf, self.nbf)]).reshape(-1))
        V = np.zeros(nspin * self.nbf * self.nbf)
        exc, nel = ctypes.c_double(), ctypes.c_double()
        fid = FUNC[func] if isinstance(func, str) else int(func)
        lib().orc_vxc(self.h, xyz, np.ascontiguousarray(w, dtype=np.float64), n, max_block, thr, ave_thr, fid, nspin,
                      Pc, V, ctypes.byref(exc), ctypes.byref(nel), threads)
        return V.reshape(nspin, self.nbf, self.nbf).transpose(0, 2, 1), exc.value, nel.value


def functional(func, rho, grad=None, max_block=0):
    """rho [nspin, n], grad [nspin, 3, n] -> (epuv [n], dfdrho [nspin, n], dfdgrad [nspin, 3, n])."""
    rho = np.ascontiguousarray(rho, dtype=np.float64)
    nspin, n = rho.shape
    fid = FUNC[func] if isinstance(func, str) else int(func)
    gga = bool(lib().orc_functional_is_gga(fid))
    g = None if grad is None else np.ascontiguousarray(grad, dtype=np.float64).reshape(-1)
    epuv = np.zeros(n)
    dr = np.zeros(nspin * n)
    dg = np.zeros(nspin * 3 * n) if gga else None
    lib().orc_functional(fid, nspin, n, max_block, rho.reshape(-1), _ptr(g), epuv, dr, _ptr(dg))
    return epuv, dr.reshape(nspin, n), (dg.reshape(nspin, 3, n) if gga else None)


PARTITION = {"becke": 0, "ssf": 1}


def becke_grid(Z, xyz_bohr, n_rad=0, n_ang=0, accuracy=0, weight_threshold=1e-14, smoothing=3, sort=True,
               lebedev_path=None, partition="becke"):
    from serenity_gb300.basis import LEBEDEV_TABLE
    Z = np.ascontiguousarray(Z, dtype=np.int32)
    xyz = np.ascontiguousarray(xyz_bohr, dtype=np.float64).reshape(-1)
    cap = len(Z) * (max(n_rad, 100) * max(n_ang, 770) + 1)
    out_x = np.zeros(3 * cap)
    out_w = np.zeros(cap)
    path = (lebedev_path or LEBEDEV_TABLE).encode()
    n = lib().orc_becke_grid(len(Z), Z, xyz, n_rad, n_ang, accuracy, weight_threshold, smoothing, int(sort), path,
                             out_x, out_w, cap, PARTITION[partition])
    if n < 0:
        raise RuntimeError("grid capacity exceeded")
    return out_x[:3 * n].reshape(n, 3).copy(), out_w[:n].copy()


def ahlrichs_radial(alpha, n):
    r, w = np.zeros(n), np.zeros(n)
    lib().orc_ahlrichs_radial(alpha, n, r, w)
    return r, w


def solid_harmonics(l, x, y, z):
    out = np.zeros(2 * l + 1)
    lib().orc_solid_harmonics(l, x, y, z, out)
    return out


def nadd_vxc(active, envs, xyz, w, func, P_active, P_envs, max_block=128, thr=1e-9, ave_thr=1e-11):
    """Non-additive XC potential and energy of subsystem DFT, composed from the oracle's
    density, functional and adder as NAddFuncPotential<M>::getMatrix does
    (NAddFuncPotential.cpp:189-243; the supersystem density is the plain sum of the
    subsystem densities, SupersystemDensityOnGridController.cpp:101-187):
        V = adder_active(dF/drho[rho_tot] - dF/drho[rho_act], dF/dgrad[tot] - dF/dgrad[act])
        E = E_xc[rho_tot] - E_xc[rho_act] - sum_env E_xc[rho_env]
    active, envs: Basis objects; P_*: [nbf, nbf] or [nspin, nbf, nbf].  Returns (V, E)."""
    w = np.asarray(w, dtype=np.float64)
    gga = bool(lib().orc_functional_is_gga(FUNC[func] if isinstance(func, str) else int(func)))
    rA, gA = active.density(xyz, P_active, max_block, thr, grad=gga)
    rT = rA.copy()
    gT = gA.copy() if gga else None
    e_env = 0.0
    for B, P in zip(envs, P_envs):
        r, g = B.density(xyz, P, max_block, thr, grad=gga)
        rT += r
        if gga:
            gT += g
        e_env += float(w @ functional(func, r, g, max_block)[0])
    eT, vT, gvT = functional(func, rT, gT, max_block)
    eA, vA, gvA = functional(func, rA, gA, max_block)
    V = active.add_scalar(xyz, w, vT - vA, (gvT - gvA) if gga else None, max_block, thr, ave_thr)
    return V, float(w @ eT) - float(w @ eA) - e_env


def xc_gradient(basis, shell_atom, natoms, xyz, w, func, P, max_block=128, thr=1e-9):
    """XC part of the nuclear gradient (FuncPotential<M>::getGeomGradients): natoms x 3.
    shell_atom[s] = atom index of shell s; P [nbf, nbf] (restricted total) or
    [nspin, nbf, nbf]."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1)
    n = xyz.size // 3
    P = np.asarray(P, dtype=np.float64)
    nspin = 1 if P.ndim == 2 else P.shape[0]
    Pc = np.ascontiguousarray(np.stack([m.T for m in P.reshape(nspin, basis.nbf, basis.nbf)]).reshape(-1))
    out = np.zeros(3 * natoms)
    L = lib()
    L.orc_xc_gradient.argtypes = [ctypes.c_void_p, _ip, ctypes.c_int, _dp, _dp, ctypes.c_long, ctypes.c_int,
                                  ctypes.c_double, ctypes.c_int, ctypes.c_int, _dp, _dp]
    L.orc_xc_gradient(basis.h, np.ascontiguousarray(shell_atom, dtype=np.int32), natoms, xyz,
                      np.ascontiguousarray(w, dtype=np.float64), n, max_block, thr, FUNC[func] if isinstance(func, str)
                      else int(func), nspin, Pc, out)
    return out.reshape(3, natoms).T


def lr_kernel(func, rho0, grad0, rho1, grad1):
    """Restricted linear-response kernel contracted with (rho1, grad rho1) on points:
    (v1 [n], g1 [3, n] or None).  rho [n], grad [3, n]."""
    fid = FUNC[func] if isinstance(func, str) else int(func)
    gga = bool(lib().orc_functional_is_gga(fid))
    rho0 = np.ascontiguousarray(rho0, dtype=np.float64).reshape(-1)
    n = rho0.size
    rho1 = np.ascontiguousarray(rho1, dtype=np.float64).reshape(-1)
    g0 = np.ascontiguousarray(grad0, dtype=np.float64).reshape(-1) if gga else None
    g1 = np.ascontiguousarray(grad1, dtype=np.float64).reshape(-1) if gga else None
    v1 = np.zeros(n)
    go = np.zeros(3 * n) if gga else None
    L = lib()
    L.orc_lr_kernel.argtypes = [ctypes.c_int, ctypes.c_long, _dp, ctypes.c_void_p, _dp, ctypes.c_void_p, _dp,
                                ctypes.c_void_p]
    L.orc_lr_kernel(fid, n, rho0, _ptr(g0), rho1, _ptr(g1), v1, _ptr(go))
    return v1, (go.reshape(3, n) if gga else None)


def lr_fock(basis, xyz, w, func, P0, D, max_block=128, thr=1e-9, ave_thr=1e-11):
    """XC-kernel part of a restricted (singlet) linear-response sigma vector
    (KernelSigmavector<RESTRICTED>::calcF, KernelSigmavector.cpp:128-253): the trial matrix
    D is symmetrised, its density rho1 = phi^T D phi and gradient are contracted with the
    ground-state kernel, and the result goes through the adder (F + F^T).  No per-element
    screening (the reference screens D_ij avg_i avg_j and the integration by block
    averages at 1e-11; here only the adder's block skip applies)."""
    D = np.asarray(D, dtype=np.float64)
    Ds = 0.5 * (D + D.T)
    gga = bool(lib().orc_functional_is_gga(FUNC[func] if isinstance(func, str) else int(func)))
    r0, g0 = basis.density(xyz, P0, max_block, thr, grad=gga)
    r1, g1 = basis.density(xyz, Ds, max_block, thr, grad=gga)
    v1, gv1 = lr_kernel(func, r0[0], g0[0] if gga else None, r1[0], g1[0] if gga else None)
    return basis.add_scalar(xyz, w, v1, gv1.reshape(1, 3, -1) if gga else None, max_block, thr, ave_thr)[0]


def lr_fock_spin(basis, xyz, w, func, P0, D, kind, max_block=128, thr=1e-9, ave_thr=1e-11):
    """XC-kernel part of a linear-response sigma vector with the spin kernels
    (KernelSigmavector.cpp:127-253, contractBlock :363-499).  kind "unrestricted": P0 and D
    [2, nbf, nbf], returns [2, nbf, nbf]; "triplet": P0 (restricted total) and D [nbf, nbf],
    returns [nbf, nbf].  Each spin's D is symmetrised."""
    fid = FUNC[func] if isinstance(func, str) else int(func)
    gga = bool(lib().orc_functional_is_gga(fid))
    code = {"triplet": 1, "unrestricted": 2}[kind]
    ns = 2 if kind == "unrestricted" else 1
    D = np.asarray(D, dtype=np.float64).reshape(ns, basis.nbf, basis.nbf)
    Ds = 0.5 * (D + np.swapaxes(D, 1, 2))
    P0 = np.asarray(P0, dtype=np.float64).reshape(ns, basis.nbf, basis.nbf)
    r0, g0 = basis.density(xyz, P0 if ns == 2 else P0[0], max_block, thr, grad=gga)
    r1, g1 = basis.density(xyz, Ds if ns == 2 else Ds[0], max_block, thr, grad=gga)
    n = r0.shape[1]
    v1 = np.zeros(ns * n)
    go = np.zeros(ns * 3 * n) if gga else None
    L = lib()
    L.orc_lr_kernel_spin.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_long, _dp, ctypes.c_void_p, _dp,
                                     ctypes.c_void_p, _dp, ctypes.c_void_p]
    c = np.ascontiguousarray
    L.orc_lr_kernel_spin(fid, code, n, c(r0.reshape(-1)), _ptr(c(g0.reshape(-1)) if gga else None),
                         c(r1.reshape(-1)), _ptr(c(g1.reshape(-1)) if gga else None), v1, _ptr(go))
    F = basis.add_scalar(xyz, w, v1.reshape(ns, n), go.reshape(ns, 3, n) if gga else None, max_block, thr, ave_thr)
    return F if ns == 2 else F[0]
