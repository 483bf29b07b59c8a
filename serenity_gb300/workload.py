"""Synthetic workloads for the XC build: water clusters, their basis sets and
random orthonormalised density matrices (seeded, reproducible on any host).

* geometry: H2O with O-H 0.96 A and H-O-H 104.5 deg, rotated by a Haar-random
  orthogonal matrix (QR of a 3x3 N(0,1) draw with the sign of R's diagonal
  folded in), its centroid placed on a cubic lattice site (3.0 A spacing) plus an
  optional uniform jitter; Angstrom -> bohr with the reference's BOHR constant.
* density: C ~ N(0,1) of shape n_bf x n_occ, Loewdin-orthonormalised in the
  overlap metric (C <- C (C^T S C)^(-1/2)); P = 2 C C^T (restricted) or
  P_a = C_a C_a^T, P_b = C_b C_b^T (unrestricted).  S is computed analytically
  (Obara-Saika recurrences) for the same normalised shells the XC path uses.
"""
import math

import numpy as np

from .basis import ANGSTROM_TO_BOHR, Shells, atomic_number


def water(rng, jitter=0.0):
    r, th = 0.96, math.radians(104.5)
    mol = np.array([[0.0, 0.0, 0.0], [r, 0.0, 0.0], [r * math.cos(th), r * math.sin(th), 0.0]])
    mol -= mol.mean(axis=0)
    q, rr = np.linalg.qr(rng.standard_normal((3, 3)))
    q = q * np.sign(np.diag(rr))
    mol = mol @ q.T
    if jitter:
        mol = mol + rng.uniform(-jitter, jitter, size=3)
    return mol


def water_cluster(nmol, seed=0, spacing=3.0, jitter=0.0, dims=None):
    """nmol waters on the first nmol sites of a lattice (dims = (nx, ny, nz) or the
    smallest cube).  Returns (symbols, coordinates in bohr)."""
    rng = np.random.default_rng(seed)
    if dims is None:
        k = int(math.ceil(round(nmol ** (1.0 / 3.0), 9)))
        dims = (k, k, k)
    sites = [(i, j, l) for l in range(dims[2]) for j in range(dims[1]) for i in range(dims[0])][:nmol]
    if len(sites) < nmol:
        raise ValueError("lattice too small")
    sym, xyz = [], []
    for s in sites:
        m = water(rng, jitter) + spacing * np.array(s, dtype=float)
        sym += ["O", "H", "H"]
        xyz += list(m)
    return sym, np.array(xyz) * ANGSTROM_TO_BOHR


def _dfact(n):
    r = 1.0
    while n > 1:
        r *= n
        n -= 2
    return r


def normalised_coefs(l, alpha, coef):
    """libint2 convention: primitive normalisation for x^l, then unit self-overlap."""
    a = np.asarray(alpha, dtype=float)
    c = np.asarray(coef, dtype=float) * np.sqrt(2.0 ** l * (2 * a) ** (l + 1.5) / (math.pi ** 1.5 * _dfact(2 * l - 1)))
    g = a[:, None] + a[None, :]
    ov = (_dfact(2 * l - 1) * math.pi ** 1.5 * c[:, None] * c[None, :] / (2.0 ** l * g ** (l + 1.5))).sum()
    return c / math.sqrt(ov)


def cart_list(l):
    return [(a, b, l - a - b) for a in range(l, -1, -1) for b in range(l - a, -1, -1)]


def solid_harmonic_matrix(l):
    """(2l+1) x ncart(l): real solid harmonics, m = -l..l, Cartesian order of cart_list."""
    f = math.factorial
    comps = cart_list(l)
    T = np.zeros((2 * l + 1, len(comps)))
    for m in range(-l, l + 1):
        am = abs(m)
        tv0 = 1 if m < 0 else 0
        N = math.sqrt(2.0 * f(l + am) * f(l - am) / (2.0 if m == 0 else 1.0)) / (2.0 ** am * f(l))
        for t in range((l - am) // 2 + 1):
            for u in range(t + 1):
                for tv in range(tv0, am + 1, 2):
                    sgn = -1.0 if (t + (tv - tv0) // 2) % 2 else 1.0
                    C = sgn * 0.25 ** t * math.comb(l, t) * math.comb(l - t, am + t) * math.comb(t, u) * math.comb(am, tv)
                    py = 2 * u + tv
                    px = 2 * t + am - py
                    T[m + l, comps.index((px, py, l - px - py))] += N * C
    return T


def _cart_norms(l):
    return np.array([math.sqrt(_dfact(2 * l - 1) / (_dfact(2 * a - 1) * _dfact(2 * b - 1) * _dfact(2 * c - 1)))
                     for a, b, c in cart_list(l)])


def _overlap_1d(la, lb, PA, PB, p):
    """S[i][j] / sqrt(pi/p) for one Cartesian direction (Obara-Saika); arrays over primitive pairs."""
    S = [[None] * (lb + 1) for _ in range(la + 1)]
    S[0][0] = np.ones_like(PA)
    for i in range(la + 1):
        for j in range(lb + 1):
            if i == 0 and j == 0:
                continue
            if i > 0:
                v = PA * S[i - 1][j]
                if i > 1:
                    v = v + (i - 1) / (2 * p) * S[i - 2][j]
                if j > 0:
                    v = v + j / (2 * p) * S[i - 1][j - 1]
            else:
                v = PB * S[i][j - 1]
                if j > 1:
                    v = v + (j - 1) / (2 * p) * S[i][j - 2]
            S[i][j] = v
    return S


def overlap_matrix(shells, cutoff=30.0):
    """Analytic overlap matrix of the (normalised) shells."""
    sh = shells.as_list()
    coefs = [normalised_coefs(s["l"], s["alpha"], s["coef"]) for s in sh]
    trans = []
    for s in sh:
        l = s["l"]
        trans.append(solid_harmonic_matrix(l) if s["pure"] else np.diag(_cart_norms(l)))
    first = np.concatenate([[0], np.cumsum(shells.nfunc)])[:-1]
    S = np.zeros((shells.nbf, shells.nbf))
    for i, a in enumerate(sh):
        A = np.array(a["center"])
        ai = np.array(a["alpha"])
        for j in range(i + 1):
            b = sh[j]
            B = np.array(b["center"])
            if np.linalg.norm(A - B) > cutoff:
                continue
            bj = np.array(b["alpha"])
            al, be = ai[:, None], bj[None, :]
            p = al + be
            P = (al[..., None] * A + be[..., None] * B) / p[..., None]
            K = np.exp(-al * be / p * np.dot(A - B, A - B)) * (math.pi / p) ** 1.5
            cc = coefs[i][:, None] * coefs[j][None, :] * K
            la, lb = a["l"], b["l"]
            S1 = [_overlap_1d(la, lb, P[..., k] - A[k], P[..., k] - B[k], p) for k in range(3)]
            ca, cb = cart_list(la), cart_list(lb)
            M = np.zeros((len(ca), len(cb)))
            for x, (ax, ay, az) in enumerate(ca):
                for y, (bx, by, bz) in enumerate(cb):
                    M[x, y] = (cc * S1[0][ax][bx] * S1[1][ay][by] * S1[2][az][bz]).sum()
            blk = trans[i] @ M @ trans[j].T
            fi, fj = first[i], first[j]
            S[fi:fi + blk.shape[0], fj:fj + blk.shape[1]] = blk
            S[fj:fj + blk.shape[1], fi:fi + blk.shape[0]] = blk.T
    return S


def orthonormal_orbitals(S, nocc, rng):
    C = rng.standard_normal((S.shape[0], nocc))
    M = C.T @ S @ C
    e, U = np.linalg.eigh(M)
    return C @ (U * e ** -0.5) @ U.T


def density_matrices(S, nocc, seed=0):
    """nocc = int (restricted, P = 2 C C^T) or (n_alpha, n_beta)."""
    rng = np.random.default_rng(seed)
    if isinstance(nocc, (tuple, list)):
        Ca = orthonormal_orbitals(S, nocc[0], rng)
        Cb = orthonormal_orbitals(S, nocc[1], rng)
        return np.stack([Ca @ Ca.T, Cb @ Cb.T])
    C = orthonormal_orbitals(S, nocc, rng)
    return 2.0 * C @ C.T


class Workload:
    """One XC build: atoms, shells, grid specification and density matrices."""

    def __init__(self, symbols, coords, basis, func, nocc, n_rad, n_ang, seed=0, spherical=True):
        self.symbols, self.coords = symbols, coords
        self.Z = np.array([atomic_number(s) for s in symbols], dtype=np.int32)
        self.basis_name, self.func = basis, func
        self.shells = Shells.for_atoms(symbols, coords, basis, spherical=spherical)
        self.nocc, self.n_rad, self.n_ang, self.seed = nocc, n_rad, n_ang, seed
        self._P = None

    @property
    def nbf(self):
        return self.shells.nbf

    @property
    def nspin(self):
        return 2 if isinstance(self.nocc, (tuple, list)) else 1

    def density(self):
        if self._P is None:
            self._P = density_matrices(overlap_matrix(self.shells), self.nocc, self.seed)
        return self._P


def config(index, seed=0):
    """The five synthetic configurations of the benchmark definition (0..2 here;
    3 and 4 are batches built from ``water_cluster``)."""
    if index == 0:
        sym, xyz = water_cluster(4, seed, jitter=0.0, dims=(2, 2, 1))
        return Workload(sym, xyz, "DEF2-SVP", "LDA", 20, 50, 194, seed)
    if index == 1:
        sym, xyz = water_cluster(32, seed, jitter=0.2, dims=(4, 4, 2))
        return Workload(sym, xyz, "DEF2-SVP", "PBE", 160, 75, 302, seed)
    if index == 2:
        sym, xyz = water_cluster(64, seed, jitter=0.2, dims=(4, 4, 4))
        return Workload(sym, xyz, "DEF2-TZVP", "PBE", (320, 319), 99, 434, seed)
    raise ValueError("config %d is a batch; build it with water_cluster" % index)
