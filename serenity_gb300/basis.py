"""Basis-set input for the XC path: Turbomole-format library files and the flat
shell arrays that the C ABI (``xcgpu_basis_create``) takes.

Parsing follows the reference's rules (BasisFunctionProvider.cpp:36-131): the
element block starts at ``<el> <BASIS>`` (case-insensitive), a ``#`` comment line
right after it is skipped, the block ends at the next ``*``, ``D+``/``D-``
exponent markers are read as ``E+``/``E-``, and each contraction is
``<nprim> <l-letter>`` followed by ``nprim`` pairs ``exponent coefficient``.
Coefficients are passed on raw; normalisation happens in the library.
"""
import functools
import os
import re

import numpy as np

DATA_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")
BASIS_DIR = os.path.join(DATA_DIR, "basis")
LEBEDEV_TABLE = os.path.join(DATA_DIR, "lebedev.txt")

ANGSTROM_TO_BOHR = 1.0 / (5.29177210544e-11 * 1.0e10)  # Constants.h:63-81
ELEMENTS = ["H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne", "Na", "Mg", "Al", "Si", "P", "S", "Cl", "Ar",
            "K", "Ca", "Sc", "Ti", "V", "Cr", "Mn", "Fe", "Co", "Ni", "Cu", "Zn", "Ga", "Ge", "As", "Se", "Br", "Kr"]
_AM = {"s": 0, "p": 1, "d": 2, "f": 3, "g": 4, "h": 5, "i": 6}


def atomic_number(symbol):
    return ELEMENTS.index(symbol.capitalize()) + 1


class BasisError(ValueError):
    pass


def read_element(name, element, library=BASIS_DIR):
    """Contractions ``[(l, exponents, coefficients), ...]`` of ``element`` in basis ``name``
    (parsed once per (file, element) and cached)."""
    return [(l, list(e), list(c)) for l, e, c in _read_element_cached(name, element.lower(), library)]


@functools.lru_cache(maxsize=None)
def _read_element_cached(name, element, library):
    return tuple((l, tuple(e), tuple(c)) for l, e, c in _parse_element(name, element, library))


def _parse_element(name, element, library):
    path = os.path.join(library, name)
    if not os.path.exists(path):
        raise BasisError("Error while parsing basis file %s: file not found" % path)
    text = open(path).read()
    el = element.lower()
    key = ("\n" + el) if len(el) == 1 else el
    m = re.search(re.escape(key) + r"\s+" + re.escape(name), text, re.IGNORECASE)
    if m is None:
        raise BasisError("Error while parsing basis set file %s for element %s: not defined" % (path, element))
    start = m.end()
    if text[start + 1:start + 2] == "#":
        start = text.index("\n", start + 1)
    end = text.find("*", start + 3)
    body = re.sub(r"D(\+|-)", r"E\1", text[start + 3:end])
    tok = body.split()
    out, i = [], 0
    while i < len(tok):
        try:
            nprim = int(tok[i])
        except ValueError:
            break
        if i + 1 >= len(tok) or tok[i + 1].lower() not in _AM:
            raise BasisError("Error while parsing basis set file %s for element %s" % (path, element))
        l = _AM[tok[i + 1].lower()]
        vals = tok[i + 2:i + 2 + 2 * nprim]
        if len(vals) != 2 * nprim:
            raise BasisError("mismatch between the number of primitives and exponent-coefficient entries")
        exps = [float(v) for v in vals[0::2]]
        coefs = [float(v) for v in vals[1::2]]
        out.append((l, exps, coefs))
        i += 2 + 2 * nprim
    return out


class Shells:
    """Flat shell arrays in the order of the atoms and of the basis file."""

    def __init__(self, shells):
        self.l = np.array([s["l"] for s in shells], dtype=np.int32)
        self.pure = np.array([int(bool(s["pure"])) for s in shells], dtype=np.int32)
        self.nprim = np.array([len(s["alpha"]) for s in shells], dtype=np.int32)
        self.centers = np.ascontiguousarray(np.array([s["center"] for s in shells], dtype=np.float64).reshape(-1))
        self.alpha = np.array([a for s in shells for a in s["alpha"]], dtype=np.float64)
        self.coef = np.array([c for s in shells for c in s["coef"]], dtype=np.float64)
        self.nfunc = np.where(self.pure == 1, 2 * self.l + 1, (self.l + 1) * (self.l + 2) // 2)
        self.nbf = int(self.nfunc.sum())
        self.nshell = len(shells)

    @staticmethod
    def for_atoms(symbols, coords_bohr, name, spherical=True, library=BASIS_DIR):
        shells = []
        for sym, xyz in zip(symbols, coords_bohr):
            for l, exps, coefs in read_element(name, sym, library):
                shells.append({"l": l, "pure": spherical, "center": list(map(float, xyz)), "alpha": exps,
                               "coef": coefs})
        return Shells(shells)

    def atom_indices(self, coords_bohr):
        """Atom index of every shell: the atom at the shell's centre."""
        xyz = np.asarray(coords_bohr, dtype=np.float64).reshape(-1, 3)
        c = np.asarray(self.centers, dtype=np.float64).reshape(-1, 3)
        return np.argmin(((c[:, None, :] - xyz[None, :, :]) ** 2).sum(-1), axis=1).astype(np.int32)

    def as_list(self):
        out, off = [], 0
        for i in range(self.nshell):
            n = int(self.nprim[i])
            out.append({"l": int(self.l[i]), "pure": int(self.pure[i]), "center": self.centers[3 * i:3 * i + 3].tolist(),
                        "alpha": self.alpha[off:off + n].tolist(), "coef": self.coef[off:off + n].tolist()})
            off += n
        return out
