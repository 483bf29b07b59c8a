"""Extract the element blocks this package needs from Serenity's Turbomole-format
basis-set library into ``serenity_gb300/data/basis/``.

Basis sets are published numerical data (def2: Weigend & Ahlrichs, PCCP 7, 3297
(2005); cc-pV5Z: Dunning and co-workers) that the reference ships as
``data/basis/<NAME>`` files exported from the Basis Set Exchange.  The extract
keeps the reference's file format unchanged (``$basis`` / ``*`` / ``<el> <NAME>``
/ ``*`` / ``<nprim> <l>`` / ``<exponent> <coefficient>`` lines, terminated by
``*``), so ``serenity_gb300.basis.read_basis`` parses both the extract and the
reference library with the same rules as BasisFunctionProvider.cpp:36-131.

Run once where the reference is mounted::

    python serenity_gb300/data/extract_basis.py /path/to/serenity
"""
import os
import re
import sys

# element blocks needed by the workloads (water clusters), the H2 end-to-end
# test systems and the spherical-normalisation test (Sc up to l = 6)
WANTED = {
    "DEF2-SVP": ["h", "c", "n", "o"],
    "DEF2-TZVP": ["h", "c", "n", "o"],
    "CC-PV5Z": ["sc"],
    "6-31GS": ["h"],  # the embedding (FDE) H2 test systems
}


def extract(ref_root, out_dir):
    for name, elements in WANTED.items():
        src = os.path.join(ref_root, "data", "basis", name)
        text = open(src).read()
        out = ["$basis", "*"]
        for el in elements:
            m = re.search(r"\n%s\s+%s\s*\n\*\n" % (re.escape(el), re.escape(name)), text, re.IGNORECASE)
            if m is None:
                raise RuntimeError("element %s not found in %s" % (el, src))
            end = text.find("*", m.end())
            body = text[m.end():end].rstrip("\n").split("\n")
            body = [ln for ln in body if not ln.lstrip().startswith("#")]
            out.append("%s   %s" % (el, name))
            out.append("*")
            out.extend(ln.rstrip() for ln in body if ln.strip())
            out.append("*")
        out.append("$end")
        with open(os.path.join(out_dir, name), "w") as f:
            f.write("\n".join(out) + "\n")


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: python serenity_gb300/data/extract_basis.py <path of the reference source tree>")
    extract(sys.argv[1], os.path.join(os.path.dirname(os.path.abspath(__file__)), "basis"))
