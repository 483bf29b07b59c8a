"""Build the xcgpu shared library (``serenity_gb300/_build/libxcgpu.so``) in tree.

Every CUDA translation unit is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, then linked into one
shared library with a plain C ABI (``include/xcgpu.h``).  No torch, no CMake.
"""
import concurrent.futures
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libxcgpu.so")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fopenmp,-O3", "--expt-relaxed-constexpr"]


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(HERE, "..", "include", "xcgpu.h")]


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def _compile(src, extra, build_dir=BUILD):
    obj = os.path.join(build_dir, os.path.basename(src) + ".o")
    cmd = [NVCC] + ARCH + FLAGS + extra + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return obj, r.stderr


def build(force=False, verbose=False, extra=(), out=None):
    """Compile and link; `out` (a path) builds a variant library elsewhere with the
    extra nvcc flags (e.g. -D switches) instead of the default in-tree library."""
    lib = out or LIB
    if not force and out is None and up_to_date():
        return LIB
    build_dir = os.path.join(os.path.dirname(lib), "obj_" + os.path.basename(lib)) if out else BUILD
    os.makedirs(build_dir, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=8) as ex:
        results = list(ex.map(lambda s: _compile(s, list(extra), build_dir), sources()))
    if verbose:
        for obj, err in results:
            if err.strip():
                sys.stderr.write(err)
    objs = [o for o, _ in results]
    tmp = lib + ".tmp"
    cmd = [NVCC] + ARCH + ["-shared", "-Xcompiler", "-fopenmp", "-o", tmp] + objs + ["-lgomp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    extra = ["-Xptxas", "-v"] if "-v" in sys.argv else []
    print(build(force=True, verbose=bool(extra), extra=extra))
