"""Builds the engine library in-tree: implicit_dpd_gb300/_build/libidpd_engine.so.

Each translation unit is compiled for sm_103a only, in parallel, then linked
into one shared library with a plain C ABI (include/idpd_engine.h).

    python -m implicit_dpd_gb300.build [--verbose]
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(OUT_DIR, "libidpd_engine.so")
SOURCES = ["engine.cu", "kernels_cells.cu", "kernels_pairs.cu", "kernels_force.cu",
           "kernels_integrate.cu",
           "kernels_chem.cu", "kernels_walks.cu", "no_alloc.cu", "formats.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def flags(verbose=False):
    f = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
                "-I", os.path.join(ROOT, "include"), "-I", CSRC]
    if verbose:
        f += ["-Xptxas", "-v"]
    return f


def _compile(src, verbose):
    obj = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc()] + flags(verbose) + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps.append(os.path.join(ROOT, "include", "idpd_engine.h"))
    deps.append(os.path.abspath(__file__))
    return all(os.path.getmtime(p) <= t for p in deps)


def build(verbose=False, force=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="--verbose" in sys.argv, force="--force" in sys.argv))
