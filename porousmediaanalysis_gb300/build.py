"""Builds the pma CUDA library (libpma.so) and the pma command-line tool in-tree.

Every translation unit is compiled by nvcc for sm_103a only, in parallel, into
porousmediaanalysis_gb300/_build/. Objects are rebuilt only when a source or header is newer.
"""
import concurrent.futures
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", "nvcc")
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + INCLUDE]
LIB_SOURCES = ["capi.cpp", "pipeline.cpp", "batch.cpp", "serve.cpp", "pma_io.cpp", "exact_ids.cpp", "edt.cu",
               "balls.cu", "geodesic.cu", "pores.cu", "watershed.cu", "resample.cu", "transfer.cu"]
LIB = os.path.join(OUT, "libpma.so")
CLI = os.path.join(OUT, "pma")


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".h")]
    hs.append(os.path.join(INCLUDE, "pma.h"))
    return hs


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src):
    path = os.path.join(CSRC, src)
    obj = os.path.join(OUT, src + ".o")
    if _newer(obj, [path] + _headers()):
        cmd = [NVCC] + ARCH + COMMON + ["-c", path, "-o", obj]
        if src.endswith(".cu"):
            cmd += ["-Xptxas", "-warn-spills", "--expt-relaxed-constexpr"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    return obj


def build(verbose=False):
    """Compiles libpma.so and the pma tool; returns the library path."""
    os.makedirs(OUT, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        objs = list(ex.map(_compile, LIB_SOURCES))
    if _newer(LIB, objs):
        cmd = [NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    main_src = os.path.join(CSRC, "pma_main.cpp")
    if _newer(CLI, [main_src, LIB]):
        cmd = [NVCC] + ARCH + COMMON + [main_src, "-o", CLI, "-L" + OUT, "-lpma",
                                        "-Xlinker", "-rpath=" + OUT]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("pma tool link failed:\n%s%s" % (r.stdout, r.stderr))
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
