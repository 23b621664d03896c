"""Builds libkamino_gb300.so in-tree (kaminogpu_gb300/lib/) with nvcc for sm_103a,
and the `kamino` executable (kamino configKamino.txt) linked against it.

Translation units compile in parallel; the shared library links against the
shared CUDA runtime.  Re-running is cheap: a unit is rebuilt only when a
source or header in csrc/ is newer than its object.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "lib")
LIB = os.path.join(OUT, "libkamino_gb300.so")
CLI = os.path.join(OUT, "kamino")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
UNITS = ["kamino_solver.cu", "kamino_batch.cu", "kamino_noalloc.cu", "kamino_frames.cu", "kamino_init.cpp"]


def _newest_header():
    t = 0.0
    for d in (CSRC, os.path.join(HERE, "..", "include")):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh")):
                t = max(t, os.path.getmtime(os.path.join(d, f)))
    return t


def _compile(unit, hdr_time, verbose):
    src = os.path.join(CSRC, unit)
    obj = os.path.join(OUT, unit + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), hdr_time):
        return obj
    if unit.endswith(".cu"):
        cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O3",
               "-Xptxas", "-v" if verbose else "-O3", "-c", src, "-o", obj]
    else:
        cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off",
               "-I" + os.path.join(CUDA, "include"), "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    hdr = _newest_header()
    units = [u for u in UNITS if os.path.exists(os.path.join(CSRC, u))]
    with ThreadPoolExecutor(max_workers=len(units)) as ex:
        objs = list(ex.map(lambda u: _compile(u, hdr, verbose), units))
    if not (os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(o) for o in objs)):
        cmd = [NVCC, *ARCH, "-shared", "--cudart", "shared", "-o", LIB, *objs,
               "-Xcompiler", "-fopenmp", "-L" + os.path.join(CUDA, "lib64"),
               "-Xlinker", "-rpath," + os.path.join(CUDA, "lib64")]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    _build_cli()
    return LIB


def _build_cli():
    """The `kamino` executable (csrc/kamino_main.cpp) over the C ABI."""
    src = os.path.join(CSRC, "kamino_main.cpp")
    if not os.path.exists(src):
        return None
    if os.path.exists(CLI) and os.path.getmtime(CLI) >= max(os.path.getmtime(src), os.path.getmtime(LIB)):
        return CLI
    cmd = ["g++", "-O2", "-std=c++17", "-I" + os.path.join(HERE, "..", "include"), src, "-o", CLI,
           "-L" + OUT, "-lkamino_gb300", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("CLI build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return CLI


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
