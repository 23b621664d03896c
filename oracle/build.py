"""Builds the test-infrastructure side: the oracle and the reference harness.

* oracle/_build/libkamino_oracle.so — the C restatement (kamino_oracle.c),
  gcc with OpenMP and -ffp-contract=off (no fused multiply-add).
* oracle/_ref/ref_{core,tdm,solver}.cubin — the reference's own kernels
  (KaminoGPU/kernel/KaminoCore.cu via ref/ref_core_probe.cu, tdm.cu,
  KaminoSolver.cu) compiled for sm_103a from the reference tree.  Only done
  where the reference tree exists; elsewhere the prebuilt cubins are used.
* oracle/_build/libkref.so — the harness that loads those cubins and runs
  them in stepForward order with cuFFT (ref/kref_harness.cpp).
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REFOUT = os.path.join(HERE, "_ref")


def _reference_tree():
    """The reference checkout (Uchanka/KaminoGPU): $KAMINO_REFERENCE, else a
    directory named `reference` beside this repository's root; None when
    neither exists (the prebuilt reference artefacts are used as they are)."""
    env = os.environ.get("KAMINO_REFERENCE")
    if env:
        return env
    sib = os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")
    return sib if os.path.isdir(os.path.join(sib, "KaminoGPU")) else None


REFSRC = _reference_tree()
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def _stale(out, *srcs):
    return not os.path.exists(out) or os.path.getmtime(out) < max(os.path.getmtime(s) for s in srcs)


def build_oracle():
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, "kamino_oracle.c"), os.path.join(HERE, "synth_state.c")]
    out = os.path.join(BUILD, "libkamino_oracle.so")
    if _stale(out, *srcs):
        _run(["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=c11",
              "-o", out, *srcs, "-lm"])
    return out


def build_ref_cubins():
    """Compile the reference kernels; returns False where the tree is absent."""
    if REFSRC is None:
        return False
    kdir = os.path.join(REFSRC, "KaminoGPU", "kernel")
    if not os.path.isdir(kdir):
        return False
    os.makedirs(REFOUT, exist_ok=True)
    inc = ["-I" + os.path.join(HERE, "ref", "shim"),  # before the vendored helper_cuda.h
           "-I" + kdir, "-I" + os.path.join(REFSRC, "KaminoGPU", "include"),
           "-I" + os.path.join(REFSRC, "KaminoGPU", "cuda_util_headers"),
           "-I" + os.path.join(REFSRC, "KaminoGPU", "partio_headers"),
           "-I" + os.path.join(REFSRC, "KaminoGPU", "opencv_headers")]
    jobs = [(os.path.join(HERE, "ref", "ref_core_probe.cu"), "ref_core.cubin"),
            (os.path.join(kdir, "tdm.cu"), "ref_tdm.cubin"),
            (os.path.join(kdir, "KaminoSolver.cu"), "ref_solver.cubin")]

    def one(job):
        src, name = job
        out = os.path.join(REFOUT, name)
        if _stale(out, src, os.path.join(kdir, "KaminoCore.cu")):
            # the reference's own flags: O3 host/device defaults, no fast math
            _run([NVCC, *ARCH, "-cubin", "-O3", "-std=c++14", "-w", *inc, "-o", out, src])
        return out

    with ThreadPoolExecutor(max_workers=3) as ex:
        list(ex.map(one, jobs))
    return True


def build_ref_fbm():
    """The reference's FBM velocity initialiser (KaminoInitializer.cu and
    vectorUtil.cu, host C++, compiled unchanged) with ref/fbm_harness.cpp into
    _ref/libref_fbm.so, for the golden vectors of tests/golden/make_golden.py.
    Only where the reference tree exists; returns the path or None."""
    if REFSRC is None:
        return None
    kg = os.path.join(REFSRC, "KaminoGPU")
    kdir = os.path.join(kg, "kernel")
    if not os.path.isdir(kdir):
        return None
    os.makedirs(REFOUT, exist_ok=True)
    harness = os.path.join(HERE, "ref", "fbm_harness.cpp")
    srcs = [os.path.join(kdir, "KaminoInitializer.cu"), os.path.join(kdir, "vectorUtil.cu")]
    out = os.path.join(REFOUT, "libref_fbm.so")
    if _stale(out, harness, *srcs):
        inc = ["-I" + os.path.join(HERE, "ref", "shim"), "-I" + os.path.join(kg, "include"),
               "-I" + os.path.join(kg, "cuda_util_headers"), "-I" + os.path.join(kg, "partio_headers"),
               "-I" + os.path.join(kg, "opencv_headers"), "-I" + os.path.join(CUDA, "include")]
        # no contraction into fused multiply-adds: the reference's own build
        # (MSVC, x86) evaluates every product and sum separately
        _run(["g++", "-O2", "-std=c++14", "-ffp-contract=off", "-fPIC", "-shared", "-w", *inc, "-o", out, harness,
              "-x", "c++", *srcs])
    return out


def have_ref_cubins():
    return all(os.path.exists(os.path.join(REFOUT, n))
               for n in ("ref_core.cubin", "ref_tdm.cubin", "ref_solver.cubin"))


def build_harness():
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "ref", "kref_harness.cpp")
    out = os.path.join(BUILD, "libkref.so")
    if _stale(out, src):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I" + os.path.join(CUDA, "include"),
              "-o", out, src, "-L" + os.path.join(CUDA, "lib64"), "-L" + os.path.join(CUDA, "lib64", "stubs"),
              "-Wl,-rpath," + os.path.join(CUDA, "lib64"), "-lcufft", "-lcudart", "-lcuda"])
    return out


def build():
    build_oracle()
    build_ref_cubins()
    build_harness()


if __name__ == "__main__":
    build()
    print("oracle built; reference cubins:", have_ref_cubins())
