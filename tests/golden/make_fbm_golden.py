"""Generates tests/golden/ref_fbm.npz from the reference's own FBM velocity
initialiser.

KaminoSolver::initialize_velocity (KaminoGPU/kernel/KaminoInitializer.cu:3-134)
is host C++.  oracle/build.py (build_ref_fbm) compiles it unchanged, with
vectorUtil.cu and the stand-in solver of oracle/ref/fbm_harness.cpp, into
oracle/_ref/libref_fbm.so; this script runs it for a radius-1 sphere of
nTheta = 64 and 256 and keeps both velocity fields.  It needs the reference
tree ($KAMINO_REFERENCE, or a directory `reference` beside this repository):

  python tests/golden/make_fbm_golden.py [out_dir]    (default: tests/golden/)
"""
import ctypes
import importlib.util
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
SIZES = (64, 256)


def main(out):
    spec = importlib.util.spec_from_file_location("oracle_build", os.path.join(ROOT, "oracle", "build.py"))
    ob = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(ob)
    so = ob.build_ref_fbm()
    if so is None:
        sys.exit("the reference tree is not on this machine")
    lib = ctypes.CDLL(so)
    lib.ref_fbm_velocity.argtypes = [ctypes.c_int, ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p]
    arrays = {}
    for nt in SIZES:
        u = np.zeros((nt, 2 * nt), np.float32)
        v = np.zeros((nt - 1, 2 * nt), np.float32)
        if lib.ref_fbm_velocity(nt, 1.0, u.ctypes.data, v.ctypes.data):
            sys.exit("ref_fbm_velocity(%d) failed" % nt)
        arrays["u_phi_%d" % nt] = u
        arrays["u_theta_%d" % nt] = v
    os.makedirs(out, exist_ok=True)
    np.savez_compressed(os.path.join(out, "ref_fbm.npz"), **arrays)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE)
