"""Generates tests/golden/*.npz from the reference's own CUDA kernels.

The reference ships no tests, fixtures or golden vectors, so the vectors here
come from running its kernels (KaminoGPU/kernel/KaminoCore.cu, tdm.cu,
KaminoSolver.cu compiled unchanged into oracle/_ref/*.cubin) through the
harness oracle/ref/kref_harness.cpp on a GB300:

  python tests/golden/make_golden.py [out_dir]    (default: tests/golden/new/)

ref_index.npz  index tuples and alphas of the reference samplers' index
               stage (its own validateCoord) for a fixed 20,000-point subset
               of the seeded coordinate sets of tests/points.py; particle
               wrap + cell indices.
ref_step.npz   seeded initial states and the reference's fields after each
               stage and after 1 and 3 steps (nTheta = 32 and 64).
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import kaminogpu_gb300 as kg  # noqa: E402
from oracle import oracle as orc  # noqa: E402
from points import index_points  # noqa: E402


KEEP = 20000  # committed points per nTheta; the GPU tests cover every grid point live


def subsample(nt, n):
    """The fixed subset of the generated points kept in the fixture."""
    return np.sort(np.random.default_rng(7 + nt).choice(n, min(KEEP, n), replace=False))


def main(out):
    os.makedirs(out, exist_ok=True)
    idx = {}
    for nt in (32, 1024):
        phi, theta = index_points(nt, n_random=4000, seed=100 + nt)
        keep = subsample(nt, len(phi))
        phi, theta = phi[keep], theta[keep]
        ref = orc.RefGPU(nt, 1.0, 0.001)
        idx["phi_%d" % nt] = phi
        idx["theta_%d" % nt] = theta
        for kind in (0, 1, 2):
            o, a = ref.probe_index(kind, phi, theta)
            idx["index_%d_%d" % (nt, kind)] = o
            idx["alpha_%d_%d" % (nt, kind)] = a
        p, t, c = ref.probe_wrap(phi, theta)
        idx["wrap_phi_%d" % nt], idx["wrap_theta_%d" % nt], idx["cells_%d" % nt] = p, t, c
        ref.close()
    np.savez_compressed(os.path.join(out, "ref_index.npz"), **idx)

    steps = {}
    for nt, dt, npart, seed in ((32, 0.005, 1024, 21), (64, 0.005, 1024, 22)):
        st = kg.make_initial_state(nt, lmax=8, seed=seed, n_particles=npart)
        pre = "nt%d_" % nt
        for k in ("u_phi", "u_theta", "thickness", "particles"):
            steps[pre + "in_" + k] = st[k]
        steps[pre + "meta"] = np.array([nt, dt, npart, seed], np.float64)
        for stage in ("advection", "geometric", "projection"):
            ref = orc.RefGPU(nt, 1.0, dt, npart)
            ref.load(st)
            getattr(ref, stage)()
            f = ref.fields()
            for k in ("u_phi", "u_theta", "thickness"):
                steps[pre + stage + "_" + k] = f[k]
            ref.close()
        for n in (1, 3):
            ref = orc.RefGPU(nt, 1.0, dt, npart)
            ref.load(st)
            ref.step(n)
            f = ref.fields()
            for k in ("u_phi", "u_theta", "thickness", "pressure", "particles"):
                steps[pre + "step%d_" % n + k] = f[k]
            ref.close()
    np.savez_compressed(os.path.join(out, "ref_step.npz"), **steps)
    print("wrote", out)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(os.path.dirname(os.path.abspath(__file__)), "new"))
