"""Pole-wrap index map and particle cell indices: bit-exact against the
reference.  The CUDA samplers' index stage (kamino_probe_index, the same device
code the step runs) is compared with (a) the reference's own validateCoord
compiled from KaminoGPU/kernel/KaminoCore.cu and run on the GPU, and (b) the
oracle's restatement in the reference's float/double arithmetic."""
import numpy as np
import pytest

from points import index_points

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("nt", [32, 64, 1024])
@pytest.mark.parametrize("kind", [0, 1, 2])
def test_index_map_bit_exact_vs_oracle(kg, orc, nt, kind):
    phi, theta = index_points(nt)
    with kg.KaminoSolver(config=kg.default_config(n_theta=nt, radius=1.0, dt=0.001)) as s:
        got, ga = s.probe_index(kind, phi, theta)
    want, wa = orc.ref_index(kind, phi, theta, nt)
    bad = np.nonzero((got != want).any(axis=1))[0]
    assert bad.size == 0, "index mismatch at %d points, first %s: got %s want %s" % (
        bad.size, (phi[bad[0]], theta[bad[0]]), got[bad[0]], want[bad[0]])
    # the alphas follow from the same rounded products
    assert np.array_equal(ga.view(np.uint32), wa.view(np.uint32))


@pytest.mark.parametrize("nt", [32, 128, 1024])
@pytest.mark.parametrize("kind", [0, 1, 2])
def test_index_map_bit_exact_vs_reference_kernels(kg, orc, nt, kind):
    if not orc.have_reference_gpu():
        pytest.skip("reference cubins not built")
    phi, theta = index_points(nt, seed=1)
    with kg.KaminoSolver(config=kg.default_config(n_theta=nt, radius=1.0, dt=0.001)) as s:
        got, _ = s.probe_index(kind, phi, theta)
    ref = orc.RefGPU(nt, 1.0, 0.001)
    want, _ = ref.probe_index(kind, phi, theta)
    ref.close()
    bad = np.nonzero((got != want).any(axis=1))[0]
    assert bad.size == 0, "index mismatch vs reference kernels at %d points, first %s: got %s want %s" % (
        bad.size, (phi[bad[0]], theta[bad[0]]), got[bad[0]], want[bad[0]])


@pytest.mark.parametrize("nt", [32, 512])
def test_particle_wrap_and_cells_bit_exact(kg, orc, nt):
    phi, theta = index_points(nt, seed=2)
    with kg.KaminoSolver(config=kg.default_config(n_theta=nt, radius=1.0, dt=0.001)) as s:
        gp, gt, gc = s.probe_wrap(phi, theta)
    wp, wt, wc = orc.ref_wrap(phi, theta, nt)
    assert np.array_equal(gp.view(np.uint32), wp.view(np.uint32))
    assert np.array_equal(gt.view(np.uint32), wt.view(np.uint32))
    assert np.array_equal(gc, wc)
    if orc.have_reference_gpu():
        ref = orc.RefGPU(nt, 1.0, 0.001)
        rp, rt, rc = ref.probe_wrap(phi, theta)
        ref.close()
        assert np.array_equal(gp.view(np.uint32), rp.view(np.uint32))
        assert np.array_equal(gt.view(np.uint32), rt.view(np.uint32))
        assert np.array_equal(gc, rc)
