"""C-ABI paths on the GPU that the parity tests do not reach: pitched host
buffers (cudaMemcpy2D, KaminoQuantity's pitched copies, KaminoQuantity.cu:
3-18), device-pointer state copies, the host-buffer step with a pitch, and
the frame loop without output (Kamino::run, KaminoCore.cu:886-904)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def solver(kg, nt=64, npart=0, frame_dt=None):
    cfg = kg.default_config(n_theta=nt, radius=1.0, dt=0.005, n_particles=npart)
    if frame_dt is not None:
        cfg.frame_dt = frame_dt
    return kg.KaminoSolver(config=cfg)


def test_pitched_host_copies_round_trip(kg):
    nt, npp, pad = 64, 128, 37
    rng = np.random.default_rng(3)
    with solver(kg, nt) as s:
        for field, rows in ((kg.U_PHI, nt), (kg.U_THETA, nt - 1), (kg.THICKNESS, nt)):
            host = rng.standard_normal((rows, npp + pad)).astype(np.float32)
            kg.check(kg.lib.kamino_set_state(s._h, field, host.ctypes.data, host.strides[0]))
            dense = s.get_state(field)
            assert np.array_equal(dense, host[:, :npp])
            back = np.full((rows, npp + pad), -7.0, np.float32)
            kg.check(kg.lib.kamino_get_state(s._h, field, back.ctypes.data, back.strides[0]))
            assert np.array_equal(back[:, :npp], host[:, :npp]) and (back[:, npp:] == -7.0).all()
        small = np.zeros((nt, npp - 1), np.float32)
        assert kg.lib.kamino_set_state(s._h, kg.U_PHI, small.ctypes.data, small.strides[0]) == kg.ERR_INVALID


def test_device_pointer_copies(kg):
    torch = pytest.importorskip("torch")
    nt, npp = 64, 128
    st = kg.make_initial_state(nt, lmax=8, seed=4)
    with solver(kg, nt) as a, solver(kg, nt) as b:
        a.load(st)
        d = {f: torch.empty((nt - (f == kg.U_THETA), npp), dtype=torch.float32, device="cuda")
             for f in (kg.U_PHI, kg.U_THETA, kg.THICKNESS)}
        for f, t in d.items():
            kg.check(kg.lib.kamino_get_state_device(a._h, f, ctypes.c_void_p(t.data_ptr()), t.stride(0) * 4))
        a.synchronize()
        for f, t in d.items():
            kg.check(kg.lib.kamino_set_state_device(b._h, f, ctypes.c_void_p(t.data_ptr()), t.stride(0) * 4))
        b.synchronize()
        a.step_n(2)
        b.step_n(2)
        fa, fb = a.fields(), b.fields()
    for k in ("u_phi", "u_theta", "thickness"):
        assert np.array_equal(fa[k], fb[k])


def test_step_host_with_a_pitch(kg):
    nt, npp, pad = 64, 128, 8
    st = kg.make_initial_state(nt, lmax=8, seed=5)

    def padded(a):
        out = np.zeros((a.shape[0], npp + pad), np.float32)
        out[:, :npp] = a
        return out

    ins = [padded(st[k]) for k in ("u_phi", "u_theta", "thickness")]
    outs = [np.zeros_like(a) for a in ins]
    with solver(kg, nt) as a, solver(kg, nt) as b:
        kg.check(kg.lib.kamino_step_host(a._h, 0.005, *[x.ctypes.data for x in ins], *[x.ctypes.data for x in outs],
                                         ins[0].strides[0]))
        b.load(st)
        b.stepForward()
        want = b.fields()
    for o, k in zip(outs, ("u_phi", "u_theta", "thickness")):
        assert np.array_equal(o[:, :npp], want[k]) and not o[:, npp:].any()


def test_run_frames_takes_the_reference_step_count(kg):
    st = kg.make_initial_state(64, lmax=8, seed=6)
    with solver(kg, frame_dt=0.0123) as a, solver(kg) as b:
        a.load(st)
        b.load(st)
        n = a.run_frames(4)
        assert n == kg.frame_steps(0.005, 0.0123, 4)
        b.step_n(n)
        assert a.time_elapsed() == b.time_elapsed()
        fa, fb = a.fields(), b.fields()
    for k in ("u_phi", "u_theta", "thickness"):
        assert np.array_equal(fa[k], fb[k])
