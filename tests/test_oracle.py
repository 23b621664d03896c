"""The oracle (test infrastructure) pinned before it is trusted:
* its FFT/solve/synthesis against numpy's FFT and a dense solve,
* its reference-arithmetic index map against an independent numpy
  restatement, and bit-exact against the reference's own validateCoord run
  on a GB300 (tests/golden/ref_index.npz, made by make_golden.py),
* its FP64 stages and steps against the reference's own kernels' outputs
  (tests/golden/ref_step.npz) within the reference's FP32 error."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_projection_solves_the_reference_mode_systems(kg, orc):
    """p satisfies A U_{i-1} + B U_i + C U_{i+1} = c_m for every m >= 1
    (precomputeABCKernel, KaminoSolver.cu:128-159), c_m = rfft(div)/nPhi."""
    nt, npp = 32, 64
    rng = np.random.default_rng(0)
    u = rng.standard_normal((nt, npp)).astype(np.float32)
    v = rng.standard_normal((nt - 1, npp)).astype(np.float32)
    o = orc.Oracle(nt)
    o.set_state(0, u)
    o.set_state(1, v)
    div = o.divergence()
    o.projection()
    p = o.get_state(3)
    h = np.pi / nt
    th = (np.arange(nt) + 0.5) * h
    P = np.fft.rfft(p, axis=1) / npp
    c = np.fft.rfft(div, axis=1) / npp
    for m in range(1, nt + 1):
        A = 1 / h ** 2 - np.cos(th) / 2 / h / np.sin(th)
        C = 1 / h ** 2 + np.cos(th) / 2 / h / np.sin(th)
        B = -2 / h ** 2 - m * m / np.sin(th) ** 2
        B[0] += A[0]
        A[0] = 0
        B[-1] += C[-1]
        C[-1] = 0
        x = P[:, m]
        lhs = B * x
        lhs[1:] += A[1:] * x[:-1]
        lhs[:-1] += C[:-1] * x[1:]
        assert np.abs(lhs - c[:, m]).max() <= 1e-10 * np.abs(c[:, m]).max(), m
    assert np.abs(p.mean(axis=1)).max() < 1e-12  # the m = 0 mode is dropped


def np_ref_index(kind, phi, theta, nt):
    """Independent restatement of KaminoCore.cu:38-52 with numpy scalars."""
    f32, f64 = np.float32, np.float64
    h = f32(np.pi / nt)
    offp = (-0.5, 0.0, 0.0)[kind]
    offt = (0.5, 1.0, 0.5)[kind]
    out = np.zeros((len(phi), 4), np.int64)
    for k in range(len(phi)):
        p = f32(f64(phi[k]) - f64(h) * offp)
        t = f32(f64(theta[k]) - f64(h) * offt)
        ret = f32(1)
        t = f32(f64(t) - int(np.floor(f32(f64(t) / (2 * np.pi)))) * (2 * np.pi))
        if f64(t) > np.pi:
            t = f32(2 * np.pi - f64(t))
            p = f32(f64(p) + np.pi)
            ret = -ret
        if t < 0:
            t = -t
            p = f32(f64(p) + np.pi)
            ret = -ret
        p = f32(f64(p) - int(np.floor(f32(f64(p) / (2 * np.pi)))) * (2 * np.pi))
        inv = f32(1.0 / f64(h))
        ip, it = int(np.floor(f32(p * inv))), int(np.floor(f32(t * inv)))
        pole_row = nt - 2 if kind == 1 else nt - 1
        out[k] = (ip % (2 * nt), it, ret == -1, (it == 0 and ret == -1) or it == pole_row)
    return out


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_ref_index_restatement_matches_numpy(orc, kind):
    from points import index_points
    phi, theta = index_points(64, n_random=3000, seed=kind)
    sel = np.random.default_rng(kind).choice(len(phi), 6000, replace=False)
    got, _ = orc.ref_index(kind, phi[sel], theta[sel], 64)
    want = np_ref_index(kind, phi[sel], theta[sel], 64)
    assert np.array_equal(got.astype(np.int64), want)


def _golden(name):
    path = os.path.join(GOLDEN, name)
    if not os.path.exists(path):
        pytest.fail("golden file %s missing; run tests/golden/make_golden.py on a GPU" % path)
    return np.load(path)


@pytest.mark.parametrize("nt", [32, 1024])
def test_ref_index_bit_exact_vs_reference_validatecoord(orc, nt):
    g = _golden("ref_index.npz")
    phi, theta = g["phi_%d" % nt], g["theta_%d" % nt]
    for kind in (0, 1, 2):
        got, _ = orc.ref_index(kind, phi, theta, nt)
        assert np.array_equal(got, g["index_%d_%d" % (nt, kind)]), kind
    p, t, c = orc.ref_wrap(phi, theta, nt)
    assert np.array_equal(p.view(np.uint32), g["wrap_phi_%d" % nt].view(np.uint32))
    assert np.array_equal(t.view(np.uint32), g["wrap_theta_%d" % nt].view(np.uint32))
    assert np.array_equal(c, g["cells_%d" % nt])


# Relative L2 bounds of the FP64 restatement against the reference's FP32
# kernels, per stage and field (u_phi, u_theta, thickness), each a few times
# what the fixtures show at nTheta = 32 and 64: the advection and the
# projection agree to FP32 rounding (~1e-6); the geometric stage's u_phi
# carries the reference's FP32 Cardano root, which cancels near the equator
# (~1.7e-4), and so does every whole step; the geometric stage leaves the
# thickness untouched (exactly equal).
ORACLE_VS_REF_TOL = {
    "advection": (5e-6, 5e-6, 1e-6),
    "geometric": (5e-4, 5e-7, 0.0),
    "projection": (5e-6, 5e-6, 0.0),
    "step": (6e-4, 3e-4, 1e-5),
}


@pytest.mark.parametrize("nt", [32, 64])
def test_fp64_oracle_vs_reference_kernels(orc, nt):
    """The FP64 restatement against the reference's FP32 kernels, stage by
    stage and after 1 and 3 steps, within the reference's own FP32 error
    (ORACLE_VS_REF_TOL); particles within 1e-5 rad (p99)."""
    g = _golden("ref_step.npz")
    pre = "nt%d_" % nt
    nt_, dt, npart, seed = g[pre + "meta"]
    st = {k: g[pre + "in_" + k] for k in ("u_phi", "u_theta", "thickness", "particles")}
    for stage in ("advection", "geometric", "projection"):
        o = orc.Oracle(nt, 1.0, dt, 0, int(npart))
        o.load(st)
        getattr(o, stage)()
        f = o.fields()
        for k, tol in zip(("u_phi", "u_theta", "thickness"), ORACLE_VS_REF_TOL[stage]):
            err = orc.rel_l2(g[pre + stage + "_" + k], f[k])
            assert err <= tol, (stage, k, err, tol)
    for n in (1, 3):
        o = orc.Oracle(nt, 1.0, dt, 0, int(npart))
        o.load(st)
        o.step(n)
        f = o.fields()
        for k, tol in zip(("u_phi", "u_theta", "thickness"), ORACLE_VS_REF_TOL["step"]):
            err = orc.rel_l2(g[pre + "step%d_" % n + k], f[k])
            assert err <= tol, (n, k, err, tol)
        d = np.abs(g[pre + "step%d_particles" % n].astype(np.float64) - f["particles"])
        d[:, 0] = np.minimum(d[:, 0], 2 * np.pi - d[:, 0])
        assert np.percentile(d, 99) < 1e-5, (n, np.percentile(d, 99))


def _py_fbm_init(nt, radius=1.0):
    """KaminoSolver::initialize_velocity written a second time, in Python:
    np.float32 for the reference's float (fReal) operations, Python floats
    for its double ones (KaminoInitializer.cu:3-134)."""
    import math
    f32 = np.float32

    def rand(x, y):  # vec2 components are double
        dot = f32(float(x) * 12.9898 + float(y) * 4.1414)
        val = f32(math.sin(float(dot) * 43758.5453))
        return f32(val - f32(math.floor(val)))

    def lerp(a, b, t):
        return f32((1.0 - float(t)) * float(a) + float(f32(t * b)))

    def noise2(x, y):
        ix, iy = f32(math.floor(x)), f32(math.floor(y))
        fx, fy = f32(x - ix), f32(y - iy)
        v1, v2 = rand(ix, iy), rand(f32(ix + f32(1)), iy)
        v3, v4 = rand(ix, f32(iy + f32(1))), rand(f32(ix + f32(1)), f32(iy + f32(1)))
        return lerp(lerp(v1, v2, fx), lerp(v3, v4, fx), fy)

    def fbm(x, y):
        total = f32(0)
        for i in range(4):
            freq, amp = f32(2.0 ** i), f32(0.5 ** i)
            total = f32(total + f32(amp * noise2(f32(f32(x * freq) / f32(0.15)), f32(f32(y * freq) / f32(0.5)))))
        return f32(f32(f32(0.5) * total) / f32(2))

    h = f32(math.pi / nt)
    np_, h2, rg, gain = 2 * nt, f32(h / f32(2)), f32(f32(radius) * h), f32(4096.0 / (2 * nt))
    u = np.empty((nt, np_), np.float32)
    v = np.empty((nt - 1, np_), np.float32)
    for j in range(nt):
        for i in range(np_):
            if i > 0:
                rx, lx = f32(f32(f32(i) * h) + h2), f32(f32(f32(i) * h) - h2)
            else:
                rx, lx = h2, f32(2 * math.pi - float(h2))
            uy, ly = f32(f32(j + 1) * h), f32(f32(j) * h)
            dl = f32(f32(fbm(rx, uy) - fbm(rx, ly)) / rg)
            dr = f32(f32(fbm(lx, uy) - fbm(lx, ly)) / rg)
            u[j, i] = f32(f32(float(f32(dl + dr)) / 2.0) * gain)
    for j in range(1, nt):
        for i in range(np_):
            rx, lx = f32(f32(i + 1) * h), f32(f32(i) * h)
            jh = f32(f32(j) * h)
            up, dn = f32(jh + h2), f32(jh - h2)
            du = f32(-f32(fbm(rx, up) - fbm(lx, up)) / rg)
            dd = f32(-f32(fbm(rx, dn) - fbm(lx, up)) / rg)
            v[j - 1, i] = f32(f32(float(f32(du + dd)) / 2.0) * gain)
    return u, v


def test_fbm_init_restatements_agree(orc):
    """The oracle's C restatement of the reference's FBM velocity initialiser
    against a second one in Python (nTheta = 16), bit for bit."""
    u, v = orc.ref_init_fbm(16, 1.0)
    pu, pv = _py_fbm_init(16, 1.0)
    assert np.all(np.isfinite(u)) and np.all(np.isfinite(v))
    assert np.array_equal(u.view(np.uint32), pu.view(np.uint32))
    assert np.array_equal(v.view(np.uint32), pv.view(np.uint32))
    assert np.abs(u).max() > 0 and np.abs(v).max() > 0


@pytest.mark.parametrize("nt,lmax,vortex,npart", [(32, 8, False, 1000), (256, 16, True, 0), (1024, 32, True, 64)])
def test_oracle_state_generator_matches_the_library(kg, orc, nt, lmax, vortex, npart):
    """The benchmark's CPU arm builds its input with the oracle's copy of the
    seeded state generator (so it never loads the product library); it must
    be the library's state bit for bit."""
    a = orc.make_initial_state(nt, lmax=lmax, seed=3, vortex=vortex, n_particles=npart, radius=1.3)
    b = kg.make_initial_state(nt, lmax=lmax, seed=3, vortex=vortex, n_particles=npart, radius=1.3)
    for k in ("u_phi", "u_theta", "thickness", "particles"):
        assert np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)), k
    assert a["vortex"] == b["vortex"]


@pytest.mark.parametrize("nt", [64, 256])
def test_fbm_restatement_vs_reference_code(orc, nt):
    """The oracle's FBM velocity restatement against the reference's own
    initialize_velocity (KaminoInitializer.cu:3-134 compiled unchanged; the
    fixture is made by tests/golden/make_fbm_golden.py): bit for bit."""
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_fbm.npz"))
    wu, wv = orc.ref_init_fbm(nt, 1.0)
    for got, key in ((wu, "u_phi_%d" % nt), (wv, "u_theta_%d" % nt)):
        ref = g[key]
        assert got.shape == ref.shape
        assert np.array_equal(np.asarray(got, np.float32).view(np.uint32), ref.view(np.uint32)), key
