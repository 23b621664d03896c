"""Host logic without a GPU: configKamino.txt parsing (main.cu:17-45), the
particle-count rule (KaminoParticles.cu:20-26), the frame-loop step rule
(KaminoCore.cu:886-895) and the seeded synthetic initial states."""
import math

import numpy as np
import pytest


def test_parse_config_positional_fields(kg, tmp_path):
    p = tmp_path / "configKamino.txt"
    p.write_text("2.5 256 4.0 0.004 0.0416667 30\n0.0 1 2 3 4\nout/frame parts/frame null sol.png null\n")
    c = kg.parse_config(p)
    assert c.radius == 2.5 and c.n_theta == 256 and c.frames == 30
    assert c.particle_density == 4.0
    assert abs(c.dt - 0.004) < 1e-9 and abs(c.frame_dt - 0.0416667) < 1e-7
    assert (c.B, c.C, c.D, c.E) == (1, 2, 3, 4)
    assert c.grid_path == b"out/frame" and c.particle_path == b"parts/frame"
    assert c.density_image == b"" and c.color_image == b""
    assert c.solid_image == b"sol.png"
    assert c.n_particles == -1  # counted from the density, as the reference does
    assert kg.particle_count(c) == 2 * int(math.sqrt(4.0) * 256) ** 2


def test_parse_config_errors(kg, tmp_path):
    with pytest.raises(kg.KaminoError) as e:
        kg.parse_config(tmp_path / "missing.txt")
    assert e.value.code == 4
    bad = tmp_path / "bad.txt"
    bad.write_text("1.0 128 2.0\n")
    with pytest.raises(kg.KaminoError) as e:
        kg.parse_config(bad)
    assert e.value.code == 4


@pytest.mark.parametrize("density,nt", [(1.0, 128), (2.0, 512), (200.0, 128), (0.5, 64)])
def test_particle_count_rule(kg, density, nt):
    c = kg.default_config(n_theta=nt, particle_density=density, n_particles=-1)
    # the density reaches KaminoParticles through a size_t parameter
    # (KaminoSolver.cu:278): its fraction is dropped, so 0.5 makes none
    lin = np.float32(np.sqrt(np.float32(int(np.float32(density)))))
    per = int(np.float32(lin * np.float32(nt)))
    assert kg.particle_count(c) == per * 2 * per


def reference_frame_steps(dt, DT, frames):
    """Kamino::run's loop (KaminoCore.cu:886-895) in float32."""
    T = np.float32(0.0)
    dt, DT = np.float32(dt), np.float32(DT)
    n = 0
    for i in range(1, frames + 1):
        while T < np.float32(i) * DT:
            n += 1
            T = np.float32(T + dt)
        n += 1
        T = np.float32(i) * DT
    return n


@pytest.mark.parametrize("dt,DT,frames", [(0.005, 1 / 24, 10), (0.001, 0.01, 7), (0.1, 0.05, 3), (0.003, 0.03, 50)])
def test_frame_step_rule(kg, dt, DT, frames):
    assert kg.frame_steps(dt, DT, frames) == reference_frame_steps(dt, DT, frames)


def test_initial_state_is_seeded_and_deterministic(kg):
    a = kg.make_initial_state(64, lmax=8, seed=5, n_particles=1000)
    b = kg.make_initial_state(64, lmax=8, seed=5, n_particles=1000)
    c = kg.make_initial_state(64, lmax=8, seed=6, n_particles=1000)
    for k in ("u_phi", "u_theta", "thickness", "particles"):
        assert np.array_equal(a[k], b[k])
        assert not np.array_equal(a[k], c[k])
    assert a["u_phi"].shape == (64, 128) and a["u_theta"].shape == (63, 128)
    vmax = max(np.abs(a["u_phi"]).max(), np.abs(a["u_theta"]).max())
    assert abs(vmax - 1.0) < 1e-6  # rescaled to max|u| = 1
    t = a["thickness"]
    assert t.min() >= 0.95 and t.max() <= 1.05 and abs(t.mean() - 1.0) < 5e-3


def test_particles_uniform_on_the_sphere(kg):
    p = kg.make_initial_state(32, lmax=2, seed=9, n_particles=200000)["particles"].astype(np.float64)
    phi, theta = p[:, 0], p[:, 1]
    assert phi.min() >= 0 and phi.max() <= 2 * np.pi + 1e-6
    assert theta.min() >= 0 and theta.max() <= np.pi + 1e-6
    # uniform on the sphere: cos(theta) ~ U(-1, 1), phi ~ U(0, 2 pi)
    assert abs(np.cos(theta).mean()) < 0.01 and abs(np.var(np.cos(theta)) - 1 / 3) < 0.01
    assert abs(phi.mean() - np.pi) < 0.02


def test_initial_velocity_is_a_curl(kg, orc):
    """u = curl(psi) at the staggered points: the reference's discrete
    divergence (fillDivergenceKernel) of it is O(h^2) relative to |u|/h."""
    for nt in (32, 64):
        st = kg.make_initial_state(nt, lmax=6, seed=3)
        o = orc.Oracle(nt)
        div = o.divergence(st["u_phi"], st["u_theta"])
        h = np.pi / nt
        scale = np.sqrt((st["u_phi"].astype(np.float64) ** 2).mean()) / h
        # interior rows (the pole rows use the reference's one-sided closure)
        ratio = np.sqrt((div[2:-2] ** 2).mean()) / scale
        assert ratio < 5 * h * h, (nt, ratio)


def test_vortex_is_recorded(kg):
    st = kg.make_initial_state(64, lmax=4, seed=2, vortex=True, vortex_sigma=0.1)
    th, ph, amp = st["vortex"]
    assert 0 <= th <= np.pi and 0 <= ph < 2 * np.pi and amp != 0
