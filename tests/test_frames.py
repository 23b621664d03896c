"""Frame output (.bgeo) without a GPU: the oracle's restatement of
write_data_bgeo / write_particles_bgeo (KaminoSolver.cu:284-423) against an
independent FP64 numpy form of the same formulas, the file layout round
trip, and argument errors at the C ABI."""
import ctypes
import struct

import numpy as np
import pytest


def numpy_grid_records(u, v, rho, nt, radius):
    """FP64 statement of write_data_bgeo's loop (KaminoSolver.cu:305-353)."""
    npp = 2 * nt
    h = np.float64(np.float32(np.pi / nt))
    i = np.arange(npp)
    j = np.arange(nt)
    ue = np.roll(u, -1, axis=1)  # iEast = i + 1, wrapping at the seam
    uphi = (u.astype(np.float64) + ue) / 2
    jn = np.clip(j - 1, 0, nt - 2)
    js = np.clip(j, 0, nt - 2)
    jn[0] = js[0] = 0
    uth = (v[jn].astype(np.float64) + v[js]) / 2
    th = ((j + 0.5) * h)[:, None] * np.ones((1, npp))
    ph = np.ones((nt, 1)) * (i * h)[None, :]
    rec = np.empty((nt, npp, 8))
    rec[..., 0] = radius * np.sin(th) * np.cos(ph)
    rec[..., 1] = radius * np.cos(th)
    rec[..., 2] = radius * np.sin(th) * np.sin(ph)
    rec[..., 3] = 1.0
    rec[..., 4] = np.cos(th) * np.cos(ph) * uth - np.sin(ph) * uphi
    rec[..., 5] = -np.sin(th) * uth
    rec[..., 6] = np.cos(th) * np.sin(ph) * uth + np.cos(ph) * uphi
    rec[..., 7] = rho
    return rec.reshape(-1, 8)


def test_oracle_grid_records_follow_the_reference_formulas(orc):
    nt, R = 64, 1.7
    rng = np.random.default_rng(5)
    u = rng.standard_normal((nt, 2 * nt)).astype(np.float32)
    v = rng.standard_normal((nt - 1, 2 * nt)).astype(np.float32)
    rho = (1 + 0.05 * rng.uniform(-1, 1, (nt, 2 * nt))).astype(np.float32)
    got = orc.frame_grid_records(u, v, rho, nt, R)
    want = numpy_grid_records(u, v, rho, nt, R)
    assert np.array_equal(got[:, 3], np.ones(nt * 2 * nt, np.float32))
    assert np.array_equal(got[:, 7], rho.reshape(-1))
    assert np.abs(got[:, :3] - want[:, :3]).max() <= 4e-7 * R
    assert np.abs(got[:, 4:7] - want[:, 4:7]).max() <= 4e-7 * np.abs(want[:, 4:7]).max()
    # every point on the sphere; the centred velocity is tangent to it
    assert np.abs(np.linalg.norm(got[:, :3].astype(np.float64), axis=1) - R).max() <= 4e-7 * R
    radial = np.einsum("ij,ij->i", got[:, :3].astype(np.float64), got[:, 4:7]) / R
    assert np.abs(radial).max() <= 1e-6 * np.abs(want[:, 4:7]).max()


def test_oracle_particle_records(orc):
    rng = np.random.default_rng(6)
    n = 1000
    part = np.stack([rng.uniform(0, 2 * np.pi, n), np.arccos(1 - 2 * rng.uniform(0, 1, n))], 1).astype(np.float32)
    rec = orc.frame_particle_records(part, 2.0)
    ph, th = part[:, 0].astype(np.float64), part[:, 1].astype(np.float64)
    want = np.stack([2 * np.sin(th) * np.cos(ph), 2 * np.cos(th), 2 * np.sin(th) * np.sin(ph)], 1)
    assert np.abs(rec[:, :3] - want).max() <= 1e-6
    assert np.array_equal(rec[:, 3], np.ones(n, np.float32))
    assert not rec[:, 4:].any()


def test_bgeo_layout_round_trip(orc):
    rec = np.arange(3 * 8, dtype=np.float32).reshape(3, 8)
    img = orc.bgeo_image(rec, orc.GRID_ATTRS)
    # header: magic, version, counts, then the two attribute definitions
    assert img[:5] == b"BgeoV" and struct.unpack(">i", img[5:9]) == (5,)
    assert struct.unpack(">8i", img[9:41]) == (3, 0, 0, 0, 2, 0, 0, 0)
    assert img[41:44] == b"\x00\x01v" and struct.unpack(">Hi", img[44:50]) == (3, 5)
    assert len(img) == 41 + (2 + 1 + 6 + 12) + (2 + 7 + 6 + 4) + 3 * 32 + 2
    assert img[-2:] == b"\x00\xff"
    attrs, back = orc.read_bgeo(img)
    assert attrs == orc.GRID_ATTRS and np.array_equal(back, rec)
    attrs, back = orc.read_bgeo(orc.bgeo_image(np.zeros((0, 10), np.float32), orc.PARTICLE_ATTRS))
    assert attrs == orc.PARTICLE_ATTRS and back.shape == (0, 10)


def test_frame_entry_points_reject_bad_arguments(kg):
    n = ctypes.c_size_t()
    assert kg.lib.kamino_frame_bytes(None, kg.FRAME_GRID, ctypes.byref(n)) == kg.ERR_INVALID
    assert kg.lib.kamino_frame_bytes(None, 7, ctypes.byref(n)) == kg.ERR_INVALID
    assert "kind" in kg._lib.last_error()
    assert kg.lib.kamino_frame_capture(None, kg.FRAME_GRID) == kg.ERR_INVALID
    assert kg.lib.kamino_frame_write(None, kg.FRAME_GRID, None, None, 0) == kg.ERR_INVALID
    assert kg.lib.kamino_run_frames_bgeo(None, -1, None, None, None) == kg.ERR_INVALID
    assert kg.lib.kamino_frame_time_pack(None, kg.FRAME_GRID, 0, 0, None) == kg.ERR_INVALID
    img = np.zeros((4, 4, 3), np.uint8)
    assert kg.lib.kamino_init_density_image(None, img.ctypes.data, 4, 4, 12) == kg.ERR_INVALID
    assert kg.lib.kamino_init_particle_colors_image(None, img.ctypes.data, 4, 4, 12) == kg.ERR_INVALID
    assert kg.lib.kamino_init_particles(None, 1) == kg.ERR_INVALID
    assert kg.lib.kamino_reference_particles(None, 1, None, 0) == kg.ERR_INVALID


@pytest.mark.parametrize("density,nt,seed", [(1.0, 32, 1), (4.0, 64, 1), (2.0, 64, 7), (3.7, 32, 1)])
def test_reference_particles_match_the_rand_restatement(kg, orc, density, nt, seed):
    """KaminoParticles' jittered grid (KaminoParticles.cu:20-62): the library's
    placement (reentrant random_r) equals the oracle's srand/rand restatement
    bit for bit, and leaves the caller's rand() sequence alone."""
    libc = ctypes.CDLL(None)
    cfg = kg.default_config(n_theta=nt, particle_density=density, n_particles=-1)
    n = kg.particle_count(cfg)
    want = orc.ref_particles(density, nt, seed)
    assert want.shape == (n, 2)
    libc.srand(5)
    first = libc.rand()
    libc.srand(5)
    got = np.empty((n, 2), np.float32)
    kg.check(kg.lib.kamino_reference_particles(ctypes.byref(cfg), seed, got.ctypes.data, n))
    assert libc.rand() == first
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    h = np.float32(np.pi / nt)
    assert got.min() >= 0 and got[:, 1].max() < np.pi + h and got[:, 0].max() < 2 * np.pi + h
    assert kg.lib.kamino_reference_particles(ctypes.byref(cfg), seed, got.ctypes.data, n + 1) == kg.ERR_INVALID


def test_cli_usage_and_config_errors(kg, tmp_path):
    import os
    import subprocess
    exe = os.path.join(os.path.dirname(kg.LIB_PATH), "kamino")
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 255 and "configKamino.txt" in r.stdout
    r = subprocess.run([exe, str(tmp_path / "missing.txt")], capture_output=True, text=True)
    assert r.returncode == 1 and "cannot open config file" in r.stderr
    bad = tmp_path / "bad.txt"
    bad.write_text("1.0 32 1.0\n")
    r = subprocess.run([exe, str(bad)], capture_output=True, text=True)
    assert r.returncode == 1 and "16 whitespace-separated fields" in r.stderr


def numpy_resample(img, dw, dh):
    """Mirrored bilinear resampling at half-pixel centres, edges clamped,
    columns then rows, float32 per operation, round half to even."""
    h, w = img.shape[:2]

    def axis(src, dst, mirror):
        f = ((np.arange(dst) + 0.5) * (src / dst) - 0.5).astype(np.float32)
        s0 = np.floor(f).astype(np.int64)
        a = (f - s0.astype(np.float32)).astype(np.float32)
        a[s0 < 0] = 0
        s0[s0 < 0] = 0
        a[s0 >= src - 1] = 0
        s0[s0 >= src - 1] = src - 1
        s1 = np.minimum(s0 + 1, src - 1)
        return (src - 1 - s0, src - 1 - s1, a) if mirror else (s0, s1, a)

    x0, x1, ax = axis(w, dw, True)
    y0, y1, ay = axis(h, dh, False)
    f = img.astype(np.float32)
    one = np.float32(1)
    bx, by = ax[None, :, None], ay[:, None, None]
    h0 = f[y0][:, x0] * (one - bx) + f[y0][:, x1] * bx
    h1 = f[y1][:, x0] * (one - bx) + f[y1][:, x1] * bx
    return np.clip(np.rint(h0 * (one - by) + h1 * by), 0, 255).astype(np.uint8)


@pytest.mark.parametrize("w,h,dw,dh", [(100, 37, 128, 64), (256, 128, 128, 64), (128, 64, 128, 64),
                                       (31, 300, 64, 32), (1, 1, 64, 32)])
def test_oracle_image_resample(orc, w, h, dw, dh):
    rng = np.random.default_rng(w * h)
    img = rng.integers(0, 256, (h, w, 3), dtype=np.uint8)
    got = orc.image_resample(img, dw, dh)
    assert np.array_equal(got, numpy_resample(img, dw, dh))
    if (w, h) == (dw, dh):  # same size: the mirrored image itself
        assert np.array_equal(got, img[:, ::-1])
    flat = orc.image_resample(np.full((h, w, 3), 77, np.uint8), dw, dh)
    assert (flat == 77).all()
    d = orc.image_density(got)
    assert d.shape == (dh, dw) and d.min() >= 0 and d.max() <= 1


def test_cli_reports_unreadable_images(kg, tmp_path):
    """The executable reads binary PPM images; anything else is reported and
    ignored, as the reference ignores an image it cannot read
    (KaminoSolver.cu:250-254, KaminoParticles.cu:8-11)."""
    import os
    import subprocess
    exe = os.path.join(os.path.dirname(kg.LIB_PATH), "kamino")
    (tmp_path / "d.png").write_bytes(b"\x89PNG\r\n\x1a\n not really")
    (tmp_path / "bad.ppm").write_bytes(b"P6\n4 4\n65535\n" + bytes(96))
    cfg = tmp_path / "configKamino.txt"
    cfg.write_text("1.0 32 1.0 0.005 0.01 0 0.0 1 1 1 1 %s %s %s null %s\n"
                   % (tmp_path / "g_", tmp_path / "p_", tmp_path / "d.png", tmp_path / "bad.ppm"))
    r = subprocess.run([exe, str(cfg)], capture_output=True, text=True, timeout=120)
    assert "density image '%s' ignored" % (tmp_path / "d.png") in r.stderr
    assert "colour image '%s' ignored" % (tmp_path / "bad.ppm") in r.stderr


def test_read_ppm_and_the_kamino_driver_config(kg, tmp_path):
    rng = np.random.default_rng(8)
    img = rng.integers(0, 256, (6, 9, 3), dtype=np.uint8)
    p = tmp_path / "a.ppm"
    p.write_bytes(b"P6\n# comment\n9 6\n255\n" + np.ascontiguousarray(img[..., ::-1]).tobytes())
    assert np.array_equal(kg.read_ppm(p), img)
    p.write_bytes(b"P6\n9 6\n65535\n" + bytes(9 * 6 * 6))
    with pytest.raises(ValueError):
        kg.read_ppm(p)
    k = kg.Kamino(2.0, 64, 3.0, 0.004, 0.02, 7, gridPath="g_", particlePath="p_")
    c = k.config
    assert (c.radius, c.n_theta, c.dt, c.frame_dt, c.frames) == (2.0, 64, 0.004, 0.02, 7)
    assert c.grid_path == b"g_" and c.particle_path == b"p_" and kg.particle_count(c) == 2 * int(np.float32(
        np.sqrt(np.float32(3.0)) * 64)) ** 2
