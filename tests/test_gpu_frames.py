"""Frame output (.bgeo) on the GPU against the oracle.

The device pack kernels build write_data_bgeo's and write_particles_bgeo's
point records (KaminoSolver.cu:284-423) in the file's byte order.  Against
the oracle's file image of the same state: header and trailer bytes equal,
w and density bit-exact, positions and velocities within a few float ulps
(only sinf / cosf differ between the device and the host C library).
Capture order and the frame loop with output (Kamino::run, KaminoCore.cu:
860-912) are checked bit for bit against frames written one by one.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

POS_ULPS = 4e-7  # |device - host| of a coordinate, relative to the radius
VEL_ULPS = 4e-7  # of a velocity component, relative to max |v|


def make_solver(kg, nt, npart=0, seed=11, radius=1.0, frame_dt=None):
    st = kg.make_initial_state(nt, lmax=8, seed=seed, n_particles=npart, radius=radius)
    cfg = kg.default_config(n_theta=nt, radius=radius, dt=0.005, n_particles=npart)
    if frame_dt is not None:
        cfg.frame_dt = frame_dt
    s = kg.KaminoSolver(config=cfg)
    s.load(st)
    return s


def check_grid_image(orc, img, s, radius):
    f = s.fields()
    want_rec = orc.frame_grid_records(f["u_phi"], f["u_theta"], f["thickness"], s.nTheta, radius)
    want = orc.bgeo_image(want_rec, orc.GRID_ATTRS)
    assert len(img) == len(want) == s.frame_bytes()
    attrs, rec = orc.read_bgeo(img)
    nrec = rec.shape[0] * rec.shape[1] * 4
    assert img[:len(img) - nrec - 2] == want[:len(want) - nrec - 2]  # header
    assert img[-2:] == b"\x00\xff"
    assert np.array_equal(rec[:, 3], want_rec[:, 3]) and np.array_equal(rec[:, 7], want_rec[:, 7])
    assert np.abs(rec[:, :3] - want_rec[:, :3]).max() <= POS_ULPS * radius
    vmax = np.abs(want_rec[:, 4:7]).max()
    assert np.abs(rec[:, 4:7] - want_rec[:, 4:7]).max() <= VEL_ULPS * vmax


@pytest.mark.parametrize("nt,radius", [(32, 1.0), (256, 1.5), (1024, 1.0), (2048, 1.0)])
def test_grid_frame_matches_oracle(kg, orc, nt, radius):
    with make_solver(kg, nt, radius=radius) as s:
        s.step_n(3)
        img = s.write_frame(kg.FRAME_GRID)
        check_grid_image(orc, img, s, radius)


def test_particle_frame_matches_oracle(kg, orc):
    nt, npart = 128, 4096
    with make_solver(kg, nt, npart=npart, radius=2.0) as s:
        s.step_n(5)
        img = s.write_frame(kg.FRAME_PARTICLES)
        part = s.get_state(kg.PARTICLES)
    want_rec = orc.frame_particle_records(part, 2.0)
    want = orc.bgeo_image(want_rec, orc.PARTICLE_ATTRS)
    assert len(img) == len(want)
    attrs, rec = orc.read_bgeo(img)
    assert attrs == orc.PARTICLE_ATTRS
    assert img[:len(img) - rec.nbytes - 2] == want[:len(want) - rec.nbytes - 2]
    assert np.array_equal(rec[:, 3:], want_rec[:, 3:])
    assert np.abs(rec[:, :3] - want_rec[:, :3]).max() <= POS_ULPS * 2.0


def test_captures_are_written_oldest_first(kg, orc):
    with make_solver(kg, 64) as s:
        s.capture_frame()
        before = s.fields()
        s.step_n(2)
        s.capture_frame()
        with pytest.raises(kg.KaminoError):  # two wait already
            s.capture_frame()
        first = s.write_frame()
        second = s.write_frame()
        now = s.write_frame()  # nothing waits: the current state
    assert second == now and first != second
    _, rec = orc.read_bgeo(first)
    assert np.array_equal(rec[:, 7], before["thickness"].reshape(-1))


def test_run_frames_bgeo_writes_every_frame(kg, orc, tmp_path):
    nt, frames, frame_dt = 64, 3, 0.012  # 0.012 / 0.005: 3 steps per frame
    with make_solver(kg, nt, npart=512, frame_dt=frame_dt) as s:
        steps = s.run_frames_bgeo(frames, str(tmp_path / "grid_"), str(tmp_path / "part_"))
        last = s.write_frame(kg.FRAME_GRID)
    assert steps == kg.frame_steps(0.005, frame_dt, frames)
    names = sorted(os.listdir(tmp_path))
    assert names == sorted(["grid_%d.bgeo" % i for i in range(frames + 1)] +
                           ["part_%d.bgeo" % i for i in range(frames + 1)])
    # the same frames written one at a time, with the frame loop's step counts
    per_frame = [kg.frame_steps(0.005, frame_dt, i) - kg.frame_steps(0.005, frame_dt, i - 1)
                 for i in range(1, frames + 1)]
    with make_solver(kg, nt, npart=512, frame_dt=frame_dt) as s:
        ref = {0: (s.write_frame(kg.FRAME_GRID), s.write_frame(kg.FRAME_PARTICLES))}
        for i, n in enumerate(per_frame, 1):
            s.step_n(n)
            ref[i] = (s.write_frame(kg.FRAME_GRID), s.write_frame(kg.FRAME_PARTICLES))
        check_grid_image(orc, ref[frames][0], s, 1.0)
    for i in range(frames + 1):
        assert (tmp_path / ("grid_%d.bgeo" % i)).read_bytes() == ref[i][0], i
        assert (tmp_path / ("part_%d.bgeo" % i)).read_bytes() == ref[i][1], i
    assert last == ref[frames][0]


def test_frame_write_reports_io_errors(kg, tmp_path):
    with make_solver(kg, 32, npart=256, frame_dt=0.012) as s:
        with pytest.raises(kg.KaminoError) as e:
            s.write_frame(kg.FRAME_GRID, path=tmp_path / "missing_dir" / "f.bgeo")
        assert e.value.code == kg._lib.ERR_IO and "cannot open" in str(e.value)
        # a frame loop that fails leaves no capture waiting behind it
        with pytest.raises(kg.KaminoError) as e:
            s.run_frames_bgeo(2, str(tmp_path / "missing_dir" / "g_"), str(tmp_path / "p_"))
        assert e.value.code == kg._lib.ERR_IO
        s.run_frames_bgeo(1, str(tmp_path / "g_"), str(tmp_path / "p_"))
        now = s.write_frame(kg.FRAME_GRID)
    assert (tmp_path / "g_1.bgeo").read_bytes() == now


def test_init_particles_uploads_the_reference_placement(kg, orc):
    cfg = kg.default_config(n_theta=64, radius=1.0, dt=0.005, particle_density=2.0, n_particles=-1)
    with kg.KaminoSolver(config=cfg) as s:
        kg.check(kg.lib.kamino_init_particles(s._h, 1))
        got = s.get_state(kg.PARTICLES)
    assert np.array_equal(got.view(np.uint32), orc.ref_particles(2.0, 64, 1).view(np.uint32))


def test_cli_runs_the_reference_frame_loop(kg, orc, tmp_path):
    """`kamino configKamino.txt` (main.cu:4-59, Kamino::run): the files it
    writes equal the library's own frame loop on the same start (FBM velocity,
    the reference's particle placement), bit for bit."""
    import subprocess
    nt, dens, dt, DT, frames = 32, 1.0, 0.005, 0.012, 3
    cfgfile = tmp_path / "configKamino.txt"
    cfgfile.write_text("1.0\n%d\n%g\n%g\n%g\n%d\n0.0 1 1 1 1\n%s\n%s\nnull\nnull\nnull\n"
                       % (nt, dens, dt, DT, frames, tmp_path / "cli_grid_", tmp_path / "cli_part_"))
    exe = os.path.join(os.path.dirname(kg.LIB_PATH), "kamino")
    r = subprocess.run([exe, str(cfgfile)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert "Frame %d is ready" % frames in r.stdout and "Performance:" in r.stdout
    cfg = kg.parse_config(cfgfile)
    with kg.KaminoSolver(config=cfg) as s:
        s.init_fbm()
        kg.check(kg.lib.kamino_init_particles(s._h, 1))
        part0 = s.get_state(kg.PARTICLES)
        s.run_frames_bgeo(frames, str(tmp_path / "lib_grid_"), str(tmp_path / "lib_part_"))
    for i in range(frames + 1):
        for k in ("grid", "part"):
            a = (tmp_path / ("cli_%s_%d.bgeo" % (k, i))).read_bytes()
            assert a == (tmp_path / ("lib_%s_%d.bgeo" % (k, i))).read_bytes(), (k, i)
    _, rec = orc.read_bgeo((tmp_path / "cli_part_0.bgeo").read_bytes())
    want = orc.frame_particle_records(part0, 1.0)
    assert rec.shape[0] == kg.particle_count(cfg) == 2 * 32 * 32
    assert np.abs(rec[:, :3] - want[:, :3]).max() <= POS_ULPS


@pytest.mark.parametrize("w,h,nt", [(100, 37, 64), (256, 128, 64), (3000, 1500, 1024)])
def test_density_image_matches_oracle(kg, orc, w, h, nt):
    """initDensityfromPic (KaminoSolver.cu:243-277) on the device: the
    thickness equals the oracle's mirrored, resampled image averaged over the
    channels, bit for bit."""
    rng = np.random.default_rng(w + h)
    img = rng.integers(0, 256, (h, w, 3), dtype=np.uint8)
    cfg = kg.default_config(n_theta=nt, radius=1.0, dt=0.005, n_particles=0)
    with kg.KaminoSolver(config=cfg) as s:
        s.initDensityfromPic(img)
        got = s.get_state(kg.THICKNESS)
    want = orc.image_density(orc.image_resample(img, 2 * nt, nt))
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_particle_colors_reach_the_particle_frames(kg, orc):
    nt = 32
    rng = np.random.default_rng(9)
    img = rng.integers(0, 256, (45, 70, 3), dtype=np.uint8)
    cfg = kg.default_config(n_theta=nt, radius=1.0, dt=0.005, particle_density=2.0, n_particles=-1)
    with kg.KaminoSolver(config=cfg) as s:
        s.initParticlesfromPic(img)
        part = s.get_state(kg.PARTICLES)
        _, rec = orc.read_bgeo(s.write_frame(kg.FRAME_PARTICLES))
    col = orc.particle_colors(orc.image_resample(img, 2 * nt, nt), part, nt)
    want = orc.written_colors(col)
    assert np.array_equal(rec[:, 7:10].view(np.uint32), want.view(np.uint32))
    assert rec[:-1, 7:10].any(axis=1).mean() > 0.9 and rec[-1, 9] == 0


def write_ppm(path, bgr):
    h, w = bgr.shape[:2]
    path.write_bytes(b"P6\n# test image\n%d %d\n255\n" % (w, h) + np.ascontiguousarray(bgr[..., ::-1]).tobytes())


def test_cli_reads_ppm_images(kg, orc, tmp_path):
    import subprocess
    nt, frames = 32, 2
    rng = np.random.default_rng(12)
    dimg = rng.integers(0, 256, (50, 90, 3), dtype=np.uint8)
    cimg = rng.integers(0, 256, (20, 33, 3), dtype=np.uint8)
    write_ppm(tmp_path / "d.ppm", dimg)
    write_ppm(tmp_path / "c.ppm", cimg)
    cfgfile = tmp_path / "configKamino.txt"
    cfgfile.write_text("1.0 %d 1.0 0.005 0.01 %d 0.0 1 1 1 1 %s %s %s null %s\n"
                       % (nt, frames, tmp_path / "g_", tmp_path / "p_", tmp_path / "d.ppm", tmp_path / "c.ppm"))
    exe = os.path.join(os.path.dirname(kg.LIB_PATH), "kamino")
    r = subprocess.run([exe, str(cfgfile)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert "ignored" not in r.stderr
    cfg = kg.parse_config(cfgfile)
    with kg.KaminoSolver(config=cfg) as s:
        s.init_fbm()
        s.initDensityfromPic(dimg)
        s.initParticlesfromPic(cimg)
        rho0 = s.get_state(kg.THICKNESS)
        s.run_frames_bgeo(frames, str(tmp_path / "lg_"), str(tmp_path / "lp_"))
    for i in range(frames + 1):
        assert (tmp_path / ("g_%d.bgeo" % i)).read_bytes() == (tmp_path / ("lg_%d.bgeo" % i)).read_bytes(), i
        assert (tmp_path / ("p_%d.bgeo" % i)).read_bytes() == (tmp_path / ("lp_%d.bgeo" % i)).read_bytes(), i
    _, rec = orc.read_bgeo((tmp_path / "g_0.bgeo").read_bytes())
    assert np.array_equal(rec[:, 7], rho0.reshape(-1))
    assert np.array_equal(rho0, orc.image_density(orc.image_resample(dimg, 2 * nt, nt)))
    # the Python mirror of Kamino::run writes the same files
    kg.Kamino.from_config(cfgfile, grid_path=str(tmp_path / "kg_"), particle_path=str(tmp_path / "kp_")).run()
    for i in range(frames + 1):
        assert (tmp_path / ("kg_%d.bgeo" % i)).read_bytes() == (tmp_path / ("g_%d.bgeo" % i)).read_bytes(), i
        assert (tmp_path / ("kp_%d.bgeo" % i)).read_bytes() == (tmp_path / ("p_%d.bgeo" % i)).read_bytes(), i


def test_image_arguments_are_checked(kg):
    img = np.zeros((4, 5, 3), np.uint8)
    cfg = kg.default_config(n_theta=32, radius=1.0, dt=0.005, n_particles=0)
    with kg.KaminoSolver(config=cfg) as s:
        for args in ((img.ctypes.data, 0, 4, 15), (img.ctypes.data, 5, 4, 14), (None, 5, 4, 15)):
            assert kg.lib.kamino_init_density_image(s._h, *args) == kg.ERR_INVALID
            assert "image" in kg._lib.last_error()
        # no particles: nothing to colour, not an error
        kg.check(kg.lib.kamino_init_particle_colors_image(s._h, img.ctypes.data, 5, 4, 15))
        kg.check(kg.lib.kamino_init_density_image(s._h, img.ctypes.data, 5, 4, 15))
        assert not s.get_state(kg.THICKNESS).any()
