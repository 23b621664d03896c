"""Checkpoint and resume (kamino_save_state / kamino_load_state): a run
resumed from a checkpoint continues bit for bit like the uninterrupted run,
and damaged or mismatched files are refused with a status."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def solver(kg, nt=64, npart=512, dt=0.005, radius=1.0, flags=0):
    cfg = kg.default_config(n_theta=nt, radius=radius, dt=dt, n_particles=npart, flags=flags)
    return kg.KaminoSolver(config=cfg)


def test_resume_continues_bitwise(kg, tmp_path):
    st = kg.make_initial_state(64, lmax=8, seed=21, n_particles=512)
    path = tmp_path / "state.bin"
    with solver(kg) as a:
        a.load(st)
        a.step_n(7)
        a.save_state(path)
        a.step_n(5)
        want = a.fields()
        t_want = a.time_elapsed()
    with solver(kg) as b:
        b.load_state(path)
        assert b.time_elapsed()[1] == 7
        b.step_n(5)
        got = b.fields()
        assert b.time_elapsed() == t_want
    for k in ("u_phi", "u_theta", "thickness", "particles"):
        assert np.array_equal(got[k].view(np.uint32), want[k].view(np.uint32)), k


def test_damaged_and_mismatched_files_are_refused(kg, tmp_path):
    path = tmp_path / "state.bin"
    with solver(kg) as a:
        a.load(kg.make_initial_state(64, lmax=8, seed=22, n_particles=512))
        a.save_state(path)
    raw = bytearray(path.read_bytes())
    bad = tmp_path / "bad.bin"
    raw[1000] ^= 0x40
    bad.write_bytes(bytes(raw))
    short = tmp_path / "short.bin"
    short.write_bytes(path.read_bytes()[:-9])
    with solver(kg) as b:
        for p, code, text in ((bad, kg._lib.ERR_IO, "checksum"), (short, kg._lib.ERR_IO, "complete"),
                              (tmp_path / "none.bin", kg._lib.ERR_IO, "cannot open")):
            with pytest.raises(kg.KaminoError) as e:
                b.load_state(p)
            assert e.value.code == code and text in str(e.value)
    with solver(kg, nt=32) as c:
        with pytest.raises(kg.KaminoError) as e:
            c.load_state(path)
        assert e.value.code == kg.ERR_INVALID and "nTheta" in str(e.value)
    with solver(kg, dt=0.002) as d:
        with pytest.raises(kg.KaminoError) as e:
            d.load_state(path)
        assert e.value.code == kg.ERR_INVALID and "dt" in str(e.value)
    for flags in (kg.F_REFERENCE_ROUNDING, kg.F_PARTICLE_RK2):
        with solver(kg, flags=flags) as f:
            with pytest.raises(kg.KaminoError) as e:
                f.load_state(path)
            assert e.value.code == kg.ERR_INVALID and "flags" in str(e.value)
