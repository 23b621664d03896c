"""Batched and served forms on the GPU.  The batched persistent kernels run
the same per-tile device code as the one-sphere kernels, so every sphere's
fields must be bit-identical alone, in a batch, and in the server's mix."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MIX = [(32, 0.7, 1, 0), (64, 1.3, 2, 256), (128, 1.0, 3, 0), (256, 1.9, 4, 1024), (64, 0.5, 5, 0),
       (512, 1.1, 6, 0), (32, 2.0, 7, 512)]


def solo(kg, nt, R, seed, npart, steps, dt=0.005, flags=0):
    st = kg.make_initial_state(nt, lmax=8, seed=seed, radius=R, n_particles=npart)
    cfg = kg.default_config(n_theta=nt, radius=R, dt=dt, n_particles=npart, flags=flags)
    with kg.KaminoSolver(config=cfg) as s:
        s.load(st)
        s.step_n(steps)
        return st, s.fields()


@pytest.mark.parametrize("flags", [0, 16])
def test_batch_matches_solo_bitwise(kg, flags):
    from kaminogpu_gb300.batch import Batch
    cfgs = [kg.default_config(n_theta=nt, radius=R, dt=0.005, n_particles=npart, flags=flags)
            for nt, R, seed, npart in MIX]
    with Batch(cfgs) as b:
        states = []
        for i, (nt, R, seed, npart) in enumerate(MIX):
            st = kg.make_initial_state(nt, lmax=8, seed=seed, radius=R, n_particles=npart)
            b.load(i, st)
            states.append(st)
        b.step_n(5)
        for i, (nt, R, seed, npart) in enumerate(MIX):
            _, want = solo(kg, nt, R, seed, npart, 5, flags=flags)
            for k, f in (("u_phi", kg.U_PHI), ("u_theta", kg.U_THETA), ("thickness", kg.THICKNESS)):
                got = b.get_state(i, f)
                assert np.array_equal(got.view(np.uint32), want[k].view(np.uint32)), (i, k)
            if npart:
                got = b.get_state(i, kg.PARTICLES)
                assert np.array_equal(got.view(np.uint32), want["particles"].view(np.uint32)), (i, "particles")


def test_autotune_keeps_the_state(kg):
    from kaminogpu_gb300.batch import Batch
    mix = MIX[:5]
    cfgs = [kg.default_config(n_theta=nt, radius=R, dt=0.005, n_particles=npart) for nt, R, seed, npart in mix]
    with Batch(cfgs) as b:
        for i, (nt, R, seed, npart) in enumerate(mix):
            b.load(i, kg.make_initial_state(nt, lmax=8, seed=seed, radius=R, n_particles=npart))
        b.step_n(2)
        chosen = b.autotune(reps=2)
        assert set(chosen) == {"adv_cta_per_sm", "fft_cta_per_sm", "solve_cta_per_sm", "adv_tiles_per_item"}
        b.step_n(3)
        for i, (nt, R, seed, npart) in enumerate(mix):
            _, want = solo(kg, nt, R, seed, npart, 5)
            got = b.get_state(i, kg.U_PHI)
            assert np.array_equal(got.view(np.uint32), want["u_phi"].view(np.uint32)), i


def test_server_results_same_alone_and_in_the_mix(kg, orc):
    from kaminogpu_gb300.batch import Server
    srv = Server(budget_bytes=8 << 30, steps_per_round=7)
    reqs = []
    plan = [(64, 21, 11), (128, 22, 30), (32, 23, 5), (256, 24, 17), (64, 25, 40), (512, 26, 9), (128, 27, 3)]
    for k, (nt, seed, steps) in enumerate(plan):
        st = kg.make_initial_state(nt, lmax=8, seed=seed)
        cfg = kg.default_config(n_theta=nt, radius=1.0, dt=0.002)
        # staggered arrivals: later requests join while earlier ones run
        reqs.append((srv.submit(cfg, st, steps, arrival=srv.now() + 0.002 * k), nt, seed, steps))
    done = 0
    deadline = time.time() + 120
    while done < len(plan) and time.time() < deadline:
        done += srv.poll()
    assert done == len(plan)
    for rid, nt, seed, steps in reqs:
        got = srv.fetch(rid)
        _, want = solo(kg, nt, 1.0, seed, 0, steps, dt=0.002)
        for k in ("u_phi", "u_theta", "thickness"):
            assert orc.rel_l2(got[k], want[k]) <= 1e-5, (rid, k)
            assert np.array_equal(got[k].view(np.uint32), want[k].view(np.uint32)), (rid, k)
    st = srv.stats()
    assert st["completed"] == len(plan) and st["p99_latency_s"] >= st["p50_latency_s"] > 0
    # the breakdown: the nTheta=512 request ran alone, the rest in batched rounds
    cells = sum(nt * 2 * nt * steps for nt, _, steps in plan)
    solo_cells = sum(nt * 2 * nt * steps for nt, _, steps in plan if nt >= 512)
    assert st["cell_steps"] == cells and st["solo_cell_steps"] == solo_cells
    assert st["batched_cell_steps"] == cells - solo_cells and st["batched_rounds"] > 0
    assert st["batched_round_seconds"] > 0 and st["solo_seconds"] > 0 and st["poll_seconds"] > 0
    srv.close()


def test_server_admission_respects_the_budget(kg):
    from kaminogpu_gb300.batch import Server
    probe = kg.KaminoSolver(config=kg.default_config(n_theta=128, radius=1.0, dt=0.002))
    one = probe.device_bytes()
    probe.close()
    srv = Server(budget_bytes=int(2.5 * one), steps_per_round=5)
    for k in range(6):
        st = kg.make_initial_state(128, lmax=4, seed=40 + k)
        srv.submit(kg.default_config(n_theta=128, radius=1.0, dt=0.002), st, 12)
    done = 0
    peak_resident = 0
    deadline = time.time() + 120
    while done < 6 and time.time() < deadline:
        done += srv.poll()
        s = srv.stats()
        peak_resident = max(peak_resident, s["resident"])
    s = srv.stats()
    assert done == 6 and peak_resident <= 2 and s["peak_resident_bytes"] <= int(2.5 * one)
    big = kg.make_initial_state(512, lmax=4, seed=1)
    srv.submit(kg.default_config(n_theta=512, radius=1.0, dt=0.002), big, 3)
    with pytest.raises(kg.KaminoError) as e:
        for _ in range(10):
            srv.poll()
    assert e.value.code == kg.ERR_BUDGET
    srv.close()


def test_solvers_of_every_size_coexist(kg):
    """Launch limits are process-wide per kernel: creating a sphere of one
    size must not break stepping a sphere of another created before it."""
    sizes = [32, 256, 64, 1024, 128, 512]
    solvers = []
    for k, nt in enumerate(sizes):
        st = kg.make_initial_state(nt, lmax=4, seed=60 + k)
        s = kg.KaminoSolver(config=kg.default_config(n_theta=nt, radius=1.0, dt=0.002))
        s.load(st)
        solvers.append(s)
    for s in solvers:
        s.step_n(2)
    for k, (nt, s) in enumerate(zip(sizes, solvers)):
        st = kg.make_initial_state(nt, lmax=4, seed=60 + k)
        with kg.KaminoSolver(config=kg.default_config(n_theta=nt, radius=1.0, dt=0.002)) as ref:
            ref.load(st)
            ref.step_n(2)
            a, b = s.fields(), ref.fields()
        for key in ("u_phi", "u_theta", "thickness"):
            assert np.array_equal(a[key].view(np.uint32), b[key].view(np.uint32)), (nt, key)
        s.close()


@pytest.mark.parametrize("fp64", [0, 4])
def test_batch_matches_solo_bitwise_large(kg, fp64):
    """The largest sphere sizes of the served mix (nTheta 512 and 1024)."""
    from kaminogpu_gb300.batch import Batch
    spheres = [(1024, 1.0, 31), (512, 0.8, 32)]
    cfgs = [kg.default_config(n_theta=nt, radius=R, dt=0.002, fp64_modes=fp64) for nt, R, _ in spheres]
    with Batch(cfgs) as b:
        for i, (nt, R, seed) in enumerate(spheres):
            b.load(i, kg.make_initial_state(nt, lmax=16, seed=seed, radius=R))
        b.step_n(3)
        for i, (nt, R, seed) in enumerate(spheres):
            st = kg.make_initial_state(nt, lmax=16, seed=seed, radius=R)
            with kg.KaminoSolver(config=cfgs[i]) as s:
                s.load(st)
                s.step_n(3)
                want = s.fields()
            bad = [k for k, f in (("u_phi", kg.U_PHI), ("u_theta", kg.U_THETA), ("thickness", kg.THICKNESS))
                   if not np.array_equal(b.get_state(i, f).view(np.uint32), want[k].view(np.uint32))]
            assert not bad, (nt, bad)

