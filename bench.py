"""Benchmark of the GB300 Kamino step: cell-steps/s at nTheta=1024 x nPhi=2048.

Workload (the precision-form configuration): one sphere, radius 1, nTheta=1024,
nPhi=2048, dt=0.001, seeded stream function with l <= 32 plus one seeded
Gaussian vortex (sigma = 0.1 rad), thickness 1 + 0.05 U(-1,1); FP32 step with
modes |m| <= 4 solved in FP64.  A "step" is one stepForward of that sphere.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

value: device time of K steps (CUDA events on the solver's stream; a 256 MiB
  buffer written and then read between steps, so each step starts from a cold
  and clean L2; the state is 25 MB and would otherwise sit in the 129 MB L2).
e2e:   the same steps through the public C ABI with host buffers: every step
  is one kamino_step_host call, which copies u_phi, u_theta, thickness in
  from pinned host memory, steps, and copies them back (the thickness
  download overlapping the projection).
--impl reference: the reference has no CPU implementation of this path, so
  the reference arm times the CPU port of its step (oracle/, FP64, all host
  threads) on the same configuration, from the same seeded state made by the
  oracle's own generator (the product library is never loaded there), plus
  the reference's own CUDA kernels on this GPU as extra information.
Extra keys of the GPU arm: fp64_modes_0 (every mode in FP32),
  reference_rounding (the same step with the reference's own sampler
  arithmetic, bit-exact index map), config2 (nTheta=512 with 2^20 RK2
  particles), batched (256 spheres), served (closed loop, and Poisson arrivals
  at 200/s for --served-seconds, 60 by default), frame_output, cpu_baseline.
With N > 1 (torchrun), every rank advances its own sphere (replicas; the
path does not shard) and rank 0 prints the aggregate.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NT, DT, LMAX, SEED = 1024, 0.001, 32, 1
METRIC = "cell-steps/s at 1024x2048, batched/served vs plain; p99 latency @1e-5 rel err"
UNIT = "cell-steps/s"
STEP_BYTES_PER_CELL = 56    # algorithmic bytes per cell-step of the whole step (3-pass minimum)
PARTICLE_BYTES = 16         # algorithmic bytes per particle-step: (phi, theta) read and written
DATA = ("synthetic: seeded l<=32 spherical-harmonic stream function + Gaussian vortex (sigma 0.1 rad), "
        "max|u|=1; thickness 1+0.05U(-1,1)")


def workload_config(ws):
    """The `config` both arms print: the workload only, nothing arm-specific."""
    return {"workload": "plain solver, one sphere nTheta=1024 nPhi=2048, radius 1, dt=0.001 (precision form)",
            "n_theta": NT, "n_phi": 2 * NT, "radius": 1.0, "dt": DT, "lmax": LMAX, "vortex_sigma": 0.1,
            "seed": SEED, "fp64_modes": 4,
            "l2": "GPU arm: a 256 MiB buffer written then read before every timed step (cold, clean L2)",
            "parallelism": "replicas" if ws > 1 else "single GPU"}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def init_dist(ws):
    if ws <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group("gloo")
    return dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def committed_traffic():
    """DRAM bytes per k_advect launch from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "k_advect_nt1024.txt")
    try:
        for line in open(path):
            if line.startswith("dram_bytes_per_launch:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


def profiler_range(start):
    """cudaProfilerStart / cudaProfilerStop of the CUDA runtime the library
    uses: an ncu run with --profile-from-start off captures only the launches
    between them; without a profiler attached both do nothing."""
    try:
        import glob
        cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
        rt = ctypes.CDLL(sorted(glob.glob(os.path.join(cuda, "lib64", "libcudart.so*")))[-1])
        (rt.cudaProfilerStart if start else rt.cudaProfilerStop)()
    except Exception:
        pass


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, device):
        self.p = None
        self.device = device

    def __enter__(self):
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device),
                 "--query-gpu=clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.p:
            time.sleep(0.25)
            self.p.terminate()
            try:
                out, _ = self.p.communicate(timeout=5)
                self.lines = [l for l in out.splitlines() if l.strip()]
            except Exception:
                self.lines = []

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, f[2:]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def run_ours(args, ws, rank, local, dist):
    import numpy as np
    import kaminogpu_gb300 as kg

    st = kg.make_initial_state(NT, lmax=LMAX, seed=SEED + rank, vortex=True)
    cfg = kg.default_config(n_theta=NT, radius=1.0, dt=DT, fp64_modes=4, device=local)
    s = kg.KaminoSolver(config=cfg)
    s.load(st)
    C = NT * 2 * NT
    s.step_n(args.warmup)
    s.synchronize()
    # per-kernel timing (events around each launch, cold L2 each step)
    kms = s.time_kernels(reps=max(3, min(args.steps, 10)), flush_l2=True)
    s.load(st)
    s.step_n(args.warmup)
    s.synchronize()
    barrier(dist)
    with Clocks(local) as ck:
        t0 = time.perf_counter()
        ms = s.time_steps(args.steps, flush_l2=True)
        wall = time.perf_counter() - t0
    barrier(dist)
    ms_max = max_over_ranks(dist, ms)
    cells_total = sum_over_ranks(dist, C * args.steps)
    value = cells_total / (ms_max / 1e3)

    # e2e through the C ABI with pinned host buffers
    L = kg.lib
    nbytes = {kg.U_PHI: NT * 2 * NT * 4, kg.U_THETA: (NT - 1) * 2 * NT * 4, kg.THICKNESS: NT * 2 * NT * 4}
    bufs = {}
    for f, n in nbytes.items():
        p = ctypes.c_void_p()
        kg.check(L.kamino_host_alloc(n, ctypes.byref(p)))
        bufs[f] = p
    src = {kg.U_PHI: st["u_phi"], kg.U_THETA: st["u_theta"], kg.THICKNESS: st["thickness"]}
    for f, p in bufs.items():
        ctypes.memmove(p, src[f].ctypes.data, nbytes[f])
    h = s._h
    pitch = 2 * NT * 4
    io = [bufs[kg.U_PHI], bufs[kg.U_THETA], bufs[kg.THICKNESS]]
    for _ in range(2):  # warm-up of the copy path
        kg.check(L.kamino_step_host(h, DT, *io, *io, pitch))
    barrier(dist)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        # upload, step and download in one C-ABI call (the same bits as
        # kamino_set_state x3, kamino_step, kamino_get_state x3)
        kg.check(L.kamino_step_host(h, DT, *io, *io, pitch))
    e2e_s = time.perf_counter() - t0
    barrier(dist)
    e2e_max = max_over_ranks(dist, e2e_s)
    e2e_value = cells_total / e2e_max
    for p in bufs.values():
        L.kamino_host_free(p)
    launches = s.launches_per_step()
    s.close()

    if rank != 0:
        return None
    hbm, src_peak = peaks()
    adv_ms = kms.get("k_advect")
    dom = max(kms, key=kms.get)
    # u_phi, u_theta, thickness read once and written once (8 bytes per point)
    adv_bytes = 8 * (NT * 2 * NT + (NT - 1) * 2 * NT + NT * 2 * NT)
    achieved = adv_bytes / (adv_ms / 1e3) / 1e9
    traffic = committed_traffic()
    step_ms = ms / args.steps
    out = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 (FP64 for Fourier modes |m|<=4)",
        "data": DATA,
        "config": workload_config(ws),
        "implementation": {"sampler": "cell-exact", "wall_s_timed_region": wall},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": sum(nbytes.values()),
                "d2h_bytes_per_step": sum(nbytes.values())},
        "gpu_launches": launches * args.steps,
        "roofline": {"bound": "hbm", "kernel": "k_advect", "achieved": achieved, "peak": hbm,
                     "peak_source": src_peak, "unit": "GB/s", "frac": achieved / hbm, "traffic": traffic,
                     "algorithmic_bytes_per_launch": adv_bytes, "avg_launch_ms": adv_ms},
        "step_roofline": {"bytes_per_cell_step": STEP_BYTES_PER_CELL,
                          "achieved": STEP_BYTES_PER_CELL * C / (step_ms / 1e3) / 1e9, "peak": hbm,
                          "frac": STEP_BYTES_PER_CELL * C / (step_ms / 1e3) / 1e9 / hbm, "unit": "GB/s"},
        "kernel_ms": kms,
        "dominant_kernel": dom,
        "clocks": ck.summary(),
    }
    out["fp64_modes_0"] = bench_fp64_modes_0(kg, local, st, steps=min(args.steps, 500))
    out["reference_rounding"] = bench_reference_rounding(kg, local, st, steps=min(args.steps, 500))
    if not args.no_config2:
        out["config2"] = bench_particles(kg, local, hbm)
    if not args.no_batched:
        out["batched"] = bench_batched(kg, local)
    if not args.no_served:
        out["served"] = bench_served(kg, local, args.served_seconds)
    if not args.no_frames:
        out["frame_output"] = bench_frames(kg, local, st, hbm)
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(st, seconds=10.0)
    return out


def bench_fp64_modes_0(kg, local, st, steps):
    """The same sphere with every Fourier mode solved in FP32 (the dominance
    form), beside the precision form's FP64 for |m| <= 4."""
    cfg = kg.default_config(n_theta=NT, radius=1.0, dt=DT, fp64_modes=0, device=local)
    with kg.KaminoSolver(config=cfg) as s:
        s.load(st)
        s.step_n(5)
        s.synchronize()
        kms = s.time_kernels(reps=10, flush_l2=True)
        s.load(st)
        s.step_n(3)
        s.synchronize()
        ms = s.time_steps(steps, flush_l2=True) / steps
    return {"ms_per_step": ms, "cell_steps_per_s": NT * 2 * NT / (ms / 1e3), "k_solve_ms": kms["k_solve"],
            "what": "fp64_modes=0: every mode solved in FP32, %d timed steps" % steps}


def bench_reference_rounding(kg, local, st, steps):
    """The same sphere with KAMINO_F_REFERENCE_ROUNDING: the samplers in
    radians with the reference's own rounding, whose pole-wrap index map is
    bit-exact with the reference's validateCoord (the drop-in's exact mode)."""
    cfg = kg.default_config(n_theta=NT, radius=1.0, dt=DT, fp64_modes=4, flags=kg.F_REFERENCE_ROUNDING, device=local)
    with kg.KaminoSolver(config=cfg) as s:
        s.load(st)
        s.step_n(5)
        s.synchronize()
        kms = s.time_kernels(reps=10, flush_l2=True)
        s.load(st)
        s.step_n(3)
        s.synchronize()
        ms = s.time_steps(steps, flush_l2=True) / steps
    return {"ms_per_step": ms, "cell_steps_per_s": NT * 2 * NT / (ms / 1e3), "k_advect_ms": kms["k_advect"],
            "kernel_ms": kms,
            "what": "KAMINO_F_REFERENCE_ROUNDING (radian samplers, the reference's index arithmetic bit for bit), "
                    "%d timed steps" % steps}


def bench_particles(kg, local, hbm, npart=1 << 20, steps=200):
    """The mid-size configuration with particles: nTheta=512, nPhi=1024,
    radius 1, dt=0.002, l<=16, 2^20 particles uniform on the sphere advected
    with RK2 every step.  Device time per step, and the particles' share of
    the advection launch (k_advect with and without the particle tiles) with
    its roofline at 16 B per particle-step."""
    nt = 512
    st = kg.make_initial_state(nt, lmax=16, seed=SEED, n_particles=npart)
    res = {}
    for n in (npart, 0):
        cfg = kg.default_config(n_theta=nt, radius=1.0, dt=0.002, n_particles=n, flags=kg.F_PARTICLE_RK2,
                                fp64_modes=4, device=local)
        with kg.KaminoSolver(config=cfg) as s:
            s.load(st)
            s.step_n(5)
            s.synchronize()
            if n:
                profiler_range(True)  # three untimed steps with particles: the ncu launch list
                s.step_n(3)
                s.synchronize()
                profiler_range(False)
            kms = s.time_kernels(reps=10, flush_l2=True)
            s.load(st)
            s.step_n(3)
            s.synchronize()
            ms = s.time_steps(steps, flush_l2=True)
        res[n] = (ms / steps, kms)
    step_ms, kms = res[npart]
    adv_p, adv_0 = kms["k_advect"], res[0][1]["k_advect"]
    part_ms = max(adv_p - adv_0, 1e-9)
    achieved = PARTICLE_BYTES * npart / (part_ms / 1e3) / 1e9
    C = nt * 2 * nt
    return {"workload": "nTheta=512 nPhi=1024, radius 1, dt=0.002, l<=16, 2^20 particles uniform on the sphere, "
                        "RK2 particle advection, fp64_modes=4, %d timed steps (cold L2 each)" % steps,
            "ms_per_step": step_ms, "cell_steps_per_s": C / (step_ms / 1e3),
            "ms_per_step_without_particles": res[0][0],
            "k_advect_ms": adv_p, "k_advect_ms_without_particles": adv_0,
            "particle_share_of_k_advect": part_ms / adv_p,
            "particle_roofline": {"bytes_per_particle_step": PARTICLE_BYTES, "achieved": achieved, "peak": hbm,
                                  "frac": achieved / hbm, "unit": "GB/s",
                                  "what": "16 B x 2^20 over the particle tiles' share of the k_advect launch"},
            "kernel_ms": kms}


def bench_frames(kg, local, st, hbm, frames=5, steps_per_frame=10):
    """.bgeo frame output of the nTheta=1024 sphere (write_data_bgeo,
    KaminoSolver.cu:284-357): the device pack kernel against the HBM roofline
    (12 B read + 32 B written per cell), and the frame loop with output
    (kamino_run_frames_bgeo: pack, copy and file write overlapping the next
    frame's steps) against the same frames with no output and against the
    reference's order (wait, copy the fields back, pack on the host with one
    thread, write; the oracle's restatement does the packing)."""
    import shutil
    import tempfile

    from oracle import oracle as orc
    dt_frame = DT * steps_per_frame  # the frame loop takes about steps_per_frame + 1 steps a frame
    cfg = kg.default_config(n_theta=NT, radius=1.0, dt=DT, fp64_modes=4, device=local)
    cfg.frame_dt = dt_frame
    s = kg.KaminoSolver(config=cfg)
    s.load(st)
    C = NT * 2 * NT
    pack_ms = s.time_frame_pack(kg.FRAME_GRID, reps=20, flush_l2=True)
    pack_bytes = 44 * C
    tmp = tempfile.mkdtemp(prefix="kamino_frames_")
    try:
        s.run_frames_bgeo(1, os.path.join(tmp, "warm_"))  # first-use buffers
        s.load(st)
        s.synchronize()
        t0 = time.perf_counter()
        steps = s.run_frames_bgeo(frames, os.path.join(tmp, "grid_"))
        wall_out = time.perf_counter() - t0
        s.load(st)
        s.synchronize()
        t0 = time.perf_counter()
        s.run_frames(frames)
        s.synchronize()
        wall_none = time.perf_counter() - t0
        s.load(st)
        threads = orc.set_threads(1)
        per_frame = [kg.frame_steps(DT, dt_frame, i) - kg.frame_steps(DT, dt_frame, i - 1)
                     for i in range(1, frames + 1)]
        t0 = time.perf_counter()
        for i in range(frames + 1):
            if i:
                s.step_n(per_frame[i - 1])
            f = s.fields()
            img = orc.bgeo_image(orc.frame_grid_records(f["u_phi"], f["u_theta"], f["thickness"], NT, 1.0),
                                 orc.GRID_ATTRS)
            with open(os.path.join(tmp, "host_%d.bgeo" % i), "wb") as fp:
                fp.write(img)
        wall_host = time.perf_counter() - t0
        orc.set_threads(os.cpu_count() or 1)
        same = open(os.path.join(tmp, "grid_%d.bgeo" % frames), "rb").read(41) == img[:41]
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    nbytes = s.frame_bytes(kg.FRAME_GRID)
    s.close()
    achieved = pack_bytes / (pack_ms / 1e3) / 1e9
    return {"workload": "nTheta=1024 sphere, %d frames of frame_dt = %d dt (%d steps in all), grid .bgeo per "
                        "frame (%.1f MB)" % (frames, steps_per_frame, steps, nbytes / 1e6),
            "steps": steps, "pack_kernel": {"avg_launch_ms": pack_ms, "algorithmic_bytes_per_launch": pack_bytes,
                                            "achieved": achieved, "peak": hbm, "frac": achieved / hbm,
                                            "unit": "GB/s"},
            "frames_with_output_s_per_frame": wall_out / frames,
            "frames_without_output_s_per_frame": wall_none / frames,
            "host_packing_order_s_per_frame": wall_host / frames, "host_packing_threads": threads,
            "headers_equal": same}


def _same(a, b):
    import numpy as np
    return all(np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)) for k in ("u_phi", "u_theta", "thickness"))


def bench_batched(kg, local, n_spheres=256, steps=500):
    """256 independent spheres, nTheta ~ U{32,64,128,256}, radius ~ U(0.5, 2),
    dt 0.005, own l<=8 stream function each, FP64 modes |m|<=4: the batched
    step (one persistent kernel per stage, one graph per step, autotuned)
    against looping the plain solver over the same spheres."""
    import numpy as np
    from kaminogpu_gb300.batch import Batch
    rng = np.random.default_rng(4)
    nts = rng.choice([32, 64, 128, 256], n_spheres)
    rads = rng.uniform(0.5, 2.0, n_spheres)
    cfgs = [kg.default_config(n_theta=int(n), radius=float(r), dt=0.005, fp64_modes=4, device=local)
            for n, r in zip(nts, rads)]
    states = [kg.make_initial_state(int(n), lmax=8, seed=1000 + i, radius=float(r))
              for i, (n, r) in enumerate(zip(nts, rads))]
    cells = int(sum(int(n) * 2 * int(n) for n in nts))
    b = Batch(cfgs)
    for i, st in enumerate(states):
        b.load(i, st)
    tuned = b.autotune(reps=3)
    for i, st in enumerate(states):
        b.load(i, st)
    profiler_range(True)  # three untimed steps of the tuned batch: the ncu launch list
    b.step_n(3)
    b.synchronize()
    profiler_range(False)
    for i, st in enumerate(states):
        b.load(i, st)
    b.synchronize()
    with Clocks(local) as ck:
        t0 = time.perf_counter()
        b.step_n(steps)
        b.synchronize()
        wall_batched = time.perf_counter() - t0
    batched_out = [{"u_phi": None} for _ in states]
    check_idx = list(range(0, n_spheres, 17))
    for i in check_idx:
        batched_out[i] = {"u_phi": b.get_state(i, kg.U_PHI), "u_theta": b.get_state(i, kg.U_THETA),
                          "thickness": b.get_state(i, kg.THICKNESS)}
    ms_dev = b.time_steps(20, flush_l2=False)
    b.close()

    solvers = [kg.KaminoSolver(config=c) for c in cfgs]
    for s, st in zip(solvers, states):
        s.load(st)
        s.step_n(3)
    for s in solvers:
        s.synchronize()
    # plain, as one simulation is run: step a sphere, wait, next sphere
    for s, st in zip(solvers, states):
        s.load(st)
    t0 = time.perf_counter()
    for s in solvers:
        s.step_n(steps)
        s.synchronize()
    wall_sync = time.perf_counter() - t0
    bitwise = all(_same(batched_out[i], solvers[i].fields()) for i in check_idx)
    # plain, every sphere's stream queued before one wait at the end
    for s, st in zip(solvers, states):
        s.load(st)
    for s in solvers:
        s.synchronize()
    t0 = time.perf_counter()
    for s in solvers:
        s.step_n(steps)
    for s in solvers:
        s.synchronize()
    wall_async = time.perf_counter() - t0
    for s in solvers:
        s.close()
    v_b = cells * steps / wall_batched
    v_s = cells * steps / wall_sync
    v_a = cells * steps / wall_async
    return {"workload": "%d spheres, nTheta~U{32,64,128,256}, radius~U(0.5,2), dt=0.005, l<=8, fp64_modes=4, "
                        "%d steps" % (n_spheres, steps),
            "cells_per_step": cells, "value": v_b, "unit": UNIT, "wall_s": wall_batched,
            "device_ms_per_step": ms_dev / 20, "autotuned": tuned,
            "plain_loop_sync": {"value": v_s, "wall_s": wall_sync},
            "plain_loop_async": {"value": v_a, "wall_s": wall_async},
            "speedup_vs_plain": v_b / max(v_s, v_a),
            "bitwise_equal_to_plain": bitwise, "spheres_compared": len(check_idx),
            "clocks": ck.summary()}


def served_requests(n, seed=5):
    import numpy as np
    rng = np.random.default_rng(seed)
    nts = 2 ** rng.integers(6, 11, n)  # log-uniform over {64, ..., 1024}
    steps = rng.integers(10, 501, n)
    return [(int(a), int(b)) for a, b in zip(nts, steps)]


def bench_served(kg, local, seconds, rate=200.0, budget=120 << 30):
    """Requests of one sphere each: nTheta log-uniform over {64..1024},
    steps ~ U[10, 500], dt 0.002, l<=16, FP64 modes |m|<=4, 120 GB budget.
    closed loop: a fixed request set drained as fast as possible, against the
    plain solver run per request (one cached handle per nTheta).  open loop:
    Poisson arrivals at 200/s for `seconds`, p50/p99 latency."""
    import numpy as np
    from kaminogpu_gb300.batch import Server
    init = {}

    def state(nt, seed):
        k = (nt, seed % 8)
        if k not in init:
            init[k] = kg.make_initial_state(nt, lmax=16, seed=2000 + seed % 8)
        return init[k]

    def cfg(nt):
        return kg.default_config(n_theta=nt, radius=1.0, dt=0.002, fp64_modes=4, device=local)

    out = {"workload": "requests: nTheta log-uniform {64..1024}, steps~U[10,500], dt=0.002, l<=16, fp64_modes=4, "
                       "120 GB admission budget"}
    # closed loop
    reqs = served_requests(120)
    cs_total = sum(nt * 2 * nt * st for nt, st in reqs)
    for i, (nt, _) in enumerate(reqs):  # initial states are inputs: made before any timing
        state(nt, i)
    srv = Server(budget_bytes=budget, steps_per_round=16, device=local)
    for i, (nt, st) in enumerate(reqs[:5]):  # warm the handle pool
        srv.submit(cfg(nt), state(nt, i), 3)
    while srv.stats()["completed"] < 5:
        srv.poll()
    srv.close()
    srv = Server(budget_bytes=budget, steps_per_round=16, device=local)
    with Clocks(local) as ck:
        t0 = time.perf_counter()
        rids = [srv.submit(cfg(nt), state(nt, i), st) for i, (nt, st) in enumerate(reqs)]
        t_submit = time.perf_counter() - t0
        done = 0
        while done < len(reqs):
            done += srv.poll()
        wall_srv = time.perf_counter() - t0
    stats = srv.stats()
    t0 = time.perf_counter()
    served_res = {i: srv.fetch(rids[i]) for i in range(0, len(reqs), 13)}
    t_fetch = (time.perf_counter() - t0) / max(1, len(served_res))
    srv.close()
    handles = {}
    for nt in sorted({nt for nt, _ in reqs}):
        handles[nt] = kg.KaminoSolver(config=cfg(nt))
        handles[nt].load(state(nt, 0))
        handles[nt].step_n(3)
        handles[nt].synchronize()
    t0 = time.perf_counter()
    bitwise = True
    for i, (nt, st) in enumerate(reqs):
        s = handles[nt]
        s.load(state(nt, i))
        s.step_n(st)
        f = s.fields()
        if i in served_res:
            bitwise = bitwise and _same(served_res[i], f)
    wall_plain = time.perf_counter() - t0
    for s in handles.values():
        s.close()
    out["closed_loop"] = {"requests": len(reqs), "cell_steps": cs_total, "value": cs_total / wall_srv,
                          "unit": UNIT, "wall_s": wall_srv, "p50_latency_s": stats["p50_latency_s"],
                          "p99_latency_s": stats["p99_latency_s"],
                          "plain_per_request": {"value": cs_total / wall_plain, "wall_s": wall_plain},
                          "speedup_vs_plain": wall_plain / wall_srv, "bitwise_equal_to_plain": bitwise,
                          "requests_compared": len(served_res), "clocks": ck.summary(),
                          "breakdown": {
                              "wall_s": wall_srv,
                              "host_submit_s": t_submit,
                              "host_poll_s": stats["poll_seconds"],
                              "host_fetch_s_per_request": t_fetch,
                              "batched_rounds": stats["batched_rounds"],
                              "batched_round_device_s": stats["batched_round_seconds"],
                              "solo_device_s_summed": stats["solo_seconds"],
                              "solo_cell_steps": stats["solo_cell_steps"],
                              "batched_cell_steps": stats["batched_cell_steps"],
                              "what": "batched rounds run one at a time on the engine's stream; one-sphere "
                                      "runs (nTheta >= 512) on their own streams, up to 3 at once, so their "
                                      "device times overlap each other and the rounds"}}
    # open loop: Poisson arrivals
    rng = np.random.default_rng(6)
    n_open = int(rate * seconds)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n_open))
    oreqs = served_requests(n_open, seed=7)
    for i, (nt, _) in enumerate(oreqs):
        state(nt, i)
    srv = Server(budget_bytes=budget, steps_per_round=16, device=local)
    t_start = srv.now()
    submitted = 0
    done = 0
    while done < n_open:
        now = srv.now() - t_start
        while submitted < n_open and arrivals[submitted] <= now:
            nt, st = oreqs[submitted]
            srv.submit(cfg(nt), state(nt, submitted), st, arrival=t_start + arrivals[submitted])
            submitted += 1
        done += srv.poll()
        if submitted < n_open and srv.stats()["resident"] == 0:
            time.sleep(max(0.0, min(0.001, arrivals[submitted] - (srv.now() - t_start))))
    wall = srv.now() - t_start
    s = srv.stats()
    srv.close()
    cs = sum(nt * 2 * nt * st for nt, st in oreqs)
    out["open_loop"] = {"rate_per_s": rate, "arrival_window_s": float(arrivals[-1]), "requests": n_open,
                        "cell_steps": cs, "value": cs / wall, "unit": UNIT, "wall_s": wall,
                        "offered_cell_steps_per_s": cs / float(arrivals[-1]),
                        "p50_latency_s": s["p50_latency_s"], "p99_latency_s": s["p99_latency_s"],
                        "mean_latency_s": s["mean_latency_s"], "peak_resident_bytes": s["peak_resident_bytes"]}
    return out


def cpu_baseline(st, seconds=10.0):
    """The oracle's FP64 CPU step on a bounded sample: as many steps of the
    same sphere as fit in about `seconds`, all host threads."""
    from oracle import oracle as orc
    cores = orc.set_threads(os.cpu_count() or 1)
    o = orc.Oracle(NT, 1.0, DT)
    o.load(st)
    t0 = time.perf_counter()
    o.step(1)
    t1 = time.perf_counter() - t0
    samples = int(max(1, min(500, seconds / max(t1, 1e-3))))
    t0 = time.perf_counter()
    o.step(samples)
    dt = time.perf_counter() - t0
    o.close()
    return {"value": NT * 2 * NT * samples / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "%d FP64 steps of the nTheta=1024 sphere after 1 untimed (%.1f s)" % (samples, dt)}


def run_reference(args, ws, rank):
    """The reference arm: the CPU port of the reference step (oracle/, FP64,
    all host threads) on the same workload, built from the same seeded state
    by the oracle's own generator -- nothing of the product library is
    loaded.  Same warm-up count as the GPU arm; the timed steps are a bounded
    sample (about 30 s of CPU work at most)."""
    if rank != 0:
        return None
    from oracle import oracle as orc
    st = orc.make_initial_state(NT, lmax=LMAX, seed=SEED, vortex=True)
    cores = orc.set_threads(os.cpu_count() or 1)
    o = orc.Oracle(NT, 1.0, DT)
    o.load(st)
    t0 = time.perf_counter()
    o.step(args.warmup)
    t1 = (time.perf_counter() - t0) / args.warmup
    n = int(max(1, min(args.steps, 30.0 / max(t1, 1e-3))))
    t0 = time.perf_counter()
    o.step(n)
    dt = time.perf_counter() - t0
    o.close()
    value = NT * 2 * NT * n / dt
    out = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": ws,
        "steps": n,
        "warmup": args.warmup,
        "ms_per_step": dt / n * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": DATA,
        "config": workload_config(ws),
        "implementation": {"what": "CPU port of the reference step (oracle/kamino_oracle.c), FP64, OpenMP",
                           "steps_requested": args.steps},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "%d FP64 steps of the nTheta=1024 sphere after %d untimed (%.1f s)"
                                   % (n, args.warmup, dt)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if orc.have_reference_gpu():
        try:
            r = orc.RefGPU(NT, 1.0, DT)
            r.load(st)
            r.step(2)
            ms, stages = r.time_steps(max(args.steps, 5))
            n = max(args.steps, 5)
            out["reference_gpu_kernels"] = {
                "value": NT * 2 * NT * n / (ms / 1e3), "unit": UNIT, "ms_per_step": ms / n,
                "stage_ms": {"advection": stages[0] / n, "geometric": stages[1] / n, "projection": stages[2] / n},
                "what": "the reference's own CUDA kernels (compiled from its sources for sm_103a) with cuFFT, "
                        "in stepForward order on this GPU"}
            r.close()
        except Exception as e:  # the CPU arm stands on its own
            out["reference_gpu_kernels"] = {"unavailable": str(e)}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-served", action="store_true")
    ap.add_argument("--no-frames", action="store_true")
    ap.add_argument("--no-config2", action="store_true")
    ap.add_argument("--served-seconds", type=float, default=60.0)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    ws, rank, local = dist_env()
    dist = init_dist(ws)
    if args.impl == "reference":
        out = run_reference(args, ws, rank)
    else:
        out = run_ours(args, ws, rank, local, dist)
    if out is not None and rank == 0:
        print(json.dumps(out), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
