"""Batched spheres and the continuous-batching server (ctypes over the C ABI)."""
import ctypes

import numpy as np

from ._lib import (PARTICLES, THICKNESS, U_PHI, U_THETA, KaminoConfig, KaminoServerConfig, KaminoServerStats,
                   check, lib)


class Batch:
    """Many independent spheres of uneven nTheta advanced by shared launches
    (kamino_batch_*).  cfgs: list of KaminoConfig."""

    def __init__(self, cfgs):
        arr = (KaminoConfig * len(cfgs))(*cfgs)
        h = ctypes.c_void_p()
        check(lib.kamino_batch_create(arr, len(cfgs), ctypes.byref(h)))
        self._h = h
        self.cfgs = list(cfgs)

    def close(self):
        if getattr(self, "_h", None):
            lib.kamino_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _shape(self, i, field):
        nt = self.cfgs[i].n_theta
        if field == PARTICLES:
            return (int(lib.kamino_particle_count(ctypes.byref(self.cfgs[i]))), 2)
        return (nt - 1 if field == U_THETA else nt, 2 * nt)

    def set_state(self, i, field, arr):
        a = np.ascontiguousarray(arr, np.float32)
        check(lib.kamino_batch_set_state(self._h, i, field, a.ctypes.data, 0))

    def get_state(self, i, field):
        out = np.empty(self._shape(i, field), np.float32)
        if out.size:
            check(lib.kamino_batch_get_state(self._h, i, field, out.ctypes.data, 0))
        return out

    def load(self, i, st):
        self.set_state(i, U_PHI, st["u_phi"])
        self.set_state(i, U_THETA, st["u_theta"])
        self.set_state(i, THICKNESS, st["thickness"])
        if self._shape(i, PARTICLES)[0]:
            self.set_state(i, PARTICLES, st["particles"])

    def step_n(self, n):
        check(lib.kamino_batch_step_n(self._h, n))

    def synchronize(self):
        check(lib.kamino_batch_synchronize(self._h))

    def time_steps(self, n, flush_l2=True):
        ms = ctypes.c_double()
        check(lib.kamino_batch_time_steps(self._h, n, int(flush_l2), ctypes.byref(ms)))
        return ms.value

    def autotune(self, reps=3):
        out = (ctypes.c_int * 4)()
        check(lib.kamino_batch_autotune(self._h, reps, out, 4))
        return dict(zip(("adv_cta_per_sm", "fft_cta_per_sm", "solve_cta_per_sm", "adv_tiles_per_item"), out))

    def cells(self):
        return int(lib.kamino_batch_cells(self._h))


class Server:
    """Continuous batching of simulate requests under an HBM budget."""

    def __init__(self, budget_bytes, max_resident=0, steps_per_round=10, device=0, solo_n_theta=0, solo_slots=0):
        """solo_n_theta: requests with n_theta >= this run as one-sphere graphs
        on their own streams (0: the library default, 512); solo_slots: how
        many of those run at once (0: the default, 3)."""
        c = KaminoServerConfig()
        c.budget_bytes, c.max_resident, c.steps_per_round, c.device = budget_bytes, max_resident, steps_per_round, device
        c.solo_n_theta, c.solo_slots = solo_n_theta, solo_slots
        h = ctypes.c_void_p()
        check(lib.kamino_server_create(ctypes.byref(c), ctypes.byref(h)))
        self._h = h
        self.shapes = {}

    def close(self):
        if getattr(self, "_h", None):
            lib.kamino_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def now(self):
        return lib.kamino_server_now(self._h)

    def submit(self, cfg, st, steps, arrival=-1.0):
        rid = ctypes.c_int64()
        u = np.ascontiguousarray(st["u_phi"], np.float32)
        v = np.ascontiguousarray(st["u_theta"], np.float32)
        r = np.ascontiguousarray(st["thickness"], np.float32)
        check(lib.kamino_server_submit(self._h, ctypes.byref(cfg), u.ctypes.data, v.ctypes.data, r.ctypes.data,
                                       steps, arrival, ctypes.byref(rid)))
        self.shapes[rid.value] = cfg.n_theta
        return rid.value

    def poll(self):
        n = ctypes.c_int()
        check(lib.kamino_server_poll(self._h, ctypes.byref(n)))
        return n.value

    def fetch(self, rid):
        nt = self.shapes[rid]
        out = {}
        for name, field, rows in (("u_phi", U_PHI, nt), ("u_theta", U_THETA, nt - 1), ("thickness", THICKNESS, nt)):
            a = np.empty((rows, 2 * nt), np.float32)
            rc = lib.kamino_server_fetch(self._h, rid, field, a.ctypes.data)
            if rc == 7:
                return None
            check(rc)
            out[name] = a
        return out

    def stats(self):
        s = KaminoServerStats()
        check(lib.kamino_server_get_stats(self._h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in KaminoServerStats._fields_}
