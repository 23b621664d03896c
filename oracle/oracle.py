"""TEST INFRASTRUCTURE: Python bindings of the oracle and the reference harness.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
legs use this module, as the checker.  It wraps
  _build/libkamino_oracle.so  the C restatement of the reference step
                              (kamino_oracle.c: FP64 step + reference-
                              arithmetic index map)
  _build/libkref.so           the reference's own kernels (cubins in _ref/)
                              run in stepForward order with cuFFT
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libkamino_oracle.so")
KREF_SO = os.path.join(HERE, "_build", "libkref.so")
REF_CUBINS = os.path.join(HERE, "_ref")

U_PHI, U_THETA, THICKNESS, PRESSURE, PARTICLES = range(5)
FL_PARTICLE_RK2, FL_POLE_SIGN_FLIP = 1, 2

_P, _I, _I64, _D, _F = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double, ctypes.c_float
_olib = None
_klib = None


def _oracle_lib():
    global _olib
    if _olib is None:
        if not os.path.exists(ORACLE_SO):
            import importlib.util
            spec = importlib.util.spec_from_file_location("oracle_build", os.path.join(HERE, "build.py"))
            mod = importlib.util.module_from_spec(spec)
            spec.loader.exec_module(mod)
            mod.build_oracle()
        L = ctypes.CDLL(ORACLE_SO)
        L.oracle_create.restype = _P
        L.oracle_create.argtypes = [_I, _D, _D, ctypes.c_uint, _I64]
        L.oracle_create_h.restype = _P
        L.oracle_create_h.argtypes = [_I, _D, _D, ctypes.c_uint, _I64, _D]
        L.oracle_destroy.argtypes = [_P]
        for f in ("oracle_advection", "oracle_geometric", "oracle_projection"):
            getattr(L, f).argtypes = [_P]
        L.oracle_step.argtypes = [_P, _I]
        L.oracle_set_state.argtypes = [_P, _I, _P]
        L.oracle_set_state_f64.argtypes = [_P, _I, _P]
        L.oracle_get_state.argtypes = [_P, _I, _P]
        L.oracle_divergence.argtypes = [_P, _P, _P, _P]
        L.oracle_set_threads.argtypes = [_I]
        L.oracle_set_threads.restype = _I
        L.oracle_ref_index.argtypes = [_I, _P, _P, _I64, _F, _I, _P, _P]
        L.oracle_ref_wrap.argtypes = [_P, _P, _I64, _F, _P]
        L.oracle_ref_init_fbm.argtypes = [_I, _F, _F, _P, _P]
        _olib = L
    return _olib


def set_threads(n):
    return _oracle_lib().oracle_set_threads(n)


def grid_h(nt):
    """gridLenGlobal = (float)(M_PI / nTheta), KaminoCore.cu:849."""
    return np.float32(np.pi / nt)


class Oracle:
    """FP64 restatement of the reference step on one sphere."""

    def __init__(self, nt, radius=1.0, dt=0.005, flags=0, n_particles=0, h=0.0):
        self.L = _oracle_lib()
        self.nt, self.np_ = nt, 2 * nt
        self.n_particles = n_particles
        self.o = self.L.oracle_create_h(nt, radius, dt, flags, n_particles, float(h))
        if not self.o:
            raise ValueError("oracle_create(nt=%d) failed" % nt)

    def close(self):
        if self.o:
            self.L.oracle_destroy(self.o)
            self.o = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _shape(self, field):
        if field == PARTICLES:
            return (self.n_particles, 2)
        return (self.nt - 1 if field == U_THETA else self.nt, self.np_)

    def set_state(self, field, arr):
        a = np.asarray(arr)
        if a.dtype == np.float64:
            a = np.ascontiguousarray(a)
            self.L.oracle_set_state_f64(self.o, field, a.ctypes.data)
        else:
            a = np.ascontiguousarray(a, np.float32)
            self.L.oracle_set_state(self.o, field, a.ctypes.data)

    def get_state(self, field):
        out = np.empty(self._shape(field), np.float64)
        if out.size:
            self.L.oracle_get_state(self.o, field, out.ctypes.data)
        return out

    def load(self, state):
        self.set_state(U_PHI, state["u_phi"])
        self.set_state(U_THETA, state["u_theta"])
        if "thickness" in state:
            self.set_state(THICKNESS, state["thickness"])
        if self.n_particles and "particles" in state:
            self.set_state(PARTICLES, state["particles"])

    def fields(self):
        out = {"u_phi": self.get_state(U_PHI), "u_theta": self.get_state(U_THETA),
               "thickness": self.get_state(THICKNESS), "pressure": self.get_state(PRESSURE)}
        if self.n_particles:
            out["particles"] = self.get_state(PARTICLES)
        return out

    def advection(self):
        self.L.oracle_advection(self.o)

    def geometric(self):
        self.L.oracle_geometric(self.o)

    def projection(self):
        self.L.oracle_projection(self.o)

    def step(self, n=1):
        self.L.oracle_step(self.o, n)

    def divergence(self, u=None, v=None):
        """The reference's discrete divergence (fillDivergenceKernel) in FP64."""
        out = np.zeros((self.nt + 2, self.np_), np.float64)
        if u is None:
            self.L.oracle_divergence(self.o, None, None, out.ctypes.data)
        else:
            u = np.ascontiguousarray(u, np.float32)
            v = np.ascontiguousarray(v, np.float32)
            self.L.oracle_divergence(self.o, u.ctypes.data, v.ctypes.data, out.ctypes.data)
        return out[: self.nt]


def ref_index(kind, phi, theta, nt):
    """Index stage of the reference samplers in the reference's arithmetic."""
    L = _oracle_lib()
    phi = np.ascontiguousarray(phi, np.float32)
    theta = np.ascontiguousarray(theta, np.float32)
    n = phi.size
    out = np.empty((n, 4), np.int32)
    alpha = np.empty((n, 2), np.float32)
    L.oracle_ref_index(kind, phi.ctypes.data, theta.ctypes.data, n, grid_h(nt), nt, out.ctypes.data,
                       alpha.ctypes.data)
    return out, alpha


def ref_init_fbm(nt, radius=1.0):
    """u_phi, u_theta of KaminoSolver::initialize_velocity in the
    reference's arithmetic (KaminoInitializer.cu:3-134)."""
    L = _oracle_lib()
    u = np.empty((nt, 2 * nt), np.float32)
    v = np.empty((nt - 1, 2 * nt), np.float32)
    L.oracle_ref_init_fbm(nt, radius, grid_h(nt), u.ctypes.data, v.ctypes.data)
    return u, v


def ref_wrap(phi, theta, nt):
    """validateCoord + particle cell index in the reference's arithmetic."""
    L = _oracle_lib()
    phi = np.array(phi, np.float32)
    theta = np.array(theta, np.float32)
    cells = np.empty((phi.size, 2), np.int32)
    L.oracle_ref_wrap(phi.ctypes.data, theta.ctypes.data, phi.size, grid_h(nt), cells.ctypes.data)
    return phi, theta, cells


# ------------------------------------------------------------ reference GPU
def _kref_lib():
    global _klib
    if _klib is None:
        if not os.path.exists(KREF_SO):
            raise FileNotFoundError("reference harness not built: %s" % KREF_SO)
        L = ctypes.CDLL(KREF_SO)
        L.kref_create.argtypes = [ctypes.c_char_p, _I, _F, _F, ctypes.c_longlong, ctypes.POINTER(_P)]
        L.kref_destroy.argtypes = [_P]
        L.kref_set_state.argtypes = [_P, _I, _P]
        L.kref_get_state.argtypes = [_P, _I, _P]
        for f in ("kref_advection", "kref_geometric", "kref_projection", "kref_synchronize"):
            getattr(L, f).argtypes = [_P]
        L.kref_step.argtypes = [_P, _I]
        L.kref_time_steps.argtypes = [_P, _I, ctypes.POINTER(_D), ctypes.POINTER(_D)]
        L.kref_probe_index.argtypes = [_P, _I, _P, _P, ctypes.c_longlong, _P, _P]
        L.kref_probe_wrap.argtypes = [_P, _P, _P, ctypes.c_longlong, _P]
        L.kref_last_error.restype = ctypes.c_char_p
        _klib = L
    return _klib


def have_reference_gpu():
    return os.path.exists(KREF_SO) and all(
        os.path.exists(os.path.join(REF_CUBINS, n)) for n in ("ref_core.cubin", "ref_tdm.cubin", "ref_solver.cubin"))


class RefGPU:
    """The reference's own CUDA kernels, driven in stepForward order."""

    def __init__(self, nt, radius=1.0, dt=0.005, n_particles=0):
        self.L = _kref_lib()
        self.nt, self.np_ = nt, 2 * nt
        self.n_particles = n_particles
        h = _P()
        if self.L.kref_create(REF_CUBINS.encode(), nt, radius, dt, n_particles, ctypes.byref(h)):
            raise RuntimeError("kref_create: %s" % self.L.kref_last_error().decode())
        self.h = h

    def _chk(self, rc):
        if rc:
            raise RuntimeError(self.L.kref_last_error().decode())

    def close(self):
        if getattr(self, "h", None):
            self.L.kref_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _shape(self, field):
        if field == PARTICLES:
            return (self.n_particles, 2)
        return (self.nt - 1 if field == U_THETA else self.nt, self.np_)

    def set_state(self, field, arr):
        a = np.ascontiguousarray(arr, np.float32)
        self._chk(self.L.kref_set_state(self.h, field, a.ctypes.data))

    def get_state(self, field):
        out = np.empty(self._shape(field), np.float32)
        self._chk(self.L.kref_get_state(self.h, field, out.ctypes.data))
        return out

    def load(self, state):
        Oracle.load(self, state)

    def fields(self):
        return Oracle.fields(self)

    def advection(self):
        self._chk(self.L.kref_advection(self.h))

    def geometric(self):
        self._chk(self.L.kref_geometric(self.h))

    def projection(self):
        self._chk(self.L.kref_projection(self.h))

    def step(self, n=1):
        self._chk(self.L.kref_step(self.h, n))

    def time_steps(self, n):
        ms, st = _D(), (_D * 3)()
        self._chk(self.L.kref_time_steps(self.h, n, ctypes.byref(ms), st))
        return ms.value, list(st)

    def probe_index(self, kind, phi, theta):
        phi = np.ascontiguousarray(phi, np.float32)
        theta = np.ascontiguousarray(theta, np.float32)
        n = phi.size
        out = np.empty((n, 4), np.int32)
        alpha = np.empty((n, 2), np.float32)
        self._chk(self.L.kref_probe_index(self.h, kind, phi.ctypes.data, theta.ctypes.data, n, out.ctypes.data,
                                          alpha.ctypes.data))
        return out, alpha

    def probe_wrap(self, phi, theta):
        phi = np.array(phi, np.float32)
        theta = np.array(theta, np.float32)
        cells = np.empty((phi.size, 2), np.int32)
        self._chk(self.L.kref_probe_wrap(self.h, phi.ctypes.data, theta.ctypes.data, phi.size, cells.ctypes.data))
        return phi, theta, cells


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    d = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (d if d > 0 else 1.0))
