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
        L.oracle_frame_grid.argtypes = [_I, _F, _F, _P, _P, _P, _P]
        L.oracle_frame_particles.argtypes = [_F, _P, _I64, _P]
        L.oracle_ref_particles.argtypes = [_F, _I, ctypes.c_uint, _P]
        L.oracle_ref_particles.restype = _I64
        L.oracle_image_resample.argtypes = [_P, _I, _I, ctypes.c_size_t, _I, _I, _P]
        L.oracle_make_initial_state.argtypes = [_I, _I, ctypes.c_uint64, _D, _D, _I, _D, _D, _D, _I64,
                                                _P, _P, _P, _P, _P]
        L.oracle_make_initial_state.restype = _I
        _olib = L
    return _olib


def make_initial_state(nt, lmax=8, seed=1, radius=1.0, thickness_noise=0.05, vortex=False, vortex_sigma=0.1,
                       velocity_scale=1.0, n_particles=0):
    """The seeded synthetic state of kamino_make_initial_state, made on the
    CPU side (synth_state.c) without the product library; same dict."""
    u = np.empty((nt, 2 * nt), np.float32)
    v = np.empty((nt - 1, 2 * nt), np.float32)
    rho = np.empty((nt, 2 * nt), np.float32)
    part = np.empty((max(n_particles, 1), 2), np.float32)
    vo = np.zeros(3, np.float64)
    rc = _oracle_lib().oracle_make_initial_state(nt, lmax, seed, radius, thickness_noise, int(bool(vortex)),
                                                 vortex_sigma, 0.0, velocity_scale, n_particles, u.ctypes.data,
                                                 v.ctypes.data, rho.ctypes.data, part.ctypes.data, vo.ctypes.data)
    if rc:
        raise ValueError("oracle_make_initial_state(nt=%d, lmax=%d) failed" % (nt, lmax))
    return {"u_phi": u, "u_theta": v, "thickness": rho, "particles": part[:n_particles], "vortex": tuple(vo)}


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


# ------------------------------------------------------------ frame output
# Partio's uncompressed BGEO layout (Houdini classic geometry), restated from
# the format: big-endian int32 magic "Bgeo", char 'V', int32 version 5, eight
# int32 counts (points, prims, point groups, prim groups, point attributes,
# vertex attributes, prim attributes, detail attributes), one definition per
# point attribute other than position (uint16 name length, name, uint16
# size, int32 type: 0 float, 5 vector, size int32 defaults 0), the points
# (x, y, z, w = 1, attribute values) and the trailer bytes 00 ff.  Partio
# itself is not in the reference tree (only its headers); the layout is
# anchored on the attribute lists of KaminoSolver.cu:290-293, 365-368.
GRID_ATTRS = (("v", 3, 5), ("density", 1, 0))
PARTICLE_ATTRS = (("v", 3, 5), ("color", 3, 5))


def frame_grid_records(u, v, rho, nt, radius):
    """write_data_bgeo's point records (KaminoSolver.cu:284-357): float32
    [nt*np, 8] = x y z 1 vx vy vz density, rows j then columns i."""
    L = _oracle_lib()
    u = np.ascontiguousarray(u, np.float32)
    v = np.ascontiguousarray(v, np.float32)
    rho = np.ascontiguousarray(rho, np.float32)
    rec = np.empty((nt * 2 * nt, 8), np.float32)
    L.oracle_frame_grid(nt, float(np.float32(radius)), float(grid_h(nt)), u.ctypes.data, v.ctypes.data,
                        rho.ctypes.data, rec.ctypes.data)
    return rec


def frame_particle_records(part, radius):
    """write_particles_bgeo's point records (KaminoSolver.cu:359-396):
    float32 [n, 10] = x y z 1 0 0 0 and a zero colour."""
    L = _oracle_lib()
    part = np.ascontiguousarray(part, np.float32).reshape(-1, 2)
    rec = np.empty((part.shape[0], 10), np.float32)
    if part.shape[0]:
        L.oracle_frame_particles(float(np.float32(radius)), part.ctypes.data, part.shape[0], rec.ctypes.data)
    return rec


def ref_particles(particle_density, nt, seed=1):
    """KaminoParticles' jittered grid (KaminoParticles.cu:20-62) drawn with
    srand(seed) / rand(): float32 [n, 2] (phi, theta)."""
    L = _oracle_lib()
    # Kamino::run hands the density to KaminoParticles through a size_t
    # parameter (KaminoSolver.cu:278): the fraction is dropped
    d = np.float32(int(np.float32(particle_density)))
    lin = np.sqrt(d)
    n_theta = int(np.float32(lin * np.float32(nt)))
    out = np.empty((2 * n_theta * n_theta, 2), np.float32)
    n = L.oracle_ref_particles(float(d), nt, seed, out.ctypes.data)
    assert n == out.shape[0]
    return out


def image_resample(img, dw, dh):
    """The mirrored, resampled 8-bit image (oracle_image_resample): uint8
    [dh, dw, 3] from uint8 [h, w, 3] (B, G, R)."""
    L = _oracle_lib()
    img = np.ascontiguousarray(img, np.uint8)
    out = np.empty((dh, dw, 3), np.uint8)
    L.oracle_image_resample(img.ctypes.data, img.shape[1], img.shape[0], img.strides[0], dw, dh, out.ctypes.data)
    return out


def image_density(px):
    """initDensityfromPic's per-cell value (KaminoSolver.cu:265-273): each
    channel / 255.0 rounded to float, a float sum, / 3.0 rounded to float."""
    c = (px.astype(np.float64) / 255.0).astype(np.float32)
    s = (c[..., 0] + c[..., 1]) + c[..., 2]
    return (s.astype(np.float64) / 3.0).astype(np.float32)


def particle_colors(px, part, nt):
    """KaminoParticles' colours (KaminoParticles.cu:56-72): (G, R, B) / 255
    of the pixel of each particle's cell, float32 [n, 3]."""
    h = grid_h(nt)
    part = np.asarray(part, np.float32).reshape(-1, 2)
    x = np.clip(np.floor(part[:, 0] / h).astype(np.int64), 0, 2 * nt - 1)
    y = np.clip(np.floor(part[:, 1] / h).astype(np.int64), 0, nt - 1)
    p = px[y, x].astype(np.float64) / 255.0
    return np.stack([p[:, 1], p[:, 2], p[:, 0]], 1).astype(np.float32)


def written_colors(col):
    """The colour write_particles_bgeo writes for particle i: components
    3i+1, 3i+2, 3i+3 of the flat (G, R, B) array (KaminoSolver.cu:375-377);
    the last particle's third one lies past the array (0 here)."""
    flat = np.concatenate([np.asarray(col, np.float32).reshape(-1), np.zeros(1, np.float32)])
    n = len(col)
    return np.stack([flat[3 * np.arange(n) + k] for k in (1, 2, 3)], 1)


def bgeo_image(records, attrs):
    """The .bgeo file bytes for float32 point records [n, 4 + sum(sizes)]."""
    import struct
    records = np.ascontiguousarray(records, np.float32)
    out = [b"Bgeo", b"V", struct.pack(">i", 5),
           struct.pack(">8i", records.shape[0], 0, 0, 0, len(attrs), 0, 0, 0)]
    for name, size, typ in attrs:
        out += [struct.pack(">H", len(name)), name.encode(), struct.pack(">Hi", size, typ),
                struct.pack(">%di" % size, *([0] * size))]
    out += [records.astype(">f4").tobytes(), b"\x00\xff"]
    return b"".join(out)


def read_bgeo(data):
    """Parses a .bgeo image of the layout above: (attrs, records float32)."""
    import struct
    if data[:5] != b"BgeoV":
        raise ValueError("not a BGEO V file")
    (version,) = struct.unpack_from(">i", data, 5)
    counts = struct.unpack_from(">8i", data, 9)
    if version != 5 or any(counts[1:4]) or any(counts[5:]):
        raise ValueError("unexpected header %r %r" % (version, counts))
    off, attrs = 41, []
    for _ in range(counts[4]):
        (n,) = struct.unpack_from(">H", data, off)
        name = data[off + 2:off + 2 + n].decode()
        size, typ = struct.unpack_from(">Hi", data, off + 2 + n)
        off += 2 + n + 6 + 4 * size
        attrs.append((name, size, typ))
    width = 4 + sum(a[1] for a in attrs)
    end = off + 4 * width * counts[0]
    if data[end:] != b"\x00\xff":
        raise ValueError("bad trailer")
    rec = np.frombuffer(data[off:end], ">f4").astype(np.float32).reshape(counts[0], width)
    return tuple(attrs), rec


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
