"""Host-side mirror of the reference's solver surface over the C ABI.

KaminoSolver keeps the reference's constructor and method names
(KaminoGPU/include/KaminoSolver.cuh:99-110, KaminoGPU/kernel/KaminoSolver.cu):
  KaminoSolver(nPhi, nTheta, radius, frameDuration, A, B, C, D, E)
  stepForward(dt)                           KaminoSolver.cu:197-221
  advection() / geometric() / projection()  KaminoCore.cu:344, 551, 749
  copyToGPU / copyBackToCPU per field       KaminoQuantity.cu:3-18
  write_data_bgeo / write_particles_bgeo    KaminoSolver.cu:284-396
Errors raise KaminoError instead of exiting the process.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import (FRAME_GRID, FRAME_PARTICLES, PARTICLES, PRESSURE, THICKNESS, U_PHI, U_THETA, KaminoConfig, KaminoInitSpec, check,
                   lib)

_FIELD_NAMES = {"velPhi": U_PHI, "velTheta": U_THETA, "density": THICKNESS, "thickness": THICKNESS,
                "p": PRESSURE, "pressure": PRESSURE, "particles": PARTICLES}


def default_config(**kw):
    c = KaminoConfig()
    check(lib.kamino_config_default(ctypes.byref(c)))
    for k, v in kw.items():
        if isinstance(v, str):
            v = v.encode()
        setattr(c, k, v)
    return c


def parse_config(path):
    """Positional configKamino.txt (KaminoGPU/kernel/main.cu:17-45)."""
    c = KaminoConfig()
    check(lib.kamino_parse_config(str(path).encode(), ctypes.byref(c)))
    return c


def particle_count(cfg):
    return int(lib.kamino_particle_count(ctypes.byref(cfg)))


def frame_steps(dt, frame_dt, frames):
    return int(lib.kamino_frame_steps(dt, frame_dt, frames))


def make_initial_state(n_theta, lmax=8, seed=1, radius=1.0, thickness_noise=0.05, vortex=False,
                       vortex_sigma=0.1, velocity_scale=1.0, n_particles=0):
    """Seeded synthetic state: returns dict of float32 arrays (+ vortex info)."""
    s = KaminoInitSpec()
    check(lib.kamino_init_spec_default(ctypes.byref(s)))
    s.n_theta, s.lmax, s.seed, s.radius = n_theta, lmax, seed, radius
    s.thickness_noise, s.vortex, s.vortex_sigma = thickness_noise, int(bool(vortex)), vortex_sigma
    s.velocity_scale, s.n_particles = velocity_scale, n_particles
    nt, npp = n_theta, 2 * n_theta
    u = np.empty((nt, npp), np.float32)
    v = np.empty((nt - 1, npp), np.float32)
    rho = np.empty((nt, npp), np.float32)
    part = np.empty((max(n_particles, 1), 2), np.float32)
    check(lib.kamino_make_initial_state(ctypes.byref(s), u.ctypes.data, v.ctypes.data, rho.ctypes.data,
                                        part.ctypes.data))
    return {"u_phi": u, "u_theta": v, "thickness": rho, "particles": part[:n_particles],
            "vortex": tuple(s.vortex_out)}


class KaminoSolver:
    """One sphere on the GPU.  Construct from a KaminoConfig (config=...) or
    with the reference's positional arguments."""

    def __init__(self, nPhi=None, nTheta=None, radius=None, frameDuration=None, A=0.0, B=1, C=1, D=1, E=1,
                 *, config=None, **ext):
        if config is None:
            if nTheta is None or nPhi != 2 * nTheta:
                raise ValueError("nPhi must be 2 * nTheta (KaminoCore.cu:849)")
            # frameDuration receives dt in Kamino::run (KaminoCore.cu:862)
            config = default_config(n_theta=nTheta, radius=radius, dt=frameDuration, A=A, B=B, C=C, D=D, E=E)
        for k, v in ext.items():
            setattr(config, k, v)
        self.config = config
        self.nTheta = config.n_theta
        self.nPhi = 2 * config.n_theta
        self.n_particles = particle_count(config)
        h = ctypes.c_void_p()
        check(lib.kamino_create(ctypes.byref(config), ctypes.byref(h)))
        self._h = h

    # ------------------------------------------------------------ lifetime
    def close(self):
        if getattr(self, "_h", None):
            lib.kamino_destroy(self._h)
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

    # -------------------------------------------------------------- state
    def _shape(self, field):
        if field == PARTICLES:
            return (self.n_particles, 2)
        return (self.nTheta - 1 if field == U_THETA else self.nTheta, self.nPhi)

    def set_state(self, field, arr):
        field = _FIELD_NAMES.get(field, field)
        a = np.ascontiguousarray(arr, dtype=np.float32)
        if a.shape != self._shape(field):
            raise ValueError("field %d expects shape %s, got %s" % (field, self._shape(field), a.shape))
        check(lib.kamino_set_state(self._h, field, a.ctypes.data, a.strides[0] if a.ndim == 2 else 0))

    def get_state(self, field):
        field = _FIELD_NAMES.get(field, field)
        out = np.empty(self._shape(field), np.float32)
        if out.size:
            check(lib.kamino_get_state(self._h, field, out.ctypes.data, out.strides[0]))
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

    # -------------------------------------------------------------- steps
    def stepForward(self, dt=None):
        check(lib.kamino_step(self._h, self.config.dt if dt is None else dt))

    def init_fbm(self):
        """The reference's FBM curl-noise velocity (kamino_init_fbm)."""
        check(lib.kamino_init_fbm(self._h))

    initialize_velocity = init_fbm  # KaminoSolver::initialize_velocity, KaminoInitializer.cu:3-85

    def initParticlesfromPic(self, image=None, seed=1):
        """KaminoSolver::initParticlesfromPic: the reference's jittered
        particle placement (kamino_init_particles) and, given a decoded image
        (uint8 [height, width, 3], B G R), the particles' colours from it."""
        check(lib.kamino_init_particles(self._h, seed))
        if image is not None:
            a = np.ascontiguousarray(image, np.uint8)
            check(lib.kamino_init_particle_colors_image(self._h, a.ctypes.data, a.shape[1], a.shape[0], a.strides[0]))

    def initDensityfromPic(self, image):
        """KaminoSolver::initDensityfromPic with a decoded image (uint8
        [height, width, 3], B G R): the thickness from the mirrored, resampled
        image (kamino_init_density_image)."""
        a = np.ascontiguousarray(image, np.uint8)
        check(lib.kamino_init_density_image(self._h, a.ctypes.data, a.shape[1], a.shape[0], a.strides[0]))

    def step_host(self, u_phi, u_theta, thickness, dt=None):
        """One step with the state in host memory (kamino_step_host): uploads
        the three fields, steps, and returns the new three as arrays."""
        ins = [np.ascontiguousarray(a, dtype=np.float32) for a in (u_phi, u_theta, thickness)]
        for f, a in zip((U_PHI, U_THETA, THICKNESS), ins):
            if a.shape != self._shape(f):
                raise ValueError("field %d expects shape %s, got %s" % (f, self._shape(f), a.shape))
        outs = [np.empty_like(a) for a in ins]
        check(lib.kamino_step_host(self._h, self.config.dt if dt is None else dt, *[a.ctypes.data for a in ins],
                                   *[o.ctypes.data for o in outs], ins[0].strides[0]))
        return outs

    def advection(self):
        check(lib.kamino_advection(self._h))

    def geometric(self):
        check(lib.kamino_geometric(self._h))

    def projection(self):
        check(lib.kamino_projection(self._h))

    def step_n(self, n):
        check(lib.kamino_step_n(self._h, n))

    def run_frames(self, frames):
        n = ctypes.c_int64()
        check(lib.kamino_run_frames(self._h, frames, ctypes.byref(n)))
        return n.value

    def synchronize(self):
        check(lib.kamino_synchronize(self._h))

    def save_state(self, path):
        """Checkpoint the sphere to a file (kamino_save_state)."""
        check(lib.kamino_save_state(self._h, str(path).encode()))

    def load_state(self, path):
        """Resume from a checkpoint of the same configuration (kamino_load_state)."""
        check(lib.kamino_load_state(self._h, str(path).encode()))

    # ------------------------------------------------------- frame output
    def frame_bytes(self, kind=FRAME_GRID):
        n = ctypes.c_size_t()
        check(lib.kamino_frame_bytes(self._h, kind, ctypes.byref(n)))
        return n.value

    def capture_frame(self, kind=FRAME_GRID):
        """Queue a snapshot of the current state as a .bgeo frame; returns at
        once (kamino_frame_capture)."""
        check(lib.kamino_frame_capture(self._h, kind))

    def write_frame(self, kind=FRAME_GRID, path=None):
        """Oldest captured frame (or the current state) as .bgeo bytes; also
        written to path when given (kamino_frame_write)."""
        buf = ctypes.create_string_buffer(self.frame_bytes(kind))
        check(lib.kamino_frame_write(self._h, kind, None if path is None else str(path).encode(), buf,
                                     len(buf)))
        return buf.raw

    def write_data_bgeo(self, s, frame):
        """KaminoSolver::write_data_bgeo: the grid frame to s + frame + ".bgeo"."""
        check(lib.kamino_frame_write(self._h, FRAME_GRID, ("%s%d.bgeo" % (s, frame)).encode(), None, 0))

    def write_particles_bgeo(self, s, frame):
        """KaminoSolver::write_particles_bgeo: the particles to s + frame + ".bgeo"."""
        check(lib.kamino_frame_write(self._h, FRAME_PARTICLES, ("%s%d.bgeo" % (s, frame)).encode(), None, 0))

    def run_frames_bgeo(self, frames, grid_path=None, particle_path=None):
        """Kamino::run with its .bgeo output (kamino_run_frames_bgeo)."""
        n = ctypes.c_int64()
        enc = lambda p: None if p is None else str(p).encode()
        check(lib.kamino_run_frames_bgeo(self._h, frames, enc(grid_path), enc(particle_path), ctypes.byref(n)))
        return n.value

    def time_frame_pack(self, kind=FRAME_GRID, reps=10, flush_l2=True):
        ms = ctypes.c_double()
        check(lib.kamino_frame_time_pack(self._h, kind, reps, int(flush_l2), ctypes.byref(ms)))
        return ms.value

    def time_elapsed(self):
        t, s = ctypes.c_double(), ctypes.c_int64()
        check(lib.kamino_time_elapsed(self._h, ctypes.byref(t), ctypes.byref(s)))
        return t.value, s.value

    # ------------------------------------------------------------ timing
    def time_steps(self, n, flush_l2=True):
        ms = ctypes.c_double()
        check(lib.kamino_time_steps(self._h, n, int(flush_l2), ctypes.byref(ms)))
        return ms.value

    def time_kernels(self, reps=5, flush_l2=True):
        ms = (ctypes.c_double * 16)()
        cnt = ctypes.c_int()
        check(lib.kamino_time_kernels(self._h, reps, int(flush_l2), ms, 16, ctypes.byref(cnt)))
        return {lib.kamino_kernel_name(i).decode(): ms[i] for i in range(cnt.value)}

    def launches_per_step(self):
        return int(lib.kamino_launches_per_step(self._h))

    def device_bytes(self):
        n = ctypes.c_size_t()
        check(lib.kamino_device_bytes(self._h, ctypes.byref(n)))
        return n.value

    # ------------------------------------------------------------ probes
    def probe_index(self, kind, phi, theta):
        phi = np.ascontiguousarray(phi, np.float32)
        theta = np.ascontiguousarray(theta, np.float32)
        n = phi.size
        out = np.empty((n, 4), np.int32)
        alpha = np.empty((n, 2), np.float32)
        check(lib.kamino_probe_index(self._h, kind, phi.ctypes.data, theta.ctypes.data, n, out.ctypes.data,
                                     alpha.ctypes.data))
        return out, alpha

    def probe_wrap(self, phi, theta):
        phi = np.array(phi, np.float32)
        theta = np.array(theta, np.float32)
        cells = np.empty((phi.size, 2), np.int32)
        check(lib.kamino_probe_wrap(self._h, phi.ctypes.data, theta.ctypes.data, phi.size, cells.ctypes.data))
        return phi, theta, cells


def read_ppm(path):
    """A binary PPM (P6, maxval 255) as uint8 [height, width, 3] in B, G, R
    order (the order the image entry points take, OpenCV's)."""
    data = open(path, "rb").read()
    fields, pos = [], 2
    if data[:2] != b"P6":
        raise ValueError("%s: not a binary PPM" % path)
    while len(fields) < 3:
        while pos < len(data) and (data[pos:pos + 1].isspace() or data[pos:pos + 1] == b"#"):
            if data[pos:pos + 1] == b"#":
                pos = data.index(b"\n", pos)
            pos += 1
        start = pos
        while pos < len(data) and data[pos:pos + 1].isdigit():
            pos += 1
        fields.append(int(data[start:pos]))
    w, h, maxval = fields
    if maxval != 255:
        raise ValueError("%s: only 8-bit PPM is supported" % path)
    pix = np.frombuffer(data, np.uint8, w * h * 3, pos + 1).reshape(h, w, 3)
    return np.ascontiguousarray(pix[..., ::-1])


class Kamino:
    """The reference's top-level driver (KaminoGPU/include/KaminoGPU.cuh:40-48,
    Kamino::run at KaminoGPU/kernel/KaminoCore.cu:860-912) over the C ABI:
    the solver with the FBM velocity, the density and colour images (binary
    PPM here; the reference reads any format with OpenCV), the particle
    placement, and the frame loop writing <gridPath><i>.bgeo and
    <particlePath><i>.bgeo for frames 0 .. frames."""

    def __init__(self, radius, nTheta, particleDensity, dt, DT, frames, A=0.0, B=1, C=1, D=1, E=1,
                 gridPath="", particlePath="", densityImage="", solidImage="", colorImage="", **ext):
        self.config = default_config(radius=radius, n_theta=nTheta, particle_density=particleDensity, dt=dt,
                                     frame_dt=DT, frames=frames, A=A, B=B, C=C, D=D, E=E, grid_path=gridPath,
                                     particle_path=particlePath, density_image=densityImage,
                                     solid_image=solidImage, color_image=colorImage, n_particles=-1, **ext)

    @classmethod
    def from_config(cls, path, **ext):
        """main(configKamino.txt) (KaminoGPU/kernel/main.cu:17-45)."""
        k = cls.__new__(cls)
        k.config = parse_config(path)
        for a, v in ext.items():
            setattr(k.config, a, v.encode() if isinstance(v, str) else v)
        return k

    def run(self):
        """Kamino::run; returns the number of steps taken."""
        c = self.config
        with KaminoSolver(config=c) as s:
            s.init_fbm()
            if c.density_image:
                s.initDensityfromPic(read_ppm(c.density_image.decode()))
            s.initParticlesfromPic(read_ppm(c.color_image.decode()) if c.color_image else None)
            return s.run_frames_bgeo(c.frames, c.grid_path.decode() or None, c.particle_path.decode() or None)
