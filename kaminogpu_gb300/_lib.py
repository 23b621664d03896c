"""ctypes binding of libkamino_gb300.so (declared in include/kamino_gb300.h).

The shared library is built in-tree by kaminogpu_gb300/build.py.  There is no
fallback: if the library is missing or fails to load, importing the package
raises, so no CPU path can stand in for the CUDA one.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libkamino_gb300.so")

# status codes (enum kamino_status)
OK, ERR_INVALID, ERR_CUDA, ERR_ALLOC, ERR_IO, ERR_BUDGET, ERR_TIMEOUT, ERR_NOT_READY, ERR_NOT_FOUND = range(9)
# fields (enum kamino_field)
U_PHI, U_THETA, THICKNESS, PRESSURE, PARTICLES = range(5)
FRAME_GRID, FRAME_PARTICLES = range(2)
# flags (enum kamino_flags)
F_PARTICLE_RK2, F_POLE_SIGN_FLIP, F_HONOR_STEP_DT, F_REFERENCE_ROUNDING = 1, 2, 4, 16


class KaminoError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("kamino status %d: %s" % (code, msg))
        self.code = code


class KaminoConfig(ctypes.Structure):
    _fields_ = [
        ("radius", ctypes.c_double),
        ("n_theta", ctypes.c_int32),
        ("frames", ctypes.c_int32),
        ("particle_density", ctypes.c_double),
        ("dt", ctypes.c_double),
        ("frame_dt", ctypes.c_double),
        ("A", ctypes.c_double),
        ("B", ctypes.c_int32),
        ("C", ctypes.c_int32),
        ("D", ctypes.c_int32),
        ("E", ctypes.c_int32),
        ("grid_path", ctypes.c_char * 256),
        ("particle_path", ctypes.c_char * 256),
        ("density_image", ctypes.c_char * 256),
        ("solid_image", ctypes.c_char * 256),
        ("color_image", ctypes.c_char * 256),
        ("n_particles", ctypes.c_int64),
        ("flags", ctypes.c_uint32),
        ("fp64_modes", ctypes.c_int32),
        ("device", ctypes.c_int32),
        ("reserved", ctypes.c_int32 * 7),
    ]


class KaminoInitSpec(ctypes.Structure):
    _fields_ = [
        ("n_theta", ctypes.c_int32),
        ("lmax", ctypes.c_int32),
        ("seed", ctypes.c_uint64),
        ("radius", ctypes.c_double),
        ("thickness_noise", ctypes.c_double),
        ("vortex", ctypes.c_int32),
        ("vortex_sigma", ctypes.c_double),
        ("vortex_amplitude", ctypes.c_double),
        ("velocity_scale", ctypes.c_double),
        ("n_particles", ctypes.c_int64),
        ("vortex_out", ctypes.c_double * 3),
    ]


class KaminoServerConfig(ctypes.Structure):
    _fields_ = [
        ("budget_bytes", ctypes.c_size_t),
        ("max_resident", ctypes.c_int32),
        ("steps_per_round", ctypes.c_int32),
        ("device", ctypes.c_int32),
        ("solo_n_theta", ctypes.c_int32),
        ("solo_slots", ctypes.c_int32),
        ("reserved", ctypes.c_int32 * 3),
    ]


class KaminoServerStats(ctypes.Structure):
    _fields_ = [
        ("submitted", ctypes.c_int64),
        ("completed", ctypes.c_int64),
        ("resident", ctypes.c_int64),
        ("queued", ctypes.c_int64),
        ("cell_steps", ctypes.c_int64),
        ("busy_seconds", ctypes.c_double),
        ("p50_latency_s", ctypes.c_double),
        ("p99_latency_s", ctypes.c_double),
        ("mean_latency_s", ctypes.c_double),
        ("resident_bytes", ctypes.c_size_t),
        ("peak_resident_bytes", ctypes.c_size_t),
        ("solo_cell_steps", ctypes.c_int64),
        ("batched_cell_steps", ctypes.c_int64),
        ("batched_rounds", ctypes.c_int64),
        ("batched_round_seconds", ctypes.c_double),
        ("solo_seconds", ctypes.c_double),
        ("poll_seconds", ctypes.c_double),
    ]


_P = ctypes.c_void_p
_I = ctypes.c_int
_I64 = ctypes.c_int64
_F = ctypes.c_float
_D = ctypes.c_double
_SZ = ctypes.c_size_t
_PF = ctypes.POINTER(ctypes.c_float)

# name: (restype, argtypes)
SIGNATURES = {
    "kamino_config_default": (_I, [ctypes.POINTER(KaminoConfig)]),
    "kamino_parse_config": (_I, [ctypes.c_char_p, ctypes.POINTER(KaminoConfig)]),
    "kamino_particle_count": (_I64, [ctypes.POINTER(KaminoConfig)]),
    "kamino_frame_steps": (_I64, [_D, _D, _I]),
    "kamino_abi_sizes": (_I, [ctypes.POINTER(_SZ), _I]),
    "kamino_create": (_I, [ctypes.POINTER(KaminoConfig), ctypes.POINTER(_P)]),
    "kamino_destroy": (_I, [_P]),
    "kamino_set_state": (_I, [_P, _I, _P, _SZ]),
    "kamino_get_state": (_I, [_P, _I, _P, _SZ]),
    "kamino_set_state_device": (_I, [_P, _I, _P, _SZ]),
    "kamino_get_state_device": (_I, [_P, _I, _P, _SZ]),
    "kamino_step": (_I, [_P, _F]),
    "kamino_step_host": (_I, [_P, _F, _P, _P, _P, _P, _P, _P, _SZ]),
    "kamino_init_fbm": (_I, [_P]),
    "kamino_reference_particles": (_I, [ctypes.POINTER(KaminoConfig), ctypes.c_uint32, _P, _I64]),
    "kamino_init_particles": (_I, [_P, ctypes.c_uint32]),
    "kamino_init_density_image": (_I, [_P, _P, _I, _I, _SZ]),
    "kamino_init_particle_colors_image": (_I, [_P, _P, _I, _I, _SZ]),
    "kamino_advection": (_I, [_P]),
    "kamino_geometric": (_I, [_P]),
    "kamino_projection": (_I, [_P]),
    "kamino_step_n": (_I, [_P, _I]),
    "kamino_projection_noalloc": (_I, [_I, _P, _P, _P, _P, _P, _P]),
    "kamino_run_frames": (_I, [_P, _I, ctypes.POINTER(_I64)]),
    "kamino_frame_bytes": (_I, [_P, _I, ctypes.POINTER(_SZ)]),
    "kamino_frame_capture": (_I, [_P, _I]),
    "kamino_frame_write": (_I, [_P, _I, ctypes.c_char_p, _P, _SZ]),
    "kamino_run_frames_bgeo": (_I, [_P, _I, ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(_I64)]),
    "kamino_frame_time_pack": (_I, [_P, _I, _I, _I, ctypes.POINTER(_D)]),
    "kamino_synchronize": (_I, [_P]),
    "kamino_save_state": (_I, [_P, ctypes.c_char_p]),
    "kamino_load_state": (_I, [_P, ctypes.c_char_p]),
    "kamino_time_elapsed": (_I, [_P, ctypes.POINTER(_D), ctypes.POINTER(_I64)]),
    "kamino_time_steps": (_I, [_P, _I, _I, ctypes.POINTER(_D)]),
    "kamino_time_kernels": (_I, [_P, _I, _I, ctypes.POINTER(_D), _I, ctypes.POINTER(_I)]),
    "kamino_kernel_name": (ctypes.c_char_p, [_I]),
    "kamino_launches_per_step": (_I, [_P]),
    "kamino_device_bytes": (_I, [_P, ctypes.POINTER(_SZ)]),
    "kamino_last_error": (ctypes.c_char_p, []),
    "kamino_host_alloc": (_I, [_SZ, ctypes.POINTER(_P)]),
    "kamino_host_free": (_I, [_P]),
    "kamino_probe_index": (_I, [_P, _I, _P, _P, _I64, _P, _P]),
    "kamino_probe_wrap": (_I, [_P, _P, _P, _I64, _P]),
    "kamino_init_spec_default": (_I, [ctypes.POINTER(KaminoInitSpec)]),
    "kamino_make_initial_state": (_I, [ctypes.POINTER(KaminoInitSpec), _P, _P, _P, _P]),
    "kamino_batch_create": (_I, [ctypes.POINTER(KaminoConfig), _I, ctypes.POINTER(_P)]),
    "kamino_batch_destroy": (_I, [_P]),
    "kamino_batch_set_state": (_I, [_P, _I, _I, _P, _SZ]),
    "kamino_batch_get_state": (_I, [_P, _I, _I, _P, _SZ]),
    "kamino_batch_step_n": (_I, [_P, _I]),
    "kamino_batch_synchronize": (_I, [_P]),
    "kamino_batch_time_steps": (_I, [_P, _I, _I, ctypes.POINTER(_D)]),
    "kamino_batch_autotune": (_I, [_P, _I, ctypes.POINTER(_I), _I]),
    "kamino_batch_cells": (_I64, [_P]),
    "kamino_server_create": (_I, [ctypes.POINTER(KaminoServerConfig), ctypes.POINTER(_P)]),
    "kamino_server_destroy": (_I, [_P]),
    "kamino_server_submit": (_I, [_P, ctypes.POINTER(KaminoConfig), _P, _P, _P, ctypes.c_int32, _D,
                                  ctypes.POINTER(_I64)]),
    "kamino_server_poll": (_I, [_P, ctypes.POINTER(_I)]),
    "kamino_server_fetch": (_I, [_P, _I64, _I, _P]),
    "kamino_server_release": (_I, [_P, _I64]),
    "kamino_server_get_stats": (_I, [_P, ctypes.POINTER(KaminoServerStats)]),
    "kamino_server_now": (_D, [_P]),
}


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            "libkamino_gb300.so not built (%s); run `python -c \"import __graft_entry__ as g; g.build()\"`"
            % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    return lib


lib = _load()


def last_error():
    s = lib.kamino_last_error()
    return s.decode() if s else ""


def check(rc):
    if rc != OK:
        raise KaminoError(rc, last_error())
    return rc
