"""ctypes binding of libsi_cuda (include/si_cuda.h). Loading fails loudly: there is no CPU path."""
import ctypes
import os

from . import build as _build

c_int32_p = ctypes.POINTER(ctypes.c_int32)
c_int64_p = ctypes.POINTER(ctypes.c_int64)
c_uint32_p = ctypes.POINTER(ctypes.c_uint32)
c_uint64_p = ctypes.POINTER(ctypes.c_uint64)
c_float_p = ctypes.POINTER(ctypes.c_float)
c_double_p = ctypes.POINTER(ctypes.c_double)
vp = ctypes.c_void_p

SI_OK, SI_EINVAL, SI_ENOMEM, SI_EDESTROYED, SI_EDEVICE, SI_ETIMEOUT, SI_EBUSY = range(7)
CODE_NAMES = {SI_EINVAL: "invalid-argument", SI_ENOMEM: "out-of-memory", SI_EDESTROYED: "destroyed",
              SI_EDEVICE: "no-device", SI_ETIMEOUT: "timeout", SI_EBUSY: "busy"}


class si_mpm_desc(ctypes.Structure):
    _fields_ = [("max_particles", ctypes.c_int64), ("grid", ctypes.c_int32), ("sort_every", ctypes.c_int32),
                ("substeps", ctypes.c_int32), ("ppc_axis", ctypes.c_int32), ("size", ctypes.c_double * 3),
                ("origin", ctypes.c_double * 3), ("gravity", ctypes.c_double * 3), ("time_scale", ctypes.c_double)]


class si_mpm_info(ctypes.Structure):
    _fields_ = [("count", ctypes.c_int64), ("max_particles", ctypes.c_int64), ("step_count", ctypes.c_int64),
                ("dims", ctypes.c_int32 * 3), ("num_materials", ctypes.c_int32), ("num_colliders", ctypes.c_int32),
                ("sort_every", ctypes.c_int32), ("substeps", ctypes.c_int32), ("ppc_axis", ctypes.c_int32),
                ("bound", ctypes.c_int32), ("num_nodes", ctypes.c_int64), ("num_blocks", ctypes.c_uint32),
                ("dx", ctypes.c_double), ("substep_dt", ctypes.c_double), ("time_scale", ctypes.c_double),
                ("origin", ctypes.c_double * 3), ("gravity", ctypes.c_double * 3), ("device_bytes", ctypes.c_int64)]


class si_material_def(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("density", ctypes.c_double), ("stiffness", ctypes.c_double),
                ("poisson", ctypes.c_double), ("viscosity", ctypes.c_double), ("hardening", ctypes.c_double),
                ("compression", ctypes.c_double), ("stretch", ctypes.c_double), ("friction_deg", ctypes.c_double)]


class si_server_stats(ctypes.Structure):
    _fields_ = [("requests_done", ctypes.c_int64), ("substeps_done", ctypes.c_int64),
                ("particle_substeps", ctypes.c_int64), ("ticks", ctypes.c_int64), ("p50_ms", ctypes.c_double),
                ("p99_ms", ctypes.c_double), ("mean_ms", ctypes.c_double), ("max_ms", ctypes.c_double),
                ("busy_s", ctypes.c_double), ("resident_bytes", ctypes.c_int64), ("budget_bytes", ctypes.c_int64),
                ("resident_scenes", ctypes.c_int32), ("queued_requests", ctypes.c_int32)]


# name: (restype, argtypes) — every function declared in include/si_cuda.h
SIGNATURES = {
    "si_last_error": (ctypes.c_char_p, []),
    "si_version": (ctypes.c_char_p, []),
    "si_world_create": (ctypes.c_int, [ctypes.POINTER(vp)]),
    "si_world_destroy": (ctypes.c_int, [vp]),
    "si_world_step": (ctypes.c_int, [vp, ctypes.c_int32]),
    "si_world_sync": (ctypes.c_int, [vp]),
    "si_world_set_graphs": (ctypes.c_int, [vp, ctypes.c_int32]),
    "si_world_set_svd_tolerance": (ctypes.c_int, [vp, ctypes.c_int32]),
    "si_world_profile": (ctypes.c_int, [vp, ctypes.c_int32, c_double_p, ctypes.c_int32]),
    "si_world_set_tuning": (ctypes.c_int, [vp, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]),
    "si_world_mark": (ctypes.c_int, [vp, ctypes.c_int32]),
    "si_world_elapsed": (ctypes.c_int, [vp, ctypes.c_int32, ctypes.c_int32, c_double_p]),
    "si_world_launches": (ctypes.c_int, [vp, c_int64_p]),
    "si_mpm_desc_default": (None, [ctypes.POINTER(si_mpm_desc)]),
    "si_mpm_create": (ctypes.c_int, [vp, ctypes.POINTER(si_mpm_desc), ctypes.POINTER(vp)]),
    "si_mpm_destroy": (ctypes.c_int, [vp]),
    "si_mpm_free": (None, [vp]),
    "si_mpm_get_info": (ctypes.c_int, [vp, ctypes.POINTER(si_mpm_info)]),
    "si_mpm_set_materials": (ctypes.c_int, [vp, c_float_p, ctypes.c_int32]),
    "si_mpm_add_particles": (ctypes.c_int, [vp, c_float_p, ctypes.c_int64, c_int64_p]),
    "si_mpm_clear": (ctypes.c_int, [vp]),
    "si_mpm_write_particles": (ctypes.c_int, [vp, c_float_p, ctypes.c_int64, ctypes.c_int64]),
    "si_mpm_read_particles": (ctypes.c_int, [vp, c_float_p, ctypes.c_int64, ctypes.c_int64]),
    "si_mpm_read_positions": (ctypes.c_int, [vp, c_float_p, ctypes.c_int64, ctypes.c_int64]),
    "si_mpm_set_colliders": (ctypes.c_int, [vp, c_float_p, ctypes.c_int32]),
    "si_mpm_set_gravity": (ctypes.c_int, [vp, c_double_p]),
    "si_mpm_set_sort_every": (ctypes.c_int, [vp, ctypes.c_int32]),
    "si_mpm_set_substep_dt": (ctypes.c_int, [vp, ctypes.c_double]),
    "si_mpm_set_frame": (ctypes.c_int, [vp, ctypes.c_int32, ctypes.c_double]),
    "si_mpm_step": (ctypes.c_int, [vp, ctypes.c_double, ctypes.c_int32]),
    "si_mpm_sort": (ctypes.c_int, [vp]),
    "si_mpm_p2g": (ctypes.c_int, [vp, ctypes.c_int32]),
    "si_mpm_grid_update": (ctypes.c_int, [vp]),
    "si_mpm_g2p": (ctypes.c_int, [vp]),
    "si_mpm_read_grid": (ctypes.c_int, [vp, c_int32_p]),
    "si_mpm_read_bins": (ctypes.c_int, [vp, c_uint32_p, c_uint32_p]),
    "si_mpm_sync": (ctypes.c_int, [vp]),
    "si_block_sort_noalloc": (ctypes.c_int, [c_float_p, ctypes.c_int64, ctypes.c_int32, c_int32_p, c_uint32_p,
                                             c_uint32_p, c_uint32_p, vp]),
    "si_material_preset": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(si_material_def)]),
    "si_material_row": (ctypes.c_int, [ctypes.POINTER(si_material_def), ctypes.c_int32, c_float_p]),
    "si_sample_shape": (ctypes.c_int, [ctypes.c_int32, c_double_p, c_double_p, ctypes.c_double, ctypes.c_double,
                                       ctypes.c_double, ctypes.c_double, ctypes.c_uint32, c_float_p, ctypes.c_int64,
                                       c_int64_p]),
    "si_make_records": (ctypes.c_int, [vp, c_float_p, ctypes.c_int64, ctypes.c_int32, c_double_p, ctypes.c_double,
                                       c_float_p]),
    "si_collider_row": (ctypes.c_int, [vp, ctypes.c_int32, c_double_p, c_double_p, ctypes.c_double, ctypes.c_double,
                                       c_double_p, ctypes.c_double, c_float_p]),
    "si_mpm_emit": (ctypes.c_int, [vp, ctypes.c_int32, c_double_p, c_double_p, ctypes.c_double, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_uint32, ctypes.c_int32, c_double_p,
                                   ctypes.POINTER(ctypes.c_int64)]),
    "si_mpm_read_positions_async": (ctypes.c_int, [vp, c_float_p, ctypes.c_int64, ctypes.c_int64, c_uint64_p]),
    "si_mpm_read_wait": (ctypes.c_int, [vp, ctypes.c_uint64]),
    "si_mpm_device_ptr": (ctypes.c_int, [vp, ctypes.c_int32, ctypes.POINTER(vp), ctypes.POINTER(ctypes.c_int64),
                                         ctypes.POINTER(ctypes.c_int64)]),
    "si_mpm_read_instances": (ctypes.c_int, [vp, c_float_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_uint32,
                                             ctypes.c_double]),
    "si_mpm_couple": (ctypes.c_int, [vp, c_float_p, ctypes.c_int32, ctypes.c_double, ctypes.c_double, ctypes.c_uint32,
                                     ctypes.c_double]),
    "si_mpm_set_bodies": (ctypes.c_int, [vp, c_float_p, ctypes.c_int32]),
    "si_mpm_read_impulses": (ctypes.c_int, [vp, c_float_p, ctypes.c_int32]),
    "si_spatial_create": (ctypes.c_int, [vp, ctypes.c_int64, c_double_p, c_double_p, ctypes.c_double,
                                         ctypes.POINTER(vp)]),
    "si_spatial_destroy": (ctypes.c_int, [vp]),
    "si_spatial_info": (ctypes.c_int, [vp, c_int32_p, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]),
    "si_spatial_build": (ctypes.c_int, [vp, c_float_p, ctypes.c_int64]),
    "si_spatial_build_mpm": (ctypes.c_int, [vp, vp]),
    "si_spatial_read": (ctypes.c_int, [vp, c_uint32_p, c_uint32_p]),
    "si_spatial_gather": (ctypes.c_int, [vp, c_float_p, c_float_p, ctypes.c_int32]),
    "si_server_create": (ctypes.c_int, [vp, ctypes.c_int64, ctypes.POINTER(vp)]),
    "si_server_destroy": (ctypes.c_int, [vp]),
    "si_server_admit": (ctypes.c_int, [vp, ctypes.POINTER(si_mpm_desc), ctypes.POINTER(vp)]),
    "si_server_retire": (ctypes.c_int, [vp, vp]),
    "si_server_submit": (ctypes.c_int, [vp, vp, ctypes.c_double, ctypes.c_int32, c_uint64_p]),
    "si_server_submit_colliders": (ctypes.c_int, [vp, vp, ctypes.c_double, ctypes.c_int32, vp, ctypes.c_int32,
                                                  c_uint64_p]),
    "si_server_poll": (ctypes.c_int, [vp, ctypes.c_uint64, c_int32_p, c_int32_p]),
    "si_server_wait": (ctypes.c_int, [vp, ctypes.c_uint64, ctypes.c_int32, c_int32_p]),
    "si_server_stats_get": (ctypes.c_int, [vp, ctypes.POINTER(si_server_stats), ctypes.c_int32]),
    "si_server_call": (ctypes.c_int, [vp, ctypes.CFUNCTYPE(None, vp), vp]),
}

_lib = None


class SIError(RuntimeError):
    """Mirror of the reference's SIError (src/core/errors.js): message + code."""

    def __init__(self, msg, code="error", status=None):
        super().__init__(msg if msg.startswith("ShaderIntel") else "ShaderIntel: " + msg)
        self.code = code
        self.status = status


def lib():
    """The loaded library (built on first use). Raises if it cannot be built or loaded."""
    global _lib
    if _lib is None:
        path = _build.LIB if os.path.exists(_build.LIB) and not _build._stale() else _build.build()
        L = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(rc):
    if rc != SI_OK:
        msg = lib().si_last_error().decode(errors="replace")
        raise SIError(msg or f"error {rc}", CODE_NAMES.get(rc, "error"), rc)
    return rc


def fptr(a):
    return a.ctypes.data_as(c_float_p)


def dptr(seq):
    return (ctypes.c_double * 3)(*[float(x) for x in seq])
