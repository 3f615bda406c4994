"""ctypes binding of libgsap.so (the C ABI declared in include/gsap.h).

The library is built in-tree by ``gsap_gb300.build`` (or
``__graft_entry__.build()``).  There is no fallback: if the shared library
is missing, importing a GPU entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgsap.so")

GSAP_OK = 0
STATUS_NAMES = {0: "GSAP_OK", 1: "GSAP_ERR_INVALID", 2: "GSAP_ERR_CAPACITY", 3: "GSAP_ERR_CUDA",
                4: "GSAP_ERR_DEVICE_TIMEOUT", 5: "GSAP_ERR_NONFINITE"}
MODE_AABB, MODE_SPHERE = 0, 1
SORT_RADIX, SORT_BUCKET = 0, 1
AXIS_PCA, AXIS_REF = 0, 1
FLAG_SORTED, FLAG_GRAPH, FLAG_TEMPORAL = 0x1, 0x2, 0x4
CONTACT_REF, CONTACT_CONFIG = 0, 1


class GsapError(RuntimeError):
    def __init__(self, status: int, msg: str):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")


class Config(C.Structure):
    _fields_ = [("mode", C.c_uint32), ("axis_mode", C.c_uint32), ("max_scenes", C.c_uint32),
                ("entry_factor", C.c_uint32), ("pair_factor", C.c_uint32), ("sort_bits", C.c_uint32),
                ("cell_factor", C.c_float), ("spin_limit", C.c_uint32), ("sort_mode", C.c_uint32),
                ("sort_tile", C.c_uint32)]


class BodyData(C.Structure):
    _fields_ = [("n_bodies", C.c_int32), ("n_total_particles", C.c_int32)] + [
        (n, C.c_void_p) for n in ("pos", "quat", "lin_vel", "ang_vel", "shape_idx", "p_start", "n_part",
                                  "inv_mass", "inv_inertia")]


class ContactParams(C.Structure):
    _fields_ = [("model", C.c_uint32), ("sp_multip", C.c_float), ("dp_multip", C.c_float),
                ("max_lin_vel", C.c_float), ("gravity_y", C.c_float), ("floor_clamp", C.c_uint32),
                ("torque_quirk", C.c_uint32), ("pair_loop_quirk", C.c_uint32), ("k", C.c_float), ("eta", C.c_float), ("kt", C.c_float),
                ("box_lo", C.c_float * 3), ("box_hi", C.c_float * 3)]


# (name, restype, argtypes) of every exported symbol of include/gsap.h and include/gsap_debug.h
P, U32, U64, I32, F32, F64 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int32, C.c_float, C.c_double
PU64 = C.POINTER(C.c_uint64)
PI32 = C.POINTER(C.c_int32)
SIGNATURES = [
    ("gsap_config_default", None, [C.POINTER(Config)]),
    ("gsap_last_error", C.c_char_p, []),
    ("gsap_sap_create", P, [U32, C.POINTER(Config)]),
    ("gsap_sap_destroy", None, [P]),
    ("gsap_sap_collision", I32, [P, F32, P, U32, P, P, PI32, PI32, U64, U64, P]),
    ("gsap_broadphase_aabb", I32, [P, P, P, U32, P, U64, P, PU64, U32, P]),
    ("gsap_broadphase_batched", I32, [P, P, P, P, U32, U32, P, U64, P, PU64, U32, P]),
    ("gsap_sap_check", I32, [P, P]),
    ("gsap_sap_scene_axes", I32, [P, U32, C.POINTER(F64), P]),
    ("gsap_sap_stage_times", C.c_int, [P, C.POINTER(F32), C.c_int]),
    ("gsap_sap_enable_timing", None, [P, C.c_int]),
    ("gsap_sap_autotune", I32, [P, P, P, P, U32, U32, P, U64, U32, C.c_int, C.POINTER(Config), P]),
    ("gsap_radix_sort_u32", I32, [P, P, P, U32, U32, P]),
    ("gsap_radix_sort_f32", I32, [P, P, P, U32, U32, C.c_int, P]),
    ("gsap_radix_sort_u32_noalloc", I32, [P, P, U32, U32, P]),
    ("gsap_rb_create", P, [I32, I32, I32]),
    ("gsap_rb_destroy", None, [P]),
    ("gsap_rb_set_body_data", I32, [P, C.POINTER(BodyData)]),
    ("gsap_rb_set_particle_data", I32, [P, P, P, I32]),
    ("gsap_rb_set_shape_inv_inertia", I32, [P, P, I32]),
    ("gsap_rb_set_contact", I32, [P, C.POINTER(ContactParams)]),
    ("gsap_rb_set_scenes", I32, [P, P, U32]),
    ("gsap_rb_update_particle_data", I32, [P, P]),
    ("gsap_rb_prepare", I32, [P, P]),
    ("gsap_rb_compute_forces", I32, [P, F32, P]),
    ("gsap_rb_update_velocity", I32, [P, F32, P]),
    ("gsap_rb_integrate", I32, [P, F32, P]),
    ("gsap_rb_pairs", P, [P]),
    ("gsap_rb_pair_entries", P, [P]),
    ("gsap_rb_set_num_pairs", I32, [P, I32, I32]),
    ("gsap_rb_particle_pos", P, [P]),
    ("gsap_rb_particle_vel", P, [P]),
    ("gsap_rb_particle_force", P, [P]),
    ("gsap_rb_step", I32, [P, P, F32, P]),
    ("gsap_rb_get_state", I32, [P, P, P, P, P, P]),
    ("gsap_rb_set_state", I32, [P, P, P, P, P, P]),
    ("gsap_rb_copy_out", I32, [P, I32, P, U64, P]),
    ("gsap_rb_copy_in", I32, [P, I32, P, U64, P]),
    ("gsap_k_integrate", I32, [P, P, P, P, F32, I32, C.POINTER(ContactParams), P]),
    ("gsap_k_update_particle_data", I32, [P, P, P, P, P, P, P, P, P, P, P, P, I32, P]),
    ("gsap_k_prepare", I32, [P, P, P, P, I32, P]),
    ("gsap_k_clear_force_and_boundary", I32, [P, P, P, P, F32, F32, I32, F32, P]),
    ("gsap_k_compute_force_on_particles", I32, [P, P, P, P, I32, I32, P, F32, F32, P, F32, I32, P]),
    ("gsap_k_update_velocity", I32, [P, P, P, P, P, P, P, P, P, P, I32, F32, F32, I32, I32, P]),
    ("gsap_debug_scene_solve", C.c_int, [C.POINTER(F64), C.POINTER(F64), C.POINTER(F64), F64, U32, U32, F32,
                                         U32, U64, C.POINTER(F64)]),
    ("gsap_debug_lookback_timeout", C.c_int, [P, U32, P]),
    ("gsap_debug_stats", C.c_int, [P, C.POINTER(U64), P]),
    ("gsap_debug_sizes", C.c_int, [C.POINTER(U32)]),
    ("gsap_debug_rb_contacts", C.c_int, [P, C.POINTER(U64), C.c_int, P]),
    ("gsap_debug_graph_cache", C.c_int, [P, U32, C.POINTER(U32)]),
]

_LIB = None


def load(path: str = LIB_PATH):
    """Load libgsap.so and bind every entry point.  Raises if it is missing."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with gsap_gb300.build.build() "
                           "(there is no CPU fallback)")
    lib = C.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def check(status: int) -> None:
    if status != GSAP_OK:
        raise GsapError(status, load().gsap_last_error().decode())


def last_error() -> str:
    return load().gsap_last_error().decode()
