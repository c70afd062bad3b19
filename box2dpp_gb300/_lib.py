"""ctypes binding of ``libbox2d_gb300.so`` (the C-ABI in ``include/box2d_gb300.h``).

The library is built in-tree by ``box2dpp_gb300.build``. There is no fallback: if the library is
missing and cannot be built, importing the world API raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

GB_OK, GB_ERR_CAPACITY, GB_ERR_TIMEOUT, GB_ERR_INVALID, GB_ERR_CUDA = 0, 1, 2, 3, 4
COLLIDE_NOALLOC_MAX_PAIRS = 4096  # GB_COLLIDE_NOALLOC_MAX_PAIRS
SOLVER_PLAIN, SOLVER_COLOURED = 0, 1
WARM_REFERENCE, WARM_LEARNED, WARM_LEARNED_ALL = 0, 1, 2
# gb_body_set properties (b2Body::SetType, SetActive, SetFixedRotation, SetBullet, SetSleepingAllowed,
# SetLinearDamping, SetAngularDamping, SetGravityScale)
(BODY_TYPE, BODY_ACTIVE, BODY_FIXED_ROTATION, BODY_BULLET, BODY_SLEEPING_ALLOWED, BODY_LINEAR_DAMPING,
 BODY_ANGULAR_DAMPING, BODY_GRAVITY_SCALE, BODY_MASS_DATA, BODY_RESET_MASS_DATA) = range(10)
# gb_fixture_set properties (b2Fixture::SetFriction, SetRestitution, SetDensity, SetSensor, SetFilterData)
FIXTURE_FRICTION, FIXTURE_RESTITUTION, FIXTURE_DENSITY, FIXTURE_SENSOR, FIXTURE_FILTER = range(5)
STATUS_NAMES = {0: "GB_OK", 1: "GB_ERR_CAPACITY", 2: "GB_ERR_TIMEOUT", 3: "GB_ERR_INVALID", 4: "GB_ERR_CUDA"}

# Every symbol include/box2d_gb300.h declares.
EXPORTS = [
    "gb_world_create", "gb_world_destroy", "gb_create_bodies", "gb_create_fixtures", "gb_create_chain",
    "gb_create_revolute_joints",
    "gb_build_world", "gb_world_upload", "gb_world_step", "gb_world_sync", "gb_world_set_stream",
    "gb_world_counts", "gb_get_bodies", "gb_get_contacts", "gb_get_proxies", "gb_world_stats", "gb_sincos",
    "gb_collide", "gb_version", "gb_world_totals", "gb_set_forces", "gb_get_transforms", "gb_set_forces_async",
    "gb_get_transforms_async", "gb_world_profile",
    "gb_collide_noalloc", "gb_world_set_solver", "gb_world_solver_stats", "gb_world_autotune",
    "gb_world_launch_plan", "gb_world_set_launch_plan", "gb_world_graph_step",
    "gb_mlp_create", "gb_mlp_destroy", "gb_mlp_param_count", "gb_mlp_set_params", "gb_mlp_get_params",
    "gb_mlp_forward", "gb_mlp_gradients", "gb_mlp_train", "gb_world_set_warm_start", "gb_world_warm_stats",
    "gb_world_set_contact_log", "gb_world_read_contact_log", "gb_world_contact_stats", "gb_world_set_events",
    "gb_world_read_events", "gb_world_query_aabb", "gb_world_raycast", "gb_create_joints",
    "gb_world_stage_times", "gb_body_edits", "gb_world_set_limits", "gb_world_set_settings", "gb_world_clear_forces", "gb_destroy_body", "gb_body_set", "gb_get_body_info", "gb_fixture_set", "gb_world_shift_origin", "gb_joint_set", "gb_get_joint_reaction", "gb_fixture_query", "gb_polygon_shape", "gb_world_track_tree", "gb_world_tree_stats", "gb_world_checkpoint", "gb_world_restore", "gb_world_set_recovery", "gb_world_recoveries", "gb_destroy_joint",
    "gb_destroy_fixture", "gb_world_raycast_all", "gb_world_get_profile", "gb_world_step_begin",
    "gb_contact_edits", "gb_world_step_end", "gb_world_set_contact_filter", "gb_world_refilter",
    "gb_world_filter_stats",
]

# gb_should_collide_fn
SHOULD_COLLIDE_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int)

# gb_contact_edit records: world, contact (list position), flags (1 enabled, 2 friction, 4 restitution,
# 8 tangent speed), enabled (int32), friction, restitution, tangent speed, reserved (float32)
CONTACT_EDIT_DTYPE = np.dtype([("world", np.int32), ("contact", np.int32), ("flags", np.int32),
                               ("enabled", np.int32), ("friction", np.float32), ("restitution", np.float32),
                               ("tangent_speed", np.float32), ("reserved", np.float32)])


# gb_body_edit ops (GB_EDIT_*) and the record layout: world, body, op, wake (int32), v[4] (float32)
EDIT_OPS = {"set_transform": 0, "set_linear_velocity": 1, "set_angular_velocity": 2, "set_awake": 3,
            "apply_force": 4, "apply_force_to_center": 5, "apply_torque": 6, "apply_linear_impulse": 7,
            "apply_angular_impulse": 8, "mouse_target": 9}
EDIT_DTYPE = np.dtype([("world", np.int32), ("body", np.int32), ("op", np.int32), ("wake", np.int32),
                       ("v", np.float32, 4)])


class GbError(RuntimeError):
    def __init__(self, status: int, where: str):
        super().__init__(f"{where} failed: {STATUS_NAMES.get(status, status)}")
        self.status = status


class WorldDef(C.Structure):
    _fields_ = [("gravity_x", C.c_float), ("gravity_y", C.c_float), ("allow_sleep", C.c_int),
                ("warm_starting", C.c_int), ("continuous_physics", C.c_int), ("sub_stepping", C.c_int)]


_f32 = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_i32 = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


class _NullableF32:
    """ctypes argtype: a C-contiguous float32 array, or None for NULL."""

    @classmethod
    def from_param(cls, obj):
        if obj is None:
            return None
        return _f32.from_param(obj)


_f32n = _NullableF32
_LIB = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load the extension (building it first when it is absent or older than its sources)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if build_if_missing:
        path = _build.build()
    if not os.path.exists(path):
        raise RuntimeError(f"box2dpp_gb300 extension not built: {path}")
    lib = C.CDLL(path)
    vp, i, f = C.c_void_p, C.c_int, C.c_float
    sig = {
        "gb_world_create": [i, C.POINTER(WorldDef), C.POINTER(vp)],
        "gb_world_destroy": [vp],
        "gb_create_bodies": [vp, i, i, _i32, _f32, _i32, _i32],
        "gb_create_fixtures": [vp, i, i, _i32, _i32, _f32, _i32, _f32, _i32, _i32],
        "gb_create_chain": [vp, i, i, _f32, i, i, vp, i, _f32, _i32, vp],
        "gb_create_revolute_joints": [vp, i, i, _i32, _i32, _f32, _i32, _i32],
        "gb_build_world": [vp, i, i, _i32, _f32, _i32, i, _i32, _i32, _f32, _i32, _f32, _i32, i, _i32, _i32, _i32, _f32,
                           _i32],
        "gb_create_joints": [vp, i, i, _i32, _i32, _i32, _f32, _i32, _i32],
        "gb_world_upload": [vp],
        "gb_world_step": [vp, f, i, i],
        "gb_world_sync": [vp],
        "gb_world_set_stream": [vp, vp],
        "gb_world_counts": [vp, i, C.POINTER(i), C.POINTER(i), C.POINTER(i), C.POINTER(i)],
        "gb_get_bodies": [vp, i, _f32],
        "gb_get_contacts": [vp, i, _i32, _f32, i, C.POINTER(i)],
        "gb_get_proxies": [vp, i, _i32, _f32],
        "gb_world_stats": [vp, i, C.POINTER(i), C.POINTER(i)],
        "gb_sincos": [_f32, _f32, _f32, i],
        "gb_collide": [i, _i32, _f32, _i32, _f32, _i32, _f32, _i32, _f32, _i32, _f32],
        "gb_collide_noalloc": [i, _i32, _f32, _i32, _f32, _i32, _f32, _i32, _f32, _i32, _f32],
        "gb_world_set_solver": [vp, i, f, i],
        "gb_world_set_limits": [vp, i, i],
        "gb_world_set_settings": [vp, i, C.POINTER(WorldDef), i],
        "gb_world_clear_forces": [vp, i],
        "gb_world_step_begin": [vp, f, i, i],
        "gb_contact_edits": [vp, i, C.c_void_p],
        "gb_world_step_end": [vp],
        "gb_world_set_contact_filter": [vp, SHOULD_COLLIDE_FN, vp],
        "gb_world_refilter": [vp, i, i],
        "gb_world_filter_stats": [vp, C.POINTER(C.c_longlong), C.POINTER(C.c_int)],
        "gb_world_raycast_all": [vp, i, _f32, _i32, _f32, i, C.POINTER(C.c_int)],
        "gb_world_get_profile": [vp, i, _f32],
        "gb_destroy_body": [vp, i, i, _i32, i, C.POINTER(C.c_int)],
        "gb_destroy_joint": [vp, i, i, _i32, i, C.POINTER(C.c_int)],
        "gb_body_set": [vp, i, i, i, _f32, _i32, i, C.POINTER(C.c_int)],
        "gb_get_body_info": [vp, i, i, _f32, C.POINTER(C.c_int)],
        "gb_fixture_set": [vp, i, i, i, _f32],
        "gb_world_shift_origin": [vp, i, f, f],
        "gb_joint_set": [vp, i, i, i, _f32],
        "gb_get_joint_reaction": [vp, i, i, f, _f32],
        "gb_fixture_query": [vp, i, i, i, _f32, _f32],
        "gb_polygon_shape": [i, _f32, i, _f32, C.POINTER(C.c_int)],
        "gb_world_track_tree": [vp, i],
        "gb_world_set_recovery": [vp, i],
        "gb_world_recoveries": [vp, C.POINTER(C.c_longlong)],
        "gb_world_checkpoint": [vp, i, C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t)],
        "gb_world_restore": [vp, i, C.c_char_p, C.c_size_t],
        "gb_world_tree_stats": [vp, i, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_float)],
        "gb_destroy_fixture": [vp, i, i, _i32, i, C.POINTER(C.c_int)],
        "gb_world_solver_stats": [vp, _i32, _i32, _f32],
        "gb_world_autotune": [vp, i],
        "gb_world_graph_step": [vp, f, i, i],
        "gb_mlp_create": [C.c_ulonglong, C.POINTER(vp)],
        "gb_world_set_warm_start": [vp, vp, i],
        "gb_world_warm_stats": [vp, _i32, _i32],
        "gb_world_set_contact_log": [vp, i],
        "gb_world_contact_stats": [vp, _f32],
        "gb_world_set_events": [vp, i],
        "gb_world_query_aabb": [vp, i, i, _f32, _i32, _i32, i, C.POINTER(i)],
        "gb_world_raycast": [vp, i, i, _f32, _i32, _f32],
        "gb_world_read_events": [vp, i, _i32, _f32, i, C.POINTER(i)],
        "gb_world_read_contact_log": [vp, _f32, _f32, i, C.POINTER(i)],
        "gb_mlp_destroy": [vp],
        "gb_mlp_set_params": [vp, _f32n, _f32n, _f32n],
        "gb_mlp_get_params": [vp, _f32, _f32, _f32],
        "gb_mlp_forward": [vp, _f32, i, _f32],
        "gb_mlp_gradients": [vp, _f32, _f32, i, _f32, C.POINTER(f)],
        "gb_mlp_train": [vp, _f32, _f32, i, i, i, f, C.c_ulonglong, _f32],
        "gb_world_launch_plan": [vp, _i32, i, C.POINTER(i), _f32, i, C.POINTER(i)],
        "gb_world_set_launch_plan": [vp, _i32, i],
        "gb_world_totals": [vp, C.POINTER(C.c_longlong)],
        "gb_set_forces": [vp, vp],
        "gb_get_transforms": [vp, vp],
        "gb_set_forces_async": [vp, vp],
        "gb_get_transforms_async": [vp, vp],
        "gb_world_profile": [vp, np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")],
        "gb_world_stage_times": [vp, f, i, i, _f32],
        "gb_body_edits": [vp, i, vp],
    }
    for name, args in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_int
    lib.gb_mlp_param_count.argtypes = []
    lib.gb_mlp_param_count.restype = C.c_int
    lib.gb_version.argtypes = []
    lib.gb_version.restype = C.c_char_p
    _LIB = lib
    return lib


def check(status: int, where: str) -> None:
    if status != GB_OK:
        raise GbError(status, where)
