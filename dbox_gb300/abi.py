"""numpy/ctypes mirror of include/dbox_gpu.h (plain-C records of the b2World boundary).

Each dtype below has exactly the byte layout of the C struct with the same name,
so arrays of them can be passed to the C ABI as pointers.
"""
import ctypes

import numpy as np

BODY_DEF = np.dtype([
    ("type", "<i4"), ("position", "<f4", 2), ("angle", "<f4"),
    ("linear_velocity", "<f4", 2), ("angular_velocity", "<f4"),
    ("linear_damping", "<f4"), ("angular_damping", "<f4"),
    ("allow_sleep", "<i4"), ("awake", "<i4"), ("fixed_rotation", "<i4"),
    ("bullet", "<i4"), ("active", "<i4"), ("gravity_scale", "<f4"),
])
assert BODY_DEF.itemsize == 60

SHAPE_DEF = np.dtype([
    ("kind", "<i4"), ("count", "<i4"), ("vertices", "<f4", (8, 2)),
    ("center", "<f4", 2), ("radius", "<f4"), ("hx", "<f4"), ("hy", "<f4"), ("angle", "<f4"),
])
assert SHAPE_DEF.itemsize == 96

FIXTURE_DEF = np.dtype([
    ("friction", "<f4"), ("restitution", "<f4"), ("density", "<f4"), ("is_sensor", "<i4"),
    ("category_bits", "<u2"), ("mask_bits", "<u2"), ("group_index", "<i2"), ("pad_", "<i2"),
])
assert FIXTURE_DEF.itemsize == 24

REVOLUTE_DEF = np.dtype([
    ("body_a", "<i4"), ("body_b", "<i4"), ("collide_connected", "<i4"),
    ("local_anchor_a", "<f4", 2), ("local_anchor_b", "<f4", 2), ("reference_angle", "<f4"),
    ("enable_limit", "<i4"), ("lower_angle", "<f4"), ("upper_angle", "<f4"),
    ("enable_motor", "<i4"), ("motor_speed", "<f4"), ("max_motor_torque", "<f4"),
])
assert REVOLUTE_DEF.itemsize == 56
DISTANCE_DEF = np.dtype([
    ("body_a", "<i4"), ("body_b", "<i4"), ("collide_connected", "<i4"),
    ("local_anchor_a", "<f4", 2), ("local_anchor_b", "<f4", 2),
    ("length", "<f4"), ("frequency_hz", "<f4"), ("damping_ratio", "<f4"),
])
assert DISTANCE_DEF.itemsize == 40
ROPE_DEF = np.dtype([
    ("body_a", "<i4"), ("body_b", "<i4"), ("collide_connected", "<i4"),
    ("local_anchor_a", "<f4", 2), ("local_anchor_b", "<f4", 2), ("max_length", "<f4"),
])
assert ROPE_DEF.itemsize == 32
WELD_DEF = np.dtype([
    ("body_a", "<i4"), ("body_b", "<i4"), ("collide_connected", "<i4"),
    ("local_anchor_a", "<f4", 2), ("local_anchor_b", "<f4", 2),
    ("reference_angle", "<f4"), ("frequency_hz", "<f4"), ("damping_ratio", "<f4"),
])
assert WELD_DEF.itemsize == 40
FRICTION_DEF = np.dtype([
    ("body_a", "<i4"), ("body_b", "<i4"), ("collide_connected", "<i4"),
    ("local_anchor_a", "<f4", 2), ("local_anchor_b", "<f4", 2), ("max_force", "<f4"), ("max_torque", "<f4"),
])
assert FRICTION_DEF.itemsize == 36
MOTOR_DEF = np.dtype([
    ("body_a", "<i4"), ("body_b", "<i4"), ("collide_connected", "<i4"),
    ("linear_offset", "<f4", 2), ("angular_offset", "<f4"), ("max_force", "<f4"), ("max_torque", "<f4"),
    ("correction_factor", "<f4"),
])
assert MOTOR_DEF.itemsize == 36
WHEEL_DEF = np.dtype([
    ("body_a", "<i4"), ("body_b", "<i4"), ("collide_connected", "<i4"),
    ("local_anchor_a", "<f4", 2), ("local_anchor_b", "<f4", 2), ("local_axis_a", "<f4", 2),
    ("enable_motor", "<i4"), ("max_motor_torque", "<f4"), ("motor_speed", "<f4"),
    ("frequency_hz", "<f4"), ("damping_ratio", "<f4"),
])
assert WHEEL_DEF.itemsize == 56
PRISMATIC_DEF = np.dtype([
    ("body_a", "<i4"), ("body_b", "<i4"), ("collide_connected", "<i4"),
    ("local_anchor_a", "<f4", 2), ("local_anchor_b", "<f4", 2), ("local_axis_a", "<f4", 2),
    ("reference_angle", "<f4"), ("enable_limit", "<i4"), ("lower_translation", "<f4"), ("upper_translation", "<f4"),
    ("enable_motor", "<i4"), ("max_motor_force", "<f4"), ("motor_speed", "<f4"),
])
assert PRISMATIC_DEF.itemsize == 64
PULLEY_DEF = np.dtype([
    ("body_a", "<i4"), ("body_b", "<i4"), ("collide_connected", "<i4"),
    ("ground_anchor_a", "<f4", 2), ("ground_anchor_b", "<f4", 2),
    ("local_anchor_a", "<f4", 2), ("local_anchor_b", "<f4", 2),
    ("length_a", "<f4"), ("length_b", "<f4"), ("ratio", "<f4"),
])
assert PULLEY_DEF.itemsize == 56
MOUSE_DEF = np.dtype([
    ("body_a", "<i4"), ("body_b", "<i4"), ("collide_connected", "<i4"),
    ("target", "<f4", 2), ("max_force", "<f4"), ("frequency_hz", "<f4"), ("damping_ratio", "<f4"),
])
assert MOUSE_DEF.itemsize == 32

GEAR_DEF = np.dtype([
    ("body_a", "<i4"), ("body_b", "<i4"), ("collide_connected", "<i4"),
    ("joint1", "<i4"), ("joint2", "<i4"), ("ratio", "<f4"),
])
assert GEAR_DEF.itemsize == 24

WORLD_HEADER = np.dtype([
    ("body_count", "<i4"), ("fixture_count", "<i4"), ("contact_count", "<i4"), ("joint_count", "<i4"),
    ("world_flags", "<u4"), ("step_complete", "<i4"), ("inv_dt0", "<f4"), ("reserved", "<i4"),
])
assert WORLD_HEADER.itemsize == 32

BODY_STATE = np.dtype([
    ("flags", "<u4"), ("type", "<i4"), ("xf", "<f4", 4), ("sweep", "<f4", 9), ("vel", "<f4", 3),
    ("force", "<f4", 3), ("sleep_time", "<f4"), ("mass", "<f4", 4),
])
assert BODY_STATE.itemsize == 104

RAY_HIT = np.dtype([("fixture", "<i4"), ("fraction", "<f4"), ("point", "<f4", 2), ("normal", "<f4", 2)])
RAY_CLOSEST = 0
RAY_ALL = 1
PROXY_STATE = np.dtype([("fat_aabb", "<f4", 4), ("moved", "<i4"), ("proxy_id", "<i4")])
assert PROXY_STATE.itemsize == 24

MANIFOLD_POINT = np.dtype([
    ("local_point", "<f4", 2), ("normal_impulse", "<f4"), ("tangent_impulse", "<f4"), ("id", "<u4"),
])
CONTACT_STATE = np.dtype([
    ("fixture_a", "<i4"), ("fixture_b", "<i4"), ("flags", "<u4"), ("toi_count", "<i4"),
    ("toi", "<f4"), ("friction", "<f4"), ("restitution", "<f4"), ("tangent_speed", "<f4"),
    ("point_count", "<i4"), ("type", "<i4"), ("local_normal", "<f4", 2), ("local_point", "<f4", 2),
    ("points", MANIFOLD_POINT, 2),
])
assert CONTACT_STATE.itemsize == 96

JOINT_STATE = np.dtype([("impulse", "<f4", 3), ("motor_impulse", "<f4"), ("limit_state", "<i4")])
assert JOINT_STATE.itemsize == 20

CONTACT_EVENT = np.dtype([
    ("kind", "<i4"), ("world", "<i4"), ("fixture_a", "<i4"), ("fixture_b", "<i4"),
    ("point_count", "<i4"), ("normal_impulses", "<f4", 2), ("tangent_impulses", "<f4", 2),
])
assert CONTACT_EVENT.itemsize == 36
EVENT_BEGIN, EVENT_END, EVENT_PRESOLVE, EVENT_POSTSOLVE = 1, 2, 3, 4   # DBOX_EVENT_*

PRESOLVE_CONTACT = np.dtype([
    ("world", "<i4"), ("enabled", "<i4"), ("friction", "<f4"), ("restitution", "<f4"), ("tangent_speed", "<f4"),
    ("contact", CONTACT_STATE),
])
assert PRESOLVE_CONTACT.itemsize == 116

PROFILE = np.dtype([(n, "<f4") for n in (
    "step", "collide", "solve", "solve_init", "solve_velocity", "solve_position", "broadphase", "solve_toi")])

STATIC, KINEMATIC, DYNAMIC = 0, 1, 2
SHAPE_CIRCLE, SHAPE_POLYGON, SHAPE_BOX, SHAPE_ORIENTED_BOX, SHAPE_EDGE = 0, 1, 2, 3, 4

# b2Body / b2Contact flag bits (dynamics/b2body.d:1118-1127, contacts/b2contact.d:242-261)
BODY_ISLAND, BODY_AWAKE, BODY_AUTOSLEEP, BODY_BULLET, BODY_FIXED_ROTATION, BODY_ACTIVE = 1, 2, 4, 8, 0x10, 0x20
CONTACT_ISLAND, CONTACT_TOUCHING, CONTACT_ENABLED, CONTACT_FILTER, CONTACT_BULLET_HIT, CONTACT_TOI = (
    1, 2, 4, 8, 0x10, 0x20)

ERRORS = {0: "ok", -1: "invalid", -2: "locked", -3: "capacity", -4: "timeout", -5: "nan", -6: "cuda",
          -7: "unsupported"}
ERR_INVALID, ERR_LOCKED, ERR_CAPACITY, ERR_TIMEOUT, ERR_NAN, ERR_CUDA, ERR_UNSUPPORTED = -1, -2, -3, -4, -5, -6, -7


def body_defs(n):
    """n b2BodyDef records with the reference defaults (dynamics/b2body.d:51-104)."""
    a = np.zeros(n, BODY_DEF)
    a["allow_sleep"] = 1
    a["awake"] = 1
    a["active"] = 1
    a["gravity_scale"] = 1.0
    return a


def fixture_defs(n):
    """n b2FixtureDef records with the reference defaults (dynamics/b2fixture.d:49-73)."""
    a = np.zeros(n, FIXTURE_DEF)
    a["friction"] = np.float32(0.2)
    a["category_bits"] = 1
    a["mask_bits"] = 0xFFFF
    return a


def ptr(a):
    """ctypes void pointer to a contiguous numpy array (or None)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return ctypes.c_void_p(a.ctypes.data)


class Vec2(ctypes.Structure):
    _fields_ = [("x", ctypes.c_float), ("y", ctypes.c_float)]
