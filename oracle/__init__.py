"""TEST INFRASTRUCTURE ONLY: Python loader for the CPU oracle (b2_oracle.cpp).

The oracle restates dbox's b2World.Step on the CPU (see b2_oracle.h for the
parity status).  Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline legs use this module; the product library never does.
"""
import ctypes
import os
import subprocess

import numpy as np

from dbox_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SRC = os.path.join(HERE, "b2_oracle.cpp")
HDRS = [os.path.join(HERE, "b2_oracle.h"), os.path.join(HERE, "..", "include", "dbox_gpu.h"),
        os.path.join(HERE, "..", "dbox_gb300", "csrc", "dbox_trig.h")]

_lib = None


def build(force=False):
    """Compile liboracle.so: -O2 -ffp-contract=off keeps every float op singly rounded."""
    os.makedirs(BUILD, exist_ok=True)
    newest = max(os.path.getmtime(p) for p in [SRC] + HDRS)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    cmd = ["g++", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-std=c++17", SRC, "-o", LIB + ".tmp"]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        vp, i32, f32 = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
        L.orc_world_create.restype = vp
        L.orc_world_create.argtypes = [f32, f32]
        L.orc_world_destroy.argtypes = [vp]
        L.orc_scene_create.argtypes = [vp, i32, vp, i32, vp, vp, vp, i32, vp]
        L.orc_joint_create_distance.argtypes = [vp, vp]
        L.orc_fixture_create_chain.argtypes = [vp, i32, vp, i32, i32, vp, vp, vp]
        L.orc_query_aabb.argtypes = [vp, f32, f32, f32, f32, vp, i32]
        L.orc_raycast.argtypes = [vp, f32, f32, f32, f32, i32, vp, i32]
        L.orc_world_dump.argtypes = [vp, ctypes.c_char_p, i32]
        L.orc_body_create.argtypes = [vp, vp]
        for fn in ("orc_body_destroy", "orc_fixture_destroy", "orc_joint_destroy"):
            getattr(L, fn).argtypes = [vp, i32]
        L.orc_fixture_create.argtypes = [vp, i32, vp, vp]
        L.orc_joint_create_revolute.argtypes = [vp, vp]
        L.orc_raycast_many.argtypes = [vp, i32, vp, vp, i32, vp, vp, i32]
        L.orc_query_aabb_many.argtypes = [vp, i32, vp, vp, vp, i32]
        L.orc_joint_create_rope.argtypes = [vp, vp]
        L.orc_joint_create_weld.argtypes = [vp, vp]
        L.orc_joint_create_friction.argtypes = [vp, vp]
        L.orc_joint_create_motor.argtypes = [vp, vp]
        L.orc_joint_create_wheel.argtypes = [vp, vp]
        L.orc_joint_create_prismatic.argtypes = [vp, vp]
        L.orc_joint_create_pulley.argtypes = [vp, vp]
        L.orc_joint_create_mouse.argtypes = [vp, vp]
        L.orc_joint_create_gear.argtypes = [vp, vp]
        L.orc_joint_set_mouse_target.argtypes = [vp, i32, f32, f32]
        L.orc_world_set_flags.argtypes = [vp, i32, i32, i32, i32, i32]
        L.orc_world_step.argtypes = [vp, f32, i32, i32]
        L.orc_world_step_n.argtypes = [vp, f32, i32, i32, i32]
        L.orc_world_export_state.argtypes = [vp, vp, vp, vp, vp, vp]
        L.orc_world_record_events.argtypes = [vp, i32]
        L.orc_world_event_count.argtypes = [vp]
        L.orc_world_get_events.argtypes = [vp, vp, i32]
        L.orc_world_clear_events.argtypes = [vp]
        L.orc_world_set_presolve.argtypes = [vp, vp, vp]
        L.orc_fixture_set_filter.argtypes = [vp, i32, i32, i32, i32]
        L.orc_fixture_set_filter_class.argtypes = [vp, i32, i32]
        L.orc_world_set_contact_filter.argtypes = [vp, vp, i32]
        L.orc_world_last_toi_events.argtypes = [vp]
        L.orc_world_last_islands.argtypes = [vp]
        L.orc_set_trig_mode.argtypes = [i32]
        L.orc_sincos.argtypes = [f32, ctypes.POINTER(f32), ctypes.POINTER(f32)]
        L.orc_sincos_array.argtypes = [i32, vp, vp, vp]
        L.orc_polygon_set.argtypes = [vp, i32, vp, vp, vp]
        L.orc_collide.argtypes = [vp, vp, vp, vp, vp]
        _lib = L
    return _lib


def set_trig_mode(mode):
    """0: host libm sinf/cosf (the reference's arithmetic); 1: the portable dbox_sincosf."""
    lib().orc_set_trig_mode(int(mode))


def sincos(a):
    s, c = ctypes.c_float(), ctypes.c_float()
    lib().orc_sincos(ctypes.c_float(a), ctypes.byref(s), ctypes.byref(c))
    return s.value, c.value


def sincos_array(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    s = np.zeros_like(a)
    c = np.zeros_like(a)
    lib().orc_sincos_array(len(a), abi.ptr(a), abi.ptr(s), abi.ptr(c))
    return s, c


def collide(shape_a, xf_a, shape_b, xf_b):
    """Narrowphase manifold of two shapes (records of abi.SHAPE_DEF) at transforms (p.x, p.y, sin, cos)."""
    sa = np.ascontiguousarray(np.array([shape_a], abi.SHAPE_DEF))
    sb = np.ascontiguousarray(np.array([shape_b], abi.SHAPE_DEF))
    xa = np.ascontiguousarray(xf_a, dtype=np.float32)
    xb = np.ascontiguousarray(xf_b, dtype=np.float32)
    out = np.zeros(1, abi.CONTACT_STATE)
    n = lib().orc_collide(abi.ptr(sa), abi.ptr(xa), abi.ptr(sb), abi.ptr(xb), abi.ptr(out))
    if n < 0:
        raise ValueError("unsupported shape pair")
    return out[0]


class OracleWorld:
    """One b2World on the CPU, built from a scene dict (dbox_gb300.scenes)."""

    def __init__(self, scene, flags=None):
        L = lib()
        g = scene.get("gravity", (0.0, -10.0))
        self.h = L.orc_world_create(float(g[0]), float(g[1]))
        b = np.ascontiguousarray(scene["bodies"])
        fb = np.ascontiguousarray(scene["fixture_body"], dtype=np.int32)
        sh = np.ascontiguousarray(scene["shapes"])
        fx = np.ascontiguousarray(scene["fixtures"])
        j = np.ascontiguousarray(scene["joints"])
        rc = L.orc_scene_create(self.h, len(b), abi.ptr(b), len(fb), abi.ptr(fb), abi.ptr(sh), abi.ptr(fx),
                                len(j), abi.ptr(j) if len(j) else None)
        if rc != 0:
            raise ValueError("oracle scene creation failed")
        for c in scene.get("chains", ()):
            fd = abi.fixture_defs(1)[0]
            fd["friction"] = c.get("friction", 0.2)
            self.create_chain(c["body"], c["vertices"], c["loop"], c.get("prev"), c.get("next"), fd)
        # joint kinds after the revolute joints, in this order (the same as the library's)
        for key, dtype, fn in (("distance_joints", abi.DISTANCE_DEF, L.orc_joint_create_distance),
                               ("rope_joints", abi.ROPE_DEF, L.orc_joint_create_rope),
                               ("weld_joints", abi.WELD_DEF, L.orc_joint_create_weld),
                               ("friction_joints", abi.FRICTION_DEF, L.orc_joint_create_friction),
                               ("motor_joints", abi.MOTOR_DEF, L.orc_joint_create_motor),
                               ("wheel_joints", abi.WHEEL_DEF, L.orc_joint_create_wheel),
                               ("prismatic_joints", abi.PRISMATIC_DEF, L.orc_joint_create_prismatic),
                               ("pulley_joints", abi.PULLEY_DEF, L.orc_joint_create_pulley),
                               ("mouse_joints", abi.MOUSE_DEF, L.orc_joint_create_mouse),
                               ("gear_joints", abi.GEAR_DEF, L.orc_joint_create_gear)):
            for d in scene.get(key, ()):
                dd = np.ascontiguousarray(np.array([d], dtype))
                if fn(self.h, abi.ptr(dd)) < 0:
                    raise ValueError("oracle %s creation failed" % key)
        if flags is not None:
            self.set_flags(**flags)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_world_destroy(self.h)
            self.h = None

    def set_flags(self, warm=1, continuous=1, substep=0, sleep=1, autoclear=1):
        lib().orc_world_set_flags(self.h, warm, continuous, substep, sleep, autoclear)

    def step(self, dt=1.0 / 60.0, vel_iters=8, pos_iters=3, steps=1):
        if steps == 1:
            lib().orc_world_step(self.h, ctypes.c_float(dt), vel_iters, pos_iters)
        else:
            lib().orc_world_step_n(self.h, ctypes.c_float(dt), vel_iters, pos_iters, steps)

    def record_events(self, on=True):
        lib().orc_world_record_events(self.h, 1 if on else 0)

    def events(self, clear=True):
        n = lib().orc_world_event_count(self.h)
        out = np.zeros(n, abi.CONTACT_EVENT)
        if n:
            lib().orc_world_get_events(self.h, abi.ptr(out), n)
        if clear:
            lib().orc_world_clear_events(self.h)
        return out

    def set_filter(self, fixture, category_bits=0x0001, mask_bits=0xFFFF, group_index=0):
        """b2Fixture.SetFilterData (and Refilter)."""
        if lib().orc_fixture_set_filter(self.h, fixture, category_bits, mask_bits, group_index) < 0:
            raise ValueError("oracle: no fixture %d" % fixture)

    def set_filter_class(self, fixture, cls):
        if lib().orc_fixture_set_filter_class(self.h, fixture, cls) < 0:
            raise ValueError("oracle: no fixture %d" % fixture)

    def set_contact_filter(self, table=None, with_default=True):
        """b2World.SetContactFilter with a user filter over a class table (None: the default)."""
        t = None if table is None else np.ascontiguousarray(table, np.uint64)
        lib().orc_world_set_contact_filter(self.h, abi.ptr(t) if t is not None else None, 1 if with_default else 0)

    _PRESOLVE_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p)

    def set_presolve(self, fn):
        """A user b2ContactListener.PreSolve: fn(records) with one abi.PRESOLVE_CONTACT record per
        call, made inside Collide and SolveTOI as the reference makes it; in-place edits of
        "enabled", "friction", "restitution" and "tangent_speed" are applied to the contact."""
        if fn is None:
            self._presolve = None
            lib().orc_world_set_presolve(self.h, None, None)
            return

        def tramp(ptr, count, user):
            buf = (ctypes.c_char * (count * abi.PRESOLVE_CONTACT.itemsize)).from_address(ptr)
            fn(np.frombuffer(buf, abi.PRESOLVE_CONTACT))

        self._presolve = OracleWorld._PRESOLVE_FN(tramp)
        lib().orc_world_set_presolve(self.h, ctypes.cast(self._presolve, ctypes.c_void_p), None)

    def last_toi_events(self):
        return lib().orc_world_last_toi_events(self.h)

    def last_islands(self):
        return lib().orc_world_last_islands(self.h)

    def create_chain(self, body, vertices, loop=False, prev=None, next=None, fixture=None):
        """b2Body.CreateFixture with a b2ChainShape, created as its child edges; returns the
        first child's fixture index."""
        v = np.ascontiguousarray(vertices, np.float32)
        pv = np.ascontiguousarray(prev, np.float32) if prev is not None else None
        nv = np.ascontiguousarray(next, np.float32) if next is not None else None
        fd = fixture if fixture is not None else abi.fixture_defs(1)[0]
        fd = np.ascontiguousarray(np.array([fd], abi.FIXTURE_DEF))
        r = lib().orc_fixture_create_chain(self.h, body, abi.ptr(v), len(v), 1 if loop else 0,
                                           abi.ptr(pv) if pv is not None else None,
                                           abi.ptr(nv) if nv is not None else None, abi.ptr(fd))
        if r < 0:
            raise ValueError("oracle chain creation failed")
        return r

    def query_aabb(self, box, capacity=4096):
        """b2World.QueryAABB through the oracle's dynamic tree: the fixtures whose fat AABB
        overlaps box = (lower x, y, upper x, y), sorted by fixture index."""
        out = np.zeros(capacity, np.int32)
        n = lib().orc_query_aabb(self.h, *[float(v) for v in box], abi.ptr(out), capacity)
        return out[:min(n, capacity)].copy()

    def raycast(self, p1, p2, mode="closest", capacity=4096):
        """b2World.RayCast through the oracle's dynamic tree.  mode "closest": the smallest
        fraction over all hits (lower fixture index on a tie); "all": every hit in fixture
        order; "clip": the reference's clipping closest-hit callback as it runs.  Returns an
        array of abi.RAY_HIT (None for p1 == p2)."""
        m = {"closest": 0, "all": 1, "clip": 2}[mode]
        out = np.zeros(capacity, abi.RAY_HIT)
        n = lib().orc_raycast(self.h, float(p1[0]), float(p1[1]), float(p2[0]), float(p2[1]), m, abi.ptr(out), capacity)
        if n < 0:
            return None
        return out[:min(n, capacity)].copy()

    _JOINTS = {"revolute": "REVOLUTE_DEF", "distance": "DISTANCE_DEF", "rope": "ROPE_DEF", "weld": "WELD_DEF",
               "friction": "FRICTION_DEF", "motor": "MOTOR_DEF", "wheel": "WHEEL_DEF", "prismatic": "PRISMATIC_DEF",
               "pulley": "PULLEY_DEF", "mouse": "MOUSE_DEF", "gear": "GEAR_DEF"}

    def create_body(self, body_def):
        dd = np.ascontiguousarray(np.array([body_def], abi.BODY_DEF))
        return lib().orc_body_create(self.h, abi.ptr(dd))

    def create_fixture(self, body, shape_def, fixture_def):
        sd = np.ascontiguousarray(np.array([shape_def], abi.SHAPE_DEF))
        fd = np.ascontiguousarray(np.array([fixture_def], abi.FIXTURE_DEF))
        r = lib().orc_fixture_create(self.h, body, abi.ptr(sd), abi.ptr(fd))
        if r < 0:
            raise ValueError("oracle fixture creation failed")
        return r

    def destroy_body(self, body):
        if lib().orc_body_destroy(self.h, body) < 0:
            raise ValueError("oracle: no body %d" % body)

    def destroy_fixture(self, fixture):
        if lib().orc_fixture_destroy(self.h, fixture) < 0:
            raise ValueError("oracle: no fixture %d" % fixture)

    def destroy_joint(self, joint):
        if lib().orc_joint_destroy(self.h, joint) < 0:
            raise ValueError("oracle: no joint %d" % joint)

    def create_joint(self, kind, d):
        dd = np.ascontiguousarray(np.array([d], getattr(abi, self._JOINTS[kind])))
        r = getattr(lib(), "orc_joint_create_" + kind)(self.h, abi.ptr(dd))
        if r < 0:
            raise ValueError("oracle %s joint creation failed" % kind)
        return r

    def dump(self):
        """b2World.Dump's text."""
        n = lib().orc_world_dump(self.h, None, 0)
        buf = ctypes.create_string_buffer(n + 1)
        lib().orc_world_dump(self.h, buf, n + 1)
        return buf.value.decode()

    def raycast_many(self, p1, p2, mode="closest", capacity=1):
        """orc_raycast over arrays of rays in one C loop: (counts, hits (n, capacity))."""
        a = np.ascontiguousarray(p1, np.float32).reshape(-1, 2)
        b = np.ascontiguousarray(p2, np.float32).reshape(-1, 2)
        counts = np.zeros(len(a), np.int32)
        hits = np.zeros((len(a), capacity), abi.RAY_HIT)
        lib().orc_raycast_many(self.h, len(a), abi.ptr(a), abi.ptr(b), {"closest": 0, "all": 1}[mode],
                               abi.ptr(counts), abi.ptr(hits), capacity)
        return counts, hits

    def query_aabb_many(self, boxes, capacity=64):
        """orc_query_aabb over an array of boxes in one C loop: (counts, fixtures (n, capacity))."""
        bx = np.ascontiguousarray(boxes, np.float32).reshape(-1, 4)
        counts = np.zeros(len(bx), np.int32)
        out = np.zeros((len(bx), capacity), np.int32)
        lib().orc_query_aabb_many(self.h, len(bx), abi.ptr(bx), abi.ptr(counts), abi.ptr(out), capacity)
        return counts, out

    def set_mouse_target(self, joint, target):
        """b2MouseJoint.SetTarget (b2mousejoint.d:83-91)."""
        if lib().orc_joint_set_mouse_target(self.h, joint, float(target[0]), float(target[1])) != 0:
            raise ValueError("not a mouse joint")

    def export_state(self):
        L = lib()
        hdr = np.zeros(1, abi.WORLD_HEADER)
        L.orc_world_export_state(self.h, abi.ptr(hdr), None, None, None, None)
        h = hdr[0]
        bodies = np.zeros(int(h["body_count"]), abi.BODY_STATE)
        proxies = np.zeros(int(h["fixture_count"]), abi.PROXY_STATE)
        contacts = np.zeros(int(h["contact_count"]), abi.CONTACT_STATE)
        joints = np.zeros(int(h["joint_count"]), abi.JOINT_STATE)
        L.orc_world_export_state(self.h, abi.ptr(hdr), abi.ptr(bodies), abi.ptr(proxies), abi.ptr(contacts),
                                 abi.ptr(joints))
        return {"header": hdr, "bodies": bodies, "proxies": proxies, "contacts": contacts, "joints": joints}


def polygon_set(points):
    """b2PolygonShape.Set on the given points: (vertices, normals, centroid) or None if degenerate."""
    pts = np.ascontiguousarray(points, dtype=np.float32).reshape(-1, 2)
    v = np.zeros((8, 2), np.float32)
    nrm = np.zeros((8, 2), np.float32)
    c = np.zeros(2, np.float32)
    n = lib().orc_polygon_set(abi.ptr(pts), len(pts), abi.ptr(v), abi.ptr(nrm), abi.ptr(c))
    if n == 0:
        return None
    return v[:n].copy(), nrm[:n].copy(), c
