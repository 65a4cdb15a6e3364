"""dbox_gb300: GPU b2World.Step behind the reference's world/body/fixture API.

The compute path is libdbox_gpu.so (hand-written sm_103a kernels behind the C
ABI of include/dbox_gpu.h); this module is a thin ctypes binding shaped like
dbox's b2World (dynamics/b2world.d): create bodies/fixtures/joints, Step(dt,
velocityIterations, positionIterations), read bodies and contacts back.

There is no CPU fallback: if the library cannot be loaded, or no GPU is
visible, World raises.
"""
import ctypes
import os

import numpy as np

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libdbox_gpu.so")

_lib = None


class DboxError(RuntimeError):
    """A failed C-ABI call; `code` is its DBOX_ERR_* status."""

    def __init__(self, msg, code=None):
        super().__init__(msg)
        self.code = code


def build(force=False):
    """Compile libdbox_gpu.so for sm_103a (see buildlib.py)."""
    from . import buildlib
    return buildlib.build(force=force)


def lib():
    """Load libdbox_gpu.so; raise if it is missing (no silent fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise DboxError("libdbox_gpu.so not built: run dbox_gb300.build() (nvcc, sm_103a)")
    L = ctypes.CDLL(LIB_PATH)
    vp, i32, f32 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_float
    L.dbox_world_create.argtypes = [abi.Vec2, i32, vp, ctypes.POINTER(vp)]
    L.dbox_world_destroy.argtypes = [vp]
    L.dbox_scene_create.argtypes = [vp, i32, i32, vp, i32, vp, vp, vp, i32, vp]
    L.dbox_body_create.argtypes = [vp, i32, vp, ctypes.POINTER(i32)]
    L.dbox_fixture_create.argtypes = [vp, i32, i32, vp, vp, ctypes.POINTER(i32)]
    L.dbox_fixture_create_chain.argtypes = [vp, i32, i32, vp, i32, i32, vp, vp, vp, ctypes.POINTER(i32)]
    L.dbox_joint_create_revolute.argtypes = [vp, i32, vp, ctypes.POINTER(i32)]
    L.dbox_joint_create_distance.argtypes = [vp, i32, vp, ctypes.POINTER(i32)]
    L.dbox_joint_create_rope.argtypes = [vp, i32, vp, ctypes.POINTER(i32)]
    L.dbox_joint_create_weld.argtypes = [vp, i32, vp, ctypes.POINTER(i32)]
    L.dbox_joint_create_friction.argtypes = [vp, i32, vp, ctypes.POINTER(i32)]
    L.dbox_joint_create_motor.argtypes = [vp, i32, vp, ctypes.POINTER(i32)]
    L.dbox_joint_create_wheel.argtypes = [vp, i32, vp, ctypes.POINTER(i32)]
    L.dbox_joint_create_prismatic.argtypes = [vp, i32, vp, ctypes.POINTER(i32)]
    L.dbox_joint_create_pulley.argtypes = [vp, i32, vp, ctypes.POINTER(i32)]
    L.dbox_joint_create_mouse.argtypes = [vp, i32, vp, ctypes.POINTER(i32)]
    L.dbox_joint_set_mouse_target.argtypes = [vp, i32, i32, abi.Vec2]
    L.dbox_joint_create_gear.argtypes = [vp, i32, vp, ctypes.POINTER(i32)]
    L.dbox_world_query_aabb.argtypes = [vp, i32, vp, vp, i32, vp, vp]
    L.dbox_world_get_stream.argtypes = [vp, ctypes.POINTER(vp)]
    L.dbox_world_get_counts.argtypes = [vp, i32, ctypes.POINTER(i32), ctypes.POINTER(i32), ctypes.POINTER(i32)]
    for fn in ("dbox_body_destroy", "dbox_fixture_destroy", "dbox_joint_destroy"):
        getattr(L, fn).argtypes = [vp, i32, i32]
    L.dbox_world_dump.argtypes = [vp, i32, ctypes.c_char_p, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64)]
    L.dbox_world_raycast.argtypes = [vp, i32, vp, vp, vp, i32, i32, vp, vp]
    L.dbox_world_query_aabb_device.argtypes = [vp, i32, vp, vp, i32, vp, vp]
    L.dbox_world_raycast_device.argtypes = [vp, i32, vp, vp, vp, i32, i32, vp, vp]
    L.dbox_world_set_flags.argtypes = [vp, i32, i32, i32, i32, i32]
    L.dbox_world_set_gravity.argtypes = [vp, abi.Vec2]
    L.dbox_world_step.argtypes = [vp, f32, i32, i32]
    L.dbox_world_step_n.argtypes = [vp, f32, i32, i32, i32]
    L.dbox_world_sync.argtypes = [vp]
    L.dbox_world_get_bodies.argtypes = [vp, vp, vp, vp, vp, vp]
    L.dbox_world_body_count.argtypes = [vp, i32, ctypes.POINTER(i32)]
    L.dbox_world_contact_count.argtypes = [vp, i32, ctypes.POINTER(i32)]
    L.dbox_world_export_state.argtypes = [vp, i32, vp, vp, vp, vp, vp]
    L.dbox_world_import_state.argtypes = [vp, i32, vp, vp, vp, vp, vp]
    L.dbox_world_get_profile.argtypes = [vp, vp]
    L.dbox_world_last_launches.argtypes = [vp, ctypes.POINTER(i32)]
    L.dbox_world_step_stats.argtypes = [vp, i32, ctypes.POINTER(i32), ctypes.POINTER(i32)]
    L.dbox_last_error.restype = ctypes.c_char_p
    L.dbox_collide_manifolds.argtypes = [i32, vp, vp, vp, vp, vp]
    L.dbox_collide_manifolds_noalloc.argtypes = [i32, vp, vp, vp, vp, vp]
    L.dbox_world_step_n_timed.argtypes = [vp, f32, i32, i32, i32, vp, vp]
    L.dbox_world_get_counters.argtypes = [vp, vp]
    L.dbox_world_set_phase_profile.argtypes = [vp, i32]
    L.dbox_world_get_phase_profile.argtypes = [vp, vp]
    L.dbox_world_apply_forces.argtypes = [vp, vp]
    L.dbox_world_get_transforms.argtypes = [vp, vp]
    L.dbox_body_def_default.argtypes = [vp]
    L.dbox_fixture_def_default.argtypes = [vp]
    u64 = ctypes.c_uint64
    L.dbox_mlp_create.argtypes = [ctypes.POINTER(vp)]
    L.dbox_mlp_destroy.argtypes = [vp]
    L.dbox_mlp_init.argtypes = [vp, u64]
    L.dbox_mlp_set_params.argtypes = [vp, vp, vp]
    L.dbox_mlp_get_params.argtypes = [vp, vp, vp]
    L.dbox_mlp_fit_normalization.argtypes = [vp, i32, vp, vp]
    L.dbox_mlp_gradient.argtypes = [vp, i32, vp, vp, vp, vp]
    L.dbox_mlp_train.argtypes = [vp, i32, vp, vp, i32, i32, f32, u64, vp]
    L.dbox_mlp_train_device.argtypes = [vp, i32, vp, i32, i32, f32, u64, vp]
    L.dbox_mlp_train_world.argtypes = [vp, vp, i32, i32, f32, u64, vp]
    L.dbox_mlp_forward.argtypes = [vp, i32, vp, vp]
    L.dbox_world_set_warmstart.argtypes = [vp, i32, vp, i32]
    L.dbox_world_set_start_source.argtypes = [vp, vp]
    L.dbox_world_copy_state.argtypes = [vp, vp]
    L.dbox_world_sample_count.argtypes = [vp, ctypes.POINTER(i32)]
    L.dbox_world_get_samples.argtypes = [vp, i32, i32, vp]
    L.dbox_world_clear_samples.argtypes = [vp]
    L.dbox_world_set_measure.argtypes = [vp, i32]
    L.dbox_world_set_wait_limit.argtypes = [vp, i32]
    L.dbox_world_set_island_solver.argtypes = [vp, i32]
    L.dbox_world_get_island_solver.argtypes = [vp, vp]
    L.dbox_world_set_fused_step.argtypes = [vp, i32]
    L.dbox_world_get_fused_step.argtypes = [vp, vp]
    L.dbox_world_set_listener.argtypes = [vp, vp, vp]
    L.dbox_world_set_presolve.argtypes = [vp, vp, vp]
    L.dbox_fixture_set_filter.argtypes = [vp, i32, i32, ctypes.c_uint16, ctypes.c_uint16, ctypes.c_int16]
    L.dbox_fixture_set_filter_class.argtypes = [vp, i32, i32, i32]
    L.dbox_world_set_contact_filter.argtypes = [vp, i32, vp, i32]
    L.dbox_world_set_mapping.argtypes = [vp, i32, i32]
    L.dbox_world_set_mapping_isolated.argtypes = [vp, i32, i32, i32]
    L.dbox_world_autotune.argtypes = [vp, f32, i32, i32, i32, vp]
    L.dbox_world_set_mapping_queue.argtypes = [vp, i32, i32, i32]
    L.dbox_world_set_world_costs.argtypes = [vp, vp]
    L.dbox_world_get_world_costs.argtypes = [vp, vp]
    L.dbox_world_get_quality.argtypes = [vp, vp]
    _lib = L
    return L


def _check(rc, what):
    if rc != 0:
        msg = lib().dbox_last_error().decode(errors="replace")
        raise DboxError("%s failed: %s (%s)" % (what, abi.ERRORS.get(rc, rc), msg), rc)


def collide_manifolds(shapes_a, xfs_a, shapes_b, xfs_b):
    """Manifolds of shape pairs on the GPU (dbox_collide_manifolds); returns abi.CONTACT_STATE records."""
    sa = np.ascontiguousarray(shapes_a, abi.SHAPE_DEF)
    sb = np.ascontiguousarray(shapes_b, abi.SHAPE_DEF)
    xa = np.ascontiguousarray(xfs_a, np.float32)
    xb = np.ascontiguousarray(xfs_b, np.float32)
    out = np.zeros(len(sa), abi.CONTACT_STATE)
    _check(lib().dbox_collide_manifolds(len(sa), abi.ptr(sa), abi.ptr(xa), abi.ptr(sb), abi.ptr(xb), abi.ptr(out)),
           "dbox_collide_manifolds")
    return out


def collide_manifolds_noalloc(shapes_a, xfs_a, shapes_b, xfs_b):
    """dbox_collide_manifolds_noalloc: same as collide_manifolds, using the library's static
    device array instead of allocating (at most 4096 pairs per call)."""
    sa = np.ascontiguousarray(shapes_a, abi.SHAPE_DEF)
    sb = np.ascontiguousarray(shapes_b, abi.SHAPE_DEF)
    xa = np.ascontiguousarray(xfs_a, np.float32)
    xb = np.ascontiguousarray(xfs_b, np.float32)
    out = np.zeros(len(sa), abi.CONTACT_STATE)
    _check(lib().dbox_collide_manifolds_noalloc(len(sa), abi.ptr(sa), abi.ptr(xa), abi.ptr(sb), abi.ptr(xb),
                                                abi.ptr(out)), "dbox_collide_manifolds_noalloc")
    return out


MLP_PARAMS, MLP_NORM, MLP_SAMPLE, MLP_FEAT = 21768, 72, 36, 32
# a world with this many fixtures or more runs the large-world kernels (block pair search, Solve,
# Collide end and SolveTOI on a 1,024-thread block each)
LARGE_WORLD_FIXTURES = 4096


class Mlp:
    """The learned warm-start network (dbox_mlp_*): 32 -> 128 -> 128 -> 4, GELU, BF16 on the
    tensor cores with FP32 accumulation.  Parameters are one flat FP32 vector (layout in
    dbox_gpu.h); norm holds feature mean/std (32 + 32) and target mean/std (4 + 4)."""

    def __init__(self, seed=None):
        h = ctypes.c_void_p()
        _check(lib().dbox_mlp_create(ctypes.byref(h)), "dbox_mlp_create")
        self.h = h
        if seed is not None:
            _check(lib().dbox_mlp_init(self.h, ctypes.c_uint64(seed)), "dbox_mlp_init")

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            lib().dbox_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, params=None, norm=None):
        p = None if params is None else np.ascontiguousarray(params, np.float32)
        q = None if norm is None else np.ascontiguousarray(norm, np.float32)
        _check(lib().dbox_mlp_set_params(self.h, abi.ptr(p) if p is not None else None,
                                         abi.ptr(q) if q is not None else None), "dbox_mlp_set_params")

    def params(self):
        p = np.zeros(MLP_PARAMS, np.float32)
        q = np.zeros(MLP_NORM, np.float32)
        _check(lib().dbox_mlp_get_params(self.h, abi.ptr(p), abi.ptr(q)), "dbox_mlp_get_params")
        return p, q

    def fit_normalization(self, feats, targets):
        f = np.ascontiguousarray(feats, np.float32)
        t = np.ascontiguousarray(targets, np.float32)
        _check(lib().dbox_mlp_fit_normalization(self.h, len(f), abi.ptr(f), abi.ptr(t)), "fit_normalization")

    def gradient(self, feats, targets):
        f = np.ascontiguousarray(feats, np.float32)
        t = np.ascontiguousarray(targets, np.float32)
        g = np.zeros(MLP_PARAMS, np.float32)
        loss = np.zeros(1, np.float32)
        _check(lib().dbox_mlp_gradient(self.h, len(f), abi.ptr(f), abi.ptr(t), abi.ptr(g), abi.ptr(loss)),
               "dbox_mlp_gradient")
        return g, float(loss[0])

    def train(self, feats, targets, epochs=1, batch=65536, lr=1e-3, seed=0):
        f = np.ascontiguousarray(feats, np.float32)
        t = np.ascontiguousarray(targets, np.float32)
        losses = np.zeros(epochs, np.float32)
        _check(lib().dbox_mlp_train(self.h, len(f), abi.ptr(f), abi.ptr(t), epochs, batch, ctypes.c_float(lr),
                                    ctypes.c_uint64(seed), abi.ptr(losses)), "dbox_mlp_train")
        return losses

    def train_device(self, rows_ptr, n, epochs=1, batch=65536, lr=1e-3, seed=0):
        """Adam on n device rows of 36 floats (features, targets) at a 16-byte aligned device address."""
        losses = np.zeros(epochs, np.float32)
        _check(lib().dbox_mlp_train_device(self.h, n, ctypes.c_void_p(rows_ptr), epochs, batch, ctypes.c_float(lr),
                                           ctypes.c_uint64(seed), abi.ptr(losses)), "dbox_mlp_train_device")
        return losses

    def train_world(self, world, epochs=1, batch=65536, lr=1e-3, seed=0):
        losses = np.zeros(epochs, np.float32)
        _check(lib().dbox_mlp_train_world(self.h, world.h, epochs, batch, ctypes.c_float(lr), ctypes.c_uint64(seed),
                                          abi.ptr(losses)), "dbox_mlp_train_world")
        return losses

    def forward(self, feats):
        f = np.ascontiguousarray(feats, np.float32)
        out = np.zeros((len(f), 4), np.float32)
        _check(lib().dbox_mlp_forward(self.h, len(f), abi.ptr(f), abi.ptr(out)), "dbox_mlp_forward")
        return out


class World:
    """One or more b2Worlds on the GPU (b2World(gravity), b2world.d:865-895).

    `scenes` is one scene dict or a list of them (see dbox_gb300.scenes); each
    becomes an independent world of the batch.
    """

    def __init__(self, scenes, gravity=None, flags=None, contacts_per_body=0):
        L = lib()
        if isinstance(scenes, dict):
            scenes = [scenes]
        if gravity is None:
            # one gravity per handle (b2World's): the scenes' own, which must agree
            gs = {tuple(float(v) for v in sc.get("gravity", (0.0, -10.0))) for sc in scenes} or {(0.0, -10.0)}
            if len(gs) != 1:
                raise ValueError("scenes with different gravity need separate World handles")
            gravity = gs.pop()
        self.n_worlds = len(scenes)
        caps = np.zeros(2, np.int32)
        caps[0] = contacts_per_body
        h = ctypes.c_void_p()
        _check(L.dbox_world_create(abi.Vec2(*gravity), self.n_worlds, abi.ptr(caps), ctypes.byref(h)), "dbox_world_create")
        self.h = h
        for i, s in enumerate(scenes):
            b = np.ascontiguousarray(s["bodies"])
            fb = np.ascontiguousarray(s["fixture_body"], dtype=np.int32)
            sh = np.ascontiguousarray(s["shapes"])
            fx = np.ascontiguousarray(s["fixtures"])
            j = np.ascontiguousarray(s["joints"])
            _check(L.dbox_scene_create(self.h, i, len(b), abi.ptr(b), len(fb), abi.ptr(fb), abi.ptr(sh), abi.ptr(fx),
                                       len(j), abi.ptr(j) if len(j) else None), "dbox_scene_create")
            for c in s.get("chains", ()):
                fd = abi.fixture_defs(1)[0]
                fd["friction"] = c.get("friction", 0.2)
                self.create_chain(i, c["body"], c["vertices"], c["loop"], c.get("prev"), c.get("next"), fd)
            # joint kinds after the revolute joints, in this order (the oracle's order too)
            for d in s.get("distance_joints", ()):
                self.create_joint(i, "distance", d)
            for d in s.get("rope_joints", ()):
                self.create_joint(i, "rope", d)
            for kind in ("weld", "friction", "motor", "wheel", "prismatic", "pulley", "mouse", "gear"):
                for d in s.get(kind + "_joints", ()):
                    self.create_joint(i, kind, d)
        self.body_counts = [len(s["bodies"]) for s in scenes]
        self.large_worlds = sum(1 for s in scenes if len(s["fixtures"]) >= LARGE_WORLD_FIXTURES)
        if flags is not None:
            self.set_flags(**flags)

    _JOINT_KINDS = {"revolute": ("REVOLUTE_DEF", "dbox_joint_create_revolute"),
                    "distance": ("DISTANCE_DEF", "dbox_joint_create_distance"),
                    "rope": ("ROPE_DEF", "dbox_joint_create_rope"),
                    "weld": ("WELD_DEF", "dbox_joint_create_weld"),
                    "friction": ("FRICTION_DEF", "dbox_joint_create_friction"),
                    "motor": ("MOTOR_DEF", "dbox_joint_create_motor"),
                    "wheel": ("WHEEL_DEF", "dbox_joint_create_wheel"),
                    "prismatic": ("PRISMATIC_DEF", "dbox_joint_create_prismatic"),
                    "pulley": ("PULLEY_DEF", "dbox_joint_create_pulley"),
                    "mouse": ("MOUSE_DEF", "dbox_joint_create_mouse"),
                    "gear": ("GEAR_DEF", "dbox_joint_create_gear")}

    def create_joint(self, world, kind, d):
        """b2World.CreateJoint with a b2DistanceJointDef / b2RopeJointDef / b2WeldJointDef /
        b2FrictionJointDef / b2MotorJointDef / b2WheelJointDef / b2PrismaticJointDef /
        b2PulleyJointDef / b2MouseJointDef (kind "distance", "rope", "weld", "friction",
        "motor", "wheel", "prismatic", "pulley" or "mouse"; d the matching *_DEF record);
        returns the joint index."""
        dtype, fn = World._JOINT_KINDS[kind]
        dd = np.ascontiguousarray(np.array([d], getattr(abi, dtype)))
        out = ctypes.c_int32()
        _check(getattr(lib(), fn)(self.h, world, abi.ptr(dd), ctypes.byref(out)), fn)
        return out.value

    def create_body(self, world, body_def):
        """b2World.CreateBody with a BODY_DEF record; returns the body index."""
        dd = np.ascontiguousarray(np.array([body_def], abi.BODY_DEF))
        out = ctypes.c_int32()
        _check(lib().dbox_body_create(self.h, world, abi.ptr(dd), ctypes.byref(out)), "dbox_body_create")
        return out.value

    def create_fixture(self, world, body, shape_def, fixture_def):
        """b2Body.CreateFixture with SHAPE_DEF and FIXTURE_DEF records; returns the fixture index."""
        sd = np.ascontiguousarray(np.array([shape_def], abi.SHAPE_DEF))
        fd = np.ascontiguousarray(np.array([fixture_def], abi.FIXTURE_DEF))
        out = ctypes.c_int32()
        _check(lib().dbox_fixture_create(self.h, world, body, abi.ptr(sd), abi.ptr(fd), ctypes.byref(out)),
               "dbox_fixture_create")
        return out.value

    def counts(self, world=0):
        """b2World.GetBodyCount / GetJointCount / GetContactCount: (bodies, joints, contacts) alive."""
        b, j, c = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        _check(lib().dbox_world_get_counts(self.h, world, ctypes.byref(b), ctypes.byref(j), ctypes.byref(c)),
               "dbox_world_get_counts")
        return b.value, j.value, c.value

    def destroy_body(self, world, body):
        """b2World.DestroyBody: its joints, contacts (EndContact to the listener) and fixtures."""
        _check(lib().dbox_body_destroy(self.h, world, body), "dbox_body_destroy")

    def destroy_fixture(self, world, fixture):
        """b2Body.DestroyFixture (a chain child destroys its chain)."""
        _check(lib().dbox_fixture_destroy(self.h, world, fixture), "dbox_fixture_destroy")

    def destroy_joint(self, world, joint):
        """b2World.DestroyJoint."""
        _check(lib().dbox_joint_destroy(self.h, world, joint), "dbox_joint_destroy")

    def create_chain(self, world, body, vertices, loop=False, prev=None, next=None, fixture=None):
        """b2Body.CreateFixture with a b2ChainShape (CreateChain / CreateLoop, SetPrevVertex /
        SetNextVertex), created as its child edges; returns the first child's fixture index."""
        v = np.ascontiguousarray(vertices, np.float32)
        pv = np.ascontiguousarray(prev, np.float32) if prev is not None else None
        nv = np.ascontiguousarray(next, np.float32) if next is not None else None
        fd = fixture if fixture is not None else abi.fixture_defs(1)[0]
        fd = np.ascontiguousarray(np.array([fd], abi.FIXTURE_DEF))
        out = ctypes.c_int32()
        _check(lib().dbox_fixture_create_chain(self.h, world, body, abi.ptr(v), len(v), 1 if loop else 0,
                                               abi.ptr(pv) if pv is not None else None,
                                               abi.ptr(nv) if nv is not None else None, abi.ptr(fd), ctypes.byref(out)),
               "dbox_fixture_create_chain")
        return out.value

    def query_aabb(self, worlds, boxes, capacity=64):
        """b2World.QueryAABB for a batch: boxes (n, 4) = lower x, y, upper x, y, one per entry of
        `worlds`.  Returns (counts (n,), fixtures (n, capacity)): every fixture whose fat AABB
        overlaps, in fixture order; counts may exceed capacity (the rest is dropped)."""
        wv = np.ascontiguousarray(np.broadcast_to(np.asarray(worlds, np.int32), (len(boxes),)))
        bv = np.ascontiguousarray(boxes, np.float32).reshape(-1, 4)
        counts = np.zeros(len(bv), np.int32)
        out = np.full((len(bv), capacity), -1, np.int32)
        _check(lib().dbox_world_query_aabb(self.h, len(bv), abi.ptr(wv), abi.ptr(bv), capacity, abi.ptr(counts),
                                           abi.ptr(out)), "dbox_world_query_aabb")
        return counts, out

    def raycast(self, worlds, p1, p2, mode="closest", capacity=None):
        """b2World.RayCast for a batch of rays p1 -> p2 (n, 2).  mode "closest": the hit with the
        smallest fraction (capacity 1); "all": every hit in fixture order.  Returns (counts,
        hits (n, capacity) of abi.RAY_HIT)."""
        m = abi.RAY_CLOSEST if mode == "closest" else abi.RAY_ALL
        cap = capacity if capacity is not None else (1 if m == abi.RAY_CLOSEST else 32)
        a = np.ascontiguousarray(p1, np.float32).reshape(-1, 2)
        b = np.ascontiguousarray(p2, np.float32).reshape(-1, 2)
        wv = np.ascontiguousarray(np.broadcast_to(np.asarray(worlds, np.int32), (len(a),)))
        counts = np.zeros(len(a), np.int32)
        hits = np.zeros((len(a), cap), abi.RAY_HIT)
        hits["fixture"] = -1
        _check(lib().dbox_world_raycast(self.h, len(a), abi.ptr(wv), abi.ptr(a), abi.ptr(b), m, cap, abi.ptr(counts),
                                        abi.ptr(hits)), "dbox_world_raycast")
        return counts, hits

    def dump(self, world=0):
        """b2World.Dump's text for one world of the handle."""
        n = ctypes.c_int64()
        _check(lib().dbox_world_dump(self.h, world, None, 0, ctypes.byref(n)), "dbox_world_dump")
        buf = ctypes.create_string_buffer(n.value + 1)
        _check(lib().dbox_world_dump(self.h, world, buf, n.value + 1, ctypes.byref(n)), "dbox_world_dump")
        return buf.value.decode()

    def stream(self):
        """The cudaStream_t (as an int) the handle's device work runs on."""
        s = ctypes.c_void_p()
        _check(lib().dbox_world_get_stream(self.h, ctypes.byref(s)), "dbox_world_get_stream")
        return s.value or 0

    def query_aabb_device(self, n, worlds_ptr, boxes_ptr, capacity, counts_ptr, out_ptr):
        """dbox_world_query_aabb_device on device addresses (ints), enqueued without a wait."""
        _check(lib().dbox_world_query_aabb_device(self.h, n, worlds_ptr, boxes_ptr, capacity, counts_ptr, out_ptr),
               "dbox_world_query_aabb_device")

    def raycast_device(self, n, worlds_ptr, p1_ptr, p2_ptr, mode, capacity, counts_ptr, hits_ptr):
        """dbox_world_raycast_device on device addresses (ints), enqueued without a wait."""
        _check(lib().dbox_world_raycast_device(self.h, n, worlds_ptr, p1_ptr, p2_ptr, mode, capacity, counts_ptr,
                                               hits_ptr), "dbox_world_raycast_device")

    def set_mouse_target(self, world, joint, target):
        """b2MouseJoint.SetTarget: wakes the dragged body and moves the target."""
        _check(lib().dbox_joint_set_mouse_target(self.h, world, joint, abi.Vec2(*target)), "dbox_joint_set_mouse_target")

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            lib().dbox_world_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_flags(self, warm=1, continuous=1, substep=0, sleep=1, autoclear=1):
        _check(lib().dbox_world_set_flags(self.h, warm, continuous, substep, sleep, autoclear), "dbox_world_set_flags")

    def step(self, dt=1.0 / 60.0, vel_iters=8, pos_iters=3, steps=1, graph=False):
        """b2World.Step(dt, velocityIterations, positionIterations) on every world."""
        if graph:
            _check(lib().dbox_world_step_n(self.h, ctypes.c_float(dt), vel_iters, pos_iters, steps), "dbox_world_step_n")
        else:
            for _ in range(steps):
                _check(lib().dbox_world_step(self.h, ctypes.c_float(dt), vel_iters, pos_iters), "dbox_world_step")

    def step_timed(self, steps, dt=1.0 / 60.0, vel_iters=8, pos_iters=3):
        """Run `steps` steps as one CUDA graph; returns (total_ms, [collide_ms, solve_ms, toi_ms])."""
        tot = np.zeros(1, np.float32)
        ph = np.zeros(3, np.float32)
        _check(lib().dbox_world_step_n_timed(self.h, ctypes.c_float(dt), vel_iters, pos_iters, steps, abi.ptr(tot),
                                             abi.ptr(ph)), "dbox_world_step_n_timed")
        return float(tot[0]), ph.astype(float).tolist()

    def counters(self):
        c = np.zeros(8, np.uint64)
        _check(lib().dbox_world_get_counters(self.h, abi.ptr(c)), "dbox_world_get_counters")
        keys = ("isl_bodies", "isl_contacts", "vsolve", "psolve", "contacts", "toi_events", "world_steps", "pairs")
        return dict(zip(keys, (int(v) for v in c)))

    def set_warmstart(self, mode, model=None, sample_capacity=0):
        """0 plain (the reference step), 1 plain + log training samples, 2 learned start with model,
        3 given start (see set_start_source)."""
        self._model = model                     # the library keeps a pointer: hold a reference
        _check(lib().dbox_world_set_warmstart(self.h, mode, model.h if model is not None else None, sample_capacity),
               "dbox_world_set_warmstart")

    def set_start_source(self, src):
        """Warm-start mode 3: new points start from src's impulses at the same contact slot."""
        self._start_src = src
        _check(lib().dbox_world_set_start_source(self.h, src.h), "dbox_world_set_start_source")

    def copy_state_from(self, src):
        """Exact device-to-device copy of src's simulation state (same worlds, same layout)."""
        _check(lib().dbox_world_copy_state(self.h, src.h), "dbox_world_copy_state")

    def sample_count(self):
        n = ctypes.c_int32()
        _check(lib().dbox_world_sample_count(self.h, ctypes.byref(n)), "dbox_world_sample_count")
        return n.value

    def samples(self, offset=0, n=None):
        """(features (n, 32), targets (n, 4)) of the logged samples."""
        if n is None:
            n = self.sample_count() - offset
        rows = np.zeros((n, MLP_SAMPLE), np.float32)
        _check(lib().dbox_world_get_samples(self.h, offset, n, abi.ptr(rows)), "dbox_world_get_samples")
        return rows[:, :MLP_FEAT].copy(), rows[:, MLP_FEAT:].copy()

    def clear_samples(self):
        _check(lib().dbox_world_clear_samples(self.h), "dbox_world_clear_samples")

    _EVENT_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p)

    def set_listener(self, fn):
        """b2World.SetContactListener: fn(events) is called after each step with the step's
        events (abi.CONTACT_EVENT records, in reference order, world by world); None removes it."""
        if fn is None:
            self._listener = None
            _check(lib().dbox_world_set_listener(self.h, None, None), "dbox_world_set_listener")
            return

        def tramp(ptr, count, user):
            buf = (ctypes.c_char * (count * abi.CONTACT_EVENT.itemsize)).from_address(ptr)
            fn(np.frombuffer(bytes(buf), abi.CONTACT_EVENT).copy())

        self._listener = World._EVENT_FN(tramp)
        _check(lib().dbox_world_set_listener(self.h, ctypes.cast(self._listener, ctypes.c_void_p), None),
               "dbox_world_set_listener")

    def set_filter(self, world, fixture, category_bits=0x0001, mask_bits=0xFFFF, group_index=0):
        """b2Fixture.SetFilterData (and Refilter)."""
        _check(lib().dbox_fixture_set_filter(self.h, world, fixture, category_bits, mask_bits, group_index),
               "dbox_fixture_set_filter")

    def set_filter_class(self, world, fixture, cls):
        """The fixture's class for a table contact filter (and Refilter)."""
        _check(lib().dbox_fixture_set_filter_class(self.h, world, fixture, cls), "dbox_fixture_set_filter_class")

    def set_contact_filter(self, world, table=None, with_default=True):
        """b2World.SetContactFilter with a class table: table (64,) uint64, bit b of row a lets
        classes a and b collide; None restores the default filter."""
        t = None if table is None else np.ascontiguousarray(table, np.uint64)
        _check(lib().dbox_world_set_contact_filter(self.h, world, abi.ptr(t) if t is not None else None,
                                                   1 if with_default else 0), "dbox_world_set_contact_filter")

    _PRESOLVE_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p)

    def set_presolve(self, fn):
        """b2ContactListener.PreSolve through the step's PreSolve window: fn(records) is called
        inside each step, after Collide, with the step's PreSolve calls (abi.PRESOLVE_CONTACT,
        world by world in reference order); it may change "enabled", "friction", "restitution"
        and "tangent_speed" in place.  None removes it."""
        if fn is None:
            self._presolve = None
            _check(lib().dbox_world_set_presolve(self.h, None, None), "dbox_world_set_presolve")
            return

        def tramp(ptr, count, user):
            buf = (ctypes.c_char * (count * abi.PRESOLVE_CONTACT.itemsize)).from_address(ptr)
            recs = np.frombuffer(buf, abi.PRESOLVE_CONTACT)        # a view: edits go straight back
            fn(recs)

        self._presolve = World._PRESOLVE_FN(tramp)
        _check(lib().dbox_world_set_presolve(self.h, ctypes.cast(self._presolve, ctypes.c_void_p), None),
               "dbox_world_set_presolve")

    def set_mapping(self, warps_per_block=4, body_budget=0, isolate=0):
        _check(lib().dbox_world_set_mapping_isolated(self.h, warps_per_block, body_budget, isolate),
               "dbox_world_set_mapping")

    def set_mapping_queue(self, heavy=0, exclusive=False, blocks_per_sm=0):
        """Queue mapping: a resident wave of warps takes worlds costliest first; the `heavy`
        costliest go one per SM sub-partition (alone there with `exclusive`); blocks_per_sm
        limits the resident four-warp blocks per SM (0: as many as fit)."""
        _check(lib().dbox_world_set_mapping_queue(self.h, heavy, 1 if exclusive else 0, blocks_per_sm),
               "dbox_world_set_mapping_queue")

    def set_world_costs(self, cost=None):
        """Per-world cost estimates for the queue order (None: body counts)."""
        if cost is None:
            _check(lib().dbox_world_set_world_costs(self.h, None), "dbox_world_set_world_costs")
            return
        c = np.ascontiguousarray(cost, np.float32)
        assert c.shape == (self.n_worlds,)
        _check(lib().dbox_world_set_world_costs(self.h, abi.ptr(c)), "dbox_world_set_world_costs")

    def world_costs(self):
        out = np.zeros(self.n_worlds, np.float32)
        _check(lib().dbox_world_get_world_costs(self.h, abi.ptr(out)), "dbox_world_get_world_costs")
        return out

    def apply_mapping(self, choice):
        """Apply a mapping returned by autotune()."""
        if choice[3]:
            self.set_mapping_queue(choice[4], bool(choice[5]))
        else:
            self.set_mapping(choice[0], choice[1], choice[2])

    def autotune_steps(self, steps):
        """Steps the worlds advance during autotune(steps): two rounds over 10 mappings, and
        with large worlds two rounds over the 2 island solvers, each trial a graph build step
        plus `steps`, after one profiled step."""
        return 1 + 20 * (steps + 1) + (4 * (steps + 1) if self.large_worlds else 0)

    def autotune(self, steps=3, dt=1.0 / 60.0, vel_iters=8, pos_iters=3):
        """Time the candidate mappings of worlds onto the solve kernel on the live worlds and
        keep the fastest; returns (warps per block, body budget, isolated largest worlds, queue,
        heavy, exclusive).  The worlds advance by autotune_steps(steps) steps."""
        out = np.zeros(6, np.int32)
        _check(lib().dbox_world_autotune(self.h, ctypes.c_float(dt), vel_iters, pos_iters, steps, abi.ptr(out)),
               "dbox_world_autotune")
        return tuple(int(v) for v in out)

    def set_wait_limit(self, polls=1 << 20):
        """Polls a bounded device wait may take before the step reports DBOX_ERR_TIMEOUT."""
        _check(lib().dbox_world_set_wait_limit(self.h, polls), "dbox_world_set_wait_limit")

    def set_island_solver(self, mode=0):
        """Large worlds' Solve on a thread-block cluster (0, default) or on a warp (1); the same results."""
        _check(lib().dbox_world_set_island_solver(self.h, mode), "dbox_world_set_island_solver")

    def island_solver(self):
        out = ctypes.c_int32()
        _check(lib().dbox_world_get_island_solver(self.h, ctypes.byref(out)), "dbox_world_get_island_solver")
        return out.value

    def set_fused_step(self, on=True):
        """Whole steps in one launch, or four launches a step (default); the same results."""
        _check(lib().dbox_world_set_fused_step(self.h, 1 if on else 0), "dbox_world_set_fused_step")

    def fused_step(self):
        out = ctypes.c_int32()
        _check(lib().dbox_world_get_fused_step(self.h, ctypes.byref(out)), "dbox_world_get_fused_step")
        return bool(out.value)

    def set_measure(self, on=True):
        _check(lib().dbox_world_set_measure(self.h, 1 if on else 0), "dbox_world_set_measure")

    def quality(self):
        """(n_worlds, 4): sum of |dlambda|^2, max |dlambda|, points, min separation of the last step."""
        out = np.zeros((self.n_worlds, 4), np.float32)
        _check(lib().dbox_world_get_quality(self.h, abi.ptr(out)), "dbox_world_get_quality")
        return out

    def set_phase_profile(self, on=True):
        _check(lib().dbox_world_set_phase_profile(self.h, 1 if on else 0), "set_phase_profile")

    def phase_profile(self):
        """(n_worlds, 32) uint64 per-world clock figures of the last step (layout in dbox_gpu.h)."""
        out = np.zeros((self.n_worlds, 32), np.uint64)
        _check(lib().dbox_world_get_phase_profile(self.h, abi.ptr(out)), "get_phase_profile")
        return out

    def apply_forces(self, force_torque):
        """ApplyForceToCenter + ApplyTorque (wake = false) on every body; (n_bodies, 3) float32, ideally pinned."""
        assert force_torque.dtype == np.float32 and force_torque.flags["C_CONTIGUOUS"]
        _check(lib().dbox_world_apply_forces(self.h, abi.ptr(force_torque)), "dbox_world_apply_forces")

    def get_transforms(self, out):
        """GetPosition + GetAngle of every body into out (n_bodies, 3) float32, ideally pinned."""
        assert out.dtype == np.float32 and out.flags["C_CONTIGUOUS"]
        _check(lib().dbox_world_get_transforms(self.h, abi.ptr(out)), "dbox_world_get_transforms")
        return out

    def sync(self):
        _check(lib().dbox_world_sync(self.h), "dbox_world_sync")

    def bodies(self):
        n = sum(self.body_counts)
        pos = np.zeros((n, 2), np.float32)
        ang = np.zeros(n, np.float32)
        vel = np.zeros((n, 2), np.float32)
        avel = np.zeros(n, np.float32)
        awake = np.zeros(n, np.int32)
        _check(lib().dbox_world_get_bodies(self.h, abi.ptr(pos), abi.ptr(ang), abi.ptr(vel), abi.ptr(avel),
                                           abi.ptr(awake)), "dbox_world_get_bodies")
        return {"position": pos, "angle": ang, "linear_velocity": vel, "angular_velocity": avel, "awake": awake}

    def export_state(self, world=0):
        L = lib()
        hdr = np.zeros(1, abi.WORLD_HEADER)
        _check(L.dbox_world_export_state(self.h, world, abi.ptr(hdr), None, None, None, None), "export header")
        h = hdr[0]
        bodies = np.zeros(int(h["body_count"]), abi.BODY_STATE)
        proxies = np.zeros(int(h["fixture_count"]), abi.PROXY_STATE)
        contacts = np.zeros(int(h["contact_count"]), abi.CONTACT_STATE)
        joints = np.zeros(int(h["joint_count"]), abi.JOINT_STATE)
        _check(L.dbox_world_export_state(self.h, world, abi.ptr(hdr), abi.ptr(bodies), abi.ptr(proxies),
                                         abi.ptr(contacts), abi.ptr(joints)), "export")
        return {"header": hdr, "bodies": bodies, "proxies": proxies, "contacts": contacts, "joints": joints}

    def import_state(self, state, world=0):
        st = {k: np.ascontiguousarray(v) for k, v in state.items()}
        _check(lib().dbox_world_import_state(self.h, world, abi.ptr(st["header"]), abi.ptr(st["bodies"]),
                                             abi.ptr(st["proxies"]), abi.ptr(st["contacts"]),
                                             abi.ptr(st["joints"])), "import")

    def stats(self, world=0):
        isl, toi = ctypes.c_int32(), ctypes.c_int32()
        _check(lib().dbox_world_step_stats(self.h, world, ctypes.byref(isl), ctypes.byref(toi)), "stats")
        return isl.value, toi.value

    def last_launches(self):
        n = ctypes.c_int32()
        _check(lib().dbox_world_last_launches(self.h, ctypes.byref(n)), "launches")
        return n.value

    def profile(self):
        p = np.zeros(1, abi.PROFILE)
        _check(lib().dbox_world_get_profile(self.h, abi.ptr(p)), "profile")
        return p[0]
