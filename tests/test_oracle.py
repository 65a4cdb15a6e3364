"""CPU checks of the oracle (the CPU restatement of b2World.Step).

The reference ships no tests or recorded outputs, so the oracle is checked
against answers derived by hand from the reference's formulas (mass, hull,
manifold, free fall), against brute force (broad-phase pairs vs. fat-AABB
overlaps, the analogue of examples/demo/tests/dynamictreetest.d:333) and
against the committed golden fixtures in tests/golden (regression pins).
"""
import math

import numpy as np
import pytest

from dbox_gb300 import abi, scenes


def _box(hx, hy):
    s = np.zeros((), abi.SHAPE_DEF)
    s["kind"] = abi.SHAPE_BOX
    s["hx"] = hx
    s["hy"] = hy
    return s


def _ulp_error(got, x, fn):
    exact = fn(x.astype(np.float64))
    r = exact.astype(np.float32)
    _, e = np.frexp(r.astype(np.float64))
    ulp = np.ldexp(1.0, e - 24)
    return np.abs(got.astype(np.float64) - exact) / ulp


def test_portable_trig_accuracy(oracle_lib):
    # dbox_sincosf: binary32 + FMA below |x| = 1024 (error < 0.75 ulp), binary64 above (correctly rounded)
    rng = np.random.default_rng(0)
    small = np.concatenate([rng.uniform(-10.0, 10.0, 300000), rng.uniform(-1024.0, 1024.0, 100000),
                            np.array([1e-30, 1e-8, np.pi / 4, np.pi / 2, 1024.0], np.float64)]).astype(np.float32)
    oracle_lib.set_trig_mode(1)
    s, c = oracle_lib.sincos_array(small)
    assert _ulp_error(s, small, np.sin).max() < 0.75
    assert _ulp_error(c, small, np.cos).max() < 0.75
    cr = (s == np.sin(small.astype(np.float64)).astype(np.float32)).mean()
    assert cr > 0.98          # glibc 2.39 sinf: 0.987 on the same kind of sample
    big = np.concatenate([rng.uniform(-1e5, 1e5, 50000), rng.uniform(-1e30, 1e30, 20000),
                          np.array([1024.0001, 131071.99, 131072.0], np.float64)]).astype(np.float32)
    big = big[np.abs(big) > 1024.0]
    s, c = oracle_lib.sincos_array(big)
    assert (s == np.sin(big.astype(np.float64)).astype(np.float32)).mean() > 1 - 1e-5
    assert (c == np.cos(big.astype(np.float64)).astype(np.float32)).mean() > 1 - 1e-5
    z = np.array([0.0, -0.0], np.float32)
    s, c = oracle_lib.sincos_array(z)
    assert np.signbit(s).tolist() == [False, True] and c.tolist() == [1.0, 1.0]


def test_libm_trig_mode_is_the_host_runtime(oracle_lib):
    xs = np.linspace(-6.0, 6.0, 1001, dtype=np.float32)
    oracle_lib.set_trig_mode(0)
    try:
        s, c = oracle_lib.sincos_array(xs)
    finally:
        oracle_lib.set_trig_mode(1)
    assert np.allclose(s, np.sin(xs.astype(np.float64)), atol=2e-7)
    assert np.allclose(c, np.cos(xs.astype(np.float64)), atol=2e-7)


def test_polygon_hull_order(oracle_lib):
    # b2PolygonShape.Set: start at the right-most (then lowest) point, wrap counter-clockwise
    pts = [(-1, 1), (1, 1), (0.1, 0.2), (1, -1), (-1, -1)]
    v, n, c = oracle_lib.polygon_set(pts)
    assert v.tolist() == [[1, -1], [1, 1], [-1, 1], [-1, -1]]
    assert n.tolist() == [[1, 0], [0, 1], [-1, 0], [0, -1]]
    assert c.tolist() == [0, 0]
    assert oracle_lib.polygon_set([(0, 0), (1, 0), (0.001, 0.001)]) is None   # welded to 2 points


def test_box_and_circle_mass(oracle_lib):
    s = scenes.hello_world()
    st = oracle_lib.OracleWorld(s).export_state()
    m = st["bodies"]["mass"][1]
    assert m[0] == np.float32(4.0) and m[1] == np.float32(0.25)           # 2x2 box, density 1
    assert abs(m[2] - 4.0 * 8.0 / 12.0) < 1e-5                            # m (w^2 + h^2) / 12
    c = scenes._boxes([(0.0, 5.0)], 1.0, 1.0, abi.DYNAMIC, 0.2, 2.0)
    c["shapes"]["kind"] = abi.SHAPE_CIRCLE
    c["shapes"]["radius"] = 0.5
    mc = oracle_lib.OracleWorld(c).export_state()["bodies"]["mass"][0]
    assert abs(mc[0] - 2.0 * math.pi * 0.25) < 1e-6
    assert abs(mc[2] - mc[0] * 0.5 * 0.25) < 1e-6


def test_polygon_manifold_known_answer(oracle_lib):
    # box B resting 0.01 m into box A: reference face is A's top edge (index 2), two points
    m = oracle_lib.collide(_box(0.5, 0.5), [0, 0, 0, 1], _box(0.5, 0.5), [0, 0.99, 0, 1])
    assert m["point_count"] == 2 and m["type"] == 1
    assert m["local_normal"].tolist() == [0.0, 1.0] and m["local_point"].tolist() == [0.0, 0.5]
    assert m["points"]["local_point"].tolist() == [[-0.5, -0.5], [0.5, -0.5]]
    # id = indexA | indexB << 8 | typeA << 16 | typeB << 24 with face = 1, vertex = 0
    assert m["points"]["id"].tolist() == [0x00010002, 0x00010102]
    far = oracle_lib.collide(_box(0.5, 0.5), [0, 0, 0, 1], _box(0.5, 0.5), [0, 1.03, 0, 1])
    assert far["point_count"] == 0


def test_circle_manifolds_known_answer(oracle_lib):
    c = np.zeros((), abi.SHAPE_DEF)
    c["kind"] = abi.SHAPE_CIRCLE
    c["radius"] = 0.5
    m = oracle_lib.collide(c, [0, 0, 0, 1], c, [0.9, 0, 0, 1])
    assert m["point_count"] == 1 and m["type"] == 0 and m["points"]["id"][0] == 0
    assert oracle_lib.collide(c, [0, 0, 0, 1], c, [1.01, 0, 0, 1])["point_count"] == 0
    m = oracle_lib.collide(_box(0.5, 0.5), [0, 0, 0, 1], c, [0, 0.95, 0, 1])
    assert m["point_count"] == 1 and m["type"] == 1
    assert m["local_normal"].tolist() == [0.0, 1.0]


def test_free_fall_matches_float32_recurrence(oracle_lib):
    s = scenes._boxes([(0.0, 100.0)], 0.5, 0.5, abi.DYNAMIC)
    w = oracle_lib.OracleWorld(s)
    h = np.float32(1.0 / 60.0)
    v = np.float32(0.0)
    y = np.float32(100.0)
    for _ in range(120):
        w.step()
        v = np.float32(v + np.float32(h * np.float32(np.float32(-10.0) + np.float32(0.0))))
        y = np.float32(y + np.float32(h * v))
    b = w.export_state()["bodies"][0]
    assert b["vel"][1] == v and b["sweep"][5] == y


def test_proxy_ids_are_tree_node_ids(oracle_lib):
    st = oracle_lib.OracleWorld(scenes.pyramid(rows=6)).export_state()
    k = np.arange(len(st["proxies"]))
    assert st["proxies"]["proxy_id"].tolist() == np.where(k == 0, 0, 2 * k - 1).tolist()


def test_contacts_cover_fat_aabb_overlaps(oracle_lib):
    # after every step each eligible pair of overlapping fat AABBs has a contact (tree query == brute force)
    s = scenes.scatter(150, 20.0, 30.0, np.random.default_rng(5))
    w = oracle_lib.OracleWorld(s)
    body = s["fixture_body"]
    dyn = s["bodies"]["type"][body] == abi.DYNAMIC
    for t in range(80):
        w.step()
        if t % 8:
            continue
        st = w.export_state()
        fat = st["proxies"]["fat_aabb"]
        have = {(min(a, b), max(a, b)) for a, b in zip(st["contacts"]["fixture_a"], st["contacts"]["fixture_b"])}
        lo, hi = fat[:, :2], fat[:, 2:]
        ov = ((lo[:, None, :] <= hi[None, :, :]) & (lo[None, :, :] <= hi[:, None, :])).all(-1)
        ia, ib = np.nonzero(np.triu(ov, 1))
        for a, b in zip(ia, ib):
            if body[a] == body[b] or not (dyn[a] or dyn[b]):
                continue
            assert (a, b) in have, "step %d: overlapping pair %s without contact" % (t, (a, b))


def test_pyramid_settles_and_sleeps(oracle_lib):
    oracle_lib.set_trig_mode(0)
    try:
        w = oracle_lib.OracleWorld(scenes.pyramid())
        w.step(steps=600)
        st = w.export_state()
    finally:
        oracle_lib.set_trig_mode(1)
    dyn = st["bodies"]["type"] == abi.DYNAMIC
    assert ((st["bodies"]["flags"][dyn] & abi.BODY_AWAKE) == 0).all()
    top = st["bodies"]["xf"][-1]
    assert abs(top[1] - 19.75) < 0.02 and abs(top[0]) < 0.5


def test_hello_world_prints_reference_line(oracle_lib):
    # examples/hello_world/hello_world.d:86-99 prints x, y, angle with %4.2f each step
    w = oracle_lib.OracleWorld(scenes.hello_world())
    for _ in range(60):
        w.step(1.0 / 60.0, 6, 2)
    b = w.export_state()["bodies"][1]
    assert "%4.2f %4.2f %4.2f" % (b["xf"][0], b["xf"][1], b["sweep"][7]) == "0.00 1.01 0.00"


def test_distance_joint_ropes_hold_their_length(oracle_lib):
    # b2DistanceJoint (joints/b2distancejoint.d): rigid ropes keep each link at the joint
    # length from its neighbour; soft ropes (4 Hz) stretch under their weight but stay bounded;
    # the joint impulses carry over between steps (warm start)
    from dbox_gb300 import scenes
    oracle_lib.set_trig_mode(1)
    s = scenes.ropes(n_ropes=2, links=10, pile=False, revolute=False)
    ow = oracle_lib.OracleWorld(s)
    ow.step(steps=240)
    st = ow.export_state()
    xy = st["bodies"]["xf"][:, :2].astype(np.float64)
    gap = 0.3
    for r, rigid in ((0, True), (1, False)):
        post = 1 + r * 11                      # ground, then per rope: post + 10 links
        d = np.linalg.norm(np.diff(xy[post:post + 11], axis=0), axis=1)
        if rigid:
            assert np.abs(d - gap).max() < 0.01, d
        else:
            assert d.max() < 4.0 * gap and d.min() > 0.5 * gap, d
    assert (st["joints"]["impulse"][:, 0] != 0).all()


def test_weld_beams_and_ropes(oracle_lib):
    # b2WeldJoint keeps rigid beams straight and near their welds' reference angle; b2RopeJoint
    # never lets its anchors get further apart than the maximum length (plus the solver slop)
    from dbox_gb300 import scenes
    oracle_lib.set_trig_mode(1)
    s = scenes.welded(n_beams=2, links=6, pile=False)
    ow = oracle_lib.OracleWorld(s)
    ow.step(steps=240)
    st = ow.export_state()
    b = st["bodies"]
    ang = b["sweep"][:, 7]
    # beam 0 (rigid welds): bodies 2..7 (ground 0, post 1); the welds hold each link close to
    # its neighbour's angle (a long weld chain sags a little under 8/3 iterations) and the
    # beam stays up
    assert np.abs(np.diff(ang[1:8])).max() < 0.2, ang[1:8]
    assert b["xf"][7, 1] > b["xf"][2, 1] - 2.0
    # rope constraints: distance between anchors within max length + 2 linear slops
    xy = b["xf"][:, :2].astype(np.float64)
    c, sn = b["xf"][:, 3].astype(np.float64), b["xf"][:, 2].astype(np.float64)

    def world_point(i, p):
        return xy[i] + np.array([c[i] * p[0] - sn[i] * p[1], sn[i] * p[0] + c[i] * p[1]])

    for r in s["rope_joints"]:
        d = np.linalg.norm(world_point(r["body_b"], r["local_anchor_b"]) - world_point(r["body_a"], r["local_anchor_a"]))
        assert d <= r["max_length"] + 0.02, (d, r["max_length"])
    n_rev, n_dist, n_rope = len(s["joints"]), len(s["distance_joints"]), len(s["rope_joints"])
    imp = st["joints"]["impulse"]
    assert (imp[n_rev + n_dist:n_rev + n_dist + n_rope, 0] <= 0).all()          # ropes only pull
    assert (st["joints"]["limit_state"][n_rev + n_dist:n_rev + n_dist + n_rope] == 2).any()


def test_friction_and_motor_joints_top_down(oracle_lib):
    # b2FrictionJoint brakes the top-down bodies (no gravity); b2MotorJoint drives its
    # platform to the offset (position and angle) from the table body
    from dbox_gb300 import scenes
    oracle_lib.set_trig_mode(1)
    s = scenes.top_down()
    ow = oracle_lib.OracleWorld(s)
    ow.step(steps=240)
    b = ow.export_state()["bodies"]
    v0 = np.abs(s["bodies"]["linear_velocity"]).sum()
    assert np.abs(b["vel"][:, :2]).sum() < 0.2 * v0
    m = s["motor_joints"][0]
    p = b["xf"][m["body_b"], :2]
    assert np.abs(p - m["linear_offset"]).max() < 0.05, p
    assert abs(b["sweep"][m["body_b"], 7] - m["angular_offset"]) < 0.02


def test_wheel_joint_cars_drive(oracle_lib):
    # b2WheelJoint: the motor-driven cars drive forward over the bumps on sprung wheels that
    # stay under the chassis (point-to-line constraint) and stay on their axles
    from dbox_gb300 import scenes
    oracle_lib.set_trig_mode(1)
    s = scenes.cars()
    ow = oracle_lib.OracleWorld(s)
    ow.step(steps=300)
    st = ow.export_state()
    b = st["bodies"]
    n = len(s["bodies"])
    for c in range(3):
        chassis, rear, front = n - 9 + 3 * c, n - 8 + 3 * c, n - 7 + 3 * c
        if c % 2 == 0:
            assert b["xf"][chassis, 0] - s["bodies"]["position"][chassis, 0] > 5.0
        # each wheel's centre stays on the chassis' suspension line (body-frame x within 1 cm)
        cx, cy, sn, cs = b["xf"][chassis]
        for wheel, ax in ((rear, -1.0), (front, 1.0)):
            dx, dy = b["xf"][wheel, 0] - cx, b["xf"][wheel, 1] - cy
            assert abs(cs * dx + sn * dy - ax) < 0.01
    assert st["joints"]["motor_impulse"][0] != 0


def test_prismatic_sliders(oracle_lib):
    # b2PrismaticJoint: motor-lifted platforms stop at their upper limit, the tilted slider
    # rests at its lower limit, the locked one holds its reference angle
    from dbox_gb300 import scenes
    oracle_lib.set_trig_mode(1)
    s = scenes.sliders()
    ow = oracle_lib.OracleWorld(s)
    ow.step(steps=240)
    st = ow.export_state()
    b, jt = st["bodies"], st["joints"]
    assert abs(b["xf"][1, 1] - 5.0) < 0.02 and jt["limit_state"][0] == 2 and jt["motor_impulse"][0] > 0
    assert jt["limit_state"][1] == 1
    assert abs(b["sweep"][1 + 3 * 6, 7] - 0.1) < 0.01 and jt["limit_state"][3] == 3


def test_pulley_and_mouse_joints(oracle_lib):
    # b2PulleyJoint keeps lengthA + ratio * lengthB at its constant (within the position
    # tolerance) while the heavier side sinks; b2MouseJoint drags its body to a moved target
    from dbox_gb300 import scenes
    oracle_lib.set_trig_mode(1)
    s = scenes.pulleys(n=2)
    ow = oracle_lib.OracleWorld(s)
    ow.step(steps=150)
    ow.set_mouse_target(2, (4.0, 3.0))
    ow.step(steps=150)
    b = ow.export_state()["bodies"]
    for p in s["pulley_joints"]:
        ya, yb = b["xf"][p["body_a"], 1] + 0.5, b["xf"][p["body_b"], 1] + 0.5
        la = np.hypot(b["xf"][p["body_a"], 0] - p["ground_anchor_a"][0], 10.0 - ya)
        lb = np.hypot(b["xf"][p["body_b"], 0] - p["ground_anchor_b"][0], 10.0 - yb)
        assert abs(la + p["ratio"] * lb - (p["length_a"] + p["ratio"] * p["length_b"])) < 0.05
    assert b["xf"][2, 1] < b["xf"][1, 1]                      # the heavier side went down
    m = s["mouse_joints"][0]["body_b"]
    assert np.hypot(b["xf"][m, 0] - 4.0, b["xf"][m, 1] - 3.0) < 0.6      # centre; the anchor is 0.28 m off it


def test_edge_shapes_collide(oracle_lib):
    # b2EdgeShape with b2CollideEdgeAndCircle / b2EPCollider: bodies come to rest on the edge
    # terrain, contacts pair an edge (fixture A) with circles and polygons (face-A and face-B
    # manifolds both occur), edges never touch edges, and the pyramid on the flat edge stands
    from dbox_gb300 import scenes
    oracle_lib.set_trig_mode(1)
    s = scenes.edge_ground()
    ow = oracle_lib.OracleWorld(s)
    ow.step(steps=300)
    st = ow.export_state()
    b, c = st["bodies"], st["contacts"]
    kind = s["shapes"]["kind"]
    ka, kb = kind[c["fixture_a"]], kind[c["fixture_b"]]
    assert ((ka == 4) & (kb != 4)).any() and not ((kb == 4) & (ka != 4)).any() and not ((ka == 4) & (kb == 4)).any()
    edge_c = c[(ka == 4) & (c["point_count"] > 0)]
    assert set(np.unique(edge_c["type"])) >= {1, 2}
    dyn = b["type"] == 2
    assert np.isfinite(b["xf"]).all() and b["xf"][dyn, 1].min() > -0.05
    pyr = slice(1 + 1 + 1, 1 + 1 + 1 + 21)                    # ground, two ramps, then the 6-row pyramid
    assert np.abs(b["sweep"][pyr, 7]).max() < 0.05             # still standing


def test_chain_shapes_collide(oracle_lib):
    # b2ChainShape as its child edges (GetChildEdge ghosts; CreateLoop closes the bowl):
    # bodies dropped into the loop bowl stay in it, the valley chain and the open chain carry
    # their bodies, every chain contact has the chain child as fixture A, and the carrier's
    # loop chain adds no mass
    from dbox_gb300 import scenes
    oracle_lib.set_trig_mode(1)
    s = scenes.chain_ground()
    n_fix = len(s["fixtures"])
    ow = oracle_lib.OracleWorld(s)
    ow.step(steps=300)
    st = ow.export_state()
    b, c = st["bodies"], st["contacts"]
    children = 20 + 11 + 2 + 4                                 # loop of 20 vertices, chains of 12 and 3, loop of 4
    assert c["fixture_a"].max() < n_fix + children
    chain_c = c[(c["fixture_a"] >= n_fix) | (c["fixture_b"] >= n_fix)]
    assert len(chain_c) and (chain_c["fixture_a"] >= n_fix).all()
    assert not ((c["fixture_a"] >= n_fix) & (c["fixture_b"] >= n_fix)).any()
    dyn = b["type"] == 2
    assert np.isfinite(b["xf"]).all()
    assert b["xf"][dyn, 1].min() > 0.5                         # nothing fell through a chain (lowest at y = 1)
    assert (chain_c["point_count"] > 0).sum() > 10


def test_gear_joints_hold_their_ratio(oracle_lib):
    # b2GearJoint keeps coordinate1 + ratio * coordinate2 at its initial value: the wheel of
    # radius 2 turns at half the speed of the radius-1 wheel, in the other sense; the rack
    # wheel moves its plate by its radius per radian; the wheels on the swinging arm keep
    # their ratio relative to it
    from dbox_gb300 import scenes
    oracle_lib.set_trig_mode(1)
    s = scenes.gears()
    ow = oracle_lib.OracleWorld(s)
    st0 = ow.export_state()["bodies"]
    ow.step(steps=120)
    st = ow.export_state()["bodies"]
    a = lambda i: float(st["sweep"][i, 7] - st0["sweep"][i, 7])
    assert abs(a(1)) > 1.0                                      # the motor turned the small wheel
    assert abs(a(1) + 2.0 * a(2)) < 0.02
    dx = float(st["xf"][4, 0] - st0["xf"][4, 0])
    assert abs(dx) > 0.5 and abs(a(3) - dx) < 0.02
    rel = lambda i: a(i) - a(5)
    assert abs(rel(6) + 0.75 * rel(7)) < 0.02
    assert np.isfinite(st["xf"]).all()


def test_concat_moves_gear_joint_indices():
    # a gear joint names its joints by creation index (all revolute joints, then distance, ...,
    # prismatic, ...); merging scenes moves those indices to the joints' new places
    from dbox_gb300 import scenes
    a, b = scenes.gears(), scenes.gears(seed=3)
    m = scenes._concat([a, b])
    na_rev, nb_rev = len(a["joints"]), len(b["joints"])
    nrev = na_rev + nb_rev
    kinds = scenes.JOINT_KINDS

    def kind_of(scene, idx):
        for k in kinds:
            n = len(scene.get(k, ()))
            if idx < n:
                return k, idx
            idx -= n
        raise IndexError(idx)

    for part, off_rev, off_pri, gears in ((a, 0, 0, m["gear_joints"][:len(a["gear_joints"])]),
                                          (b, na_rev, len(a["prismatic_joints"]), m["gear_joints"][len(a["gear_joints"]):])):
        for g_old, g_new in zip(part["gear_joints"], gears):
            for f in ("joint1", "joint2"):
                k, i = kind_of(part, int(g_old[f]))
                want = off_rev + i if k == "joints" else nrev + len(m["distance_joints"]) + len(m["rope_joints"]) + \
                    len(m["weld_joints"]) + len(m["friction_joints"]) + len(m["motor_joints"]) + \
                    len(m["wheel_joints"]) + off_pri + i
                assert int(g_new[f]) == want, (f, k, i)
    assert m["gear_joints"][len(a["gear_joints"]):]["body_a"].min() >= len(a["bodies"])
