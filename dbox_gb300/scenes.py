"""Seeded synthetic scenes for the b2World.Step workloads.

Each scene is a dict of plain records (see abi.py): bodies, fixture_body,
shapes, fixtures, joints, plus gravity.  The same records feed the GPU library
(dbox_scene_create) and the CPU oracle, so both build identical worlds.

Workloads (sizes as named in the benchmark configuration):
  pyramid   - static ground box 50x10 half extents at y=-10; 20-row pyramid of
              210 dynamic SetAsBox(0.5, 0.5) boxes, base row centred at y=0.75,
              spacing 1.125 m horizontal / 1.0 m vertical, each row shifted by
              half a spacing (the layout of examples/demo/tests/pyramid.d:51-67
              with a box ground); density 1, friction 0.6.
  scatter   - static container of 4 box walls; n dynamic bodies, half circles
              (r ~ U[0.25,0.5]) and half convex polygons (3..8 points at sorted
              angles U[0, 2pi) conditioned on gaps in (0.25, pi) rad, radius
              U[0.3,0.6], hull by b2PolygonShape.Set) on
              a jittered grid (spacing 1.3 m, jitter U[-0.1,0.1]), friction
              U[0.2,0.8], velocity N(0,1) per axis.
  stacks    - ground box plus columns of unit boxes 1..30 high.
  batch     - n worlds with body counts log-uniform in [8,512], one third each
              pyramid / scatter (40 m container) / stacks.
Random numbers come from numpy's PCG64 generator with the given seed.
"""
import math

import numpy as np

from . import abi

F32 = np.float32


def _empty():
    return {
        "bodies": abi.body_defs(0), "fixture_body": np.zeros(0, np.int32),
        "shapes": np.zeros(0, abi.SHAPE_DEF), "fixtures": abi.fixture_defs(0),
        "joints": np.zeros(0, abi.REVOLUTE_DEF), "distance_joints": np.zeros(0, abi.DISTANCE_DEF),
        "rope_joints": np.zeros(0, abi.ROPE_DEF), "weld_joints": np.zeros(0, abi.WELD_DEF),
        "friction_joints": np.zeros(0, abi.FRICTION_DEF), "motor_joints": np.zeros(0, abi.MOTOR_DEF),
        "wheel_joints": np.zeros(0, abi.WHEEL_DEF), "prismatic_joints": np.zeros(0, abi.PRISMATIC_DEF),
        "pulley_joints": np.zeros(0, abi.PULLEY_DEF), "mouse_joints": np.zeros(0, abi.MOUSE_DEF),
        "gear_joints": np.zeros(0, abi.GEAR_DEF),
        "chains": [], "gravity": (0.0, -10.0), "name": "",
    }


# joint kinds in creation order: a scene's joints are created kind by kind in this order, so a
# joint's index is the count of the earlier kinds plus its place in its own kind
JOINT_KINDS = ("joints", "distance_joints", "rope_joints", "weld_joints", "friction_joints", "motor_joints",
               "wheel_joints", "prismatic_joints", "pulley_joints", "mouse_joints", "gear_joints")


def _concat(parts):
    """Concatenate scene parts; fixture_body / joint body indices are offset per part, and a
    gear joint's joint indices are moved to the joints' places in the concatenated order."""
    out = _empty()
    nb = 0
    counts = [[len(p.get(k, ())) for k in JOINT_KINDS] for p in parts]
    totals = [sum(c[i] for c in counts) for i in range(len(JOINT_KINDS))]
    for pi, p in enumerate(parts):
        g = p.get("gear_joints", np.zeros(0, abi.GEAR_DEF)).copy()
        g["body_a"] += nb
        g["body_b"] += nb
        for f in ("joint1", "joint2"):
            for r in range(len(g)):
                idx, k = int(g[r][f]), 0
                while idx >= counts[pi][k]:
                    idx -= counts[pi][k]
                    k += 1
                g[r][f] = sum(totals[:k]) + sum(c[k] for c in counts[:pi]) + idx
        out["gear_joints"] = np.concatenate([out["gear_joints"], g])
        out["bodies"] = np.concatenate([out["bodies"], p["bodies"]])
        out["fixture_body"] = np.concatenate([out["fixture_body"], p["fixture_body"] + nb]).astype(np.int32)
        out["shapes"] = np.concatenate([out["shapes"], p["shapes"]])
        out["fixtures"] = np.concatenate([out["fixtures"], p["fixtures"]])
        j = p["joints"].copy()
        j["body_a"] += nb
        j["body_b"] += nb
        out["joints"] = np.concatenate([out["joints"], j])
        for key, dtype in (("distance_joints", abi.DISTANCE_DEF), ("rope_joints", abi.ROPE_DEF),
                           ("weld_joints", abi.WELD_DEF), ("friction_joints", abi.FRICTION_DEF),
                           ("motor_joints", abi.MOTOR_DEF), ("wheel_joints", abi.WHEEL_DEF),
                           ("prismatic_joints", abi.PRISMATIC_DEF), ("pulley_joints", abi.PULLEY_DEF),
                           ("mouse_joints", abi.MOUSE_DEF)):
            d = p.get(key, np.zeros(0, dtype)).copy()
            d["body_a"] += nb
            d["body_b"] += nb
            out[key] = np.concatenate([out[key], d])
        out["chains"] = out["chains"] + [dict(c, body=c["body"] + nb) for c in p.get("chains", ())]
        nb += len(p["bodies"])
    return out


def _boxes(centers, hx, hy, btype, friction=0.6, density=1.0):
    n = len(centers)
    s = _empty()
    b = abi.body_defs(n)
    b["type"] = btype
    b["position"] = np.asarray(centers, F32)
    s["bodies"] = b
    s["fixture_body"] = np.arange(n, dtype=np.int32)
    sh = np.zeros(n, abi.SHAPE_DEF)
    sh["kind"] = abi.SHAPE_BOX
    sh["hx"] = hx
    sh["hy"] = hy
    s["shapes"] = sh
    f = abi.fixture_defs(n)
    f["friction"] = F32(friction)
    f["density"] = F32(density if btype == abi.DYNAMIC else 0.0)
    s["fixtures"] = f
    return s


def ground_box(hx=50.0, hy=10.0, y=-10.0):
    return _boxes([(0.0, y)], hx, hy, abi.STATIC)


def pyramid(rows=20, box=0.5, dx=1.125, dy=1.0, y0=0.75, friction=0.6, density=1.0, ground=True):
    """Pyramid of rows*(rows+1)/2 boxes; positions accumulate in float32 like pyramid.d:59-70."""
    centers = []
    x = np.array([-(rows - 1) * dx / 2.0, y0], F32)
    delta_x = np.array([dx / 2.0, dy], F32)
    delta_y = np.array([dx, 0.0], F32)
    for i in range(rows):
        y = x.copy()
        for _ in range(i, rows):
            centers.append(y.copy())
            y = (y + delta_y).astype(F32)
        x = (x + delta_x).astype(F32)
    parts = []
    if ground:
        parts.append(ground_box())
    parts.append(_boxes(centers, box, box, abi.DYNAMIC, friction, density))
    s = _concat(parts)
    s["name"] = "pyramid%d" % rows
    return s


def container(width, height, thick=1.0):
    """Four static box walls enclosing [-width/2, width/2] x [0, height]."""
    hw = width / 2.0
    parts = [
        _boxes([(0.0, -thick)], hw + thick, thick, abi.STATIC),
        _boxes([(0.0, height + thick)], hw + thick, thick, abi.STATIC),
        _boxes([(-hw - thick, height / 2.0)], thick, height / 2.0 + 2 * thick, abi.STATIC),
        _boxes([(hw + thick, height / 2.0)], thick, height / 2.0 + 2 * thick, abi.STATIC),
    ]
    return _concat(parts)


def scatter(n, width, height, rng, spacing=1.3, jitter=0.1, y_base=1.0):
    """n mixed circles/polygons on a jittered grid inside a width x height container."""
    cols = max(1, int((width - 2.0) // spacing))
    rows = (n + cols - 1) // cols
    idx = np.arange(n)
    gx = (idx % cols).astype(np.float64)
    gy = (idx // cols).astype(np.float64)
    x0 = -(cols - 1) * spacing / 2.0
    pos = np.stack([x0 + gx * spacing, y_base + 0.65 + gy * spacing], 1)
    pos += rng.uniform(-jitter, jitter, size=(n, 2))
    kinds = rng.permutation(np.arange(n) % 2)  # half circles, half polygons
    b = abi.body_defs(n)
    b["type"] = abi.DYNAMIC
    b["position"] = pos.astype(F32)
    b["linear_velocity"] = rng.normal(0.0, 1.0, size=(n, 2)).astype(F32)
    sh = np.zeros(n, abi.SHAPE_DEF)
    circ = kinds == 0
    sh["kind"][circ] = abi.SHAPE_CIRCLE
    sh["radius"][circ] = rng.uniform(0.25, 0.5, size=int(circ.sum())).astype(F32)
    poly = np.nonzero(~circ)[0]
    sh["kind"][poly] = abi.SHAPE_POLYGON
    for i in poly:
        k = int(rng.integers(3, 9))
        while True:
            # rejection sampling keeps b2PolygonShape.Set away from welded / sliver hulls:
            # every gap between sorted angles above 0.25 rad, the largest below pi
            ang = np.sort(rng.uniform(0.0, 2.0 * math.pi, size=k))
            gaps = np.diff(np.concatenate([ang, ang[:1] + 2.0 * math.pi]))
            if gaps.min() > 0.25 and gaps.max() < math.pi:
                break
        r = rng.uniform(0.3, 0.6)
        sh["count"][i] = k
        sh["vertices"][i, :k, 0] = (r * np.cos(ang)).astype(F32)
        sh["vertices"][i, :k, 1] = (r * np.sin(ang)).astype(F32)
    f = abi.fixture_defs(n)
    f["density"] = F32(1.0)
    f["friction"] = rng.uniform(0.2, 0.8, size=n).astype(F32)
    s = _empty()
    s["bodies"] = b
    s["fixture_body"] = np.arange(n, dtype=np.int32)
    s["shapes"] = sh
    s["fixtures"] = f
    height = max(height, y_base + rows * spacing + 4.0)
    out = _concat([container(width, height), s])
    out["name"] = "scatter%d" % n
    return out


def scatter_world(n=16384, seed=1, width=200.0, height=400.0):
    """Single large world: n mixed bodies in a 200 m x 400 m container."""
    return scatter(n, width, height, np.random.default_rng(seed))


def stacks(n, height, spacing=2.0, box=0.5):
    cols = (n + height - 1) // height
    centers = []
    x0 = -(cols - 1) * spacing / 2.0
    for i in range(n):
        c, r = divmod(i, height)
        centers.append((x0 + c * spacing, box + r * (2 * box)))
    g = ground_box(hx=max(50.0, cols * spacing), hy=10.0)
    s = _concat([g, _boxes(centers, box, box, abi.DYNAMIC, 0.6, 1.0)])
    s["name"] = "stacks%dx%d" % (cols, height)
    return s


def chains(n_chains=4, links=32, hx=0.125, hy=0.025, x0=-12.0, spacing=6.0, y=12.0, pile=True):
    """Revolute-joint chains (b2RevoluteJointDef, joints/b2revolutejoint.d:30-110): each chain
    is `links` boxes of half-extents hx x hy laid out horizontally from a static post and
    joined end to end; odd chains limit their joints to +-0.5 rad, every third chain drives
    its first joint with a motor.  Optional box stacks on the ground below."""
    parts = [ground_box()]
    if pile:
        parts.append(stacks(4 * n_chains, 4, spacing=spacing / 2.0))
    for c in range(n_chains):
        x = x0 + c * spacing
        post = _boxes([(x, y)], 0.1, 0.1, abi.STATIC)
        chain = _boxes([(x + hx + 2 * hx * i, y) for i in range(links)], hx, hy, abi.DYNAMIC, 0.4, 20.0)
        part = _concat([post, chain])
        j = np.zeros(links, abi.REVOLUTE_DEF)
        for i in range(links):
            j[i]["body_a"] = i               # the post for i = 0, else link i-1
            j[i]["body_b"] = i + 1
            j[i]["local_anchor_a"] = (0.0, 0.0) if i == 0 else (hx, 0.0)
            j[i]["local_anchor_b"] = (-hx, 0.0)
            if c % 2 == 1:
                j[i]["enable_limit"] = 1
                j[i]["lower_angle"] = -0.5
                j[i]["upper_angle"] = 0.5
        if c % 3 == 0:
            j[0]["enable_motor"] = 1
            j[0]["motor_speed"] = 1.0
            j[0]["max_motor_torque"] = 50.0
        part["joints"] = j
        parts.append(part)
    out = _concat(parts)
    out["name"] = "chains"
    return out


def ropes(n_ropes=4, links=20, box=0.1, gap=0.3, x0=-9.0, spacing=6.0, y=14.0, pile=True, revolute=True):
    """Distance-joint ropes (b2DistanceJointDef, joints/b2distancejoint.d:33-93): each rope is
    `links` small boxes hanging in a horizontal line from a static post, consecutive boxes
    joined by a distance joint of length `gap` between their centres (the first from the
    post); even ropes are rigid, odd ropes soft (4 Hz, damping ratio 0.5), and the last
    link of every third rope is tied back to the post by a long soft joint.  With `revolute`,
    a revolute chain hangs beside them (the revolute joints are created first), and box
    stacks stand on the ground below when `pile` is set."""
    parts = [ground_box()]
    if pile:
        parts.append(stacks(4 * n_ropes, 3, spacing=spacing / 2.0))
    if revolute:
        c = chains(n_chains=1, links=12, x0=x0 + n_ropes * spacing, y=y, pile=False)
        parts.append({k: c[k] for k in ("bodies", "fixture_body", "shapes", "fixtures", "joints")})
    for r in range(n_ropes):
        x = x0 + r * spacing
        post = _boxes([(x, y)], 0.1, 0.1, abi.STATIC)
        rope = _boxes([(x + gap * (i + 1), y) for i in range(links)], box, box, abi.DYNAMIC, 0.4, 5.0)
        part = _concat([post, rope])
        soft = r % 2 == 1
        tie = r % 3 == 0
        d = np.zeros(links + (1 if tie else 0), abi.DISTANCE_DEF)
        for i in range(links):
            d[i]["body_a"] = i               # the post for i = 0, else link i-1
            d[i]["body_b"] = i + 1
            d[i]["length"] = gap
            if soft:
                d[i]["frequency_hz"] = 4.0
                d[i]["damping_ratio"] = 0.5
        if tie:
            d[links]["body_a"] = 0
            d[links]["body_b"] = links
            d[links]["local_anchor_b"] = (box, 0.0)
            d[links]["length"] = gap * links * 0.7
            d[links]["frequency_hz"] = 1.5
            d[links]["damping_ratio"] = 0.2
        part["distance_joints"] = d
        parts.append(part)
    out = _concat(parts)
    out["name"] = "ropes"
    return out


def welded(n_beams=3, links=8, hx=0.3, hy=0.08, x0=-8.0, spacing=6.0, y=10.0, pile=True):
    """Weld and rope joints (b2WeldJointDef joints/b2weldjoint.d:30-86, b2RopeJointDef
    joints/b2ropejoint.d:30-52): each beam is `links` boxes welded end to end and to a
    static post (rigid welds on even beams, angularly soft welds, 3 Hz, on odd beams); a
    rope of maximum length 1.5 m ties the free end of each beam to a box hanging below it,
    and a second, taut rope ties that box to a point on the ground below it.  Box stacks stand below when `pile` is set."""
    parts = [ground_box()]
    if pile:
        parts.append(stacks(3 * n_beams, 3, spacing=spacing / 2.0))
    for b in range(n_beams):
        x = x0 + b * spacing
        post = _boxes([(x, y)], 0.2, 0.2, abi.STATIC)
        beam = _boxes([(x + 0.2 + hx + 2 * hx * i, y) for i in range(links)], hx, hy, abi.DYNAMIC, 0.5, 2.0)
        weight = _boxes([(x + 0.2 + 2 * hx * links, y - 1.2)], 0.25, 0.25, abi.DYNAMIC, 0.5, 1.0)
        part = _concat([post, beam, weight])
        soft = b % 2 == 1
        wj = np.zeros(links, abi.WELD_DEF)
        for i in range(links):
            wj[i]["body_a"] = i                      # the post for i = 0, else beam link i-1
            wj[i]["body_b"] = i + 1
            wj[i]["local_anchor_a"] = (0.2, 0.0) if i == 0 else (hx, 0.0)
            wj[i]["local_anchor_b"] = (-hx, 0.0)
            if soft:
                wj[i]["frequency_hz"] = 3.0
                wj[i]["damping_ratio"] = 0.4
        rj = np.zeros(1, abi.ROPE_DEF)
        rj[0]["body_a"] = links                      # the last beam link
        rj[0]["body_b"] = links + 1                  # the weight
        rj[0]["local_anchor_a"] = (hx, 0.0)
        rj[0]["max_length"] = 1.5
        part["weld_joints"] = wj
        part["rope_joints"] = rj
        parts.append(part)
    out = _concat(parts)
    # ropes from each weight to the ground body (body 0)
    weights = np.nonzero(np.isclose(out["bodies"]["position"][:, 1], y - 1.2))[0]
    extra = np.zeros(len(weights), abi.ROPE_DEF)
    for k, wi in enumerate(weights):
        extra[k]["body_a"] = 0
        extra[k]["body_b"] = wi
        extra[k]["local_anchor_a"] = (float(out["bodies"]["position"][wi, 0]), 10.0)
        extra[k]["max_length"] = (y - 1.2) - 0.8        # taut: pulls the weight 0.8 m down
    out["rope_joints"] = np.concatenate([out["rope_joints"], extra])
    out["name"] = "welded"
    return out


def top_down(n=12, seed=5, width=16.0):
    """Zero-gravity table top (the reference testbed's top-down use of b2FrictionJoint,
    joints/b2frictionjoint.d:30-73, and b2MotorJoint, joints/b2motorjoint.d:30-80): boxes and
    circles with a friction joint each to a static table body (max force ~ mass, max torque ~
    mass), pushed by their initial velocities; two platforms are driven by motor joints
    towards offsets from the table (one rotated, one translated) and push the others."""
    rng = np.random.default_rng(seed)
    table = _boxes([(0.0, 0.0)], 0.5, 0.5, abi.STATIC)
    walls = container(width, width, thick=0.5)
    walls["bodies"]["position"][:, 1] -= width / 2.0
    items = []
    for i in range(n):
        x, y = rng.uniform(-width / 2 + 1.5, width / 2 - 1.5, 2)
        items.append(_boxes([(x, y)], 0.4, 0.3, abi.DYNAMIC, 0.3, 1.0))
    platforms = _boxes([(-3.0, -4.0), (3.0, 4.0)], 1.2, 0.2, abi.DYNAMIC, 0.3, 2.0)
    out = _concat([table, walls] + items + [platforms])
    out["gravity"] = (0.0, 0.0)
    nb = len(out["bodies"])
    dyn = np.nonzero(out["bodies"]["type"] == abi.DYNAMIC)[0]
    out["bodies"]["linear_velocity"][dyn] = rng.normal(0.0, 3.0, (len(dyn), 2))
    out["bodies"]["angular_velocity"][dyn] = rng.normal(0.0, 2.0, len(dyn))
    fj = np.zeros(len(dyn) - 2, abi.FRICTION_DEF)
    for k, b in enumerate(dyn[:-2]):
        fj[k]["body_a"] = 0                      # the table
        fj[k]["body_b"] = b
        fj[k]["collide_connected"] = 1
        fj[k]["max_force"] = 0.12 * 10.0 * 0.48   # mu * g * mass of a 0.8 x 0.6 box, density 1
        fj[k]["max_torque"] = 0.12 * 10.0 * 0.48 * 0.3
    mj = np.zeros(2, abi.MOTOR_DEF)
    for k, b in enumerate(dyn[-2:]):
        mj[k]["body_a"] = 0
        mj[k]["body_b"] = b
        mj[k]["collide_connected"] = 1
        mj[k]["linear_offset"] = (-2.0, 1.0) if k == 0 else (4.0, -3.0)
        mj[k]["angular_offset"] = 1.2 if k == 0 else 0.0
        mj[k]["max_force"] = 40.0
        mj[k]["max_torque"] = 20.0
        mj[k]["correction_factor"] = 0.3
    out["friction_joints"] = fj
    out["motor_joints"] = mj
    out["name"] = "top_down"
    assert nb == len(out["bodies"])
    return out


def cars(n_cars=3, x0=-20.0, spacing=8.0, bumps=12, seed=7):
    """Wheel joints (b2WheelJointDef, joints/b2wheeljoint.d:30-99): cars with a box chassis
    and two circle wheels on spring suspensions (4 Hz, damping ratio 0.7, vertical axis), the
    rear wheel driven by a motor (max torque 20, speed -10 rad/s; every other car without a
    motor), driving over small box bumps on the ground."""
    rng = np.random.default_rng(seed)
    parts = [ground_box(hx=80.0)]
    parts.append(_boxes([(float(x), 0.1) for x in rng.uniform(-15.0, 35.0, bumps)], 0.4, 0.1, abi.STATIC, 0.8))
    for c in range(n_cars):
        x = x0 + c * spacing
        chassis = _boxes([(x, 1.0)], 1.5, 0.25, abi.DYNAMIC, 0.6, 1.0)
        wheels = _boxes([(x - 1.0, 0.4), (x + 1.0, 0.4)], 0.4, 0.4, abi.DYNAMIC, 0.9, 1.0)
        wheels["shapes"]["kind"] = abi.SHAPE_CIRCLE
        wheels["shapes"]["radius"] = 0.4
        part = _concat([chassis, wheels])
        wj = np.zeros(2, abi.WHEEL_DEF)
        for k in range(2):
            wj[k]["body_a"] = 0
            wj[k]["body_b"] = 1 + k
            wj[k]["local_anchor_a"] = (-1.0 if k == 0 else 1.0, -0.6)
            wj[k]["local_axis_a"] = (0.0, 1.0)
            wj[k]["frequency_hz"] = 4.0
            wj[k]["damping_ratio"] = 0.7
        if c % 2 == 0:
            wj[0]["enable_motor"] = 1
            wj[0]["max_motor_torque"] = 20.0
            wj[0]["motor_speed"] = -10.0
        part["wheel_joints"] = wj
        parts.append(part)
    out = _concat(parts)
    out["name"] = "cars"
    return out


def sliders(n=4, x0=-12.0, spacing=7.0, boxes=5):
    """Prismatic joints (b2PrismaticJointDef, joints/b2prismaticjoint.d:30-158): platforms on
    axes to the ground body, each loaded with a small stack of boxes.  Platform k: vertical
    axis with a motor (k even: lifting at 1 m/s, max force 400) and translation limits
    [-0.5, 3]; odd platforms slide on a tilted axis (30 degrees) with limits [-2, 2] and no
    motor; the last platform has equal limits (locked) and a reference angle of 0.1 rad."""
    parts = [ground_box()]
    for k in range(n):
        x = x0 + k * spacing
        plat = _boxes([(x, 2.0)], 1.5, 0.2, abi.DYNAMIC, 0.6, 2.0)
        load = _boxes([(x, 2.7 + 0.5 * i) for i in range(boxes)], 0.25, 0.25, abi.DYNAMIC, 0.6, 1.0)
        parts.append(_concat([plat, load]))
    out = _concat(parts)
    pj = np.zeros(n, abi.PRISMATIC_DEF)
    for k in range(n):
        body = 1 + k * (boxes + 1)
        x = x0 + k * spacing
        pj[k]["body_a"] = 0
        pj[k]["body_b"] = body
        pj[k]["local_anchor_a"] = (x, 12.0)                       # (x, 2) in the world
        if k % 2 == 0:
            pj[k]["local_axis_a"] = (0.0, 2.0)                    # normalised on creation
            pj[k]["enable_motor"] = 1
            pj[k]["motor_speed"] = 1.0
            pj[k]["max_motor_force"] = 400.0
            pj[k]["enable_limit"] = 1
            pj[k]["lower_translation"] = -0.5
            pj[k]["upper_translation"] = 3.0
        else:
            pj[k]["local_axis_a"] = (0.8660254, 0.5)
            pj[k]["enable_limit"] = 1
            pj[k]["lower_translation"] = -2.0
            pj[k]["upper_translation"] = 2.0
        if k == n - 1:
            pj[k]["enable_motor"] = 0
            pj[k]["lower_translation"] = 0.5
            pj[k]["upper_translation"] = 0.5
            pj[k]["reference_angle"] = 0.1
    out["prismatic_joints"] = pj
    out["name"] = "sliders"
    return out


def pulleys(n=3, x0=-10.0, spacing=8.0):
    """Pulley and mouse joints (b2PulleyJointDef joints/b2pulleyjoint.d:30-97, b2MouseJointDef
    joints/b2mousejoint.d:28-58): pairs of boxes hanging from two ground anchors 10 m up, one
    side heavier (ratio 1, 1.5 and 2 for the three pulleys), so the heavy side sinks onto the
    ground; a mouse joint drags a box on the ground towards a target above it (max force 200,
    5 Hz, damping 0.7)."""
    parts = [ground_box()]
    for k in range(n):
        x = x0 + k * spacing
        parts.append(_boxes([(x - 1.5, 5.0)], 0.5, 0.5, abi.DYNAMIC, 0.6, 1.0))
        parts.append(_boxes([(x + 1.5, 5.0)], 0.5, 0.5, abi.DYNAMIC, 0.6, 1.5 + 0.5 * k))
    parts.append(_boxes([(x0 + n * spacing, 0.5)], 0.4, 0.4, abi.DYNAMIC, 0.6, 1.0))
    out = _concat(parts)
    pj = np.zeros(n, abi.PULLEY_DEF)
    for k in range(n):
        x = x0 + k * spacing
        pj[k]["body_a"] = 1 + 2 * k
        pj[k]["body_b"] = 2 + 2 * k
        pj[k]["ground_anchor_a"] = (x - 1.5, 10.0)
        pj[k]["ground_anchor_b"] = (x + 1.5, 10.0)
        pj[k]["local_anchor_a"] = (0.0, 0.5)
        pj[k]["local_anchor_b"] = (0.0, 0.5)
        pj[k]["length_a"] = 4.5
        pj[k]["length_b"] = 4.5
        pj[k]["ratio"] = 1.0 + 0.5 * k
    mj = np.zeros(1, abi.MOUSE_DEF)
    mj[0]["body_a"] = 0
    mj[0]["body_b"] = 1 + 2 * n
    mj[0]["target"] = (x0 + n * spacing + 0.2, 0.7)
    mj[0]["max_force"] = 200.0
    mj[0]["frequency_hz"] = 5.0
    mj[0]["damping_ratio"] = 0.7
    out["pulley_joints"] = pj
    out["mouse_joints"] = mj
    out["name"] = "pulleys"
    return out


def _circles(centers, radius, btype=abi.DYNAMIC, density=1.0, friction=0.6):
    s = _boxes(centers, radius, radius, btype, friction, density)
    s["shapes"]["kind"] = abi.SHAPE_CIRCLE
    s["shapes"]["radius"] = radius
    return s


def gears(boxes=12, seed=9):
    """Gear joints (b2GearJointDef, joints/b2gearjoint.d:30-168) over revolute and prismatic
    joints: two wheels on ground pivots geared by their radii (1 and 2, the small one driven
    by a motor); a motor-driven wheel geared to a plate sliding on a prismatic axis (a rack);
    a swinging arm on a ground pivot carrying
    two wheels geared to each other through pivots on the arm (the gear's C and D bodies are
    the dynamic arm); boxes dropped onto the machinery."""
    rng = np.random.default_rng(seed)
    parts = [ground_box()]
    parts.append(_circles([(-10.0, 8.0)], 1.0))                   # 1: small wheel
    parts.append(_circles([(-7.0, 8.0)], 2.0))                    # 2: large wheel
    parts.append(_circles([(2.0, 7.0)], 1.0))                     # 3: rack wheel
    parts.append(_boxes([(2.0, 5.5)], 3.0, 0.25, abi.DYNAMIC, 0.6, 1.0))   # 4: sliding plate
    parts.append(_boxes([(12.0, 9.0)], 3.0, 0.2, abi.DYNAMIC, 0.6, 1.0))   # 5: arm
    parts.append(_circles([(10.0, 9.0)], 0.8))                    # 6: arm wheel 1
    parts.append(_circles([(14.0, 9.0)], 0.6))                    # 7: arm wheel 2
    xs = rng.uniform(-12.0, 14.0, boxes)
    parts.append(_boxes([(float(x), 14.0 + 0.8 * i) for i, x in enumerate(xs)], 0.3, 0.3, abi.DYNAMIC, 0.6, 1.0))
    out = _concat(parts)
    ground_y = -10.0
    rj = np.zeros(6, abi.REVOLUTE_DEF)
    for k, (b, x, y) in enumerate([(1, -10.0, 8.0), (2, -7.0, 8.0), (3, 2.0, 7.0), (5, 12.0, 9.0)]):
        rj[k]["body_a"], rj[k]["body_b"] = 0, b
        rj[k]["local_anchor_a"] = (x, y - ground_y)
    rj[0]["enable_motor"], rj[0]["motor_speed"], rj[0]["max_motor_torque"] = 1, 2.0, 500.0
    rj[2]["enable_motor"], rj[2]["motor_speed"], rj[2]["max_motor_torque"] = 1, -1.0, 300.0
    for k, (b, dx) in enumerate([(6, -2.0), (7, 2.0)]):          # wheels pinned to the arm
        rj[4 + k]["body_a"], rj[4 + k]["body_b"] = 5, b
        rj[4 + k]["local_anchor_a"] = (dx, 0.0)
    out["joints"] = rj
    pj = np.zeros(1, abi.PRISMATIC_DEF)
    pj[0]["body_a"], pj[0]["body_b"] = 0, 4
    pj[0]["local_anchor_a"] = (2.0, 5.5 - ground_y)
    pj[0]["local_axis_a"] = (1.0, 0.0)
    pj[0]["enable_limit"], pj[0]["lower_translation"], pj[0]["upper_translation"] = 1, -4.0, 4.0
    out["prismatic_joints"] = pj
    gj = np.zeros(3, abi.GEAR_DEF)
    gj[0]["body_a"], gj[0]["body_b"], gj[0]["joint1"], gj[0]["joint2"], gj[0]["ratio"] = 1, 2, 0, 1, 2.0   # r2 / r1
    gj[1]["body_a"], gj[1]["body_b"], gj[1]["joint1"], gj[1]["joint2"], gj[1]["ratio"] = 3, 4, 2, 6, -1.0
    gj[2]["body_a"], gj[2]["body_b"], gj[2]["joint1"], gj[2]["joint2"], gj[2]["ratio"] = 6, 7, 4, 5, 0.6 / 0.8
    out["gear_joints"] = gj
    out["name"] = "gears"
    return out


def _edges(points, ghosts=True, body_type=abi.STATIC, friction=0.6):
    """One body at the origin with an edge fixture per segment of the polyline `points`
    (b2EdgeShape, shapes/b2edgeshape.d); with `ghosts` each segment knows its neighbours
    (hasVertex0 / hasVertex3), as a chain's child edges do."""
    pts = np.asarray(points, F32)
    n = len(pts) - 1
    s = _empty()
    b = abi.body_defs(1)
    b["type"] = body_type
    s["bodies"] = b
    s["fixture_body"] = np.zeros(n, np.int32)
    sh = np.zeros(n, abi.SHAPE_DEF)
    sh["kind"] = abi.SHAPE_EDGE
    for i in range(n):
        sh["vertices"][i, 0] = pts[i]
        sh["vertices"][i, 1] = pts[i + 1]
        flags = 0
        if ghosts and i > 0:
            sh["vertices"][i, 2] = pts[i - 1]
            flags |= 1
        if ghosts and i + 1 < n:
            sh["vertices"][i, 3] = pts[i + 2]
            flags |= 2
        sh["count"][i] = flags
    s["shapes"] = sh
    fx = abi.fixture_defs(n)
    fx["friction"] = friction
    fx["density"] = 0.0
    s["fixtures"] = fx
    return s


def edge_ground(n=40, seed=13, pyramid_rows=6):
    """Edge shapes (b2EdgeShape, b2CollideEdgeAndCircle / b2EPCollider, collision/b2collideedge.d):
    a terrain of connected edges with ghost vertices (smooth collision across the joints),
    loose edges without neighbours, circles and convex polygons dropped onto it, a small box
    pyramid standing on a flat edge (the reference's pyramid demo uses an edge ground), and a
    dynamic body carrying an edge fixture next to its box (edges never touch edges)."""
    rng = np.random.default_rng(seed)
    xs = np.linspace(-30.0, 30.0, 25)
    ys = np.where(np.abs(xs) < 8.0, 0.0, 0.15 * (np.abs(xs) - 8.0) + 0.4 * np.sin(xs))
    parts = [_edges(np.stack([xs, ys], 1))]
    parts.append(_edges([(-12.0, 6.0), (-4.0, 4.0)], ghosts=False))                 # a loose ramp
    parts.append(_edges([(4.0, 4.0), (12.0, 6.0)], ghosts=False))
    if pyramid_rows:
        pyr = pyramid(rows=pyramid_rows, ground=False)
        pyr["bodies"]["position"][:, 1] -= 0.25                         # resting on y = 0
        parts.append(pyr)
    k = n // 2
    circ = _boxes([(float(x), 10.0 + float(y)) for x, y in zip(rng.uniform(-25.0, 25.0, k), rng.uniform(0.0, 8.0, k))],
                  0.3, 0.3, abi.DYNAMIC, 0.5, 1.0)
    circ["shapes"]["kind"] = abi.SHAPE_CIRCLE
    circ["shapes"]["radius"] = rng.uniform(0.2, 0.5, k).astype(F32)
    parts.append(circ)
    polys = _boxes([(float(x), 12.0 + float(y)) for x, y in zip(rng.uniform(-25.0, 25.0, n - k), rng.uniform(0.0, 8.0, n - k))],
                   0.3, 0.3, abi.DYNAMIC, 0.5, 1.0)
    polys["shapes"]["kind"] = abi.SHAPE_POLYGON
    for i in range(n - k):
        m = int(rng.integers(3, 9))
        ang = np.sort(rng.uniform(0.0, 2.0 * np.pi, m))
        r = rng.uniform(0.3, 0.6)
        polys["shapes"]["count"][i] = m
        polys["shapes"]["vertices"][i, :m, 0] = r * np.cos(ang)
        polys["shapes"]["vertices"][i, :m, 1] = r * np.sin(ang)
    parts.append(polys)
    carrier = _boxes([(20.0, 3.0)], 0.5, 0.25, abi.DYNAMIC, 0.5, 1.0)   # box + an edge fixture below it
    e = _edges([(-0.6, -0.4), (0.6, -0.4)], ghosts=False)
    carrier["fixture_body"] = np.concatenate([carrier["fixture_body"], np.zeros(1, np.int32)])
    carrier["shapes"] = np.concatenate([carrier["shapes"], e["shapes"]])
    carrier["fixtures"] = np.concatenate([carrier["fixtures"], e["fixtures"]])
    parts.append(carrier)
    out = _concat(parts)
    out["name"] = "edge_ground"
    return out


def chain_ground(n=40, seed=17):
    """Chain shapes (b2ChainShape, collision/shapes/b2chainshape.d, created as their child
    edges): a closed loop (CreateLoop) forming an irregular bowl, an open chain (CreateChain)
    with SetPrevVertex / SetNextVertex ghosts across a valley, a second open chain without
    ghosts, and circles and convex polygons dropped into them; a dynamic box carries a
    small loop chain (no mass of its own).  Chains are created after the scene's fixtures,
    in list order."""
    rng = np.random.default_rng(seed)
    ground = abi.body_defs(2)
    ground["type"] = abi.STATIC
    ground["position"][1] = (0.0, 0.5)
    base = _empty()
    base["bodies"] = ground
    ang = np.linspace(np.pi * 1.05, np.pi * 1.95, 18)
    bowl = np.concatenate([np.stack([14.0 * np.cos(ang), 10.0 + 8.0 * np.sin(ang) + 0.3 * np.sin(5 * ang)], 1),
                           [(12.0, 14.0), (-12.0, 14.0)]])
    xs = np.linspace(-34.0, -16.0, 12)
    valley = np.stack([xs, 4.0 + 0.05 * (xs + 25.0) ** 2 - 3.0], 1)
    base["chains"] = [
        dict(body=0, vertices=bowl.astype(F32), loop=True, prev=None, next=None, friction=0.6),
        dict(body=0, vertices=valley.astype(F32), loop=False, prev=(-36.0, 9.0), next=(-14.0, 9.0), friction=0.4),
        dict(body=1, vertices=np.array([(16.0, 0.0), (22.0, 1.5), (30.0, 1.0)], F32), loop=False, prev=None,
             next=None, friction=0.6),
    ]
    parts = [base]
    k = n // 2
    circ = _boxes([(float(x), 9.0 + float(y)) for x, y in zip(rng.uniform(-10.0, 10.0, k), rng.uniform(0.0, 4.0, k))],
                  0.3, 0.3, abi.DYNAMIC, 0.5, 1.0)
    circ["shapes"]["kind"] = abi.SHAPE_CIRCLE
    circ["shapes"]["radius"] = rng.uniform(0.2, 0.5, k).astype(F32)
    parts.append(circ)
    m = n - k
    polys = _boxes([(float(x), 12.0 + float(y)) for x, y in zip(
        np.concatenate([rng.uniform(-9.0, 9.0, m - 6), rng.uniform(-30.0, -20.0, 3), rng.uniform(18.0, 28.0, 3)]),
        rng.uniform(0.0, 4.0, m))], 0.3, 0.3, abi.DYNAMIC, 0.5, 1.0)
    polys["shapes"]["kind"] = abi.SHAPE_POLYGON
    for i in range(m):
        c = int(rng.integers(3, 9))
        a = np.sort(rng.uniform(0.0, 2.0 * np.pi, c))
        r = rng.uniform(0.3, 0.6)
        polys["shapes"]["count"][i] = c
        polys["shapes"]["vertices"][i, :c, 0] = r * np.cos(a)
        polys["shapes"]["vertices"][i, :c, 1] = r * np.sin(a)
    parts.append(polys)
    carrier = _boxes([(0.0, 20.0)], 0.5, 0.5, abi.DYNAMIC, 0.5, 1.0)
    carrier["chains"] = [dict(body=0, vertices=np.array([(-0.8, -0.8), (0.8, -0.8), (0.8, 0.8), (-0.8, 0.8)], F32),
                              loop=True, prev=None, next=None, friction=0.5)]
    parts.append(carrier)
    out = _concat(parts)
    out["name"] = "chain_ground"
    return out


def features(seed=23):
    """The less common parts of a step in one world: sensor fixtures (a static sensor region
    and a sensor beside a solid fixture on one dynamic body: b2Contact.Update's sensor branch,
    contacts/b2contact.d:283-296); a bullet circle fired into a box stack and a fast non-bullet
    box flying at a thin static wall (b2World.SolveTOI with bullets and static bodies,
    b2world.d:1172-1188); a kinematic platform sliding and turning through boxes; collision
    filtering (b2ContactFilter.ShouldCollide, b2worldcallbacks.d:52-64): a negative group that
    overlaps itself, a positive group, and category / mask pairs that skip each other; a bouncy
    ball (restitution), damped bodies, a body with gravity scale 0.5 and a fixed-rotation box."""
    rng = np.random.default_rng(seed)
    parts = [ground_box(hx=60.0)]                                          # 0: ground
    parts.append(_boxes([(30.0, 4.0)], 0.1, 4.0, abi.STATIC))              # 1: thin wall
    sensor = _boxes([(-20.0, 3.0)], 3.0, 3.0, abi.STATIC)                  # 2: sensor region
    sensor["fixtures"]["is_sensor"] = 1
    parts.append(sensor)
    stack = _boxes([(18.0, 0.5 + k) for k in range(6)], 0.5, 0.5, abi.DYNAMIC, 0.5, 1.0)   # 3..8
    parts.append(stack)
    bullet = _circles([(-5.0, 2.5)], 0.1, abi.DYNAMIC, 4.0, 0.3)           # 9: bullet
    bullet["bodies"]["bullet"] = 1
    bullet["bodies"]["linear_velocity"] = (150.0, 0.0)
    parts.append(bullet)
    fast = _boxes([(0.0, 5.0)], 0.15, 0.15, abi.DYNAMIC, 0.4, 1.0)         # 10: fast, not a bullet
    fast["bodies"]["linear_velocity"] = (120.0, 4.0)
    fast["bodies"]["angular_velocity"] = 3.0
    parts.append(fast)
    plat = _boxes([(-32.0, 1.2)], 3.0, 0.25, abi.KINEMATIC)                # 11: kinematic platform
    plat["bodies"]["linear_velocity"] = (1.5, 0.0)
    plat["bodies"]["angular_velocity"] = 0.15
    parts.append(plat)
    riders = _boxes([(-33.5 + 1.1 * k, 2.2) for k in range(4)], 0.4, 0.4, abi.DYNAMIC, 0.6, 1.0)   # 12..15
    parts.append(riders)
    # falling through the sensor region: circles and boxes
    xs = rng.uniform(-22.5, -17.5, 8)
    fall = _concat([_circles([(float(x), 8.0 + 1.2 * k)], 0.3) for k, x in enumerate(xs[:4])] +
                   [_boxes([(float(x), 13.0 + 1.2 * k)], 0.3, 0.3, abi.DYNAMIC) for k, x in enumerate(xs[4:])])
    parts.append(fall)                                                      # 16..23
    # two-fixture body: a solid box and a sensor circle around it
    two = _boxes([(-14.0, 6.0)], 0.5, 0.5, abi.DYNAMIC, 0.6, 1.0)          # 24
    sc = np.zeros(1, abi.SHAPE_DEF)
    sc["kind"] = abi.SHAPE_CIRCLE
    sc["radius"] = 1.5
    sf = abi.fixture_defs(1)
    sf["is_sensor"] = 1
    sf["density"] = 0.0
    two["shapes"] = np.concatenate([two["shapes"], sc])
    two["fixtures"] = np.concatenate([two["fixtures"], sf])
    two["fixture_body"] = np.array([0, 0], np.int32)
    parts.append(two)
    # filtering: a negative group stacked into itself (its members never collide with each other)
    neg = _boxes([(-8.0, 1.0), (-7.7, 1.5), (-8.2, 2.0), (-7.9, 2.6)], 0.5, 0.5, abi.DYNAMIC)   # 25..28
    neg["fixtures"]["group_index"] = -3
    parts.append(neg)
    pos = _boxes([(-3.0, 0.5), (-3.0, 1.5), (-3.0, 2.5)], 0.5, 0.5, abi.DYNAMIC)               # 29..31
    pos["fixtures"]["group_index"] = 2
    pos["fixtures"]["category_bits"] = 0x0002
    pos["fixtures"]["mask_bits"] = 0x0001                                  # ground only, but the group wins
    parts.append(pos)
    cat_a = _boxes([(4.0, 0.5), (4.2, 1.5)], 0.5, 0.5, abi.DYNAMIC)       # 32..33: category 4
    cat_a["fixtures"]["category_bits"] = 0x0004
    cat_a["fixtures"]["mask_bits"] = 0xFFFF & ~0x0008
    parts.append(cat_a)
    cat_b = _boxes([(4.1, 2.6), (4.3, 3.7)], 0.5, 0.5, abi.DYNAMIC)       # 34..35: category 8, skips 4
    cat_b["fixtures"]["category_bits"] = 0x0008
    cat_b["fixtures"]["mask_bits"] = 0xFFFF & ~0x0004
    parts.append(cat_b)
    ball = _circles([(10.0, 6.0)], 0.4)                                     # 36: restitution 0.8
    ball["fixtures"]["restitution"] = 0.8
    parts.append(ball)
    damped = _boxes([(12.0, 3.0), (13.5, 3.0)], 0.4, 0.4, abi.DYNAMIC)    # 37..38
    damped["bodies"]["linear_damping"] = 0.5
    damped["bodies"]["angular_damping"] = 0.8
    damped["bodies"]["angular_velocity"] = (4.0, -4.0)
    parts.append(damped)
    light = _boxes([(15.0, 6.0)], 0.4, 0.4, abi.DYNAMIC)                    # 39: gravity scale 0.5
    light["bodies"]["gravity_scale"] = 0.5
    parts.append(light)
    fixed = _boxes([(7.0, 4.0)], 0.6, 0.3, abi.DYNAMIC)                     # 40: fixed rotation
    fixed["bodies"]["fixed_rotation"] = 1
    fixed["bodies"]["angular_velocity"] = 2.0
    parts.append(fixed)
    out = _concat(parts)
    out["name"] = "features"
    return out


def _hanging_chain(x, y, links, hx=0.125, hy=0.025):
    """A static post at (x, y) and `links` boxes of half-extents hx x hy hanging straight down
    from it, joined end to end by revolute joints (link density 20, friction 0.4)."""
    post = _boxes([(x, y)], 0.1, 0.1, abi.STATIC)
    chain = _boxes([(x, y - hx - 2 * hx * i) for i in range(links)], hy, hx, abi.DYNAMIC, 0.4, 20.0)
    part = _concat([post, chain])
    j = np.zeros(links, abi.REVOLUTE_DEF)
    for i in range(links):
        j[i]["body_a"] = i                   # the post for i = 0, else link i-1
        j[i]["body_b"] = i + 1
        j[i]["local_anchor_a"] = (0.0, 0.0) if i == 0 else (0.0, -hx)
        j[i]["local_anchor_b"] = (0.0, hx)
    part["joints"] = j
    return part


def stress(piles=64, per_pile=2048, chains_per_pile=4, links=32, width=40.0, seed=5, gap=4.0):
    """Large-island stress world: `piles` separate containers (width x tall enough for the grid)
    side by side, each filled with `per_pile` mixed circles / polygons drawn as in scatter (they
    fall into one pile, one large island per container), and `chains_per_pile` revolute-joint
    chains of `links` 0.25 x 0.05 m box links hanging from static posts over each container into
    its pile.  The default sizes are 64 piles x 2,048 bodies and 256 chains x 32 links."""
    rng = np.random.default_rng(seed)
    parts = []
    for k in range(piles):
        pile = scatter(per_pile, width, 0.0, rng)
        height = float(pile["bodies"]["position"][:, 1].max()) + 2.0
        dx = k * (width + 2.0 + gap)
        pile["bodies"]["position"][:, 0] += F32(dx)
        parts.append(pile)
        for c in range(chains_per_pile):
            x = dx - width / 2.0 + width * (c + 1) / (chains_per_pile + 1)
            parts.append(_hanging_chain(x, height + 2.0 * 0.125 * links + 1.0, links))
    out = _concat(parts)
    out["name"] = "stress%dx%d" % (piles, per_pile)
    return out


def _shifted(scene, dx):
    """The scene moved by dx along x (bodies, pulley ground anchors, mouse targets)."""
    out = dict(scene)
    out["bodies"] = scene["bodies"].copy()
    out["bodies"]["position"][:, 0] += F32(dx)
    for key, fields in (("pulley_joints", ("ground_anchor_a", "ground_anchor_b")), ("mouse_joints", ("target",))):
        d = scene.get(key)
        if d is not None and len(d):
            d = d.copy()
            for f in fields:
                d[f][:, 0] += F32(dx)
            out[key] = d
    return out


def large_mixed(seed=11, n=4000):
    """One world of over 4,096 fixtures holding every joint scene side by side, 110 m apart
    (revolute chains, distance ropes, welded beams, friction / motor joints of the table top,
    wheel-joint cars, prismatic sliders, pulleys and a mouse joint, gears, edge and chain
    grounds; under gravity), and a 60 m container of `n` scattered mixed bodies."""
    parts = [chains(), ropes(), welded(), top_down(), cars(), sliders(), pulleys(), gears(), edge_ground(),
             chain_ground()]
    parts = [_shifted(p, 110.0 * (k + 1)) for k, p in enumerate(parts)]
    rng = np.random.default_rng(seed)
    parts.append(_concat([container(60.0, 60.0), scatter(n, 58.0, 58.0, rng)]))
    out = _concat(parts)
    out["name"] = "large_mixed"
    return out


def batch(n_worlds=4096, seed=3, lo=8, hi=512):
    """Batched workload: per-world body counts log-uniform in [lo, hi]; thirds of
    pyramids, 40 m-container scatters and box stacks."""
    rng = np.random.default_rng(seed)
    counts = np.exp(rng.uniform(math.log(lo), math.log(hi), size=n_worlds)).astype(np.int64)
    worlds = []
    for w in range(n_worlds):
        n = int(counts[w])
        kind = w % 3
        if kind == 0:
            rows = int((math.sqrt(8 * n + 1) - 1) // 2)
            worlds.append(pyramid(rows=max(rows, 1)))
        elif kind == 1:
            worlds.append(scatter(n, 40.0, 40.0, rng))
        else:
            worlds.append(stacks(n, int(rng.integers(1, 31))))
    return worlds


def hello_world():
    """examples/hello_world/hello_world.d:31-103: ground box + one 1x1 box at y=4."""
    g = ground_box()
    b = _boxes([(0.0, 4.0)], 1.0, 1.0, abi.DYNAMIC, 0.3, 1.0)
    s = _concat([g, b])
    s["name"] = "hello_world"
    return s


def dynamic_body_count(scene):
    return int((scene["bodies"]["type"] == abi.DYNAMIC).sum())
