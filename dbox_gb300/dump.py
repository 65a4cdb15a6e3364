"""Read b2World.Dump text back into creation calls (scenario exchange).

b2World.Dump (dynamics/b2world.d:796-855) logs statements that rebuild a world: a body
block per body (b2BodyDef fields, CreateBody, then one block per fixture with its
b2FixtureDef and shape), then one block per joint.  `parse` reads that text, and the
hand-edited variants of it that testbed scenes carry (``bd.awake = true;``,
``b2BodyType.b2_dynamicBody``, ``auto shape = new b2PolygonShape();``,
``shape.Set(vs[0 .. n]);``), into records of this package's ABI; `replay` makes the same
creation calls, in the same order, on a World handle or an oracle world.  Statements the
format does not use are ignored; a mouse joint is dumped as a "not supported" line and
is not replayed (the reference cannot replay it either).
"""
import re

import numpy as np

from . import abi

_NUM = r"[-+0-9.eEinfa]+f?"
_BODY_TYPES = {"b2_staticBody": 0, "b2_kinematicBody": 1, "b2_dynamicBody": 2}
_JOINT_KINDS = {"Revolute": "revolute", "Distance": "distance", "Rope": "rope", "Weld": "weld",
                "Friction": "friction", "Motor": "motor", "Wheel": "wheel", "Prismatic": "prismatic",
                "Pulley": "pulley", "Gear": "gear"}
_JOINT_DEFS = {"revolute": abi.REVOLUTE_DEF, "distance": abi.DISTANCE_DEF, "rope": abi.ROPE_DEF,
               "weld": abi.WELD_DEF, "friction": abi.FRICTION_DEF, "motor": abi.MOTOR_DEF,
               "wheel": abi.WHEEL_DEF, "prismatic": abi.PRISMATIC_DEF, "pulley": abi.PULLEY_DEF,
               "gear": abi.GEAR_DEF}
_JOINT_FIELDS = {"maxLength": "max_length", "localAxisA": "local_axis_a"}


def _snake(name):
    return _JOINT_FIELDS.get(name) or re.sub(r"([A-Z])", lambda m: "_" + m.group(1).lower(), name)


def _value(text):
    """A scalar of the dump: float literal with an f suffix, bool(n), uint16(n), int16(n),
    b2BodyType(n) / b2BodyType.b2_*Body, true / false, or a plain integer."""
    t = text.strip()
    m = re.fullmatch(r"(?:bool|uint16|int16|b2BodyType)\((-?\d+)\)", t)
    if m:
        return int(m.group(1))
    m = re.fullmatch(r"b2BodyType\.(\w+)", t)
    if m:
        return _BODY_TYPES[m.group(1)]
    if t in ("true", "false"):
        return 1 if t == "true" else 0
    if t.endswith("f"):
        t = t[:-1]
    return np.float32(float(t))


def parse(text):
    """Parse dump text into {"gravity": (x, y), "bodies": BODY_DEF array, "fixtures": [ops],
    "joints": [(kind, record, dump index)]} where each fixture op is ("fixture", body, SHAPE_DEF record,
    FIXTURE_DEF record) or ("chain", body, vertices, prev or None, next or None,
    FIXTURE_DEF record), in the text's order."""
    gravity = (0.0, -10.0)
    bodies, fixtures, joints = [], [], []
    body = fd = shape = jd = None
    verts = {}
    for raw in text.splitlines():
        line = re.sub(r"\s+", "", raw)
        if not line or line.startswith("//"):
            continue
        m = re.fullmatch(r"b2Vec2g(?:=b2Vec2)?\((%s),(%s)\);" % (_NUM, _NUM), line)
        if m:
            gravity = (float(_value(m.group(1))), float(_value(m.group(2))))
            continue
        if line == "b2BodyDefbd;":
            body = abi.body_defs(1)[0]
            continue
        m = re.fullmatch(r"bd\.(\w+)\.Set\((%s),(%s)\);" % (_NUM, _NUM), line)
        if m and body is not None:
            body[_snake(m.group(1))] = (_value(m.group(2)), _value(m.group(3)))
            continue
        m = re.fullmatch(r"bd\.(\w+)=(.+);", line)
        if m and body is not None:
            v = _value(m.group(2))
            f = _snake(m.group(1))
            body[f] = (1 if v else 0) if f in ("allow_sleep", "awake", "fixed_rotation", "bullet", "active") else v
            continue
        m = re.fullmatch(r"bodies\[(\d+)\]=m_world\.CreateBody\(&bd\);", line)
        if m:
            assert int(m.group(1)) == len(bodies), "bodies out of order"
            bodies.append(body)
            body = None
            continue
        if line == "b2FixtureDeffd;":
            fd = abi.fixture_defs(1)[0]
            shape, verts = None, {}
            continue
        m = re.fullmatch(r"fd\.(?:filter\.)?(\w+)=(.+);", line)
        if m and fd is not None and m.group(1) != "shape":
            v = _value(m.group(2))
            f = _snake(m.group(1))
            fd[f] = (1 if v else 0) if f == "is_sensor" else v
            continue
        m = re.fullmatch(r"(?:b2(\w+)Shapeshape;|autoshape=newb2(\w+)Shape\(\);)", line)
        if m:
            shape = {"kind": m.group(1) or m.group(2)}
            continue
        m = re.fullmatch(r"vs\[(\d+)\]\.Set\((%s),(%s)\);" % (_NUM, _NUM), line)
        if m:
            verts[int(m.group(1))] = (_value(m.group(2)), _value(m.group(3)))
            continue
        m = re.fullmatch(r"shape\.(Set|CreateChain|CreateLoop)\(vs(?:,(\d+)|\[0\.\.(\d+)\])\);", line)
        if m and shape is not None:
            shape["count"] = int(m.group(2) or m.group(3))
            shape["loop"] = m.group(1) == "CreateLoop"
            continue
        m = re.fullmatch(r"shape\.(\w+)\.Set\((%s),(%s)\);" % (_NUM, _NUM), line)
        if m and shape is not None:
            shape[m.group(1)] = (_value(m.group(2)), _value(m.group(3)))
            continue
        m = re.fullmatch(r"shape\.(\w+)=(.+);", line)
        if m and shape is not None:
            shape[m.group(1)] = _value(m.group(2))
            continue
        m = re.fullmatch(r"bodies\[(\d+)\]\.CreateFixture\(&fd\);", line)
        if m:
            fixtures.append(_fixture_op(int(m.group(1)), shape, verts, fd))
            fd = shape = None
            continue
        m = re.fullmatch(r"b2(\w+)JointDefjd;", line)
        if m:
            kind = _JOINT_KINDS.get(m.group(1))
            jd = (kind, np.zeros(1, _JOINT_DEFS[kind])[0]) if kind else None
            continue
        m = re.fullmatch(r"jd\.joint([12])=joints\[(\d+)\];", line)
        if m and jd is not None:
            jd[1]["joint" + m.group(1)] = int(m.group(2))
            continue
        m = re.fullmatch(r"jd\.body([AB])=bodies\[(\d+)\];", line)
        if m and jd is not None:
            jd[1]["body_" + m.group(1).lower()] = int(m.group(2))
            continue
        m = re.fullmatch(r"jd\.(\w+)\.Set\((%s),(%s)\);" % (_NUM, _NUM), line)
        if m and jd is not None:
            jd[1][_snake(m.group(1))] = (_value(m.group(2)), _value(m.group(3)))
            continue
        m = re.fullmatch(r"jd\.(\w+)=(.+);", line)
        if m and jd is not None:
            jd[1][_snake(m.group(1))] = _value(m.group(2))
            continue
        m = re.fullmatch(r"joints\[(\d+)\]=m_world\.CreateJoint\(&jd\);", line)
        if m and jd is not None:
            joints.append((jd[0], jd[1], int(m.group(1))))
            jd = None
    out = abi.body_defs(len(bodies))
    for i, b in enumerate(bodies):
        out[i] = b
    return {"gravity": gravity, "bodies": out, "fixtures": fixtures, "joints": joints}


def _fixture_op(body, shape, verts, fd):
    kind = shape["kind"]
    vs = [verts[i] for i in range(shape.get("count", 0))]
    if kind == "Chain":
        prev = shape.get("m_prevVertex") if shape.get("m_hasPrevVertex") else None
        nxt = shape.get("m_nextVertex") if shape.get("m_hasNextVertex") else None
        return ("chain", body, np.array(vs, np.float32), prev, nxt, shape.get("loop", False), fd)
    sd = np.zeros(1, abi.SHAPE_DEF)[0]
    if kind == "Circle":
        sd["kind"] = abi.SHAPE_CIRCLE
        sd["radius"] = shape["m_radius"]
        sd["center"] = shape.get("m_p", (0.0, 0.0))
    elif kind == "Edge":
        sd["kind"] = abi.SHAPE_EDGE
        sd["vertices"][0] = shape["m_vertex1"]
        sd["vertices"][1] = shape["m_vertex2"]
        sd["vertices"][2] = shape.get("m_vertex0", (0.0, 0.0))
        sd["vertices"][3] = shape.get("m_vertex3", (0.0, 0.0))
        sd["count"] = (1 if shape.get("m_hasVertex0") else 0) | (2 if shape.get("m_hasVertex3") else 0)
    else:
        sd["kind"] = abi.SHAPE_POLYGON
        sd["count"] = len(vs)
        sd["vertices"][:len(vs)] = vs
    return ("fixture", body, sd, fd)


def replay(parsed, target, world=None):
    """Make the dump's creation calls on `target`: a World handle (then `world` names the world
    of the handle, which should be empty) or an oracle world (world None).  Returns the body
    indices created, in dump order."""
    args = () if world is None else (world,)
    base = [target.create_body(*args, b) for b in parsed["bodies"]]
    for op in parsed["fixtures"]:
        if op[0] == "fixture":
            target.create_fixture(*args, base[op[1]], op[2], op[3])
        else:
            _, b, vs, prev, nxt, loop, fd = op
            target.create_chain(*args, base[b], vs, loop, prev, nxt, fd)
    made = {}                                           # dump index -> joint created
    for kind, d, k in parsed["joints"]:
        d = d.copy()
        d["body_a"] = base[d["body_a"]]
        d["body_b"] = base[d["body_b"]]
        if kind == "gear":
            d["joint1"] = made[int(d["joint1"])]
            d["joint2"] = made[int(d["joint2"])]
        made[k] = target.create_joint(*args, kind, d)
    return base
