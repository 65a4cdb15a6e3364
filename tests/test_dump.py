"""b2World.Dump text (dynamics/b2world.d:796-855, b2body.d:992-1022, b2fixture.d:280-358, the
joints' Dump) and its replay: the oracle against a hand-written expectation of the reference's
format, dump -> replay round trips, the reference's own dumped test scene; the library's dump
against the oracle's, bit for bit."""
import json
import os

import numpy as np
import pytest

from dbox_gb300 import abi, dump, scenes
from compare import exact_diff

HERE = os.path.dirname(os.path.abspath(__file__))
Z = "0.000000000000000e+00f"


def _tiny_scene():
    s = scenes._empty()
    b = abi.body_defs(2)
    b["type"] = (abi.STATIC, abi.DYNAMIC)
    b["position"][1] = (1.0, 3.0)
    b["angle"][1] = 0.25
    s["bodies"] = b
    s["fixture_body"] = np.array([0, 1], np.int32)
    sh = np.zeros(2, abi.SHAPE_DEF)
    sh["kind"] = (abi.SHAPE_BOX, abi.SHAPE_CIRCLE)
    sh["hx"][0], sh["hy"][0] = 2.0, 0.5
    sh["radius"][1] = 0.5
    s["shapes"] = sh
    fx = abi.fixture_defs(2)
    fx["friction"][0] = 0.6
    fx["density"][1] = 1.0
    fx["group_index"][1] = -3
    s["fixtures"] = fx
    j = np.zeros(1, abi.REVOLUTE_DEF)
    j["body_a"], j["body_b"] = 0, 1
    j["local_anchor_a"] = (1.0, 3.0)
    j["enable_limit"] = 1
    j["lower_angle"], j["upper_angle"] = -0.5, 0.5
    s["joints"] = j
    return s


def _body(index, btype, pos, angle, awake):
    return [
        "{", "  b2BodyDef bd;", "  bd.type = b2BodyType(%d);" % btype,
        "  bd.position.Set(%s, %s);" % pos, "  bd.angle = %s;" % angle,
        "  bd.linearVelocity.Set(%s, %s);" % (Z, Z), "  bd.angularVelocity = %s;" % Z,
        "  bd.linearDamping = %s;" % Z, "  bd.angularDamping = %s;" % Z,
        "  bd.allowSleep = bool(4);", "  bd.awake = bool(%d);" % awake, "  bd.fixedRotation = bool(0);",
        "  bd.bullet = bool(0);", "  bd.active = bool(32);", "  bd.gravityScale = 1.000000000000000e+00f;",
        "  bodies[%d] = m_world.CreateBody(&bd);" % index, ""]


def _fixture_head(friction, density, group):
    return ["  {", "    b2FixtureDef fd;", "    fd.friction = %s;" % friction, "    fd.restitution = %s;" % Z,
            "    fd.density = %s;" % density, "    fd.isSensor = bool(0);",
            "    fd.filter.categoryBits = uint16(1);", "    fd.filter.maskBits = uint16(65535);",
            "    fd.filter.groupIndex = int16(%d);" % group]


def _fixture_tail(body):
    return ["", "    fd.shape = &shape;", "", "    bodies[%d].CreateFixture(&fd);" % body, "  }", "}"]


def test_dump_text_known_answer(oracle_lib):
    # the statements b2World.Dump logs for a static box and a dynamic circle joined by a
    # limited revolute joint, before any step: newest body first, %.15e floats with an 'f'
    # suffix, the body flags as their masked bit values
    want = ["b2Vec2 g(%s, -1.000000000000000e+01f);" % Z, "m_world.SetGravity(g);",
            "b2Body** bodies = cast(b2Body**)b2Alloc(2 * (b2Body*).sizeof);",
            "b2Joint joints = cast(b2Joint)b2Alloc(1 * (b2Joint).sizeof);"]
    want += _body(0, 2, ("1.000000000000000e+00f", "3.000000000000000e+00f"), "2.500000000000000e-01f", 2)
    want += _fixture_head("2.000000029802322e-01f", "1.000000000000000e+00f", -3)
    want += ["    b2CircleShape shape;", "    shape.m_radius = 5.000000000000000e-01f",
             "    shape.m_p.Set(%s, %s);" % (Z, Z)]
    want[-2] += ";"
    want += _fixture_tail(0)
    want += _body(1, 0, (Z, Z), Z, 2)
    want += _fixture_head("6.000000238418579e-01f", Z, 0)
    want += ["    b2PolygonShape shape;", "    b2Vec2 vs[8];",
             "    vs[0].Set(-2.000000000000000e+00f, -5.000000000000000e-01f);",
             "    vs[1].Set(2.000000000000000e+00f, -5.000000000000000e-01f);",
             "    vs[2].Set(2.000000000000000e+00f, 5.000000000000000e-01f);",
             "    vs[3].Set(-2.000000000000000e+00f, 5.000000000000000e-01f);", "    shape.Set(vs, 4);"]
    want += _fixture_tail(1)
    want += ["{", "  b2RevoluteJointDef jd;", "  jd.bodyA = bodies[1];", "  jd.bodyB = bodies[0];",
             "  jd.collideConnected = bool(0);",
             "  jd.localAnchorA.Set(1.000000000000000e+00f, 3.000000000000000e+00f);",
             "  jd.localAnchorB.Set(%s, %s);" % (Z, Z), "  jd.referenceAngle = %s;" % Z,
             "  jd.enableLimit = bool(1);", "  jd.lowerAngle = -5.000000000000000e-01f;",
             "  jd.upperAngle = 5.000000000000000e-01f;", "  jd.enableMotor = bool(0);",
             "  jd.motorSpeed = %s;" % Z, "  jd.maxMotorTorque = %s;" % Z,
             "  joints[0] = m_world.CreateJoint(&jd);", "}",
             "b2Free(joints);", "b2Free(bodies);", "joints = null;", "bodies = null;"]
    got = oracle_lib.OracleWorld(_tiny_scene()).dump()
    assert got == "\n".join(want) + "\n"


def _empty_oracle(oracle_lib, g):
    e = scenes._empty()
    e["gravity"] = g
    return oracle_lib.OracleWorld(e)


def _drop_velocity(text):
    return "\n".join(l for l in text.splitlines() if "bd.linearVelocity" not in l)


@pytest.mark.parametrize("name", ["ropes", "welded", "cars", "sliders", "pulleys", "top_down", "edge_ground",
                                  "chain_ground", "gears"])
def test_dump_replay_round_trip(oracle_lib, name):
    # dump -> parse -> replay reverses the list orders; twice restores them.  Replaying a dump
    # of a replayed world gives the same text again, except the linear velocity of bodies whose
    # centre of mass is off their origin: b2Body.ResetMassData adds w x (c - c_old) to it when
    # each fixture is created (b2body.d:548-549), in the reference too
    oracle_lib.set_trig_mode(1)
    s = dict(getattr(scenes, name)())
    s["mouse_joints"] = np.zeros(0, abi.MOUSE_DEF)
    w1 = oracle_lib.OracleWorld(s)
    w1.step(steps=20)
    t1 = w1.dump()
    p1 = dump.parse(t1)
    assert len(p1["bodies"]) == len(s["bodies"])
    n_chain_children = sum(len(c["vertices"]) - (0 if c["loop"] else 1) for c in s.get("chains", ()))
    assert len(p1["fixtures"]) == len(s["fixtures"]) + len(s.get("chains", ()))
    assert n_chain_children >= 0
    texts = [t1]
    for _ in range(3):
        w = _empty_oracle(oracle_lib, p1["gravity"])
        dump.replay(dump.parse(texts[-1]), w)
        texts.append(w.dump())
    centred = name not in ("edge_ground", "chain_ground")
    if centred:
        assert texts[1] == texts[3]
    else:
        assert _drop_velocity(texts[1]) == _drop_velocity(texts[3])
    # positions, angles and joint definitions survive the double round trip unchanged
    p3 = dump.parse(texts[2])
    for f in ("position", "angle", "angular_velocity", "type", "awake"):
        assert np.array_equal(p1["bodies"][f], p3["bodies"][f]), f
    assert [(k, d.tobytes(), i) for k, d, i in p1["joints"]] == [(k, d.tobytes(), i) for k, d, i in p3["joints"]]


def test_mouse_joint_dump_line(oracle_lib):
    w = oracle_lib.OracleWorld(scenes.pulleys())
    t = w.dump()
    assert "{\nMouse joint dumping is not supported.\n}\n" in t
    assert len(dump.parse(t)["joints"]) == len(scenes.pulleys()["pulley_joints"])


def dumpshell_scene():
    """The reference's DumpShell test scene (a dumped world, Box2D issue 304) as a scene dict."""
    d = json.load(open(os.path.join(HERE, "golden", "dumpshell_scene.json")))
    s = scenes._empty()
    s["gravity"] = tuple(d["gravity"])
    b = abi.body_defs(len(d["bodies"]))
    for i, body in enumerate(d["bodies"]):
        for k, v in body.items():
            b[i][k] = v
    s["bodies"] = b
    fx = d["fixtures"]
    s["fixture_body"] = np.array([f["body"] for f in fx], np.int32)
    sh = np.zeros(len(fx), abi.SHAPE_DEF)
    fd = abi.fixture_defs(len(fx))
    for i, f in enumerate(fx):
        sh[i]["kind"] = f["kind"]
        sh[i]["count"] = f["count"]
        sh[i]["vertices"][:f["count"]] = f["vertices"]
        for k in ("friction", "restitution", "density", "is_sensor", "category_bits", "mask_bits", "group_index"):
            fd[i][k] = f[k]
    s["shapes"] = sh
    s["fixtures"] = fd
    return s


def test_dumpshell_scene(oracle_lib):
    # the reference's own dumped test scene loads, its dump gives back the scene's positions
    # and angles, and it simulates: the small box comes to rest on the static polygon, the
    # long plank dropped on the polygon's narrow top tips off it
    oracle_lib.set_trig_mode(1)
    s = dumpshell_scene()
    ow = oracle_lib.OracleWorld(s)
    p = dump.parse(ow.dump())
    assert np.array_equal(p["bodies"]["position"][::-1], s["bodies"]["position"])
    assert np.array_equal(p["bodies"]["angle"][::-1], s["bodies"]["angle"])
    ow.step(steps=300)
    b = ow.export_state()["bodies"]
    assert np.isfinite(b["xf"]).all()
    assert np.abs(b["vel"][2]).max() < 1e-3 and 5.6 < b["xf"][2, 1] < 5.8
    assert b["xf"][1, 1] < 0.0


@pytest.mark.gpu
def test_dump_exact(oracle_lib, gpu_lib):
    # the library's dump of each world of a handle is the oracle's text, byte for byte, after
    # 60 steps (positions, angles, velocities, awake flags as the step left them)
    oracle_lib.set_trig_mode(1)
    groups = [[scenes.ropes(), scenes.welded(), scenes.cars(), scenes.sliders(), scenes.pulleys(), scenes.gears()],
              [scenes.top_down()], [scenes.edge_ground(), scenes.chain_ground(), dumpshell_scene()]]
    for worlds in groups:
        gw = gpu_lib.World(worlds)
        ows = [oracle_lib.OracleWorld(s) for s in worlds]
        assert [gw.dump(i) for i in range(len(worlds))] == [ow.dump() for ow in ows]
        gw.step(steps=60)
        for ow in ows:
            ow.step(steps=60)
        for i, ow in enumerate(ows):
            assert gw.dump(i) == ow.dump(), i


@pytest.mark.gpu
def test_dump_replay_exact(oracle_lib, gpu_lib):
    # a dump replayed into an empty world of the library and into the oracle gives the same
    # world: the same text, and bit-identical states over 120 further steps
    oracle_lib.set_trig_mode(1)
    for s in (scenes.ropes(), scenes.chain_ground(), scenes.sliders()):
        src = oracle_lib.OracleWorld(s)
        src.step(steps=30)
        p = dump.parse(src.dump())
        e = scenes._empty()
        e["gravity"] = p["gravity"]
        gw = gpu_lib.World([e])
        dump.replay(p, gw, 0)
        ow = _empty_oracle(oracle_lib, p["gravity"])
        dump.replay(p, ow)
        assert gw.dump(0) == ow.dump()
        for t in range(4):
            gw.step(steps=30)
            ow.step(steps=30)
            d = exact_diff(ow.export_state(), gw.export_state(0))
            assert not d, (t, d[:6])


def test_dump_after_destruction(oracle_lib):
    # destroyed bodies, fixtures and joints leave the world lists: the dump counts and indexes
    # only the live ones, and the text replays (twice round, the same text)
    oracle_lib.set_trig_mode(1)
    s = scenes._concat([scenes.pyramid(rows=5), scenes.chains(n_chains=1, links=6, pile=False), scenes.gears()])
    ow = oracle_lib.OracleWorld(s)
    ow.step(steps=30)
    nb, nj = len(s["bodies"]), sum(len(s[k]) for k in scenes.JOINT_KINDS)
    ow.destroy_body(2)
    ow.destroy_body(1 + 15 + 1 + 2)                    # a chain link with two joints
    ow.destroy_fixture(5)
    p = dump.parse(ow.dump())
    assert len(p["bodies"]) == nb - 2
    assert len(p["joints"]) == nj - 2
    texts = [ow.dump()]
    for _ in range(3):
        w = _empty_oracle(oracle_lib, p["gravity"])
        dump.replay(dump.parse(texts[-1]), w)
        texts.append(w.dump())
    assert _drop_velocity(dump_bodies_only(texts[0])).count("b2BodyDef bd;") == nb - 2
    # a replayed world's box vertices come back in b2PolygonShape.Set's hull order, so texts
    # of replayed worlds are compared
    assert _drop_velocity(dump_bodies_only(texts[1])) == _drop_velocity(dump_bodies_only(texts[3]))
    assert texts[1].count("JointDef jd;") == texts[3].count("JointDef jd;") == nj - 2


def dump_bodies_only(text):
    """The body and fixture statements of a dump (joint blocks left out)."""
    i = text.find("JointDef jd;")
    return text if i < 0 else text[:text.rfind("{\n", 0, i)]


def test_parse_hand_edited_loop_and_circle(oracle_lib):
    # testbed-style statements the reference's Dump never writes but scenes carry:
    # CreateLoop, `true` flags, a bare b2BodyType member, an `auto shape = new ...` circle
    text = """
    b2Vec2 g = b2Vec2(0.000000000000000e+00f, -1.000000000000000e+01f);
    m_world.SetGravity(g);
    {
        b2BodyDef bd;
        bodies[0] = m_world.CreateBody(&bd);
        {
            b2FixtureDef fd;
            fd.friction = 6.000000238418579e-01f;
            b2ChainShape shape;
            b2Vec2 vs[4];
            vs[0].Set(-5.0f, 0.0f);
            vs[1].Set(5.0f, 0.0f);
            vs[2].Set(5.0f, 10.0f);
            vs[3].Set(-5.0f, 10.0f);
            shape.CreateLoop(vs, 4);
            fd.shape = &shape;
            bodies[0].CreateFixture(&fd);
        }
    }
    {
        b2BodyDef bd;
        bd.type = b2BodyType.b2_dynamicBody;
        bd.position.Set(0.0f, 5.0f);
        bd.bullet = true;
        bodies[1] = m_world.CreateBody(&bd);
        {
            b2FixtureDef fd;
            fd.density = 2.0f;
            auto shape = new b2CircleShape();
            shape.m_radius = 5.000000000000000e-01f;
            fd.shape = shape;
            bodies[1].CreateFixture(&fd);
        }
    }
    """
    p = dump.parse(text)
    assert len(p["bodies"]) == 2 and p["bodies"]["type"][1] == abi.DYNAMIC and p["bodies"]["bullet"][1] == 1
    assert p["fixtures"][0][0] == "chain" and p["fixtures"][0][5] is True
    assert p["fixtures"][1][0] == "fixture" and p["fixtures"][1][2]["kind"] == abi.SHAPE_CIRCLE
    oracle_lib.set_trig_mode(1)
    ow = _empty_oracle(oracle_lib, p["gravity"])
    dump.replay(p, ow)
    ow.step(steps=120)
    st = ow.export_state()
    assert len(st["proxies"]) == 4 + 1                  # a loop of 4 vertices has 4 child edges
    assert 0.0 < st["bodies"]["xf"][1, 1] < 1.0         # the ball rests on the loop's floor
    t = ow.dump()
    assert "shape.CreateChain(vs, 5);" in t and "shape.m_hasPrevVertex = bool(1);" in t
