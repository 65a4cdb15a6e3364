"""World queries (b2World.QueryAABB / RayCast, dynamics/b2world.d:563-587): the oracle against
analytic answers and brute force on CPU; the device index against the oracle, bit for bit."""
import numpy as np
import pytest

from dbox_gb300 import abi, scenes
from compare import exact_diff


def _one_body_scene(kind, **kw):
    s = scenes._empty()
    b = abi.body_defs(1)
    b["type"] = abi.STATIC
    b["position"][0] = kw.get("pos", (0.0, 0.0))
    b["angle"][0] = kw.get("angle", 0.0)
    s["bodies"] = b
    s["fixture_body"] = np.zeros(1, np.int32)
    sh = np.zeros(1, abi.SHAPE_DEF)
    sh["kind"] = kind
    if kind == abi.SHAPE_CIRCLE:
        sh["radius"] = kw["radius"]
        sh["vertices"][0, 0] = kw.get("center", (0.0, 0.0))
    elif kind == abi.SHAPE_EDGE:
        sh["vertices"][0, 0] = kw["v1"]
        sh["vertices"][0, 1] = kw["v2"]
    else:
        hx, hy = kw["half"]
        sh["count"] = 4
        sh["vertices"][0, :4] = [(-hx, -hy), (hx, -hy), (hx, hy), (-hx, hy)]
    s["shapes"] = sh
    s["fixtures"] = abi.fixture_defs(1)
    return s


def test_raycast_known_answers(oracle_lib):
    # analytic hits: a box face, a circle, an edge from either side, a rotated box, a miss,
    # a ray starting inside a box (b2PolygonShape.RayCast reports no hit from inside)
    ow = oracle_lib.OracleWorld(_one_body_scene(abi.SHAPE_POLYGON, half=(0.5, 0.5)))
    h = ow.raycast((-5.0, 0.0), (5.0, 0.0), "closest")
    assert len(h) == 1 and h[0]["fixture"] == 0
    assert abs(h[0]["fraction"] - 0.45) < 1e-6 and np.allclose(h[0]["normal"], (-1.0, 0.0)) and np.allclose(h[0]["point"], (-0.5, 0.0))
    assert len(ow.raycast((0.0, 0.0), (5.0, 0.0), "all")) == 0
    assert len(ow.raycast((-5.0, 2.0), (5.0, 2.0), "all")) == 0
    ow = oracle_lib.OracleWorld(_one_body_scene(abi.SHAPE_CIRCLE, radius=1.0, pos=(3.0, 0.0)))
    h = ow.raycast((0.0, 0.0), (10.0, 0.0), "closest")
    assert len(h) == 1 and abs(h[0]["fraction"] - 0.2) < 1e-6 and np.allclose(h[0]["normal"], (-1.0, 0.0))
    ow = oracle_lib.OracleWorld(_one_body_scene(abi.SHAPE_EDGE, v1=(0.0, -1.0), v2=(0.0, 1.0)))
    h = ow.raycast((-2.0, 0.0), (2.0, 0.0), "closest")
    assert len(h) == 1 and abs(h[0]["fraction"] - 0.5) < 1e-6 and np.allclose(h[0]["normal"], (-1.0, 0.0))
    h = ow.raycast((2.0, 0.5), (-2.0, 0.5), "closest")                   # from the other side
    assert len(h) == 1 and abs(h[0]["fraction"] - 0.5) < 1e-6 and np.allclose(h[0]["normal"], (1.0, 0.0))
    ow = oracle_lib.OracleWorld(_one_body_scene(abi.SHAPE_POLYGON, half=(1.0, 1.0), angle=np.pi / 4))
    h = ow.raycast((-5.0, 0.0), (5.0, 0.0), "closest")
    assert len(h) == 1 and abs(h[0]["point"][0] + np.sqrt(2.0)) < 1e-5
    assert np.allclose(h[0]["normal"], (-np.sqrt(0.5), np.sqrt(0.5)), atol=1e-6) or np.allclose(
        h[0]["normal"], (-np.sqrt(0.5), -np.sqrt(0.5)), atol=1e-6)
    assert ow.raycast((1.0, 1.0), (1.0, 1.0), "closest") is None         # p1 == p2


def _settled(oracle_lib, scene, steps):
    oracle_lib.set_trig_mode(1)
    ow = oracle_lib.OracleWorld(scene)
    ow.step(steps=steps)
    return ow


def _random_boxes(rng, n, lo, hi, size):
    c = rng.uniform(lo, hi, (n, 2)).astype(np.float32)
    e = rng.uniform(0.05, size, (n, 2)).astype(np.float32)
    return np.concatenate([c - e, c + e], 1)


def test_query_aabb_matches_fat_aabbs(oracle_lib):
    # the tree walk reports exactly the fixtures whose fat AABB overlaps (b2TestOverlap)
    ow = _settled(oracle_lib, scenes.edge_ground(), 60)
    px = ow.export_state()["proxies"]
    fat = px["fat_aabb"]
    rng = np.random.default_rng(3)
    for box in _random_boxes(rng, 200, (-30.0, -2.0), (30.0, 15.0), 4.0):
        got = ow.query_aabb(box)
        want = np.nonzero((px["proxy_id"] >= 0) & ~((fat[:, 0] - box[2] > 0) | (fat[:, 1] - box[3] > 0) |
                                                     (box[0] - fat[:, 2] > 0) | (box[1] - fat[:, 3] > 0)))[0]
        assert np.array_equal(got, want)


def test_raycast_closest_matches_clipping_callback(oracle_lib):
    # the closest hit over all hits equals what the reference's clipping callback ends with
    # (fraction, point and normal; the fixture too, ties aside), and every hit of "all" lies
    # on the ray, no nearer than the closest
    for scene in (scenes.edge_ground(), scenes.chain_ground(), scenes.pyramid(rows=12)):
        ow = _settled(oracle_lib, scene, 90)
        rng = np.random.default_rng(5)
        hits = 0
        for _ in range(150):
            p1 = rng.uniform((-30.0, -2.0), (30.0, 20.0)).astype(np.float32)
            p2 = (p1 + rng.uniform(-25.0, 25.0, 2)).astype(np.float32)
            a = ow.raycast(p1, p2, "closest")
            c = ow.raycast(p1, p2, "clip")
            al = ow.raycast(p1, p2, "all")
            assert len(a) == len(c) == min(len(al), 1)
            if len(a):
                hits += 1
                assert a[0]["fraction"] == c[0]["fraction"]
                if (al["fraction"] == a[0]["fraction"]).sum() == 1:
                    assert a[0]["fixture"] == c[0]["fixture"] and np.array_equal(a[0]["normal"], c[0]["normal"])
                assert (al["fraction"] >= a[0]["fraction"]).all() and (al["fraction"] <= 1.0).all()
                assert np.all(np.diff(al["fixture"]) > 0)
        assert hits > 20


def _gpu_vs_oracle(gpu_lib, oracle_lib, worlds, steps, n_boxes, n_rays, seed):
    oracle_lib.set_trig_mode(1)
    gw = gpu_lib.World(worlds)
    ows = [oracle_lib.OracleWorld(s) for s in worlds]
    gw.step(steps=steps)
    for ow in ows:
        ow.step(steps=steps)
    for i, ow in enumerate(ows):
        assert not exact_diff(ow.export_state(), gw.export_state(i))
    rng = np.random.default_rng(seed)
    W = len(worlds)
    wid = rng.integers(0, W, n_boxes).astype(np.int32)
    boxes = _random_boxes(rng, n_boxes, (-30.0, -2.0), (30.0, 20.0), 6.0)
    cap = 512
    counts, fx = gw.query_aabb(wid, boxes, cap)
    for q in range(n_boxes):
        want = ows[wid[q]].query_aabb(boxes[q])
        assert counts[q] == len(want), q
        assert np.array_equal(fx[q, :min(cap, len(want))], want[:cap]), q
    rid = rng.integers(0, W, n_rays).astype(np.int32)
    p1 = rng.uniform((-30.0, -2.0), (30.0, 20.0), (n_rays, 2)).astype(np.float32)
    p2 = (p1 + rng.uniform(-30.0, 30.0, (n_rays, 2))).astype(np.float32)
    for mode, cap in (("closest", 1), ("all", 64)):
        counts, hits = gw.raycast(rid, p1, p2, mode, cap)
        nz = 0
        for q in range(n_rays):
            want = ows[rid[q]].raycast(p1[q], p2[q], mode)
            assert counts[q] == len(want), (mode, q)
            got = hits[q, :min(cap, len(want))]
            assert got.tobytes() == want[:cap].tobytes(), (mode, q, got, want)
            nz += len(want) > 0
        assert nz > n_rays // 10
    return gw


@pytest.mark.gpu
def test_queries_exact_small_worlds(oracle_lib, gpu_lib):
    # pyramids, edge and chain terrain, scatter: the device index gives the oracle's sets,
    # fractions, points and normals bit for bit
    worlds = [scenes.pyramid(rows=10), scenes.edge_ground(), scenes.chain_ground(), scenes.pyramid(rows=4),
              scenes.chains(n_chains=2, links=12)]
    _gpu_vs_oracle(gpu_lib, oracle_lib, worlds, 90, 600, 600, 11)


@pytest.mark.gpu
def test_queries_exact_large_world(oracle_lib, gpu_lib):
    # one world of 2,500+ proxies: three index levels are used (more than 32 x 32 proxies)
    rng = np.random.default_rng(2)
    s = scenes._concat([scenes.container(60.0, 40.0), scenes.scatter(2400, 58.0, 38.0, rng)])
    gw = _gpu_vs_oracle(gpu_lib, oracle_lib, [s], 20, 300, 300, 13)
    # empty results (entries past the count are unspecified), a box covering everything (count
    # above capacity), a ray naming no world, a ray of zero length
    counts, fx = gw.query_aabb([0], np.array([[1e6, 1e6, 1e6 + 1, 1e6 + 1]], np.float32), 8)
    assert counts[0] == 0
    counts, fx = gw.query_aabb([0], np.array([[-1e4, -1e4, 1e4, 1e4]], np.float32), 8)
    assert counts[0] == len(s["fixtures"]) and np.array_equal(fx[0], np.arange(8))
    counts, _ = gw.raycast([5], [(0.0, 0.0)], [(1.0, 1.0)])
    assert counts[0] == -1
    counts, _ = gw.raycast([0], [(1.0, 1.0)], [(1.0, 1.0)])
    assert counts[0] == -1
