"""b2World.DestroyBody / DestroyJoint and b2Body.DestroyFixture (dynamics/b2world.d:105-360,
dynamics/b2body.d:179-247) between steps: the proxy-id rule the library uses, pinned against
the oracle's restated b2DynamicTree; then the library against the oracle, bit for bit,
including the EndContact events the destruction reports and the ids new proxies take."""
import numpy as np
import pytest

from dbox_gb300 import abi, dump, scenes
from compare import exact_diff


class ProxyIdModel:
    """The library's proxy-id rule (api.cu ProxyIds): freed nodes come back last in, first
    out, before never-used ones; a proxy takes a leaf and, unless the tree is empty, a parent;
    destroying one frees its parent (unless it was the root), then the leaf."""

    def __init__(self):
        self.free, self.fresh, self.live = [], 0, 0

    def _take(self):
        if self.free:
            return self.free.pop()
        self.fresh += 1
        return self.fresh - 1

    def create(self):
        i = self._take()
        if self.live > 0:
            self._take()
        self.live += 1
        return i

    def destroy(self, i):
        if self.live > 1:
            self.free.append(-1)
        self.free.append(i)
        self.live -= 1


def _box(x, y, btype=abi.DYNAMIC):
    b = abi.body_defs(1)[0]
    b["type"] = btype
    b["position"] = (x, y)
    sd = np.zeros(1, abi.SHAPE_DEF)[0]
    sd["kind"] = abi.SHAPE_BOX
    sd["hx"] = sd["hy"] = 0.5
    fd = abi.fixture_defs(1)[0]
    fd["density"] = 1.0
    return b, sd, fd


def test_proxy_ids_follow_the_free_list(oracle_lib):
    # random creations and destructions with steps between them (the tree moves, rotates and
    # rebalances): every new proxy gets the id the free-list rule predicts
    oracle_lib.set_trig_mode(1)
    rng = np.random.default_rng(7)
    ow = oracle_lib.OracleWorld(scenes.ground_box())
    model = ProxyIdModel()
    model.create()                                      # the ground's proxy
    live = {}                                           # fixture -> (body, proxy id)
    for it in range(120):
        op = rng.random()
        if op < 0.55 or len(live) < 3:
            b, sd, fd = _box(float(rng.uniform(-20, 20)), float(rng.uniform(1, 12)))
            body = ow.create_body(b)
            f = ow.create_fixture(body, sd, fd)
            want = model.create()
            got = int(ow.export_state()["proxies"]["proxy_id"][f])
            assert got == want, (it, got, want)
            live[f] = (body, got)
        elif op < 0.8:
            f = int(rng.choice(list(live)))
            body, pid = live.pop(f)
            ow.destroy_body(body)
            model.destroy(pid)
        else:
            f = int(rng.choice(list(live)))
            body, pid = live.pop(f)
            ow.destroy_fixture(f)
            model.destroy(pid)
        if it % 5 == 4:
            ow.step(steps=3)
    st = ow.export_state()
    assert (st["proxies"]["proxy_id"] >= 0).sum() == len(live) + 1


def test_destroy_behaviour(oracle_lib):
    # destroying a resting pyramid box reports EndContact for its touching contacts and wakes
    # the boxes it touched (b2Contact.Destroy); destroying a chain link removes its joints;
    # destroyed items export as zero records and the rest keeps simulating
    oracle_lib.set_trig_mode(1)
    s = scenes._concat([scenes.pyramid(rows=6), scenes.chains(n_chains=1, links=8, pile=False)])
    ow = oracle_lib.OracleWorld(s)
    ow.step(steps=90)
    before = ow.export_state()
    touching = set()
    for c in before["contacts"]:
        fa, fb = int(c["fixture_a"]), int(c["fixture_b"])
        if 3 in (fa, fb) and c["point_count"] > 0:
            touching.add(fa + fb - 3)
    assert touching and all(before["bodies"]["flags"][i] & 2 == 0 for i in touching if i)   # asleep
    ow.record_events(True)
    ow.destroy_body(3)                                  # bottom row of the pyramid
    ev = ow.events()
    assert len(ev) > 0 and (ev["kind"] == abi.EVENT_END).all()
    st = ow.export_state()
    assert all(st["bodies"]["flags"][i] & 2 for i in touching)
    njoints = len(s["joints"])
    link = 1 + 21 + 1 + 3                               # ground, 21 boxes, post, 4th link
    ow.destroy_body(link)
    st = ow.export_state()
    zero = lambda rec: not np.frombuffer(rec.tobytes(), np.uint8).any()
    assert zero(st["bodies"][3]) and zero(st["bodies"][link])
    assert st["proxies"]["proxy_id"][3] == -1 and st["proxies"]["proxy_id"][link] == -1
    assert sum(not zero(j) for j in st["joints"]) <= njoints - 2
    ow.step(steps=60)
    assert np.isfinite(ow.export_state()["bodies"]["xf"]).all()


def _compare(ow, gw, tag):
    d = exact_diff(ow.export_state(), gw.export_state(0))
    assert not d, (tag, d[:6])
    text = ow.dump()
    assert text == gw.dump(0), tag
    p = dump.parse(text)                                # b2World.GetBodyCount / GetJointCount / GetContactCount
    assert gw.counts(0) == (len(p["bodies"]), len(p["joints"]), int(ow.export_state()["header"][0]["contact_count"])), tag


@pytest.mark.gpu
def test_destroy_exact(oracle_lib, gpu_lib):
    # destroy bodies (with contacts and joints), fixtures (one a chain child: the whole chain
    # goes), joints; create new bodies whose proxies reuse the freed ids; the library matches
    # the oracle bit for bit at every phase, and reports the same EndContact events
    oracle_lib.set_trig_mode(1)
    s = scenes._concat([scenes.pyramid(rows=8), scenes.chains(n_chains=2, links=10, pile=False),
                        scenes.chain_ground(n=16, seed=3)])
    ow = oracle_lib.OracleWorld(s)
    gw = gpu_lib.World([s])
    got = []
    gw.set_listener(lambda e: got.append(e))
    ow.record_events(True)
    gw.step(steps=60)
    ow.step(steps=60)
    ow.events()
    got.clear()
    _compare(ow, gw, "before")
    nb = len(s["bodies"])
    nf = len(s["fixtures"])
    chain_child = nf + 5                                # a child of the first chain shape
    # the low ids freed last come back first: the new fixtures below get ids under those of
    # older fixtures, so the broad-phase must walk proxies by id, not by fixture index
    for kind, idx in (("body", nb - 1), ("fixture", chain_child), ("joint", 3), ("fixture", 10), ("body", 37),
                      ("body", 4)):
        getattr(ow, "destroy_" + kind)(idx)
        getattr(gw, "destroy_" + kind)(0, idx)
        ref = ow.events()
        ev = np.concatenate(got) if got else np.zeros(0, abi.CONTACT_EVENT)
        got.clear()
        assert ev.tobytes() == ref.tobytes(), (kind, idx, len(ev), len(ref))
        _compare(ow, gw, "after destroying %s %d" % (kind, idx))
    ow.events()
    for t in range(3):
        gw.step(steps=30)
        ow.step(steps=30)
        got.clear()
        ow.events()
        _compare(ow, gw, "step %d" % (30 * (t + 1)))
    for k in range(5):                                  # new proxies take the freed ids
        b, sd, fd = _box(-3.0 + 1.2 * k, 10.0 + 0.1 * k)
        ob = ow.create_body(b)
        gb = gw.create_body(0, b)
        assert ob == gb
        assert ow.create_fixture(ob, sd, fd) == gw.create_fixture(0, gb, sd, fd)
    _compare(ow, gw, "after creating")
    ids = gw.export_state(0)["proxies"]["proxy_id"]
    live = ids[ids >= 0]
    assert (np.diff(live) < 0).any()                    # proxy ids no longer rise with the index
    gw.step(steps=90)
    ow.step(steps=90)
    _compare(ow, gw, "end")


def test_chain_proxy_ids_follow_the_free_list(oracle_lib):
    # a chain's child proxies are created and destroyed as the reference's one chain fixture:
    # created in child order, freed in child order (b2Fixture.CreateProxies / DestroyProxies),
    # so a new chain on freed ids gets them back last freed first
    oracle_lib.set_trig_mode(1)
    ow = oracle_lib.OracleWorld(scenes.ground_box())
    model = ProxyIdModel()
    model.create()
    b = abi.body_defs(1)[0]
    b["type"] = abi.STATIC
    body = ow.create_body(b)
    verts = np.array([(-5.0, 1.0), (-2.0, 2.0), (1.0, 1.5), (4.0, 2.5), (6.0, 1.0)], np.float32)
    first = ow.create_chain(body, verts, loop=True)
    ids = [model.create() for _ in range(len(verts))]
    got = ow.export_state()["proxies"]["proxy_id"][first:first + len(verts)]
    assert list(got) == ids
    ow.step(steps=3)
    ow.destroy_fixture(first + 2)                       # a child destroys its whole chain
    for i in ids:
        model.destroy(i)
    st = ow.export_state()["proxies"]["proxy_id"]
    assert (st[first:first + len(verts)] == -1).all()
    second = ow.create_chain(body, verts[:4], loop=False)
    want = [model.create() for _ in range(3)]
    assert list(ow.export_state()["proxies"]["proxy_id"][second:second + 3]) == want


def test_gear_dependencies_block_destruction(oracle_lib):
    # the reference leaves a gear dangling when one of its joints, or a body that carries one
    # of its joints but is neither of the gear's own bodies (joint1's and joint2's B bodies),
    # is destroyed first; here that is refused until the gear is gone.  Destroying one of the
    # gear's own bodies is well defined (its joints go newest first, the gear before them).
    oracle_lib.set_trig_mode(1)
    s = scenes.gears()
    ow = oracle_lib.OracleWorld(s)
    ow.step(steps=10)
    nrev, npri = len(s["joints"]), len(s["prismatic_joints"])
    gear0, gear2 = nrev + npri, nrev + npri + 2         # gear joints are created last
    with pytest.raises(ValueError):
        ow.destroy_joint(0)                             # joint1 of the first gear
    with pytest.raises(ValueError):
        ow.destroy_body(0)                              # the ground: the A body of gear 0's joints
    with pytest.raises(ValueError):
        ow.destroy_body(5)                              # the arm: the A body of gear 2's joints
    ow.destroy_body(1)                                  # gear 0's body A: the gear goes first
    assert not np.frombuffer(ow.export_state()["joints"][gear0].tobytes(), np.uint8).any()
    ow.destroy_joint(gear2)
    ow.destroy_body(5)
    ow.step(steps=10)
    assert np.isfinite(ow.export_state()["bodies"]["xf"]).all()


@pytest.mark.gpu
def test_gear_body_destruction_exact(oracle_lib, gpu_lib):
    # destroying a gear's own body takes the gear with it, in the library as in the oracle;
    # a body that would leave a gear dangling is refused by both
    oracle_lib.set_trig_mode(1)
    s = scenes.gears()
    ow = oracle_lib.OracleWorld(s)
    gw = gpu_lib.World([s])
    ow.step(steps=20)
    gw.step(steps=20)
    with pytest.raises(gpu_lib.DboxError):
        gw.destroy_body(0, 0)
    with pytest.raises(ValueError):
        ow.destroy_body(0)
    for body in (1, 7):                                 # gear 0's body A, gear 2's body B
        ow.destroy_body(body)
        gw.destroy_body(0, body)
        _compare(ow, gw, "after destroying body %d" % body)
    gw.step(steps=40)
    ow.step(steps=40)
    _compare(ow, gw, "40 steps later")
