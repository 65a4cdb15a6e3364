"""Contact-listener events (b2ContactListener, dynamics/b2worldcallbacks.d:87-128) against
the oracle's recording listener: BeginContact / EndContact / PreSolve from Collide and the
TOI updates, PostSolve from b2Island.Report, in reference order, every step.  With the
portable sin/cos the events must match field for field, impulses to the bit."""
import numpy as np
import pytest

from dbox_gb300 import abi, scenes

pytestmark = pytest.mark.gpu


def _run(oracle_lib, gpu_lib, scene, steps):
    oracle_lib.set_trig_mode(1)
    ow = oracle_lib.OracleWorld(scene)
    ow.record_events(True)
    gw = gpu_lib.World(scene)
    got = []
    gw.set_listener(lambda ev: got.append(ev))
    kinds = np.zeros(5, np.int64)
    for t in range(steps):
        ow.step()
        got.clear()
        gw.step()
        ref = ow.events()
        ev = got[0] if got else np.zeros(0, abi.CONTACT_EVENT)
        assert len(ev) == len(ref), "step %d: %d events vs %d" % (t + 1, len(ev), len(ref))
        assert ev.tobytes() == ref.tobytes(), "step %d: first difference at event %d" % (
            t + 1, int(np.nonzero(ev.view(np.uint8).reshape(len(ev), -1) != ref.view(np.uint8).reshape(len(ref), -1))[0][0]))
        np.add.at(kinds, ev["kind"], 1)
    return kinds


def test_scatter_events_match(oracle_lib, gpu_lib):
    s = scenes.scatter(250, 30.0, 40.0, np.random.default_rng(31))
    kinds = _run(oracle_lib, gpu_lib, s, 200)
    assert kinds[abi.EVENT_BEGIN] > 0 and kinds[abi.EVENT_PRESOLVE] > 0 and kinds[abi.EVENT_POSTSOLVE] > 0
    assert kinds[abi.EVENT_END] > 0


def test_pyramid_and_chain_events_match(oracle_lib, gpu_lib):
    _run(oracle_lib, gpu_lib, scenes.pyramid(rows=10), 120)
    _run(oracle_lib, gpu_lib, scenes.chains(n_chains=3, links=12), 120)


def test_batch_events_are_world_by_world(oracle_lib, gpu_lib):
    rng = np.random.default_rng(32)
    worlds = [scenes.scatter(80, 20.0, 20.0, rng) for _ in range(3)]
    oracle_lib.set_trig_mode(1)
    ows = [oracle_lib.OracleWorld(s) for s in worlds]
    for o in ows:
        o.record_events(True)
    gw = gpu_lib.World(worlds)
    got = []
    gw.set_listener(lambda ev: got.append(ev))
    for t in range(60):
        got.clear()
        gw.step()
        ref = []
        for i, o in enumerate(ows):
            o.step()
            e = o.events()
            e["world"] = i
            ref.append(e)
        ref = np.concatenate(ref)
        ev = got[0] if got else np.zeros(0, abi.CONTACT_EVENT)
        assert ev.tobytes() == ref.tobytes(), "step %d" % (t + 1)
