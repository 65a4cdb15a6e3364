"""b2ContactListener.PreSolve with contact edits (b2worldcallbacks.d:101-115, called by
b2Contact.Update, contacts/b2contact.d:354): the library's PreSolve window between Collide and
Solve against the oracle's listener, which calls the same rule inside Collide as the reference
does.  The rule disables some contacts (b2Contact.SetEnabled, for this step only), and sets
friction, restitution and a conveyor tangent speed on others (persistent); the calls each side
sees, and the worlds, must match bit for bit every step."""
import numpy as np
import pytest

from compare import CONTACT_FLAG_MASK, exact_diff
from dbox_gb300 import abi, scenes

pytestmark = pytest.mark.gpu


def make_rule(static_fixtures):
    """A user's PreSolve: decisions from the fixtures of each contact.  It edits only contacts
    between two non-bullet dynamic bodies: b2World.SolveTOI calls b2Contact.Update (and so
    PreSolve) again only for contacts with a static, kinematic or bullet body
    (b2world.d:1194-1208, 1287, 1345-1372), where the library keeps the window's decisions
    instead of calling back (a contact that first touches inside a sub-step gets none)."""
    static = np.asarray(static_fixtures, bool)

    def rule(r):
        fa, fb = r["contact"]["fixture_a"], r["contact"]["fixture_b"]
        dyn = ~static[fa] & ~static[fb]
        r["enabled"][((fa % 7 == 3) | (fb % 7 == 3)) & dyn] = 0     # SetEnabled(false): this step only
        r["friction"][((fa + fb) % 5 == 1) & dyn] = np.float32(0.05)           # SetFriction
        r["restitution"][((fa + fb) % 9 == 4) & dyn] = np.float32(0.6)         # SetRestitution
        r["tangent_speed"][((fa + fb) % 4 == 2) & dyn] = np.float32(1.5)       # SetTangentSpeed
    return rule


def _key(recs):
    """Record bytes without the fields the comparison of states leaves out too: solver-internal
    flag bits, the cached TOI fraction and unused manifold points."""
    r = recs.copy()
    c = r["contact"]
    c["flags"] &= CONTACT_FLAG_MASK
    c["toi"] = 0
    for k in range(2):
        unused = c["point_count"] <= k
        c["points"][unused, k] = np.zeros(1, c["points"].dtype.base)
    r["contact"] = c
    return r.tobytes()


def test_presolve_window_matches_listener(oracle_lib, gpu_lib):
    oracle_lib.set_trig_mode(1)
    worlds = [scenes.pyramid(rows=10), scenes.scatter(120, 20.0, 20.0, np.random.default_rng(41))]
    rules = [make_rule((s["bodies"]["type"][s["fixture_body"]] != abi.DYNAMIC) |
                       (s["bodies"]["bullet"][s["fixture_body"]] != 0)) for s in worlds]
    gw = gpu_lib.World(worlds)
    ows = [oracle_lib.OracleWorld(s) for s in worlds]
    got, want = [], [[] for _ in worlds]

    def gpu_rule(r):
        got.append(r.copy())                                         # as the callback received them
        for i, rl in enumerate(rules):
            sub = r[r["world"] == i]
            rl(sub)
            r[r["world"] == i] = sub

    for i, ow in enumerate(ows):
        def orc_rule(r, i=i):
            if r["world"][0] == 0:                                   # Collide's calls (the window's)
                c = r.copy()
                c["world"] = i
                want[i].append(c)
            rules[i](r)
        ow.set_presolve(orc_rule)
    gw.set_presolve(gpu_rule)
    disabled = 0
    for t in range(150):
        got.clear()
        for lst in want:
            lst.clear()
        gw.step()
        for ow in ows:
            ow.step()
        g = np.concatenate(got) if got else np.zeros(0, abi.PRESOLVE_CONTACT)
        parts = [np.concatenate(lst) for lst in want if lst]
        o = np.concatenate(parts) if parts else np.zeros(0, abi.PRESOLVE_CONTACT)
        assert len(g) == len(o), "step %d: %d PreSolve calls vs %d" % (t + 1, len(g), len(o))
        assert _key(g) == _key(o), "step %d: PreSolve calls differ" % (t + 1)
        for i, rl in enumerate(rules):
            chk = g[g["world"] == i].copy()
            rl(chk)
            disabled += int((chk["enabled"] == 0).sum())
        if (t + 1) % 10 == 0:
            for i, ow in enumerate(ows):
                d = exact_diff(ow.export_state(), gw.export_state(i))
                assert not d, "world %d step %d: %s" % (i, t + 1, d[:6])
    assert disabled > 0
    gw.set_presolve(None)
    for ow in ows:
        ow.set_presolve(None)
    for _ in range(20):
        gw.step()
        for ow in ows:
            ow.step()
    for i, ow in enumerate(ows):
        assert not exact_diff(ow.export_state(), gw.export_state(i))
