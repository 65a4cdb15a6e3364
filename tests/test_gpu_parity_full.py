"""GPU step parity at the benchmark's own sizes and on the less common branches of a step.

- the 16,384-body single world and the full 4,096-world batch, bit for bit against the
  oracle with the portable sin/cos (every world of the batch compared);
- the same workloads against the reference's arithmetic (host libm sinf/cosf): the GPU is
  re-seeded from the oracle's state before each step, then pair set, contact order, point
  counts and feature ids must be identical and the bodies within 1e-5 m, 1e-5 rad, 1e-4 m/s
  (any step beyond that must be the oracle's own step with the device's sin/cos, bit for bit);
- one world with sensors, a bullet, a fast body against a thin wall, a kinematic platform,
  group / category / mask filtering, restitution and damping, stepped with varying dt
  (b2TimeStep.dtRatio, b2world.d:392) and with each b2World flag changed in turn
  (SetWarmStarting, SetContinuousPhysics, SetSubStepping, SetAllowSleeping): states and
  listener events bit for bit, TOI event counts equal.
"""
import numpy as np
import pytest

from compare import body_error, exact_diff, structure_diff
from dbox_gb300 import abi, scenes

pytestmark = pytest.mark.gpu


def test_scatter_16384_exact(oracle_lib, gpu_lib):
    # the single large world of the benchmark: 16,384 mixed circles / polygons in a 200 x 400 m
    # container, velocities N(0, 1), dt 1/60, 8/3 iterations
    oracle_lib.set_trig_mode(1)
    s = scenes.scatter_world(seed=3)
    assert scenes.dynamic_body_count(s) == 16384
    ow = oracle_lib.OracleWorld(s)
    gw = gpu_lib.World(s)
    d = exact_diff(ow.export_state(), gw.export_state())
    assert not d, d[:6]
    for t in range(60):
        ow.step()
        gw.step()
        if (t + 1) % 10 == 0:
            d = exact_diff(ow.export_state(), gw.export_state())
            assert not d, "step %d: %s" % (t + 1, d[:6])
    assert gw.export_state()["header"][0]["contact_count"] > 1000


def test_batch_4096_exact(oracle_lib, gpu_lib):
    # the benchmark's batch itself: 4,096 worlds, bodies log-uniform in [8, 512], thirds
    # pyramid / scatter / stacks, seed 3; every world compared after 20 steps
    import oracle_pool
    worlds = scenes.batch(n_worlds=4096, seed=3)
    want = oracle_pool.step_all(worlds, 20, trig=1)
    gw = gpu_lib.World(worlds)
    gw.step(steps=20, graph=True)
    bad = []
    for i in range(len(worlds)):
        d = exact_diff(want[i], gw.export_state(i))
        if d:
            bad.append((i, d[:3]))
    assert not bad, "%d worlds differ, first: %s" % (len(bad), bad[:3])


def _beyond_tolerance(a, b):
    """(bodies, bodies beyond 1e-5 m / 1e-5 rad / 1e-4 m/s) between two exported states."""
    ba, bb = a["bodies"], b["bodies"]
    dp = np.abs(ba["xf"][:, :2].astype(np.float64) - bb["xf"][:, :2]).max(1)
    da = np.abs(ba["sweep"][:, 7].astype(np.float64) - bb["sweep"][:, 7])
    dv = np.abs(ba["vel"].astype(np.float64) - bb["vel"]).max(1)
    return len(ba), int(((dp > 1e-5) | (da > 1e-5) | (dv > 1e-4)).sum())


def _reference_trig_run(oracle_lib, gpu_lib, worlds, pre_steps, steps):
    """Re-seeded one-step check against the host libm trig.

    Every step: the GPU is re-seeded from the libm oracle, both take one step, and the pair
    set, contact order, point counts and feature ids must be identical.  Positions, angles and
    velocities must agree within 1e-5 m, 1e-5 rad and 1e-4 m/s for at least 99.5 % of the
    body-steps.  A (world, step) with a body beyond that tolerance must be explained by the sin/cos alone:
    the oracle, stepped from the same state with the device's sin/cos instead of the libm's,
    reproduces the GPU's state bit for bit (the reference's block solver and position solver
    switch cases on last-bit differences of a rotation).  Returns (worst errors, outliers)."""
    from compare import exact_diff
    oracle_lib.set_trig_mode(0)
    try:
        ows = [oracle_lib.OracleWorld(s) for s in worlds]
        for ow in ows:
            ow.step(steps=pre_steps)
        gw = gpu_lib.World(worlds)
        worst = [0.0, 0.0, 0.0]
        outliers = []
        body_steps = bad_bodies = 0
        for t in range(steps):
            for i, ow in enumerate(ows):
                gw.import_state(ow.export_state(), i)
            for ow in ows:
                ow.step()
            gw.step()
            for i, ow in enumerate(ows):
                a, b = ow.export_state(), gw.export_state(i)
                sd = structure_diff(a, b)
                assert not sd, "world %d step %d: %s" % (i, pre_steps + t + 1, sd[:4])
                e = body_error(a, b)
                worst = [max(u, v) for u, v in zip(worst, e)]
                nb, nbad = _beyond_tolerance(a, b)
                body_steps += nb
                bad_bodies += nbad
                if nbad:
                    outliers.append((i, pre_steps + t + 1, e, b))
        assert bad_bodies <= 0.005 * body_steps, "%d of %d body-steps beyond tolerance: %s" % (
            bad_bodies, body_steps, [o[:3] for o in outliers[:4]])
        for i, step, e, b in outliers[:3]:
            x = oracle_lib.OracleWorld(worlds[i])
            x.step(steps=step - 1)                         # the libm trajectory up to the step
            oracle_lib.set_trig_mode(1)
            x.step()                                       # the step itself with the device's sin/cos
            oracle_lib.set_trig_mode(0)
            d = exact_diff(x.export_state(), b)
            assert not d, "world %d step %d beyond tolerance %s and not the sin/cos alone: %s" % (i, step, e, d[:4])
        return worst, outliers
    finally:
        oracle_lib.set_trig_mode(1)


def test_scatter_16384_reference_trig_one_step(oracle_lib, gpu_lib):
    # the 16,384-body world after 150 steps (bodies colliding, piles forming), 40 re-seeded steps
    worst, _ = _reference_trig_run(oracle_lib, gpu_lib, [scenes.scatter_world(seed=3)], 150, 40)
    assert max(worst) > 0.0          # the two sin/cos do differ somewhere


def test_batch_sample_reference_trig_one_step(oracle_lib, gpu_lib):
    # every 64th world of the benchmark's batch (pyramids, scatters and stacks of all sizes)
    worlds = scenes.batch(n_worlds=4096, seed=3)[::64]
    _reference_trig_run(oracle_lib, gpu_lib, worlds, 30, 60)


FLAG_CASES = [None, dict(warm=0), dict(continuous=0), dict(substep=1), dict(sleep=0)]


@pytest.mark.parametrize("flags", FLAG_CASES, ids=["default", "no_warm_start", "no_continuous", "sub_stepping",
                                                   "no_sleep"])
def test_features_exact(oracle_lib, gpu_lib, flags):
    oracle_lib.set_trig_mode(1)
    s = scenes.features()
    ow = oracle_lib.OracleWorld(s, flags)
    ow.record_events(True)
    gw = gpu_lib.World(s, flags=flags)
    got = []
    gw.set_listener(lambda ev: got.append(ev))
    # dt changes give b2TimeStep.dtRatio != 1 (warm-start impulses scaled), and a few steps
    # with other iteration counts
    sched = [(1 / 60, 8, 3)] * 40 + [(1 / 30, 8, 3)] * 20 + [(1 / 120, 10, 4)] * 20 + [(1 / 60, 6, 2)] * 60
    toi_total = 0
    kinds = np.zeros(5, np.int64)
    for t, (dt, vi, pi) in enumerate(sched):
        got.clear()
        ow.step(dt, vi, pi)
        gw.step(dt, vi, pi)
        ref = ow.events()
        ev = np.concatenate(got) if got else np.zeros(0, abi.CONTACT_EVENT)
        assert ev.tobytes() == ref.tobytes(), "step %d: events differ (%d vs %d)" % (t + 1, len(ev), len(ref))
        np.add.at(kinds, ev["kind"], 1)
        toi = gw.stats(0)[1]
        assert toi == ow.last_toi_events(), "step %d: TOI events %d vs %d" % (t + 1, toi, ow.last_toi_events())
        toi_total += toi
        if (t + 1) % 10 == 0:
            d = exact_diff(ow.export_state(), gw.export_state())
            assert not d, "step %d: %s" % (t + 1, d[:6])
    assert kinds[abi.EVENT_BEGIN] > 0 and kinds[abi.EVENT_END] > 0
    if flags == dict(continuous=0):
        assert toi_total == 0
    else:
        assert toi_total > 0


@pytest.mark.parametrize("per_pile,solver", [(300, 0), (1100, 0), (1100, 1)],
                         ids=["warp_path", "large_world_path", "large_world_warp_solve"])
def test_stress_reduced_exact(oracle_lib, gpu_lib, per_pile, solver):
    # the large-island stress world at reduced size: 4 container piles of mixed bodies with 4
    # revolute chains of 16 links hanging into each (with 1,100 bodies a pile the world has over
    # 4,096 fixtures and takes the large-world kernels; its Solve on a block, or on a warp)
    oracle_lib.set_trig_mode(1)
    s = scenes.stress(piles=4, per_pile=per_pile, chains_per_pile=4, links=16)
    ow = oracle_lib.OracleWorld(s)
    gw = gpu_lib.World(s)
    gw.set_island_solver(solver)
    toi = 0
    for t in range(120):
        ow.step()
        gw.step()
        toi += gw.stats(0)[1]
        assert gw.stats(0)[1] == ow.last_toi_events(), "step %d: TOI events" % (t + 1)
        if (t + 1) % 30 == 0:
            d = exact_diff(ow.export_state(), gw.export_state())
            assert not d, "step %d: %s" % (t + 1, d[:6])
    st = gw.export_state()
    assert st["header"][0]["contact_count"] > 4 * per_pile
    assert np.abs(st["joints"]["impulse"]).max() > 0
    assert toi > 100                     # SolveTOI's event loop runs many events a step


@pytest.mark.parametrize("solver", [0, 1], ids=["block_solve", "warp_solve"])
def test_large_mixed_world_exact(oracle_lib, gpu_lib, solver):
    # every joint type (gears with dynamic C / D bodies included), edge and chain grounds and a
    # 4,000-body pile in one world of over 4,096 fixtures: b2World.Solve on a block (union-find
    # islands, one search per thread, levels over the block) and on a warp; states and listener
    # events bit for bit against the oracle for 240 steps, bodies falling asleep on the way
    oracle_lib.set_trig_mode(1)
    s = scenes.large_mixed()
    assert len(s["fixtures"]) >= 4096
    ow = oracle_lib.OracleWorld(s)
    ow.record_events(True)
    gw = gpu_lib.World(s)
    gw.set_island_solver(solver)
    got = []
    gw.set_listener(lambda ev: got.append(ev))
    toi = 0
    for t in range(240):
        got.clear()
        ow.step()
        gw.step()
        toi += gw.stats(0)[1]
        assert gw.stats(0)[1] == ow.last_toi_events(), "step %d: TOI events" % (t + 1)
        ref = ow.events()
        ev = np.concatenate(got) if got else np.zeros(0, abi.CONTACT_EVENT)
        assert ev.tobytes() == ref.tobytes(), "step %d: events differ (%d vs %d)" % (t + 1, len(ev), len(ref))
        if (t + 1) % 60 == 0:
            d = exact_diff(ow.export_state(), gw.export_state())
            assert not d, "step %d: %s" % (t + 1, d[:6])
    st = gw.export_state()
    dyn = st["bodies"]["type"] == abi.DYNAMIC
    assert ((st["bodies"]["flags"][dyn] & abi.BODY_AWAKE) == 0).any()
    assert st["header"][0]["joint_count"] == sum(len(s[k]) for k in scenes.JOINT_KINDS)
    assert toi > 100


def test_two_large_worlds_and_small_ones_exact(oracle_lib, gpu_lib):
    # two worlds of 4,096+ fixtures in one handle (each on its own cluster of blocks) beside
    # small worlds on warps: every world bit for bit against the oracle
    oracle_lib.set_trig_mode(1)
    rng = np.random.default_rng(29)
    big_a = scenes._concat([scenes.container(90.0, 90.0), scenes.scatter(4300, 88.0, 88.0, rng)])
    big_b = scenes.stress(piles=4, per_pile=1100, chains_per_pile=2, links=12, seed=8)
    worlds = [scenes.pyramid(rows=8), big_a, scenes.chains(n_chains=2, links=8), big_b]
    assert len(big_a["fixtures"]) >= 4096 and len(big_b["fixtures"]) >= 4096
    gw = gpu_lib.World(worlds)
    ows = [oracle_lib.OracleWorld(s) for s in worlds]
    for t in range(90):
        gw.step()
        for ow in ows:
            ow.step()
        if (t + 1) % 30 == 0:
            for i, ow in enumerate(ows):
                d = exact_diff(ow.export_state(), gw.export_state(i))
                assert not d, "world %d step %d: %s" % (i, t + 1, d[:6])
