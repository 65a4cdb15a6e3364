"""GPU step parity against the CPU oracle (b2World.Step restated on the CPU).

Bit-exact cases run the oracle with the portable sin/cos (dbox_sincosf), which
the GPU library also uses; every exported field must then match to the bit on
every step.  The reference-arithmetic cases run the oracle with the host libm
sinf/cosf (as the reference does), re-seed the GPU from the oracle's state
before each step and require: identical pair set, contact list order, point
counts and feature ids, and body state within 1e-5 m, 1e-5 rad, 1e-4 m/s.
"""
import numpy as np
import pytest

from compare import body_error, exact_diff, structure_diff

pytestmark = pytest.mark.gpu


def _pair(oracle_lib, gpu_lib, scene, flags=None):
    ow = oracle_lib.OracleWorld(scene, flags)
    gw = gpu_lib.World(scene, flags=flags)
    return ow, gw


def _run_exact(oracle_lib, gpu_lib, scene, steps, every=1, flags=None, vi=8, pi=3):
    oracle_lib.set_trig_mode(1)
    ow, gw = _pair(oracle_lib, gpu_lib, scene, flags)
    d = exact_diff(ow.export_state(), gw.export_state())
    assert not d, "creation state differs: %s" % d[:6]
    for t in range(steps):
        ow.step(1.0 / 60.0, vi, pi)
        gw.step(1.0 / 60.0, vi, pi)
        if (t + 1) % every == 0 or t + 1 == steps:
            d = exact_diff(ow.export_state(), gw.export_state())
            assert not d, "step %d: %s" % (t + 1, d[:6])
    return ow, gw


def test_hello_world_exact(oracle_lib, gpu_lib):
    from dbox_gb300 import scenes
    _run_exact(oracle_lib, gpu_lib, scenes.hello_world(), 60, vi=6, pi=2)


def test_pyramid_600_steps_exact(oracle_lib, gpu_lib):
    from dbox_gb300 import scenes
    ow, gw = _run_exact(oracle_lib, gpu_lib, scenes.pyramid(), 600, every=1)
    st = gw.export_state()
    assert len(st["contacts"]) > 400
    assert int(((st["bodies"]["flags"] & 2) == 0).sum()) > 0   # the pyramid fell asleep


def test_scatter_exact(oracle_lib, gpu_lib):
    from dbox_gb300 import scenes
    s = scenes.scatter(300, 30.0, 40.0, np.random.default_rng(7))
    _run_exact(oracle_lib, gpu_lib, s, 400, every=5)


def test_large_scatter_exact(oracle_lib, gpu_lib):
    # more than 1,024 proxies: the broad-phase takes the sweep-and-prune path
    from dbox_gb300 import scenes
    s = scenes.scatter(1500, 60.0, 60.0, np.random.default_rng(9))
    _run_exact(oracle_lib, gpu_lib, s, 120, every=10)


def test_stacks_exact(oracle_lib, gpu_lib):
    from dbox_gb300 import scenes
    _run_exact(oracle_lib, gpu_lib, scenes.stacks(60, 12), 300, every=10)


def test_revolute_chains_exact(oracle_lib, gpu_lib):
    # revolute joints (b2revolutejoint.d:319-636): plain, limited and motor-driven chains
    # falling onto box stacks, joints in the islands with contacts
    from dbox_gb300 import scenes
    ow, gw = _run_exact(oracle_lib, gpu_lib, scenes.chains(n_chains=4, links=16), 300, every=5)
    st = gw.export_state()
    assert len(st["joints"]) == 64
    assert np.abs(st["joints"]["impulse"]).max() > 0


def test_batch_exact(oracle_lib, gpu_lib):
    from dbox_gb300 import scenes
    oracle_lib.set_trig_mode(1)
    worlds = scenes.batch(n_worlds=9, seed=11, lo=8, hi=96)
    gw = gpu_lib.World(worlds)
    ows = [oracle_lib.OracleWorld(s) for s in worlds]
    for t in range(240):
        gw.step()
        for ow in ows:
            ow.step()
        if (t + 1) % 20 == 0:
            for i, ow in enumerate(ows):
                d = exact_diff(ow.export_state(), gw.export_state(i))
                assert not d, "world %d step %d: %s" % (i, t + 1, d[:6])


def test_mappings_and_autotune_keep_results(oracle_lib, gpu_lib):
    # the world-to-block mapping (warps per block, shared-memory budget, or the world queue)
    # and the autotuner's choice among mappings change where worlds run, never what they compute
    from dbox_gb300 import scenes
    oracle_lib.set_trig_mode(1)
    worlds = scenes.batch(n_worlds=9, seed=12, lo=8, hi=200)
    gw = gpu_lib.World(worlds)
    ows = [oracle_lib.OracleWorld(s) for s in worlds]
    steps = 0
    for wpb, budget, iso in ((1, 0, 0), (2, 2048, 0), (4, 0, 3)):
        gw.set_mapping(wpb, budget, iso)
        for _ in range(30):
            gw.step()
        steps += 30
    # queue mappings: plain, heavy worlds spread over sub-partitions, exclusive; graph and single steps
    for heavy, excl in ((0, False), (4, False), (3, True)):
        gw.set_mapping_queue(heavy, excl)
        gw.step(steps=10, graph=True)
        for _ in range(10):
            gw.step()
        steps += 20
    gw.set_world_costs(np.arange(len(worlds), dtype=np.float32))
    gw.step(steps=10, graph=True)
    steps += 10
    choice = gw.autotune(steps=2)
    assert choice[3] in (0, 1) and (choice[3] == 1 or choice[0] in (1, 2, 4))
    steps += gw.autotune_steps(2)
    for _ in range(30):
        gw.step()
    steps += 30
    for ow in ows:
        ow.step(steps=steps)
    for i, ow in enumerate(ows):
        d = exact_diff(ow.export_state(), gw.export_state(i))
        assert not d, "world %d: %s" % (i, d[:6])


def test_queue_mapping_with_more_worlds_than_warps_exact(oracle_lib, gpu_lib):
    # more worlds than the resident warps of the queue mapping, so warps take several worlds
    # one after another in a step (and carry their row ring from world to world)
    from dbox_gb300 import scenes
    oracle_lib.set_trig_mode(1)
    worlds = scenes.batch(n_worlds=2000, seed=14, lo=8, hi=40)
    gw = gpu_lib.World(worlds)
    ows = [oracle_lib.OracleWorld(s) for s in worlds]
    gw.set_mapping_queue(64, False)
    gw.step(steps=12, graph=True)
    for _ in range(4):
        gw.step()
    gw.set_mapping_queue(32, True)
    gw.step(steps=4, graph=True)
    for ow in ows:
        ow.step(steps=20)
    for i, ow in enumerate(ows):
        d = exact_diff(ow.export_state(), gw.export_state(i))
        assert not d, "world %d: %s" % (i, d[:6])


def test_fused_and_split_steps_exact(oracle_lib, gpu_lib):
    # one launch per step (each world's warp from its Collide straight to its Solve and TOI), all
    # the steps of a step_n call in one launch, and four launches a step: the same bits, on
    # both mappings (packed blocks and the world queue, where warps take several worlds)
    from dbox_gb300 import scenes
    oracle_lib.set_trig_mode(1)
    worlds = scenes.batch(n_worlds=600, seed=15, lo=8, hi=160)
    gw = gpu_lib.World(worlds)
    ows = [oracle_lib.OracleWorld(s) for s in worlds]
    assert not gw.fused_step()
    steps = 0
    for queue in (False, True):
        if queue:
            gw.set_mapping_queue(16, False)
        for fused in (True, False):
            gw.set_fused_step(fused)
            gw.step(steps=7, graph=True)
            for _ in range(3):
                gw.step()
            steps += 10
            assert gw.last_launches() == (1 if fused else 4)
            tot, ph = gw.step_timed(5)
            steps += 5
            assert gw.last_launches() == (1 if fused else 20)
            assert tot > 0.0 and (ph[0] == 0.0) == fused
    for ow in ows:
        ow.step(steps=steps)
    for i, ow in enumerate(ows):
        d = exact_diff(ow.export_state(), gw.export_state(i))
        assert not d, "world %d: %s" % (i, d[:6])


def test_graph_replay_matches_single_steps(oracle_lib, gpu_lib):
    from dbox_gb300 import scenes
    s = scenes.scatter(200, 25.0, 30.0, np.random.default_rng(3))
    a = gpu_lib.World(s)
    b = gpu_lib.World(s)
    a.step(steps=120)
    b.step(steps=120, graph=True)
    assert not exact_diff(a.export_state(), b.export_state())


def test_pyramid_reference_trig_one_step(oracle_lib, gpu_lib):
    from dbox_gb300 import scenes
    oracle_lib.set_trig_mode(0)
    try:
        s = scenes.pyramid()
        ow, gw = _pair(oracle_lib, gpu_lib, s)
        worst = [0.0, 0.0, 0.0]
        for t in range(600):
            gw.import_state(ow.export_state())
            ow.step()
            gw.step()
            a, b = ow.export_state(), gw.export_state()
            assert not structure_diff(a, b), "step %d: %s" % (t + 1, structure_diff(a, b)[:4])
            dp, da, dv = body_error(a, b)
            worst = [max(worst[0], dp), max(worst[1], da), max(worst[2], dv)]
            assert dp <= 1e-5 and da <= 1e-5 and dv <= 1e-4, "step %d: %s" % (t + 1, (dp, da, dv))
    finally:
        oracle_lib.set_trig_mode(1)


def test_distance_joint_ropes_exact(oracle_lib, gpu_lib):
    # distance joints (rigid, soft, a long soft tie) beside a revolute chain and box stacks:
    # bit-exact against the oracle, in one world and in a batch with other worlds
    from dbox_gb300 import scenes
    oracle_lib.set_trig_mode(1)
    worlds = [scenes.ropes(), scenes.ropes(n_ropes=3, links=8, revolute=False),
              scenes.pyramid(rows=6), scenes.chains(n_chains=2, links=10)]
    gw = gpu_lib.World(worlds)
    ows = [oracle_lib.OracleWorld(s) for s in worlds]
    for t in range(150):
        gw.step()
        for ow in ows:
            ow.step()
        if t % 30 == 29:
            for i, ow in enumerate(ows):
                d = exact_diff(ow.export_state(), gw.export_state(i))
                assert not d, "world %d step %d: %s" % (i, t + 1, d[:6])


def test_weld_and_rope_joints_exact(oracle_lib, gpu_lib):
    # rigid and soft weld beams, ropes at and below their maximum length, beside stacks and
    # the other joint kinds: bit-exact against the oracle
    from dbox_gb300 import scenes
    oracle_lib.set_trig_mode(1)
    worlds = [scenes.welded(), scenes.welded(n_beams=2, links=5, pile=False), scenes.ropes(n_ropes=2, links=6)]
    gw = gpu_lib.World(worlds)
    ows = [oracle_lib.OracleWorld(s) for s in worlds]
    for t in range(150):
        gw.step()
        for ow in ows:
            ow.step()
        if t % 30 == 29:
            for i, ow in enumerate(ows):
                d = exact_diff(ow.export_state(), gw.export_state(i))
                assert not d, "world %d step %d: %s" % (i, t + 1, d[:6])


def test_friction_and_motor_joints_exact(oracle_lib, gpu_lib):
    # zero-gravity top-down worlds with friction joints to a table body and two motor-driven
    # platforms: bit-exact against the oracle
    from dbox_gb300 import scenes
    oracle_lib.set_trig_mode(1)
    # zero gravity: one handle for the top-down worlds (a handle has one gravity, as a b2World)
    worlds = [scenes.top_down(), scenes.top_down(n=20, seed=9)]
    gw = gpu_lib.World(worlds)
    ows = [oracle_lib.OracleWorld(s) for s in worlds]
    for t in range(150):
        gw.step()
        for ow in ows:
            ow.step()
        if t % 30 == 29:
            for i, ow in enumerate(ows):
                d = exact_diff(ow.export_state(), gw.export_state(i))
                assert not d, "world %d step %d: %s" % (i, t + 1, d[:6])


def test_wheel_joint_cars_exact(oracle_lib, gpu_lib):
    # sprung, motor-driven wheels over bumps (circle wheels against boxes), batched with
    # the other joint kinds: bit-exact against the oracle
    from dbox_gb300 import scenes
    oracle_lib.set_trig_mode(1)
    worlds = [scenes.cars(), scenes.cars(n_cars=2, seed=11), scenes.welded(n_beams=1, links=4, pile=False),
              scenes.ropes(n_ropes=1, links=5)]
    gw = gpu_lib.World(worlds)
    ows = [oracle_lib.OracleWorld(s) for s in worlds]
    for t in range(180):
        gw.step()
        for ow in ows:
            ow.step()
        if t % 30 == 29:
            for i, ow in enumerate(ows):
                d = exact_diff(ow.export_state(), gw.export_state(i))
                assert not d, "world %d step %d: %s" % (i, t + 1, d[:6])


def test_prismatic_joints_exact(oracle_lib, gpu_lib):
    # prismatic platforms with motors, limits (lower, upper, equal) and a reference angle,
    # batched with wheels and welds: bit-exact against the oracle
    from dbox_gb300 import scenes
    oracle_lib.set_trig_mode(1)
    worlds = [scenes.sliders(), scenes.sliders(n=3, boxes=3), scenes.cars(n_cars=1),
              scenes.welded(n_beams=1, links=3, pile=False)]
    gw = gpu_lib.World(worlds)
    ows = [oracle_lib.OracleWorld(s) for s in worlds]
    for t in range(180):
        gw.step()
        for ow in ows:
            ow.step()
        if t % 30 == 29:
            for i, ow in enumerate(ows):
                d = exact_diff(ow.export_state(), gw.export_state(i))
                assert not d, "world %d step %d: %s" % (i, t + 1, d[:6])


def test_pulley_and_mouse_joints_exact(oracle_lib, gpu_lib):
    # pulleys of three ratios and a mouse joint whose target moves twice (SetTarget wakes the
    # body), batched with prismatic sliders: bit-exact against the oracle
    from dbox_gb300 import scenes
    oracle_lib.set_trig_mode(1)
    worlds = [scenes.pulleys(), scenes.pulleys(n=2, x0=-4.0), scenes.sliders(n=2, boxes=2)]
    gw = gpu_lib.World(worlds)
    ows = [oracle_lib.OracleWorld(s) for s in worlds]
    targets = {60: (6.0, 4.0), 120: (-2.0, 1.5)}
    for t in range(180):
        if t in targets:
            for i in (0, 1):
                mj = len(worlds[i]["pulley_joints"])          # the mouse joint comes after the pulleys
                gw.set_mouse_target(i, mj, targets[t])
                ows[i].set_mouse_target(mj, targets[t])
        gw.step()
        for ow in ows:
            ow.step()
        if t % 30 == 29:
            for i, ow in enumerate(ows):
                d = exact_diff(ow.export_state(), gw.export_state(i))
                assert not d, "world %d step %d: %s" % (i, t + 1, d[:6])


def test_edge_shapes_exact(oracle_lib, gpu_lib):
    # edge terrain with ghost vertices, loose edges, circles and polygons, a pyramid on an
    # edge ground, an edge on a dynamic body: bit-exact against the oracle (contact list,
    # manifolds with feature ids, bodies)
    from dbox_gb300 import scenes
    oracle_lib.set_trig_mode(1)
    worlds = [scenes.edge_ground(), scenes.edge_ground(n=24, seed=21, pyramid_rows=4)]
    gw = gpu_lib.World(worlds)
    ows = [oracle_lib.OracleWorld(s) for s in worlds]
    for t in range(240):
        gw.step()
        for ow in ows:
            ow.step()
        if t % 30 == 29:
            for i, ow in enumerate(ows):
                d = exact_diff(ow.export_state(), gw.export_state(i))
                assert not d, "world %d step %d: %s" % (i, t + 1, d[:6])


def test_chain_shapes_exact(oracle_lib, gpu_lib):
    # chain shapes (a loop bowl, open chains with and without prev/next ghosts, a loop on a
    # dynamic body) created as their child edges after the scene's fixtures: bit-exact
    # against the oracle
    from dbox_gb300 import scenes
    oracle_lib.set_trig_mode(1)
    worlds = [scenes.chain_ground(), scenes.chain_ground(n=24, seed=29)]
    gw = gpu_lib.World(worlds)
    ows = [oracle_lib.OracleWorld(s) for s in worlds]
    for t in range(240):
        gw.step()
        for ow in ows:
            ow.step()
        if t % 30 == 29:
            for i, ow in enumerate(ows):
                d = exact_diff(ow.export_state(), gw.export_state(i))
                assert not d, "world %d step %d: %s" % (i, t + 1, d[:6])


def test_gear_joints_exact(oracle_lib, gpu_lib):
    # gear joints over revolute / revolute, revolute / prismatic, and two wheels on a swinging
    # arm (the gear's C and D bodies dynamic, so its schedule level depends on four bodies),
    # with boxes falling onto the machinery: bit-exact against the oracle
    from dbox_gb300 import scenes
    oracle_lib.set_trig_mode(1)
    worlds = [scenes.gears(), scenes.gears(boxes=20, seed=4)]
    gw = gpu_lib.World(worlds)
    ows = [oracle_lib.OracleWorld(s) for s in worlds]
    for t in range(240):
        gw.step()
        for ow in ows:
            ow.step()
        if t % 30 == 29:
            for i, ow in enumerate(ows):
                d = exact_diff(ow.export_state(), gw.export_state(i))
                assert not d, "world %d step %d: %s" % (i, t + 1, d[:6])


def test_large_world_block_pairs_exact(oracle_lib, gpu_lib):
    # a world of 4,500 bodies (at least 4,096 fixtures) generates its end-of-Solve pairs on a
    # block of its own and finishes AddPair + SolveTOI in a separate warp; a small world in the
    # same handle keeps the one-warp path: both bit-exact against the oracle
    from dbox_gb300 import scenes
    oracle_lib.set_trig_mode(1)
    rng = np.random.default_rng(12)
    big = scenes._concat([scenes.container(90.0, 90.0), scenes.scatter(4500, 88.0, 88.0, rng)])
    worlds = [big, scenes.pyramid(rows=10)]
    assert len(big["fixtures"]) >= 4096
    gw = gpu_lib.World(worlds)
    ows = [oracle_lib.OracleWorld(s) for s in worlds]
    for t in range(90):
        gw.step()
        for ow in ows:
            ow.step()
        if t % 30 == 29:
            for i, ow in enumerate(ows):
                d = exact_diff(ow.export_state(), gw.export_state(i))
                assert not d, "world %d step %d: %s" % (i, t + 1, d[:6])
    assert gw.export_state(0)["header"][0]["contact_count"] > 1000
