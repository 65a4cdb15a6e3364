"""Learned warm start on the GPU: the plumbing leaves the reference step untouched, the
plain solver logs usable samples, and a network trained on them gives a smaller velocity
residual than the zero start at the same iteration count."""
import numpy as np
import pytest

from dbox_gb300 import scenes

pytestmark = pytest.mark.gpu


def _scatter(n_worlds, bodies, seed):
    rng = np.random.default_rng(seed)
    return [scenes.scatter(bodies, 40.0, 40.0, rng) for _ in range(n_worlds)]


def test_zero_network_is_the_plain_step(gpu_lib):
    # a network that predicts 0 for every new point: learned mode must give the plain step bit for bit
    worlds = _scatter(12, 150, 21)
    m = gpu_lib.Mlp()
    norm = np.concatenate([np.zeros(32), np.ones(32), np.zeros(4), np.ones(4)]).astype(np.float32)
    m.set_params(np.zeros(gpu_lib.MLP_PARAMS, np.float32), norm)
    plain, learned = gpu_lib.World(worlds), gpu_lib.World(worlds)
    learned.set_warmstart(2, m)
    for _ in range(60):
        plain.step()
        learned.step()
    for i in range(len(worlds)):
        a, b = plain.export_state(i), learned.export_state(i)
        assert a["bodies"].tobytes() == b["bodies"].tobytes()
        ca, cb = a["contacts"].copy(), b["contacts"].copy()
        cb["flags"] &= ~np.uint32(0xC0)                 # the learned mode's new-point marks
        assert ca.tobytes() == cb.tobytes()
        assert (a["contacts"]["flags"] & 0xC0).sum() == 0


def test_plain_solver_logs_samples(gpu_lib):
    w = gpu_lib.World(_scatter(32, 128, 22))
    w.set_warmstart(1, None, 200000)
    w.step(steps=100, graph=True)
    n = w.sample_count()
    assert n > 1000
    f, t = w.samples()
    assert np.isfinite(f).all() and np.isfinite(t).all()
    assert set(np.unique(f[:, 26])) <= {1.0, 2.0}            # point count
    assert (t[:, [0, 2]] >= 0).all()                         # converged normal impulses are clamped at 0
    assert (t[f[:, 26] == 1.0][:, 2:] == 0).all()            # one-point contacts have no second point


def test_quality_measure_orders_iteration_counts(gpu_lib):
    res = {}
    for vi in (3, 8):
        w = gpu_lib.World(_scatter(16, 128, 23))
        w.step(steps=80, graph=True)
        w.set_measure(True)
        acc = []
        for _ in range(10):
            w.step(vel_iters=vi)
            q = w.quality()
            acc.append(np.sqrt(q[:, 0].sum() / max(q[:, 2].sum(), 1)))
        res[vi] = np.mean(acc)
    assert res[8] < res[3]


def test_trained_start_lowers_the_residual(gpu_lib):
    worlds = _scatter(96, 200, 24)
    log = gpu_lib.World(worlds)
    log.set_warmstart(1, None, 1_000_000)
    log.step(steps=250, graph=True)
    f, t = log.samples(0, min(log.sample_count(), 300000))
    m = gpu_lib.Mlp(seed=3)
    m.fit_normalization(f, t)
    losses = m.train_world(log, epochs=20, batch=16384, lr=1e-3, seed=4)
    assert losses[-1] < 0.8 * losses[0]

    def measure(mode, model):
        w = gpu_lib.World(worlds)
        w.step(steps=250, graph=True)
        w.set_warmstart(mode, model, 0)
        w.set_measure(True)
        mx, rms = [], []
        for _ in range(30):
            w.step(vel_iters=5)
            q = w.quality()
            mx.append(q[:, 1].max())
            rms.append(np.sqrt(q[:, 0].sum() / max(q[:, 2].sum(), 1)))
        return np.mean(mx), np.mean(rms)

    plain_max, plain_rms = measure(0, None)
    learned_max, learned_rms = measure(2, m)
    assert learned_max < plain_max
    assert learned_rms <= 1.02 * plain_rms


def test_copy_state_is_an_exact_checkpoint(oracle_lib, gpu_lib):
    # dbox_world_copy_state: a twin handle continues exactly where the source stood
    from compare import exact_diff
    oracle_lib.set_trig_mode(1)
    worlds = _scatter(6, 120, 25) + [scenes.pyramid(rows=9), scenes.chains(n_chains=2, links=8)]
    a = gpu_lib.World(worlds)
    b = gpu_lib.World(worlds)
    b.step()                                            # both on the device, b one step apart
    a.step(steps=40, graph=True)
    b.copy_state_from(a)
    a.step(steps=25)
    b.step(steps=25, graph=True)
    ows = [oracle_lib.OracleWorld(s) for s in worlds]
    for i, ow in enumerate(ows):
        ow.step(steps=65)
        assert not exact_diff(ow.export_state(), b.export_state(i)), i
        assert not exact_diff(a.export_state(i), b.export_state(i)), i


def test_given_start_slots_line_up(gpu_lib):
    # warm-start mode 3 reads the start of each new point from the source handle's contact at
    # the same slot.  With no velocity iterations on the source, its impulses at those slots
    # after its step are the reference's zero start, so the given-start step is the plain one
    from compare import exact_diff
    worlds = _scatter(32, 160, 26)
    plain = gpu_lib.World(worlds)
    given = gpu_lib.World(worlds)
    src = gpu_lib.World(worlds)
    for h in (plain, given, src):
        h.step(steps=60, graph=True)
    given.set_warmstart(3)
    given.set_start_source(src)
    for _ in range(10):
        src.copy_state_from(given)
        src.step(vel_iters=0)
        given.step(vel_iters=0)
        plain.step(vel_iters=0)
    for i in range(len(worlds)):
        assert not exact_diff(plain.export_state(i), given.export_state(i)), i
    # with iterations on the source the given start changes the step (new points start elsewhere)
    src.copy_state_from(given)
    src.step(vel_iters=8)
    given.step(vel_iters=4)
    plain.step(vel_iters=4)
    assert any(exact_diff(plain.export_state(i), given.export_state(i)) for i in range(len(worlds)))


def _large_world():
    rng = np.random.default_rng(27)
    big = scenes._concat([scenes.container(90.0, 90.0), scenes.scatter(4500, 88.0, 88.0, rng)])
    assert len(big["fixtures"]) >= 4096
    return big


def test_warm_start_modes_on_a_large_world(gpu_lib):
    # a world of 4,096+ fixtures runs its Solve on a block: every warm-start mode gives there the
    # same bits as on a warp (mode 2 with an untrained network, whose predictions are far from
    # zero; mode 1's logged samples as a set, their slots being taken in any order; mode 3 from
    # a source handle's step)
    from compare import exact_diff
    big = _large_world()
    m = gpu_lib.Mlp(seed=5)
    hs = {}
    for solver in (0, 1):
        w = gpu_lib.World(big)
        w.set_island_solver(solver)
        w.step(steps=40, graph=True)
        w.set_warmstart(2, m)
        w.step(steps=20)
        hs[solver] = w
    d = exact_diff(hs[0].export_state(), hs[1].export_state())
    assert not d, d[:6]
    samples = {}
    for solver in (0, 1):
        w = hs[solver]
        w.set_warmstart(1, None, 200000)
        w.step(steps=5)
        n = w.sample_count()
        f, t = w.samples(0, n)
        rows = np.concatenate([f, t], 1)
        samples[solver] = rows[np.lexsort(rows.T[::-1])]
    assert len(samples[0]) > 100 and samples[0].tobytes() == samples[1].tobytes()
    src = gpu_lib.World(big)
    src.step()
    for solver in (0, 1):
        w = hs[solver]
        w.set_warmstart(3)
        w.set_start_source(src)
    for _ in range(3):
        src.copy_state_from(hs[0])
        src.step(vel_iters=8)
        hs[0].step(vel_iters=4)
        hs[1].step(vel_iters=4)
    d = exact_diff(hs[0].export_state(), hs[1].export_state())
    assert not d, d[:6]
