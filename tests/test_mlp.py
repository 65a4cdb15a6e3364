"""The learned warm-start network: oracle self-check, then the GPU forward / gradient /
training kernels against the oracle (oracle/mlp_ref.py)."""
import numpy as np
import pytest

from oracle import mlp_ref


def _data(n, seed):
    rng = np.random.default_rng(seed)
    feats = rng.normal(0.0, 1.0, (n, 32)).astype(np.float32) * np.linspace(0.5, 3.0, 32).astype(np.float32)
    targets = np.stack([np.tanh(feats[:, 0]) + 0.5 * feats[:, 4], 0.3 * feats[:, 5] * feats[:, 24],
                        np.maximum(feats[:, 13], 0.0), np.sin(feats[:, 14])], 1).astype(np.float32)
    return feats, targets


def _norm(feats, targets):
    return np.concatenate([feats.mean(0), feats.std(0), targets.mean(0), targets.std(0)]).astype(np.float32)


def test_oracle_gradient_matches_finite_differences():
    feats, targets = _data(40, 1)
    params = mlp_ref.init_params(3).astype(np.float64)
    norm = _norm(feats, targets)
    _, g = mlp_ref.loss_and_grad(params, norm, feats, targets, bf16=False)
    rng = np.random.default_rng(2)
    idx = np.concatenate([rng.integers(0, mlp_ref.NW1, 6), mlp_ref.NW1 + rng.integers(0, mlp_ref.NW2, 6),
                          [mlp_ref.NW1 + mlp_ref.NW2 + 8 * 5 + 1, mlp_ref.NPARAMS - 8, mlp_ref.NPARAMS - 140]])
    for i in idx:
        e = 1e-6
        pp, pm = params.copy(), params.copy()
        pp[i] += e
        pm[i] -= e
        fd = (mlp_ref.loss_and_grad(pp, norm, feats, targets, bf16=False)[0] -
              mlp_ref.loss_and_grad(pm, norm, feats, targets, bf16=False)[0]) / (2 * e)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(g[i]), (i, fd, g[i])


@pytest.mark.gpu
def test_gpu_gradient_matches_oracle(gpu_lib):
    feats, targets = _data(300, 4)
    params = mlp_ref.init_params(5)
    norm = _norm(feats, targets)
    m = gpu_lib.Mlp()
    m.set_params(params, norm)
    g_gpu, loss_gpu = m.gradient(feats, targets)
    loss_ref, g_ref = mlp_ref.loss_and_grad(params, norm, feats, targets, bf16=True)
    assert abs(loss_gpu - loss_ref) <= 1e-3 * abs(loss_ref)
    # per parameter block: relative L2 error and direction (BF16 products, FP32 sums in any order)
    o = np.cumsum([0, mlp_ref.NW1, mlp_ref.NW2, mlp_ref.NW3, 128, 128, 8])
    for a, b in zip(o[:-1], o[1:]):
        d, r = g_gpu[a:b].astype(np.float64), g_ref[a:b]
        if np.linalg.norm(r) == 0:
            continue
        assert np.linalg.norm(d - r) <= 2e-2 * np.linalg.norm(r), (a, b)
        assert d @ r >= 0.999 * np.linalg.norm(d) * np.linalg.norm(r)


@pytest.mark.gpu
def test_gpu_gradient_many_tiles_matches_oracle(gpu_lib):
    # more 128-sample tiles than the GPU has SMs: each CTA keeps its gradients in tensor memory
    # across several tiles; the last tile is partial
    feats, targets = _data(152 * 128 * 2 + 77, 6)
    params = mlp_ref.init_params(7)
    norm = _norm(feats, targets)
    m = gpu_lib.Mlp()
    m.set_params(params, norm)
    g_gpu, loss_gpu = m.gradient(feats, targets)
    loss_ref, g_ref = mlp_ref.loss_and_grad(params, norm, feats, targets, bf16=True)
    assert abs(loss_gpu - loss_ref) <= 1e-3 * abs(loss_ref)
    o = np.cumsum([0, mlp_ref.NW1, mlp_ref.NW2, mlp_ref.NW3, 128, 128, 8])
    for a, b in zip(o[:-1], o[1:]):
        d, r = g_gpu[a:b].astype(np.float64), g_ref[a:b]
        if np.linalg.norm(r) == 0:
            continue
        assert np.linalg.norm(d - r) <= 2e-2 * np.linalg.norm(r), (a, b)


@pytest.mark.gpu
def test_gpu_forward_matches_oracle(gpu_lib):
    feats, targets = _data(200, 6)
    params = mlp_ref.init_params(7)
    norm = _norm(feats, targets)
    m = gpu_lib.Mlp()
    m.set_params(params, norm)
    out = m.forward(feats)
    ref = mlp_ref.forward(params, norm, feats, bf16=True)
    assert np.abs(out - ref).max() <= 2e-2 * np.abs(ref).max()


@pytest.mark.gpu
def test_gpu_training_lowers_the_loss(gpu_lib):
    feats, targets = _data(20000, 8)
    m = gpu_lib.Mlp(seed=11)
    m.fit_normalization(feats, targets)
    losses = m.train(feats, targets, epochs=20, batch=1024, lr=1e-3, seed=1)
    assert np.isfinite(losses).all()
    assert losses[-1] < 0.3 * losses[0]
    # the trained parameters give the same loss through the oracle
    p, q = m.params()
    loss_ref, _ = mlp_ref.loss_and_grad(p, q, feats[:2000], targets[:2000])
    _, loss_gpu = m.gradient(feats[:2000], targets[:2000])
    assert abs(loss_ref - loss_gpu) <= 2e-2 * loss_ref
