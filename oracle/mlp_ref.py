"""Test oracle for the learned warm-start network (test infrastructure only: imported by
tests/ to check the GPU kernels, never by the library).

A numpy restatement of the library's 32 -> 128 -> 128 -> 4 GELU network: the forward pass
and the gradient of the mean squared error over samples and outputs, in normalised units.
`bf16=True` rounds at the places the GPU rounds (normalised inputs, weights, activations,
pre-activations kept for the backward pass, back-propagated errors) and accumulates in
float64; `bf16=False` is the same network in float64 throughout (used to check the
gradient against finite differences).  Parameter layout: w1[32][128], w2[128][128],
w3[128][8] (columns 4..7 unused), b1[128], b2[128], b3[8]; normalisation: feature mean[32],
std[32], target mean[4], std[4].
"""
import numpy as np

FEAT, HID, OUT, OUTPAD = 32, 128, 4, 8
NW1, NW2, NW3 = FEAT * HID, HID * HID, HID * OUTPAD
NPARAMS = NW1 + NW2 + NW3 + HID + HID + OUTPAD
K0, K1 = 0.7978845608028654, 0.044715


def round_bf16(x):
    """float32 -> nearest bfloat16 (ties to even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params):
    p = np.asarray(params, np.float64)
    w1 = p[:NW1].reshape(FEAT, HID)
    w2 = p[NW1:NW1 + NW2].reshape(HID, HID)
    w3 = p[NW1 + NW2:NW1 + NW2 + NW3].reshape(HID, OUTPAD)
    o = NW1 + NW2 + NW3
    return w1, w2, w3, p[o:o + HID], p[o + HID:o + 2 * HID], p[o + 2 * HID:o + 2 * HID + OUTPAD]


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(K0 * (x + K1 * x ** 3)))


def gelu_grad(x):
    t = np.tanh(K0 * (x + K1 * x ** 3))
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * K0 * (1.0 + 3.0 * K1 * x * x)


def _norm(norm):
    q = np.asarray(norm, np.float64)
    return q[:FEAT], q[FEAT:2 * FEAT], q[2 * FEAT:2 * FEAT + OUT], q[2 * FEAT + OUT:]


def _forward(params, norm, feats, bf16):
    r = round_bf16 if bf16 else (lambda v: np.asarray(v, np.float64))
    w1, w2, w3, b1, b2, b3 = unpack(params)
    fm, fs, _, _ = _norm(norm)
    x = r(((np.asarray(feats, np.float32) - fm.astype(np.float32)) / fs.astype(np.float32)))
    w1r, w2r, w3r = r(w1), r(w2), r(w3)
    pre1 = x @ w1r + b1
    h1 = r(gelu(pre1))
    pre2 = h1 @ w2r + b2
    h2 = r(gelu(pre2))
    y = h2 @ w3r + b3
    return x, w1r, w2r, w3r, pre1, h1, pre2, h2, y


def forward(params, norm, feats, bf16=True):
    """Predicted impulses (n x 4) in target units."""
    _, _, tm, ts = _norm(norm)
    y = _forward(params, norm, feats, bf16)[-1][:, :OUT]
    return y * ts + tm


def loss_and_grad(params, norm, feats, targets, bf16=True):
    """(loss, gradient (NPARAMS,)) of mean((MLP(x) - t')^2) with t' the normalised targets."""
    r = round_bf16 if bf16 else (lambda v: np.asarray(v, np.float64))
    x, w1r, w2r, w3r, pre1, h1, pre2, h2, y = _forward(params, norm, feats, bf16)
    _, _, tm, ts = _norm(norm)
    t = (np.asarray(targets, np.float32) - tm.astype(np.float32)) / ts.astype(np.float32)
    n = len(x)
    diff = y[:, :OUT] - t
    loss = float((diff ** 2).sum() / (4.0 * n))
    d = np.zeros((n, OUTPAD))
    d[:, :OUT] = 2.0 * diff / (4.0 * n)
    dy = r(d)
    gb3 = d.sum(0)
    gw3 = h2.T @ dy
    g2 = r(gelu_grad(pre2))            # the GELU derivative, kept in BF16 from the forward pass
    dh2 = (dy @ w3r.T) * g2
    d2 = r(dh2)
    gb2 = d2.sum(0)                    # column sums of the rounded operand (a tensor-core product with ones)
    gw2 = h1.T @ d2
    g1 = r(gelu_grad(pre1))
    dh1 = (d2 @ w2r.T) * g1
    d1 = r(dh1)
    gb1 = d1.sum(0)
    gw1 = x.T @ d1
    gw3[:, OUT:] = 0.0
    gb3[OUT:] = 0.0
    grad = np.concatenate([gw1.ravel(), gw2.ravel(), gw3.ravel(), gb1, gb2, gb3])
    return loss, grad


def init_params(seed):
    """A float32 parameter vector with uniform fan-in scaling (for tests)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAMS, np.float32)
    p[:NW1] = rng.uniform(-1, 1, NW1) * np.sqrt(3.0 / FEAT)
    p[NW1:NW1 + NW2] = rng.uniform(-1, 1, NW2) * np.sqrt(3.0 / HID)
    w3 = rng.uniform(-1, 1, (HID, OUTPAD)) * np.sqrt(3.0 / HID)
    w3[:, OUT:] = 0.0
    p[NW1 + NW2:NW1 + NW2 + NW3] = w3.ravel()
    return p
