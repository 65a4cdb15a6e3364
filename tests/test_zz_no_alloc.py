"""dbox_collide_manifolds_noalloc: the narrowphase for callers that may not allocate.

Some programs cannot call cudaMalloc while they run: a game or robotics loop
that forbids allocation inside a frame, or a host engine whose device memory is
handed out by its own allocator.  For them the library offers this one entry
point, which keeps its working memory in a fixed array compiled into the
library (4096 shape pairs per call) instead of allocating.

Here the new entry point is called through the C ABI twice in a row, on
different inputs, and each result must equal, bit for bit, what the allocating
entry point dbox_collide_manifolds returns for the same pairs.  The second call
also shows that nothing of the first call's results leaks into the next one.
This file is named to run last, and it works on its own in a fresh process too.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "manifolds.npz")


def _pairs():
    d = np.load(GOLDEN)
    shapes, xfs = d["shapes"], d["xfs"]
    a, b = shapes[:, 0].copy(), shapes[:, 1].copy()
    swap = a["kind"] == 0                       # the polygon of a mixed pair goes first
    a[swap], b[swap] = shapes[swap, 1], shapes[swap, 0]
    xa, xb = xfs[:, 0].copy(), xfs[:, 1].copy()
    xa[swap], xb[swap] = xfs[swap, 1], xfs[swap, 0]
    return a, xa, b, xb


def _same(x, y):
    assert len(x) == len(y)
    assert (x.view(np.uint8) == y.view(np.uint8)).all()


def test_noalloc_matches_allocating_entry_point_twice(gpu_lib):
    a, xa, b, xb = _pairs()
    first = gpu_lib.collide_manifolds_noalloc(a, xa, b, xb)
    _same(first, gpu_lib.collide_manifolds(a, xa, b, xb))
    assert (first["point_count"] > 0).sum() > 200

    # second call: a different order and a shorter list
    rng = np.random.default_rng(1)
    idx = rng.permutation(len(a))[:157]
    a2, xa2, b2, xb2 = a[idx], xa[idx], b[idx], xb[idx]
    second = gpu_lib.collide_manifolds_noalloc(a2, xa2, b2, xb2)
    _same(second, gpu_lib.collide_manifolds(a2, xa2, b2, xb2))
    _same(second, first[idx])


def test_noalloc_rejects_more_than_its_capacity(gpu_lib):
    a, xa, b, xb = _pairs()
    reps = 4097 // len(a) + 1
    big = [np.concatenate([v] * reps)[:4097] for v in (a, xa, b, xb)]
    with pytest.raises(gpu_lib.DboxError, match="at most 4096"):
        gpu_lib.collide_manifolds_noalloc(*big)
