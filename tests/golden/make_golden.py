"""Regenerate the golden fixtures in this folder from the CPU oracle.

    python tests/golden/make_golden.py

Fixtures (numpy .npz, float32 kept bit-exact):
  hello_world.npz  examples/hello_world/hello_world.d:31-103 (dt 1/60, 6/2 iterations, 60 steps):
                   per-step x, y, angle of the box; `libm` uses the host sinf/cosf (the reference's
                   arithmetic), `portable` the dbox_sincosf the GPU library uses.
  pyramid8.npz     8-row pyramid on the box ground, 120 steps of 8/3 iterations, portable trig:
                   full exported state after steps 30, 60 and 120.
  manifolds.npz    300 seeded polygon/circle pairs at random poses: manifold of each pair.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from dbox_gb300 import abi, scenes  # noqa: E402


def hello_world():
    out = {}
    for name, mode in (("libm", 0), ("portable", 1)):
        oracle.set_trig_mode(mode)
        w = oracle.OracleWorld(scenes.hello_world())
        rows = []
        for _ in range(60):
            w.step(1.0 / 60.0, 6, 2)
            b = w.export_state()["bodies"][1]
            rows.append([b["xf"][0], b["xf"][1], b["sweep"][7]])
        out[name] = np.array(rows, np.float32)
    oracle.set_trig_mode(1)
    np.savez(os.path.join(HERE, "hello_world.npz"), **out)


def pyramid8():
    oracle.set_trig_mode(1)
    w = oracle.OracleWorld(scenes.pyramid(rows=8))
    out = {}
    done = 0
    for stop in (30, 60, 120):
        w.step(steps=stop - done)
        done = stop
        st = w.export_state()
        for k, v in st.items():
            out["s%d_%s" % (stop, k)] = v
    np.savez(os.path.join(HERE, "pyramid8.npz"), **out)


def shape_cases(n=300, seed=9):
    rng = np.random.default_rng(seed)
    shapes = np.zeros((n, 2), abi.SHAPE_DEF)
    xfs = np.zeros((n, 2, 4), np.float32)
    for i in range(n):
        for j in range(2):
            s = shapes[i, j]
            kind = rng.integers(0, 3) if j == 0 else rng.integers(0, 2)
            if kind == 0 and j == 0:
                kind = 2
            if kind == 0:
                s["kind"] = abi.SHAPE_CIRCLE
                s["radius"] = rng.uniform(0.2, 0.6)
                s["center"] = rng.uniform(-0.1, 0.1, 2)
            elif kind == 1:
                k = int(rng.integers(3, 9))
                while True:
                    ang = np.sort(rng.uniform(0, 2 * np.pi, k))
                    gaps = np.diff(np.concatenate([ang, ang[:1] + 2 * np.pi]))
                    if gaps.min() > 0.25 and gaps.max() < np.pi:
                        break
                r = rng.uniform(0.3, 0.6)
                s["kind"] = abi.SHAPE_POLYGON
                s["count"] = k
                s["vertices"][:k, 0] = r * np.cos(ang)
                s["vertices"][:k, 1] = r * np.sin(ang)
            else:
                s["kind"] = abi.SHAPE_BOX
                s["hx"] = rng.uniform(0.2, 0.7)
                s["hy"] = rng.uniform(0.2, 0.7)
            a = rng.uniform(-3.2, 3.2)
            xfs[i, j] = [rng.uniform(-0.6, 0.6) if j else 0.0, rng.uniform(-0.6, 0.6) if j else 0.0,
                         np.float32(np.sin(a)), np.float32(np.cos(a))]
    return shapes, xfs


def manifolds():
    shapes, xfs = shape_cases()
    out = np.zeros(len(shapes), abi.CONTACT_STATE)
    for i in range(len(shapes)):
        a, b = shapes[i, 0], shapes[i, 1]
        if a["kind"] == abi.SHAPE_CIRCLE:
            a, b = b, a
        out[i] = oracle.collide(a, xfs[i, 0], b, xfs[i, 1])
    np.savez(os.path.join(HERE, "manifolds.npz"), shapes=shapes, xfs=xfs, manifolds=out)


if __name__ == "__main__":
    oracle.build()
    hello_world()
    pyramid8()
    manifolds()
    print("golden fixtures written to", HERE)
