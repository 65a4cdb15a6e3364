"""Oracle worlds stepped in parallel host processes (test helper).

The pool is started with the "spawn" method: a process forked after the GPU library has
created a CUDA context would inherit it and hang.  Each worker builds its share of the
worlds from their scene dicts, steps them and returns their exported states.
"""
import multiprocessing as mp
import os


def _worker(task):
    import oracle
    scenes_list, steps, trig = task
    oracle.set_trig_mode(trig)
    out = []
    for s in scenes_list:
        w = oracle.OracleWorld(s)
        w.step(steps=steps)
        out.append(w.export_state())
    return out


def step_all(worlds, steps, trig=1, processes=None):
    """Export states of every world after `steps` oracle steps (dt 1/60, 8/3 iterations)."""
    n = processes or max(1, min(len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else 4, 32))
    chunks = [list(range(i, len(worlds), 4 * n)) for i in range(4 * n)]
    chunks = [c for c in chunks if c]
    with mp.get_context("spawn").Pool(n) as pool:
        res = pool.map(_worker, [([worlds[i] for i in c], steps, trig) for c in chunks])
    out = [None] * len(worlds)
    for c, states in zip(chunks, res):
        for i, st in zip(c, states):
            out[i] = st
    return out
