"""Benchmark: body-steps/s of b2World.Step on one GB300 (plain solver, batched worlds).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload batch|scatter|pyramid|stress|train]

Workload (default "batch"): 4,096 independent worlds in one handle, body counts
log-uniform in [8, 512], one third each pyramid / scatter in a 40 m container /
box stacks (dbox_gb300.scenes.batch), float32, dt = 1/60, 8 velocity and 3 position
iterations.  A "step" is one b2World.Step of every world.  The timed steps follow
W untimed warm-up steps, so the timed window is steps W+1 .. W+K of the simulation.

value  = dynamic body-steps / device time of K steps replayed from one CUDA graph
         (world state resident in HBM; CUDA events on the library's stream).
e2e    = the same K steps (on a twin handle built from the same scenes and warmed up
         the same way) through the C ABI from host buffers: each step uploads a
         (fx, fy, torque) array for every body from pinned host memory
         (dbox_world_apply_forces; zero forces, so the trajectory is unchanged),
         steps, and reads every body's (x, y, angle) back into pinned memory
         (dbox_world_get_transforms); host wall clock around the K steps.
cpu_baseline / --impl reference: the CPU oracle (a C++ restatement of the dbox
         step; the D reference cannot be compiled on these machines) on every world
         of the workload and the same step window, worlds spread largest first over
         all host cores, wall clock of the whole pool.
Under torchrun each rank runs its own 4,096-world batch (weak scaling, no
collective on the data path); rank 0 prints the max-over-ranks timing.
"""
import argparse
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

DT = 1.0 / 60.0
VI, PI = 8, 3
METRIC = "body-steps/s on 1 GB300 (plain GPU solver, batched worlds)"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=60)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="batch", choices=["batch", "scatter", "pyramid", "stress", "train"],
                   help="train: the learned warm-start MLP's Adam training alone, on synthetic device rows")
    p.add_argument("--train-rows", type=int, default=1 << 20)
    p.add_argument("--train-epochs", type=int, default=3)
    p.add_argument("--worlds", type=int, default=4096)
    p.add_argument("--seed", type=int, default=3)
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-learned", action="store_true", help="skip the learned warm-start comparison")
    p.add_argument("--no-autotune", action="store_true", help="keep the default world-to-block mapping")
    p.add_argument("--mapping", default="auto", choices=["auto", "default", "queue"],
                   help="auto: the autotuner's choice; default: default block packing; queue: world queue")
    p.add_argument("--queries", type=int, default=1 << 20, help="rays / boxes per world-query batch")
    p.add_argument("--no-queries", action="store_true", help="skip the world-query measurement")
    p.add_argument("--learned-worlds", type=int, default=1024)
    p.add_argument("--learned-log-steps", type=int, default=2000)
    p.add_argument("--stress-warmup", type=int, default=60, help="steps before the stress world is measured")
    p.add_argument("--stress-steps", type=int, default=3)
    p.add_argument("--no-stress", action="store_true", help="skip the large-island stress world")
    p.add_argument("--fused-step", action="store_true",
                   help="whole steps in one launch (dbox_world_set_fused_step) instead of four launches a step")
    return p.parse_args()


def make_worlds(args, rank):
    from dbox_gb300 import scenes
    from dbox_gb300.dist import rank_seed
    if args.workload == "batch":
        return scenes.batch(n_worlds=args.worlds, seed=rank_seed(args.seed, rank)), {
            "workload": "batched worlds: %d worlds, bodies log-uniform [8,512], thirds pyramid/scatter/stacks"
                        % args.worlds, "worlds": args.worlds}
    if args.workload == "scatter":
        return [scenes.scatter_world(seed=rank_seed(args.seed, rank))], {
            "workload": "single world: 16,384 mixed circles/polygons in a 200x400 m container", "worlds": 1}
    if args.workload == "stress":
        return [scenes.stress(seed=rank_seed(args.seed, rank))], {
            "workload": "single world: 64 container piles x 2,048 mixed circles/polygons + 256 revolute chains "
                        "x 32 links", "worlds": 1}
    return [scenes.pyramid()], {"workload": "single world: 20-row pyramid, 210 boxes", "worlds": 1}


def dynamic_bodies(worlds):
    from dbox_gb300 import scenes
    return sum(scenes.dynamic_body_count(s) for s in worlds)


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ CPU oracle legs
def _cpu_worker(scenes_list, warmup, steps, barrier, out):
    """One host core: build the oracle worlds of its share, step them through the warm-up,
    wait for every core at the barrier, then time steps warmup+1 .. warmup+steps."""
    import oracle
    from dbox_gb300 import scenes
    oracle.set_trig_mode(0)
    ows = [oracle.OracleWorld(s) for s in scenes_list]
    for w in ows:
        w.step(DT, VI, PI, steps=warmup)
    barrier.wait()
    t0 = time.monotonic()
    for w in ows:
        w.step(DT, VI, PI, steps=steps)
    t1 = time.monotonic()
    out.put((t0, t1, sum(scenes.dynamic_body_count(s) for s in scenes_list) * steps))


def _cpu_cost_worker(task):
    """Calibration (untimed): per world, the time of the timed window (steps warmup+1 ..
    warmup+steps) on one core."""
    import oracle
    scenes_list, warmup, steps = task
    oracle.set_trig_mode(0)
    out = []
    for s in scenes_list:
        w = oracle.OracleWorld(s)
        w.step(DT, VI, PI, steps=warmup)
        t0 = time.perf_counter()
        w.step(DT, VI, PI, steps=steps)
        out.append(time.perf_counter() - t0)
    return out


def lpt_shares(costs, bins):
    """Longest-processing-time assignment: items by cost, largest first, each to the least
    loaded bin; returns the item indices of each non-empty bin."""
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * bins
    out = [[] for _ in range(bins)]
    for i in order:
        k = min(range(bins), key=lambda b: (load[b], b))
        out[k].append(i)
        load[k] += costs[i]
    return [o for o in out if o]


def cpu_leg(args, worlds=None):
    """The oracle step (dbox's float32 step restated in C++, host libm trig) on the host cores,
    on every world of the workload and the same step window as the GPU leg: worlds spread over
    all cores largest first (one world list per core), each core warms its worlds up, a barrier,
    then the wall clock of the whole pool's timed steps.  Returns (body-steps/s, cores, sample)."""
    import oracle
    from dbox_gb300 import scenes
    oracle.build()
    if worlds is None:
        worlds, _ = make_worlds(args, 0)
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    ctx = mp.get_context("spawn")
    # per-world cost from an untimed calibration pass over all worlds (the cost per body differs
    # between pyramids, stacks and scatter worlds), then a largest-first assignment
    nb = min(cores, len(worlds))
    if len(worlds) == 1:
        shares = [[0]]                            # one world: one core, nothing to balance
    else:
        chunks = [list(range(i, len(worlds), 4 * nb)) for i in range(4 * nb)]
        chunks = [c for c in chunks if c]
        with ctx.Pool(nb) as pool:
            timed = pool.map(_cpu_cost_worker, [([worlds[i] for i in c], args.warmup, args.steps) for c in chunks])
        costs = [0.0] * len(worlds)
        for c, t in zip(chunks, timed):
            for i, v in zip(c, t):
                costs[i] = v
        shares = lpt_shares(costs, nb)
    barrier = ctx.Barrier(len(shares))
    out = ctx.Queue()
    procs = [ctx.Process(target=_cpu_worker, args=([worlds[i] for i in sh], args.warmup, args.steps, barrier, out))
             for sh in shares]
    for p in procs:
        p.start()
    res = [out.get() for _ in procs]
    for p in procs:
        p.join()
        if p.exitcode != 0:
            raise RuntimeError("CPU oracle worker failed (exit code %s)" % p.exitcode)
    wall = max(r[1] for r in res) - min(r[0] for r in res)
    work = sum(r[2] for r in res)
    busy = [r[1] - r[0] for r in res]
    if len(worlds) == 1:
        sample = ("the one world, steps %d..%d, one process (one core); wall clock %.2f s; oracle with host libm trig"
                  % (args.warmup + 1, args.warmup + args.steps, wall))
    else:
        sample = ("%d of %d worlds, steps %d..%d, %d processes (worlds spread costliest first over the cores, "
                  "costs from an untimed calibration pass), "
                  "wall clock of the pool; per-process busy %.2f-%.2f s; oracle with host libm trig"
                  % (len(worlds), len(worlds), args.warmup + 1, args.warmup + args.steps, len(shares), min(busy),
                     max(busy)))
    return work / wall, len(shares), sample


# ------------------------------------------------------------------ GPU leg
def algorithmic_solve_bytes(c):
    """Bytes the solve part of the fused solve + SolveTOI kernel must move, by the reference
    struct sizes (the SolveTOI part is not counted, so the figure is a lower bound):
    96 per island body (integrate + copy back), per island contact 244 (b2ContactVelocity/
    PositionConstraint build) + 156 (velocity init) + 16 (store impulses), 220 per contact
    velocity solve (vc 156 + two 24-byte body states read and written, 16 of impulses) and
    136 per contact position solve (pc 88 + two 24-byte positions)."""
    return 96 * c["isl_bodies"] + (244 + 156 + 16) * c["isl_contacts"] + 220 * c["vsolve"] + 136 * c["psolve"]


def solver_chain(w):
    """Cycles per Gauss-Seidel level of the deepest world, from one profiled step (clock64
    stamps at the solve kernel's phase boundaries): the velocity sweeps' cycles over (levels x
    velocity iterations), the position sweeps' over (levels x position iterations, the most
    that can run before the early exit)."""
    w.set_phase_profile(True)
    w.step(DT, VI, PI)
    p = w.phase_profile().astype(np.int64)
    w.set_phase_profile(False)
    span = p[:, 11] - p[:, 0]
    k = int(np.argmax(span))
    lv = int(p[k, 12])
    if lv <= 0:
        return None
    return {"world": k, "bodies": int(p[k, 14]), "contacts": int(p[k, 13]), "levels": lv,
            "solve_cycles": int(span[k]),
            "velocity_cycles_per_level": float(p[k, 6] - p[k, 5]) / (lv * VI),
            "position_cycles_per_level": float(p[k, 8] - p[k, 7]) / (lv * PI)}


def gpu_leg(args, rank, world_size):
    import torch
    import dbox_gb300
    from dbox_gb300.dist import max_over_ranks
    dbox_gb300.build()
    torch.cuda.set_device(0 if world_size == 1 else int(os.environ.get("LOCAL_RANK", rank)))
    worlds, cfg = make_worlds(args, rank)
    nbody_dyn = dynamic_bodies(worlds)
    nbody = sum(len(s["bodies"]) for s in worlds)
    # the autotuner picks the world-to-block mapping on a throwaway handle of the same worlds
    # (it advances the worlds it times); the measured handles then use that mapping
    mapping = None
    if args.mapping == "queue":
        mapping = (0, 0, 0, 1, 0, 0)
        costs = None
    elif not args.no_autotune and args.mapping == "auto":
        wt = dbox_gb300.World(worlds)
        wt.set_fused_step(args.fused_step)
        wt.step(DT, VI, PI, steps=args.warmup, graph=True)
        mapping = wt.autotune(steps=3, dt=DT, vel_iters=VI, pos_iters=PI)
        costs = wt.world_costs()
        wt.close()
    w = dbox_gb300.World(worlds)
    # twin handle for the end-to-end leg: the same scenes and warm-up, so it replays exactly
    # the steps the device-timed leg measures
    we = dbox_gb300.World(worlds)
    for h in (w, we):
        h.set_fused_step(args.fused_step)
    if mapping:
        for h in (w, we):
            if costs is not None:
                h.set_world_costs(costs)
            h.apply_mapping(mapping)
    w.step(DT, VI, PI, steps=args.warmup, graph=True)
    we.step(DT, VI, PI, steps=args.warmup, graph=True)
    w.sync()
    we.sync()
    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    c0 = w.counters()
    if world_size > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    total_ms, phase_ms = w.step_timed(args.steps, DT, VI, PI)
    clk = clocks.stop()
    c1 = w.counters()
    cdiff = {k: c1[k] - c0[k] for k in c1}
    total_ms_max = max_over_ranks(total_ms, "cuda")
    value = nbody_dyn * args.steps * world_size / (total_ms_max / 1e3)
    launches = w.last_launches()                 # kernels of the timed call, all its steps
    fused = w.fused_step() and phase_ms[0] == 0.0
    # end to end through the C ABI with pinned host buffers
    forces = torch.zeros((nbody, 3), dtype=torch.float32).pin_memory().numpy()
    xya = torch.zeros((nbody, 3), dtype=torch.float32).pin_memory().numpy()
    if world_size > 1:
        torch.distributed.barrier()
    we.sync()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        we.apply_forces(forces)
        we.step(DT, VI, PI)
        we.get_transforms(xya)
    e2e_s = time.perf_counter() - t0
    e2e = nbody_dyn * args.steps * world_size / max_over_ranks(e2e_s, "cuda")
    assert np.isfinite(xya).all()
    solve_bytes = algorithmic_solve_bytes(cdiff) / args.steps
    solve_ms = phase_ms[1] / args.steps          # the solve + SolveTOI kernel (the whole step when fused)
    achieved = solve_bytes / (solve_ms / 1e3) / 1e9
    hbm = peaks.get("hbm_gbs")
    chain = solver_chain(w)
    out = {
        "metric": METRIC, "value": value, "unit": "body-steps/s", "n_gpus": world_size, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic seeded scenes (numpy PCG64 seed %d)" % args.seed,
        "config": dict(cfg, dt=DT, velocity_iterations=VI, position_iterations=PI, dynamic_bodies=nbody_dyn,
                       parallelism="replicas: one batch of worlds per GPU",
                       mapping=mapping_report(mapping, args.mapping),
                       l2="working set (bodies, contacts, constraint rows) larger than the 129 MB L2",
                       timing=("one launch of K whole steps (k_step_fused), CUDA events around it" if fused else
                               "one CUDA graph of K steps with per-phase CUDA events")),
        "e2e": {"value": e2e, "unit": "body-steps/s", "h2d_bytes_per_step": int(forces.nbytes),
                "d2h_bytes_per_step": int(xya.nbytes)},
        "gpu_launches": launches,
        "phases_ms_per_step": ({"whole_step_kernel": solve_ms} if fused else
                               {"collide": phase_ms[0] / args.steps, "solve_and_toi": solve_ms}),
        "work_per_step": {k: v / args.steps for k, v in cdiff.items()},
        # The fused solve + SolveTOI kernel is bound by the dependent Gauss-Seidel chain of the
        # deepest worlds (levels in sequence, each level a few hundred cycles of dependent
        # arithmetic), not by HBM: the bandwidth fraction below is what that chain leaves.
        "roofline": {"bound": "latency", "kernel": "k_step_fused" if fused else "k_solve_toi", "achieved": achieved,
                     "peak": hbm, "unit": "GB/s", "frac": (achieved / hbm) if hbm else None,
                     "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if hbm else "fallback 6800",
                     "algorithmic_bytes_per_launch": solve_bytes,
                     "algorithmic_bytes_cover": "the island solve only (bodies, constraint build, velocity and "
                                                "position solves, impulse store); SolveTOI and Collide not counted"
                                                + ("; the kernel time is the whole step" if fused else ""),
                     "solve_share_of_step": solve_ms / (total_ms_max / args.steps),
                     "traffic": None,
                     "traffic_note": "DRAM bytes come from a separate ncu capture of this kernel, not from the "
                                     "timed run",
                     "critical_chain": chain},
        "clocks": clk,
    }
    if out["roofline"]["peak"] is None:
        out["roofline"]["peak"] = 6800.0
        out["roofline"]["frac"] = achieved / 6800.0
    if world_size == 1 and not args.no_queries:
        out["world_queries"] = queries_leg(args, w, worlds, out["roofline"]["peak"])
    w.close()
    return out, worlds


def _query_inputs(rng, n, worlds, xy):
    """n seeded queries over the worlds: a random world, a random body of it; the ray starts
    within 2 m of the body and runs 8 m in a random direction; the box is 2 m x 2 m around it."""
    nb = np.array([len(s["bodies"]) for s in worlds])
    starts = np.concatenate([[0], np.cumsum(nb)[:-1]])
    wid = rng.integers(0, len(worlds), n).astype(np.int32)
    b = starts[wid] + (rng.random(n) * nb[wid]).astype(np.int64)
    ang = rng.uniform(0.0, 2.0 * np.pi, n)
    p1 = (xy[b] + rng.uniform(-2.0, 2.0, (n, 2))).astype(np.float32)
    p2 = (p1 + 8.0 * np.stack([np.cos(ang), np.sin(ang)], 1)).astype(np.float32)
    boxes = np.concatenate([xy[b] - 1.0, xy[b] + 1.0], 1).astype(np.float32)
    return wid, p1, p2, boxes


def queries_leg(args, w, worlds, hbm_peak):
    """b2World.RayCast (closest hit, all hits) and b2World.QueryAABB as batches of queries over
    the measured handle's worlds after its timed steps.  Device-resident batches are timed
    with CUDA events on the handle's stream, L2 flushed before each timed batch; the index
    build (once per step) is timed on the first batch after one more step; e2e is the host
    API with host arrays; the CPU figure is the oracle's b2DynamicTree walk on a sample."""
    import torch
    import oracle
    n = args.queries
    nbody = sum(len(s["bodies"]) for s in worlds)
    xya = np.zeros((nbody, 3), np.float32)
    w.get_transforms(xya)
    rng = np.random.default_rng(args.seed + 101)
    wid, p1, p2, boxes = _query_inputs(rng, n, worlds, xya[:, :2])
    dev = torch.device("cuda")
    t_w, t_p1, t_p2, t_box = (torch.from_numpy(a).to(dev) for a in (wid, p1, p2, boxes))
    cap_all, cap_box = 16, 32
    t_cnt = torch.zeros(n, dtype=torch.int32, device=dev)
    t_hits = torch.zeros((n, cap_all, 6), dtype=torch.float32, device=dev)        # dbox_ray_hit, 24 bytes
    t_fx = torch.zeros((n, cap_box), dtype=torch.int32, device=dev)
    stream = torch.cuda.ExternalStream(w.stream())
    flush = torch.empty(64 << 20, dtype=torch.float32, device=dev)              # 256 MB, twice the L2

    def run(kind):
        if kind == "query_aabb":
            w.query_aabb_device(n, t_w.data_ptr(), t_box.data_ptr(), cap_box, t_cnt.data_ptr(), t_fx.data_ptr())
        else:
            mode, cap = (0, 1) if kind == "raycast_closest" else (1, cap_all)
            w.raycast_device(n, t_w.data_ptr(), t_p1.data_ptr(), t_p2.data_ptr(), mode, cap, t_cnt.data_ptr(),
                             t_hits.data_ptr())

    def timed(kind, reps):
        ts = []
        for _ in range(reps):
            with torch.cuda.stream(stream):
                flush.fill_(1.0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            run(kind)
            e1.record(stream)
            stream.synchronize()
            ts.append(e0.elapsed_time(e1))
        return float(np.median(ts))

    res = {"queries_per_batch": n,
           "workload": "the bench's worlds after its timed steps; per query a random world and body, a ray from "
                       "within 2 m of the body running 8 m in a random direction, a 2 m x 2 m box around the body"}
    for kind in ("raycast_closest", "raycast_all", "query_aabb"):
        for _ in range(3):
            run(kind)
        ms = timed(kind, 5)
        cnt = t_cnt.cpu().numpy()
        in_bytes = 4 + (16 if kind == "query_aabb" else 16)
        out_bytes = 4 + (4 * np.minimum(cnt, cap_box).mean() if kind == "query_aabb" else
                         24 * np.minimum(cnt, 1 if kind == "raycast_closest" else cap_all).mean())
        gbs = n * (in_bytes + out_bytes) / (ms / 1e3) / 1e9
        res[kind] = {"value": n / (ms / 1e3), "unit": "queries/s", "ms_per_batch": ms,
                     "mean_results": float(cnt.mean()), "io_gbs": gbs, "io_frac_of_hbm": gbs / hbm_peak}
    w.step(DT, VI, PI)                                                           # the index goes stale
    res["raycast_closest"]["ms_first_batch_after_step"] = timed("raycast_closest", 1)
    res["index_build_ms"] = res["raycast_closest"]["ms_first_batch_after_step"] - res["raycast_closest"]["ms_per_batch"]
    # end to end: host arrays in, host arrays out, through the C ABI
    w.raycast(wid[:1024], p1[:1024], p2[:1024], "closest", 1)
    t0 = time.perf_counter()
    w.raycast(wid, p1, p2, "closest", 1)
    e2e_s = time.perf_counter() - t0
    res["raycast_closest"]["e2e"] = {"value": n / e2e_s, "unit": "queries/s", "h2d_bytes": int(n * 20),
                                     "d2h_bytes": int(n * 28)}
    # CPU: the oracle's tree walk (b2DynamicTree.RayCast + b2World.RayCast's wrapper), one core
    if not args.no_cpu:
        sample = list(range(min(len(worlds), 32)))
        oracle.set_trig_mode(0)
        ows = [oracle.OracleWorld(worlds[i]) for i in sample]
        for ow in ows:
            ow.step(DT, VI, PI, steps=args.warmup + args.steps)
        per = 2048
        cpu_t = 0.0
        for ow, i in zip(ows, sample):
            xy = ow.export_state()["bodies"]["xf"][:, :2].astype(np.float32)
            _, a, b, _ = _query_inputs(np.random.default_rng(args.seed + i), per, [worlds[i]], xy)
            t0 = time.perf_counter()
            ow.raycast_many(a, b, "closest", 1)
            cpu_t += time.perf_counter() - t0
        res["raycast_closest"]["cpu_baseline"] = {
            "value": per * len(sample) / cpu_t, "unit": "queries/s", "cores": 1, "kind": "port",
            "sample": "%d rays in each of the first %d worlds, oracle stepped %d steps, one core"
                      % (per, len(sample), args.warmup + args.steps)}
    return res


def learned_leg(args):
    """Learned warm start vs the plain solver (the project's learned-start configuration):
    1,024 scatter worlds of 256 bodies in 40 m containers.  The plain solver logs up to 10M
    new-contact samples over its first steps; the MLP (32-128-128-4, BF16 tensor cores) is
    trained with Adam (lr 1e-3, batch 65,536, 20 epochs); then new-seed worlds run plain with
    8 and 5 velocity iterations and learned with 5 and 4, each from the same warmed-up state:
    velocity residual (one extra non-mutating sweep per step), deepest penetration and
    body-steps/s (CUDA graph of the timed steps, measurement off)."""
    import dbox_gb300
    from dbox_gb300 import scenes
    rng = np.random.default_rng(args.seed + 77)
    train_worlds = [scenes.scatter(256, 40.0, 40.0, rng) for _ in range(args.learned_worlds)]
    eval_worlds = [scenes.scatter(256, 40.0, 40.0, rng) for _ in range(args.learned_worlds)]
    nd = sum(scenes.dynamic_body_count(s) for s in eval_worlds)
    log = dbox_gb300.World(train_worlds)
    log.set_warmstart(1, None, 10_000_000)
    t0 = time.perf_counter()
    log.step(DT, VI, PI, steps=args.learned_log_steps, graph=True)
    log.sync()
    t_log = time.perf_counter() - t0
    n = log.sample_count()
    f, tg = log.samples(0, min(n, 1_000_000))
    model = dbox_gb300.Mlp(seed=args.seed)
    model.fit_normalization(f, tg)
    t0 = time.perf_counter()
    losses = model.train_world(log, epochs=20, batch=65536, lr=1e-3, seed=args.seed)
    t_train = time.perf_counter() - t0
    log.close()
    res = {}
    for label, mode, vi in (("plain_8", 0, 8), ("plain_5", 0, 5), ("learned_5", 2, 5), ("learned_4", 2, 4)):
        w = dbox_gb300.World(eval_worlds)
        w.step(DT, VI, PI, steps=100, graph=True)
        w.set_warmstart(mode, model if mode == 2 else None, 0)
        w.set_measure(True)
        rms, mx, pen = [], [], []
        for _ in range(30):
            w.step(DT, vi, PI)
            q = w.quality()
            rms.append(float(np.sqrt(q[:, 0].sum() / max(q[:, 2].sum(), 1.0))))
            mx.append(float(q[:, 1].max()))
            pen.append(float(-q[:, 3].min()))
        w.set_measure(False)
        w.step(DT, vi, PI, steps=3, graph=True)
        tot_ms, _ = w.step_timed(30, DT, vi, PI)
        res[label] = {"velocity_iterations": vi, "residual_rms": float(np.mean(rms)),
                      "residual_max": float(np.mean(mx)), "penetration_max_m": float(np.max(pen)),
                      "body_steps_per_s": nd * 30 / (tot_ms / 1e3)}
        w.close()
    # upper bound of any learned start: new points start from the impulses a 50-iteration solve
    # of the same step converged to (a perfect prediction), persistent points keep Box2D's
    # warm start; each step a twin handle copies the state, takes the 50-iteration step first
    for label, vi in (("perfect_5", 5), ("perfect_4", 4)):
        w = dbox_gb300.World(eval_worlds)
        src = dbox_gb300.World(eval_worlds)
        w.step(DT, VI, PI, steps=100, graph=True)
        src.step(DT, VI, PI)
        w.set_warmstart(3)
        w.set_start_source(src)
        w.set_measure(True)
        rms, mx, pen = [], [], []
        for _ in range(30):
            src.copy_state_from(w)
            src.step(DT, 50, PI)
            w.step(DT, vi, PI)
            q = w.quality()
            rms.append(float(np.sqrt(q[:, 0].sum() / max(q[:, 2].sum(), 1.0))))
            mx.append(float(q[:, 1].max()))
            pen.append(float(-q[:, 3].min()))
        res[label] = {"velocity_iterations": vi, "residual_rms": float(np.mean(rms)),
                      "residual_max": float(np.mean(mx)), "penetration_max_m": float(np.max(pen)),
                      "start": "new points from the converged impulses of a 50-iteration solve of the same step"}
        w.close()
        src.close()
    p8, l5 = res["plain_8"], res["learned_5"]
    u5 = res["perfect_5"]
    args._model = model                        # for the large-island stress leg
    return {
        "config": "%d scatter worlds x 256 bodies (40 m containers), dt 1/60, %d position iterations; "
                  "samples from %d plain steps, evaluation on new-seed worlds after 100 steps, 30 steps"
                  % (args.learned_worlds, PI, args.learned_log_steps),
        "samples": n, "log_seconds": t_log, "train_seconds": t_train,
        # forward 2 (32*128 + 128*128 + 128*4) FLOP per sample, training about 3x that
        "train_tflops": 3 * 41984 * n * 20 / t_train / 1e12,
        "train_kernel": "k_mlp_train: tcgen05.mma (bf16 in shared memory, f32 accumulators in tensor memory)",
        "loss_first_epoch": float(losses[0]), "loss_last_epoch": float(losses[-1]),
        "runs": res,
        "speedup_learned_5_vs_plain_8": l5["body_steps_per_s"] / p8["body_steps_per_s"],
        "learned_5_reaches_plain_8_residual": bool(l5["residual_rms"] <= p8["residual_rms"] and
                                                   l5["residual_max"] <= p8["residual_max"]),
        "perfect_start_5_reaches_plain_8_residual": bool(u5["residual_rms"] <= p8["residual_rms"] and
                                                         u5["residual_max"] <= p8["residual_max"]),
    }


def stress_leg(args, model):
    """The large-island stress world: one world of 64 container piles x 2,048 mixed circles /
    polygons (one large island per pile) and 256 revolute chains x 32 links hanging into them.
    Plain 8/3 iterations and the learned start with 5 velocity iterations, each from the same
    warmed-up state: body-steps/s (CUDA events), velocity residual and penetration, and the
    algorithmic bandwidth of the solve phase."""
    import dbox_gb300
    from dbox_gb300 import scenes
    s = scenes.stress(seed=args.seed)
    nd = scenes.dynamic_body_count(s)
    base = dbox_gb300.World(s)
    base.step(DT, VI, PI, steps=args.stress_warmup, graph=True)
    res = {"config": "1 world: 64 piles x 2,048 bodies + 256 chains x 32 links, %d dynamic bodies; steps %d..%d"
                     % (nd, args.stress_warmup + 1, args.stress_warmup + args.stress_steps), "dynamic_bodies": nd}
    runs = [("plain_8", 0, VI), ("learned_5", 2, 5)] if model is not None else [("plain_8", 0, VI)]
    for label, mode, vi in runs:
        w = dbox_gb300.World(s)
        w.step()                                  # on the device, then the same state as `base`
        w.copy_state_from(base)
        w.set_warmstart(mode, model if mode == 2 else None, 0)
        w.set_measure(True)
        rms, mx, pen = [], [], []
        for _ in range(2):
            w.step(DT, vi, PI)
            q = w.quality()
            rms.append(float(np.sqrt(q[:, 0].sum() / max(q[:, 2].sum(), 1.0))))
            mx.append(float(q[:, 1].max()))
            pen.append(float(-q[:, 3].min()))
        w.set_measure(False)
        c0 = w.counters()
        tot_ms, ph = w.step_timed(args.stress_steps, DT, vi, PI)
        c1 = w.counters()
        cd = {k: (c1[k] - c0[k]) / args.stress_steps for k in c1}
        solve_ms = ph[1] / args.stress_steps
        res[label] = {"velocity_iterations": vi, "body_steps_per_s": nd * args.stress_steps / (tot_ms / 1e3),
                      "ms_per_step": tot_ms / args.stress_steps, "residual_rms": float(np.mean(rms)),
                      "residual_max": float(np.mean(mx)), "penetration_max_m": float(np.max(pen)),
                      "phases_ms_per_step": {"collide": ph[0] / args.stress_steps, "solve_and_toi": solve_ms},
                      "solve_algorithmic_gbs": algorithmic_solve_bytes(cd) / (solve_ms / 1e3) / 1e9,
                      "collide_contacts_per_step": cd["contacts"]}
        w.close()
    base.close()
    return res


def mapping_report(mapping, how):
    """The world-to-warp mapping of the measured handles, for the JSON line."""
    if not mapping:
        return "default"
    by = "autotuner" if how == "auto" else "--mapping " + how
    if mapping[3]:
        return {"queue": 1, "heavy_worlds_one_per_subpartition": mapping[4], "exclusive": mapping[5], "chosen_by": by}
    return {"warps_per_block": mapping[0], "body_budget": mapping[1], "isolated_largest_worlds": mapping[2],
            "chosen_by": by}


def train_only(args):
    """The MLP trainer alone: --train-rows normal random rows (32 features, 4 targets) resident
    in device memory, one untimed epoch, then --train-epochs epochs of Adam in batches of
    65,536 (dbox_mlp_train_device), timed on the host around the synchronous call."""
    import torch
    import dbox_gb300
    rng = np.random.default_rng(args.seed)
    n = args.train_rows
    f = rng.normal(size=(n, 32)).astype(np.float32)
    t = rng.normal(size=(n, 4)).astype(np.float32)
    m = dbox_gb300.Mlp(seed=args.seed)
    m.fit_normalization(f, t)
    rows = torch.from_numpy(np.concatenate([f, t], 1)).cuda()
    m.train_device(rows.data_ptr(), n, epochs=1, batch=65536, lr=1e-3, seed=args.seed)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    loss = m.train_device(rows.data_ptr(), n, epochs=args.train_epochs, batch=65536, lr=1e-3, seed=args.seed)
    dt = time.perf_counter() - t0
    flop = 3.0 * 41984.0 * n * args.train_epochs
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    bf = json.load(open(pk)).get("bf16_tflops") if os.path.exists(pk) else None
    out = {"metric": "MLP training TFLOP/s (learned warm-start network, Adam, batch 65,536)",
           "value": flop / dt / 1e12, "unit": "TFLOP/s", "n_gpus": 1, "higher_is_better": True, "dtype": "bf16",
           "data": "synthetic normal rows (seed %d), device resident" % args.seed,
           "config": {"workload": "MLP 32-128-128-4 training", "rows": n, "epochs": args.train_epochs},
           "seconds": dt, "loss": [float(v) for v in loss],
           "peak": bf or 1900.0, "peak_source": "measured (MEASURED_PEAKS.json bf16_tflops)" if bf else "fallback 1900"}
    out["frac"] = out["value"] / out["peak"]
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    world_size = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.workload == "train":
        if rank == 0 and args.impl == "ours":
            train_only(args)
        elif rank == 0:
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no trainer for this network"}))
        return
    if args.impl == "reference":
        if rank != 0:
            return
        worlds, cfg = make_worlds(args, 0)
        rate, cores, sample = cpu_leg(args, worlds)
        out = {"metric": METRIC, "value": rate, "unit": "body-steps/s", "n_gpus": world_size, "steps": args.steps,
               "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
               "dtype": "f32", "data": "synthetic seeded scenes (numpy PCG64 seed %d)" % args.seed,
               "impl": "reference",
               "config": dict(cfg, dt=DT, velocity_iterations=VI, position_iterations=PI,
                              dynamic_bodies=dynamic_bodies(worlds)),
               "cpu_baseline": {"value": rate, "unit": "body-steps/s", "cores": cores, "kind": "port",
                                "sample": sample},
               "e2e": {"value": rate, "unit": "body-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(out), flush=True)
        return
    if world_size > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    out, worlds = gpu_leg(args, rank, world_size)
    if rank == 0:
        if world_size == 1 and not args.no_learned:
            out["learned_warmstart"] = lw = learned_leg(args)
            pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
            bf = json.load(open(pk)).get("bf16_tflops") if os.path.exists(pk) else None
            lw["train_tflops_peak"] = bf or 1900.0
            lw["train_tflops_peak_source"] = "measured (MEASURED_PEAKS.json bf16_tflops)" if bf else "fallback 1900"
            lw["train_tflops_frac"] = lw["train_tflops"] / lw["train_tflops_peak"]
        if world_size == 1 and not args.no_stress and args.workload == "batch":
            out["large_island_stress"] = stress_leg(args, getattr(args, "_model", None))
        if world_size == 1 and not args.no_cpu:
            rate, cores, sample = cpu_leg(args, worlds)
            out["cpu_baseline"] = {"value": rate, "unit": "body-steps/s", "cores": cores, "kind": "port",
                                   "sample": sample}
        print(json.dumps(out), flush=True)
    if world_size > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
