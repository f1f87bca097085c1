"""Benchmark: batched ODE world stepping (collide + QuickStep) on GB300.

Workload (one "step" = one collide+QuickStep step of every world of the batch):
4096 independent worlds, N in [4,64] bodies log-uniform (spheres r U[0.1,0.5]
or boxes edges U[0.2,1.0], density 1000), ~25% of bodies in ball-joint chains
of 2-6 links, on plane z=0; mu=0.5, Approx1|SoftERP|SoftCFM, erp 0.2,
cfm 1e-5, dt=0.01, 20 iterations, w=1.3, <=4 contacts per pair; seeded
synthetic scene. Metric: world-steps/s (higher is better).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU restatement of ODE's algorithm (the oracle
port, oracle/liboracle.so) on a bounded sample of the same workload with all
host threads.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "ode-0.12_gb300"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

METRIC = "world-steps/s, batched collide+QuickStep (4096 worlds)"
N_WORLDS = 4096
WORKLOAD = "batched_worlds: 4096 worlds, N~logU[4,64] spheres/boxes, 25% ball chains, plane"
SCENE_SEED = 1
# The timed window starts from the rollout's state at this step: the piles have
# settled (about 130 constraint rows per world), where the steady-state cost
# of a step lies. Steps 0-20 are mostly free fall (about 15 rows per world).
SETTLE_STEP = 150
# CPU timings repeat their window from the same state until at least this long
CPU_MIN_SECONDS = 2.0


def _set_worlds(n):
    """Resize the batched workload (profiling of a smaller case)."""
    global N_WORLDS, WORKLOAD, METRIC
    if n < 1:
        raise SystemExit("--worlds must be >= 1")
    WORKLOAD = WORKLOAD.replace(f"{N_WORLDS} worlds", f"{n} worlds")
    METRIC = METRIC.replace(f"({N_WORLDS} worlds)", f"({n} worlds)")
    N_WORLDS = n


def bench_config(steps, iters=20):
    """The workload description both arms print (identical for the same
    --steps)."""
    return {"workload": WORKLOAD, "n_worlds": N_WORLDS, "iterations": iters, "dt": 0.01,
            "rollout": f"steps {SETTLE_STEP}..{SETTLE_STEP + steps - 1} of the rollout (state at step "
                       f"{SETTLE_STEP} reached untimed)",
            "l2": "flushed between timed GPU steps (256 MB write)"}


def rank_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def rank_scene_seed(rank):
    """Weak scaling: every rank steps its own batch of the workload, seeded by rank."""
    return SCENE_SEED + rank


def max_over_ranks(value, device="cpu"):
    """Max of a per-rank number over the process group (the value itself
    without one): the timed region ends when the slowest rank ends."""
    import torch
    import torch.distributed as tdist
    if not (tdist.is_available() and tdist.is_initialized()) or tdist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return float(t.item())


def build_scene(n_worlds, seed=SCENE_SEED):
    from odegpu import scene as S
    return S.batched_worlds(n_worlds=n_worlds, seed=seed)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    def __init__(self, gpu_index=0):
        self.proc = None
        self.lines = []
        self.idx = gpu_index

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(mx)) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def algorithmic_bytes(sc, nc, nr, iters=20):
    """Sweep-model bytes of one batched step: per world
    208*nb + 56*nc + sum_joints Bj + m*(248 + 236*iters) (ball joint Bj=40)."""
    nb = np.diff(sc.body_off)
    nj = np.diff(sc.joint_off)
    return float(np.sum(208.0 * nb + 56.0 * nc + 40.0 * nj + nr * (248.0 + 236.0 * iters)))


def solve_bytes(nr, iters=20):
    """Sweep-model bytes of one world_solve_kernel launch: 236 B per
    row-iteration (J', iMJ, b', Ad', lo, hi, findex, jb, order = 32 words; lambda
    r/w; lambda[findex]; fc r/w of two bodies)."""
    return float(np.sum(nr) * 236.0 * iters)


SOLVE_PROFILE = os.path.join(ROOT, "profiles", "world_solve_kernel_batched_512_settled.md")


def solve_traffic_per_row_iter():
    """DRAM bytes (read + write) per row-iteration of one world_solve_kernel
    launch, from the committed ncu capture summary (None without it)."""
    try:
        with open(SOLVE_PROFILE) as f:
            for line in f:
                if line.startswith("dram_bytes_per_row_iteration:"):
                    return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


def cpu_baseline(sc, n_worlds_sample, n_steps, threads=None):
    """Oracle port (FP64 restatement of ODE's algorithm, oracle/liboracle.so) on
    worlds [0, n_worlds_sample) for n_steps from the initial state, all host
    threads (one world per thread at a time); returns world-steps/s."""
    import oracle_lib as O
    L = O.oracle()
    threads = threads or (os.cpu_count() or 1)
    t0 = time.perf_counter()
    L.oracle_run_worlds(C.byref(sc.c), 0, n_worlds_sample, n_steps, threads, None)
    dt = time.perf_counter() - t0
    return n_worlds_sample * n_steps / dt, threads, dt


def cpu_window(sc, start_step, n_steps, threads=None, min_seconds=CPU_MIN_SECONDS):
    """The oracle port on every world of the workload: its own FP64 rollout
    to `start_step` (untimed), then the window of n_steps steps from that state
    timed on all host threads, repeated from the same state until at least
    min_seconds have been timed. Returns (world-steps/s, threads, seconds
    timed, repeats)."""
    import oracle_lib as O
    threads = threads or (os.cpu_count() or 1)
    x, seeds, _ = O.step_worlds_from(sc, 0, start_step, threads=threads, counts=False)
    done, t_sum, reps = 0, 0.0, 0
    while t_sum < min_seconds or reps == 0:
        t0 = time.perf_counter()
        O.step_worlds_from(sc, start_step, n_steps, state=x, seeds=seeds, threads=threads, counts=False)
        t_sum += time.perf_counter() - t0
        done += sc.n_worlds * n_steps
        reps += 1
    return done / t_sum, threads, t_sum, reps


ADJ_WORKLOAD = ("hinge_chains: 1024 worlds x 8-link hinge chains (0.5x0.1x0.1 m, 1 kg), per-step torques "
                "U[-2,2], plane z=-2, 100 steps, dt 0.01, 20 iterations, checkpoints every 10; "
                "loss |p_end - target|^2")


def run_adjoint(local_rank, reps=3):
    """Batched forward + hand-written adjoint on the differentiable-batch
    workload: world-steps/s of (checkpointed forward rollout + backward), and
    of the forward rollout alone, timed with CUDA events on the batch stream."""
    import torch
    from odegpu import scene as S
    from odegpu.batch import Batch
    n_w, n_steps, ckpt = 1024, 100, 10
    sc = S.hinge_chains(n_worlds=n_w, steps=n_steps)
    B = Batch(sc, device=local_rank)
    stream = torch.cuda.ExternalStream(B.stream_handle())
    seeds = B.seeds()
    x0n = B.state()
    B.step(20)
    B.sync()
    B.autotune(4)
    B.set_state(x0n)
    B.set_seeds(seeds)
    B.set_step_index(0)
    x0 = torch.tensor(x0n, dtype=torch.float32, device="cuda")
    nbt = B.nb_total
    g_final = torch.zeros((nbt, 13), dtype=torch.float32, device="cuda")
    ends = torch.tensor(sc.body_off[1:] - 1, dtype=torch.long, device="cuda")
    g_final[ends, 0:3] = 1.0
    g_init = torch.empty_like(g_final)
    g_jt = torch.zeros((n_steps, B.nj_total, 2), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    fwd_ms, tot_ms = [], []
    launches0 = B.launch_count()
    for r in range(reps + 1):
        B.set_seeds(seeds)
        B.set_step_index(0)
        B.write_state_async(x0.data_ptr())
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        with torch.cuda.stream(stream):
            e0.record(stream)
        B.rollout_forward(n_steps, ckpt)
        with torch.cuda.stream(stream):
            e1.record(stream)
        B.rollout_backward(g_final.data_ptr(), g_init.data_ptr(), g_jt.data_ptr(), None)
        with torch.cuda.stream(stream):
            e2.record(stream)
        B.sync()
        if r > 0:                    # the first repetition is the warm-up
            fwd_ms.append(e0.elapsed_time(e1))
            tot_ms.append(e0.elapsed_time(e2))
    launches = (B.launch_count() - launches0) // (reps + 1)
    status = B.adjoint_status()
    B.close()
    t_tot = float(np.median(tot_ms)) / 1e3
    t_fwd = float(np.median(fwd_ms)) / 1e3
    return {"metric": "world-steps/s, batched forward + adjoint", "value": n_w * n_steps / t_tot,
            "unit": "world-steps/s", "forward_only": n_w * n_steps / t_fwd,
            "ms_forward_plus_backward": 1e3 * t_tot, "ms_forward": 1e3 * t_fwd,
            "workload": ADJ_WORKLOAD, "gpu_launches_per_rollout": int(launches),
            "worlds_with_unmodelled_terms": int((status != 0).sum()),
            "unmodelled_by_bit": {"joint": int(((status & 1) != 0).sum()), "contact": int(((status & 2) != 0).sum()),
                                  "too_large": int(((status & 4) != 0).sum()),
                                  "body_body_case_switch": int(((status & 8) != 0).sum())},
            "gradient_check": "tests/test_gpu_adjoint.py (FP64 central differences of the oracle)"}


def run_vehicles(local_rank, steps=300):
    """Vehicle batch: 2048 cars (box chassis, four sphere wheels on hinge2
    joints) on a 256 x 256 heightfield at 0.5 m, per-step steering stops and
    wheel torques; world-steps/s of the 300-step rollout from the initial
    state, timed with CUDA events on the batch stream."""
    import torch
    from odegpu import scene as S
    from odegpu.batch import Batch
    sc = S.vehicles(n_worlds=2048, steps=steps)
    B = Batch(sc, device=local_rank)
    stream = torch.cuda.ExternalStream(B.stream_handle())
    x0, seeds = B.state(), B.seeds()
    B.step(30)
    B.sync()
    B.autotune(4)
    B.set_state(x0)
    B.set_seeds(seeds)
    B.set_step_index(0)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    B.set_timing(True)
    with torch.cuda.stream(stream):
        e0.record(stream)
    B.step(steps)
    with torch.cuda.stream(stream):
        e1.record(stream)
    B.sync()
    t = e0.elapsed_time(e1) / 1e3
    kern_ms, kern_steps = B.kernel_times()
    B.set_timing(False)
    nc, nr, _ = B.counts()
    status = B.status()
    # forward + adjoint of the final chassis positions with respect to the
    # control sequence (drive torques), checkpoints every 10 steps
    B.set_state(x0)
    B.set_seeds(seeds)
    B.set_step_index(0)
    nbt = B.nb_total
    g_final = torch.zeros((nbt, 13), dtype=torch.float32, device="cuda")
    chassis = torch.tensor(sc.body_off[:-1], dtype=torch.long, device="cuda")
    g_final[chassis, 0:3] = 1.0
    g_jt = torch.zeros((steps, B.nj_total, 2), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        a0.record(stream)
    B.rollout_forward(steps, 10)
    B.rollout_backward(g_final.data_ptr(), None, g_jt.data_ptr(), None)
    with torch.cuda.stream(stream):
        a1.record(stream)
    B.sync()
    t_adj = a0.elapsed_time(a1) / 1e3
    adj_status = B.adjoint_status()
    B.close()
    return {"metric": "world-steps/s, vehicle batch (heightfield + hinge2)", "value": 2048 * steps / t,
            "forward_plus_adjoint": 2048 * steps / t_adj,
            "adjoint_worlds_with_unmodelled_terms": int((adj_status != 0).sum()),
            "unit": "world-steps/s", "ms_per_step": 1e3 * t / steps,
            "workload": "vehicles: 2048 cars (2x1x0.5 m 1000 kg chassis, 4 sphere wheels r 0.35 m 20 kg, "
                        "hinge2 suspension ERP 0.4 CFM 0.01), 256x256 fractal heightfield (0.5 m, sigma 0.3), "
                        "steer U[-0.4,0.4] rad, throttle U[0,1]*400 N m, 300 steps from the initial state",
            "contacts_last_step": int(nc.sum()), "rows_last_step": int(nr.sum()),
            "kernel_ms_per_step": {"collide": kern_ms[0] / max(1, kern_steps),
                                   "setup": kern_ms[1] / max(1, kern_steps),
                                   "solve": kern_ms[2] / max(1, kern_steps)},
            "worlds_with_status": int((status != 0).sum())}


def run_large_world(local_rank, steps=100, cpu_steps=20):
    """Large single world: 10,000 spheres (r U[0.1,0.3] m, density 1000) on a
    jittered grid in a 6 x 6 x 20 m box of five static planes, mu 0.8, 50
    iterations, dt 0.005, stepped by the large-world pipeline; ms per step over
    the first `steps` steps from the initial state (the pile settling), timed
    with CUDA events on the batch stream, and the FP64 oracle port (grid
    broadphase, same canonical pairs) on one host core over the first
    `cpu_steps` steps, against the GPU over the same steps."""
    import torch
    import oracle_lib as O
    from odegpu import scene as S
    from odegpu.batch import Batch
    sc = S.sphere_pile(n=10000)
    B = Batch(sc, device=local_rank)
    stream = torch.cuda.ExternalStream(B.stream_handle())
    x0, seeds = B.state(), B.seeds()
    B.step(3)
    B.sync()

    def timed(n):
        B.set_state(x0)
        B.set_seeds(seeds)
        B.set_step_index(0)
        B.large_world_stats(reset=True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            e0.record(stream)
        B.step(n)
        with torch.cuda.stream(stream):
            e1.record(stream)
        B.sync()
        return e0.elapsed_time(e1) / 1e3, B.large_world_stats(reset=True)

    t_cpu_span, _ = timed(cpu_steps)
    t, st = timed(steps)
    nc, nr, ni = B.counts()
    status = int(B.status()[0])
    B.close()
    t0 = time.perf_counter()
    O.run_world(O.oracle().oracle_run_world, sc, 0, cpu_steps, max_rec=1)
    t_cpu = time.perf_counter() - t0
    return {"metric": "steps/s, one 10k-sphere world", "value": steps / t, "unit": "steps/s",
            "ms_per_step": 1e3 * t / steps,
            "workload": "large world: 10,000 spheres r U[0.1,0.3] m, density 1000, jittered grid in a 6x6x20 m box "
                        "of 5 static planes, mu 0.8, 50 iterations, w 1.3, dt 0.005; first %d steps from the "
                        "initial state" % steps,
            "contacts_last_step": int(nc[0]), "rows_last_step": int(nr[0]), "islands_last_step": int(ni[0]),
            "status": status,
            "phase_ms_per_step": {"island_walk": st["walk_ms"] / steps, "levels": st["sweep_first_ms"] / steps,
                                  "level_sort": st["sort_ms"] / steps,
                                  "level_sweeps": st["sweep_rest_ms"] / steps},
            "levels_max": st["levels_max"], "sweep_cluster_ctas": st["cluster"],
            "cpu_port": {"ms_per_step": 1e3 * t_cpu / cpu_steps, "cores": 1,
                         "sample": f"FP64 oracle port, first {cpu_steps} steps from the initial state",
                         "gpu_ms_per_step_same_steps": 1e3 * t_cpu_span / cpu_steps,
                         "gpu_speedup_same_steps": (t_cpu / cpu_steps) / (t_cpu_span / cpu_steps)}}


def run_exact(local_rank, steps=100, cpu_worlds=N_WORLDS, n_worlds=N_WORLDS):
    """dWorldStep (the exact stepper: dense LCP per island, the reference's
    Dantzig pivoting) on the batched-worlds workload: world-steps/s of the
    first `steps` steps from the initial state, timed with CUDA events on the
    batch stream, beside the FP64 oracle port of dWorldStep on all host
    threads over worlds [0, cpu_worlds) for the same steps."""
    import torch
    import oracle_lib as O
    from odegpu.batch import Batch
    sc = build_scene(n_worlds)
    B = Batch(sc, device=local_rank)
    B.set_stepper(True)
    stream = torch.cuda.ExternalStream(B.stream_handle())
    x0, seeds = B.state(), B.seeds()
    B.step(3)
    B.sync()
    B.set_state(x0)
    B.set_seeds(seeds)
    B.set_step_index(0)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        e0.record(stream)
    B.step(steps)
    with torch.cuda.stream(stream):
        e1.record(stream)
    B.sync()
    t = e0.elapsed_time(e1) / 1e3
    nc, nr, ni = B.counts()
    status = B.status()
    B.close()
    with O.exact_stepper():
        v_cpu, thr, dt = cpu_baseline(sc, min(cpu_worlds, n_worlds), steps)
    return {"metric": f"world-steps/s, batched collide + dWorldStep ({n_worlds} worlds)", "value": n_worlds * steps / t,
            "unit": "world-steps/s", "ms_per_step": 1e3 * t / steps,
            "workload": WORKLOAD.replace("4096 worlds", f"{n_worlds} worlds") +
                        f"; dWorldStep, first {steps} steps from the initial state",
            "rows_last_step": int(nr.sum()), "contacts_last_step": int(nc.sum()),
            "worlds_with_status": int((status != 0).sum()),
            "worlds_with_lcp_stop": int(((status & 256) != 0).sum()),
            "cpu_port": {"value": v_cpu, "unit": "world-steps/s", "cores": thr,
                         "sample": f"FP64 oracle port of dWorldStep, worlds 0..{min(cpu_worlds, n_worlds) - 1}, {steps} steps "
                                   f"from the initial state ({dt:.1f} s)"}}


def run_reference(args):
    rank, world_size, _ = rank_env()
    if rank != 0:
        return
    sc = build_scene(N_WORLDS)
    import oracle_lib as O
    O.build_oracle()
    threads = os.cpu_count() or 1
    # warm-up: W steps of every world from the initial state
    O.step_worlds_from(sc, 0, max(1, args.warmup), threads=threads, counts=False)
    value, _, dt, reps = cpu_window(sc, SETTLE_STEP, args.steps, threads)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "world-steps/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * N_WORLDS / value, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": bench_config(args.steps),
            "cpu_baseline": {"value": value, "unit": "world-steps/s", "cores": threads, "kind": "port",
                             "sample": f"all {N_WORLDS} worlds, steps {SETTLE_STEP}..{SETTLE_STEP + args.steps - 1} "
                                       f"of the oracle's own rollout, repeated {reps}x ({dt:.1f} s timed), "
                                       f"{threads} threads, one world per thread at a time"},
            "e2e": {"value": value, "unit": "world-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def state_error_sample(sc, B, x_start, seeds_start, step, n_sample=64):
    """One GPU step from the batch's FP32 state at `step` against one oracle
    step from the same state, on n_sample worlds spread over the batch: max
    abs position error (m), max position error relative to the world's
    extent, max linear / angular velocity error."""
    import oracle_lib as O
    B.set_state(x_start)
    B.set_seeds(seeds_start)
    B.set_step_index(step)
    B.step(1)
    g = B.state()
    ws = np.linspace(0, sc.n_worlds - 1, n_sample).astype(int)
    pos_abs = pos_rel = lv = av = 0.0
    for w in ws:
        b0, b1 = sc.world_bodies(int(w))
        o, _, _ = O.step_worlds_from(sc, step, 1, state=x_start[b0:b1], seeds=seeds_start[w:w + 1],
                                     w_begin=int(w), w_end=int(w) + 1, threads=1, counts=False)
        e = np.abs(g[b0:b1] - o)
        pos_abs = max(pos_abs, float(e[:, 0:3].max()))
        pos_rel = max(pos_rel, float(e[:, 0:3].max() / max(1.0, np.abs(o[:, 0:3]).max())))
        lv = max(lv, float(e[:, 7:10].max()))
        av = max(av, float(e[:, 10:13].max()))
    return {"pos_abs_m": pos_abs, "pos_rel": pos_rel, "lvel_abs": lv, "avel_abs": av,
            "sample": f"{n_sample} worlds, one step from the GPU's FP32 state at step {step} against "
                      f"one FP64 oracle step from the same state"}


def run_ours(args):
    import torch
    from odegpu.batch import Batch

    rank, world_size, local_rank = rank_env()
    dist = world_size > 1
    if dist:
        import torch.distributed as tdist
        tdist.init_process_group("nccl")
    torch.cuda.set_device(local_rank)
    # weak scaling (default): every rank steps its own 4096-world batch
    # (distinct seeds). --split (strong scaling): the ranks share one
    # 4096-world scene, each stepping its contiguous block of worlds
    # (odegpu.shard). Either way the step has no collective; only the timing
    # is reduced.
    if args.split and world_size > 1:
        from odegpu.shard import bodies_per_world, slice_scene, world_blocks
        full = build_scene(N_WORLDS)
        b0, b1 = world_blocks(N_WORLDS, world_size, weights=bodies_per_world(full))[rank]
        sc = slice_scene(full, b0, b1)
        total_worlds, scaling = N_WORLDS, "strong"
    else:
        sc = build_scene(N_WORLDS, seed=rank_scene_seed(rank))
        total_worlds, scaling = N_WORLDS * world_size, "weak"
    B = Batch(sc, device=local_rank)
    stream = torch.cuda.ExternalStream(B.stream_handle())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    iters = sc.world_params[0].iterations
    init_state, init_seeds = B.state(), B.seeds()

    def barrier():
        if dist:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # the rollout to the settled state (untimed)
    B.step(SETTLE_STEP)
    B.sync()
    settled_state, settled_seeds = B.state(), B.seeds()

    def reset(to_initial=False):
        B.set_state(init_state if to_initial else settled_state)
        B.set_seeds(init_seeds if to_initial else settled_seeds)
        B.set_step_index(0 if to_initial else SETTLE_STEP)

    # launch shapes picked by the library's autotuner on the settled state
    # (outside the timed region; the state is restored below)
    launch_cfg = B.autotune(4)
    if args.step_kernels != "auto":
        B.set_step_kernels(args.step_kernels == "fused")
    reset()
    for _ in range(args.warmup):
        B.step(1)
    B.sync()

    def timed_window(from_initial=False):
        reset(from_initial)
        barrier()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
        rec = dict(bytes=[], solve_bytes=0.0, rows=0)
        B.set_timing(True)                # events around each kernel, on the batch stream
        B.kernel_times()                  # reset the per-kernel sums
        launches0 = B.launch_count()
        barrier()
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.add_(1.0)           # evict L2 between timed steps (256 MB > 129 MB L2)
                ev[k][0].record(stream)
            B.step(1)
            with torch.cuda.stream(stream):
                ev[k][1].record(stream)
            nc, nr, _ = B.counts()        # host read between steps, outside the events
            rec["bytes"].append(algorithmic_bytes(sc, nc, nr, iters))
            rec["solve_bytes"] += solve_bytes(nr, iters)
            rec["rows"] += int(np.sum(nr))
        B.sync()
        barrier()
        rec["launches"] = B.launch_count() - launches0
        rec["kern_ms"], rec["kern_steps"] = B.kernel_times()
        B.set_timing(False)
        rec["times"] = np.array([a.elapsed_time(b) for a, b in ev]) / 1e3
        rec["status"] = B.status()
        return rec

    clocks = ClockSampler(local_rank)
    clocks.start()
    main = timed_window()
    clk = clocks.stop()
    t_kernel = float(main["times"].sum())
    t_max = max_over_ranks(t_kernel, device="cuda")
    value = total_worlds * args.steps / t_max
    first = timed_window(from_initial=True)
    t_first = max_over_ranks(float(first["times"].sum()), device="cuda")

    # e2e through the C ABI with host buffers: per step H2D of the state from
    # pinned memory, the step, D2H of the new state, synchronised
    nbt = B.nb_total
    h_in = torch.empty(nbt * 13, dtype=torch.float32, pin_memory=True)
    h_out = torch.empty(nbt * 13, dtype=torch.float32, pin_memory=True)
    reset()
    B.read_state_async(h_in.data_ptr())
    B.sync()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        B.write_state_async(h_in.data_ptr())
        B.step(1)
        B.read_state_async(h_out.data_ptr())
        B.sync()
        h_in, h_out = h_out, h_in
    barrier()
    t_e2e = max_over_ranks(time.perf_counter() - t0, device="cuda")
    e2e = total_worlds * args.steps / t_e2e

    if rank == 0:
        hbm, src = peaks()
        kern_ms, kern_steps = main["kern_ms"], main["kern_steps"]
        step_achieved = float(np.sum(main["bytes"])) / t_kernel / 1e9
        fused, fused_wpb, fused_carve = B.step_kernels()
        if fused:
            # one kernel per step (the autotuner picked the fused step kernel):
            # its roofline is the whole step's byte model
            t_dom = kern_ms[0] / 1e3
            achieved = float(np.sum(main["bytes"])) / t_dom / 1e9
            traffic = None
            dom = {"kernel": "world_step_kernel (collide + setup + SOR_LCP + integration)",
                   "bytes_model": "208*nb + 56*nc + 40*n_ball + m*(248 + 236*iters) per world",
                   "launch_ms_avg": kern_ms[0] / max(1, kern_steps), "traffic_source": None}
            share_d = {"world_step_kernel": 1.0}
        else:
            t_solve = kern_ms[2] / 1e3
            achieved = main["solve_bytes"] / t_solve / 1e9
            tpr = solve_traffic_per_row_iter()
            traffic = tpr * main["rows"] * iters / args.steps if tpr is not None else None
            dom = {"kernel": "world_solve_kernel (SOR_LCP + integration)",
                   "bytes_model": "236 B per row-iteration (rows x iterations of the launch)",
                   "launch_ms_avg": kern_ms[2] / max(1, kern_steps),
                   "traffic_source": "ncu dram bytes per row-iteration (profiles/) x rows x iters"}
            share = kern_ms / kern_ms.sum()
            share_d = {"world_collide_kernel": share[0], "world_setup_kernel": share[1],
                       "world_solve_kernel": share[2]}
        times = main["times"]
        line = {"metric": METRIC, "value": value, "unit": "world-steps/s", "n_gpus": world_size,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps,
                "higher_is_better": True, "scaling": scaling, "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded)",
                "config": bench_config(args.steps, iters),
                "window": {"rows_per_world_avg": main["rows"] / (args.steps * sc.n_worlds),
                           "bodies": int(nbt), "worlds_with_status": int((main["status"] != 0).sum()),
                           "launch_shape": {"collide": launch_cfg[0], "setup": launch_cfg[1],
                                            "solve": launch_cfg[2],
                                            "solve_registers": 128 if B.launch_config_ex(2)[2] else 168,
                                            "fused_step": [fused_wpb, fused_carve],
                                            "step_kernels": "fused" if fused else "collide, setup, solve"},
                           "step_ms_min_median_max": [float(1e3 * times.min()), float(1e3 * np.median(times)),
                                                      float(1e3 * times.max())]},
                "from_initial_state": {"value": total_worlds * args.steps / t_first,
                                       "unit": "world-steps/s",
                                       "rollout": f"steps 0..{args.steps - 1} from the initial state",
                                       "rows_per_world_avg": first["rows"] / (args.steps * sc.n_worlds)},
                "roofline": dict({"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                                  "frac": achieved / hbm, "peak_source": src, "traffic": traffic}, **dom),
                "step_roofline": {"achieved": step_achieved, "frac": step_achieved / hbm,
                                  "bytes_model": "208*nb + 56*nc + 40*n_ball + m*(248 + 236*iters) per world"},
                "kernel_share": share_d,
                "e2e": {"value": e2e, "unit": "world-steps/s", "h2d_bytes_per_step": nbt * 13 * 4,
                        "d2h_bytes_per_step": nbt * 13 * 4},
                "gpu_launches": main["launches"], "clocks": clk}
        if not args.no_cpu:
            line["state_err"] = state_error_sample(sc, B, settled_state, settled_seeds, SETTLE_STEP)
        if not args.no_plain:
            # plain comparator: the same kernels, one world per launch, first
            # 512 worlds x 20 steps from the initial state, against the batched
            # path over the same worlds and steps
            pw = 512
            sub = build_scene(pw)
            P = Batch(sub, device=local_rank)
            P.step_plain(2)
            P.sync()
            t0 = time.perf_counter()
            P.step_plain(20)
            P.sync()
            tp = time.perf_counter() - t0
            line["plain_gpu"] = {"value": pw * 20 / tp, "unit": "world-steps/s",
                                 "sample": f"first {pw} worlds x 20 steps, one world per launch",
                                 "batched_from_initial_over_plain": sc.n_worlds * args.steps / t_first / (pw * 20 / tp)}
            P.close()
        if not args.no_adjoint:
            line["adjoint"] = run_adjoint(local_rank)
        if not args.no_vehicles:
            line["vehicles"] = run_vehicles(local_rank)
        if not args.no_large:
            line["large_world"] = run_large_world(local_rank)
        if not args.no_exact:
            line["exact_step"] = run_exact(local_rank)
        if not args.no_cpu:
            v, thr, dt, reps = cpu_window(sc, SETTLE_STEP, args.steps)
            line["cpu_baseline"] = {"value": v, "unit": "world-steps/s", "cores": thr, "kind": "port",
                                    "sample": f"all {N_WORLDS} worlds, steps {SETTLE_STEP}..{SETTLE_STEP + args.steps - 1} "
                                              f"of the oracle's own rollout, repeated {reps}x ({dt:.1f} s timed)"}
        print(json.dumps(line), flush=True)
    B.close()
    if dist:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-vehicles", action="store_true")
    ap.add_argument("--only-adjoint", action="store_true",
                    help="print only the forward + adjoint measurement (for profiling)")
    ap.add_argument("--only-vehicles", action="store_true",
                    help="print only the vehicle-batch measurement (for profiling)")
    ap.add_argument("--no-large", action="store_true")
    ap.add_argument("--no-exact", action="store_true")
    ap.add_argument("--only-exact", action="store_true",
                    help="print only the dWorldStep measurement (for profiling)")
    ap.add_argument("--exact-worlds", type=int, default=N_WORLDS)
    ap.add_argument("--split", action="store_true",
                    help="under torchrun: the ranks share one 4096-world scene (strong scaling)")
    ap.add_argument("--exact-steps", type=int, default=100)
    ap.add_argument("--only-large", action="store_true",
                    help="print only the large-world measurement (for profiling)")
    ap.add_argument("--step-kernels", default="auto", choices=["auto", "split", "fused"],
                    help="one fused kernel per step, the collide / setup / solve kernels, or the "
                         "autotuner's choice (under a profiler the autotuner's timings are distorted)")
    ap.add_argument("--worlds", type=int, default=N_WORLDS,
                    help="worlds of the batched workload (a smaller case for profiling; the "
                         "benchmark configuration is 4096)")
    args = ap.parse_args()
    _set_worlds(args.worlds)
    if args.impl == "reference":
        run_reference(args)
    elif args.only_adjoint or args.only_vehicles or args.only_large or args.only_exact:
        import torch
        _, _, local_rank = rank_env()
        torch.cuda.set_device(local_rank)
        out = (run_adjoint(local_rank) if args.only_adjoint else
               run_vehicles(local_rank) if args.only_vehicles else
               run_exact(local_rank, steps=args.exact_steps, n_worlds=args.exact_worlds) if args.only_exact
               else run_large_world(local_rank))
        print(json.dumps(out), flush=True)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
