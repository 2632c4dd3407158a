#!/usr/bin/env python
"""Benchmark of the per-frame particle physics step on GB300.

Metric: particle-steps/s (particles x frames / s).  Workload: 1,000,000
particles on a jittered lattice in a 1920x1080 box, cell size 1, extended
physics (3x3-cell neighbourhood, 4 Jacobi iterations, gravity 0.1 px/frame^2,
walls, velocity clamp 1).  A step is one frame: solve + rebin.

  value    device-timed frames of the workload's 1000-frame trajectory
           (timed K frames = K/1000 passes over it, the initial state
           re-uploaded untimed between passes), state resident in HBM, L2
           flushed (a 256 MiB write) before every timed frame; CUDA events on
           the library's stream around each frame
  e2e      the same metric through the C ABI with pinned host buffers:
           every step uploads the particles (wrach_set_particles: H2D and
           the device re-pack), runs one frame and reads the frame back
           (wrach_read: D2H of positions, velocities and the table)
  roofline the dominant kernel's algorithmic bytes / its mean CUDA-event
           duration on eager frames sampled within the timed frames 1..K,
           against the measured HBM copy bandwidth

`--impl reference` times the reference's CPU path (the oracle port of the
shader crate, all host threads) on the same workload and metric.
Multi-GPU: one independent replica per rank (the single-world step does not
shard), value = all ranks' particle-steps / the slowest rank's time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PUBLISHED_PARTICLE_STEPS = 39.0e6  # README.md:14-18 of the reference: ~39 fps at 1M particles
FALLBACK_HBM_GBS = 6800.0
METRIC = "particle-steps/s at 1M particles (plain CUDA step)"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=2000)
    p.add_argument("--trajectory", type=int, default=1000)
    p.add_argument("--warmup", type=int, default=20)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--e2e-steps", type=int, default=50)
    p.add_argument("--profile-frames", type=int, default=10)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--cpu-seconds", type=float, default=15.0)
    p.add_argument("--workload", default="lattice",
                   choices=["lattice", "blobs", "small", "reference", "surrogate", "batch", "viewport"],
                   help="lattice: the headline line; surrogate and batch print their own line")
    return p.parse_args()


L2_NOTE = "flushed before every timed GPU frame (256 MiB write), flush not timed"


def workload(name="lattice", trajectory=1000):
    """The 1M jittered lattice (the headline), the same lattice under the
    reference's own physics (per-cell Gauss-Seidel, no gravity), or the 4M
    clustered field (32 Gaussian blobs falling into a basin).  Both arms
    print the description returned here as their `config`."""
    desc, dims, pos, vel, cfg = _workload(name)
    desc = dict(desc, trajectory_frames=trajectory, timed_frames="frames 1..K of the trajectory",
                l2=L2_NOTE)
    return dims, pos, vel, cfg, desc


def _workload(name):
    from wrach_gb300 import workloads
    cfg = dict(cell_size=1, mode=1, iterations=4, gravity=0.1)
    if name == "small":
        dims, pos, vel = workloads.small()
        desc = {"workload": "small-16K", "particles": int(len(pos)), "box": list(dims),
                "cell_size": 1, "physics": "extended (3x3 cells, 4 Jacobi iterations)",
                "gravity": 0.1, "init": "uniform in 512x512, vel N(0,2), seed 0",
                "note": "2.6 MB of state: L2-resident and launch-bound, not rooflined"}
        return desc, dims, pos, vel, cfg
    if name == "reference":
        dims, pos, vel = workloads.lattice()
        cfg = dict(cell_size=1, mode=0, iterations=1, gravity=0.0)
        desc = {"workload": "lattice-1M, reference physics", "particles": int(len(pos)),
                "box": list(dims), "cell_size": 1,
                "physics": "reference (per-cell Gauss-Seidel, cap 9, no gravity)",
                "init": "jittered lattice 1334x750 sites, jitter U(-0.25,0.25), vel N(0,1), seed 0"}
        return desc, dims, pos, vel, cfg
    if name == "blobs":
        dims, pos, vel = workloads.blobs()
        desc = {"workload": "blobs-4M", "particles": int(len(pos)), "box": list(dims),
                "cell_size": 1, "physics": "extended (3x3 cells, 4 Jacobi iterations)",
                "gravity": 0.1, "init": "32 Gaussian blobs, sigma 40 px, centres U(box), clipped to the box, vel N(0,1), seed 0"}
        return desc, dims, pos, vel, cfg
    dims, pos, vel = workloads.lattice()
    desc = {"workload": "lattice-1M", "particles": int(len(pos)), "box": list(dims),
            "cell_size": 1, "physics": "extended (3x3 cells, 4 Jacobi iterations)",
            "gravity": 0.1, "init": "jittered lattice 1334x750 sites, jitter U(-0.25,0.25), vel N(0,1), seed 0"}
    return desc, dims, pos, vel, cfg


def ncu_figure(workload_name, table, kernel=None):
    """One figure of the committed ncu summary (profiles/ncu_traffic.json):
    `table` ("dram_bytes_per_launch" or "warp_instructions_per_launch") of
    `kernel` in a capture of this very workload (with no kernel: the entry
    `table` itself, e.g. "frame", the captured frame), or None when that
    workload has no capture."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.json")) as f:
            entry = json.load(f)["workloads"][workload_name][table]
        return entry if kernel is None else entry.get(kernel)
    except Exception:
        return None


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 100 ms."""
    FIELDS = ("index,timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def stop(self):
        if not self.proc:
            return
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out, _ = self.proc.communicate()
        self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 10:
                continue
            try:
                sm.append(float(parts[2]))
                mx = float(parts[3])
            except ValueError:
                continue
            for name, val in zip(names, parts[6:10]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def oracle_setup(dims, pos, vel, cfg):
    from oracle import oracle as O
    w = O.world(dims[0], dims[1], cfg["cell_size"])
    if cfg["mode"]:
        ph = O.extended_physics(cfg["iterations"], cfg["gravity"])
    else:
        ph = O.reference_physics()
    table, p, v = O.pack(w, pos, vel, O.max_particles_per_frame(w))
    return O, w, ph, table, p, v


def cpu_frames(dims, pos, vel, cfg, frames, seconds):
    """The oracle (C port of the reference's shader crate), all host threads,
    stepping frames 1..k of the trajectory from the initial state: the same
    frames as the GPU line's timed window, k = frames, or fewer when the
    steps (taken 10 frames at a time) pass about `seconds`.  Returns
    (particle-steps/s, k, seconds taken, threads)."""
    O, w, ph, table, p, v = oracle_setup(dims, pos, vel, cfg)
    k, dt = 0, 0.0
    while k < frames and (k == 0 or dt < seconds):
        chunk = min(10, frames - k)
        t0 = time.perf_counter()
        table, p, v, _ = O.step(w, ph, table, p, v, chunk)
        dt += time.perf_counter() - t0
        k += chunk
    return len(pos) * k / dt, k, dt, O.num_threads()


def cpu_on_states(dims, cfg, states):
    """The oracle timed on one frame from each (frame, table, pos, vel) state
    sampled along the trajectory.  The GPU path is bit-exact with the oracle,
    so the GPU's state at frame f is the oracle's state at frame f: this
    gives the CPU's rate over the whole trajectory without stepping it all on
    the host."""
    from oracle import oracle as O
    w = O.world(dims[0], dims[1], cfg["cell_size"])
    ph = O.extended_physics(cfg["iterations"], cfg["gravity"]) if cfg["mode"] else O.reference_physics()
    total, units = 0.0, 0
    for _, table, p, v in states:
        t0 = time.perf_counter()
        O.step(w, ph, table.copy(), p.copy(), v.copy(), 1)
        total += time.perf_counter() - t0
        units += int(table[-1])
    return units / total, total


def run_reference(args):
    world, rank, _ = dist_setup()
    if rank != 0:
        return 0
    dims, pos, vel, cfg, desc = workload(trajectory=args.trajectory)
    O, w, ph, table0, p0, v0 = oracle_setup(dims, pos, vel, cfg)
    # warm-up frames, then the timed frames 1..K from the initial state, the
    # window the GPU arm times; each step is one frame of the full workload
    table, p, v, _ = O.step(w, ph, table0.copy(), p0.copy(), v0.copy(), args.warmup)
    steps = max(1, min(args.steps, 100))
    table, p, v = table0.copy(), p0.copy(), v0.copy()
    t0 = time.perf_counter()
    table, p, v, _ = O.step(w, ph, table, p, v, steps)
    dt = time.perf_counter() - t0
    value = len(pos) * steps / dt
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "particle-steps/s",
            "n_gpus": args.gpus, "steps": steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * dt / steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": value / PUBLISHED_PARTICLE_STEPS, "dtype": "f32",
            "data": "synthetic", "config": desc,
            "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": O.num_threads(),
                             "kind": "port",
                             "sample": "frames 1-%d of the full workload on the host cores" % steps},
            "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# algorithmic bytes of each launch of a frame (n particles, c cells)
def launch_bytes(kind, n, c, n_tp=None):
    if kind == "jacobi":            # over the n_tp taking-part particles (default: all)
        return 20 * (n if n_tp is None else n_tp) + 4 * c  # q in + q out + cell, capped table once
    if kind == "jacobi_final":
        return 40 * n + 4 * c       # q, vel, cell_of in; pos, vel, key out
    if kind == "solve_reference":
        return 36 * n + 4 * c       # pos, vel in; pos, vel, key out
    if kind == "rebin":
        return 40 * n + 8 * c       # key, pos, vel in; pos, vel, cell_of out; table in + out
    if kind == "rebin_count":
        return 8 * n                # keys in, tickets out
    if kind == "rebin_scan":
        return 12 * c               # counts in; cell-start and capped tables out
    if kind == "rebin_scatter":
        return 20 * n               # keys, tickets, starts in; source and cell out
    if kind == "rebin_place":
        return 64 * n               # slots in; pos, vel in; pos, vel, cell and compacted copies out
    return 0


# the launches of the rebin (a stable counting sort), in order; the first is
# left out of extended-physics frames, whose last Jacobi pass takes the tickets
REBIN_STEPS = ["count", "scan", "scatter", "place", "large_cells"]


def run_ours(args):
    import numpy as np
    import torch

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import wrach_gb300 as W
    W.build()
    dims, pos, vel, cfg, desc = workload(args.workload if args.workload in ("blobs", "reference", "small")
                                         else "lattice", args.trajectory)
    n = len(pos)
    sim = W.Simulation(W.WrachConfig(dimensions=dims, device=local, **cfg))
    sim.add_particles(pos, vel)
    cells = sim.cells()
    stream = torch.cuda.ExternalStream(sim.stream, device=torch.device("cuda", local))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def flush_l2():
        with torch.cuda.stream(stream):
            flush.fill_(1)

    for _ in range(args.warmup):
        flush_l2()
        sim.step(1)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    clocks = ClockSampler(local).start()
    time.sleep(0.25)
    barrier()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    launches = 0
    for k in range(args.steps):
        if k % args.trajectory == 0:
            # a new pass over the trajectory: restart from the initial state
            torch.cuda.synchronize()
            sim.set_particles(pos, vel)
        flush_l2()
        l0 = sim.kernel_launches
        starts[k].record(stream)
        sim.step(1)
        ends[k].record(stream)
        launches += sim.kernel_launches - l0
    barrier()
    clocks.stop()
    frame_ms = np.array([s.elapsed_time(e) for s, e in zip(starts, ends)])
    dev_ms = float(frame_ms.sum())
    from wrach_gb300 import replicas
    max_ms, units = replicas.aggregate(dev_ms, n * args.steps, device="cuda")
    value = units / (max_ms / 1000.0)
    traj = frame_ms[: min(args.trajectory, args.steps)]
    head = min(100, len(traj))
    phases = {"frames_1_%d_ms" % head: float(traj[:head].mean())}
    if len(traj) > 100:
        phases["frames_%d_%d_ms" % (len(traj) - 99, len(traj))] = float(traj[-100:].mean())

    # per-kernel durations of eager frames sampled over the timed window
    # (frames 1..K of the trajectory), the frames the line's value covers
    solve_kinds = (["jacobi"] * (cfg["iterations"] - 1) + ["jacobi_final"] if cfg["mode"] else
                   ["solve_reference"])
    # extended frames take the rebin's tickets in their last Jacobi pass
    rebin_kinds = REBIN_STEPS[1:] if cfg["mode"] else REBIN_STEPS
    kinds = solve_kinds + ["rebin_" + s for s in rebin_kinds]
    sim.set_particles(pos, vel)
    window = min(args.steps, args.trajectory)
    every_prof = max(1, window // max(1, args.profile_frames))
    every = max(1, args.trajectory // 10)
    prof, nprof = np.zeros(len(kinds)), 0
    # the taking-part particles of the profiled frames (the first
    # cell_capacity of each cell), whose compacted iterates the Jacobi
    # launches read and write
    cell_cap = W.WrachConfig().cell_capacity
    n_tp = 0.0
    # states along the trajectory for the CPU baseline's trajectory-wide rate
    want_states = rank == 0 and world == 1 and not args.no_cpu_baseline
    states = []
    for k in range(args.trajectory):
        if want_states and k % every == 0:
            p_k, v_k, t_k = sim.read_frame()
            states.append((k, t_k.copy(), p_k.copy(), v_k.copy()))
        if k < window and k % every_prof == every_prof - 1:
            if cfg["mode"]:
                counts = np.diff(sim.read_frame()[2][1:].astype(np.int64))
                n_tp += float(np.minimum(counts, cell_cap).sum())
            flush_l2()
            prof += np.array(sim.profile_frame())
            nprof += 1
        else:
            sim.step(1)
    prof /= max(nprof, 1)
    n_tp = n_tp / max(nprof, 1) if cfg["mode"] else float(n)
    per_kind = {}
    for k, ms in zip(solve_kinds, prof):
        per_kind.setdefault(k, []).append(ms)
    rebin_steps = {s: float(ms) for s, ms in zip(rebin_kinds, prof[len(solve_kinds):])}
    # the dominant kernel: the most time per frame of one kernel (the
    # rebin's launches each count on their own)
    for step, ms in rebin_steps.items():
        per_kind["rebin_" + step] = [ms]
    dom = max(per_kind, key=lambda k: sum(per_kind[k]))
    per_kind["rebin"] = [float(sum(rebin_steps.values()))]
    dom_ms = statistics.mean(per_kind[dom])
    peak, peak_kind = measured_peak()
    achieved = launch_bytes(dom, n, cells, n_tp) / (dom_ms / 1000.0) / 1e9
    step_bytes = 32 * n + 8 * cells
    kernels = {k: {"launches_per_step": len(v), "mean_ms": statistics.mean(v),
                   "gbs": launch_bytes(k, n, cells, n_tp) / (statistics.mean(v) / 1000.0) / 1e9}
               for k, v in per_kind.items()}

    # end to end through the C ABI with pinned host buffers
    e2e = None
    if args.e2e_steps > 0:
        cap = sim.capacity()
        h_pos = torch.empty((n, 2), dtype=torch.float32, pin_memory=True).numpy()
        h_vel = torch.empty((n, 2), dtype=torch.float32, pin_memory=True).numpy()
        h_pos[:] = pos
        h_vel[:] = vel
        o_pos = torch.empty((cap, 2), dtype=torch.float32, pin_memory=True).numpy()
        o_vel = torch.empty((cap, 2), dtype=torch.float32, pin_memory=True).numpy()
        o_idx = torch.empty(cells + 2, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
        for _ in range(2):
            sim.set_particles(h_pos, h_vel)
            sim.step(1)
            sim.read(out=(o_pos, o_vel, o_idx))
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            sim.set_particles(h_pos, h_vel)
            sim.step(1)
            sim.read(out=(o_pos, o_vel, o_idx))
        barrier()
        dt = time.perf_counter() - t0
        max_dt, e2e_units = replicas.aggregate(dt, n * args.e2e_steps, device="cuda")
        e2e = {"value": e2e_units / max_dt, "unit": "particle-steps/s",
               "h2d_bytes_per_step": 16 * n, "d2h_bytes_per_step": 16 * n + 4 * (cells + 1),
               "steps": args.e2e_steps,
               "ms_per_step": 1000.0 * max_dt / args.e2e_steps}

    lattice = args.workload == "lattice"
    clock_summary = clocks.summary()
    # the Jacobi is bound by instruction issue: its warp instructions per
    # launch (one ncu capture of this workload) over its live mean duration,
    # against one instruction per scheduler per cycle on every SM
    # (only when the timed window is the early frames around the captured
    # one: the instruction count changes along the trajectory)
    issue = None
    inst = ncu_figure(desc["workload"], "warp_instructions_per_launch", dom)
    cap_frame = ncu_figure(desc["workload"], "frame")
    if inst and cap_frame and cap_frame <= window <= 100 and clock_summary.get("sm_max_mhz"):
        sms = torch.cuda.get_device_properties(local).multi_processor_count
        ipeak = sms * 4 * clock_summary["sm_max_mhz"] * 1e6
        issue = {"kernel": dom, "warp_instructions_per_launch": inst,
                 "source": "profiles/ncu_traffic.json (ncu smsp__inst_executed.sum, one launch)",
                 "achieved": inst / (dom_ms / 1000.0), "peak": ipeak,
                 "peak_source": "%d SMs x 4 schedulers x %.0f MHz" % (sms, clock_summary["sm_max_mhz"]),
                 "unit": "warp instructions/s", "frac": inst / (dom_ms / 1000.0) / ipeak}
    other = {"blobs": "particle-steps/s at 4M particles, clustered (plain CUDA step)",
             "reference": "particle-steps/s at 1M particles, the reference's own physics",
             "small": "particle-steps/s at 16K particles (plain CUDA step)"}
    line = {
        "metric": METRIC if lattice else other[args.workload],
        "value": value, "unit": "particle-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": max_ms / args.steps,
        "higher_is_better": True, "scaling": "weak",
        # the published number is quoted at 1M particles only
        "vs_baseline": value / PUBLISHED_PARTICLE_STEPS if lattice else None,
        "dtype": "f32", "data": "synthetic",
        "config": desc,
        "parallelism": "replicas" if world > 1 else "single GPU",
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                     "peak_source": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": ncu_figure(desc["workload"], "dram_bytes_per_launch", dom),
                     "traffic_source": "profiles/ncu_traffic.json (ncu dram__bytes_read+write, one launch"
                                       " of this workload at frame %s; null: no capture of it)" % cap_frame,
                     "algorithmic_bytes_per_launch": launch_bytes(dom, n, cells, n_tp),
                     "taking_part_particles": n_tp},
        "step_roofline": {"algorithmic_bytes_per_step": step_bytes,
                          "achieved": step_bytes / (max_ms / args.steps / 1000.0) / 1e9,
                          "frac": step_bytes / (max_ms / args.steps / 1000.0) / 1e9 / peak},
        "kernels": kernels,
        "rebin_steps_ms": rebin_steps,
        "trajectory": dict(phases, frames=args.trajectory,
                           note="frames of one pass; late frames are the collapsed floor"),
        "issue_roofline": issue,
        "gpu_launches": launches,
        "clocks": clock_summary,
        "e2e": e2e,
        "flags": sim.flags(),
    }
    if want_states:
        v_cpu, k_cpu, dt_cpu, threads = cpu_frames(dims, pos, vel, cfg, args.steps, args.cpu_seconds)
        v_traj, dt_traj = cpu_on_states(dims, cfg, states)
        line["cpu_baseline"] = {
            "value": v_cpu, "unit": "particle-steps/s", "cores": threads, "kind": "port",
            "sample": "frames 1-%d of the %d-particle trajectory from the initial state, the GPU"
                      " line's timed frames%s (%.1f s)"
                      % (k_cpu, n, "" if k_cpu >= args.steps else " (the first %d of them)" % k_cpu,
                         dt_cpu),
            "full_trajectory": {
                "value": v_traj, "unit": "particle-steps/s",
                "sample": "one frame from each of %d states sampled every %d frames along the"
                          " %d-frame trajectory (the GPU's states, bit-exact with the oracle's;"
                          " %.1f s)" % (len(states), every, args.trajectory, dt_traj)}}
    sim.close()
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_surrogate(args):
    """The learned surrogate at the lattice-1M geometry (1M particles,
    1920x1080 px, cell 1 px, extended physics, 4 iterations, gravity 0.1).
    The network is trained on plain-solver frames of the trajectory, then
    1000 frames are timed twice from the same initial state: plain frames
    (graph-launched) and surrogate frames (one fused features + network +
    correction pass and the last plain iteration, the gate on the device:
    fallback when the mean overlap exceeds the latest plain frame's by 0.2 px
    or the kinetic energy deviates by 1%; every 32nd frame a plain
    calibration frame)."""
    import numpy as np
    import torch
    import wrach_gb300 as W
    W.build()
    dims, pos, vel, cfg, desc = workload()
    n = len(pos)
    sim = W.Simulation(W.WrachConfig(dimensions=dims, **cfg))
    sim.add_particles(pos, vel)
    # training rows from 2,000 plain frames of the trajectory: every 20th
    # frame, every 4th taking-part particle of it (25 M rows)
    train_frames, every, stride = 2000, 20, 4
    sim.surrogate_init(0, (train_frames // every) * (n // stride + 1))
    t0 = time.perf_counter()
    for f in range(train_frames):
        if f % every == 0:
            rows = sim.surrogate_collect(stride)
        sim.step(1)
    sim.sync()
    collect_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    loss = sim.surrogate_train(4000, 16384, 2e-3)
    train_s = time.perf_counter() - t0
    net, zero = sim.surrogate_evaluate()
    # the network alone on the tensor cores: features of the current frame
    # precomputed, then the forward kernel timed with CUDA events
    x = torch.zeros((n, 64), dtype=torch.int16, device="cuda")
    yout = torch.zeros((n, 2), dtype=torch.float32, device="cuda")
    sim.surrogate_features(x.data_ptr(), n)
    sim.sync()
    fstream = torch.cuda.ExternalStream(sim.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 20
    filler = torch.empty(1 << 30, dtype=torch.uint8, device="cuda")

    def gpu_ms(fn):
        """GPU time of one call of fn (a launch on the library's stream): a
        long fill queued first keeps the GPU busy while the host queues the
        timed calls, so host-side call overhead does not enter the events."""
        for _ in range(3):
            fn()
        sim.sync()
        with torch.cuda.stream(fstream):
            for _ in range(40):
                filler.fill_(1)
        e0.record(fstream)
        for _ in range(reps):
            fn()
        e1.record(fstream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    fwd_s = gpu_ms(lambda: sim.surrogate_forward(x.data_ptr(), n, yout.data_ptr(), kernel="tcgen05")) / 1000.0
    mma_s = gpu_ms(lambda: sim.surrogate_forward(x.data_ptr(), n, yout.data_ptr(), kernel="mma")) / 1000.0

    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            bf16_peak, peak_source = float(json.load(f)["bf16_tflops"]), "measured (burst)"
    except Exception:
        bf16_peak, peak_source = 1900.0, "fallback"
    flop_per_particle = 2 * (50 * 64 + 64 * 64 + 64 * 2)  # the unpadded network
    net_tflops = flop_per_particle * n / fwd_s / 1e12
    frames = 1000 if args.steps >= 1000 else max(64, args.steps)
    stream = torch.cuda.ExternalStream(sim.stream)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]

    def timed(fn):
        sim.set_particles(pos, vel)
        sim.sync()
        torch.cuda.synchronize()
        ev[0].record(stream)
        out = fn()
        ev[1].record(stream)
        torch.cuda.synchronize()
        return ev[0].elapsed_time(ev[1]) / 1000.0, out

    # the plain frame's launches, eager, on an early frame: a surrogate
    # frame keeps the last iteration and the rebin, so with a free surrogate
    # pass it would take the plain frame minus its first iterations
    sim.set_particles(pos, vel)
    sim.step(7)
    prof = [float(x) for x in sim.profile_frame()]
    iters = cfg["iterations"] - 1
    # the fused surrogate pass alone (features from the 3x3 candidates, the
    # network, the correction) on this lattice frame, where every particle
    # takes part
    corr = torch.zeros((n, 2), dtype=torch.float32, device="cuda")
    fused_ms = gpu_ms(lambda: sim.surrogate_correction(corr.data_ptr()))
    del filler
    sim.set_particles(pos, vel)
    sim.step(3)                        # the plain frame graphs
    sim.surrogate_step(3, 0.2, 0.01)   # the fused kernel's set-up
    clocks = ClockSampler(0).start()
    time.sleep(0.25)
    plain_s, _ = timed(lambda: sim.step(frames))
    pen_plain = sim.frame_metrics()
    sur_s, st = timed(lambda: sim.surrogate_step(frames, 0.2, 0.01))
    pen_sur = sim.frame_metrics()
    clocks.stop()
    # the error bounds over time: both runs again from the initial state in
    # chunks of 32 frames (one calibration frame and 31 gated surrogate frames
    # each, as in one run), the overlap and kinetic energy sampled after each
    # chunk and averaged over the last 10 samples (frames 705-1024)
    samples = {"plain": [], "surrogate": []}
    for name, fn in (("plain", lambda: sim.step(32)),
                     ("surrogate", lambda: sim.surrogate_step(32, 0.2, 0.01))):
        sim.set_particles(pos, vel)
        for _ in range(32):
            fn()
            samples[name].append(sim.frame_metrics())
    late = {k: np.array(v[-10:]) for k, v in samples.items()}
    quality = {"frames": 1024, "sampled_every": 32, "averaged_over": "the last 10 samples",
               "excess_mean_overlap_px": float(late["surrogate"][:, 0].mean() - late["plain"][:, 0].mean()),
               "kinetic_energy_ratio": float(late["surrogate"][:, 2].mean() / late["plain"][:, 2].mean())}
    line = {"metric": "particle-steps/s at 1M particles, surrogate frames (gated) vs plain frames",
            "value": n * frames / sur_s, "unit": "particle-steps/s", "n_gpus": 1, "steps": frames,
            "higher_is_better": True, "dtype": "bf16 network / f32 physics", "data": "synthetic",
            "config": dict(desc, workload="lattice-1M surrogate"),
            "plain": {"value": n * frames / plain_s, "ms_per_step": 1000 * plain_s / frames},
            "surrogate": {"ms_per_step": 1000 * sur_s / frames, "frames": st["frames"],
                          "calibrations": st["calibrations"], "fallbacks": st["fallbacks"],
                          "mean_penetration_before_last_iteration_px": st["mean_penetration"],
                          "reference_penetration_px": st["reference_penetration"],
                          "max_energy_drift": st["max_energy_drift"]},
            "speedup_vs_plain": plain_s / sur_s, "clocks": clocks.summary(),
            "bound": {"plain_frame_launch_ms": prof,
                      "replaced_iterations_ms": sum(prof[:iters]),
                      "kept_ms": sum(prof[iters:]),
                      "speedup_with_a_free_surrogate_pass": sum(prof) / sum(prof[iters:]),
                      "fused_surrogate_pass_ms": fused_ms,
                      "note": "eager launches of frame 8 (L2 warm), the fused pass on frame 9; a"
                              " surrogate frame keeps the last iteration and the rebin and adds two"
                              " gate launches"},
            "network_roofline": {"bound": "tensor", "kernel": "k_mlp_forward_tc (features precomputed)",
                                 "achieved": net_tflops, "peak": bf16_peak, "peak_source": peak_source,
                                 "unit": "TFLOP/s", "frac": net_tflops / bf16_peak,
                                 "flop_per_particle": flop_per_particle, "ms": 1000 * fwd_s,
                                 "note": "tcgen05.mma kind::f16 (M 128, N 64/64/16, K 64), BF16 operands in"
                                         " shared memory, FP32 accumulators in TMEM, two 128-row tiles"
                                         " in flight per CTA; tanh-form GELU on packed FP16 pairs"
                                         " (tanh.approx.f16x2)",
                                 "mma_sync": {"kernel": "k_mlp_forward", "ms": 1000 * mma_s,
                                              "achieved": flop_per_particle * n / mma_s / 1e12,
                                              "frac": flop_per_particle * n / mma_s / 1e12 / bf16_peak}},
            "error_bounds_over_time": quality,
            "final_frame": {"plain_mean_penetration_px": pen_plain[0],
                            "surrogate_mean_penetration_px": pen_sur[0],
                            "excess_penetration_px": pen_sur[0] - pen_plain[0],
                            "plain_kinetic_energy": pen_plain[2],
                            "surrogate_kinetic_energy": pen_sur[2],
                            "kinetic_energy_ratio": pen_sur[2] / pen_plain[2] if pen_plain[2] else None},
            "training": {"samples": rows, "frames": train_frames,
                         "sampling": "every %dth frame, every %dth taking-part particle" % (every, stride),
                         "steps": 4000, "batch": 16384,
                         "final_loss": loss, "collect_s": collect_s, "train_s": train_s,
                         "held_out_mse_ratio_vs_no_network": net / zero if zero else None}}
    sim.close()
    print(json.dumps(line))
    return 0


def batch_worlds(rank, world_size):
    """The worlds of the 256-world batch (sides U[128, 1024], counts
    log-uniform in [1024, 65536]) that `rank` of `world_size` steps: a
    contiguous shard, no data-path collective.  Returns (first world, end,
    dims, positions, velocities)."""
    from wrach_gb300 import replicas, workloads
    dims, poss, vels = workloads.batch()
    lo, hi = replicas.shard(len(poss), rank, world_size)
    return lo, hi, dims[lo:hi], poss[lo:hi], vels[lo:hi]


def run_batch(args):
    """Config 3: 256 independent worlds stepped together in one context
    (one graph launch per frame), the launch shape picked by the autotuner.
    The line's value is the configured cell size 1; cell size 2, which
    changes which particles share a cell and so the physics, is timed beside
    it.  Over N GPUs the worlds are sharded (each rank a contiguous range of
    them, no data-path collective)."""
    import torch
    import wrach_gb300 as W
    from wrach_gb300 import autotune, replicas
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if world > 1:
        torch.distributed.init_process_group("nccl", device_id=torch.device("cuda", local))
    W.build()
    lo, hi, dims, poss, vels = batch_worlds(rank, world)
    n = int(sum(len(p) for p in poss))
    base = W.WrachConfig(cell_size=1, mode=1, iterations=4, gravity=0.1, device=local,
                         capacity=int(max(len(p) for p in poss)))
    steps = max(10, min(args.steps, 500))

    def measure(cell_size):
        cfg = W.WrachConfig(**dict(base.__dict__, cell_size=cell_size))
        t0 = time.perf_counter()
        tuned, table = autotune.tune(cfg, poss, vels, worlds=dims.tolist(), frames=6,
                                     use_cache=False)
        tune_s = time.perf_counter() - t0
        sim = W.Simulation(tuned, worlds=dims.tolist())
        for w, (p, v) in enumerate(zip(poss, vels)):
            sim.set_particles(p, v, world=w)
        stream = torch.cuda.ExternalStream(sim.stream)
        sim.step(max(3, args.warmup))
        torch.cuda.synchronize()
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        clocks = ClockSampler(local).start()
        time.sleep(0.25)
        torch.cuda.synchronize()
        l0 = sim.kernel_launches
        start.record(stream)
        sim.step(steps)
        end.record(stream)
        torch.cuda.synchronize()
        launches = sim.kernel_launches - l0
        clocks.stop()
        st = sim.stats()
        sim.close()
        max_s, units = replicas.aggregate(start.elapsed_time(end) / 1000.0, n * steps, device="cuda")
        return {"value": units / max_s, "ms_per_step": 1000.0 * max_s / steps, "cells": st["cells"],
                "gpu_launches": launches, "clocks": clocks.summary(),
                "autotune": {"choice": autotune.launch_shape(tuned), "ms_per_frame": table,
                             "seconds": tune_s}}

    cs1 = measure(1)
    cs2 = measure(2)
    line = {"metric": "particle-steps/s, 256 batched worlds", "value": cs1["value"],
            "unit": "particle-steps/s", "n_gpus": world, "steps": steps,
            "ms_per_step": cs1["ms_per_step"], "higher_is_better": True, "dtype": "f32",
            "data": "synthetic", "scaling": "strong (the 256 worlds sharded over the GPUs)",
            "config": {"workload": "batch-256", "worlds_on_rank_0": len(poss), "particles_on_rank_0": n,
                       "cells": cs1["cells"], "cell_size": 1,
                       "physics": "extended (4 iterations, gravity 0.1)",
                       "l2": "working set above L2 (tables of %d cells)" % cs1["cells"]},
            "gpu_launches": cs1["gpu_launches"], "clocks": cs1["clocks"], "autotune": cs1["autotune"],
            "cell_size_2": dict(cs2, note="cell size 2 changes which particles share a cell, and so"
                                          " the physics: opt-in, not the configured workload")}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_viewport(args):
    """Viewport streaming at the lattice-1M geometry: the 1,000,000 lattice
    particles in the 1920x1080 viewport plus 1,000,000 more spread over the
    3840x2160 area around it, in the world's store.  After 10 frames, each
    timed move writes the frame back into the store (2 M particles
    classified and compacted) and re-packs the frame under an anchor shifted
    by 64 whole cells (and back), then runs one frame."""
    import numpy as np
    import torch
    import wrach_gb300 as W
    W.build()
    dims, pos, vel, cfg, desc = workload()
    rng = np.random.default_rng(1)
    far = rng.uniform((-960.0, -540.0), (2880.0, 1620.0), size=(1_000_000, 2)).astype(np.float32)
    far_vel = rng.normal(0, 1, size=far.shape).astype(np.float32)
    cfg = dict(cfg, capacity=1_600_000)
    sim = W.Simulation(W.WrachConfig(dimensions=dims, **cfg))
    sim.add_particles(np.concatenate([pos, far]), np.concatenate([vel, far_vel]))
    sim.step(10)
    sim.sync()
    moves = max(4, min(args.steps, 40))
    anchors = [(64.0, 32.0), (0.0, 0.0)]
    for k in range(2):  # warm-up: the store and staging buffers reach their size
        sim.set_viewport(anchors[k % 2])
        sim.step(1)
    sim.sync()
    stream = torch.cuda.ExternalStream(sim.stream)
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    clocks = ClockSampler(0).start()
    time.sleep(0.25)
    t0 = time.perf_counter()
    s0.record(stream)
    frame_n = []
    for k in range(moves):
        sim.set_viewport(anchors[k % 2])
        frame_n.append(sim.settings().particles_in_frame_count)
        sim.step(1)
    s1.record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clocks.stop()
    store_n = len(sim.store()[0])
    line = {"metric": "viewport moves/s (write-back + re-pack + 1 frame), 2M particles",
            "value": moves / wall, "unit": "moves/s", "n_gpus": 1, "steps": moves,
            "ms_per_step": 1000 * wall / moves, "higher_is_better": True, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "lattice-1M viewport streaming", "frame_particles": int(np.mean(frame_n)),
                       "store_particles": store_n, "move_cells": [64, 32]},
            "device_ms_per_step": s0.elapsed_time(s1) / moves, "clocks": clocks.summary(),
            "note": "host-timed: a move blocks (it reads the kept count and the per-world counts back)"}
    sim.close()
    print(json.dumps(line))
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "surrogate":
        return run_surrogate(args)
    if args.workload == "batch":
        return run_batch(args)
    if args.workload == "viewport":
        return run_viewport(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
