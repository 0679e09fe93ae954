"""Benchmark of libbhgpu's per-step Barnes-Hut pipeline (one JSON line on stdout).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

Default workload ("plummer-4m"): one Plummer sphere, N = 2^22 bodies (FP32 state), theta 0.5,
softening 0.005, leaf capacity 16, dt 5e-4, root edge 2S, quadrupole multipoles. A step is one
full frame of the reference's sequence: bounds, Morton keys, sort, kick+drift, tree build,
upsweep, walk + force, kick.

  value  body-steps/s over K timed steps with the state resident in HBM; every bh_step call
         (without stats, so its graph records no stage events) is bracketed by CUDA events on
         the library's stream and the L2 is flushed between steps (outside the events); the
         per-step working set (~0.6 GB) is also larger than L2. A second pass of K steps with
         bh_stats gives the stage split, the rooflines and the launch count.
  e2e    the same metric through the C ABI with host buffers: bh_step_host uploads positions and
         velocities from pinned host memory, runs one step and downloads them, its copies
         overlapped with the step on a second stream; CUDA events around the whole call.
  roofline  the tree walk (the dominant kernel) against the measured FP32 FMA peak of this GPU
         (bh_measure_fp32_peak); the Morton sort against MEASURED_PEAKS.json's HBM copy peak.
  cpu_baseline  the oracle port of the reference's step on this host: one whole step of the same
         workload (every body walked) with all host threads; cpu_serial: whole steps of the
         N = 16 384 configuration on one thread, as the reference runs.
  ensemble / adjoint  the batched and reverse-mode halves of the metric, measured in the same run
         (the ensemble-4096 and adjoint-64k workloads, 5 timed steps each; --no-modes skips them).

--impl reference: the reference's CPU implementation of the same step (the oracle port: the
reference's own sources cannot be compiled on this machine), W + K whole steps with all host
threads, the K steps timed.
Multi-GPU (torchrun): independent replicas, one per GPU (the single-system step does not
shard); value = sum of per-rank body-steps / max-over-ranks time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "plummer-4m": dict(n=1 << 22, theta=0.5, eps=0.005, leaf=16, dt=5e-4, edge=2.0, kind="plummer", seed=0,
                       desc="Plummer sphere N=2^22, theta=0.5, eps=0.005, leaf 16, dt=5e-4, quadrupole, edge 2S"),
    "plummer-4m-theta0.3": dict(n=1 << 22, theta=0.3, eps=0.005, leaf=16, dt=5e-4, edge=2.0, kind="plummer", seed=0,
                                desc="Plummer sphere N=2^22, theta=0.3, eps=0.005, leaf 16, dt=5e-4, quadrupole, edge 2S"),
    "plummer-4m-theta0.7": dict(n=1 << 22, theta=0.7, eps=0.005, leaf=16, dt=5e-4, edge=2.0, kind="plummer", seed=0,
                                desc="Plummer sphere N=2^22, theta=0.7, eps=0.005, leaf 16, dt=5e-4, quadrupole, edge 2S"),
    "plummer-16k": dict(n=16384, theta=0.5, eps=0.01, leaf=1, dt=1e-3, edge=2.0, kind="plummer", seed=0,
                        desc="Plummer sphere N=16384, theta=0.5, eps=0.01, leaf 1, dt=1e-3, quadrupole, edge 2S"),
    # profiling sizes of the headline recipe (small enough for full ncu captures / larger than L2)
    "plummer-1m": dict(n=1 << 20, theta=0.5, eps=0.005, leaf=16, dt=5e-4, edge=2.0, kind="plummer", seed=0,
                       desc="Plummer sphere N=2^20, theta=0.5, eps=0.005, leaf 16, dt=5e-4, quadrupole, edge 2S"),
    "plummer-8m": dict(n=1 << 23, theta=0.5, eps=0.005, leaf=16, dt=5e-4, edge=2.0, kind="plummer", seed=0,
                       desc="Plummer sphere N=2^23, theta=0.5, eps=0.005, leaf 16, dt=5e-4, quadrupole, edge 2S"),
    "two-spheres-4m": dict(n=1 << 22, theta=0.5, eps=0.001, leaf=8, dt=2e-4, edge=2.0, kind="two", seed=0,
                           desc="two Plummer spheres of 2^21 (B: a=0.1, M=0.1 at (10,0,0)), theta=0.5, "
                                "eps=0.001, leaf 8, dt=2e-4"),
    # the reference app's own frame (src/ofApp.h:60,62; src/ofApp.cpp:96; src/HashedOctree.hpp:151):
    # its solar-system scene in SI units, theta 1, dt 1e-3, softening 0.025, leaf capacity 1, root
    # edge S, the pseudo-barycentre (literal) multipoles and the unsorted acceleration array
    "app-solar-4444": dict(n=4444, theta=1.0, eps=0.025, leaf=1, dt=1e-3, edge=1.0, kind="solar", seed=1,
                           multipole="literal", acc_follows_body=0,
                           desc="the reference app's frame: SetupSolarSystem scene N=4444 (SI units), theta=1, "
                                "eps=0.025, leaf 1, dt=1e-3, literal multipoles, root edge S"),
}
METRIC = "body-steps/s @theta=0.5, acc err<=1e-3: plain vs batched/adjoint, 1 GB300 vs CPU"
# algorithmic flops per interaction (an FMA counts 2): point mass 20 (3 sub, r^2 + eps^2 6, rsqrt,
# 2 mul, m d r^-3 6); quadrupole cell 57 (the point-mass terms plus Q.d 15, r^-5 2, update 6,
# d.Q.d 5, scale 2, update 7)
FLOPS_P2P, FLOPS_CELL_QUAD = 20, 57
SORT_PASSES = 8
# steps of the ensemble and adjoint figures carried in the default workload's line
MODE_STEPS, MODE_WARMUP = 5, 3


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    def __init__(self):
        self.ws, self.rank, self.local = dist_env()
        self.pg = None
        if self.ws > 1:
            import torch.distributed as td

            td.init_process_group("gloo")
            self.td = td

    def device(self):
        """This rank's GPU: the local rank under torchrun (one replica per GPU), else 0."""
        return self.local if self.ws > 1 else 0

    def simulation(self, bh, n):
        """A context on this rank's GPU. A rank whose GPU cannot be opened fails (a replica never
        moves onto another rank's GPU)."""
        return bh.Simulation(n, device=self.device())

    def gpu_index(self):
        """nvidia-smi index of this rank's GPU (BH_GPU_INDEX overrides)."""
        return int(os.environ.get("BH_GPU_INDEX", str(self.device())))

    def barrier(self):
        if self.ws > 1:
            self.td.barrier()

    def max(self, x):
        if self.ws == 1:
            return x
        import torch

        t = torch.tensor([float(x)], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x):
        if self.ws == 1:
            return x
        import torch

        t = torch.tensor([float(x)], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.SUM)
        return float(t.item())


def make_inputs(bh, w, seed, sim=None):
    """Initial (pos_m, vel) float32 (n, 4) arrays of a workload. The solar scene comes from the
    library's device generator through `sim`, or, without one (the CPU arm), from the oracle's
    restatement of the same generator (the same draws; within 1e-5 of the device scene)."""
    if w["kind"] == "two":
        return bh.two_spheres(seed, w["n"])
    if w["kind"] == "solar":
        n = w["n"]
        if sim is not None:
            sim.solar_system_device(seed, n, bh.UNITS_SI)
            p, v, _ = sim.get_bodies()
            return np.ascontiguousarray(p), np.ascontiguousarray(v)
        from oracle.oracle import Restatement

        rows = Restatement().solar_system(seed, n)
        pm = np.zeros((n, 4), np.float32)
        vel = np.zeros((n, 4), np.float32)
        pm[:, :3], pm[:, 3], vel[:, :3] = rows[:, :3], rows[:, 6], rows[:, 3:6]
        return pm, vel
    return bh.plummer(seed, w["n"])


def multipole_mode(bh, w):
    """(library multipole constant, oracle mode) of a workload: quadrupoles unless it asks for the
    reference's literal pseudo-barycentres."""
    if w.get("multipole") == "literal":
        return bh.BH_MULTIPOLE_LITERAL, 0
    return bh.BH_MULTIPOLE_QUADRUPOLE, 1


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 50 ms during the timed region (the
    sampler is running, with a first sample written, before the region starts)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.f = None

    def __enter__(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "50"], stdout=self.f, stderr=subprocess.DEVNULL)
            t0 = time.time()
            while time.time() - t0 < 3.0 and self.proc.poll() is None and os.path.getsize(self.f.name) == 0:
                time.sleep(0.02)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.f:
            return None
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    idx = int(parts[0])
                except ValueError:
                    continue
                if idx != self.gpu:
                    continue
                rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except Exception:
        return {}


def ncu_traffic():
    """DRAM bytes per body of one walk launch, from the committed ncu summary (a line
    'walk_dram_bytes_per_body: X'), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", "k_walk_quadrupole_plummer1m.md")) as f:
            for line in f:
                if line.startswith("walk_dram_bytes_per_body:"):
                    return {"bytes_per_body": float(line.split(":")[1])}
    except Exception:
        pass
    return None


def accuracy_vs_direct(w, pm, acc_by_theta, orc, nthreads, ntarget=4096, ntarget_walk=65536, tree=None, mode=1):
    """Median / p99 relative error of the step-0 accelerations against the FP64 direct sum on a
    seeded subsample (the <= 1e-3 accuracy gate at theta 0.5), for the workload's theta and the others
    of the at-scale sweep; and against the reference's tree walk (the oracle restatement) on a
    seeded 65 536-body subsample."""
    from oracle.oracle import relerr

    rng = np.random.default_rng(1234)
    tgt = np.sort(rng.choice(len(pm), min(ntarget, len(pm)), replace=False)).astype(np.uint32)
    pos = pm[:, :3].astype(np.float64)
    mass = pm[:, 3].astype(np.float64)
    d = orc.direct(pos, mass, w["eps"], targets=tgt, nthreads=nthreads)
    out = {}
    for theta, acc in acc_by_theta.items():
        err = relerr(acc[tgt], d)
        out[f"{theta:g}"] = {"median": float(np.median(err)), "p99": float(np.percentile(err, 99))}
    main = out[f"{w['theta']:g}"]
    res = {"median_rel_err_vs_direct_fp64": main["median"], "p99": main["p99"], "targets": int(len(tgt)),
           "by_theta": out}
    if tree is not None:
        # the reference's tree walk (the oracle restatement, FP64) at the same theta, softening,
        # leaf size and root cube, on the same targets
        c, edge = tree
        tw = np.sort(np.random.default_rng(4321).choice(len(pm), min(ntarget_walk, len(pm)),
                                                        replace=False)).astype(np.uint32)
        ref, _, _ = orc.force(pos, mass, c, edge, w["leaf"], mode, w["theta"], w["eps"], targets=tw,
                              nthreads=nthreads)
        err = relerr(acc_by_theta[w["theta"]][tw], ref)
        res["vs_reference_walk"] = {"median": float(np.median(err)), "p99": float(np.percentile(err, 99)),
                                    "targets": int(len(tw))}
    return res


def cpu_whole_steps(bh, w, pm, vel, nthreads, nsteps, acc=None):
    """The oracle port of the reference's per-frame step (bounds, Morton keys, sort, kick+drift,
    tree build, walk + force over every body, kick; src/ofApp.cpp:169-177, 248-282), nsteps whole
    steps from (pm, vel) with nthreads walk threads (the rest of the step is serial, as in the
    reference). Returns the end state and the wall seconds of the call."""
    from oracle.oracle import Restatement

    orc = Restatement()
    pos = pm[:, :3].astype(np.float64)
    v = vel[:, :3].astype(np.float64)
    m = pm[:, 3].astype(np.float64)
    a = np.zeros_like(pos) if acc is None else acc
    t0 = time.perf_counter()
    r = orc.steps(pos, v, m, a, w["dt"], w["theta"], w["eps"], w["edge"], w["leaf"], multipole_mode(bh, w)[1],
                  nsteps, acc_follows_body=w.get("acc_follows_body", 1), nthreads=nthreads)
    r["wall_s"] = time.perf_counter() - t0
    return r


def cpu_state(r):
    """(pos_m, vel) float32 arrays of an oracle end state (the next call's start)."""
    pm = np.zeros((len(r["pos"]), 4), np.float32)
    vel = np.zeros_like(pm)
    pm[:, :3], pm[:, 3], vel[:, :3] = r["pos"], r["mass"], r["vel"]
    return pm, vel


STAGE_NAMES = ("bounds_keys", "sort_reorder", "kick_drift", "build", "walk_force", "kick")


def cpu_baseline_whole_step(bh, w, pm, vel, nthreads):
    """cpu_baseline: one whole step of the same workload (every body walked) by the oracle port
    on nthreads host threads; no sampling, no extrapolation."""
    r = cpu_whole_steps(bh, w, pm, vel, nthreads, 1)
    n = len(pm)
    return {"value": n / r["wall_s"], "unit": "body-steps/s", "cores": nthreads, "kind": "port",
            "sample": (f"1 whole step of the same workload ({n} bodies, every body walked) by the oracle port on "
                       f"{nthreads} host thread(s) (walk threaded, the rest serial): {r['wall_s']:.3g} s"),
            "stage_s": dict(zip(STAGE_NAMES, (float(x) for x in r["stage_s"])))}


def cpu_serial_config0(bh, nsteps=10):
    """The serial figure: whole steps of the small Plummer configuration (N = 16 384, theta 0.5,
    eps 0.01, leaf 1, dt 1e-3) by the oracle port on one thread, as the reference runs."""
    w = WORKLOADS["plummer-16k"]
    pm, vel = make_inputs(bh, w, w["seed"])
    r = cpu_whole_steps(bh, w, pm, vel, 1, nsteps)
    return {"value": w["n"] * nsteps / r["wall_s"], "unit": "body-steps/s", "cores": 1, "kind": "port",
            "workload": "plummer-16k", "steps": nsteps, "seconds_per_step": r["wall_s"] / nsteps,
            "sample": f"{nsteps} whole steps of the N=16384 Plummer configuration (theta 0.5, eps 0.01, leaf 1), "
                      f"1 thread"}


def cpu_steps_sample(systems, theta, eps, dt, leaf, edge, nthreads=1):
    """Oracle port of one reference step (bounds, keys, sort, kick+drift, build, walk, kick) on
    each (pos_m, vel) system given; returns the seconds of each."""
    from oracle.oracle import Restatement

    orc = Restatement()
    out = []
    for pm, vel in systems:
        pos = pm[:, :3].astype(np.float64)
        t0 = time.perf_counter()
        orc.steps(pos, vel[:, :3].astype(np.float64), pm[:, 3].astype(np.float64), np.zeros_like(pos), dt, theta,
                  eps, edge, leaf, 1, 1, acc_follows_body=1, nthreads=nthreads)
        out.append(time.perf_counter() - t0)
    return out


def workload_config(args, w):
    """The `config` object of a workload line; both arms print the same one."""
    return {"workload": args.workload, "bodies": w["n"], "desc": w["desc"]}


def run_reference(args, w, dist):
    """CPU reference arm: the oracle port of the reference's step, whole steps on every body, with
    all host threads: W untimed warm-up steps, then K timed steps continuing the same trajectory.
    Under torchrun only rank 0 runs."""
    if dist.rank != 0:
        return
    import __graft_entry__

    bh = __graft_entry__.package()
    pm, vel = make_inputs(bh, w, w["seed"])
    nthreads = os.cpu_count() or 1
    acc = None
    if args.warmup > 0:
        r = cpu_whole_steps(bh, w, pm, vel, nthreads, args.warmup)
        pm, vel = cpu_state(r)
        acc = r["acc"]
    r = cpu_whole_steps(bh, w, pm, vel, nthreads, args.steps, acc=acc)
    wall = r["wall_s"]
    value = w["n"] * args.steps / wall
    sample = (f"{args.steps} whole steps of the workload ({w['n']} bodies, every body walked) by the oracle port "
              f"on {nthreads} host threads (walk threaded, the rest serial), after {args.warmup} untimed warm-up "
              f"steps: {wall:.3g} s")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "body-steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args, w),
            "timing": "wall clock around the K timed steps (one call into the oracle port)",
            "cpu_baseline": {"value": value, "unit": "body-steps/s", "cores": nthreads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "body-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "stage_s_per_step": {k: float(x) / args.steps for k, x in zip(STAGE_NAMES, r["stage_s"])},
            "steps_timed": args.steps, "wall_s": wall}
    print(json.dumps(line), flush=True)


def run_ours(args, w, dist):
    import __graft_entry__

    bh = __graft_entry__.package()
    bh.load()
    n = w["n"]
    mp, mode = multipole_mode(bh, w)
    prm = bh.default_params(theta=w["theta"], eps=w["eps"], dt=w["dt"], leaf_capacity=w["leaf"],
                            multipole=mp, edge_factor=w["edge"], acc_follows_body=w.get("acc_follows_body", 1))
    sim = dist.simulation(bh, n)
    pm, vel = make_inputs(bh, w, w["seed"] + dist.rank, sim)
    sim.set_bodies(pm, vel)

    # step-0 accelerations for the accuracy gate (rank 0, before stepping)
    accuracy = None
    if dist.rank == 0 and not args.no_accuracy:
        from oracle.oracle import Restatement

        c, size = sim.bounds()
        sim.build(c, size * w["edge"], w["leaf"], mp)
        accs = {th: sim.force(th, w["eps"]) for th in sorted({0.3, 0.5, 0.7, w["theta"]})}
        accuracy = accuracy_vs_direct(w, pm, accs, Restatement(), os.cpu_count() or 1,
                                      tree=(c, size * w["edge"]), mode=mode)
        sim.set_bodies(pm, vel)

    fp32_peak = sim.fp32_peak_tflops()
    # the first warm-up step builds a tree; the autotuner picks the walk's launch shape on it
    sim.step(prm, 1, stats=False)
    tune = sim.autotune(w["theta"], w["eps"], trials=3)
    for _ in range(args.warmup - 1):
        sim.step(prm, 1, stats=False)
    sim.synchronize()
    energy0 = sim.energy(w["theta"], w["eps"])  # over the tree of the last warm-up step

    gpu_index = dist.gpu_index()
    # a literal cell is a point mass at its pseudo-barycentre (Q = 0): the point-mass flops
    cell_flops = FLOPS_CELL_QUAD if mode == 1 else FLOPS_P2P
    per_step_ms, walk_ms, sort_ms, flops, inter, util_cell, util_pt = [], [], [], [], [], [], []
    stage = {}
    launches = 0
    dist.barrier()
    sim.synchronize()
    with ClockSampler(gpu_index) as clocks:
        t_wall = time.perf_counter()
        for k in range(args.steps):
            # the step as a caller runs it: bh_step without stats (its graph records no stage
            # events), timed by CUDA events on the library stream around the call
            sim.flush_l2()
            sim.event_record(0)
            sim.step(prm, 1, stats=False)
            sim.event_record(1)
            per_step_ms.append(sim.event_elapsed_ms(0, 1))
        sim.synchronize()
        wall = time.perf_counter() - t_wall
    dist.barrier()
    energy1 = sim.energy(w["theta"], w["eps"])
    p_now, v_now, _ = sim.get_bodies()
    mv = float(np.sum(p_now[:, 3].astype(np.float64) * np.linalg.norm(v_now[:, :3].astype(np.float64), axis=1)))
    # a second pass of K steps with bh_stats (stage events inside the graph, interaction counts)
    # for the stage split, the rooflines and the launch count; outside the timed region
    for k in range(args.steps):
        sim.flush_l2()
        st = sim.step(prm, 1, stats=True)
        walk_ms.append(st.ms_walk)
        sort_ms.append(st.ms_sort)
        flops.append(FLOPS_P2P * st.interactions_p2p + cell_flops * st.interactions_cell)
        inter.append(st.interactions_p2p + st.interactions_cell)
        util_cell.append((st.interactions_cell, st.walk_cell_evals))
        util_pt.append((st.interactions_p2p, st.walk_point_evals))
        launches += st.kernel_launches
        for key, val in st.as_dict().items():
            if key.startswith("ms_"):
                stage[key] = stage.get(key, 0.0) + val
    conservation = {
        "steps": args.steps,
        "energy_drift": (energy1["total"] - energy0["total"]) / abs(energy0["total"]),
        "momentum_drift": float(np.linalg.norm(np.subtract(energy1["momentum"], energy0["momentum"]))) / mv,
        "angular_momentum_drift": float(np.linalg.norm(np.subtract(energy1["angular_momentum"],
                                                                   energy0["angular_momentum"]))) / mv,
        "energy_start": energy0, "energy_end": energy1,
        "potential": "tree potential (bh_energy_diag) at the run's theta, eps and quadrupoles; momentum "
                     "drifts relative to sum m|v|"}
    total_ms = dist.max(sum(per_step_ms))
    bodies_all = dist.sum(n * args.steps)
    value = bodies_all / (total_ms * 1e-3)

    # end to end through the C ABI with host buffers (pinned), one step per sample
    e2e_ms = []
    pin_p = bh.PinnedArray((n, 4))
    pin_v = bh.PinnedArray((n, 4))
    pin_p.array[:] = pm
    pin_v.array[:] = vel
    out_p = bh.PinnedArray((n, 4))
    out_v = bh.PinnedArray((n, 4))
    # one warm-up call captures the step with its copies; the timed calls replay it
    sim.set_bodies(pm, vel)
    sim.step_host(prm, pin_p.array, pin_v.array, out_p.array, out_v.array, stats=False)
    for k in range(max(3, min(args.steps, 10))):
        sim.flush_l2()
        sim.event_record(0)
        sim.step_host(prm, pin_p.array, pin_v.array, out_p.array, out_v.array, stats=False)
        sim.event_record(1)
        e2e_ms.append(sim.event_elapsed_ms(0, 1))
    e2e_value = dist.sum(n) / (dist.max(statistics.median(e2e_ms)) * 1e-3)
    for a in (pin_p, pin_v, out_p, out_v):
        a.free()

    mean_walk = statistics.mean(walk_ms)
    walk_flops = statistics.mean(flops)
    # a stage time the library could not read comes back as 0: no rate is derived from it
    achieved_tflops = walk_flops / (mean_walk * 1e-3) / 1e12 if mean_walk > 0 else None
    peaks = measured_peaks()
    hbm_peak = peaks.get("hbm_gbs")
    sort_bytes = n * (8 + 24 * SORT_PASSES)
    sort_gbs = sort_bytes / (statistics.mean(sort_ms) * 1e-3) / 1e9 if statistics.mean(sort_ms) > 0 else None
    nodes = int(st.n_nodes)
    build_bytes = n * 24 + nodes * (64 + 16) + nodes * 64
    build_ms = (stage.get("ms_build", 0.0) + stage.get("ms_upsweep", 0.0)) / args.steps
    traffic = ncu_traffic()
    walk_traffic = None
    if traffic and traffic.get("bytes_per_body"):
        walk_traffic = traffic["bytes_per_body"] * n

    line = {
        "metric": METRIC, "value": value, "unit": "body-steps/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (keys, bounds and tree geometry in f64; node masses and centres in float-float)",
        "data": "synthetic", "impl": "ours",
        "config": workload_config(args, w),
        "timing": "per-step CUDA events on the library stream around each bh_step call (graph launch "
                  "included; no stage events in the graph); L2 flushed between steps; the stage split, "
                  "rooflines and launch count come from a second pass of K steps with bh_stats",
        "parallelism": f"replicas x{args.gpus}" if args.gpus > 1 else "single GPU",
        "e2e": {"value": e2e_value, "unit": "body-steps/s", "h2d_bytes_per_step": 32 * n, "d2h_bytes_per_step": 32 * n,
                "ms_per_step": statistics.median(e2e_ms)},
        "interactions_per_s": dist.sum(sum(inter)) / (total_ms * 1e-3),
        "interactions_per_body": statistics.mean(inter) / n,
        "roofline": {"kernel": "k_walk<quadrupole>" if mode == 1 else "k_walk<literal>", "bound": "fp32", "achieved": achieved_tflops,
                     "peak": fp32_peak, "unit": "TFLOP/s", "frac": achieved_tflops / fp32_peak if achieved_tflops else None,
                     "peak_source": "measured FP32 FMA peak of this GPU (bh_measure_fp32_peak)",
                     "traffic": walk_traffic,
                     "flops_per_launch": walk_flops, "ms_per_launch": mean_walk},
        "roofline_sort": {"kernel": "onesweep radix sort (Morton keys)", "bound": "hbm", "achieved": sort_gbs,
                          "peak": hbm_peak, "unit": "GB/s",
                          "frac": (sort_gbs / hbm_peak) if hbm_peak and sort_gbs else None,
                          "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)",
                          "bytes_per_launch": sort_bytes},
        # node discovery + multipoles: N x 24 B (keys, positions) + M x (64 + 16) B (walk records,
        # node keys and ranges) + M x 64 B (upsweep records), M = nodes of the step
        "roofline_build": {"kernel": "k_nodes_count/scan/write/link + k_upsweep_links + k_upsweep", "bound": "hbm",
                           "achieved": build_bytes / (build_ms * 1e-3) / 1e9 if build_ms > 0 else None,
                           "peak": hbm_peak, "unit": "GB/s",
                           "frac": (build_bytes / (build_ms * 1e-3) / 1e9 / hbm_peak) if hbm_peak and build_ms > 0
                           else None,
                           "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)",
                           "bytes_per_step": build_bytes, "nodes": nodes,
                           "note": "node records at all depths at once; the upsweep is latency-bound (float-float chains per leaf, see profiles)"},
        "stage_ms_per_step": {k[3:]: v / args.steps for k, v in stage.items()},
        "walk_lane_utilization": {
            "cells": sum(a for a, _ in util_cell) / max(1, 32 * sum(b for _, b in util_cell)),
            "points": sum(a for a, _ in util_pt) / max(1, 32 * sum(b for _, b in util_pt)),
            "cell_share": sum(a for a, _ in util_cell) / max(1, sum(inter))},
        "gpu_launches": launches,
        "wall_s_timed_loop": wall,
        "accuracy": accuracy,
        "conservation": conservation,
        "autotune": tune,
    }
    if dist.rank == 0:
        line["clocks"] = clocks.summary()
    sim.close()
    if args.workload == "plummer-4m" and not args.no_modes:
        # the batched and reverse-mode halves of the metric, measured in the same run
        line["ensemble"] = ensemble_summary(measure_ensemble(bh, dist, MODE_STEPS, MODE_WARMUP, args.loop_sample,
                                                             with_cpu=False))
        line["adjoint"] = adjoint_summary(measure_adjoint(bh, dist, MODE_STEPS, MODE_WARMUP, with_cpu=False))
    if dist.rank == 0:
        if dist.ws == 1 and not args.no_cpu_baseline:
            nthreads = os.cpu_count() or 1
            line["cpu_baseline"] = cpu_baseline_whole_step(bh, w, pm, vel, nthreads)
            line["cpu_serial"] = cpu_serial_config0(bh)
        print(json.dumps(line), flush=True)


ENSEMBLE = dict(nsys=4096, nmin=256, nmax=65536, theta=0.6, eps=0.01, leaf=8, dt=1e-3, edge=2.0, seed=1000,
                desc="4096 Plummer systems (device generator, seed 1000 + s), N_s = round(exp(U ln 256 + ln 256)) "
                     "in [256, 65536], M = a = 1 each, theta=0.6, eps=0.01, leaf 8, dt=1e-3, quadrupole, edge 2S")


def measure_ensemble(bh, dist, steps, warmup, loop_sample, with_cpu):
    """Batched ensemble: all systems in one bh_batch_step per step (graph-replayed), against the
    plain path looped over the systems (each system resident in its own context, one bh_step
    call per system per step, wall-clock), estimated from a seeded sample of systems. Returns the
    workload's JSON line (every rank; rank 0 prints it)."""
    e = ENSEMBLE
    rng = np.random.default_rng(e["seed"])
    u = rng.uniform(0.0, 1.0, e["nsys"])
    sizes = np.round(np.exp(u * np.log(e["nmax"] / e["nmin"]) + np.log(e["nmin"]))).astype(np.int64)
    off = np.concatenate([[0], np.cumsum(sizes)]).astype(np.uint32)
    n = int(off[-1])
    prm = bh.default_params(theta=e["theta"], eps=e["eps"], dt=e["dt"], leaf_capacity=e["leaf"],
                            multipole=bh.BH_MULTIPOLE_QUADRUPOLE, edge_factor=e["edge"], acc_follows_body=1)
    sim = dist.simulation(bh, n)
    # the ensemble's initial conditions come from the device generator (system s: seed + s)
    sim.batch_plummer_device(e["seed"], off)
    pos, vel, _ = sim.get_bodies()
    fp32_peak = sim.fp32_peak_tflops()
    sim.batch_step(prm, 1, stats=False)
    tune = sim.autotune(e["theta"], e["eps"], trials=2)  # walk launch shape for this ensemble
    for _ in range(warmup - 1):  # re-captures the step graph with the chosen walk
        sim.batch_step(prm, 1, stats=False)
    per_step, flops, walk_ms, util = [], [], [], []
    stage = {}
    launches = 0
    dist.barrier()
    with ClockSampler(dist.gpu_index()) as clocks:
        for _ in range(steps):
            sim.flush_l2()
            st = sim.batch_step(prm, 1)
            launches += st.kernel_launches
            per_step.append(st.ms_step)
            walk_ms.append(st.ms_walk)
            flops.append(FLOPS_P2P * st.interactions_p2p + FLOPS_CELL_QUAD * st.interactions_cell)
            util.append((st.interactions_cell, st.walk_cell_evals, st.interactions_p2p, st.walk_point_evals))
            for key, val in st.as_dict().items():
                if key.startswith("ms_"):
                    stage[key] = stage.get(key, 0.0) + val
    total_ms = dist.max(sum(per_step))
    value = dist.sum(n * steps) / (total_ms * 1e-3)
    # end to end: bh_batch_step_host uploads every system's positions and velocities from pinned
    # host memory, steps the ensemble and downloads them, its copies beside the step (one call
    # captures; the timed calls replay)
    pp, pv = bh.PinnedArray((n, 4)), bh.PinnedArray((n, 4))
    op, ov = bh.PinnedArray((n, 4)), bh.PinnedArray((n, 4))
    cur_p, cur_v, _ = sim.get_bodies()
    pp.array[:] = cur_p
    pv.array[:] = cur_v
    sim.batch_step_host(prm, pp.array, pv.array, op.array, ov.array, stats=False)
    e2e = []
    # seven calls, the median reported: some runs showed one or two calls of 150-230 ms among
    # ~118 ms ones (the 1.5 GB host copies), and three calls let two such outliers set the median
    for _ in range(7):
        sim.event_record(0)
        sim.batch_step_host(prm, pp.array, pv.array, op.array, ov.array, stats=False)
        sim.event_record(1)
        e2e.append(sim.event_elapsed_ms(0, 1))
    for a in (pp, pv, op, ov):
        a.free()
    sim.close()
    # the plain path looped over the systems, on a seeded sample of systems
    rng = np.random.default_rng(7)
    sample = np.sort(rng.choice(e["nsys"], min(loop_sample, e["nsys"]), replace=False))
    loop_s = []
    for s in sample:
        a, b = int(off[s]), int(off[s + 1])
        with dist.simulation(bh, b - a) as one:
            one.set_bodies(pos[a:b], vel[a:b])
            for _ in range(2):
                one.step(prm, 1, stats=False)
            t = []
            for _ in range(3):
                t0 = time.perf_counter()
                one.step(prm, 1, stats=False)
                t.append(time.perf_counter() - t0)
            loop_s.append(statistics.median(t))
    loop_step_s = sum(loop_s) * e["nsys"] / len(sample)
    walk_tflops = statistics.mean(flops) / (statistics.mean(per_step) * 1e-3) / 1e12
    walk_only_tflops = statistics.mean(flops) / (statistics.mean(walk_ms) * 1e-3) / 1e12 if min(walk_ms) > 0 else None
    cpu = None
    if dist.rank == 0 and with_cpu:
        # the oracle port on one core over 12 seeded systems, scaled by sum N log N
        sizes = np.diff(off).astype(np.float64)
        pick = np.sort(np.random.default_rng(8).choice(e["nsys"], 12, replace=False))
        secs = cpu_steps_sample([(pos[off[s]:off[s + 1]], vel[off[s]:off[s + 1]]) for s in pick], e["theta"],
                                e["eps"], e["dt"], e["leaf"], e["edge"])
        nlogn = sizes * np.log(sizes)
        cpu_step_s = sum(secs) * float(nlogn.sum() / nlogn[pick].sum())
        cpu = {"value": n / cpu_step_s, "unit": "body-steps/s", "cores": 1, "kind": "port",
               "sample": f"one oracle-port step of 12 seeded systems ({sum(secs):.1f} s, "
                         f"{int(sizes[pick].sum())} bodies), scaled by sum N log N to all {e['nsys']} systems: "
                         f"{cpu_step_s:.0f} s per ensemble step"}
    line = {"metric": METRIC, "value": value, "unit": "body-steps/s", "n_gpus": dist.ws, "steps": steps,
            "warmup": warmup, "ms_per_step": total_ms / steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "ours",
            "config": {"workload": "ensemble-4096", "systems": e["nsys"], "bodies": n, "desc": e["desc"]},
            "timing": "per-step CUDA events inside the captured step; L2 flushed between steps",
            "e2e": {"value": n / (statistics.median(e2e) * 1e-3), "unit": "body-steps/s",
                    "h2d_bytes_per_step": 32 * n, "d2h_bytes_per_step": 32 * n,
                    "ms_per_step": statistics.median(e2e), "samples_ms": e2e},
            "plain_loop": {"value": n / loop_step_s, "unit": "body-steps/s", "seconds_per_step": loop_step_s,
                           "sample": (f"all {e['nsys']} systems" if len(sample) == e["nsys"] else
                                      f"{len(sample)} seeded systems, sum scaled by {e['nsys']}/{len(sample)}") +
                                     ", each in its own context, wall-clock bh_step (median of 3)"},
            "batched_speedup_vs_plain_loop": loop_step_s / (total_ms / steps * 1e-3),
            "flops_per_step": statistics.mean(flops), "tflops": walk_tflops,
            "fp32_peak_tflops": fp32_peak, "gpu_launches": launches, "autotune": tune,
            "roofline": {"kernel": "k_walk<quadrupole> (ensemble groups)", "bound": "fp32",
                         "achieved": walk_only_tflops, "peak": fp32_peak, "unit": "TFLOP/s",
                         "frac": (walk_only_tflops / fp32_peak) if walk_only_tflops and fp32_peak else None,
                         "peak_source": "measured FP32 FMA peak of this GPU (bh_measure_fp32_peak)",
                         "traffic": None, "flops_per_launch": statistics.mean(flops),
                         "ms_per_launch": statistics.mean(walk_ms)},
            "stage_ms_per_step": {k[3:]: v / steps for k, v in stage.items()},
            "walk_lane_utilization": {
                "cells": sum(u[0] for u in util) / max(1, 32 * sum(u[1] for u in util)),
                "points": sum(u[2] for u in util) / max(1, 32 * sum(u[3] for u in util))},
            "interactions_per_body": statistics.mean(u[0] + u[2] for u in util) / n,
            "clocks": clocks.summary()}
    if cpu:
        line["cpu_baseline"] = cpu
    return line


def ensemble_summary(line):
    """The ensemble figures carried in the headline line."""
    keys = ("value", "unit", "ms_per_step", "steps", "warmup", "batched_speedup_vs_plain_loop", "gpu_launches")
    out = {k: line[k] for k in keys}
    out["plain_loop_ms_per_step"] = line["plain_loop"]["seconds_per_step"] * 1e3
    out["plain_loop_sample"] = line["plain_loop"]["sample"]
    out["e2e"] = line["e2e"]
    out["config"] = line["config"]
    out["walk_frac"] = line["roofline"]["frac"]
    return out


def run_ensemble(args, dist):
    import __graft_entry__

    bh = __graft_entry__.package()
    bh.load()
    line = measure_ensemble(bh, dist, args.steps, args.warmup, args.loop_sample, not args.no_cpu_baseline)
    if dist.rank == 0:
        print(json.dumps(line), flush=True)


ADJOINT = dict(n=65536, nsteps=200, every=20, theta=0.5, eps=0.01, leaf=8, dt=1e-3, edge=1.0, seed=1, tseed=2,
               desc="Plummer sphere N=65536 (seed 1), 200 KDK steps, dt=1e-3, theta=0.5, eps=0.01, leaf 8, "
                    "quadrupole; loss = mean squared distance of final positions to the final positions of a run "
                    "with lognormal(0.1) mass factors (seed 2); checkpoints every 20 steps")


def measure_adjoint(bh, dist, steps, warmup, with_cpu):
    """Reverse mode: a step is one gradient of the loss over the whole 200-step trajectory
    (bh_adjoint_forward with checkpoints + bh_step_backward with recomputation). Beside it, the
    plain forward path (bh_step) over the same 200 steps, so the backward/forward cost ratio is
    measured in the same run. Returns the workload's JSON line."""
    a = ADJOINT
    n, ns = a["n"], a["nsteps"]
    pm, vel = bh.plummer(a["seed"], n)
    prm = bh.default_params(theta=a["theta"], eps=a["eps"], dt=a["dt"], leaf_capacity=a["leaf"],
                            multipole=bh.BH_MULTIPOLE_QUADRUPOLE, edge_factor=a["edge"], acc_follows_body=1)
    sim = dist.simulation(bh, n)
    tpm = pm.copy()
    tpm[:, 3] *= np.random.default_rng(a["tseed"]).lognormal(0.0, 0.1, n).astype(np.float32)
    sim.set_bodies(tpm, vel)
    sim.adjoint_forward(prm, ns, ns)
    target = sim.get_bodies()[0][:, :3].copy()

    def gradient(timed):
        sim.set_bodies(pm, vel)
        if timed:
            sim.flush_l2()
        f = sim.adjoint_forward(prm, ns, a["every"])
        p = sim.get_bodies()[0]
        dl = (2.0 * (p[:, :3] - target) / n).astype(np.float32)
        if timed:
            sim.flush_l2()
        g = sim.step_backward(dl, None, stats=True)
        return f, g[3], float(np.mean(np.sum((p[:, :3] - target) ** 2, axis=1)))

    for _ in range(warmup):
        gradient(False)
    fwd, bwd, launches = [], [], 0
    dist.barrier()
    with ClockSampler(dist.gpu_index()) as clocks:
        for _ in range(steps):
            f, b, loss = gradient(True)
            fwd.append(f.ms_step)
            bwd.append(b.ms_step)
            launches += f.kernel_launches + b.kernel_launches
        # the plain forward path over the same trajectory length
        plain = []
        for _ in range(max(2, steps)):
            sim.set_bodies(pm, vel)
            sim.flush_l2()
            plain.append(sim.step(prm, ns).ms_step)
    total_ms = dist.max(sum(fwd) + sum(bwd))
    value = dist.sum(n * ns * steps) / (total_ms * 1e-3)
    # end to end through the C ABI: host state in, loss cotangent in, gradients out
    pp, pv, pd = bh.PinnedArray((n, 4)), bh.PinnedArray((n, 4)), bh.PinnedArray((n, 4))
    pp.array[:] = pm
    pv.array[:] = vel
    e2e = []
    for _ in range(2):
        sim.event_record(0)
        sim.set_bodies(pp.array, pv.array)
        sim.adjoint_forward(prm, ns, a["every"], stats=False)
        p = sim.get_bodies()[0]
        pd.array[:, :3] = 2.0 * (p[:, :3] - target) / n
        sim.step_backward(pd.array, None)
        sim.event_record(1)
        e2e.append(sim.event_elapsed_ms(0, 1))
    for x in (pp, pv, pd):
        x.free()
    sim.close()
    plain_ms = statistics.median(plain)
    cpu = None
    if dist.rank == 0 and with_cpu:
        secs = cpu_steps_sample([(pm, vel)] * 2, a["theta"], a["eps"], a["dt"], a["leaf"], a["edge"])
        per = statistics.mean(secs)
        cpu = {"value": n / per, "unit": "body-steps/s (forward only)", "cores": 1, "kind": "port",
               "sample": f"two oracle-port forward steps of the N={n} system ({sum(secs):.1f} s); the reference "
                         f"has no reverse mode, so this is its forward cost per step"}
    line = {"metric": METRIC, "value": value, "unit": "body-steps/s (differentiated)", "n_gpus": dist.ws,
            "steps": steps, "warmup": warmup, "ms_per_step": total_ms / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "impl": "ours",
            "config": {"workload": "adjoint-64k", "bodies": n, "kdk_steps": ns, "checkpoint_every": a["every"],
                       "desc": a["desc"]},
            "timing": "a step = one gradient over the 200-step trajectory; CUDA events around "
                      "bh_adjoint_forward and bh_step_backward; L2 flushed before each",
            "forward_ms": statistics.median(fwd), "backward_ms": statistics.median(bwd),
            "plain_forward_ms": plain_ms,
            "backward_over_forward": statistics.median(bwd) / plain_ms,
            "gradient_over_forward": (statistics.median(fwd) + statistics.median(bwd)) / plain_ms,
            "loss": loss,
            "gradient_checks": "tests/test_gpu_adjoint.py (FP64 frozen-list central differences, FP64 "
                               "direct-sum adjoint)",
            "e2e": {"value": n * ns / (statistics.median(e2e) * 1e-3), "unit": "body-steps/s (differentiated)",
                    "h2d_bytes_per_step": 48 * n, "d2h_bytes_per_step": 32 * n + 36 * n,
                    "ms_per_step": statistics.median(e2e)},
            "gpu_launches": launches, "clocks": clocks.summary()}
    if cpu:
        line["cpu_baseline"] = cpu
    return line


def adjoint_summary(line):
    """The reverse-mode figures carried in the headline line."""
    keys = ("value", "unit", "ms_per_step", "steps", "warmup", "forward_ms", "backward_ms", "plain_forward_ms",
            "backward_over_forward", "gradient_over_forward", "gpu_launches", "e2e", "config")
    return {k: line[k] for k in keys}


def run_adjoint(args, dist):
    import __graft_entry__

    bh = __graft_entry__.package()
    bh.load()
    line = measure_adjoint(bh, dist, args.steps, args.warmup, not args.no_cpu_baseline)
    if dist.rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="plummer-4m",
                    choices=sorted(WORKLOADS) + ["ensemble-4096", "adjoint-64k"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--no-modes", action="store_true",
                    help="skip the ensemble and adjoint figures of the default workload's line")
    ap.add_argument("--loop-sample", type=int, default=4096,
                    help="systems of the ensemble timed in the per-system loop of the plain path (all 4096 by default)")
    args = ap.parse_args()
    if args.warmup < 3:
        log("warning: fewer than 3 warm-up steps")
    dist = Dist()
    if args.workload in ("ensemble-4096", "adjoint-64k") and args.impl == "reference":
        if dist.rank == 0:
            why = ("the reference has no batched mode" if args.workload == "ensemble-4096"
                   else "the reference has no reverse mode")
            print(json.dumps({"impl": "reference", "unavailable": why}), flush=True)
        return
    if args.workload == "ensemble-4096":
        run_ensemble(args, dist)
        return
    if args.workload == "adjoint-64k":
        run_adjoint(args, dist)
        return
    w = WORKLOADS[args.workload]
    if args.impl == "reference":
        run_reference(args, w, dist)
    else:
        run_ours(args, w, dist)


if __name__ == "__main__":
    main()
