"""Benchmark of the red.cuda hot path on GB300 (one JSON line on stdout).

Workload (default): one planetesimal disk of N = 16384 bodies -- 1 star, 16
protoplanets of 0.05 M_earth spaced 10 mutual Hill radii from 0.5 AU, 16367
planetesimals log-uniform in [0.5, 3] AU -- integrated with adaptive RKF7(8)
at tolerance 1e-10, collision detection on, mixed precision (FP32 pairwise
gravity on double-single coordinates, FP64 star term, state and step control).
A step is one try of the integrator over the disk (13 force evaluations, the
error norm, step control, y_{n+1}, the collision check).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--config c2|c1|c3|c4|c5|dense|cube] [--precision mixed|fp64|fp32|fp64_exact]

Timing: CUDA events on the integration stream around each step, L2 flushed
(a 256 MiB write) between timed steps; value = total interactions over all
ranks / max over ranks of the summed step time.  `e2e` is the same metric
through the C ABI with the state of every system copied host->device before
and device->host after every step (red_set_states / red_step /
red_get_states, pinned host arrays).
`--impl reference` times red's path on the host CPU: the oracle's
restatement of red's code (the reference's own sources are not on the GPU
host), with all host threads.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time
import types

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
import __graft_entry__  # noqa: E402

K_GAUSS = 0.01720209895
YEAR = 365.25
METRIC = "interactions/s and sim-years/s vs plain FP64 on same GPU at |ΔE/E|≤1e-9"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def workload(rg, name, rank=0, world=1):
    """(systems, integrator kwargs, description) of one rank: the ensemble is
    split by systems (rank r owns its own 512 seeded disks), a single disk
    is replicated on every rank."""
    ic = rg.ic
    if name == "c1":
        s = ic.config1()
        return [s], dict(integrator="rk4", adaptive=False, dt=0.5 * K_GAUSS, collision_factor=1.0), \
            "config1: 1 star + 4 protoplanets + 2048 planetesimals, RK4 fixed dt = 0.5 d, collisions on"
    if name == "c3":
        s = ic.config3()
        gas = ic.gas_params(ic.gas_disk_config3())
        return [s], dict(integrator="rkf78", adaptive=True, tolerance=1e-10, dt=1.0 * K_GAUSS, gas=gas,
                         collision_factor=1.0), \
            "config3: 1 star + 32 protoplanets + 65503 planetesimals (1-100 km), analytic gas drag, RKF7(8) tol 1e-10"
    if name == "c4":
        first, count = rg.shard.ensemble_range(512, rank, world)
        systems = ic.config4(n_systems=count, first=first)
        return systems, dict(integrator="rkf78", adaptive=True, tolerance=1e-10, dt=1.0 * K_GAUSS,
                             collision_factor=1.0), \
            "config4: 512 disks, N ~ U[128, 4096], 2-8 protoplanets each, RKF7(8) tol 1e-10, per-system dt"
    if name == "c5":
        first, count = rg.shard.ensemble_range(512, rank, world)
        systems = ic.config4(n_systems=count, first=first)
        return systems, dict(integrator="rkf78", adaptive=True, tolerance=1e-10, dt=1.0 * K_GAUSS,
                             collision_factor=1.0), \
            "config5: the config4 ensemble with learned step proposals (BF16 MLP 12-64-64-1 trained on the GPU " \
            "on the feature log of plain runs of the same ensemble), RKF7(8) tol 1e-10"
    if name == "dense":
        s = ic.config2().relabel_all_SI()
        return [s], dict(integrator="rkf78", adaptive=True, tolerance=1e-10, dt=1.0 * K_GAUSS,
                         collision_factor=0.0), \
            "config2 relabelled all-SI (every pair interacts, N = 16384), RKF7(8) tol 1e-10"
    if name == "cube":
        s = ic.benchmark_cube(16384)
        return [s], dict(integrator="rk4", adaptive=False, dt=1e-3, collision_factor=0.0), \
            "red's benchmark cube: 16384 unit masses in [-50, 50]^3, all pairs, RK4 fixed step"
    s = ic.config2()
    return [s], dict(integrator="rkf78", adaptive=True, tolerance=1e-10, dt=1.0 * K_GAUSS,
                     collision_factor=1.0), \
        "config2: 1 star + 16 protoplanets + 16367 planetesimals, RKF7(8) tol 1e-10, collisions on"


def n_stage(kw):
    if kw["integrator"] == "rk4":
        return 5 if kw.get("adaptive") else 4
    return 13 if kw.get("adaptive") else 11


class ClockSampler:
    """nvidia-smi clocks / throttle reasons every 200 ms while running."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
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
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def flush_l2(torch, buf):
    buf.add_(1.0)


def timed_steps(torch, sim, stream, steps, flush):
    """Per-step CUDA events on the integration stream; L2 flushed between steps."""
    tot = 0.0
    for _ in range(steps):
        if flush is not None:
            with torch.cuda.stream(stream):
                flush_l2(torch, flush)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.launch_tries(1)
        e1.record(stream)
        e1.synchronize()
        tot += e0.elapsed_time(e1)
    return tot


def drain_events(sim):
    _, n_halted = sim.synchronize()
    if n_halted:
        sim.handle_events()


def roofline_for(rg, sim, systems, kw, peaks, traffic_per_launch):
    """Average launch duration of each kernel kind over a few kernel-by-kernel
    tries, and the roofline of the kind that takes the most time."""
    tot = {}
    cnt = {}
    for _ in range(5):
        ms, kind = sim.profile_try()
        for m, k in zip(ms, kind):
            tot[int(k)] = tot.get(int(k), 0.0) + float(m)
            cnt[int(k)] = cnt.get(int(k), 0) + 1
        drain_events(sim)
    names = {0: "stage", 1: "control", 2: "finish", 3: "collision", 4: "ejhc", 5: "proposer"}
    share = {names[k]: tot[k] / sum(tot.values()) for k in tot}
    ms_by_kind = {names[k]: tot[k] / 5 for k in tot}   # ms per try of each kind (5 profiled tries)
    dom = max(tot, key=lambda k: tot[k])
    avg_ms = tot[dom] / cnt[dom]
    n_body = sum(s.n for s in systems)
    hbm = peaks.get("hbm_gbs", 6800.0)
    ns = n_stage(kw)
    if names[dom] == "stage":
        # RKF7(8): (nnz_r + 2) * 48 B per body for stage r, + 4 * 48 B error read, over 13 launches
        if kw["integrator"] == "rkf78":
            nnz = [0, 1, 2, 2, 3, 3, 4, 4, 6, 7, 8, 6, 9]
            per_try = sum((nnz[r] + 2) * 48 for r in range(1, ns)) + (4 * 48 if kw.get("adaptive") else 0)
        else:
            per_try = 3 * 3 * 48 + (2 * 48 if kw.get("adaptive") else 0)
        per_launch = per_try * n_body / ns
    elif names[dom] == "finish":
        per_launch = 9 * 48 * n_body
    elif names[dom] == "collision":
        per_launch = 32 * n_body
    else:
        per_launch = 48 * n_body
    achieved = per_launch / (avg_ms * 1e-3) / 1e9
    out = {"kernel": names[dom], "bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
           "frac": achieved / hbm, "traffic": traffic_per_launch.get(names[dom]), "avg_launch_ms": avg_ms,
           "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if "hbm_gbs" in peaks else "fallback",
           "share": share, "ms_per_try_by_kind": ms_by_kind}
    if names[dom] == "stage":
        # the same launch against the FP32 pipe: 20 FLOP per directed interaction
        tflops = 20.0 * sim.interactions_per_eval / (avg_ms * 1e-3) / 1e12
        peak32 = FP32_NOMINAL_TFLOPS
        out["gravity_fp32"] = {"achieved": tflops, "peak": peak32, "unit": "TFLOP/s", "frac": tflops / peak32,
                               "peak_source": "nominal: 152 SMs x 128 FP32 lanes x 2 FLOP x 2.07 GHz"}
    return out


def cpu_baseline_sample(systems, kw, seconds=10.0):
    """The oracle restatement of red's step on a bounded sample of the
    workload, all host threads; interactions/s counted like the GPU arm."""
    import oracle
    s = systems[0]
    nth = os.cpu_count() or 1
    b = oracle.Body(s.r, s.v, s.p, s.md, s.playing)
    kind = oracle.RK4 if kw["integrator"] == "rk4" else oracle.RKF78
    ig = oracle.make_integrator(kind, kw["dt"], adaptive=kw.get("adaptive", False), tol=kw.get("tolerance", 0.0),
                                nthreads=nth)
    ipe = oracle.interactions_per_eval(s.playing)
    ns = n_stage(kw)
    t = 0.0
    t0 = time.perf_counter()
    tries = 0
    steps = 0
    sim_t = 0.0
    while time.perf_counter() - t0 < seconds or steps == 0:
        before = ig.n_tried
        rc, t_new = oracle.step(ig, b, t)
        if rc:
            raise RuntimeError("oracle step failed %d" % rc)
        if kw.get("collision_factor", 0.0) > 0.0:
            oracle.check_collision(b, t_new, kw["collision_factor"], nthreads=nth)
        sim_t += t_new - t
        t = t_new
        tries += ig.n_tried - before
        steps += 1
    el = time.perf_counter() - t0
    inter = ipe * ns * tries
    return {"value": inter / el, "unit": "interactions/s", "cores": nth, "kind": "port",
            "sample": "%d oracle steps (%d tries) of the workload's first system, %.1f s" % (steps, tries, el),
            "sim_years_per_s": sim_t / K_GAUSS / YEAR / el}


FP32_NOMINAL_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12   # GB300 FP32 FMA, nominal
PROPOSER_WARMUP_TRIES = 400   # tries before the timed region in the learned-proposal workload


def train_proposer(rg, systems, kw, args, local_rank, stream, log_tries=PROPOSER_WARMUP_TRIES):
    """The proposer's training data and network: a plain run of the ensemble
    logs (features, accepted log|dt|) records on the device; the network is
    trained on the GPU by the library's own kernels."""
    sim = rg.Sim(systems, precision=args.precision, device=local_rank, stream=stream.cuda_stream, **kw)
    sim.log_features(1 << 22)
    for _ in range(log_tries // 100):
        sim.launch_tries(100)
        drain_events(sim)
    recs = sim.feature_log(cap=1 << 22)
    sim.close()
    t0 = time.perf_counter()
    bits, nm, hist = rg.proposer.train(recs, epochs=30, batch=2048, lr=2e-3)
    return {"bits": bits, "norm": nm, "records": int(len(recs)), "train_s": time.perf_counter() - t0,
            "val_loss": hist[-1][2]}


def plain_comparison(rg, systems, kw, args, local_rank, stream, flush):
    """The same ensemble with the classical controller, timed the same way."""
    import torch
    sim = rg.Sim(systems, precision=args.precision, device=local_rank, stream=stream.cuda_stream, **kw)
    for _ in range(max(3, args.warmup)):
        sim.launch_tries(1)
    drain_events(sim)
    for _ in range(PROPOSER_WARMUP_TRIES // 100):
        sim.launch_tries(100)
        drain_events(sim)
    info0 = [sim.info(k) for k in range(sim.n_systems)]
    ms = timed_steps(torch, sim, stream, args.steps, flush)
    drain_events(sim)
    info1 = [sim.info(k) for k in range(sim.n_systems)]
    sim.close()
    tried = sum(b.n_tried - a.n_tried for a, b in zip(info0, info1))
    failed = sum(b.n_failed - a.n_failed for a, b in zip(info0, info1))
    sim_dt = sum(b.t - a.t for a, b in zip(info0, info1))
    return {"rejected_fraction": failed / tried if tried else None,
            "sim_years_per_s": sim_dt / K_GAUSS / YEAR / (ms * 1e-3), "ms_per_step": ms / args.steps}


def run_reference(args, rg, rank, world):
    systems, kw, desc = workload(rg, args.config)
    if rank != 0:
        return
    import oracle
    oracle.build()
    sample_s = float(os.environ.get("REDGB_REF_SECONDS", "10"))
    for _ in range(args.warmup):
        pass
    res = cpu_baseline_sample(systems, kw, seconds=sample_s * max(1, args.steps) / 20.0)
    line = {"metric": METRIC, "value": res["value"], "unit": "interactions/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": desc, "seed": 2},
            "sim_years_per_s": res["sim_years_per_s"],
            "cpu_baseline": {"value": res["value"], "unit": "interactions/s", "cores": res["cores"],
                             "kind": res["kind"], "sample": res["sample"]},
            "e2e": {"value": res["value"], "unit": "interactions/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, rg, rank, world, local_rank):
    import torch
    torch.cuda.set_device(local_rank)
    t_ic = time.perf_counter()
    systems, kw, desc = workload(rg, args.config, rank, world)
    t_ic = time.perf_counter() - t_ic
    ic_gpu = None
    if args.config in ("c4", "c5"):
        # the same ensemble layout drawn by the GPU generator (red_populate_disks)
        first, count = rg.shard.ensemble_range(512, rank, world)
        rg.ic.config4_gpu(n_systems=1, first=first, device=local_rank)   # first call: library and context warm
        t_gpu = time.perf_counter()
        gen = rg.ic.config4_gpu(n_systems=count, first=first, device=local_rank)
        t_gpu = time.perf_counter() - t_gpu
        ic_gpu = {"bodies": int(sum(s.n for s in gen)), "host_numpy_s": t_ic, "gpu_s": t_gpu,
                  "api": "red_populate_disks (records copied to host memory)"}
        del gen
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    stream = torch.cuda.Stream()
    sim = rg.Sim(systems, precision=args.precision, device=local_rank, stream=stream.cuda_stream, **kw)
    ipe = sim.interactions_per_eval
    ns = n_stage(kw)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")   # 256 MiB > L2
    proposer = None
    if args.config == "c5":
        proposer = train_proposer(rg, systems, kw, args, local_rank, stream)
        sim.set_step_proposer(proposer["bits"], proposer["norm"], safety=1.0, ratio_lo=0.25, ratio_hi=4.0)
    # warm-up (graph capture happens on the first launch); the learned-proposal
    # workload first runs past the start-up phase its network was trained on
    for _ in range(max(3, args.warmup)):
        sim.launch_tries(1)
    drain_events(sim)
    if proposer is not None:
        for _ in range(PROPOSER_WARMUP_TRIES // 100):
            sim.launch_tries(100)
            drain_events(sim)
    E0 = sim.energy_interacting(0)
    t_before = [sim.info(k).t for k in range(sim.n_systems)]
    tried_before = sum(sim.info(k).n_tried for k in range(sim.n_systems))
    failed_before = sum(sim.info(k).n_failed for k in range(sim.n_systems))
    launches0 = sim.kernel_launches
    clocks = ClockSampler(local_rank)
    rg.shard.barrier(local_rank)
    torch.cuda.synchronize()
    clocks.start()
    ms = timed_steps(torch, sim, stream, args.steps, flush)
    torch.cuda.synchronize()
    rg.shard.barrier(local_rank)
    clk = clocks.stop()
    launches = sim.kernel_launches - launches0
    drain_events(sim)
    infos = [sim.info(k) for k in range(sim.n_systems)]
    tried = sum(i.n_tried for i in infos) - tried_before
    failed = sum(i.n_failed for i in infos) - failed_before
    n_fail_tries = args.steps * sim.n_systems - tried  # systems that were finished / halted
    sim_dt = float(np.sum([infos[k].t - t_before[k] for k in range(sim.n_systems)]))
    E1 = sim.energy_interacting(0)
    dE = abs((E1[0] - E0[0]) / E0[0])
    inter = ipe * ns * args.steps
    t_max = rg.shard.max_over_ranks(ms, device="cuda")
    value = inter * world / (t_max * 1e-3)
    sim_years = sim_dt / K_GAUSS / YEAR
    # roofline of the dominant kernel (kernel-by-kernel tries, CUDA events)
    try:
        traffic = json.load(open(os.path.join(ROOT, "profiles", "traffic.json"))).get(args.config, {})
    except (OSError, ValueError):
        traffic = {}
    roof = roofline_for(rg, sim, systems, kw, peaks, traffic)

    # end to end through the C ABI with host buffers: the state of every system
    # of the workload in and out each step
    n_all = sim.bodies()
    st = types.SimpleNamespace()
    host = {}
    for f, dt in (("r", rg.types.VAR4), ("v", rg.types.VAR4), ("p", rg.types.PARAM), ("md", rg.types.BMD)):
        host[f] = torch.zeros(n_all * dt.itemsize, dtype=torch.uint8).pin_memory()
        setattr(st, f, host[f].numpy().view(dt))
    sim.get_states(st)
    e2e_steps = max(3, args.steps // 2)
    torch.cuda.synchronize()
    rg.shard.barrier(local_rank)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        sim.set_states(st, parts="rv")      # inputs from pinned host memory
        sim.step()
        sim.get_states(st, parts="rv")      # results into the same pinned buffers
    e2e_s = rg.shard.max_over_ranks(time.perf_counter() - t0, device="cuda")
    drain_events(sim)
    e2e_value = ipe * ns * e2e_steps * world / e2e_s
    bytes_state = n_all * (32 + 32)

    # the plain FP64 path on the same GPU, same workload (fewer steps)
    fp64 = None
    if args.precision != "fp64" and not args.no_fp64:
        sim64 = rg.Sim(systems, precision="fp64", device=local_rank, stream=stream.cuda_stream, **kw)
        for _ in range(3):
            sim64.launch_tries(1)
        drain_events(sim64)
        k64 = max(3, args.steps // 4)
        ms64 = timed_steps(torch, sim64, stream, k64, flush)
        drain_events(sim64)
        fp64 = {"value": ipe * ns * k64 * world / (ms64 * 1e-3), "ms_per_step": ms64 / k64}
        sim64.close()

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline_sample(systems, kw, seconds=float(os.environ.get("REDGB_CPU_SECONDS", "10")))
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "interactions/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_max / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32 pairs + f64 state" if args.precision in ("mixed", "fp32") else "f64",
                "data": "synthetic",
                "config": {"workload": desc, "precision": args.precision, "l2": "flushed (256 MiB write) between timed steps",
                           "n_bodies": int(sum(s.n for s in systems)), "systems": len(systems),
                           "interactions_per_eval": ipe, "evals_per_step": ns},
                "sim_years_per_s": sim_years * world / (t_max * 1e-3),
                "dE_over_E": dE,
                "tries_in_timed_region": int(tried),
                "accept_fraction": (1.0 - failed / tried) if tried else None,
                "e2e": {"value": e2e_value, "unit": "interactions/s", "h2d_bytes_per_step": bytes_state,
                        "d2h_bytes_per_step": bytes_state, "steps": e2e_steps,
                        "api": "red_set_states(r, v) + red_step + red_get_states(r, v), every system"},
                "roofline": roof,
                "cpu_baseline": cpu,
                "plain_fp64_same_gpu": fp64,
                "vs_plain_fp64": (value / fp64["value"]) if fp64 else None,
                "clocks": clk,
                "gpu_launches": int(launches)}
        if ic_gpu is not None:
            line["initial_conditions"] = ic_gpu
        if proposer is not None:
            plain = plain_comparison(rg, systems, kw, args, local_rank, stream, flush)
            line["proposer"] = {
                "records": proposer["records"], "train_s": proposer["train_s"],
                "val_loss": proposer["val_loss"],
                "rejected_fraction": (failed / tried) if tried else None,
                "rejected_fraction_plain": plain["rejected_fraction"],
                "sim_years_per_s": sim_years * world / (t_max * 1e-3),
                "sim_years_per_s_plain": plain["sim_years_per_s"],
                "ms_per_step_plain": plain["ms_per_step"],
                "overhead_ms_per_try": t_max / args.steps - plain["ms_per_step"],
                "kernels_ms_per_try": roof["ms_per_try_by_kind"].get("proposer")}
        print(json.dumps(line), flush=True)
    sim.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c2", choices=["c1", "c2", "c3", "c4", "c5", "dense", "cube"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64", "fp32", "fp64_exact"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    rg = __graft_entry__.load_package()
    if args.impl == "reference":
        run_reference(args, rg, rank, world)
        return
    rg.build()
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    run_ours(args, rg, rank, world, local_rank)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
