"""Benchmark of the red.cuda hot path on GB300 (one JSON line on stdout).

Workload (default): one planetesimal disk of N = 16384 bodies -- 1 star, 16
protoplanets of 0.05 M_earth spaced 10 mutual Hill radii from 0.5 AU, 16367
planetesimals log-uniform in [0.5, 3] AU -- integrated with adaptive RKF7(8)
at tolerance 1e-10, collision detection on, mixed precision (FP32 pairwise
gravity on double-single coordinates, FP64 star term, state and step control).

A step is a run of `tries_per_step` consecutive tries of the integrator over
the disk (each try: 13 force evaluations, the error norm, step control,
y_{n+1}, the collision check), back to back as an integration runs them; the
count per workload makes a step last ~50 ms, so that the timed region spans
about a second and the clock record covers it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--config c2|c1|c3|c4|c5|dense|cube|cube65536] [--precision mixed|fp64|fp32|fp64_exact]
                  [--accuracy-years T] [--plan-only]

Timing: CUDA events on the integration stream around each step, L2 flushed
(a 256 MiB write) between timed steps, after W warm-up steps and a settling
run past the start-up adaptation of the step size; value = interactions of
the tries run on all ranks / max over ranks of the summed step time.  `e2e`
is the same metric through the C ABI with the state of every system copied
host->device before and device->host after every integrator step
(red_set_states / red_step / red_get_states, pinned host arrays).
`plain_fp64_same_gpu` is red's own FP64 GPU path, built from its unmodified
sources for sm_103a (oracle/ref_gpu.py), started from the same settled state.
`--impl reference` times red's path on the host CPU: the oracle's
restatement of red's code (red's CPU path cannot integrate planetesimals),
with all host threads.
`--gpus N` without torchrun starts N local ranks itself.
"""
import argparse
import json
import os
import socket
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

# tries per timed step (~50 ms of GPU time each) and untimed tries before the
# timed region that take the step size past its start-up adaptation
TRIES_PER_STEP = {"c1": 1000, "c2": 400, "c3": 120, "c4": 20, "c5": 20, "dense": 20, "cube": 60, "cube65536": 6}
SETTLE_TRIES = {"c1": 0, "c2": 600, "c3": 200, "c4": 200, "c5": 400, "dense": 100, "cube": 0, "cube65536": 0}
# steps of red's own GPU path per system (it is slower), and the ensemble's sample
RED_GPU_STEPS = {"c1": 200, "c2": 20, "c3": 4, "c4": 6, "c5": 6, "dense": 4, "cube": 10, "cube65536": 1}
RED_GPU_ENSEMBLE_SAMPLE = 16


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
    if name in ("c4", "c5"):
        first, count = rg.shard.ensemble_range(512, rank, world)
        systems = ic.config4(n_systems=count, first=first)
        kw = dict(integrator="rkf78", adaptive=True, tolerance=1e-10, dt=1.0 * K_GAUSS, collision_factor=1.0)
        if name == "c4":
            return systems, kw, \
                "config4: 512 disks, N ~ U[128, 4096], 2-8 protoplanets each, RKF7(8) tol 1e-10, per-system dt"
        return systems, kw, \
            "config5: the config4 ensemble with learned step proposals (BF16 MLP 12-64-64-1 trained on the GPU " \
            "on the feature log of plain runs of the same ensemble), RKF7(8) tol 1e-10"
    if name == "dense":
        s = ic.config2().relabel_all_SI()
        return [s], dict(integrator="rkf78", adaptive=True, tolerance=1e-10, dt=1.0 * K_GAUSS,
                         collision_factor=0.0), \
            "config2 relabelled all-SI (every pair interacts, N = 16384), RKF7(8) tol 1e-10"
    if name in ("cube", "cube65536"):
        n = 65536 if name == "cube65536" else 16384
        s = ic.benchmark_cube(n)
        return [s], dict(integrator="rk4", adaptive=False, dt=1e-3, collision_factor=0.0), \
            "red's benchmark cube: %d unit masses in [-50, 50]^3, all pairs, RK4 fixed step" % n
    s = ic.config2()
    return [s], dict(integrator="rkf78", adaptive=True, tolerance=1e-10, dt=1.0 * K_GAUSS,
                     collision_factor=1.0), \
        "config2: 1 star + 16 protoplanets + 16367 planetesimals, RKF7(8) tol 1e-10, collisions on"


def n_stage(kw):
    if kw["integrator"] == "rk4":
        return 5 if kw.get("adaptive") else 4
    return 13 if kw.get("adaptive") else 11


def ipe_of(playing):
    """Directed interactions of one force evaluation over red's interaction
    bounds (red_type.h:670-692): SI x (massive - 1) + NSI x SI + NI x massive."""
    pl = np.asarray(playing, dtype=np.int64)
    nsi, nnsi, nni = int(pl[:4].sum()), int(pl[4:6].sum()), int(pl[6])
    nm = nsi + nnsi
    return (nsi * (nm - 1) if nsi else 0) + nnsi * nsi + nni * nm


def config_object(args, systems, kw, desc, world):
    """The `config` of the JSON line; both arms print the same object."""
    return {"workload": desc, "precision": args.precision,
            "l2": "flushed (256 MiB write) between timed steps; the tries within a step run back to back",
            "tries_per_step": tries_per_step(args), "settle_tries": SETTLE_TRIES[args.config],
            "n_bodies": int(sum(s.n for s in systems)), "systems": len(systems),
            "interactions_per_eval": int(sum(ipe_of(s.playing) for s in systems)), "evals_per_step": n_stage(kw),
            "parallelism": ("ensemble split by systems over %d ranks" % world) if args.config in ("c4", "c5")
            else ("replicas of one disk on %d ranks" % world)}


def tries_per_step(args):
    return args.tries_per_step or TRIES_PER_STEP[args.config]


class ClockSampler:
    """nvidia-smi clocks / throttle reasons every 100 ms while running."""
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
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            time.sleep(0.3)     # the first sample lands before the timed region
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
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "power_w_max": float(max(power)) if power else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def timed_steps(torch, sim, stream, steps, flush, tps):
    """`steps` timed steps of `tps` tries each, enqueued back to back with a
    CUDA event pair around each step and the L2 flush between steps; one
    synchronisation at the end.  Returns the summed step time in ms."""
    evs = []
    for _ in range(steps):
        if flush is not None:
            with torch.cuda.stream(stream):
                flush.add_(1.0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.launch_tries(tps)
        e1.record(stream)
        evs.append((e0, e1))
    evs[-1][1].synchronize()
    return float(sum(e0.elapsed_time(e1) for e0, e1 in evs))


def drain_events(sim):
    _, n_halted = sim.synchronize()
    if n_halted:
        sim.handle_events()


def snapshot(sim):
    infos = [sim.info(k) for k in range(sim.n_systems)]
    return {"t": np.array([i.t for i in infos]), "tried": np.array([i.n_tried for i in infos], np.int64),
            "failed": np.array([i.n_failed for i in infos], np.int64),
            "collisions": np.array([i.n_collision[0] for i in infos], np.int64),   # total (red_type.h:156)
            "ipe": np.array([ipe_of(list(i.playing)) for i in infos], np.int64)}


FP32_NOMINAL_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12   # GB300 FP32 FMA, nominal
KIND_NAMES = {0: "stage", 1: "control", 2: "finish", 3: "collision", 4: "ejhc", 5: "proposer"}


def roofline_for(sim, systems, kw, peaks, traffic_per_launch, ms_per_try):
    """The kernel kind with the largest share of a try, against its roof.

    Each kind's share of a try comes from tries run kernel by kernel with CUDA
    events (red_profile_try); its time inside the timed graph is that share of
    the measured try time (ms_per_try), so the kinds add up to the step.
    `achieved` divides the algorithmic bytes of one launch by the launch's
    in-graph time."""
    tot, cnt = {}, {}
    for _ in range(5):
        ms, kind = sim.profile_try()
        for m, k in zip(ms, kind):
            tot[int(k)] = tot.get(int(k), 0.0) + float(m)
            cnt[int(k)] = cnt.get(int(k), 0) + 1
        drain_events(sim)
    share = {KIND_NAMES[k]: tot[k] / sum(tot.values()) for k in tot}
    dom = max(tot, key=lambda k: tot[k])
    launches_per_try = cnt[dom] / 5.0
    alone_ms = tot[dom] / cnt[dom]
    in_graph_ms = ms_per_try * share[KIND_NAMES[dom]] / launches_per_try
    n_body = sum(s.n for s in systems)
    hbm = peaks.get("hbm_gbs", 6800.0)
    ns = n_stage(kw)
    name = KIND_NAMES[dom]
    if name == "stage":
        # RKF7(8): (nnz_r + 2) * 48 B per body for stage r, + 4 * 48 B error read, over the try's launches
        if kw["integrator"] == "rkf78":
            nnz = [0, 1, 2, 2, 3, 3, 4, 4, 6, 7, 8, 6, 9]
            per_try = sum((nnz[r] + 2) * 48 for r in range(1, ns)) + (4 * 48 if kw.get("adaptive") else 0)
        else:
            per_try = 3 * 3 * 48 + (2 * 48 if kw.get("adaptive") else 0)
        per_launch = per_try * n_body / ns
    elif name == "finish":
        per_launch = 9 * 48 * n_body
    elif name == "collision":
        per_launch = 32 * n_body
    else:
        per_launch = 48 * n_body
    achieved = per_launch / (in_graph_ms * 1e-3) / 1e9
    out = {"kernel": name, "bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
           "frac": achieved / hbm, "traffic": traffic_per_launch.get(name), "algorithmic_bytes": per_launch,
           "avg_launch_ms": in_graph_ms, "avg_launch_ms_alone": alone_ms,
           "timing": "in-graph launch time = measured try time x the kind's share of kernel-by-kernel tries",
           "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if "hbm_gbs" in peaks else "fallback",
           "share": share, "ms_per_try_by_kind": {KIND_NAMES[k]: ms_per_try * share[KIND_NAMES[k]] for k in tot}}
    if name == "stage":
        # the same launch against the FP32 pipe: 20 FLOP per directed interaction
        ipe = sum(ipe_of(s.playing) for s in systems)
        tflops = 20.0 * ipe / (in_graph_ms * 1e-3) / 1e12
        out["gravity_fp32"] = {"achieved": tflops, "peak": FP32_NOMINAL_TFLOPS, "unit": "TFLOP/s",
                               "frac": tflops / FP32_NOMINAL_TFLOPS,
                               "peak_source": "nominal: 152 SMs x 128 FP32 lanes x 2 FLOP x 2.07 GHz"}
    return out


def cpu_baseline_sample(systems, kw, seconds=10.0, warmup=0, state=None):
    """The oracle restatement of red's step on a bounded sample of the
    workload (its first system), all host threads; interactions/s counted
    like the GPU arm.  `warmup` untimed oracle steps come first."""
    import oracle
    s = state if state is not None else systems[0]
    nth = os.cpu_count() or 1
    b = oracle.Body(s.r, s.v, s.p, s.md, s.playing)
    kind = oracle.RK4 if kw["integrator"] == "rk4" else oracle.RKF78
    ig = oracle.make_integrator(kind, kw["dt"], adaptive=kw.get("adaptive", False), tol=kw.get("tolerance", 0.0),
                                nthreads=nth)
    ipe = oracle.interactions_per_eval(s.playing)
    ns = n_stage(kw)
    t = 0.0
    for _ in range(warmup):
        rc, t = oracle.step(ig, b, t)
        if rc:
            raise RuntimeError("oracle step failed %d" % rc)
    t0 = time.perf_counter()
    tried0 = ig.n_tried
    steps = 0
    sim_t = 0.0
    while time.perf_counter() - t0 < seconds or steps == 0:
        rc, t_new = oracle.step(ig, b, t)
        if rc:
            raise RuntimeError("oracle step failed %d" % rc)
        if kw.get("collision_factor", 0.0) > 0.0:
            oracle.check_collision(b, t_new, kw["collision_factor"], nthreads=nth)
        sim_t += t_new - t
        t = t_new
        steps += 1
    el = time.perf_counter() - t0
    tries = ig.n_tried - tried0
    inter = ipe * ns * tries
    return {"value": inter / el, "unit": "interactions/s", "cores": nth, "kind": "port",
            "sample": "%d oracle steps (%d tries) of the workload's first system after %d warm-up steps, %.1f s"
                      % (steps, tries, warmup, el),
            "sim_years_per_s": sim_t / K_GAUSS / YEAR / el}


def red_gpu_baseline(rg, args, kw, states):
    """red's own FP64 GPU path (unmodified sources built for sm_103a,
    -fmad=false, every launch followed by a device synchronisation as red
    ships it), run system by system from `states` = [(System, dt)], each for
    RED_GPU_STEPS integrator steps after red's own thread-per-block search.
    interactions/s and sim-years/s over the summed step-loop wall time."""
    from oracle import ref_gpu
    if not ref_gpu.available():
        return {"unavailable": "red's sources are not staged under baseline/_ref (oracle/ref_stage.sh)"}
    ref_gpu.build()
    gas_keys = rg.ic.gas_disk_config3() if "gas" in kw else None
    n = RED_GPU_STEPS[args.config]
    ns = n_stage(kw)
    inter = sim_t = secs = 0.0
    tried = 0
    tpb = []
    for s, dt in states:
        r = ref_gpu.run(rg, s, kw["integrator"], dt, n, adaptive=kw.get("adaptive", False),
                        tol=kw.get("tolerance", 1e-10), gas_keys=gas_keys)
        k = int(r["steps"]["tried"][-1]) if kw.get("adaptive") else n
        inter += ipe_of(s.playing) * ns * k
        tried += k
        sim_t += float(r["steps"]["t"][-1]) - 0.0
        secs += r["seconds"]
        tpb.append(r["tpb"])
    return {"value": inter / secs, "unit": "interactions/s", "sim_years_per_s": sim_t / K_GAUSS / YEAR / secs,
            "ms_per_try": 1e3 * secs / max(1, tried), "tries": tried, "systems": len(states),
            "threads_per_block": sorted(set(tpb)),
            "kind": "red's own GPU path: calc_grav_accel_naive + rk8/rk4 stage kernels + thrust error max + host "
                    "controller, unmodified sources built here for sm_103a (-fmad=false); started from the same "
                    "settled state"}


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


def settle(sim, tries):
    """Untimed tries in batches of 100, handling collision events between batches."""
    done = 0
    while done < tries:
        k = min(100, tries - done)
        sim.launch_tries(k)
        drain_events(sim)
        done += k


def measure(torch, sim, stream, args, flush, steps, tps, stats=None):
    """Timed steps plus the work the tries did: (ms, interactions, sim-time, tries, failed)."""
    a = snapshot(sim)
    ms = timed_steps(torch, sim, stream, steps, flush, tps)
    drain_events(sim)
    b = snapshot(sim)
    tried = b["tried"] - a["tried"]
    if stats is not None:
        stats["collisions"] = int(np.sum(b["collisions"] - a["collisions"]))
    return ms, float(np.sum(b["ipe"] * tried)), float(np.sum(b["t"] - a["t"])), int(tried.sum()), \
        int(np.sum(b["failed"] - a["failed"]))


def plain_comparison(rg, systems, kw, args, local_rank, stream, flush, ns):
    """The same ensemble with the classical controller, timed the same way."""
    import torch
    sim = rg.Sim(systems, precision=args.precision, device=local_rank, stream=stream.cuda_stream, **kw)
    tps = tries_per_step(args)
    settle(sim, max(3, args.warmup) * tps + SETTLE_TRIES[args.config])
    ms, inter, sim_dt, tried, failed = measure(torch, sim, stream, args, flush, args.steps, tps)
    sim.close()
    return {"rejected_fraction": failed / tried if tried else None,
            "sim_years_per_s": sim_dt / K_GAUSS / YEAR / (ms * 1e-3), "ms_per_step": ms / args.steps,
            "value": inter * ns / (ms * 1e-3)}


def run_reference(args, rg, rank, world):
    systems, kw, desc = workload(rg, args.config)
    kw, desc = with_tolerance(args, kw, desc)
    if rank != 0:
        return
    import oracle
    oracle.build()
    sample_s = float(os.environ.get("REDGB_REF_SECONDS", "10")) * max(1, args.steps) / 20.0
    res = cpu_baseline_sample(systems, kw, seconds=sample_s, warmup=max(0, args.warmup))
    line = {"metric": METRIC, "value": res["value"], "unit": "interactions/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_object(args, systems, kw, desc, world),
            "sim_years_per_s": res["sim_years_per_s"],
            "cpu_baseline": {"value": res["value"], "unit": "interactions/s", "cores": res["cores"],
                             "kind": res["kind"], "sample": res["sample"]},
            "e2e": {"value": res["value"], "unit": "interactions/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def with_tolerance(args, kw, desc):
    """--tolerance overrides the workload's RKF7(8) tolerance (named in the description)."""
    if args.tolerance and kw.get("adaptive"):
        kw = dict(kw, tolerance=args.tolerance)
        desc = desc.replace("tol 1e-10", "tol %g" % args.tolerance)
    return kw, desc


def run_ours(args, rg, rank, world, local_rank):
    import torch
    torch.cuda.set_device(local_rank)
    t_ic = time.perf_counter()
    systems, kw, desc = workload(rg, args.config, rank, world)
    kw, desc = with_tolerance(args, kw, desc)
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
    ns = n_stage(kw)
    tps = tries_per_step(args)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")   # 256 MiB > L2
    proposer = None
    if args.config == "c5":
        proposer = train_proposer(rg, systems, kw, args, local_rank, stream)
        sim.set_step_proposer(proposer["bits"], proposer["norm"], safety=1.0, ratio_lo=0.25, ratio_hi=4.0)
    tuned = None
    if not args.no_autotune:
        t0 = time.perf_counter()
        tuned = sim.autotune()
        tuned["seconds"] = time.perf_counter() - t0
    # W warm-up steps (the graph is captured on the first launch), then the
    # rest of the settling run past the step size's start-up adaptation
    settle(sim, max(3, args.warmup) * tps)
    settle(sim, max(0, SETTLE_TRIES[args.config] - max(3, args.warmup) * tps))
    E0 = [sim.energy_interacting(k) for k in range(sim.n_systems)]
    launches0 = sim.kernel_launches
    clocks = ClockSampler(local_rank)
    clocks.start()
    rg.shard.barrier(local_rank)
    torch.cuda.synchronize()
    stats = {}
    coll0 = snapshot(sim)["collisions"]
    ms, inter, sim_dt, tried, failed = measure(torch, sim, stream, args, flush, args.steps, tps, stats)
    torch.cuda.synchronize()
    rg.shard.barrier(local_rank)
    clk = clocks.stop()
    launches = sim.kernel_launches - launches0
    # |dE/E| over the systems that had no merge in the timed region (a perfect
    # merge changes E by design)
    merged = snapshot(sim)["collisions"] - coll0
    dEs = [abs((sim.energy_interacting(k)[0] - E0[k][0]) / E0[k][0]) for k in range(sim.n_systems) if not merged[k]]
    dE = max(dEs) if dEs else None   # null when every system had a merge (perfect merging changes E)
    t_max = rg.shard.max_over_ranks(ms, device="cuda")
    inter_all = rg.shard.sum_over_ranks(inter * ns, device="cuda")
    value = inter_all / (t_max * 1e-3)
    sim_years_all = rg.shard.sum_over_ranks(sim_dt / K_GAUSS / YEAR, device="cuda")
    ms_per_try = ms / (args.steps * tps)
    try:
        traffic = json.load(open(os.path.join(ROOT, "profiles", "traffic.json"))).get(args.config, {})
    except (OSError, ValueError):
        traffic = {}
    roof = roofline_for(sim, systems, kw, peaks, traffic, ms_per_try)

    # end to end through the C ABI with host buffers: the state of every system
    # of the workload in and out of pinned host memory around each integrator step
    n_all = sim.bodies()
    st = types.SimpleNamespace()
    host = {}
    for f, dt in (("r", rg.types.VAR4), ("v", rg.types.VAR4), ("p", rg.types.PARAM), ("md", rg.types.BMD)):
        host[f] = torch.zeros(n_all * dt.itemsize, dtype=torch.uint8).pin_memory()
        setattr(st, f, host[f].numpy().view(dt))
    sim.get_states(st)
    e2e_steps = max(10, args.steps * tps // 8)
    a = snapshot(sim)
    torch.cuda.synchronize()
    rg.shard.barrier(local_rank)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        sim.set_states(st, parts="rv")      # inputs from pinned host memory
        sim.step()
        sim.get_states(st, parts="rv")      # results into the same pinned buffers
    e2e_s = rg.shard.max_over_ranks(time.perf_counter() - t0, device="cuda")
    drain_events(sim)
    b = snapshot(sim)
    e2e_value = rg.shard.sum_over_ranks(float(np.sum(b["ipe"] * (b["tried"] - a["tried"]))) * ns,
                                        device="cuda") / e2e_s
    bytes_state = n_all * (32 + 32)

    # the settled state, the start of the baselines below
    settled = []
    pick = range(sim.n_systems)
    if sim.n_systems > 1:
        pick = sorted(np.random.Generator(np.random.MT19937(5)).choice(
            sim.n_systems, min(RED_GPU_ENSEMBLE_SAMPLE, sim.n_systems), replace=False))
    for k in pick:
        settled.append((sim.get_state(int(k)), sim.info(int(k)).dt_next))

    # this library's FP64 mode on the same workload (fewer steps)
    fp64 = None
    if args.precision != "fp64" and not args.no_fp64:
        sim64 = rg.Sim(systems, precision="fp64", device=local_rank, stream=stream.cuda_stream, **kw)
        tps64 = max(1, tps // 4)
        settle(sim64, 3 * tps64 + SETTLE_TRIES[args.config])
        m64, i64, d64, _, _ = measure(torch, sim64, stream, args, flush, max(3, args.steps // 4), tps64)
        fp64 = {"value": i64 * ns / (m64 * 1e-3), "sim_years_per_s": d64 / K_GAUSS / YEAR / (m64 * 1e-3),
                "ms_per_try": m64 / (max(3, args.steps // 4) * tps64),
                "kind": "this library's FP64 mode (FP64 pairs with FMA, the same fused stages)"}
        sim64.close()

    red_gpu = None
    cpu = None
    if rank == 0 and not args.no_red_gpu:
        try:
            red_gpu = red_gpu_baseline(rg, args, kw, settled)
        except Exception as e:     # the baseline is reported, never required
            red_gpu = {"unavailable": "red's GPU path failed: %s" % str(e).splitlines()[0][:200]}
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline_sample(systems, kw, seconds=float(os.environ.get("REDGB_CPU_SECONDS", "10")),
                                  state=settled[0][0])
    if rank == 0:
        denom = red_gpu if red_gpu and "value" in red_gpu else None
        line = {"metric": METRIC, "value": value, "unit": "interactions/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_max / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32 pairs + f64 state" if args.precision in ("mixed", "fp32") else "f64",
                "data": "synthetic",
                "config": config_object(args, systems, kw, desc, world),
                "sim_years_per_s": sim_years_all / (t_max * 1e-3),
                "dE_over_E": dE,
                "dE_over_E_note": "largest over the systems without a merge in the timed region (null if every "
                                  "system merged), E over the interacting pairs; the FP64 runs drift the same at "
                                  "this tolerance (--accuracy-years)",
                "collisions_in_timed_region": stats.get("collisions"),
                "systems_with_merges": int(np.count_nonzero(merged)),
                "tries_in_timed_region": int(tried),
                "ms_per_try": ms_per_try,
                "accept_fraction": (1.0 - failed / tried) if tried else None,
                "e2e": {"value": e2e_value, "unit": "interactions/s", "h2d_bytes_per_step": bytes_state,
                        "d2h_bytes_per_step": bytes_state, "steps": e2e_steps,
                        "api": "red_set_states(r, v) + red_step + red_get_states(r, v), every system"},
                "roofline": roof,
                "cpu_baseline": cpu,
                "plain_fp64_same_gpu": denom or fp64,
                "vs_plain_fp64": (value / denom["value"]) if denom else ((value / fp64["value"]) if fp64 else None),
                "sim_years_vs_plain_fp64": ((sim_years_all / (t_max * 1e-3)) / denom["sim_years_per_s"])
                if denom else None,
                "library_fp64": fp64,
                "vs_library_fp64": (value / fp64["value"]) if fp64 else None,
                "autotune": tuned,
                "clocks": clk,
                "gpu_launches": int(launches)}
        if ic_gpu is not None:
            line["initial_conditions"] = ic_gpu
        if proposer is not None:
            plain = plain_comparison(rg, systems, kw, args, local_rank, stream, flush, ns)
            line["proposer"] = {
                "records": proposer["records"], "train_s": proposer["train_s"],
                "val_loss": proposer["val_loss"],
                "rejected_fraction": (failed / tried) if tried else None,
                "rejected_fraction_plain": plain["rejected_fraction"],
                "sim_years_per_s": sim_years_all / (t_max * 1e-3),
                "sim_years_per_s_plain": plain["sim_years_per_s"],
                "ms_per_step_plain": plain["ms_per_step"],
                "overhead_ms_per_step": t_max / args.steps - plain["ms_per_step"],
                "kernels_ms_per_try": roof["ms_per_try_by_kind"].get("proposer")}
        print(json.dumps(line), flush=True)
    sim.close()


def run_accuracy(args, rg, local_rank=0):
    """The accuracy statement: the 16384-body disk over T years (1000 orbits at
    1 AU for T = 1000) in MIXED precision against this library's FP64 mode,
    the same start and the same tolerance.  Collisions are off in both runs so
    that they integrate the same bodies (a merge changes E by design).  Each
    run stops past T and one fixed RKF7(8) step of the remaining (tiny) time
    brings it to T exactly, so positions compare at the same instant.
    Reported: |dE/E| (E over the interacting pairs), the relative drift of the
    angular momentum, and the relative position error of every body against
    the FP64 run (median, 90th percentile, largest; the protoplanets apart).
    The disk is chaotic (close encounters), so a third run -- MIXED again,
    from a start that differs by one ulp in one planetesimal's x -- measures
    the divergence that any difference of rounding grows into over T: the
    floor under which no precision can bring the position error."""
    import torch
    torch.cuda.set_device(local_rank)
    systems, kw, desc = workload(rg, "c2")
    kw = dict(kw, collision_factor=0.0, tolerance=args.tolerance or kw["tolerance"])
    T = args.accuracy_years * YEAR * K_GAUSS

    def one(prec, s0):
        sim = rg.Sim(s0, precision=prec, length=T, device=local_rank, **kw)
        E0 = sim.energy_interacting(0)
        t0 = time.perf_counter()
        while True:
            sim.launch_tries(2000)
            act, halted = sim.synchronize()
            if halted:
                sim.handle_events()
            if not act:
                break
        wall = time.perf_counter() - t0
        info = sim.info(0)
        st = sim.get_state(0)
        tried, failed = info.n_tried, info.n_failed
        sim.close()
        # one fixed step from just past T back to T
        fix = dict(kw, adaptive=False, dt=T - info.t)
        fix.pop("tolerance", None)
        with rg.Sim(st, precision=prec, device=local_rank, t0=info.t, **fix) as s2:
            s2.step()
            E1 = s2.energy_interacting(0)
            fin = s2.get_state(0)
            t_end = s2.info(0).t
        return {"wall_s": wall, "tries": int(tried), "failed": int(failed), "t_end": t_end,
                "dE_over_E": abs((E1[0] - E0[0]) / E0[0]),
                "dC_over_C": float(np.linalg.norm(E1[1:] - E0[1:]) / np.linalg.norm(E0[1:])),
                "sim_years_per_s": args.accuracy_years / wall,
                "r": np.stack([fin.r["x"], fin.r["y"], fin.r["z"]], axis=1)}

    s = systems[0]
    res = {"mixed": one("mixed", s), "fp64": one("fp64", s)}
    if not args.no_chaos:
        sp = s.copy()
        k = s.n_SI + 100
        sp.r["x"][k] = np.nextafter(sp.r["x"][k], np.inf)
        res["mixed_1ulp"] = one("mixed", sp)
    n_si = s.n_SI

    def err(a, b):
        rel = np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1)
        return {"median": float(np.median(rel[1:])), "p90": float(np.percentile(rel[1:], 90)),
                "max": float(rel[1:].max()), "protoplanets_max": float(rel[1:n_si].max()),
                "star_abs": float(np.linalg.norm(a[0] - b[0]))}
    out = {"accuracy": {
        "workload": desc.replace(", collisions on", "") + ", collisions off", "years": args.accuracy_years,
        "tolerance": kw["tolerance"],
        "reference": "this library's FP64 mode (FP64 pairs with FMA), same start, same tolerance",
        "runs": {k: {q: v for q, v in r.items() if q != "r"} for k, r in res.items()},
        "position_error_mixed_vs_fp64": err(res["mixed"]["r"], res["fp64"]["r"]),
        "chaos_floor_mixed_1ulp_vs_mixed": err(res["mixed_1ulp"]["r"], res["mixed"]["r"])
        if "mixed_1ulp" in res else None}}
    print(json.dumps(out), flush=True)


def run_proposer_eval(args, rg, local_rank=0):
    """The learned step proposer at the scale of its specification: the 512-disk
    ensemble integrated plainly for `proposer_train_years` (~2e6 logged
    records), the network trained on the GPU on two targets (the step accepted
    next; the largest step that would have met the tolerance), then three runs
    of `proposer_years` from the same start: the classical controller, and the
    controller with either network's proposals.  Reported per run: tries,
    rejected fraction, simulated years per second (wall clock of the whole
    run, events handled), |dE/E| (largest over the disks without a merge) and
    the proposer kernels' share of a try."""
    import torch
    torch.cuda.set_device(local_rank)
    systems, kw, desc = workload(rg, "c4")
    stream = torch.cuda.Stream()
    YR = YEAR * K_GAUSS

    def integrate(sim):
        while True:
            sim.launch_tries(500)
            act, halted = sim.synchronize()
            if halted:
                sim.handle_events()
            if not act:
                break

    t0 = time.perf_counter()
    sim = rg.Sim(systems, length=args.proposer_train_years * YR, device=local_rank, stream=stream.cuda_stream, **kw)
    sim.log_features(1 << 23)
    integrate(sim)
    recs = sim.feature_log(cap=1 << 23)
    sim.close()
    log_s = time.perf_counter() - t0
    nets = {}
    for target in ("accepted", "largest"):
        t0 = time.perf_counter()
        bits, nm, hist = rg.proposer.train(recs, epochs=args.proposer_epochs, batch=8192, lr=2e-3, target=target)
        nets[target] = (bits, nm, {"train_s": time.perf_counter() - t0, "val_loss": hist[-1][2]})

    def arm(name, net=None, safety=1.0):
        sim = rg.Sim(systems, length=args.proposer_years * YR, device=local_rank, stream=stream.cuda_stream, **kw)
        if net is not None:
            sim.set_step_proposer(net[0], net[1], safety=safety, ratio_lo=0.25, ratio_hi=4.0)
        E0 = [sim.energy_interacting(k)[0] for k in range(sim.n_systems)]
        c0 = snapshot(sim)["collisions"]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        integrate(sim)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        snap = snapshot(sim)
        merged = snap["collisions"] - c0
        dE = max([abs((sim.energy_interacting(k)[0] - E0[k]) / E0[k]) for k in range(sim.n_systems)
                  if not merged[k]] or [0.0])
        share = None
        if net is not None:
            tot = {}
            for _ in range(3):
                ms, kind = sim.profile_try()
                for m, k in zip(ms, kind):
                    tot[int(k)] = tot.get(int(k), 0.0) + float(m)
            share = tot.get(5, 0.0) / sum(tot.values()) if tot else None
        tried, failed = int(snap["tried"].sum()), int(snap["failed"].sum())
        sim.close()
        return name, {"tries": tried, "rejected_fraction": failed / tried, "wall_s": wall,
                      "sim_years_per_s": float(np.sum(snap["t"])) / YR / wall, "dE_over_E": dE,
                      "proposer_share_of_try": share, "safety": safety if net is not None else None}

    runs = dict([arm("classical"), arm("learned_accepted", nets["accepted"], 1.0),
                 arm("learned_largest", nets["largest"], 0.9)])
    base = runs["classical"]["sim_years_per_s"]
    for r in runs.values():
        r["sim_years_per_s_vs_classical"] = r["sim_years_per_s"] / base
    print(json.dumps({"proposer_eval": {
        "workload": desc, "train_years": args.proposer_train_years, "eval_years": args.proposer_years,
        "records": int(len(recs)), "log_run_s": log_s,
        "training": {k: v[2] for k, v in nets.items()}, "runs": runs}}), flush=True)


def run_plan_only(args, rg, rank, world):
    """Each rank builds its slice of the workload and reports it (no GPU work);
    rank 0 prints the gathered slices.  Checks the launcher and the split."""
    systems, kw, desc = workload(rg, args.config, rank, world)
    mine = {"rank": rank, "world": world, "systems": len(systems), "bodies": int(sum(s.n for s in systems)),
            "first_x": [float(s.r["x"][1]) for s in systems[:3]]}
    if world > 1:
        import torch.distributed as dist
        got = [None] * world
        dist.all_gather_object(got, mine)
    else:
        got = [mine]
    if rank == 0:
        print(json.dumps({"plan_only": True, "config": args.config, "ranks": got}), flush=True)


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def launch_ranks(n):
    """bench.py --gpus N started without a launcher: run this file again under
    torch.distributed.run with N local ranks (one per GPU)."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=%d" % n,
           "--master-addr=127.0.0.1", "--master-port=%d" % free_port(), os.path.abspath(__file__)] + sys.argv[1:]
    return subprocess.call(cmd)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c2", choices=["c1", "c2", "c3", "c4", "c5", "dense", "cube", "cube65536"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64", "fp32", "fp64_exact"])
    ap.add_argument("--tries-per-step", type=int, default=0)
    ap.add_argument("--accuracy-years", type=float, default=0.0)
    ap.add_argument("--tolerance", type=float, default=0.0)
    ap.add_argument("--no-chaos", action="store_true")
    ap.add_argument("--plan-only", action="store_true")
    ap.add_argument("--proposer-eval", action="store_true")
    ap.add_argument("--proposer-years", type=float, default=100.0)
    ap.add_argument("--proposer-train-years", type=float, default=20.0)
    ap.add_argument("--proposer-epochs", type=int, default=10)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-red-gpu", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    args = ap.parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(launch_ranks(args.gpus))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    rg = __graft_entry__.load_package()
    if args.plan_only:
        if world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
        run_plan_only(args, rg, rank, world)
        if world > 1:
            dist.destroy_process_group()
        return
    if args.impl == "reference":
        run_reference(args, rg, rank, world)
        return
    rg.build()
    if args.accuracy_years > 0:
        if rank == 0:
            run_accuracy(args, rg, local_rank)
        return
    if args.proposer_eval:
        if rank == 0:
            run_proposer_eval(args, rg, local_rank)
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    run_ours(args, rg, rank, world, local_rank)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
