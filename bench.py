"""Benchmark of the NeuCor simulation step on GB300.

Workload (the plain single-network GPU configuration): 100,000 neurons uniform in a
cube at the reference's spawn density, each connected to its 100 nearest neighbours
(10M synapses), U[0,1) fp32 weights, int16 delays from distance; 200 input neurons in 10
correlated Poisson groups at 5-40 Hz (+-2-step jitter); STDP on; background firing on.
One bench step = 1,000 simulation steps (1 s of simulated time at 1 ms per step);
the default 20 timed steps are the configuration's 20,000-step horizon.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N > 1 runs N independent replicas (one per GPU, launched by torch.distributed.run);
the networks do not interact, so there is no collective on the data path.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_NEURONS = 100_000
FANOUT = 100
SIM_STEPS_PER_STEP = 1000
N_GROUPS, GROUP_SIZE = 10, 20
METRIC = "synaptic events/s"
UNIT = "events/s"
STEP_MODES = {"dense": 0, "event": 1, "auto": 2}
FORM_NAMES = {0: "dense", 1: "event"}
REF_PREWARM_STEPS = 40


def workload_groups():
    rates = np.linspace(5.0, 40.0, N_GROUPS)
    return [dict(first=GROUP_SIZE * g, count=GROUP_SIZE, rate_hz=float(rates[g]), correlated=1, jitter=2)
            for g in range(N_GROUPS)]


def workload_config(extra=None):
    cfg = {"workload": "plain single network: 100k neurons x 100 nearest targets (10M synapses), "
                       "200 inputs in 10 correlated Poisson groups 5-40 Hz, STDP on, 20,000 steps",
           "neurons": N_NEURONS, "synapses": N_NEURONS * FANOUT, "sim_steps_per_bench_step": SIM_STEPS_PER_STEP,
           "dt_ms": 1.0, "l2": "inputs larger than L2 (synapse tables ~350 MB)", "parallelism": "replicas"}
    if extra:
        cfg.update(extra)
    return cfg


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during a region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.lines = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.device)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        return False

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def ncu_traffic(kernel):
    """DRAM bytes per launch of `kernel` from its committed ncu summary (profiles/)."""
    for name in (f"{kernel}_c2.txt", f"{kernel}_event_c2.txt"):
        try:
            for line in open(os.path.join(ROOT, "profiles", name)):
                if line.startswith("dram_bytes_per_launch_scaled:"):
                    return float(line.split(":")[1])
        except OSError:
            continue
    return None


def build_network(G, seed):
    xyz, pre, post, w = G.build_knn(N_NEURONS, FANOUT, 8.0, seed=seed)
    return xyz, pre, post, w


class CpuPort:
    """The oracle port (the reference's step restated on CPU, single-threaded like the
    reference) on the same workload; `replicas` independent networks run on as many
    host threads (the C code runs outside the GIL)."""

    def __init__(self, net_arrays, groups, seed, replicas=1):
        from oracle import oracle as O
        xyz, pre, post, w = net_arrays
        self.sims = [None] * replicas

        def make(r):
            self.sims[r] = O.OracleS(xyz, pre, post, w, params=O.default_params(seed=seed + r), groups=groups)

        self._parallel(make)

    def _parallel(self, fn):
        ths = [threading.Thread(target=fn, args=(r,)) for r in range(len(self.sims))]
        for th in ths:
            th.start()
        for th in ths:
            th.join()

    def timed(self, sim_steps):
        """Runs sim_steps on every replica at once; returns (events, wall seconds)."""
        before = [s.stats()["launched"] for s in self.sims]
        t0 = time.perf_counter()
        self._parallel(lambda r: self.sims[r].run(sim_steps))
        wall = time.perf_counter() - t0
        return sum(s.stats()["launched"] - b for s, b in zip(self.sims, before)), wall

    def fires(self):
        return sum(s.stats()["fires"] for s in self.sims)

    def budgeted(self, budget_s, chunk=10, cap=5000):
        events, wall, steps = 0, 0.0, 0
        while wall < budget_s and steps < cap:
            e, dt = self.timed(chunk)
            events, wall, steps = events + e, wall + dt, steps + chunk
        return events, wall, steps


def host_threads():
    n = os.cpu_count() or 1
    try:
        with open("/proc/meminfo") as fh:
            avail_kb = next(int(l.split()[1]) for l in fh if l.startswith("MemAvailable"))
        n = max(1, min(n, int(avail_kb / (1.2 * 1024 * 1024))))  # ~1 GB per 10M-synapse replica
    except (OSError, StopIteration, ValueError):
        pass
    return n


def run_reference_arm(args):
    """The reference's step on the host cores: the oracle port (the reference's CPU
    algorithm restated in C and pinned to the reference's own code), one independent
    replica of the workload per host thread.  The network comes from the oracle's own
    kNN restatement: nothing of the GPU library is loaded on this arm."""
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import oracle as O
    groups = workload_groups()
    arrays = O.build_knn(N_NEURONS, FANOUT, 8.0, seed=1)
    threads = host_threads()
    port = CpuPort(arrays, groups, seed=100, replicas=threads)
    # the workload saturates within its first ~30 steps (one fire per refractory period,
    # 333 Hz); the GPU arm is timed at saturation, so this arm is too
    port.timed(REF_PREWARM_STEPS)
    chunk = 10  # one reference-arm step: 10 simulation steps on every replica
    for _ in range(args.warmup):
        port.timed(chunk)
    events, wall, fires0 = 0, 0.0, port.fires()
    for _ in range(args.steps):
        e, dt = port.timed(chunk)
        events, wall = events + e, wall + dt
    fires = port.fires() - fires0
    value = events / wall
    first = REF_PREWARM_STEPS + args.warmup * chunk
    rate = fires / (threads * N_NEURONS * chunk * args.steps / 1000.0)
    sample = (f"{threads} replica(s) of the 100k x 100 network on {threads} host thread(s); each step = "
              f"{chunk} simulation steps per replica; timed steps {first + 1}-{first + chunk * args.steps} "
              f"of the horizon, at saturation (mean rate {rate:.1f} Hz, as in the GPU arm)")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(),
            "stats": {"mean_rate_hz": rate, "neuron_steps_per_s": threads * N_NEURONS * chunk * args.steps / wall},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------ batched / served
def c3_nets(G, n_nets, horizon, seed=3):
    """Batched workload: sizes log-uniform over 1k-64k neurons, fan-out uniform over
    20-200 nearest neighbours, per-network seed, input rate 5-50 Hz and 1-8 correlated
    groups of 10 input neurons."""
    rng = np.random.default_rng(seed)
    nets = []
    for q in range(n_nets):
        n = int(np.exp(rng.uniform(np.log(1000), np.log(64000))))
        k = min(int(rng.integers(20, 201)), n - 1)
        rate = float(rng.uniform(5.0, 50.0))
        ng = int(rng.integers(1, 9))
        nseed = seed * 100003 + q
        xyz, pre, post, w = G.build_knn(n, k, 8.0, seed=nseed)
        groups = [dict(first=10 * g, count=10, rate_hz=rate, correlated=1, jitter=2) for g in range(ng)]
        nets.append(dict(xyz=xyz, pre=pre, post=post, weight=w, seed=nseed, groups=groups, horizon=horizon))
    return nets


def c4_requests(n_req, horizon_scale, seed=4):
    """Served workload: Poisson arrivals at 50 requests/s; sizes log-uniform over
    500-200k neurons, fan-out 20-150, horizons log-uniform over 1k-100k steps (times
    horizon_scale), each with a random input pattern of 1-8 groups.  A request is the
    parameters of its kNN network (the server builds it)."""
    rng = np.random.default_rng(seed)
    t, reqs = 0.0, []
    for q in range(n_req):
        t += float(rng.exponential(1.0 / 50.0))
        n = int(np.exp(rng.uniform(np.log(500), np.log(200000))))
        k = min(int(rng.integers(20, 151)), n - 1)
        h = max(1, int(np.exp(rng.uniform(np.log(1000), np.log(100000))) * horizon_scale))
        ng = int(rng.integers(1, 9))
        groups = [dict(first=10 * g, count=10, rate_hz=float(rng.uniform(5.0, 50.0)), correlated=int(rng.integers(0, 2)),
                       jitter=int(rng.integers(0, 4))) for g in range(ng)]
        nseed = seed * 100003 + q
        reqs.append(dict(knn=(n, k, nseed), seed=nseed, groups=groups, horizon=h, arrival=t))
    return reqs


def one_at_a_time(G, nets, mode, arrivals=None, device_build=False):
    """The plain drop-in, one network after another: create, run the horizon, read the
    counters, destroy.  Returns (events, busy seconds, run-only seconds, per-request
    latency or None); run-only leaves out building and uploading each network."""
    events, busy, run_s, clock, lat = 0, 0.0, 0.0, 0.0, []
    for q, d in enumerate(nets):
        t0 = time.perf_counter()
        if "knn" in d and device_build:  # the drop-in's device kNN builder (dense form)
            n, k, kseed = d["knn"]
            net = G.NeuCor.knn(n, k, 8.0, seed=kseed, params=G.default_params(seed=d["seed"], step_mode=mode))
        elif "knn" in d:  # built on the host, as the server's builder threads do
            n, k, kseed = d["knn"]
            xyz, pre, post, w = G.build_knn(n, k, 8.0, seed=kseed)
            net = G.NeuCor.from_arrays(xyz, pre, post, w, params=G.default_params(seed=d["seed"], step_mode=mode))
        else:
            net = G.NeuCor.from_arrays(d["xyz"], d["pre"], d["post"], d["weight"],
                                       params=G.default_params(seed=d["seed"], step_mode=mode))
        net.set_input_groups(d["groups"])
        net.sync()
        t1 = time.perf_counter()
        net.run(d["horizon"])
        st = net.stats()
        t2 = time.perf_counter()
        net.close()
        dt = time.perf_counter() - t0
        events += st["launched"]
        busy += dt
        run_s += t2 - t1
        if arrivals is not None:
            start = max(arrivals[q], clock)
            clock = start + dt
            lat.append(clock - arrivals[q])
    return events, busy, run_s, lat


def measure_batched(G, n_nets, horizon, mode, one_at_a_time_sample=None):
    t_gen = time.perf_counter()
    nets = c3_nets(G, n_nets, horizon)
    t_build = time.perf_counter()
    b = G.Batch([dict(xyz=d["xyz"], pre=d["pre"], post=d["post"], weight=d["weight"],
                      params=G.default_params(seed=d["seed"], step_mode=mode), groups=d["groups"],
                      horizon=d["horizon"]) for d in nets])
    t_tune = time.perf_counter()
    cfg = b.autotune(steps_per_trial=8)
    t_run = time.perf_counter()
    done = b.step(0)
    before = sum(b.stats(q)["launched"] for q in range(n_nets))
    ms = b.time(horizon - done)
    events = sum(b.stats(q)["launched"] for q in range(n_nets)) - before
    neurons = sum(int(d["xyz"].shape[0]) for d in nets)
    synapses = sum(int(d["pre"].shape[0]) for d in nets)
    b.close()
    t_one = time.perf_counter()
    sub = nets if not one_at_a_time_sample else nets[:one_at_a_time_sample]
    ev1, busy1, run1, _ = one_at_a_time(G, sub, mode)
    t_end = time.perf_counter()
    rate = events * 1000.0 / ms
    return {"workload": f"{n_nets} networks, sizes log-uniform 1k-64k neurons, fan-out 20-200 nearest, "
                        f"input rate 5-50 Hz, 1-8 correlated groups, {horizon} steps each",
            "networks": n_nets, "neurons": neurons, "synapses": synapses, "steps": horizon,
            "timed_steps": horizon - done, "launch_config": cfg, "events_per_s": rate,
            "wall_s": {"generate": t_build - t_gen, "create": t_tune - t_build, "autotune": t_run - t_tune,
                       "run": t_one - t_run, "one_at_a_time": t_end - t_one},
            "one_at_a_time_sample": f"{'all' if len(sub) == len(nets) else 'the first ' + str(len(sub))} of the "
                                    "networks, each created, run for its horizon and read back alone",
            "one_at_a_time_events_per_s": ev1 / run1,
            "one_at_a_time_events_per_s_with_build": ev1 / busy1,
            "speedup_vs_one_at_a_time": rate / (ev1 / run1)}


def measure_served(G, n_req, horizon_scale, budget, mode):
    reqs = c4_requests(n_req, horizon_scale)
    srv = G.Server(budget, max_networks=256, steps_per_batch=64, build_threads=min(16, os.cpu_count() or 1),
                   step_mode=mode)
    t0 = time.perf_counter()
    for r in reqs:
        wait = t0 + r["arrival"] - time.perf_counter()
        if wait > 0:
            time.sleep(wait)
        n, k, kseed = r["knn"]
        srv.submit_knn(n, k, 8.0, kseed, r["horizon"], params=G.default_params(seed=r["seed"], step_mode=mode),
                       groups=r["groups"])
    srv.drain()
    done = srv.poll()
    sst = srv.stats()
    srv.close()
    ok = [d for d in done if d["status"] == 0]
    lat = np.array([d["done_s"] - d["submit_s"] for d in ok])
    span = max(d["done_s"] for d in ok) - min(d["submit_s"] for d in ok)
    events = sum(d["launched"] for d in ok)
    t_one = time.perf_counter()
    arr = [r["arrival"] for r in reqs]
    ev1, busy1, _, lat1 = one_at_a_time(G, reqs, mode, arrivals=arr)
    span1 = max(a + l for a, l in zip(arr, lat1)) - reqs[0]["arrival"]
    t_dev = time.perf_counter()
    ev2, _, _, lat2 = one_at_a_time(G, reqs, mode, arrivals=arr, device_build=True)
    span2 = max(a + l for a, l in zip(arr, lat2)) - reqs[0]["arrival"]
    t_end = time.perf_counter()
    return {"workload": f"{n_req} requests, Poisson arrivals at 50/s, 500-200k neurons, fan-out 20-150, "
                        f"horizons log-uniform 1k-100k steps x {horizon_scale}, 1-8 input groups each; "
                        "served: each sent as kNN parameters and built on the host by the server's builder "
                        "threads; one at a time: each built on the host (as the server does), run and read "
                        "back; and again with the drop-in's device kNN builder",
            "wall_s": {"served": t_one - t0, "one_at_a_time": t_dev - t_one, "one_at_a_time_device_build": t_end - t_dev},
            "requests": n_req, "finished": len(ok), "horizon_scale": horizon_scale, "arrival_rate_per_s": 50,
            "budget_gb": budget / 1e9, "events_per_s": events / span, "p50_latency_s": float(np.percentile(lat, 50)),
            "p99_latency_s": float(np.percentile(lat, 99)), "peak_resident_networks": sst["peak_resident_networks"],
            "peak_resident_gb": sst["peak_resident_bytes"] / 1e9,
            "one_at_a_time_events_per_s": ev1 / span1,
            "one_at_a_time_p50_latency_s": float(np.percentile(lat1, 50)),
            "one_at_a_time_p99_latency_s": float(np.percentile(lat1, 99)),
            "speedup_vs_one_at_a_time": (events / span) / (ev1 / span1),
            "one_at_a_time_device_build_events_per_s": ev2 / span2,
            "one_at_a_time_device_build_p50_latency_s": float(np.percentile(lat2, 50)),
            "one_at_a_time_device_build_p99_latency_s": float(np.percentile(lat2, 99)),
            "speedup_vs_one_at_a_time_device_build": (events / span) / (ev2 / span2)}


def measure_large(G, mode, sim_steps=100, timed=5):
    """The large single network: 2,000,000 neurons x 200 nearest targets (400M synapses),
    2,000 inputs in 20 correlated groups at 10-40 Hz, STDP on, built on the device
    (nc_create_knn), timed over a prefix of the 100,000-step horizon."""
    n, k = 2_000_000, 200
    rates = np.linspace(10.0, 40.0, 20)
    groups = [dict(first=100 * g, count=100, rate_hz=float(rates[g]), correlated=1, jitter=2) for g in range(20)]
    t0 = time.perf_counter()
    net = G.NeuCor.knn(n, k, 8.0, seed=5, params=G.default_params(seed=5, step_mode=mode))
    net.sync()
    build_s = time.perf_counter() - t0
    net.set_input_groups(groups)
    net.run(3 * sim_steps)
    st0 = net.stats()
    ms, _ = net.time_steps(timed * sim_steps)
    st1 = net.stats()
    _, per = net.time_steps(20, per_kernel=True)
    events = st1["launched"] - st0["launched"]
    secs = ms / 1e3
    st = timed * sim_steps
    out = {"workload": "2M neurons x 200 nearest targets (400M synapses), 2,000 inputs in 20 correlated "
                       "groups 10-40 Hz, STDP on", "steps_timed": st, "warmup_steps": 3 * sim_steps,
           "device_build_s": build_s, "events_per_s": events / secs, "neuron_steps_per_s": n * st / secs,
           "ms_per_sim_step": ms / st, "mean_rate_hz": (st1["fires"] - st0["fires"]) / (n * st / 1000.0),
           "kernel_ms": per}
    net.close()
    return out


def measure_sparse(G, arrays, groups, seed, warm=2000, timed=2000):
    """The same network with its weights scaled by 0.05: activity stays near the input
    and background rates (a few Hz), the regime where the event form is the fast one.
    Timed in each form and in the automatic choice."""
    xyz, pre, post, w = arrays
    ws = (w * np.float32(0.05)).astype(np.float32)
    out = {"workload": "100k x 100 network as the headline, weights x 0.05 (quiet), "
                       f"{timed} steps after {warm}"}
    for label in ("auto", "dense", "event"):
        net = G.NeuCor.from_arrays(xyz, pre, post, ws, params=G.default_params(seed=seed, step_mode=STEP_MODES[label]))
        net.set_input_groups(groups)
        net.run(warm)
        st0 = net.stats()
        ms, _ = net.time_steps(timed)
        st1 = net.stats()
        out[label] = {"form": FORM_NAMES[net.step_form], "us_per_sim_step": ms * 1e3 / timed,
                      "events_per_s": (st1["launched"] - st0["launched"]) / (ms / 1e3),
                      "mean_rate_hz": (st1["fires"] - st0["fires"]) / (N_NEURONS * timed / 1000.0)}
        net.close()
    return out


def aggregate_over_ranks(pg, secs, e2e_secs, events, e2e_events):
    """The whole job's timing and work: the slowest rank's seconds (timed region and end
    to end) and the events of all ranks.  pg: torch.distributed, or None for one rank."""
    if not pg:
        return secs, e2e_secs, events, e2e_events
    import torch
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    t = torch.tensor([secs, e2e_secs], dtype=torch.float64, device=dev)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    c = torch.tensor([events, e2e_events], dtype=torch.float64, device=dev)
    pg.all_reduce(c)
    return float(t[0]), float(t[1]), float(c[0]), float(c[1])


def run_ours(args):
    world, rank, local = dist_env()
    pg = None
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
        pg = dist
    import neurocorrelation_gb300 as G

    G.load_library()
    if G.device_count() < 1:
        raise RuntimeError("no CUDA device")
    G.set_device(local)
    groups = workload_groups()
    seed = 1 + rank
    arrays = build_network(G, seed=seed)
    mode = STEP_MODES[args.step_mode]
    net = G.NeuCor.from_arrays(*arrays, params=G.default_params(seed=seed, step_mode=mode))
    net.set_input_groups(groups)
    S = SIM_STEPS_PER_STEP

    def barrier():
        if pg:
            import torch
            t = torch.zeros(1, device="cuda" if torch.cuda.is_available() else "cpu")
            pg.all_reduce(t)

    net.run(args.warmup * S)
    net.sync()
    st0 = net.stats()
    barrier()
    with ClockSampler(local) as clk:
        ms, _ = net.time_steps(args.steps * S)
    barrier()
    st1 = net.stats()
    events = st1["launched"] - st0["launched"]
    fires = st1["fires"] - st0["fires"]
    # per-kernel timing pass (outside the timed region)
    kpass = 200
    stk0 = net.stats()
    _, per = net.time_steps(kpass, per_kernel=True)
    stk1 = net.stats()
    ev_per_step_k = (stk1["launched"] - stk0["launched"]) / (2 * kpass)
    # end to end through the public API with host buffers: the step's input definition
    # in, the step's spike raster and potentials/activities out
    e2e_steps = min(args.steps, 5)
    net.record_raster(S)
    h2d = 0
    d2h = 0
    st_e0 = net.stats()
    barrier()
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        net.set_input_groups(groups)
        net.record_raster(S)
        net.run(S)
        r = net.raster()
        pa = net.potAct
        h2d = 20 * len(groups)
        d2h = r.nbytes + pa.nbytes
    net.sync()
    e2e_wall = time.perf_counter() - t0
    barrier()
    st_e1 = net.stats()
    e2e_events = st_e1["launched"] - st_e0["launched"]

    # aggregate over ranks
    secs, e2e_secs, tot_events, tot_e2e = aggregate_over_ranks(pg, ms / 1e3, e2e_wall, events, e2e_events)
    if rank != 0:
        if pg:
            pg.destroy_process_group()
        return 0

    value = tot_events / secs
    neuron_steps = N_NEURONS * args.steps * S * world / secs
    peak, peak_kind = measured_peak()
    n_ms, l_ms = per
    form = FORM_NAMES[net.step_form]  # the form the timed steps ran in (auto: the one it chose)
    if form == "dense":
        # the synapse pass moves the 14 bytes per synaptic event (index 4, delay 2,
        # weight read + write 8), the neuron pass the 16 per neuron
        kernels = {"k_dense_synapses": n_ms, "k_dense_neurons": l_ms}
        dominant = "k_dense_synapses" if n_ms >= l_ms else "k_dense_neurons"
        alg = 14.0 * ev_per_step_k if dominant == "k_dense_synapses" else 16.0 * N_NEURONS
    else:
        kernels = {"k_neuron_step": n_ms, "k_spike_launch": l_ms}
        dominant = "k_neuron_step" if n_ms >= l_ms else "k_spike_launch"
        # algorithmic bytes (16 per neuron + 14 per synaptic event per step): the neuron
        # update moves 16 per neuron and 8 per event (weight read+write of plasticity),
        # the spike launch 6 per event (target index 4 + delay 2)
        alg = 16.0 * N_NEURONS + 8.0 * ev_per_step_k if dominant == "k_neuron_step" else 6.0 * ev_per_step_k
    dur = kernels[dominant] / 1e3
    achieved = alg / dur / 1e9
    traffic = ncu_traffic(dominant)
    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        port = CpuPort(arrays, groups, seed=seed, replicas=1)
        ev, wall, nst = port.budgeted(args.cpu_budget)
        cpu = {"value": ev / wall, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"first {nst} steps of the same 100k x 100 network on 1 thread ({wall:.1f} s)"}
    step_alg = (16.0 * N_NEURONS * args.steps * S + 14.0 * events) / secs / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": secs * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(),
        "stats": {"step_mode": args.step_mode, "form": form, "neuron_steps_per_s": neuron_steps,
                  "spikes_per_s": fires * world / secs,
                  "mean_rate_hz": fires / (N_NEURONS * args.steps * S / 1000.0),
                  "timed_steps": f"{args.warmup * S + 1}-{(args.warmup + args.steps) * S}",
                  "step_alg_gbs": step_alg},
        "gpu_launches": 2 * args.steps * S,  # two kernels per simulation step in either form
        "clocks": clk.summary(),
        "roofline": {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                     "kernel_ms": kernels,
                     "events_per_step_in_kernel_pass": ev_per_step_k,
                     # the DRAM bytes the kernel actually moves (ncu, per launch) over its
                     # CUDA-event time: how well it uses HBM, beside the algorithmic fraction
                     "traffic_gbs": traffic / dur / 1e9 if traffic else None,
                     "traffic_frac": traffic / dur / 1e9 / peak if traffic else None},
        "e2e": {"value": tot_e2e / e2e_secs, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "cpu_baseline": cpu,
    }
    if world == 1 and not args.no_sparse:
        line["sparse_variant"] = measure_sparse(G, arrays, groups, seed)
    # the batched and served forms run one form for all their networks, and the device
    # builder of the large network makes the dense form: the automatic choice resolves to
    # the dense form there (these workloads saturate)
    fixed = mode if mode != STEP_MODES["auto"] else STEP_MODES["dense"]
    if world == 1 and args.large:
        line["large_network"] = measure_large(G, fixed)
    if world == 1 and args.forms:
        line["forms"] = {"batched": measure_batched(G, args.batched_nets, args.batched_steps, fixed,
                                                    args.batched_one_at_a_time),
                         "served": measure_served(G, args.served_requests, args.served_horizon_scale,
                                                  args.served_budget_gb * 1e9, fixed)}
    print(json.dumps(line), flush=True)
    if pg:
        pg.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-large", dest="large", action="store_false",
                    help="skip the 2M x 200 network (built on the device, timed over a prefix)")
    ap.add_argument("--step-mode", default="auto", choices=sorted(STEP_MODES),
                    help="form of the step kernels (results are the same in all); auto switches by activity")
    ap.add_argument("--no-sparse", action="store_true",
                    help="skip the quiet variant of the workload (weights x 0.05)")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--no-forms", dest="forms", action="store_false",
                    help="skip the batched and served samples")
    ap.add_argument("--batched-nets", type=int, default=256)
    ap.add_argument("--batched-steps", type=int, default=1000)
    ap.add_argument("--batched-one-at-a-time", type=int, default=0,
                    help="networks of the batched mix timed one at a time (0 = all)")
    ap.add_argument("--served-requests", type=int, default=200)
    ap.add_argument("--served-horizon-scale", type=float, default=0.1)
    ap.add_argument("--served-budget-gb", type=float, default=120.0)
    ap.add_argument("--sim-steps-per-step", type=int, default=SIM_STEPS_PER_STEP,
                    help="simulation steps per bench step (smaller values make ncu-sized cases)")
    args = ap.parse_args()
    globals()["SIM_STEPS_PER_STEP"] = args.sim_steps_per_step
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        return run_reference_arm(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
