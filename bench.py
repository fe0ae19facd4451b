"""Benchmark of the sparse-lattice D3Q19 BGK step on one GB300.

Workload (default): 256^3 periodic sphere pack, seed 1, sphere radius
uniform in [4, 10], porosity 0.35, tau 0.8, body force 5e-7 along x,
FP64 distributions.  One bench step = one lattice time step over every fluid
node (one fused pull-stream + collide launch).  The distributions (2 x 19 x
8 B per node, about 1.8 GB) exceed L2, so no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line.  ``--impl reference`` times the CPU implementation of
the reference algorithm on the host cores (the oracle port, z-slab ranks as
threads) on the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "fluid MLUPS"
DATA = "synthetic sphere pack (seeded splitmix64 generator)"
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM = 6800.0

# algorithmic bytes per fluid-node update: 19 loads + 19 stores of the
# distribution + 18 int32 neighbour words
BYTES_PER_NODE = {"fp64_exact": 376, "fp64": 376, "fp64_fma": 376, "fp32": 224,
                  "fp16dev": 148, "bf16dev": 148}

# DRAM bytes (read + write) of one step-kernel launch come from one-pass ncu
# captures summarised in profiles/*.md, each with a line
#   traffic-record: workload=W form=F num_node=N order=O bytes=B source=D
# where O is the node order of the run and D is source_digest() of the
# step-kernel sources it was captured from.  A record is reported only
# while the kernel sources are unchanged.
PROFILES = os.path.join(ROOT, "profiles")
STEP_SOURCES = ("plb_step.cu", "plb_fx.h", "plb_emu.h", "plb_internal.h")


def source_digest():
    import hashlib
    h = hashlib.sha256()
    for name in STEP_SOURCES:
        with open(os.path.join(ROOT, "porelb_gb300", "csrc", name), "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()[:16]


def recorded_traffic(workload, form, num_node, order):
    """(bytes, profile file) of the matching capture, or (None, reason)."""
    digest = source_digest()
    stale = None
    try:
        names = sorted(os.listdir(PROFILES))
    except OSError:
        return None, "no profiles"
    for name in names:
        if not name.endswith(".md"):
            continue
        with open(os.path.join(PROFILES, name)) as fh:
            for line in fh:
                if not line.startswith("traffic-record:"):
                    continue
                kv = dict(t.split("=", 1) for t in line.split()[1:] if "=" in t)
                if (kv.get("workload"), kv.get("form"), kv.get("num_node"),
                        kv.get("order")) != (workload, form, str(num_node), order):
                    continue
                if kv.get("source") == digest:
                    return int(kv["bytes"]), "profiles/" + name
                stale = "profiles/" + name
    if stale:
        return None, f"{stale} was captured from other kernel sources"
    return None, "no capture of this workload and form"


WORKLOADS = {
    # plain FP64 at scale (the configuration the metric is quoted on)
    "c2_256": dict(dims=(256, 256, 256), seed=1, rmin=4.0, rmax=10.0,
                   porosity=0.35, tau=0.8, force=5e-7),
    # the plain FP64 workload at 128^3 (profiling size: state > L2, ~0.5 GB)
    "prof_128": dict(dims=(128, 128, 128), seed=1, rmin=4.0, rmax=10.0,
                     porosity=0.35, tau=0.8, force=5e-7),
    # the CPU-runnable plain case
    "c1_64": dict(dims=(64, 64, 64), seed=0, rmin=6.0, rmax=6.0,
                  porosity=0.40, tau=1.0, force=1e-6),
}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x, world, device="cuda"):
    """Largest value of x over the ranks (the step time the job takes)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def hbm_peak():
    try:
        with open(PEAKS) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.result = None
        if self.proc is None:
            return
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out = ""
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for line in out.strip().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) != 6:
                continue
            try:
                sm.append(float(parts[0]))
                mx = max(mx, float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[2:]):
                if v.lower() == "active":
                    reasons.add(n)
        if sm:
            self.result = {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx,
                           "reasons": sorted(reasons), "samples": len(sm)}


def make_geometry(w):
    import porelb_gb300 as P
    flag, ns, phi = P.sphere_pack(w["seed"], *w["dims"], w["rmin"], w["rmax"],
                                  w["porosity"])
    return flag, ns, phi


def workload_config(name, w, num_node, phi, precision):
    """The `config` object of both arms' JSON lines: the same keys and values
    for the same workload."""
    return {"workload": name, "dims": list(w["dims"]), "seed": w["seed"],
            "radius": [w["rmin"], w["rmax"]], "porosity_target": w["porosity"],
            "num_node": int(num_node), "porosity": phi, "tau": w["tau"],
            "force": w["force"], "precision": precision,
            "l2": "inputs larger than L2 (no flush)"}


def cpu_port_mlups(V, vs, dims, w, budget_s, threads):
    """The oracle port (push-form reference algorithm, z-slab ranks as
    threads) on a bounded number of steps of the workload."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py
    s = oracle_py.OracleSim(V, *dims, vs, w["tau"], w["force"])
    s.init()
    t0 = time.perf_counter()
    s.run(1, threads=threads)
    one = time.perf_counter() - t0
    steps = max(1, min(200, int(budget_s / max(one, 1e-6))))
    t0 = time.perf_counter()
    s.run(steps, threads=threads, it_begin=1)
    el = time.perf_counter() - t0
    s.close()
    return len(V) * steps / el / 1e6, steps, el


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def slab_count(nz, cores):
    p = max(1, cores)
    while p > 1 and nz % p:
        p -= 1
    return p


def run_reference(args, rank, world):
    """The reference algorithm on the host cores: the oracle port (push-form
    stream and collision in the reference's operation order, z-slab ranks as
    threads), on a table and geometry the oracle builds itself (its own
    sphere-pack generator and build_V restatement), so that nothing of the
    GPU library is loaded."""
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py
    w = WORKLOADS[args.workload]
    dims = w["dims"]
    flag, _, phi = oracle_py.sphere_pack(w["seed"], *dims, w["rmin"], w["rmax"],
                                         w["porosity"])
    cores = host_threads()
    p = slab_count(dims[2], cores)
    V, vs = oracle_py.build_v(flag, *dims, p)
    # one oracle solve for the whole run: W single warm-up steps, then K
    # bench steps of `per` lattice steps each, `per` sized so that the K
    # steps take about --ref-budget seconds in all
    s = oracle_py.OracleSim(V, *dims, vs, w["tau"], w["force"])
    s.init()
    it = 0
    t0 = time.perf_counter()
    s.run(1, threads=p, it_begin=it)
    it += 1
    one = time.perf_counter() - t0
    for _ in range(args.warmup):
        s.run(1, threads=p, it_begin=it)
        it += 1
    per = max(1, int(args.ref_budget / max(args.steps, 1) / max(one, 1e-6)))
    vals = []
    total = 0.0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        s.run(per, threads=p, it_begin=it)
        el = time.perf_counter() - t0
        it += per
        total += el
        vals.append(len(V) * per / el / 1e6)
    s.close()
    detail = (per, total)
    value = statistics.median(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3),
        "unit": "MLUPS", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": DATA,
        "config": workload_config(args.workload, w, len(V), phi, "fp64"),
        "parallelism": f"{p} z-slab ranks on host threads",
        "cpu_baseline": {"value": round(value, 3), "unit": "MLUPS",
                         "cores": p, "kind": "port",
                         "sample": f"{detail[0]} lattice step(s) of the full "
                                   f"workload per bench step, {args.steps} bench "
                                   f"steps ({detail[1]:.1f} s in all), {p} z-slab "
                                   f"ranks on {p} threads"},
        "e2e": {"value": round(value, 3), "unit": "MLUPS",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_gpu(args, rank, world, local):
    import torch
    import porelb_gb300 as P

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    w = WORKLOADS[args.workload]
    dims = w["dims"]
    flag, _, phi = make_geometry(w)
    V, vs = P.build_table(flag, *dims, 1)
    N = len(V)
    prec = args.precision

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    kv = args.kernel_variant
    sim = P.Simulation(V, *dims, vs, tau=w["tau"], force=w["force"],
                       precision=prec, device=local, kernel_variant=kv)
    sim.init_dist_macro()
    stream = torch.cuda.ExternalStream(sim.stream, device=local)
    it = 0
    sim.step(args.warmup, it_begin=it)
    it += args.warmup
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(stream)
        sim.step_async(args.steps, it_begin=it)
        e1.record(stream)
        sim.sync()
        barrier()
    it += args.steps
    ms = max_over_ranks(e0.elapsed_time(e1), world)
    ms_step = ms / args.steps
    value = N * args.steps * world / (ms * 1e-3) / 1e6
    kd, _ = sim.permeability()
    # untimed: continue the same solve to steady state (relative change of
    # <u_x> below 1e-7 over 1000 steps) for the FP64 permeability of the
    # workload, within a bounded wall time
    steady = None
    clk_steady = None
    if args.steady_wall > 0 and rank == 0:
        t0 = time.perf_counter()
        prev = kd
        # the same kernel runs for seconds here: its clocks are sampled too
        # (the timed region itself can be shorter than one sample)
        with ClockSampler(local) as cs:
            while time.perf_counter() - t0 < args.steady_wall:
                sim.step(1000, it_begin=it)
                it += 1000
                k, ki = sim.permeability()
                if prev and abs(k - prev) <= 1e-7 * abs(k):
                    steady = {"k_darcy": k, "k_intrinsic": ki, "steps": it,
                              "tol": 1e-7, "interval": 1000}
                    break
                prev = k
        clk_steady = cs.result
        if steady is None:
            steady = {"unconverged_after_steps": it}
    sim.close()

    # End to end through the C ABI from host buffers, every call: the host
    # flag grid (preprocess's input) goes up, preprocess + alloc run on the
    # device (plb_create_from_flag), init, S lattice steps, and the macros
    # come back.  S defaults to 1000, the reference's interval between
    # part-file dumps (porelb.c:436); the table is built again on every call.
    # The same through the V.bin table (plb_create from 152-byte records) is
    # reported beside it.
    e2e_steps = args.e2e_steps

    def pinned(a):
        """a copy of a in page-locked host memory (the tensor is kept alive
        by the closure's list)"""
        t = torch.empty(a.nbytes, dtype=torch.uint8, pin_memory=True)
        keep.append(t)
        v = t.numpy().view(a.dtype).reshape(a.shape)
        v[...] = a
        return v

    keep = []
    Vh = pinned(np.ascontiguousarray(V))
    fh = pinned(np.ascontiguousarray(flag))
    rho = pinned(np.zeros((4, N)))

    def e2e_rate(make):
        vals = []
        for k in range(args.e2e_reps + 1 if args.e2e_reps > 0 else 0):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s2 = make()
            s2.init_dist_macro()
            s2.step(e2e_steps)
            s2.macros(out=rho)
            s2.close()
            el = time.perf_counter() - t0
            if k > 0:
                vals.append(N * e2e_steps / el / 1e6)
        if not vals:
            return None
        # whole-job rate: the slowest rank's time for the same per-rank work
        t_rank = N * e2e_steps / (statistics.median(vals) * 1e6)
        return N * e2e_steps * world / max_over_ranks(t_rank, world) / 1e6

    e2e = e2e_rate(lambda: P.Simulation.from_flag(
        fh, *dims, tau=w["tau"], force=w["force"], precision=prec,
        device=local, kernel_variant=kv))
    e2e_v = e2e_rate(lambda: P.Simulation(
        Vh, *dims, vs, tau=w["tau"], force=w["force"], precision=prec,
        device=local, kernel_variant=kv))

    peak, peak_kind = hbm_peak()
    order = P.auto_ordering(N, dims[2], prec, local)
    traffic, traffic_src = recorded_traffic(args.workload, prec, N, order)
    bpn = BYTES_PER_NODE[prec]
    achieved = bpn * N / (ms_step * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "MLUPS",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms_step, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if prec.startswith("fp64") else "f32",
        "data": DATA,
        "config": workload_config(args.workload, w, N, phi, prec),
        "parallelism": f"replicas{world}",
        "layout": "SoA f[19][npad] ping-pong, %s node order" % order,
        "k_darcy_after_run": kd, "steady_state": steady,
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1),
                     "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4),
                     "traffic": traffic,
                     "traffic_source": traffic_src,
                     "bytes_per_node": bpn, "peak_kind": peak_kind},
        # one end-to-end call = upload, device build, init, e2e_steps lattice
        # steps and the macros back; the per-step bytes are the call's bytes
        # spread over its lattice steps
        "e2e": {"value": round(e2e, 3) if e2e else None, "unit": "MLUPS",
                "h2d_bytes_per_step": round(fh.nbytes / e2e_steps, 1),
                "d2h_bytes_per_step": round(rho.nbytes / e2e_steps, 1),
                "h2d_bytes_per_call": int(fh.nbytes),
                "d2h_bytes_per_call": int(rho.nbytes),
                "lattice_steps_per_call": e2e_steps,
                "host_memory": "pinned",
                "path": "host flag grid -> plb_create_from_flag -> steps -> macros"},
        "e2e_vbin": {"value": round(e2e_v, 3) if e2e_v else None,
                     "unit": "MLUPS",
                     "h2d_bytes_per_step": round(Vh.nbytes / e2e_steps, 1),
                     "d2h_bytes_per_step": round(rho.nbytes / e2e_steps, 1),
                     "h2d_bytes_per_call": int(Vh.nbytes),
                     "d2h_bytes_per_call": int(rho.nbytes),
                     "lattice_steps_per_call": e2e_steps,
                     "path": "host V.bin table -> plb_create -> steps -> macros"},
        "gpu_launches": args.steps,
        "clocks": clk.result,
        "clocks_steady_run": clk_steady,
    }
    if rank == 0 and not args.no_cpu:
        cores = host_threads()
        p = slab_count(dims[2], cores)
        Vp, vsp = P.build_table(flag, *dims, p)
        v, steps, el = cpu_port_mlups(Vp, vsp, dims, w, args.cpu_budget, p)
        line["cpu_baseline"] = {
            "value": round(v, 3), "unit": "MLUPS", "cores": p, "kind": "port",
            "sample": f"{steps} lattice steps of the full workload "
                      f"({el:.1f} s), {p} z-slab ranks on {p} threads"}
    if rank == 0 and world == 1 and not args.no_extras:
        # the rest of the metric: served permeability solves (solves/s and
        # latency, answers against FP64) and the batched pool against the
        # plain kernel; bounded runs of the serving and batched workloads
        t0 = time.perf_counter()
        served = served_result(args.extra_requests, args.extra_rate,
                               args.budget_gb, args.serve_precision,
                               args.serve_check_every, args.max_steps,
                               max_wall=args.extra_wall, fp64_check=0,
                               plain_fp64=True)
        ks64 = served.pop("_plain_ks")
        line["served"] = served
        # the serving configuration as specified: FP16 deviation storage
        # (with the hand-off to FP32 that lets tight tolerances finish), on
        # the same requests, answers against the same FP64 plain solves
        if args.serve_precision != "fp16dev":
            c5 = served_result(args.extra_requests, args.extra_rate,
                               args.budget_gb, "fp16dev", args.serve_check_every,
                               args.max_steps, max_wall=args.extra_wall,
                               fp64_check=0, plain_ks=ks64)
            c5.pop("_plain_ks")
            line["served_fp16"] = c5
        line["batched"] = batched_result(args.samples, args.check_every,
                                         args.max_steps, args.plain_steps)
        line["extras_wall_s"] = round(time.perf_counter() - t0, 1)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)


# ------------------------------------------------------------- batched / served

def _steady_batch(samples, precision, K, max_steps, capacity=None):
    """Run samples (workloads.Sample) to steady state in one pool; returns
    {index: result}, node-steps and wall time."""
    import porelb_gb300 as P  # noqa: F401
    from porelb_gb300.batch import Batch
    cap = capacity or sum(int(s.edge ** 3 * s.porosity * 1.05) + 512
                          for s in samples)
    b = Batch(cap, max(len(samples), 1), precision, check_every=K)
    ids = {}
    for smp in samples:
        sid = b.add_packed(smp.seed, smp.edge, smp.edge, smp.edge, smp.rmin,
                           smp.rmax, smp.porosity, smp.tau, smp.force,
                           tol=smp.tol, max_steps=max_steps)
        ids[sid] = (smp.index, b.num_nodes(sid))
    out = {}
    node_steps = 0
    t0 = time.perf_counter()
    while True:
        live = b.info()["used_nodes"]
        if live == 0:
            break
        node_steps += sum(n for sid, (_, n) in ids.items()
                          if b.result(sid)["status"] == 0) * K
        if b.run(1) == 0:
            pass
        for sid in b.poll():
            idx, n = ids[sid]
            r = b.result(sid)
            r["nodes"] = n
            out[idx] = r
    wall = time.perf_counter() - t0
    b.close()
    return out, node_steps, wall


def run_pool(args):
    """Throughput of the batch step on a fixed pool: --samples sphere packs of
    --edge^3 (seeds 100, 101, ...; R ~ U[3, 6], porosity 0.35, tau 0.8,
    F 5e-7) in the --precision form, stepped for --steps lattice steps in
    intervals of --check-every (no sample retires), timed by wall clock
    around the intervals after one warm-up interval."""
    import torch
    from porelb_gb300.batch import Batch
    torch.cuda.set_device(0)
    K = args.check_every
    cap = int(args.samples * (args.edge ** 3 * 0.40 + 512))
    groups = {"off": False, "l2": True}.get(args.l2_groups)
    if groups is None:
        groups = int(args.l2_groups)
    b = Batch(cap, max(args.samples, 1), args.precision, check_every=K,
              l2_groups=groups)
    n = 0
    for k in range(args.samples):
        sid = b.add_packed(100 + k, args.edge, args.edge, args.edge, 3.0, 6.0, 0.35,
                           0.8, 5e-7, tol=0.0, max_steps=10 ** 9)
        n += b.num_nodes(sid)
    b.run(1)
    torch.cuda.synchronize()
    intervals = max(1, args.steps // K)
    t0 = time.perf_counter()
    b.run(intervals)
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    b.close()
    line = {"metric": f"fluid MLUPS (batch step, {args.precision})",
            "value": round(n * intervals * K / el / 1e6, 1), "unit": "MLUPS",
            "steps": intervals * K, "num_node": n,
            "config": {"workload": f"pool of {args.samples} sphere packs of "
                                   f"{args.edge}^3, seeds 100+",
                       "check_every": K, "precision": args.precision,
                       "l2_groups": args.l2_groups}}
    print(json.dumps(line), flush=True)


def batched_result(n_samples, K, max_steps, plain_steps):
    """The batched workload (n_samples samples of seed 3, FP32 storage, each
    to its 1e-7 steady-state test) in one pool, against looping the plain
    FP32 kernel and the plain FP64 form over the samples, with each
    sample's permeability against the FP64 pool's."""
    import torch
    import porelb_gb300 as P
    from porelb_gb300.workloads import batched_samples
    from porelb_gb300 import tune
    samples = batched_samples(n_samples, 3)
    # the pools take the launch tuner's choice for their form
    launch = {f: {k: v for k, v in tune.ensure_pool(f).items() if k != "tune_s"}
              for f in ("fp32", "fp64")}
    res32, ns32, wall32 = _steady_batch(samples, "fp32", K, max_steps)
    res64, ns64, wall64 = _steady_batch(samples, "fp64", K, max_steps)
    # plain kernel per sample (FP32, and the FP64 plain form), timed on a
    # fixed step count, then each loop over the samples is costed with each
    # sample's own step count in its pool
    loop_s = 0.0
    loop64_s = 0.0
    for smp in samples:
        for prec in ("fp32", "fp64"):
            sim = P.Simulation.packed(smp.seed, smp.edge, smp.edge, smp.edge,
                                      smp.rmin, smp.rmax, smp.porosity,
                                      tau=smp.tau, force=smp.force,
                                      precision=prec)
            sim.init_dist_macro()
            sim.step(20)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            sim.step(plain_steps, it_begin=20)
            el = time.perf_counter() - t0
            sim.close()
            if prec == "fp32":
                loop_s += el / plain_steps * res32[smp.index]["steps"]
            else:
                loop64_s += el / plain_steps * res64[smp.index]["steps"]
    errs = [abs(res32[i]["k_darcy"] - res64[i]["k_darcy"]) /
            abs(res64[i]["k_darcy"]) for i in res32 if res64[i]["k_darcy"]]
    conv = sum(1 for r in res32.values() if r["status"] == 1)
    return {
        "metric": "fluid MLUPS (batched, FP32)",
        "value": round(ns32 / wall32 / 1e6, 1), "unit": "MLUPS",
        "plain_loop_mlups": round(ns32 / loop_s / 1e6, 1),
        "speedup_vs_plain_loop": round(loop_s / wall32, 3),
        # the plain form (FP64, one sample at a time) on the same samples
        "plain_fp64_loop_mlups": round(ns64 / loop64_s / 1e6, 1),
        "mlups_ratio_vs_plain_fp64_loop": round((ns32 / wall32) / (ns64 / loop64_s), 3),
        "fp64_batched_mlups": round(ns64 / wall64 / 1e6, 1),
        "samples": len(samples), "converged": conv,
        "k_rel_err_vs_fp64": {"max": max(errs), "median": statistics.median(errs),
                              "within_1e-3": sum(e <= 1e-3 for e in errs),
                              "of": len(errs)},
        "wall_s": round(wall32, 2), "check_every": K,
        "pool_launch_tuned": launch,
        "config": {"workload": f"batched {len(samples)} samples, seed 3",
                   "edges": [s.edge for s in samples],
                   "tol": 1e-7, "force": 1e-6, "max_steps": max_steps},
    }


def run_batched(args):
    import torch
    torch.cuda.set_device(0)
    print(json.dumps(batched_result(args.samples, args.check_every, args.max_steps,
                                    args.plain_steps)), flush=True)


def _plain_fp64_fcfs(reqs, K, max_steps):
    """The FP64 plain form serving the same requests one at a time, first
    come first served: each request is solved alone (FP64 fixed-point step,
    same steady-state test every K steps); queueing is replayed on the
    arrival times with the measured solve times."""
    import torch
    import porelb_gb300 as P
    ks, service = {}, []
    node_steps, stepping_s = 0, 0.0
    for r in reqs:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sim = P.Simulation.packed(r.seed, r.edge, r.edge, r.edge, r.rmin,
                                  r.rmax, r.porosity, tau=r.tau, force=r.force,
                                  precision="fp64")
        sim.init_dist_macro()
        it, prev, k, checks = 0, None, None, 0
        while it < max_steps:
            ts = time.perf_counter()
            sim.step(K, it_begin=it)
            it += K
            k = sim.permeability()[0]
            stepping_s += time.perf_counter() - ts
            node_steps += sim.N * K
            checks += 1
            if checks >= 2 and k != 0 and abs(k - prev) <= r.tol * abs(k):
                break
            prev = k
        sim.close()
        service.append(time.perf_counter() - t0)
        ks[r.index] = k
    t_free, lat = 0.0, []
    for r, sv in zip(reqs, service):
        start = max(r.arrival, t_free)
        t_free = start + sv
        lat.append(t_free - r.arrival)
    span = t_free - reqs[0].arrival
    return ks, dict(solves_per_s=len(reqs) / span if span > 0 else None,
                    p50_latency_s=float(np.percentile(lat, 50)),
                    p99_latency_s=float(np.percentile(lat, 99)),
                    mean_solve_s=float(np.mean(service)),
                    fluid_mlups_stepping=(node_steps / stepping_s / 1e6
                                          if stepping_s > 0 else None))


SERVE_FORMS = {"fp16dev": "FP16 deviations", "bf16dev": "BF16 deviations",
               "fp32": "FP32", "fp64": "FP64"}


def served_result(n_requests, rate, budget_gb, precision, K, max_steps,
                  max_wall=None, fp64_check=32, plain_fp64=False, plain_ks=None):
    """The serving workload (n_requests Poisson requests of seed 4 at `rate`
    per second) through the continuous-batching server, with the
    permeabilities checked against FP64: a pooled FP64 solve of the first
    fp64_check answered requests, and with plain_fp64 the FP64 plain form
    serving every answered request one at a time (first come first
    served), which also gives that form's solves/s and latencies.  plain_ks
    (request index -> k of the FP64 plain form, from an earlier run on the
    same requests) compares the answers without solving them again.  The
    result's "_plain_ks" holds the FP64 plain form's k per request."""
    from porelb_gb300.serve import Server
    from porelb_gb300.workloads import serving_requests
    reqs = serving_requests(n_requests, 4, rate)
    srv = Server(budget_gb * 1e9, precision, check_every=K)
    done, summ = srv.serve(reqs, max_wall=max_wall)
    srv.close()
    by = {d["index"]: d for d in done}
    sub = [r for r in reqs if r.index in by][:fp64_check]
    res64, ns64, wall64 = (_steady_batch(sub, "fp64", K, max_steps) if sub
                           else ({}, 0, 0.0))
    errs = [abs(by[i]["k_darcy"] - r["k_darcy"]) / abs(r["k_darcy"])
            for i, r in res64.items() if r["k_darcy"]]
    plain = None
    ks64 = dict(plain_ks or {})
    if plain_fp64:
        served = [r for r in reqs if r.index in by]
        ks64, plain = _plain_fp64_fcfs(served, K, max_steps)
        perr = [abs(by[i]["k_darcy"] - k) / abs(k) for i, k in ks64.items() if k]
        if plain["fluid_mlups_stepping"] and summ["fluid_mlups_busy"]:
            plain["mlups_ratio_served_busy_vs_plain_fp64"] = round(
                summ["fluid_mlups_busy"] / plain["fluid_mlups_stepping"], 3)
        plain["k_rel_err_served_vs_plain_fp64"] = {
            "max": max(perr) if perr else None,
            "median": statistics.median(perr) if perr else None,
            "within_1e-3": sum(e <= 1e-3 for e in perr), "of": len(perr)}
    aerr = [abs(by[i]["k_darcy"] - k) / abs(k) for i, k in ks64.items() if k and i in by]
    return {
        "metric": "perm solves/s (served, %s)" % SERVE_FORMS[precision],
        "value": round(summ["solves_per_s"], 3), "unit": "solves/s",
        "p50_latency_s": round(summ["p50_latency_s"], 3),
        "p99_latency_s": round(summ["p99_latency_s"], 3),
        "fluid_mlups": round(summ["fluid_mlups"], 1),
        "fluid_mlups_gpu_busy": (round(summ["fluid_mlups_busy"], 1)
                                 if summ["fluid_mlups_busy"] else None),
        "requests_done": summ["requests"], "requests": len(reqs),
        "rejected": len(summ["rejected"]),
        "k_rel_err_vs_fp64": {"checked": len(errs),
                              "max": max(errs) if errs else None,
                              "median": statistics.median(errs) if errs else None,
                              "within_1e-3": sum(e <= 1e-3 for e in errs)},
        "fp64_mlups_on_checked": round(ns64 / wall64 / 1e6, 1) if wall64 else None,
        "plain_fp64_fcfs": plain,
        # every answer against the FP64 plain form's k of the same request
        "k_rel_err_vs_plain_fp64": ({"max": max(aerr), "median": statistics.median(aerr),
                                     "within_1e-3": sum(e <= 1e-3 for e in aerr),
                                     "of": len(aerr)} if aerr else None),
        "_plain_ks": ks64,
        "time_split_s": {"admission_overlapped": round(summ["admit_s"], 2),
                         "waiting_for_intervals": round(summ["wait_s"], 2),
                         "gpu_busy": round(summ["gpu_busy_s"], 2),
                         "wall": round(summ["wall_s"], 2)},
        "gpu_idle_frac": (round(summ["gpu_idle_frac"], 4)
                          if summ["gpu_idle_frac"] is not None else None),
        "handoffs": summ["handoffs"], "handoff_tol": summ["handoff_tol"],
        "pool_launch_tuned": summ["pool_launch"],
        "config": {"workload": f"{len(reqs)} Poisson requests, seed 4",
                   "rate_per_s": rate, "budget_gb": budget_gb,
                   "check_every": K, "storage": precision,
                   "capacity_nodes": summ["capacity_nodes"]},
    }


def run_served(args):
    import torch
    torch.cuda.set_device(0)
    res = served_result(args.requests, args.rate, args.budget_gb,
                        args.serve_precision, args.serve_check_every,
                        args.max_steps, args.max_wall, args.fp64_check,
                        args.plain_fp64)
    res.pop("_plain_ks")
    print(json.dumps(res), flush=True)


def _steady_flag(flag, dims, precision, tau, force, tol, K, max_steps):
    """One sample from a host flag grid run to its steady-state test in a
    pool of its own: the pool's result record."""
    from porelb_gb300.batch import Batch
    n = int((flag == 1).sum())
    with Batch(n + 1024, 2, precision, check_every=K) as b:
        sid = b.add_flag(flag, *dims, tau, force, tol=tol, max_steps=max_steps)
        while b.run(1):
            pass
        return b.result(sid)


def run_precision(args):
    """1024^3, porosity 0.20, R 8, seed 2, tau 0.9, F 5e-7 at four storage
    forms (MLUPS), and the permeability of the pack's 256^3 corner
    subvolume (cells [0, 256)^3 of the same flag field, run as a periodic
    sample) at each form, every form to its own steady-state test, against
    the FP64 solve of that subvolume (the 16-bit forms' test capped at 30000
    steps: their <u_x> wanders by more than 1e-7 of itself)."""
    import torch
    import porelb_gb300 as P
    torch.cuda.set_device(0)
    n = args.edge
    out = {}
    forms = ("fp64", "fp32", "fp16dev", "bf16dev")
    for prec in forms:
        sim = P.Simulation.packed(2, n, n, n, 8.0, 8.0, 0.20, tau=0.9,
                                  force=5e-7, precision=prec)
        sim.init_dist_macro()
        sim.step(3)
        stream = torch.cuda.ExternalStream(sim.stream, device=0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.step_async(args.steps, it_begin=3)
        e1.record(stream)
        sim.sync()
        ms = e0.elapsed_time(e1)
        out[prec] = dict(mlups=round(sim.N * args.steps / (ms * 1e-3) / 1e6, 1),
                         bytes_per_node=BYTES_PER_NODE[prec],
                         num_node=sim.N, device_bytes=sim.info()["device_bytes"])
        sim.close()
    flag, _, _ = P.sphere_pack_device(2, n, n, n, 8.0, 8.0, 0.20)
    m = min(256, n)
    sub = np.ascontiguousarray(flag.reshape(n, n, n)[:m, :m, :m])
    ks = {}
    for prec in forms:
        cap = args.max_steps if prec in ("fp64", "fp32") else min(args.max_steps, 30000)
        ks[prec] = _steady_flag(sub, (m, m, m), prec, 0.9, 5e-7, 1e-7, args.check_every, cap)
    for prec in forms[1:]:
        out[prec]["k_rel_err_vs_fp64_256"] = abs(ks[prec]["k_darcy"] - ks["fp64"]["k_darcy"]) / abs(ks["fp64"]["k_darcy"])
    line = {"metric": "fluid MLUPS by storage form", "unit": "MLUPS",
            "value": out["fp16dev"]["mlups"], "forms": out,
            "k_256": {p: ks[p]["k_darcy"] for p in ks},
            "steps_256": {p: ks[p]["steps"] for p in ks},
            "status_256": {p: ks[p]["status"] for p in ks},
            "config": {"workload": f"{n}^3 sphere pack seed 2 R 8 porosity 0.20",
                       "tau": 0.9, "force": 5e-7,
                       "subvolume": f"cells [0, {m})^3 of the same flag field, periodic"}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c2_256", choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="fp64",
                    choices=sorted(BYTES_PER_NODE))
    ap.add_argument("--kernel-variant", type=int, default=0,
                    help="FP64 step kernel (0 = the library default)")
    ap.add_argument("--steady-wall", type=float, default=60.0,
                    help="seconds allowed for the untimed run to steady state "
                         "(0 = skip)")
    ap.add_argument("--e2e-steps", type=int, default=1000,
                    help="lattice steps per end-to-end call (default: the "
                         "reference's interval between part-file dumps)")
    ap.add_argument("--e2e-reps", type=int, default=2)
    ap.add_argument("--cpu-budget", type=float, default=10.0,
                    help="seconds of the GPU arm's CPU-baseline sample")
    ap.add_argument("--ref-budget", type=float, default=60.0,
                    help="seconds of CPU work in all for --impl reference")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--mode", default="plain",
                    choices=["plain", "batched", "served", "precision", "pool"])
    ap.add_argument("--samples", type=int, default=64)
    ap.add_argument("--check-every", type=int, default=1000,
                    help="steady-state check interval of the batched and "
                         "precision runs (the 1000 steps of the plain FP64 "
                         "workload's steady-state definition)")
    ap.add_argument("--serve-check-every", type=int, default=250,
                    help="check interval of the served runs (the requests "
                         "name a tolerance, not an interval; 250 steps give "
                         "answers within 2e-6 of FP64 solves checked every "
                         "1000 steps, and twice the solves/s of 1000)")
    ap.add_argument("--max-steps", type=int, default=200000)
    ap.add_argument("--plain-steps", type=int, default=200)
    ap.add_argument("--requests", type=int, default=2000)
    ap.add_argument("--rate", type=float, default=5.0)
    ap.add_argument("--budget-gb", type=float, default=80.0)
    ap.add_argument("--max-wall", type=float, default=None)
    ap.add_argument("--fp64-check", type=int, default=32)
    ap.add_argument("--serve-precision", default="fp32",
                    choices=sorted(SERVE_FORMS))
    ap.add_argument("--plain-fp64", action="store_true",
                    help="also serve the same requests with the FP64 plain "
                         "form, one at a time (first come first served)")
    ap.add_argument("--edge", type=int, default=1024)
    ap.add_argument("--l2-groups", default="off",
                    help="pool mode: the pool's L2 groups (off, l2 = 60%% of "
                         "the L2, or a budget in KiB)")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the served and batched runs of the default line")
    ap.add_argument("--extra-requests", type=int, default=200,
                    help="requests of the served run in the default line")
    ap.add_argument("--extra-rate", type=float, default=20.0)
    ap.add_argument("--extra-wall", type=float, default=120.0,
                    help="wall-clock cap of the served run in the default line")
    args = ap.parse_args()
    if args.mode == "batched":
        return run_batched(args)
    if args.mode == "served":
        return run_served(args)
    if args.mode == "pool":
        return run_pool(args)
    if args.mode == "precision":
        return run_precision(args)
    args.warmup = max(args.warmup, 3)
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_gpu(args, rank, world, local)


if __name__ == "__main__":
    main()
