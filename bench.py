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
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM = 6800.0

# algorithmic bytes per fluid-node update: 19 loads + 19 stores of the
# distribution + 18 int32 neighbour words
BYTES_PER_NODE = {"fp64_exact": 376, "fp64": 376, "fp64_fma": 376, "fp32": 224,
                  "fp16dev": 148, "bf16dev": 148}

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
                 "--format=csv,noheader,nounits", "-lms", "200"],
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
    if rank != 0:
        return
    import porelb_gb300 as P
    w = WORKLOADS[args.workload]
    dims = w["dims"]
    flag, _, phi = make_geometry(w)
    cores = host_threads()
    p = slab_count(dims[2], cores)
    V, vs = P.build_table(flag, *dims, p)
    for _ in range(args.warmup):
        cpu_port_mlups(V, vs, dims, w, 1.0, p)
    vals = []
    detail = None
    for _ in range(args.steps):
        v, steps, el = cpu_port_mlups(V, vs, dims, w, args.cpu_budget, p)
        vals.append(v)
        detail = (steps, el)
    value = statistics.median(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3),
        "unit": "MLUPS", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": args.workload, "dims": list(dims),
                   "num_node": int(len(V)), "porosity": phi,
                   "tau": w["tau"], "force": w["force"]},
        "cpu_baseline": {"value": round(value, 3), "unit": "MLUPS",
                         "cores": p, "kind": "port",
                         "sample": f"{detail[0]} lattice steps of the full "
                                   f"workload per bench step ({detail[1]:.1f} s),"
                                   f" {p} z-slab ranks on {p} threads"},
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

    sim = P.Simulation(V, *dims, vs, tau=w["tau"], force=w["force"],
                       precision=prec, device=local)
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
    ms = e0.elapsed_time(e1)
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    ms_step = ms / args.steps
    value = N * args.steps * world / (ms * 1e-3) / 1e6
    kd, _ = sim.permeability()
    sim.close()

    # end to end through the C ABI from host buffers: table upload and
    # device build, init, S steps, macro read-back, every step
    e2e_steps = args.e2e_steps
    Vh = np.ascontiguousarray(V)
    rho = np.empty((4, N))
    e2e_vals = []
    for k in range(args.e2e_reps + 1 if args.e2e_reps > 0 else 0):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s2 = P.Simulation(Vh, *dims, vs, tau=w["tau"], force=w["force"],
                          precision=prec, device=local)
        s2.init_dist_macro()
        s2.step(e2e_steps)
        rho[:] = s2.macros()
        s2.close()
        el = time.perf_counter() - t0
        if k > 0:
            e2e_vals.append(N * e2e_steps / el / 1e6)
    e2e = statistics.median(e2e_vals) * world if e2e_vals else None

    peak, peak_kind = hbm_peak()
    bpn = BYTES_PER_NODE[prec]
    achieved = bpn * N / (ms_step * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "MLUPS",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(ms_step, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if prec.startswith("fp64") else "f32",
        "data": "synthetic sphere pack (seeded splitmix64 generator)",
        "config": {"workload": args.workload, "dims": list(dims),
                   "num_node": int(N), "porosity": phi, "tau": w["tau"],
                   "force": w["force"], "precision": prec,
                   "ordering": "morton",
                   "l2": "inputs larger than L2 (no flush)",
                   "parallelism": f"replicas{world}",
                   "k_darcy_after_run": kd},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1),
                     "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": None,
                     "bytes_per_node": bpn, "peak_kind": peak_kind},
        "e2e": {"value": round(e2e, 3) if e2e else None, "unit": "MLUPS",
                "h2d_bytes_per_step": int(Vh.nbytes),
                "d2h_bytes_per_step": int(rho.nbytes),
                "lattice_steps_per_call": e2e_steps},
        "gpu_launches": args.steps,
        "clocks": clk.result,
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
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c2_256", choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="fp64",
                    choices=sorted(BYTES_PER_NODE))
    ap.add_argument("--e2e-steps", type=int, default=200)
    ap.add_argument("--e2e-reps", type=int, default=2)
    ap.add_argument("--cpu-budget", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_gpu(args, rank, world, local)


if __name__ == "__main__":
    main()
