"""Autotuner for the step launch: threads per block, register budget and
node ordering.

For one geometry and storage form it builds a solver per candidate
(block size in {64, 128, 256}; register budgets: default, tighter, tightest;
Morton or reference node order), times a few steps with CUDA events on the
solver's stream after a warm-up, and keeps the fastest.  Results are cached
per (form, boundary, node-count bucket) for the process; ``best`` returns the
cached choice when one exists.
"""
import math

from .api import Simulation

BLOCKS = (64, 128, 256)
ORDERINGS = ("morton", "reference")
_cache = {}


def _bucket(n):
    return int(round(math.log2(max(n, 1)) * 2))


def time_config(flag, dims, precision, block, ordering, tau=0.8, force=1e-5,
                steps=20, warmup=5, boundary="reference", variant=0):
    """Mean milliseconds per step of one configuration."""
    import torch
    sim = Simulation.from_flag(flag, *dims, tau=tau, force=force,
                               precision=precision, ordering=ordering,
                               block_size=block, boundary=boundary,
                               kernel_variant=variant)
    try:
        sim.init_dist_macro()
        sim.step(warmup)
        stream = torch.cuda.ExternalStream(sim.stream)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sim.step_async(steps, it_begin=warmup)
        e1.record(stream)
        sim.sync()
        return e0.elapsed_time(e1) / steps, sim.N
    finally:
        sim.close()


def tune(flag, dims, precision="fp64", boundary="reference", steps=20):
    """Time every candidate; returns (best, [(block, ordering, variant, ms)])."""
    table = []
    n = None
    variants = (0, 1, 3) if precision in ("fp64", "fp32", "fp16dev", "bf16dev") else (0,)
    for ordering in ORDERINGS:
        for block in BLOCKS:
            for v in variants:
                ms, n = time_config(flag, dims, precision, block, ordering,
                                    steps=steps, boundary=boundary, variant=v)
                table.append((block, ordering, v, ms))
    best = min(table, key=lambda r: r[3])
    choice = dict(block_size=best[0], ordering=best[1], kernel_variant=best[2])
    _cache[(precision, boundary, _bucket(n))] = choice
    return dict(choice, ms=best[3]), table


def best(precision, n, boundary="reference"):
    """Cached choice for this form and size, or the defaults."""
    return _cache.get((precision, boundary, _bucket(n)),
                      dict(block_size=0, ordering="morton", kernel_variant=0))
