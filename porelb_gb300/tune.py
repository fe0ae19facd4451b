"""Autotuner for the step launches: threads per block, register budget, node
ordering and L2 prefetch.

* ``tune`` (plain solver): for one geometry and storage form it builds a
  solver per candidate (block size in {64, 128, 256}; register budgets:
  default, tighter, tightest; Morton or reference node order), times a few
  steps with CUDA events on the solver's stream after a warm-up, and keeps
  the fastest.  Cached per (form, boundary, node-count bucket);
  ``best`` returns the cached choice, which ``Simulation(..., tuned=True)``
  uses.
* ``tune_pool`` (batched pool and server): for one storage form it builds a
  pool of synthetic sphere packs per candidate (batch-step CTAs of 128 or
  256 threads, L2 prefetch of the pool block half a wave ahead on or off,
  Morton or reference node order within each sample), times intervals of
  the batch step, and keeps the fastest.  Cached per
  form; every ``Batch`` created without an explicit launch takes the cached
  choice (``best_pool``), and ``Server`` tunes its pools' form when it
  starts.

The choices change no result: every candidate runs the same arithmetic on
the same nodes (tests/test_gpu_tune.py checks the bits).
"""
import math
import time

from .api import Simulation

BLOCKS = (64, 128, 256)
ORDERINGS = ("morton", "reference")
POOL_CTAS = (128, 256)
POOL_PREFETCH = (False, True)
POOL_ORDERINGS = ("morton", "reference")
_cache = {}
_pool_cache = {}


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
                      dict(block_size=0, ordering="auto", kernel_variant=0))


def time_pool(precision, cta_threads, l2_prefetch, samples=8, edge=64, K=20,
              intervals=3, device=0, ordering="morton"):
    """Milliseconds per lattice step of a pool of `samples` sphere packs of
    edge^3 (seeds 200+, R ~ U[3, 6], porosity 0.35) with this launch."""
    from .batch import Batch
    cap = int(samples * (edge ** 3 * 0.40 + 512))
    with Batch(cap, samples, precision, check_every=K, device=device,
               cta_threads=cta_threads, l2_prefetch=l2_prefetch, ordering=ordering) as b:
        for k in range(samples):
            b.add_packed(200 + k, edge, edge, edge, 3.0, 6.0, 0.35, 0.8, 5e-7,
                         tol=0.0, max_steps=10 ** 9)
        b.run(1)
        ms = []
        for _ in range(intervals):
            b.launch()
            b.finish()
            ms.append(b.interval_ms())
        return min(ms) / K


def tune_pool(precision, samples=8, edge=64, K=20, device=0):
    """Time every pool launch candidate for this form; caches and returns
    (best, [(cta_threads, l2_prefetch, ordering, ms per step)])."""
    table = []
    for order in POOL_ORDERINGS:
        for cta in POOL_CTAS:
            for pf in POOL_PREFETCH:
                table.append((cta, pf, order, time_pool(precision, cta, pf, samples, edge, K,
                                                        device=device, ordering=order)))
    best = min(table, key=lambda r: r[3])
    choice = dict(cta_threads=best[0], l2_prefetch=best[1], ordering=best[2])
    _pool_cache[precision] = choice
    return dict(choice, ms=best[3]), table


def best_pool(precision):
    """Cached pool launch for this form, or the library defaults (None)."""
    return _pool_cache.get(precision, dict(cta_threads=None, l2_prefetch=None,
                                           ordering=None))


def ensure_pool(precision, device=0):
    """The cached pool launch for this form, tuning it first if needed
    (about a second)."""
    if precision not in _pool_cache:
        t0 = time.perf_counter()
        tune_pool(precision, device=device)
        _pool_cache[precision]["tune_s"] = time.perf_counter() - t0
    return _pool_cache[precision]
