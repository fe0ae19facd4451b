"""The launch tuner: it times every candidate (block size, register
budget, node order), keeps the fastest, and the solver built with its
choice gives the same bits as the default launch."""
import pytest

import porelb_gb300 as P
from porelb_gb300 import tune

from helpers import pack_flag

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "fp16dev"])
def test_tune_picks_a_candidate_and_changes_no_result(precision):
    dims = (40, 32, 24)
    flag = pack_flag(dims, 21, 2.0, 5.0, 0.4)
    best, table = tune.tune(flag, dims, precision, steps=4)
    assert len(table) == 2 * 3 * 3
    assert all(ms > 0 for *_, ms in table)
    assert best["ms"] == min(ms for *_, ms in table)
    n = P.Simulation.from_flag(flag, *dims, precision=precision).N
    choice = tune.best(precision, n)
    assert choice == {k: best[k] for k in ("block_size", "ordering", "kernel_variant")}
    out = []
    for kw in ({}, choice):
        sim = P.Simulation.from_flag(flag, *dims, tau=0.8, force=1e-4, precision=precision,
                                     **kw)
        sim.init_dist_macro()
        sim.step(6)
        out.append(sim.macros())
        sim.close()
    # the node order may differ; the macros come back in reference order
    assert all((a == b).all() for a, b in zip(out[0], out[1]))


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_pool_tuner_picks_a_candidate_caches_it_and_changes_no_result(precision):
    """The pool tuner times batch-step CTAs of 128 and 256 threads with the
    L2 prefetch on and off, caches the fastest for the form, and a pool
    built afterwards takes it; every candidate gives the same bits."""
    from porelb_gb300.batch import Batch
    best, table = tune.tune_pool(precision, samples=4, edge=40, K=10)
    assert len(table) == 8 and all(ms > 0 for *_, ms in table)
    assert best["ms"] == min(ms for *_, ms in table)
    assert tune.best_pool(precision) == {k: best[k] for k in
                                         ("cta_threads", "l2_prefetch", "ordering")}
    with Batch(100000, 4, precision, check_every=10) as b:
        assert b.launch_choice == tune.best_pool(precision)
    dims = (24, 20, 16)
    flag = pack_flag(dims, 5, 2.0, 4.0, 0.4)
    ks = []
    for cta, pf, order in [(c, p, o) for c in tune.POOL_CTAS for p in tune.POOL_PREFETCH
                           for o in tune.POOL_ORDERINGS]:
        with Batch(50000, 2, precision, check_every=10, cta_threads=cta,
                   l2_prefetch=pf, ordering=order) as b:
            sid = b.add_flag(flag, *dims, 0.8, 1e-4, tol=0.0)
            b.run(3)
            ks.append((b.result(sid)["k_darcy"], b.get_f(sid)))
    assert all(k == ks[0][0] and (f == ks[0][1]).all() for k, f in ks)


def test_auto_ordering_picks_row_order_while_three_planes_fit_in_l2():
    """PLB_ORDER_AUTO: row (reference) order for the 256^3 FP64 workload and
    the 512^3 16-bit form, Morton for 512^3 and 1024^3 FP64 (measured
    fastest on GB300 in each case); both orders give the same bits."""
    assert P.auto_ordering(5871717, 256, "fp64") == "reference"
    assert P.auto_ordering(46976000, 512, "fp16dev") == "reference"
    assert P.auto_ordering(46976000, 512, "fp64") == "morton"
    assert P.auto_ordering(214748328, 1024, "fp64") == "morton"
    dims = (40, 32, 24)
    flag = pack_flag(dims, 21, 2.0, 5.0, 0.4)
    out = []
    for order in ("auto", "morton", "reference"):
        with P.Simulation.from_flag(flag, *dims, tau=0.8, force=1e-4, precision="fp64",
                                    ordering=order) as sim:
            sim.init_dist_macro()
            sim.step(5)
            out.append((sim.get_f(), sim.macros()))
    for f, m in out[1:]:
        assert (f == out[0][0]).all() and all((a == b).all() for a, b in zip(m, out[0][1]))
