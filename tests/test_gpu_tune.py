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
