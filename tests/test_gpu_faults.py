"""Allocation failures, injected on the host.

The reference exits when an allocation fails (porelb.c:18-22,65-69); the
library returns PLB_ERR_NOMEM instead and must leave nothing behind.  Each
test counts the device allocations a call makes (plb_alloc_count), then
makes each of them fail in turn (plb_fault_inject_alloc: the allocation
reports out-of-memory without calling cudaMalloc, so no GPU fault is
involved), and checks that the call fails with PLB_ERR_NOMEM, that device
memory comes back, and that the same call then succeeds with the same
result."""
import numpy as np
import pytest

import porelb_gb300 as P
from porelb_gb300 import _lib
from porelb_gb300.batch import Batch

from helpers import pack_flag

pytestmark = pytest.mark.gpu

DIMS = (20, 18, 16)


def free_bytes():
    import torch
    torch.cuda.synchronize()
    return torch.cuda.mem_get_info()[0]


def each_allocation_fails(call, check=None):
    """Run call() once to count its allocations, then once per allocation
    with that allocation failing."""
    lib = _lib.load()
    n0 = lib.plb_alloc_count()
    ref = call()
    n = lib.plb_alloc_count() - n0
    assert n > 0
    before = free_bytes()
    for k in range(1, n + 1):
        lib.plb_fault_inject_alloc(k)
        with pytest.raises(P.PorelbError) as e:
            call()
        lib.plb_fault_inject_alloc(0)
        assert e.value.status == _lib.ERR_NOMEM, f"allocation {k} of {n}: {e.value}"
    # nothing left allocated (a few MiB of slack for the driver's own pools)
    assert before - free_bytes() < 64 << 20
    again = call()
    if check is not None:
        check(ref, again)
    return n


def test_create_paths_fail_cleanly():
    flag = pack_flag(DIMS, 3, 2.0, 4.0, 0.45)
    V, vs = P.build_table(flag, *DIMS, 1)

    def solve(make):
        def call():
            with make() as sim:
                sim.init_dist_macro()
                sim.step(5)
                return sim.get_f()
        return call

    same = lambda a, b: np.testing.assert_array_equal(a, b)  # noqa: E731
    for prec in ("fp64_exact", "fp16dev"):
        each_allocation_fails(solve(lambda: P.Simulation(V, *DIMS, vs, tau=0.8, force=1e-4,
                                                         precision=prec)), same)
        each_allocation_fails(solve(lambda: P.Simulation.from_flag(
            flag, *DIMS, tau=0.8, force=1e-4, precision=prec)), same)
    each_allocation_fails(solve(lambda: P.Simulation.packed(
        3, *DIMS, 2.0, 4.0, 0.45, tau=0.8, force=1e-4, precision="fp64")), same)


def test_readback_fails_cleanly_and_the_solver_goes_on():
    flag = pack_flag(DIMS, 3, 2.0, 4.0, 0.45)
    with P.Simulation.from_flag(flag, *DIMS, tau=0.8, force=1e-4,
                                precision="fp64_exact") as sim:
        sim.init_dist_macro()
        sim.step(3)
        each_allocation_fails(sim.get_f, lambda a, b: np.testing.assert_array_equal(a, b))
        each_allocation_fails(sim.macros, lambda a, b: np.testing.assert_array_equal(a, b))
        sim.step(3, it_begin=3)
        assert sim.permeability()[0] > 0


def test_pool_create_and_admission_fail_cleanly():
    each_allocation_fails(lambda: Batch(20000, 4, "fp32", check_every=10).close())
    with Batch(60000, 8, "fp32", check_every=10) as b:
        ids = []

        def admit():
            sid = b.add_packed(7, *DIMS, 2.0, 4.0, 0.45, 0.8, 1e-4, tol=0.0)
            ids.append(sid)
            return sid

        each_allocation_fails(admit)
        # a failed admission takes no pool room: the two that went through
        # are the only residents and they step
        blocks = -(-b.num_nodes(ids[0]) // 256) * 256
        assert len(ids) == 2 and b.info()["used_nodes"] == 2 * blocks
        b.run(2)
        r = [b.result(s) for s in ids]
        assert r[0]["steps"] == r[1]["steps"] == 20
        assert r[0]["k_darcy"] == r[1]["k_darcy"]


def test_transfer_allocates_nothing():
    """Moving a parked sample between pools uses the pools' own memory: it
    makes no allocation that could fail."""
    with Batch(60000, 4, "fp16dev", check_every=10) as h, \
            Batch(60000, 4, "fp32", check_every=10) as t:
        sid = h.add_packed(7, *DIMS, 2.0, 4.0, 0.45, 0.8, 1e-4, tol=1e-12, handoff_tol=0.5)
        while h.run(1):
            pass
        res = h.result(sid)
        assert res["status"] == 4
        lib = _lib.load()
        n0 = lib.plb_alloc_count()
        nid = h.transfer(sid, t)
        assert lib.plb_alloc_count() == n0
        h.release(sid)
        t.run(1)
        assert t.result(nid)["steps"] == res["steps"] + 10
