"""Batched pool: each sample's result equals its single-solve result (bit for
bit in the same form), whatever else shares the pool; convergence retires
samples and frees their blocks for new ones."""
import numpy as np
import pytest

import porelb_gb300 as P
from porelb_gb300.batch import Batch

from helpers import max_rel, pack_flag

pytestmark = pytest.mark.gpu

SAMPLES = [((20, 18, 16), 3, 3.0, 4.0, 0.45, 0.8, 2e-4),
           ((12, 12, 12), 4, 2.0, 3.0, 0.40, 1.1, 1e-4),
           ((24, 16, 20), 5, 2.5, 5.0, 0.35, 0.65, 5e-5)]


def single(flag, dims, tau, force, steps, precision):
    sim = P.Simulation.from_flag(flag, *dims, tau=tau, force=force,
                                 precision=precision)
    sim.init_dist_macro()
    sim.step(steps)
    f = sim.get_f()
    kd = sim.permeability()[0]
    sim.close()
    return f, kd


@pytest.mark.parametrize("precision", ["fp64", "fp32", "fp16dev"])
def test_batch_samples_equal_single_solves(precision):
    K = 20
    with Batch(200000, 16, precision, check_every=K) as b:
        ids = []
        flags = []
        for dims, seed, rmin, rmax, phi, tau, force in SAMPLES:
            flag = pack_flag(dims, seed, rmin, rmax, phi)
            flags.append(flag)
            ids.append(b.add_flag(flag, *dims, tau, force, tol=0.0))
        b.run(2)
        for sid, flag, (dims, _, _, _, _, tau, force) in zip(ids, flags, SAMPLES):
            f_b = b.get_f(sid)
            if precision == "fp16dev":
                # the batch adapts the 16-bit scale; compare at tolerance
                f_s, _ = single(flag, dims, tau, force, 2 * K, "fp64")
                assert max_rel(f_b, f_s) < 1e-3
            else:
                f_s, _ = single(flag, dims, tau, force, 2 * K, precision)
                assert (f_b == f_s).all()


def test_batch_result_same_alone_and_in_mix():
    K = 20
    dims, seed, rmin, rmax, phi, tau, force = SAMPLES[0]
    flag = pack_flag(dims, seed, rmin, rmax, phi)
    with Batch(50000, 4, "fp32", check_every=K) as alone:
        a = alone.add_flag(flag, *dims, tau, force, tol=0.0, max_steps=3 * K)
        alone.run(5)
        ra = alone.result(a)
    with Batch(200000, 16, "fp32", check_every=K) as mix:
        other = [mix.add_flag(pack_flag(d, s, r0, r1, p), *d, t, fo, tol=0.0)
                 for d, s, r0, r1, p, t, fo in SAMPLES[1:]]
        mix.run(1)
        m = mix.add_flag(flag, *dims, tau, force, tol=0.0, max_steps=3 * K)
        mix.run(5)
        rm = mix.result(m)
        assert other
    assert ra["status"] == 2 and rm["status"] == 2
    assert ra["steps"] == rm["steps"] == 3 * K
    assert ra["k_darcy"] == rm["k_darcy"]


def test_batch_convergence_retires_and_backfills():
    K = 50
    with Batch(12000, 8, "fp32", check_every=K) as b:
        dims = (12, 12, 12)
        s0 = b.add_packed(11, *dims, 2.0, 3.0, 0.5, 0.9, 1e-5, tol=1e-4)
        s1 = b.add_packed(12, *dims, 2.0, 3.0, 0.5, 0.9, 1e-5, tol=1e-4)
        # the pool is now too small for a third sample of this size
        assert b.try_add_packed(13, 40, 40, 40, 2.0, 3.0, 0.5, 0.9, 1e-5) is None
        done = []
        for _ in range(400):
            if b.run(1) == 0:
                break
            done += b.poll()
        done += b.poll()
        assert sorted(done) == sorted([s0, s1])
        for sid in (s0, s1):
            r = b.result(sid)
            assert r["status"] == 1 and r["k_darcy"] > 0
            b.release(sid)
        assert b.info()["used_nodes"] == 0
        s2 = b.add_packed(13, 16, 16, 16, 2.0, 3.0, 0.5, 0.9, 1e-5, tol=1e-4)
        assert s2 >= 0


GROUP_SAMPLES = [((20, 18, 16), 3, 3.0, 4.0, 0.45, 0.8, 2e-4),
                 ((12, 12, 12), 4, 2.0, 3.0, 0.40, 1.1, 1e-4),
                 ((40, 36, 32), 6, 3.0, 6.0, 0.40, 0.9, 1e-4),
                 ((24, 16, 20), 5, 2.5, 5.0, 0.35, 0.65, 5e-5),
                 ((16, 16, 16), 7, 2.0, 4.0, 0.50, 1.3, 2e-4),
                 ((28, 28, 28), 8, 3.0, 5.0, 0.30, 0.7, 1e-4)]


@pytest.mark.parametrize("precision", ["fp32", "fp16dev", "bf16dev"])
def test_l2_groups_change_no_bit(precision):
    """The pool's L2 groups (samples that fit a budget step their interval
    group by group) against one chain over every sample: the same f and
    the same results.  A 1 MiB budget makes several groups and leaves the
    40x36x32 sample outside them; True takes 60% of the L2 (one group)."""
    K = 20
    out = {}
    for groups in (False, 1024, True):
        with Batch(400000, 16, precision, check_every=K, l2_groups=groups) as b:
            ids = [b.add_flag(pack_flag(dims, seed, rmin, rmax, phi), *dims, tau, force,
                              tol=0.0, max_steps=3 * K)
                   for dims, seed, rmin, rmax, phi, tau, force in GROUP_SAMPLES]
            b.run(2)
            fs = [b.get_f(sid) for sid in ids]
            b.run(3)
            res = [b.result(sid) for sid in ids]
            out[groups] = (fs, res)
    base_f, base_r = out[False]
    for groups in (1024, True):
        fs, res = out[groups]
        for a, c in zip(fs, base_f):
            assert np.array_equal(a, c), groups
        for a, c in zip(res, base_r):
            assert a["k_darcy"] == c["k_darcy"] and a["steps"] == c["steps"], groups
            assert a["status"] == c["status"] == 2, groups
