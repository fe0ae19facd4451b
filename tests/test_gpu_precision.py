"""Reduced-precision storage forms against FP64, at steady state.

Each storage form (FP32 deviations, scaled FP16 deviations, BF16 deviations)
solves a sphere pack to the steady-state test; its permeability must lie
within 1e-3 relative of the bit-exact FP64 form's (which equals the
reference's collision, porelb.c:318-365, bit for bit) on the same pack
after the same number of steps.  The plain kernel and the batched pool are
both checked, and a batched FP32 mix of uneven samples is checked sample by
sample against FP64 solves of each sample alone.  The measured error is in
every assertion message."""
import pytest

import porelb_gb300 as P
from porelb_gb300.batch import Batch

from helpers import pack_flag

pytestmark = pytest.mark.gpu

K_TOL = 1e-3
# the 64^3 plain configuration's geometry and physics: seed 0, R 6,
# porosity 0.40, tau 1.0, F 1e-6
DIMS = (64, 64, 64)
TAU, FORCE = 1.0, 1e-6
CHECK = 500


@pytest.fixture(scope="module")
def c1():
    return pack_flag(DIMS, 0, 6.0, 6.0, 0.40)


def steady_exact(flag, dims, tau, force, tol, check=CHECK, cap=40000):
    """The bit-exact FP64 form run to the steady-state test (relative change
    of <u_x> over `check` steps at most tol): (k, steps)."""
    with P.Simulation.from_flag(flag, *dims, tau=tau, force=force,
                                precision="fp64_exact") as sim:
        sim.init_dist_macro()
        it, prev = 0, None
        while it < cap:
            sim.step(check, it_begin=it)
            it += check
            k = sim.permeability()[0]
            if prev is not None and abs(k - prev) <= tol * abs(k):
                return k, it
            prev = k
    raise AssertionError(f"FP64 not steady after {cap} steps")


def exact_k_at(flag, dims, tau, force, steps):
    with P.Simulation.from_flag(flag, *dims, tau=tau, force=force,
                                precision="fp64_exact") as sim:
        sim.init_dist_macro()
        sim.step(steps)
        return sim.permeability()[0]


@pytest.fixture(scope="module")
def c1_exact(c1):
    return steady_exact(c1, DIMS, TAU, FORCE, 1e-7)


@pytest.mark.parametrize("precision", ["fp32", "fp16dev", "bf16dev"])
def test_plain_form_permeability_within_1e3_of_fp64(c1, c1_exact, precision):
    k64, steps = c1_exact
    with P.Simulation.from_flag(c1, *DIMS, tau=TAU, force=FORCE,
                                precision=precision) as sim:
        sim.init_dist_macro()
        sim.step(steps)
        k = sim.permeability()[0]
    err = abs(k - k64) / abs(k64)
    assert err <= K_TOL, f"{precision}: k {k!r} vs FP64 {k64!r}, rel err {err:.3e}"


@pytest.mark.parametrize("precision,tol", [("fp32", 1e-7), ("fp16dev", 1e-6),
                                           ("bf16dev", 1e-6)])
def test_pool_form_steady_permeability_within_1e3_of_fp64(c1, c1_exact, precision, tol):
    """The pool runs the form to its own steady-state test; FP64 is taken
    at the same step count."""
    with Batch(200000, 4, precision, check_every=CHECK) as b:
        sid = b.add_flag(c1, *DIMS, TAU, FORCE, tol=tol, max_steps=60000)
        while b.run(1):
            pass
        r = b.result(sid)
    assert r["status"] == 1, f"{precision}: not steady ({r})"
    k64 = exact_k_at(c1, DIMS, TAU, FORCE, r["steps"])
    err = abs(r["k_darcy"] - k64) / abs(k64)
    assert err <= K_TOL, (f"{precision}: k {r['k_darcy']!r} after {r['steps']} steps "
                          f"vs FP64 {k64!r}, rel err {err:.3e}")


MIX = [((40, 40, 40), 31, 3.0, 5.0, 0.45, 0.7),
       ((32, 32, 32), 32, 3.0, 4.0, 0.30, 1.3),
       ((48, 40, 36), 33, 4.0, 8.0, 0.50, 0.9),
       ((28, 28, 28), 34, 3.0, 3.0, 0.25, 0.6),
       ((36, 36, 36), 35, 3.0, 6.0, 0.40, 1.5)]


def test_batched_fp32_mix_each_sample_within_1e3_of_fp64_alone():
    K = 200
    with Batch(400000, 8, "fp32", check_every=K) as b:
        ids = {}
        for dims, seed, r0, r1, phi, tau in MIX:
            flag = pack_flag(dims, seed, r0, r1, phi)
            ids[b.add_flag(flag, *dims, tau, 1e-6, tol=1e-7, max_steps=60000)] = \
                (flag, dims, tau)
        while b.run(1):
            pass
        res = {sid: b.result(sid) for sid in ids}
    errs = []
    for sid, (flag, dims, tau) in ids.items():
        r = res[sid]
        assert r["status"] == 1, f"sample {sid} not steady: {r}"
        k64 = exact_k_at(flag, dims, tau, 1e-6, r["steps"])
        errs.append(abs(r["k_darcy"] - k64) / abs(k64))
    assert max(errs) <= K_TOL, f"per-sample rel err vs FP64 alone: {errs}"
