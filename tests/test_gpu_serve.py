"""The permeability server: requests that arrive while others run are
admitted as pool space frees up, and every answer is the one the request
gets solved alone (bit for bit in the server's storage form)."""
import pytest

from porelb_gb300.batch import Batch
from porelb_gb300.serve import Server
from porelb_gb300.workloads import Sample

pytestmark = pytest.mark.gpu


def requests():
    # (index, edge, porosity, rmin, rmax, tau, force, tol, seed, arrival)
    return [Sample(0, 40, 0.40, 3.0, 5.0, 0.8, 1e-6, 1e-6, 31, 0.00),
            Sample(1, 32, 0.35, 2.0, 4.0, 1.0, 1e-6, 1e-7, 32, 0.00),
            Sample(2, 48, 0.45, 3.0, 6.0, 0.7, 1e-6, 1e-6, 33, 0.01),
            Sample(3, 36, 0.30, 2.0, 4.0, 0.9, 1e-6, 1e-7, 34, 0.02),
            Sample(4, 44, 0.40, 3.0, 5.0, 1.2, 1e-6, 1e-6, 35, 0.02),
            Sample(5, 28, 0.50, 2.0, 3.0, 0.6, 1e-6, 1e-7, 36, 0.03)]


def alone(r, check_every):
    with Batch(int(r.edge ** 3 * 0.6) + 4096, 2, "fp32", check_every=check_every) as b:
        sid = b.add_packed(r.seed, r.edge, r.edge, r.edge, r.rmin, r.rmax, r.porosity,
                           r.tau, r.force, tol=r.tol)
        while b.run(1):
            pass
        return b.result(sid)


def test_server_answers_equal_solves_alone():
    K = 100
    # a budget that holds about two of these requests at once, so later ones
    # wait for retirements and backfill their blocks
    srv = Server(2 * 48 ** 3 * 0.5 * 224, "fp32", check_every=K)
    try:
        done, summary = srv.serve(requests())
    finally:
        srv.close()
    assert summary["requests"] == len(requests())
    by = {d["index"]: d for d in done}
    # the budget forced at least one request to wait for a retirement
    first_finish = min(d["finished"] for d in done)
    assert any(d["admitted"] >= first_finish for d in done)
    for r in requests():
        d = by[r.index]
        assert d["status"] == 1  # converged
        ref = alone(r, K)
        assert d["steps"] == ref["steps"]
        assert d["k_darcy"] == ref["k_darcy"]
        assert d["latency"] >= 0.0
    assert summary["p99_latency_s"] >= summary["p50_latency_s"] > 0.0


def served(reqs, K, precision, budget, **kw):
    srv = Server(budget, precision, check_every=K, **kw)
    try:
        return srv.serve(reqs)
    finally:
        srv.close()


def test_fp16_handoff_answers_same_alone_and_in_mix_and_within_1e3_of_fp64():
    """FP16-deviation storage with the hand-off to FP32 at a relative change
    of 1e-5: a request answers the same bits alone and among others that
    share (and fill) both pools, it finishes in the FP32 pool at its own
    tolerance, and its permeability is within 1e-3 of the bit-exact FP64
    form's after the same number of steps."""
    import porelb_gb300 as P
    K = 100
    reqs = requests()
    # the 16-bit pool holds two or three requests, the FP32 pool (half the
    # budget) the largest one
    budget = 3 * 48 ** 3 * 0.5 * 224
    mix, summ = served(reqs, K, "fp16dev", budget, handoff_share=0.5)
    assert summ["requests"] == len(reqs) and summ["handoffs"] >= 1
    by = {d["index"]: d for d in mix}
    for r in reqs[:3]:
        one, _ = served([r], K, "fp16dev", budget, handoff_share=0.5)
        a, m = one[0], by[r.index]
        assert a["status"] == m["status"] == 1
        assert a["handed_off"] and m["handed_off"]
        assert a["steps"] == m["steps"] and a["k_darcy"] == m["k_darcy"]
        sim = P.Simulation.packed(r.seed, r.edge, r.edge, r.edge, r.rmin, r.rmax,
                                  r.porosity, tau=r.tau, force=r.force,
                                  precision="fp64_exact")
        sim.init_dist_macro()
        sim.step(a["steps"])
        k64 = sim.permeability()[0]
        sim.close()
        err = abs(a["k_darcy"] - k64) / abs(k64)
        assert err <= 1e-3, f"request {r.index}: k {a['k_darcy']!r} vs FP64 {k64!r}, {err:.2e}"


def test_pool_launch_finish_overlaps_admission():
    """A sample admitted while an interval runs joins at the next launch and
    gives the same answer as when admitted between intervals."""
    K = 100
    r0, r1 = requests()[0], requests()[1]
    with Batch(200000, 4, "fp32", check_every=K) as b:
        s0 = b.add_packed(r0.seed, r0.edge, r0.edge, r0.edge, r0.rmin, r0.rmax,
                          r0.porosity, r0.tau, r0.force, tol=r0.tol)
        assert b.launch() == 1
        s1 = b.add_packed(r1.seed, r1.edge, r1.edge, r1.edge, r1.rmin, r1.rmax,
                          r1.porosity, r1.tau, r1.force, tol=r1.tol)
        b.finish()
        assert b.result(s1)["steps"] == 0
        while b.run(1):
            pass
        res = {0: b.result(s0), 1: b.result(s1)}
    for i, r in ((0, r0), (1, r1)):
        ref = alone(r, K)
        assert res[i]["steps"] == ref["steps"] and res[i]["k_darcy"] == ref["k_darcy"]


def test_transfer_fp16_to_fp32_keeps_state_and_history():
    """A parked FP16 sample moved into an FP32 pool continues from its
    state: its distributions convert exactly, and its step count carries
    over."""
    K = 100
    r = requests()[0]
    with Batch(200000, 4, "fp16dev", check_every=K) as h, \
            Batch(200000, 4, "fp32", check_every=K) as t:
        sid = h.add_packed(r.seed, r.edge, r.edge, r.edge, r.rmin, r.rmax, r.porosity,
                           r.tau, r.force, tol=1e-12, handoff_tol=1e-4)
        while h.run(1):
            pass
        res = h.result(sid)
        assert res["status"] == 4
        f16 = h.get_f(sid)
        nid = h.transfer(sid, t)
        h.release(sid)
        f32 = t.get_f(nid)
        # a scaled FP16 deviation is exact in FP32 (power-of-two scales)
        assert abs(f32 - f16).max() <= 1e-12
        assert t.result(nid)["steps"] == res["steps"]
        t.run(1)
        assert t.result(nid)["steps"] == res["steps"] + K
