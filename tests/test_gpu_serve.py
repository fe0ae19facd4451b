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
