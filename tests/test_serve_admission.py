"""Admission logic of the permeability server on the CPU, with a stand-in
pool: a request larger than the whole pool is rejected (it used to wait
forever), a request that does not fit now waits without its geometry being
built, and every other request is answered."""
from types import SimpleNamespace

from porelb_gb300.serve import Server


class FakePool:
    """The Batch calls the server makes, over a pool of `cap` nodes; a
    sample needs edge^3 * porosity nodes and converges after `life`
    intervals."""

    def __init__(self, cap, K=100, life=2):
        self.cap, self.check_every, self.life = cap, K, life
        self.used, self.live, self.finished = 0, {}, []
        self.adds = 0
        self.next = 0

    def info(self):
        return dict(capacity_nodes=self.cap)

    def free_nodes(self):
        free = self.cap - self.used
        return free, free

    def try_add_packed(self, seed, nx, ny, nz, rmin, rmax, phi, tau, force, tol,
                       handoff_tol=0.0):
        self.adds += 1
        n = int(nx * ny * nz * phi)
        if n > self.cap - self.used:
            return None
        sid = self.next
        self.next += 1
        self.used += n
        self.live[sid] = [n, self.life]
        return sid

    def num_nodes(self, sid):
        return self.live[sid][0]

    def launch(self):
        self.stepping = [sid for sid, v in self.live.items() if v[1] > 0]
        return len(self.stepping)

    def finish(self):
        for sid in getattr(self, "stepping", []):
            v = self.live[sid]
            v[1] -= 1
            if v[1] == 0:
                self.finished.append(sid)
        self.stepping = []

    def interval_ms(self):
        return 0.0

    def poll(self):
        out, self.finished = self.finished, []
        return out

    def result(self, sid):
        return dict(steps=self.check_every * self.life, k_darcy=1.0, status=1)

    def release(self, sid):
        self.used -= self.live.pop(sid)[0]


def req(i, edge, arrival=0.0, phi=0.5):
    return SimpleNamespace(index=i, edge=edge, arrival=arrival, seed=i, porosity=phi,
                           rmin=3.0, rmax=5.0, tau=0.8, force=1e-6, tol=1e-6)


def test_oversize_request_is_rejected_not_waiting_forever():
    pool = FakePool(cap=1024)
    srv = Server(0, batch=pool)
    reqs = [req(0, 20), req(1, 8), req(2, 9)]  # 4000 nodes > 1024; 256; 364
    done, summ = srv.serve(reqs, max_wall=30.0)
    assert summ["rejected"] == [0]
    assert sorted(d["index"] for d in done) == [1, 2]
    assert summ["wall_s"] < 5.0


def test_request_that_fits_only_an_empty_pool_waits_then_runs():
    pool = FakePool(cap=1024, life=3)
    srv = Server(0, batch=pool)
    # 9^3 * 0.5 = 364 nodes: two fit at once, the third waits for a slot
    reqs = [req(0, 9), req(1, 9), req(2, 9), req(3, 12)]  # 864 nodes: waits for all
    done, summ = srv.serve(reqs, max_wall=30.0)
    assert summ["rejected"] == []
    assert sorted(d["index"] for d in done) == [0, 1, 2, 3]
    # the waiting requests were not built at every interval
    assert pool.adds <= 8


def test_request_estimated_to_fit_but_larger_than_the_empty_pool():
    """The estimate is below the pool but the built geometry is not: the
    failed add into an empty pool rejects it."""
    pool = FakePool(cap=1024)
    srv = Server(0, batch=pool)
    # a stand-in whose built size is above its estimate: 0.9 * 1100 < 1024
    # passes the pre-check, but 1100 nodes do not fit
    reqs = [req(0, 10, phi=1.1)]
    done, summ = srv.serve(reqs, max_wall=30.0)
    assert summ["rejected"] == [0] and done == []
