"""Permeability-solve server with continuous batching.

Requests (geometry seed and size, porosity, sphere radius, tau, force,
tolerance) arrive over time.  The server keeps device node pools
(``Batch``) sized from an HBM budget.  Each round it launches one interval
(K lattice steps, one CUDA-graph replay) on every pool that has work and,
while those run, admits waiting requests that fit (first come first served,
smaller requests may pass a head that does not fit): their geometry and node
table are built on the pool's admission stream, concurrently with the
interval, and they join at the next launch.  Then it waits for the
intervals, answers converged requests and backfills their blocks.  Work of
requests that arrive while others run overlaps on the device with theirs.

Storage forms:
* one pool in FP32 (default), FP64, FP16 or BF16 deviations;
* ``"fp16dev"`` with ``handoff_tol``: requests start in a pool of scaled
  FP16 deviations (148 B per lattice update against FP32's 224) and, once
  the relative change of <u_x> over an interval falls below handoff_tol,
  move with their state and history into an FP32 pool, where the
  steady-state test finishes at the request's own tolerance.  FP16
  storage alone cannot finish at tight tolerances: once a sample is
  steady, its <u_x> keeps wandering by 2e-7 to 5e-7 of itself from check
  to check (FP32: below 4e-9), so a 1e-7 test passes only by chance.

Latency of a request = completion time - arrival time (wall clock).
"""
import time

import numpy as np

from .batch import PARKED, Batch

# a request whose estimated fluid nodes exceed the free room by more than
# this factor is not tried: the generator stops at or just below the target
# porosity, so edge^3 * porosity over-estimates its nodes by a few percent
_EST_SLACK = 0.9

BLOCK = 256  # pool block (nodes)


def _blocks_nodes(n):
    return -(-int(n) // BLOCK) * BLOCK


class Server:
    def __init__(self, hbm_budget_bytes, precision="fp32", check_every=250,
                 max_samples=4096, device=0, lookahead=64, batch=None,
                 handoff_tol=None, handoff_share=0.35, tuned=True):
        """precision: the storage form requests start in.  handoff_tol (only
        with "fp16dev"; default 1e-5): move a request to an FP32 pool once
        its relative change is below it; handoff_share: the FP32 pool's
        share of the budget.  tuned: time the pool launch candidates of
        the forms first (tune.ensure_pool, about a second per form, once per
        process) and build the pools with the fastest.  batch: a ready pool
        (tests)."""
        self.precision = precision
        self.lookahead = lookahead
        if precision == "fp16dev" and handoff_tol is None:
            handoff_tol = 1e-5
        self.handoff_tol = handoff_tol if precision == "fp16dev" else None
        self.tail = None
        if batch is None and tuned:
            from . import tune
            tune.ensure_pool(precision, device)
            if self.handoff_tol:
                tune.ensure_pool("fp32", device)
        if batch is None:
            share = handoff_share if self.handoff_tol else 0.0
            cap = int(hbm_budget_bytes * (1 - share) // Batch.bytes_per_node(precision))
            batch = Batch(cap, max_samples, precision, check_every, device=device)
            if self.handoff_tol:
                cap32 = int(hbm_budget_bytes * share // Batch.bytes_per_node("fp32"))
                self.tail = Batch(cap32, max_samples, "fp32", check_every, device=device)
        self.batch = batch
        self.capacity = int(batch.info()["capacity_nodes"])
        self.pool_launch = getattr(batch, "launch_choice", None)

    @staticmethod
    def estimated_nodes(r):
        """Fluid nodes a request will have, estimated before its geometry is
        built (edge^3 * porosity)."""
        return r.edge ** 3 * r.porosity

    def close(self):
        self.batch.close()
        if self.tail is not None:
            self.tail.close()

    def pools(self):
        return [self.batch] + ([self.tail] if self.tail is not None else [])

    def _answer(self, done, v, res, t0, time_scale, status=None, handed_off=False):
        end = time.perf_counter() - t0
        r = v["req"]
        done.append(dict(index=r.index, edge=r.edge, nodes=v["nodes"],
                         arrival=r.arrival * time_scale, admitted=v["admitted"],
                         finished=end, latency=end - r.arrival * time_scale,
                         steps=res["steps"], k_darcy=res["k_darcy"],
                         status=res["status"] if status is None else status,
                         tau=r.tau, tol=r.tol, handed_off=handed_off,
                         handoff_steps=v.get("handoff_steps")))

    def serve(self, requests, time_scale=1.0, max_wall=None):
        """Serve requests (objects with .arrival in seconds, .edge, .seed,
        .porosity, .rmin, .rmax, .tau, .force, .tol) in real time.  Returns a
        list of per-request records and a summary."""
        pending = sorted(requests, key=lambda r: r.arrival)
        waiting = []
        live = {}        # (pool index, sid) -> record
        parked = []      # sids parked in the first pool, waiting for room
        done = []
        rejected = []
        t0 = time.perf_counter()
        node_steps = 0
        rounds = 0
        t_admit = t_wait = busy_ms = 0.0
        handoffs = 0
        pools = self.pools()
        K = self.batch.check_every
        head = self.batch
        while pending or waiting or live:
            now = time.perf_counter() - t0
            if max_wall is not None and now > max_wall:
                break
            while pending and pending[0].arrival * time_scale <= now:
                waiting.append(pending.pop(0))
            # one interval on every pool with work, asynchronously
            stepping = [p.launch() for p in pools]
            node_steps += sum(v["nodes"] for (pi, _), v in live.items()
                              if stepping[pi] and not v.get("parked")) * K
            # admissions while the intervals run
            ta = time.perf_counter()
            admitted = []
            room = head.free_nodes()[0]
            for r in waiting[: self.lookahead]:
                est = _EST_SLACK * self.estimated_nodes(r)
                if est > self.capacity:
                    # larger than the whole pool: it can never be admitted
                    rejected.append(self._reject(r, t0, time_scale))
                    admitted.append(r)
                    continue
                if live and _blocks_nodes(est) > room:
                    continue  # no room now: skip building its geometry
                sid = head.try_add_packed(
                    r.seed, r.edge, r.edge, r.edge, r.rmin, r.rmax, r.porosity,
                    r.tau, r.force, tol=r.tol,
                    handoff_tol=self.handoff_tol or 0.0)
                if sid is not None:
                    live[(0, sid)] = dict(req=r, admitted=time.perf_counter() - t0,
                                          nodes=head.num_nodes(sid))
                    admitted.append(r)
                    room = head.free_nodes()[0]
                elif not live and not any(stepping):
                    # it did not fit into the empty pool: it never will
                    rejected.append(self._reject(r, t0, time_scale))
                    admitted.append(r)
                else:
                    room = head.free_nodes()[0]
            for r in admitted:
                waiting.remove(r)
            t_admit += time.perf_counter() - ta
            if not any(stepping):
                if not live and pending:
                    time.sleep(max(0.0, pending[0].arrival * time_scale -
                                   (time.perf_counter() - t0)))
                if not parked:
                    continue
            tw = time.perf_counter()
            for p in pools:
                p.finish()
            t_wait += time.perf_counter() - tw
            busy_ms += max(p.interval_ms() if s else 0.0 for p, s in zip(pools, stepping))
            rounds += 1
            for pi, p in enumerate(pools):
                for sid in p.poll():
                    res = p.result(sid)
                    if res["status"] == PARKED:
                        live[(pi, sid)]["parked"] = True
                        live[(pi, sid)]["handoff_steps"] = res["steps"]
                        parked.append(sid)
                        continue
                    self._answer(done, live.pop((pi, sid)), res, t0, time_scale,
                                 handed_off=pi == 1)
                    p.release(sid)
            # parked 16-bit samples move to the FP32 pool when it has room
            still = []
            tail_busy = any(pi == 1 for pi, _ in live)
            for sid in parked:
                nid = self.batch.try_transfer(sid, self.tail)
                if nid is None and not tail_busy:
                    # larger than the whole FP32 pool: answered at the
                    # handoff tolerance, marked as such (PLB_ERR_NOMEM)
                    self._answer(done, live.pop((0, sid)), self.batch.result(sid), t0,
                                 time_scale, status=-5)
                    self.batch.release(sid)
                    continue
                if nid is None:
                    still.append(sid)
                    continue
                v = live.pop((0, sid))
                v.pop("parked", None)
                live[(1, nid)] = v
                self.batch.release(sid)
                handoffs += 1
            parked = still
        wall = time.perf_counter() - t0
        lat = np.array([d["latency"] for d in done]) if done else np.zeros(1)
        summary = dict(requests=len(done), wall_s=wall,
                       solves_per_s=len(done) / wall if wall > 0 else 0.0,
                       p50_latency_s=float(np.percentile(lat, 50)),
                       p99_latency_s=float(np.percentile(lat, 99)),
                       fluid_mlups=node_steps / wall / 1e6 if wall > 0 else 0.0,
                       fluid_mlups_busy=(node_steps / (busy_ms / 1e3) / 1e6
                                         if busy_ms > 0 else None),
                       intervals=rounds, capacity_nodes=self.capacity,
                       admit_s=t_admit, wait_s=t_wait,
                       gpu_busy_s=busy_ms / 1e3,
                       gpu_idle_frac=max(0.0, 1.0 - busy_ms / 1e3 / wall) if wall > 0 else None,
                       handoffs=handoffs, handoff_tol=self.handoff_tol,
                       pool_launch=self.pool_launch,
                       precision=self.precision, check_every=K,
                       rejected=[d["index"] for d in rejected])
        return done, summary

    @staticmethod
    def _reject(r, t0, time_scale):
        """Record of a request that cannot fit into the pool even when the
        pool is empty (status PLB_ERR_NOMEM)."""
        return dict(index=r.index, edge=r.edge, status=-5,
                    arrival=r.arrival * time_scale,
                    finished=time.perf_counter() - t0)
