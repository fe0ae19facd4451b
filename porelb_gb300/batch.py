"""Batched permeability solves: many porous samples in one device pool
(C ABI plb_batch_*, include/porelb_gpu.h).

Each sample runs porelb's step loop (porelb.c:426-437) with its own tau and
force; all samples advance together in one launch per lattice step, K steps
per CUDA-graph replay, and each is retired when the relative change of its
mean u_x over an interval drops below its tolerance.
"""
import ctypes

import numpy as np

from . import _lib
from .api import ORDERINGS, PRECISIONS, PorelbError, _check, _ptr

STATUS = {0: "running", 1: "converged", 2: "step limit", 3: "released",
          4: "parked"}
PARKED = 4


class Batch:
    def __init__(self, capacity_nodes, max_samples=1024, precision="fp32",
                 check_every=1000, keep_macros=False, device=0, cta_threads=None,
                 l2_prefetch=None, ordering=None, l2_groups=None):
        """cta_threads (128 or 256), l2_prefetch (True/False) and ordering
        ("morton" or "reference"): the batch step's launch and the samples'
        node order; None takes the launch tuner's cached choice for this
        form (porelb_gb300.tune.tune_pool), else the library default.
        l2_groups: L2 groups of the samples that fit a budget (each group
        steps its interval while it stays in L2): None or False = off,
        True = 60% of the L2, or a budget in KiB."""
        self._lib = _lib.load()
        self.precision = precision
        self.check_every = check_every
        if cta_threads is None or l2_prefetch is None or ordering is None:
            from . import tune
            choice = tune.best_pool(precision)
            if cta_threads is None:
                cta_threads = choice["cta_threads"]
            if l2_prefetch is None:
                l2_prefetch = choice["l2_prefetch"]
            if ordering is None:
                ordering = choice["ordering"]
        bp = _lib.BatchParams()
        bp.capacity_nodes = int(capacity_nodes)
        bp.max_samples = max_samples
        bp.precision = PRECISIONS[precision]
        bp.check_every = check_every
        bp.keep_macros = int(keep_macros)
        bp.device = device
        bp.cta_threads = int(cta_threads or 0)
        bp.l2_prefetch = 0 if l2_prefetch is None else (1 if l2_prefetch else -1)
        bp.ordering = ORDERINGS[ordering or "auto"]
        bp.l2_group_kb = (0 if l2_groups is None or l2_groups is False else
                          (-1 if l2_groups is True else int(l2_groups)))
        h = ctypes.c_void_p()
        _check(self._lib.plb_batch_create_ex(ctypes.byref(bp), ctypes.byref(h)),
               "plb_batch_create_ex")
        self._h = h
        self.launch_choice = dict(cta_threads=cta_threads, l2_prefetch=l2_prefetch,
                                  ordering=ordering)
        self.meta = {}

    @staticmethod
    def bytes_per_node(precision, keep_macros=False):
        return _lib.load().plb_batch_bytes_per_node(PRECISIONS[precision],
                                                    int(keep_macros))

    @staticmethod
    def _sp(tau, force, tol, max_steps, handoff_tol=0.0):
        sp = _lib.SampleParams()
        sp.tau, sp.force_x, sp.tol, sp.max_steps = tau, force, tol, max_steps
        sp.handoff_tol = handoff_tol
        return sp

    def add_flag(self, flag, nx, ny, nz, tau, force, tol=1e-7, max_steps=0,
                 handoff_tol=0.0):
        flag = np.ascontiguousarray(flag, dtype=np.uint8).reshape(-1)
        sid = ctypes.c_int(-1)
        sp = self._sp(tau, force, tol, max_steps, handoff_tol)
        _check(self._lib.plb_batch_add_flag(self._h, _ptr(flag), nx, ny, nz,
                                            ctypes.byref(sp),
                                            ctypes.byref(sid)),
               "plb_batch_add_flag")
        self.meta[sid.value] = dict(dims=(nx, ny, nz), tau=tau, force=force)
        return sid.value

    def add_packed(self, seed, nx, ny, nz, rmin, rmax, porosity, tau, force,
                   tol=1e-7, max_steps=0, handoff_tol=0.0):
        sid = ctypes.c_int(-1)
        ns = ctypes.c_int(0)
        phi = ctypes.c_double(0.0)
        sp = self._sp(tau, force, tol, max_steps, handoff_tol)
        _check(self._lib.plb_batch_add_packed(
            self._h, ctypes.c_uint64(seed), nx, ny, nz, rmin, rmax, porosity,
            ctypes.byref(sp), ctypes.byref(sid), ctypes.byref(ns),
            ctypes.byref(phi)), "plb_batch_add_packed")
        self.meta[sid.value] = dict(dims=(nx, ny, nz), tau=tau, force=force,
                                    spheres=ns.value, porosity=phi.value)
        return sid.value

    def try_add_packed(self, *args, **kw):
        """add_packed, or None when the pool has no room (PLB_ERR_NOMEM)."""
        try:
            return self.add_packed(*args, **kw)
        except PorelbError as e:
            if e.status == _lib.ERR_NOMEM:
                return None
            raise

    def launch(self):
        """Start one interval without waiting; returns the samples it steps
        (0: nothing launched)."""
        act = ctypes.c_int(0)
        _check(self._lib.plb_batch_launch(self._h, ctypes.byref(act)), "plb_batch_launch")
        return act.value

    def finish(self):
        """Wait for the interval in flight and check its samples."""
        _check(self._lib.plb_batch_finish(self._h), "plb_batch_finish")

    def interval_ms(self):
        """Device time of the last completed interval (ms)."""
        ms = ctypes.c_float(0.0)
        _check(self._lib.plb_batch_interval_ms(self._h, ctypes.byref(ms)), "interval_ms")
        return ms.value

    def transfer(self, sid, dst):
        """Move parked sample sid into pool dst (converting its storage);
        returns its id there.  The caller releases it here."""
        nid = ctypes.c_int(-1)
        _check(self._lib.plb_batch_transfer(self._h, sid, dst._h, ctypes.byref(nid)),
               "plb_batch_transfer")
        return nid.value

    def try_transfer(self, sid, dst):
        """transfer, or None when dst has no room (PLB_ERR_NOMEM)."""
        try:
            return self.transfer(sid, dst)
        except PorelbError as e:
            if e.status == _lib.ERR_NOMEM:
                return None
            raise

    def run(self, intervals=1):
        act = ctypes.c_int(0)
        _check(self._lib.plb_batch_run(self._h, intervals, ctypes.byref(act)),
               "plb_batch_run")
        return act.value

    def poll(self, max_ids=4096):
        ids = (ctypes.c_int * max_ids)()
        c = ctypes.c_int(0)
        _check(self._lib.plb_batch_poll(self._h, ids, max_ids,
                                        ctypes.byref(c)), "plb_batch_poll")
        return list(ids[:c.value])

    def result(self, sid):
        k, u = ctypes.c_double(), ctypes.c_double()
        st, status = ctypes.c_longlong(), ctypes.c_int()
        _check(self._lib.plb_batch_result(self._h, sid, ctypes.byref(k),
                                          ctypes.byref(u), ctypes.byref(st),
                                          ctypes.byref(status)), "result")
        return dict(k_darcy=k.value, mean_ux=u.value, steps=st.value,
                    status=status.value)

    def release(self, sid):
        _check(self._lib.plb_batch_release(self._h, sid), "release")
        self.meta.pop(sid, None)

    def num_nodes(self, sid):
        n = ctypes.c_int(0)
        _check(self._lib.plb_batch_sample_nodes(self._h, sid, ctypes.byref(n)),
               "sample_nodes")
        return n.value

    def get_f(self, sid):
        out = np.empty(self.num_nodes(sid) * _lib.Q)
        _check(self._lib.plb_batch_get_f(self._h, sid, _ptr(out)), "get_f")
        return out

    def macros(self, sid):
        n = self.num_nodes(sid)
        out = np.empty((4, n))
        _check(self._lib.plb_batch_get_macros(self._h, sid, _ptr(out[0]),
                                              _ptr(out[1]), _ptr(out[2]),
                                              _ptr(out[3])), "get_macros")
        return out

    def free_nodes(self):
        """(largest free block range, all free ranges) in nodes; the largest
        range is 0 when no sample slot is free."""
        big, tot = ctypes.c_longlong(), ctypes.c_longlong()
        _check(self._lib.plb_batch_free_nodes(self._h, ctypes.byref(big),
                                              ctypes.byref(tot)), "free_nodes")
        return big.value, tot.value

    def info(self):
        t, used, cap = (ctypes.c_longlong() for _ in range(3))
        act = ctypes.c_int()
        b = ctypes.c_size_t()
        _check(self._lib.plb_batch_info(self._h, ctypes.byref(t),
                                        ctypes.byref(act), ctypes.byref(used),
                                        ctypes.byref(cap), ctypes.byref(b)),
               "info")
        return dict(t=t.value, active=act.value, used_nodes=used.value,
                    capacity_nodes=cap.value, device_bytes=b.value)

    @property
    def stream(self):
        return self._lib.plb_batch_stream(self._h)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.plb_batch_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
