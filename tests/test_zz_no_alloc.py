"""plb_reduce_noalloc: the macro reduction for callers that cannot let a
library allocate device memory (a framework owning all device memory through
its own pool and budget, a serving loop admitting work against a fixed HBM
budget, code that must not synchronise the device).  Checked against the
allocating path, plb_reduce, on two calls in a row.  Named so that pytest
collects it last."""
import ctypes

import numpy as np
import pytest

import porelb_gb300 as P
from porelb_gb300 import _lib

pytestmark = pytest.mark.gpu


def test_reduce_noalloc_matches_plb_reduce():
    torch = pytest.importorskip("torch")
    dims = (40, 36, 32)
    flag, _, _ = P.sphere_pack(17, *dims, 3.0, 5.0, 0.4)
    sim = P.Simulation.from_flag(flag, *dims, tau=0.9, force=1e-4,
                                 precision="fp64")
    sim.init_dist_macro()
    sim.step(50)
    sum_ux, mass = sim.reduce()
    mac = sim.macros()
    sim.close()
    lib = _lib.load()
    ux = torch.tensor(mac[1], dtype=torch.float64, device="cuda")
    rho = torch.tensor(mac[0], dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    for call in range(2):
        out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
        st = lib.plb_reduce_noalloc(ctypes.c_void_p(ux.data_ptr()),
                                    ctypes.c_void_p(rho.data_ptr()),
                                    ux.numel(), ctypes.c_void_p(out.data_ptr()),
                                    ctypes.c_void_p(stream.cuda_stream))
        assert st == _lib.OK, call
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert abs(got[0] - sum_ux) <= 1e-12 * abs(sum_ux), (call, got[0], sum_ux)
        assert abs(got[1] - mass) <= 1e-12 * abs(mass), (call, got[1], mass)


def test_reduce_noalloc_rejects_oversize():
    lib = _lib.load()
    dummy = ctypes.c_void_p(16)
    st = lib.plb_reduce_noalloc(dummy, dummy, _lib.REDUCE_NOALLOC_MAX_NODES + 1,
                                dummy, None)
    assert st == _lib.ERR_ARG
