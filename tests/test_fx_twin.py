"""The integer-pipe FP64 collision (porelb_gb300/csrc/plb_fx.h) built for the
CPU (tests/native/fx_twin.cpp): checked against the oracle here, and bit for
bit against the GPU kernel in the GPU suite."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import oracle_py as O
import porelb_gb300 as P

from helpers import max_rel, noise_flag, pack_flag

HERE = os.path.dirname(os.path.abspath(__file__))
W = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)


@pytest.fixture(scope="module")
def twin(tmp_path_factory):
    out = tmp_path_factory.mktemp("fx") / "fx_twin.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC",
                    "-shared", "-o", str(out),
                    os.path.join(HERE, "native", "fx_twin.cpp")], check=True)
    lib = ctypes.CDLL(str(out))
    v = ctypes.c_void_p
    lib.fx_twin_step.restype = ctypes.c_int
    lib.fx_twin_step.argtypes = [v, v, ctypes.c_int, v, v, v, v,
                                 ctypes.c_double, ctypes.c_double, ctypes.c_int]
    return lib


def twin_run(lib, V, vs, tau, force, steps):
    kind, src = O.pull_table(V, vs)
    N = len(V)
    f0 = np.tile(W, N)
    f1, fo = f0.copy(), f0.copy()
    mac = np.zeros((4, N))
    p = lambda a: ctypes.c_void_p(a.ctypes.data)  # noqa: E731
    bad = 0
    for it in range(steps):
        r = lib.fx_twin_step(p(kind), p(src), N, p(f0), p(f1), p(fo), p(mac),
                             tau, force, it)
        assert r >= 0
        bad += r
        f0, fo = fo, f0
    return f0, mac, bad


@pytest.mark.parametrize("case", [((24, 20, 16), 3, 3.0, 5.0, 0.45, 0.8, 1e-4, 150),
                                  ((16, 16, 16), 5, 3.0, 3.0, 0.4, 0.8, 1e-3, 200)])
def test_twin_within_1e12_of_oracle(twin, case):
    dims, seed, rmin, rmax, phi, tau, force, steps = case
    flag = pack_flag(dims, seed, rmin, rmax, phi)
    V, vs = P.build_table(flag, *dims, 1)
    f, mac, bad = twin_run(twin, V, vs, tau, force, steps)
    assert bad == 0
    s = O.OracleSim(V, *dims, vs, tau, force)
    s.init()
    assert s.run(steps)[0] == 0
    assert max_rel(f, s.f0()) <= 1e-12
    assert max_rel(mac[0], s.macros()[0]) <= 1e-13


def test_twin_flags_out_of_range_nodes(twin):
    """A node whose populations leave the fixed-point range is reported for
    the native-FP64 fallback instead of being computed wrongly."""
    dims = (6, 6, 6)
    flag = noise_flag(dims, 0.2, 4)
    V, vs = P.build_table(flag, *dims, 1)
    kind, src = O.pull_table(V, vs)
    N = len(V)
    f0 = np.tile(W, N)
    f0[5 * 19] = 1e-3  # rest population below the fixed-point bound 2^-8
    f1, fo, mac = f0.copy(), f0.copy(), np.zeros((4, N))
    p = lambda a: ctypes.c_void_p(a.ctypes.data)  # noqa: E731
    r = twin.fx_twin_step(p(kind), p(src), N, p(f0), p(f1), p(fo), p(mac),
                          0.8, 1e-4, 1)
    assert r >= 1
