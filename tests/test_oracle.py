"""The oracle pinned to the reference.

* against the committed golden fixtures, which the compiled reference wrote
  (tests/golden/make_golden.py): always;
* against the reference compiled from its own sources (oracle/_ref), live,
  on fresh random cases: when the reference tree is present.
"""
import hashlib
import os
import tempfile

import numpy as np
import pytest

import oracle_py as O
import porelb_gb300 as P

from helpers import (golden_arrays, golden_meta, noise_flag, pack_flag,
                     table_fields)

META = golden_meta()
SMALL = ["noise_10x8x6_p1", "noise_8x6x8_p2", "tiny_2x2x2_p1"]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("name", SMALL)
def test_oracle_table_matches_golden(name):
    m, g = META[name], golden_arrays(name)
    V, vs = O.build_v(g["flag"], *m["dims"], m["num_p"])
    xyz, t, ident, pid = table_fields(V)
    assert list(vs) == m["v_sub_start"]
    assert (xyz == g["xyz"]).all() and (t == g["type"]).all()
    assert (ident == g["node_id"]).all() and (pid == g["node_pid"]).all()
    # the product's host builder gives the same bytes as the oracle's
    Vp, vsp = P.build_table(g["flag"], *m["dims"], m["num_p"])
    assert Vp.tobytes() == V.tobytes() and (vsp == vs).all()


@pytest.mark.parametrize("name", SMALL)
def test_oracle_solver_matches_golden(name):
    m, g = META[name], golden_arrays(name)
    V, vs = P.build_table(g["flag"], *m["dims"], m["num_p"])
    s = O.OracleSim(V, *m["dims"], vs, m["tau"], m["force"])
    s.init()
    st, _, _ = s.run(m["steps"], threads=m["num_p"])
    assert st == 0
    assert (s.f0() == g["f0"]).all()
    assert (s.f1() == g["f1"]).all()
    assert (s.macros() == g["macros"]).all()
    f0, f1, mac = O.pull_run(V, vs, m["tau"], m["force"], m["steps"],
                             remote_wins=m["num_p"] > 1)
    assert (f0 == g["f0"]).all() and (f1 == g["f1"]).all()
    assert (mac == g["macros"]).all()


def test_oracle_c1_1000_steps_matches_golden_hash():
    """Plain configuration (64^3, seed 0, R 6, porosity 0.40, tau 1, F 1e-6):
    the oracle's f after 1000 steps is the reference's, bit for bit."""
    m = META["c1_64_seed0"]
    geo = m["geometry"]
    flag, ns, phi = P.sphere_pack(geo["seed"], *m["dims"], geo["rmin"],
                                  geo["rmax"], geo["porosity"])
    assert sha(flag) == geo["sha_flag"] and ns == geo["spheres"]
    V, vs = P.build_table(flag, *m["dims"], 1)
    xyz, t, ident, pid = table_fields(V)
    assert sha(np.concatenate([xyz.ravel().view(np.uint8), t.ravel(),
                               ident.ravel().view(np.uint8),
                               pid.ravel().view(np.uint8)])) == m["sha_table"]
    s = O.OracleSim(V, *m["dims"], vs, m["tau"], m["force"])
    s.init()
    assert s.run(m["steps"])[0] == 0
    assert sha(s.f0()) == m["sha_f0"]
    assert sha(s.macros()) == m["sha_macros"]


def test_oracle_multirank_matches_golden_hash():
    m = META["c1_64_seed0_p4_100"]
    flag = pack_flag(m["dims"], 0, 6.0, 6.0, 0.40)
    V, vs = P.build_table(flag, *m["dims"], m["num_p"])
    s = O.OracleSim(V, *m["dims"], vs, m["tau"], m["force"])
    s.init()
    assert s.run(m["steps"], threads=4)[0] == 0
    assert sha(s.f0()) == m["sha_f0"]
    assert sha(s.macros()) == m["sha_macros"]
    g = golden_arrays(m["name"])
    assert (s.f0().reshape(-1, 19)[g["sample_idx"]] == g["sample_f0"]).all()


def test_pull_form_equals_push_form_on_noise():
    for seed, p_solid, dims, num_p in [(1, 0.2, (7, 9, 6), 1),
                                       (2, 0.5, (8, 8, 8), 2),
                                       (3, 0.4, (5, 3, 12), 4),
                                       (4, 0.0, (3, 3, 3), 1)]:
        flag = noise_flag(dims, p_solid, seed)
        V, vs = P.build_table(flag, *dims, num_p)
        s = O.OracleSim(V, *dims, vs, 0.75, 2e-3)
        s.init()
        assert s.run(12, threads=num_p)[0] == 0
        f0, f1, mac = O.pull_run(V, vs, 0.75, 2e-3, 12, remote_wins=num_p > 1)
        assert (f0 == s.f0()).all() and (f1 == s.f1()).all()
        assert (mac == s.macros()).all()


def test_oracle_density_guard():
    dims = (8, 8, 8)
    flag = noise_flag(dims, 0.3, 21)
    V, vs = P.build_table(flag, *dims, 1)
    s = O.OracleSim(V, *dims, vs, 0.505, 0.2)
    s.init()
    st, bad_it, bad_node = s.run(500)
    assert st == -6 and bad_it > 0 and 0 <= bad_node < len(V)


needs_ref = pytest.mark.skipif(not O.ref_available(),
                               reason="reference tree not compiled here")


@needs_ref
@pytest.mark.parametrize("case", [((11, 7, 9), 0.35, 31, 1), ((10, 6, 8), 0.3, 32, 2),
                                  ((6, 6, 12), 0.45, 33, 4), ((4, 1, 3), 0.2, 34, 1),
                                  ((1, 1, 1), 0.0, 35, 1)])
def test_live_reference_table(case):
    dims, p_solid, seed, num_p = case
    flag = noise_flag(dims, p_solid, seed)
    Vr, vr = O.ref_build_v(flag, *dims, num_p)
    Vp, vp = P.build_table(flag, *dims, num_p)
    assert (vr == vp).all()
    for a, b in zip(table_fields(Vr), table_fields(Vp)):
        assert (a == b).all()


@needs_ref
@pytest.mark.parametrize("case", [((12, 9, 8), 0.3, 41, 1, 0.8, 1e-3, 25),
                                  ((8, 8, 8), 0.4, 42, 2, 1.0, 1e-4, 25),
                                  ((9, 5, 12), 0.25, 43, 3, 0.6, 5e-4, 20)])
def test_live_reference_solver(case):
    dims, p_solid, seed, num_p, tau, force, steps = case
    flag = noise_flag(dims, p_solid, seed)
    with tempfile.TemporaryDirectory() as d:
        O.ref_write_vbin(flag, *dims, num_p, os.path.join(d, "V.bin"))
        f0r, f1r, macr, _ = O.ref_run(d, num_p, steps, tau, force)
        V, vs, _ = P.read_vbin(os.path.join(d, "V.bin"))
    s = O.OracleSim(V, *dims, vs, tau, force)
    s.init()
    assert s.run(steps, threads=num_p)[0] == 0
    assert (s.f0() == f0r).all() and (s.f1() == f1r).all()
    assert (s.macros() == macr).all()


@needs_ref
def test_live_reference_dump_schedule(tmp_path):
    """main dumps at it % 1000 == 0 (state after it+1 steps) and once more at
    the end tagged it_max (porelb.c:436,440)."""
    dims = (6, 6, 6)
    flag = noise_flag(dims, 0.3, 51)
    O.ref_write_vbin(flag, *dims, 1, str(tmp_path / "V.bin"))
    O.ref_run(str(tmp_path), 1, 12, 0.8, 1e-3, save=True, save_every=5)
    names = sorted(f for f in os.listdir(tmp_path) if f.startswith("part_"))
    assert names == ["part_000_0000000.bin", "part_000_0000005.bin",
                     "part_000_0000010.bin", "part_000_0000012.bin"]
    V, vs, _ = P.read_vbin(tmp_path / "V.bin")
    s = O.OracleSim(V, *dims, vs, 0.8, 1e-3)
    s.init()
    s.run(1)
    got = np.fromfile(tmp_path / "part_000_0000000.bin", np.float64).reshape(4, -1)
    assert (got == s.macros()).all()


@pytest.mark.parametrize("case", [
    (0, 64, 64, 64, 6.0, 6.0, 0.40),      # the 64^3 plain configuration
    (1, 256, 256, 256, 4.0, 10.0, 0.35),  # the 256^3 plain FP64 workload
    (7, 20, 9, 13, 3.0, 11.0, 0.30),      # spheres wider than the box
])
def test_oracle_sphere_pack_equals_library(case):
    """The oracle's own generator (which the CPU baseline builds its input
    with) gives the library's flag field byte for byte."""
    seed, nx, ny, nz, rmin, rmax, phi = case
    fo, no, po = O.sphere_pack(seed, nx, ny, nz, rmin, rmax, phi)
    fp, npk, pp = P.sphere_pack(seed, nx, ny, nz, rmin, rmax, phi)
    assert no == npk and po == pp
    assert np.array_equal(fo, fp)
    assert po <= phi and 0 < fo.sum() < fo.size
