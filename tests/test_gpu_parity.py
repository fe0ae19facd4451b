"""Parity of the CUDA path with the reference (golden fixtures written by
the compiled reference) and with the oracle, through the C ABI.

Tolerances: FP64_EXACT is bit-exact (== on every double); FP64 (FMA form) is
within 1e-12 relative on f and 1e-10 relative on the permeability."""
import hashlib
import os

import numpy as np
import pytest

import oracle_py as O
import porelb_gb300 as P
from porelb_gb300 import _lib

from helpers import golden_arrays, golden_meta, max_rel, noise_flag, pack_flag

pytestmark = pytest.mark.gpu
META = golden_meta()


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def gpu_run(V, dims, vs, tau, force, steps, precision="fp64_exact",
            ordering="morton", halo="auto", chunks=None):
    sim = P.Simulation(V, *dims, vs, tau=tau, force=force,
                       precision=precision, ordering=ordering, halo=halo)
    sim.init_dist_macro()
    if chunks is None:
        sim.step(steps)
    else:
        for c in chunks:
            sim.step(c)
    return sim


@pytest.mark.parametrize("ordering", ["morton", "reference"])
@pytest.mark.parametrize("name", ["noise_10x8x6_p1", "noise_8x6x8_p2",
                                  "tiny_2x2x2_p1"])
def test_exact_matches_golden(name, ordering):
    m, g = META[name], golden_arrays(name)
    V, vs = P.build_table(g["flag"], *m["dims"], m["num_p"])
    with gpu_run(V, m["dims"], vs, m["tau"], m["force"], m["steps"],
                 ordering=ordering) as sim:
        assert (sim.get_f() == g["f0"]).all()
        assert (sim.macros() == g["macros"]).all()


def test_exact_c1_1000_steps_hash_and_dumps(tmp_path):
    """64^3 sphere pack, seed 0, tau 1, F 1e-6, 1000 steps: f, macros and the
    part files of the reference's dump schedule are the reference's bytes."""
    m = META["c1_64_seed0"]
    geo = m["geometry"]
    flag = pack_flag(m["dims"], geo["seed"], geo["rmin"], geo["rmax"],
                     geo["porosity"])
    assert sha(flag) == geo["sha_flag"]
    V, vs = P.build_table(flag, *m["dims"], 1)
    sim = P.Simulation(V, *m["dims"], vs, tau=m["tau"], force=m["force"])
    sim.init_dist_macro()
    sim.step(1)
    sim.save_data(str(tmp_path), tag=0)
    sim.step(999)
    sim.save_data(str(tmp_path), tag=1000)
    assert sha(sim.get_f()) == m["sha_f0"]
    assert sha(sim.macros()) == m["sha_macros"]
    for fn, h in m["parts"].items():
        with open(tmp_path / fn, "rb") as fh:
            assert hashlib.sha256(fh.read()).hexdigest() == h, fn
    kd, _ = sim.permeability()
    assert abs(kd - m["k_darcy"]) <= 1e-10 * abs(m["k_darcy"])
    su, mass = sim.reduce()
    assert abs(mass - m["mass"]) <= 1e-12 * m["mass"]
    sim.close()


def test_exact_multirank_hash():
    m = META["c1_64_seed0_p4_100"]
    flag = pack_flag(m["dims"], 0, 6.0, 6.0, 0.40)
    V, vs = P.build_table(flag, *m["dims"], m["num_p"])
    with gpu_run(V, m["dims"], vs, m["tau"], m["force"], m["steps"]) as sim:
        assert sha(sim.get_f()) == m["sha_f0"]
        assert sha(sim.macros()) == m["sha_macros"]


CASES = [((7, 9, 6), 0.2, 1, 1), ((8, 8, 8), 0.5, 2, 2), ((5, 3, 12), 0.4, 3, 4),
         ((3, 3, 3), 0.0, 4, 1), ((1, 1, 2), 0.0, 5, 1), ((2, 2, 2), 0.3, 6, 1),
         ((13, 1, 17), 0.3, 7, 1), ((33, 17, 9), 0.45, 8, 3)]


@pytest.mark.parametrize("case", CASES)
def test_exact_matches_oracle_on_noise(case):
    dims, p_solid, seed, num_p = case
    flag = noise_flag(dims, p_solid, seed)
    V, vs = P.build_table(flag, *dims, num_p)
    s = O.OracleSim(V, *dims, vs, 0.7, 3e-3)
    s.init()
    assert s.run(15, threads=num_p)[0] == 0
    with gpu_run(V, dims, vs, 0.7, 3e-3, 15) as sim:
        assert (sim.get_f() == s.f0()).all()
        assert (sim.macros() == s.macros()).all()


def test_single_rank_semantics_on_multirank_table():
    """halo='single' on a 3-slab table gives the one-rank result."""
    dims = (10, 8, 9)
    flag = noise_flag(dims, 0.35, 12)
    V1, vs1 = P.build_table(flag, *dims, 1)
    V3, vs3 = P.build_table(flag, *dims, 3)
    with gpu_run(V1, dims, vs1, 0.9, 1e-3, 20) as a, \
            gpu_run(V3, dims, vs3, 0.9, 1e-3, 20, halo="single") as b:
        assert (a.get_f() == b.get_f()).all()


def test_chunked_steps_equal_one_call():
    dims = (12, 10, 8)
    flag = noise_flag(dims, 0.3, 13)
    V, vs = P.build_table(flag, *dims, 1)
    with gpu_run(V, dims, vs, 0.8, 1e-3, 17) as a, \
            gpu_run(V, dims, vs, 0.8, 1e-3, 17, chunks=[1, 5, 11]) as b:
        assert (a.get_f() == b.get_f()).all()
        assert (a.macros() == b.macros()).all()


@pytest.mark.parametrize("precision", ["fp64", "fp64_fma"])
def test_fp64_forms_within_1e12_of_reference_c1(precision):
    """f within 1e-12 relative and k within 1e-10 relative of the reference
    after 1000 steps of the 64^3 plain configuration."""
    m = META["c1_64_seed0"]
    flag = pack_flag(m["dims"], 0, 6.0, 6.0, 0.40)
    V, vs = P.build_table(flag, *m["dims"], 1)
    ref = gpu_run(V, m["dims"], vs, m["tau"], m["force"], m["steps"])
    fast = gpu_run(V, m["dims"], vs, m["tau"], m["force"], m["steps"],
                   precision=precision)
    assert sha(ref.get_f()) == m["sha_f0"]
    assert max_rel(fast.get_f(), ref.get_f()) <= 1e-12
    kd = fast.permeability()[0]
    assert abs(kd - m["k_darcy"]) <= 1e-10 * abs(m["k_darcy"])
    assert max_rel(fast.macros()[0], ref.macros()[0]) <= 1e-12
    ref.close()
    fast.close()


@pytest.mark.parametrize("case", [((32, 32, 32), 5, 4.0, 4.0, 0.4, 0.8, 1e-3, 300),
                                  ((24, 20, 16), 6, 2.0, 5.0, 0.3, 0.6, 1e-4, 200)])
def test_fp64_fixed_point_within_1e12_high_velocity(case):
    dims, seed, rmin, rmax, phi, tau, force, steps = case
    flag = pack_flag(dims, seed, rmin, rmax, phi)
    V, vs = P.build_table(flag, *dims, 1)
    s = O.OracleSim(V, *dims, vs, tau, force)
    s.init()
    assert s.run(steps)[0] == 0
    with gpu_run(V, dims, vs, tau, force, steps, precision="fp64") as sim:
        assert max_rel(sim.get_f(), s.f0()) <= 1e-12
        assert max_rel(sim.macros()[0], s.macros()[0]) <= 1e-12


def oracle_pull_from(V, vs, f0, tau, force, it_begin, steps):
    """The oracle's pull-form restatement stepped from the state f0 (AoS,
    reference order); slots no push or bounce writes keep w_j, as the
    reference's f1 does from its initialisation (porelb.c:224-238)."""
    import ctypes
    lib = O.orc()
    kind, src = O.pull_table(V, vs)
    N = len(V)
    f0 = np.ascontiguousarray(f0, dtype=np.float64).copy()
    f1 = np.tile(np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12), N)
    mac = np.zeros((4, N))
    bad = ctypes.c_int()
    p = lambda a: ctypes.c_void_p(a.ctypes.data)
    for it in range(it_begin, it_begin + steps):
        assert lib.orc_pull_step(p(kind), p(src), N, p(f0), p(f1), p(mac[0]), p(mac[1]),
                                 p(mac[2]), p(mac[3]), tau, force, it,
                                 ctypes.byref(bad)) == 0
    return f0, mac


def test_exact_form_native_path_for_out_of_range_nodes():
    """The bit-exact form multiplies on the integer pipes only for nodes
    whose values and density lie in [2^-64, 2^64); other nodes (an exact
    zero, a value of 2^-100, a subnormal value, and the neighbours they
    stream to) take native multiplies.  The kernel reports it, and the
    result equals the oracle bit for bit."""
    dims, tau, force, steps = (20, 18, 16), 0.8, 1e-4, 2
    flag = pack_flag(dims, 9, 2.5, 4.0, 0.45)
    V, vs = P.build_table(flag, *dims, 1)
    N = len(V)
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    rng = np.random.default_rng(11)
    f = np.tile(w, (N, 1)) * (1 + 0.05 * rng.uniform(-1, 1, (N, 19)))
    nodes = rng.choice(N, 40, replace=False)
    for q, i in enumerate(nodes):
        f[i, 1 + q % 18] = (0.0, 2.0 ** -100, 1e-310)[q % 3]
    ref_f, ref_mac = oracle_pull_from(V, vs, f.reshape(-1), tau, force, 1, steps)
    with gpu_run(V, dims, vs, tau, force, 0, precision="fp64_exact") as sim:
        sim.set_f(f.reshape(-1))
        sim.step(steps, it_begin=1)
        assert sim.kernel_flags() & 2, "the native path did not run"
        got = sim.get_f()
        assert np.array_equal(got.view(np.uint64), ref_f.view(np.uint64))
        assert np.array_equal(sim.macros().view(np.uint64), ref_mac.view(np.uint64))
    # a state inside the range keeps the integer path everywhere
    with gpu_run(V, dims, vs, tau, force, 20, precision="fp64_exact") as sim:
        assert not sim.kernel_flags() & 2


def test_fixed_point_fallback_fires_and_stays_within_1e12():
    """A state whose populations lie far outside the fixed-point form's range
    (deviations up to 60% of the weights at one node in twenty): those
    nodes are recomputed in native FP64, the kernel reports it, and the
    result stays within 1e-12 of the oracle; the bit-exact form equals it."""
    dims, tau, force, steps = (20, 18, 16), 0.8, 1e-4, 3
    flag = pack_flag(dims, 9, 2.5, 4.0, 0.45)
    V, vs = P.build_table(flag, *dims, 1)
    N = len(V)
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    rng = np.random.default_rng(5)
    f = np.tile(w, (N, 1)) * (1 + 0.05 * rng.uniform(-1, 1, (N, 19)))
    hit = rng.random(N) < 0.05
    f[hit] = w * (1 + 0.6 * rng.uniform(-1, 1, (int(hit.sum()), 19)))
    f /= f.sum(axis=1, keepdims=True)  # density 1 at every node
    dev = np.abs(f / w - 1)
    assert (dev[hit] > 0.45).any(axis=1).mean() > 0.9
    ref_f, ref_mac = oracle_pull_from(V, vs, f.reshape(-1), tau, force, 1, steps)
    for prec in ("fp64", "fp64_exact"):
        with gpu_run(V, dims, vs, tau, force, 0, precision=prec) as sim:
            sim.set_f(f.reshape(-1))
            sim.step(steps, it_begin=1)
            got = sim.get_f()
            if prec == "fp64":
                assert sim.kernel_flags() & 2, "the native-FP64 fallback did not fire"
                assert max_rel(got, ref_f) <= 1e-12
                assert max_rel(sim.macros()[0], ref_mac[0]) <= 1e-12
            else:
                assert (got == ref_f).all()
    # a state inside the range does not fire it
    with gpu_run(V, dims, vs, tau, force, 40, precision="fp64") as sim:
        assert sim.kernel_flags() == 0


@pytest.mark.parametrize("dims", [(96, 96, 96), (12, 10, 9)])
def test_fp64_kernel_variants_agree_bitwise(dims):
    """Every FP64 step kernel (128-, 80- and 64-register, with and without
    the L2 prefetch) runs the same integer collision: distributions, macros
    and permeability agree bit for bit."""
    flag = pack_flag(dims, 11, 3.0, 6.0, 0.4)
    runs = {}
    for v in (0, 1, 2, 3, "off"):
        sim = P.Simulation.from_flag(flag, *dims, tau=0.7, force=1e-4,
                                     precision="fp64",
                                     kernel_variant=0 if v == "off" else v,
                                     prefetch=False if v == "off" else None)
        sim.init_dist_macro()
        sim.step(7)
        sim.step(6, it_begin=7)
        runs[v] = (sim.get_f(), sim.macros(), sim.permeability()[0])
        sim.close()
    f1, m1, k1 = runs[0]
    for v in (1, 2, 3, "off"):
        f, m, k = runs[v]
        assert (f == f1).all(), v
        assert all((a == b).all() for a, b in zip(m, m1)), v
        assert k == k1, v


@pytest.mark.parametrize("precision", ["fp32", "fp16dev"])
def test_prefetch_changes_no_result(precision):
    """The L2 prefetch (off by default for the deviation forms) moves no
    value: forced on, the results are the same bits."""
    dims = (64, 48, 40)
    flag = pack_flag(dims, 12, 3.0, 6.0, 0.4)
    out = []
    for pf in (None, True):
        sim = P.Simulation.from_flag(flag, *dims, tau=0.9, force=1e-4,
                                     precision=precision, prefetch=pf)
        sim.init_dist_macro()
        sim.step(9)
        out.append((sim.get_f(), sim.macros()))
        sim.close()
    assert (out[0][0] == out[1][0]).all()
    assert all((a == b).all() for a, b in zip(out[0][1], out[1][1]))


def test_set_get_roundtrip_and_restart():
    dims = (9, 8, 7)
    flag = noise_flag(dims, 0.3, 14)
    V, vs = P.build_table(flag, *dims, 1)
    with gpu_run(V, dims, vs, 0.8, 1e-3, 10) as a, \
            gpu_run(V, dims, vs, 0.8, 1e-3, 0) as b:
        f = a.get_f()
        b.set_f(f)
        assert (b.get_f() == f).all()
        a.step(5)
        b.step(5, it_begin=10)
        assert (a.get_f() == b.get_f()).all()


def test_density_guard_matches_oracle():
    dims = (8, 8, 8)
    flag = noise_flag(dims, 0.3, 21)
    V, vs = P.build_table(flag, *dims, 1)
    s = O.OracleSim(V, *dims, vs, 0.505, 0.2)
    s.init()
    st, bad_it, bad_node = s.run(500)
    assert st == -6
    sim = P.Simulation(V, *dims, vs, tau=0.505, force=0.2)
    sim.init_dist_macro()
    with pytest.raises(P.PorelbError) as e:
        sim.step(500)
    assert e.value.status == _lib.ERR_DENSITY
    err = sim.last_error()
    assert err["it"] == bad_it and err["node"] == bad_node
    assert (err["x"], err["y"], err["z"]) == (int(V["x"][bad_node]),
                                             int(V["y"][bad_node]),
                                             int(V["z"][bad_node]))
    sim.close()


def test_rejects_bad_tables_and_order():
    dims = (6, 5, 4)
    flag = noise_flag(dims, 0.25, 15)
    V, vs = P.build_table(flag, *dims, 1)
    bad = V.copy()
    k = np.argwhere(bad["nb_info"]["node_type"][0] == 0)[0, 0]
    bad["nb_info"]["node_id"][0, k] = len(V) + 5
    with pytest.raises(P.PorelbError) as e:
        P.Simulation(bad, *dims, vs)
    assert e.value.status == _lib.ERR_TABLE
    dup = V.copy()
    dup["x"][1], dup["y"][1], dup["z"][1] = dup["x"][0], dup["y"][0], dup["z"][0]
    with pytest.raises(P.PorelbError) as e:
        P.Simulation(dup, *dims, vs)
    assert e.value.status == _lib.ERR_TABLE
    sim = P.Simulation(V, *dims, vs)
    with pytest.raises(P.PorelbError) as e:
        sim.step(1)
    assert e.value.status == _lib.ERR_STATE
    sim.close()


def test_empty_domain():
    V, vs = P.build_table(np.zeros(8, np.uint8), 2, 2, 2)
    with gpu_run(V, (2, 2, 2), vs, 0.8, 1e-3, 3) as sim:
        assert sim.get_f().size == 0
        assert sim.reduce() == (0.0, 0.0)


def test_fp64_fixed_point_matches_cpu_twin_bitwise(tmp_path):
    """The GPU's integer collision and its CPU build give identical bits."""
    import ctypes
    import subprocess
    here = os.path.dirname(os.path.abspath(__file__))
    so = tmp_path / "fx_twin.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC",
                    "-shared", "-o", str(so),
                    os.path.join(here, "native", "fx_twin.cpp")], check=True)
    lib = ctypes.CDLL(str(so))
    v = ctypes.c_void_p
    lib.fx_twin_step.restype = ctypes.c_int
    lib.fx_twin_step.argtypes = [v, v, ctypes.c_int, v, v, v, v,
                                 ctypes.c_double, ctypes.c_double, ctypes.c_int]
    dims = (20, 18, 16)
    flag = pack_flag(dims, 9, 3.0, 4.0, 0.4)
    V, vs = P.build_table(flag, *dims, 1)
    kind, src = O.pull_table(V, vs)
    N = len(V)
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    f0 = np.tile(w, N)
    f1, fo, mac = f0.copy(), f0.copy(), np.zeros((4, N))
    p = lambda a: ctypes.c_void_p(a.ctypes.data)  # noqa: E731
    for it in range(60):
        assert lib.fx_twin_step(p(kind), p(src), N, p(f0), p(f1), p(fo),
                                p(mac), 0.7, 2e-4, it) == 0
        f0, fo = fo, f0
    with gpu_run(V, dims, vs, 0.7, 2e-4, 60, precision="fp64") as sim:
        assert (sim.get_f() == f0).all()
        assert (sim.macros()[0] == mac[0]).all()


def test_dropin_porelb_x_dumps_match_reference(tmp_path):
    """preprocess.x + porelb.x on the 64^3 configuration write the
    reference's part files byte for byte (FP64_EXACT form)."""
    import subprocess
    bin_dir = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                           "porelb_gb300", "bin")
    m = META["c1_64_seed0"]
    geo = m["geometry"]
    flag = pack_flag(m["dims"], geo["seed"], geo["rmin"], geo["rmax"],
                     geo["porosity"])
    flag.tofile(tmp_path / "flag.bin")
    subprocess.run([os.path.join(bin_dir, "preprocess.x"), "1",
                    *map(str, m["dims"])], cwd=tmp_path, check=True,
                   capture_output=True)
    r = subprocess.run([os.path.join(bin_dir, "porelb.x"), "1000", "--tau",
                        repr(m["tau"]), "--force", repr(m["force"]),
                        "--precision", "fp64_exact"], cwd=tmp_path,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for fn, h in m["parts"].items():
        with open(tmp_path / fn, "rb") as fh:
            assert hashlib.sha256(fh.read()).hexdigest() == h, fn


@pytest.mark.parametrize("num_p,halfway", [(1, False), (3, False), (1, True)])
def test_streamed_state_equals_reference_next_stream(num_p, halfway):
    """plb_get_f_streamed is what the reference's f1 holds after one more
    stream of the current f0 (stream_inner_nodes, porelb.c:285-300, with its
    double-written and never-written slots; with num_p > 1 the halo order
    of porelb.c:428-433), computed from the oracle's pull table."""
    dims = (12, 9, 9)
    flag = noise_flag(dims, 0.3, 17)
    V, vs = P.build_table(flag, *dims, num_p)
    f0, _, _ = O.pull_run(V, vs, 0.8, 1e-3, 7, remote_wins=num_p > 1, halfway=halfway)
    kind, src = O.pull_table(V, vs, num_p > 1, halfway)
    N = len(V)
    w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
    g = f0.reshape(N, 19)
    f1 = np.tile(w, (N, 1))
    f1[:, 0] = g[:, 0]
    opp = [0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17]
    k, sidx = kind.reshape(N, 18), src.reshape(N, 18)
    for j in range(1, 19):
        pull, bnc = k[:, j - 1] == 0, k[:, j - 1] == 1
        f1[pull, j] = g[sidx[pull, j - 1], j]
        f1[bnc, j] = g[bnc, opp[j]]
    with P.Simulation(V, *dims, vs, tau=0.8, force=1e-3, precision="fp64_exact",
                      boundary="halfway" if halfway else "reference") as sim:
        sim.init_dist_macro()
        sim.step(7)
        assert (sim.get_f() == f0).all()
        assert (sim.get_f_streamed() == f1.reshape(-1)).all()
