"""Writes the golden fixtures of tests/golden from the reference itself.

The reference (porelb.c / preprocess.c) is compiled from its own sources by
oracle/Makefile into oracle/_ref/ (needs the reference tree, so this runs in
the development container, not on the GPU machine).  Geometry comes from the
library's sphere-pack generator or a seeded numpy noise field; both are
recorded in the fixtures.

    python tests/golden/make_golden.py
"""
import hashlib
import json
import math
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle_py as O  # noqa: E402
import porelb_gb300 as P  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def table_fields(V):
    """Fields of a node table that the reference defines (SOLID id/pid and
    padding are leftovers of a reused temporary and are zeroed here)."""
    t = V["nb_info"]["node_type"].astype(np.uint8)
    ident = np.where(t == 1, 0, V["nb_info"]["node_id"]).astype(np.uint32)
    pid = np.where(t == 1, 0, V["nb_info"]["node_pid"]).astype(np.uint16)
    xyz = np.stack([V["x"], V["y"], V["z"]]).astype(np.uint16)
    return xyz, t, ident, pid


def run_case(name, flag, dims, num_p, steps, tau, force, full, save=False):
    nx, ny, nz = dims
    with tempfile.TemporaryDirectory() as d:
        vpath = os.path.join(d, "V.bin")
        O.ref_write_vbin(flag, nx, ny, nz, num_p, vpath)
        V, vs, _ = P.read_vbin(vpath)
        f0, f1, mac, _ = O.ref_run(d, num_p, steps, tau, force, save=save)
        parts = {}
        if save:
            for fn in sorted(os.listdir(d)):
                if fn.startswith("part_"):
                    with open(os.path.join(d, fn), "rb") as fh:
                        parts[fn] = hashlib.sha256(fh.read()).hexdigest()
    xyz, t, ident, pid = table_fields(V)
    tau_eff = 0.8 if math.isnan(tau) else tau
    f_eff = 1e-3 if math.isnan(force) else force
    nu = 1.0 / 3.0 * (tau_eff - 0.5)
    sum_ux = math.fsum(mac[1])
    meta = dict(name=name, dims=[nx, ny, nz], num_p=num_p, steps=steps,
                tau=tau_eff, force=f_eff, num_node=int(len(V)),
                v_sub_start=[int(x) for x in vs],
                sha_table=sha(np.concatenate([xyz.ravel().view(np.uint8),
                                              t.ravel(), ident.ravel().view(np.uint8),
                                              pid.ravel().view(np.uint8)])),
                sha_f0=sha(f0), sha_f1=sha(f1), sha_macros=sha(mac),
                sum_ux=sum_ux, mass=math.fsum(mac[0]),
                k_darcy=sum_ux / (nx * ny * nz) * nu / f_eff,
                parts=parts)
    arrays = dict(flag=np.asarray(flag, np.uint8).reshape(-1))
    if full:
        arrays.update(xyz=xyz, type=t, node_id=ident, node_pid=pid, f0=f0,
                      f1=f1, macros=mac)
    else:
        rng = np.random.default_rng(123)
        idx = np.sort(rng.choice(len(V), size=min(64, len(V)), replace=False))
        arrays.update(sample_idx=idx, sample_f0=f0.reshape(-1, 19)[idx],
                      sample_macros=mac[:, idx])
        # the flag of a large case is regenerated from its seed
        del arrays["flag"]
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **arrays)
    return meta


def main():
    if not O.ref_available():
        sys.exit("oracle/_ref is not built: run make -C oracle with the reference tree present")
    cases = []
    rng = np.random.default_rng(11)
    flag = (rng.random(10 * 8 * 6) > 0.3).astype(np.uint8)
    # reference defaults: tau 0.8, force 1e-3 (NaN keeps init_para's values)
    cases.append(run_case("noise_10x8x6_p1", flag, (10, 8, 6), 1, 30,
                          float("nan"), float("nan"), True))
    rng = np.random.default_rng(12)
    flag = (rng.random(8 * 6 * 8) > 0.35).astype(np.uint8)
    cases.append(run_case("noise_8x6x8_p2", flag, (8, 6, 8), 2, 30, 0.9,
                          5e-4, True))
    flag = np.ones(2 * 2 * 2, np.uint8)
    flag[3] = 0
    cases.append(run_case("tiny_2x2x2_p1", flag, (2, 2, 2), 1, 7, 0.7, 1e-3,
                          True))
    # Plain-method configuration: 64^3 periodic sphere pack, seed 0, R = 6,
    # porosity 0.40, tau 1.0, body force 1e-6, 1000 steps; part files dumped
    # on the reference's schedule.
    flag, ns, phi = P.sphere_pack(0, 64, 64, 64, 6.0, 6.0, 0.40)
    meta = run_case("c1_64_seed0", flag, (64, 64, 64), 1, 1000, 1.0, 1e-6,
                    False, save=True)
    meta.update(geometry=dict(seed=0, rmin=6.0, rmax=6.0, porosity=0.40,
                              spheres=ns, porosity_out=phi,
                              sha_flag=sha(flag)))
    cases.append(meta)
    # the same geometry decomposed into 4 z-slabs (mpirun -np 4 semantics)
    meta = run_case("c1_64_seed0_p4_100", flag, (64, 64, 64), 4, 100, 1.0,
                    1e-6, False)
    cases.append(meta)
    with open(os.path.join(OUT, "golden.json"), "w") as fh:
        json.dump(dict(generator="tests/golden/make_golden.py", cases=cases),
                  fh, indent=1)
    print(json.dumps([(c["name"], c["num_node"]) for c in cases]))


if __name__ == "__main__":
    main()
