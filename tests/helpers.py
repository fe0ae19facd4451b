"""Shared helpers of the test suite: geometries, golden fixtures and the
comparison of device results with the oracle."""
import json
import os

import numpy as np

import porelb_gb300 as P

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
W = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)


def noise_flag(dims, p_solid, seed):
    rng = np.random.default_rng(seed)
    n = dims[0] * dims[1] * dims[2]
    return (rng.random(n) >= p_solid).astype(np.uint8)


def pack_flag(dims, seed, rmin, rmax, porosity):
    flag, _, _ = P.sphere_pack(seed, *dims, rmin, rmax, porosity)
    return flag


def golden_meta():
    with open(os.path.join(GOLDEN, "golden.json")) as fh:
        return {c["name"]: c for c in json.load(fh)["cases"]}


def golden_arrays(name):
    return dict(np.load(os.path.join(GOLDEN, f"{name}.npz")))


def table_fields(V):
    t = V["nb_info"]["node_type"].astype(np.uint8)
    ident = np.where(t == 1, 0, V["nb_info"]["node_id"]).astype(np.uint32)
    pid = np.where(t == 1, 0, V["nb_info"]["node_pid"]).astype(np.uint16)
    xyz = np.stack([V["x"], V["y"], V["z"]]).astype(np.uint16)
    return xyz, t, ident, pid


def max_rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300))) if a.size else 0.0
