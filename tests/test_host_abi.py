"""Host-side checks of the C ABI that need no GPU: exports, struct layout,
V.bin I/O, table checks, the geometry generator and loud failure without a
device."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import porelb_gb300 as P
from porelb_gb300 import _lib

from helpers import noise_flag

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "porelb_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(plb_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    names = declared_functions()
    assert len(names) >= 20
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (plb_\w+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        assert getattr(lib, n) is not None
    assert set(names) == set(_lib.exported_symbols())


def test_struct_layout_matches_reference():
    # NEIGHBOR_INFO: type@0 pid@2 id@4, 8 B; NODE_INFO: 152 B (porelb.h:58-76)
    assert P.NB_DTYPE.itemsize == 8
    assert P.NB_DTYPE.fields["node_pid"][1] == 2
    assert P.NB_DTYPE.fields["node_id"][1] == 4
    assert P.NODE_DTYPE.itemsize == 152
    assert P.NODE_DTYPE.fields["nb_info"][1] == 8


def test_vbin_roundtrip(tmp_path):
    dims = (9, 7, 6)
    flag = noise_flag(dims, 0.3, 5)
    V, vs = P.build_table(flag, *dims, num_p=3)
    path = tmp_path / "V.bin"
    P.write_vbin(path, V, vs, *dims)
    V2, vs2, d2 = P.read_vbin(path)
    assert d2 == dims
    assert (vs2 == vs).all()
    assert V2.tobytes() == V.tobytes()
    raw = np.fromfile(path, np.int32, 5 + 3)
    assert list(raw[:5]) == [len(V), 3, *dims]
    assert os.path.getsize(path) == 4 * (5 + 3) + 152 * len(V)


def test_read_vbin_errors(tmp_path):
    with pytest.raises(P.PorelbError) as e:
        P.read_vbin(tmp_path / "missing.bin")
    assert e.value.status == _lib.ERR_IO
    p = tmp_path / "short.bin"
    np.array([10, 1, 4, 4, 4, 0], np.int32).tofile(p)
    with pytest.raises(P.PorelbError):
        P.read_vbin(p)


def test_build_table_rejects_uneven_slabs():
    # the reference writes out of bounds when nz % num_p != 0 (preprocess.c:107)
    flag = np.ones(4 * 4 * 6, np.uint8)
    with pytest.raises(P.PorelbError) as e:
        P.build_table(flag, 4, 4, 6, num_p=4)
    assert e.value.status == _lib.ERR_ARG
    with pytest.raises(P.PorelbError):
        P.build_table(flag, 4, 4, 6, num_p=7)


def test_build_table_empty_and_full():
    V, vs = P.build_table(np.zeros(27, np.uint8), 3, 3, 3)
    assert len(V) == 0 and list(vs) == [0]
    V, vs = P.build_table(np.ones(27, np.uint8), 3, 3, 3)
    assert len(V) == 27
    assert (V["nb_info"]["node_type"] == 0).all()


def test_check_table():
    dims = (6, 5, 4)
    flag = noise_flag(dims, 0.25, 9)
    V, vs = P.build_table(flag, *dims, num_p=2)
    assert P.check_table(V, *dims, vs) == 0
    bad = V.copy()
    k = np.argwhere(bad["nb_info"]["node_type"][0] == 0)[0, 0]
    bad["nb_info"]["node_id"][0, k] = 10 ** 6
    assert P.check_table(bad, *dims, vs) == _lib.ERR_TABLE
    bad = V.copy()
    bad["x"][3] = dims[0]
    assert P.check_table(bad, *dims, vs) == _lib.ERR_TABLE
    assert P.check_table(V, *dims, np.array([0, len(V) + 1], np.int32)) == _lib.ERR_NUMP


def test_sphere_pack_is_deterministic():
    a, na, pa = P.sphere_pack(7, 24, 20, 16, 2.5, 4.0, 0.45)
    b, nb, pb = P.sphere_pack(7, 24, 20, 16, 2.5, 4.0, 0.45)
    c, _, _ = P.sphere_pack(8, 24, 20, 16, 2.5, 4.0, 0.45)
    assert (a == b).all() and na == nb and pa == pb
    assert not (a == c).all()
    assert set(np.unique(a)) <= {0, 1}
    assert pa <= 0.45 and abs(pa - a.mean()) < 1e-15
    # one sphere fewer would still be above the target
    assert pa > 0.45 - 0.05


def test_sphere_pack_wraps_periodically():
    # a sphere near a corner covers cells on the opposite faces
    flag, ns, _ = P.sphere_pack(3, 16, 16, 16, 5.0, 5.0, 0.97)
    assert ns >= 1
    f = flag.reshape(16, 16, 16)
    solid = np.argwhere(f == 0)
    span = solid.max(0) - solid.min(0)
    assert (span <= 15).all()


def test_sphere_pack_rejects_bad_args():
    with pytest.raises(P.PorelbError):
        P.sphere_pack(0, 8, 8, 8, 0.0, 1.0, 0.5)
    with pytest.raises(P.PorelbError):
        P.sphere_pack(0, 8, 8, 8, 2.0, 1.0, 0.5)


def test_missing_library_fails_loudly(monkeypatch):
    monkeypatch.setattr(_lib, "LIB_PATH", "/nonexistent/libporelb_gpu.so")
    monkeypatch.setattr(_lib, "_lib", None)
    with pytest.raises(ImportError):
        _lib.load()


def test_create_without_device_reports_cuda_error():
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a CUDA device is present")
    V, vs = P.build_table(np.ones(8, np.uint8), 2, 2, 2)
    with pytest.raises(P.PorelbError) as e:
        P.Simulation(V, 2, 2, 2, vs)
    assert e.value.status == _lib.ERR_CUDA


def test_size_limits_rejected_before_any_device_work():
    """Neighbour words are signed offsets within two planes of the
    distribution array, so a solve holds fewer than 2^30 - 512 nodes; sizes
    beyond that are argument errors, found before any device call."""
    import ctypes
    lib = _lib.load()
    p = _lib.Params()
    lib.plb_default_params(ctypes.byref(p))
    p.precision = _lib.FP16DEV
    h = ctypes.c_void_p()
    start = (ctypes.c_int * 1)(0)
    V = (ctypes.c_char * 152)()
    rc = lib.plb_create(V, (1 << 30) - 512, 1024, 1024, 1024, 1, start,
                        ctypes.byref(p), ctypes.byref(h))
    assert rc == _lib.ERR_ARG
    rc = lib.plb_batch_create(ctypes.c_size_t(1 << 30), 4,
                              _lib.FP16DEV, 500, 0, 0,
                              ctypes.byref(h))
    assert rc == _lib.ERR_ARG


def test_tuner_defaults_without_a_measurement():
    from porelb_gb300 import tune
    assert tune.best("fp32", 12345) == dict(block_size=0, ordering="auto",
                                            kernel_variant=0)
    assert tune.best_pool("bf16dev") == dict(cta_threads=None, l2_prefetch=None,
                                             ordering=None)
