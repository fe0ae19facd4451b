"""Drop-in executables: preprocess.x writes the reference's V.bin, and
postprocess.x writes the reference's slice files from the same part files
(last column masked: the reference prints an int through %e there, an
undefined value)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle_py as O
import porelb_gb300 as P

from helpers import noise_flag, table_fields

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BIN = os.path.join(ROOT, "porelb_gb300", "bin")
needs_ref = pytest.mark.skipif(
    not (O.ref_available() and os.path.exists(O.REF_POST_PATH)),
    reason="reference tree not compiled here")


def test_preprocess_x_writes_reference_table(tmp_path):
    dims = (10, 9, 8)
    flag = noise_flag(dims, 0.3, 61)
    flag.tofile(tmp_path / "flag.bin")
    subprocess.run([os.path.join(BIN, "preprocess.x"), "2", *map(str, dims)],
                   cwd=tmp_path, check=True, capture_output=True)
    V, vs, d = P.read_vbin(tmp_path / "V.bin")
    Vo, vso = O.build_v(flag, *dims, 2)
    assert d == dims and (vs == vso).all()
    for a, b in zip(table_fields(V), table_fields(Vo)):
        assert (a == b).all()


def strip_last_column(text):
    out = []
    for line in text.splitlines():
        parts = line.split()
        if len(parts) == 7 and not line.startswith(("TITLE", "Variables", "ZONE")):
            parts = parts[:6]
            out.append(" ".join(parts))
        else:
            out.append(line)
    return out


@needs_ref
@pytest.mark.parametrize("mode,n", [("X", 3), ("Y", 0), ("Z", 5)])
def test_postprocess_slices_match_reference(tmp_path, mode, n):
    dims = (9, 7, 6)
    flag = noise_flag(dims, 0.3, 62)
    ref_dir = tmp_path / "ref"
    our_dir = tmp_path / "our"
    ref_dir.mkdir()
    flag.tofile(ref_dir / "flag.bin")
    O.ref_write_vbin(flag, *dims, 2, str(ref_dir / "V.bin"))
    O.ref_run(str(ref_dir), 2, 6, 0.8, 1e-3, save=True, save_every=5)
    shutil.copytree(ref_dir, our_dir)
    one_dir = tmp_path / "one"
    shutil.copytree(ref_dir, one_dir)
    # the reference leaves the last time's data in every slice file of a
    # multi-time call; PLB_SLICE_COMPAT=1 reproduces that
    assert O.ref_postprocess(str(ref_dir), [mode, n, 0, 6]) == 0
    env = dict(os.environ, PLB_SLICE_COMPAT="1")
    subprocess.run([os.path.join(BIN, "postprocess.x"), mode, str(n), "0", "6"],
                   cwd=our_dir, check=True, capture_output=True, env=env)
    for tag in (0, 6):
        fn = f"Slice_{mode}_{tag:07d}.dat"
        a = strip_last_column((ref_dir / fn).read_text())
        b = strip_last_column((our_dir / fn).read_text())
        assert a == b
    # default: each file holds its own time, as the reference gives for a
    # one-time call
    subprocess.run([os.path.join(BIN, "postprocess.x"), mode, str(n), "0", "6"],
                   cwd=our_dir, check=True, capture_output=True)
    for tag in (0, 6):
        assert O.ref_postprocess(str(one_dir), [mode, n, tag]) == 0
        fn = f"Slice_{mode}_{tag:07d}.dat"
        a = strip_last_column((one_dir / fn).read_text())
        b = strip_last_column((our_dir / fn).read_text())
        assert a == b


def test_postprocess_raw_full_grid(tmp_path):
    dims = (5, 4, 3)
    flag = noise_flag(dims, 0.3, 63)
    flag.tofile(tmp_path / "flag.bin")
    V, vs = P.build_table(flag, *dims, 1)
    P.write_vbin(tmp_path / "V.bin", V, vs, *dims)
    N = len(V)
    mac = np.arange(4 * N, dtype=np.float64).reshape(4, N) + 0.5
    mac.tofile(tmp_path / "part_000_0000007.bin")
    subprocess.run([os.path.join(BIN, "postprocess.x"), "R", "7"], cwd=tmp_path,
                   check=True, capture_output=True)
    raw = np.fromfile(tmp_path / "full_0000007.raw", np.int32, 3)
    assert list(raw) == list(dims)
    data = np.fromfile(tmp_path / "full_0000007.raw", np.float64, offset=12)
    grid = data.reshape(4, -1)
    loc = (V["z"].astype(int) * dims[1] + V["y"]) * dims[0] + V["x"]
    assert (grid[:, loc] == mac).all()
    solid = np.ones(grid.shape[1], bool)
    solid[loc] = False
    assert (grid[:, solid] == 0).all()


def test_postprocess_tecplot_mode_unavailable(tmp_path):
    r = subprocess.run([os.path.join(BIN, "postprocess.x"), "A", "0"], cwd=tmp_path,
                       capture_output=True, text=True)
    assert r.returncode != 0 and "TECIO" in r.stderr
