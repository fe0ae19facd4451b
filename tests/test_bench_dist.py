"""The multi-rank plumbing of bench.py on CPU with gloo (world size 2):
max-over-ranks timing, and the reference arm printing on rank 0 only."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    got = bench.max_over_ranks(10.0 * (rank + 1), world, device="cpu")
    r, w, _ = bench.dist_env()
    dist.destroy_process_group()
    q.put((rank, got, r, w))


def test_max_over_ranks_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [20.0, 20.0]
    assert [(r[2], r[3]) for r in res] == [(0, 2), (1, 2)]


def test_reference_arm_silent_off_rank0(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference"])
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    bench.main()
    assert capsys.readouterr().out == ""


def test_reference_arm_line_on_rank0(monkeypatch, capsys):
    """The reference arm's JSON line: the contract's keys, its CPU work
    bounded by --ref-budget whatever --steps is."""
    import json
    import time
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--workload",
                                      "c1_64", "--steps", "50", "--warmup", "3",
                                      "--ref-budget", "2"])
    monkeypatch.setenv("RANK", "0")
    monkeypatch.setenv("WORLD_SIZE", "1")
    t0 = time.perf_counter()
    bench.main()
    took = time.perf_counter() - t0
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["metric"] == "fluid MLUPS"
    assert line["value"] > 0 and line["unit"] == "MLUPS" and line["steps"] == 50
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    assert took < 60


def test_reference_arm_loads_no_library_code():
    """The reference arm builds its geometry and table with the oracle and
    runs the oracle port: the GPU library is neither imported nor mapped,
    and its config equals the GPU arm's for the same workload."""
    import json
    import subprocess
    code = (
        "import sys, json; sys.argv = ['bench.py', '--impl', 'reference', "
        "'--workload', 'c1_64', '--steps', '3', '--warmup', '3', '--ref-budget', '1'];"
        "import bench; bench.main();"
        "maps = open('/proc/self/maps').read();"
        "print(json.dumps({'lib_mapped': 'libporelb_gpu' in maps, "
        "'pkg': 'porelb_gb300' in sys.modules}))")
    out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True,
                         text=True, timeout=300, env=dict(os.environ, RANK="0",
                                                          WORLD_SIZE="1"))
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [json.loads(x) for x in out.stdout.strip().splitlines() if x.startswith("{")]
    probe, line = lines[-1], lines[-2]
    assert probe == {"lib_mapped": False, "pkg": False}
    sys.path.insert(0, ROOT)
    import bench
    import porelb_gb300 as P
    w = bench.WORKLOADS["c1_64"]
    flag, _, phi = P.sphere_pack(w["seed"], *w["dims"], w["rmin"], w["rmax"], w["porosity"])
    V, _ = P.build_table(flag, *w["dims"], 1)
    assert line["config"] == bench.workload_config("c1_64", w, len(V), phi, "fp64")
