"""Host logic of the multi-GPU replica mode of bench.py on CPU (gloo, world size 2): every rank
renders its own replica, the ranks meet at a barrier, and the step time is the maximum over ranks.
No collective touches the data path.  Also: under torchrun the reference arm runs on rank 0 only."""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _worker(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, str(ROOT))
    import bench

    r, w, local, td = bench.dist()
    assert (r, w, local) == (rank, world, rank) and td is not None
    td.barrier()
    m = bench.reduce_max(td, 10.0 + 5.0 * rank)
    out.put((rank, m))
    td.destroy_process_group()


def test_two_rank_barrier_and_max_over_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 1000)
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == {0: 15.0, 1: 15.0}


def test_single_process_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.dist() == (0, 1, 0, None)
    assert bench.reduce_max(None, 3.5) == 3.5


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1"],
                       capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""


def test_reference_arm_line_shape(monkeypatch):
    """The reference arm's JSON line on a tiny photograph (the oracle's tile renders patched out)."""
    sys.path.insert(0, str(ROOT))
    import numpy as np
    import bench

    seen = []
    monkeypatch.setattr(bench, "oracle_tiles",
                        lambda jobs, threads: (seen.extend(jobs), (2.0, [np.zeros_like(j[2]) for j in jobs]))[1])
    lines = []
    monkeypatch.setattr("builtins.print", lambda s, *a, **k: lines.append(s))

    class A:
        steps, warmup, gpus, film_side = 2, 1, 2, 64

    monkeypatch.setenv("RANK", "0")
    bench.run_reference(A())
    d = json.loads(lines[-1])
    assert d["impl"] == "reference" and d["unit"] == "Mpx/s" and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["n_gpus"] == 2 and d["config"]["workload"].startswith(bench.C4_WORKLOAD)
    assert d["steps"] == 2 and d["warmup"] == 1 and len(seen) == 1 + 4 * 2  # one tile per warm-up step
    assert all(j[0] == "t-max" and abs(j[1] - 1 / 1.1) < 1e-15 for j in seen)


def test_reference_arm_imports_nothing_of_the_product():
    """The reference arm runs the oracle only: after a (tiny, patched) run no module of the
    product package is loaded in the process."""
    code = (
        "import sys, numpy as np; sys.path.insert(0, %r); import bench\n"
        "bench.oracle_tiles = lambda jobs, threads: (1.0, [np.zeros_like(j[2]) for j in jobs])\n"
        "class A: steps, warmup, gpus, film_side = 1, 0, 1, 64\n"
        "bench.run_reference(A())\n"
        "print(sorted(m for m in sys.modules if m.startswith('fgrain_gb300')))\n" % str(ROOT))
    env = dict(os.environ, RANK="0", WORLD_SIZE="1")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip().splitlines()[-1] == "[]"
