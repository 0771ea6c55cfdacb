"""The N > 1 path of bench.py on CPU with the gloo backend (world size 2):
ranks are independent replicas; the only cross-rank operations are a
barrier and the max of the per-rank times, and rank 0 alone prints."""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.barrier(world)
        t = bench.allmax(1.5 + rank, world)  # rank 1 is the slower replica
        with open(os.path.join(out_dir, f"r{rank}.txt"), "w") as fh:
            fh.write(repr(t))
    finally:
        dist.destroy_process_group()


def test_allmax_over_two_gloo_ranks(tmp_path):
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn")
    for r in range(2):
        assert float((tmp_path / f"r{r}.txt").read_text()) == 2.5


def test_reference_arm_under_torchrun_prints_once(lgb, oracle):
    port = _free_port()
    env = dict(os.environ, LGB_REF_BUDGET_S="5")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py",
           "--impl", "reference", "--gpus", "2", "--steps", "2", "--warmup", "1",
           "--grid", "24"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    rec = json.loads(lines[0])
    assert rec["impl"] == "reference" and rec["unit"] == "MLUPS" and rec["value"] > 0
    assert rec["cpu_baseline"]["kind"] == "port"
    assert rec["e2e"]["h2d_bytes_per_step"] == 0


def test_lettuce_arm_cpu_leg():
    """``bench.py --impl lettuce`` with its GPU legs off: lettuce's own torch
    CPU path on a small grid, one JSON line with the sample stated; and the
    main line's ``lettuce_cpu`` entry built from it. Skipped when lettuce
    is not installed in baseline/_ref."""
    if not os.path.isfile(os.path.join(ROOT, "baseline", "_ref", "lettuce", "__init__.py")):
        pytest.skip("lettuce is not installed in baseline/_ref")
    env = dict(os.environ, LGB_LETTUCE_CPU_ONLY="1", LGB_LETTUCE_CPU_GRID="12,10,8")
    cmd = [sys.executable, "bench.py", "--impl", "lettuce", "--steps", "3", "--warmup", "1"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    rec = json.loads(lines[0])
    assert rec["impl"] == "lettuce" and rec["lettuce"]["version"]
    leg = rec["torch_cpu"]
    assert leg["mlups"] > 0 and leg["cores"] >= 1 and "12x10x8" in leg["sample"]
    assert "cuda_native" not in rec
    sys.path.insert(0, ROOT)
    import bench
    os.environ["LGB_LETTUCE_CPU_GRID"] = "12,10,8"
    try:
        got = bench.lettuce_cpu_sample()
    finally:
        del os.environ["LGB_LETTUCE_CPU_GRID"]
    assert got["kind"] == "lettuce torch CPU path" and got["value"] > 0
