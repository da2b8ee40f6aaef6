"""The multi-rank path of bench.py on CPU: world size 2 over gloo.

The solver step does not shard (the SIP recurrences are global), so N GPUs
run N independent replicas; the only cross-rank operations are the barrier
around the timed region and the max over ranks of the timings, plus the rule
that rank 0 alone prints.  Both are exercised here without a GPU."""
import json
import os
import pathlib
import socket
import subprocess
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import bench
    g = bench.Group(2)
    g.barrier()
    m = g.max(10.0 * (rank + 1))   # rank 0: 10, rank 1: 20
    g.barrier()
    g.close()
    (pathlib.Path(out_dir) / f"rank{rank}.txt").write_text(repr(m))


def test_group_barrier_and_max_two_ranks(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    for r in range(2):
        assert float((tmp_path / f"rank{r}.txt").read_text()) == 20.0


def test_reference_arm_prints_once_under_torchrun(oracle_mod):
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0", "--size", "8"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=str(ROOT))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    rec = lines[0]
    assert rec["impl"] == "reference" and rec["n_gpus"] == 2 and rec["value"] > 0
    assert rec["cpu_baseline"]["kind"] == "port" and rec["e2e"]["h2d_bytes_per_step"] == 0
