"""The multi-process path of bench.py on CPU ranks (gloo, world size 2): the
step time is the slowest rank's, the reported value aggregates all ranks, and
under torchrun only rank 0 prints the reference arm's line."""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, out_dir):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    ms = bench.max_over_ranks(100.0 + 25.0 * rank, ws)
    rate = bench.whole_job_rate(1e12, ms, ws)
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump({"ms": ms, "rate": rate}, f)
    dist.destroy_process_group()


def test_max_over_ranks_and_whole_job_rate_gloo(tmp_path):
    import torch.multiprocessing as mp
    ws, port = 2, _free_port()
    mp.start_processes(_rank_main, args=(ws, port, str(tmp_path)), nprocs=ws, start_method="spawn")
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(ws)]
    for r in res:
        assert r["ms"] == 125.0                       # the slowest rank's step
        assert r["rate"] == pytest.approx(2 * 1e12 / 0.125 / 1e12)   # both ranks' work


def test_single_rank_is_identity():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(7.5, 1) == 7.5
    assert bench.whole_job_rate(2e12, 1000.0, 1) == pytest.approx(2.0)


def test_reference_arm_under_torchrun_prints_once():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0", "--nocc", "6", "--nvirt", "16", "--cpu-frac", "0.5"]
    p = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
