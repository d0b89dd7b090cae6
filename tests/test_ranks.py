"""The multi-GPU form of bench.py on the host (no GPU): N replicas, one
process per GPU under torchrun, meeting only at a barrier and a max over the
ranks' times (cubelets are independent, so there is no exchange step).  Two
gloo ranks on 127.0.0.1 stand in for two GPUs."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.rank_barrier(dist)
        local_ms = [3.5, 7.25][rank]  # the second rank is the slow one
        got = bench.rank_max(dist, local_ms)
        bench.rank_barrier(dist)
        with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
            json.dump({"max": got}, f)
    finally:
        dist.destroy_process_group()


def test_rank_max_and_barrier_two_gloo_ranks(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    for r in range(2):
        assert json.load(open(tmp_path / f"rank{r}.json"))["max"] == 7.25


def test_rank_helpers_on_one_rank():
    sys.path.insert(0, ROOT)
    import bench
    bench.rank_barrier(None)  # nothing to wait for
    assert bench.rank_max(None, 4.5) == 4.5
    # whole-job throughput: every rank's bytes over the slowest rank's time
    assert bench.replica_gbs(2, 1e9, 500.0) == pytest.approx(4.0)
    assert bench.replica_gbs(1, 668e6, 4.67) == pytest.approx(668e6 / 4.67e-3 / 1e9)


def test_reference_arm_under_torchrun_two_ranks():
    """Rank 0 alone runs the reference arm and prints its line; the other
    rank exits 0 without work."""
    pytest.importorskip("torch")
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
           "--warmup", "0", "--cubelets", "16"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
