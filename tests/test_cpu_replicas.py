"""The bench's multi-GPU mode is replicas only (every rank integrates on its own,
no collective on the data path): the rank bookkeeping -- process group, barrier,
max over ranks of the timed region, rank 0 printing one line -- runs here as
two gloo ranks on the CPU."""

import json
import os
import socket
import subprocess
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist

    r, w, local = bench.dist_setup(world)
    assert (r, w, local) == (rank, world, rank)
    assert dist.get_backend() == "gloo"
    bench.barrier(w)
    slowest = bench.max_over_ranks(1.5 + rank, w)  # rank 1 "took" longer
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as fh:
        json.dump({"slowest": slowest}, fh)
    dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks(tmp_path):
    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    got = [json.load(open(tmp_path / f"rank{r}.json"))["slowest"] for r in range(2)]
    assert got == [2.5, 2.5]


def test_reference_arm_under_torchrun_prints_once():
    """`torchrun --nproc-per-node 2 bench.py --impl reference`: rank 0 times the
    CPU restatement and prints one JSON line, rank 1 exits 0 without work."""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0"]
    proc = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert proc.returncode == 0, proc.stderr[-2000:]
    lines = [ln for ln in proc.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["value"] > 0 and line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0
