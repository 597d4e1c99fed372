"""The multi-rank host logic of bench.py on CPU (gloo, world size 2): the barrier and the max over
ranks that time a replicated run, and the reference arm under torchrun (rank 0 alone measures and
prints; the other ranks exit without work)."""
import json
import multiprocessing as mp
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, port: int, q) -> None:
    os.environ.update(WORLD_SIZE="2", RANK=str(rank), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist
    world, r, local = bench.dist_setup(0)
    bench.barrier(world)
    m = bench.max_over_ranks(1.5 + rank, world, "cpu")
    bench.barrier(world)
    dist.destroy_process_group()
    q.put((r, world, local, m))


def test_barrier_and_max_over_ranks_with_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 2, 0, 2.5), (1, 2, 1, 2.5)]


def test_reference_arm_under_torchrun_prints_one_line():
    pytest.importorskip("torch.distributed.run")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "all"], check=True)
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--workload", "c1", "--steps", "1", "--warmup", "0",
           "--ref-sample-s", "0.3"]
    res = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [l for l in res.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"


def test_training_hbm_accounting_counts_each_tensor_once():
    """The training line's HBM roofline rests on bench.train_bytes_per_row: per row of the width-256
    step, the features written once and read by the first layer's forward and backward (128 B each),
    four hidden layers each reading its input and writing Z and A (3 x 512 B, the first reading the
    features instead), the head reading A3 and the targets (8 floats and a class byte) and writing dY
    (32 B), and the backward reading dY / dZ, Z and the layer input and writing dZ (not dZ0)."""
    sys.path.insert(0, ROOT)
    import bench
    a, f, o = 512, 128, 32
    forward = (f + 2 * a) + 3 * (3 * a) + (a + 33 + o)
    backward = (o + 3 * a) + 2 * (4 * a) + (2 * a + f)
    assert bench.train_bytes_per_row(256) == f + forward + backward == 13281
    # width 64 keeps a separate head weight gradient (dY^T and A3 read again, dY written twice)
    a = 128
    assert bench.train_bytes_per_row(64) == f + ((f + 2 * a) + 3 * (3 * a) + (a + 33 + 2 * o)) + \
        ((o + a) + (o + 3 * a) + 2 * (4 * a) + (2 * a + f))
