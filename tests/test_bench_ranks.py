"""The replica (multi-GPU) host logic of bench.py on CPU ranks (gloo, world size 2): the job's
time is the slowest rank's, throughput counts every rank's batch, each rank evaluates its own
C_l vectors, and the reference arm prints from rank 0 only.  No device is used."""
import json
import os
import socket
import subprocess
import sys

import numpy as np
import torch.multiprocessing as mp

from conftest import ROOT

sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=world)
    ms = [12.5, 30.25][rank]
    got = bench.max_over_ranks(ms, world)
    dist.barrier()
    dist.destroy_process_group()
    with open(os.path.join(out, "r%d.json" % rank), "w") as f:
        json.dump({"max": got, "value": bench.job_throughput(256, world, got)}, f)


def test_max_over_ranks_and_job_throughput(tmp_path):
    mp.spawn(_rank_main, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    for r in range(2):
        d = json.load(open(tmp_path / ("r%d.json" % r)))
        assert d["max"] == 30.25
        assert abs(d["value"] - 2 * 256 / 0.03025) < 1e-6


def test_single_rank_is_identity():
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.job_throughput(256, 1, 32.0) == 8000.0


def test_ranks_draw_different_batches():
    from cosmopp_gb300 import workload as W
    a = W.make(bench.WORKLOAD, batch=4, batch_seed=bench.rank_batch_seed(0)).cl_batch
    b = W.make(bench.WORKLOAD, batch=4, batch_seed=bench.rank_batch_seed(1)).cl_batch
    assert a.shape == b.shape and not np.array_equal(a, b)


def test_reference_arm_prints_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], capture_output=True, text=True, env=env, timeout=300)
    assert p.returncode == 0, p.stderr
    assert p.stdout.strip() == ""
