"""The N > 1 host path of bench.py on the CPU: two ranks over gloo.

The hot path does not shard (independent discs, replicas only), so the only
multi-process logic is the launch contract: a barrier before each timed
region, every timed figure taken as the maximum over ranks, rank 0 alone
printing the JSON line, and the reference arm run on rank 0 only while the
other ranks exit 0 without work.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    sys.path.insert(0, ROOT)
    import bench
    r, w, _ = bench.rank_info()
    dist = bench.dist_init(w)
    dist.barrier()
    mx = bench.max_over_ranks(dist, 1.5 + r)
    with open(os.path.join(out_dir, "rank%d" % r), "w") as f:
        f.write(repr(mx))
    dist.destroy_process_group()


def test_max_over_ranks_gloo(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_rank_main, args=(world, free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    got = [float((tmp_path / ("rank%d" % r)).read_text()) for r in range(world)]
    assert got == [2.5, 2.5]


class FakeDevices:
    """Stands in for the binding's device calls: records what each rank binds."""

    def __init__(self, ndev):
        self.ndev = ndev
        self.cur = 0

    def use_device(self, ordinal):
        if not 0 <= ordinal < self.ndev:
            raise RuntimeError("bad ordinal")
        self.cur = ordinal

    def current_device(self):
        return self.cur


def _rank_device(rank, world, port, out_dir):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       # a launcher that already exports the whole device list
                       "CUDA_VISIBLE_DEVICES": ",".join(str(d) for d in range(world))})
    sys.path.insert(0, ROOT)
    import bench
    r, w, local = bench.rank_info()
    dist = bench.dist_init(w)
    dev = bench.select_device(FakeDevices(w), local, w)
    dist.barrier()
    with open(os.path.join(out_dir, "dev%d" % r), "w") as f:
        f.write(repr(dev))
    dist.destroy_process_group()


def test_each_rank_binds_its_own_device(tmp_path):
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_rank_device, args=(world, free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    got = [int((tmp_path / ("dev%d" % r)).read_text()) for r in range(world)]
    assert got == [0, 1]


def test_one_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.dist_init(1) is None
    assert bench.max_over_ranks(None, 3.25) == 3.25


def test_reference_arm_under_torchrun_prints_once(tmp_path):
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--size", "24x16x20",
           "--steps", "1", "--warmup", "0"]
    r = subprocess.run(cmd, capture_output=True, text=True, cwd=str(tmp_path), timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    out = json.loads(lines[0])
    assert out["impl"] == "reference" and out["n_gpus"] == 2
    assert out["cpu_baseline"]["kind"] == "port" and out["value"] > 0
    assert out["e2e"]["h2d_bytes_per_step"] == 0 and out["e2e"]["d2h_bytes_per_step"] == 0
