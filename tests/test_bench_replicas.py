"""The multi-GPU path of bench.py on CPU: every rank lays out its own replica
(the layout has no data-parallel split without a per-batch exchange), the
job's time is the slowest rank's, and the value is the units of all ranks
over that time.  Two `gloo` ranks on this host stand in for two GPUs."""
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


def _rank(rank, port, out_dir):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=2)
    # rank 1 is the slow one: 500 ms against 300 ms for 10 steps of 1,000 units
    value, job_ms = bench.replica_throughput(dist, 2, 1000, 10, 300.0 if rank == 0 else 500.0, "cpu")
    with open(os.path.join(out_dir, f"r{rank}.json"), "w") as f:
        json.dump({"value": value, "job_ms": job_ms}, f)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_throughput_two_gloo_ranks(tmp_path):
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    mp.start_processes(_rank, args=(free_port(), str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    got = [json.load(open(tmp_path / f"r{r}.json")) for r in range(2)]
    for g in got:
        assert g["job_ms"] == 500.0  # the slowest rank
        assert g["value"] == pytest.approx(2 * 1000 * 10 / 0.5)


def test_replica_throughput_one_rank():
    sys.path.insert(0, ROOT)
    import bench
    value, job_ms = bench.replica_throughput(None, 1, 1000, 10, 250.0, "cpu")
    assert job_ms == 250.0 and value == pytest.approx(40000.0)


def test_reference_arm_other_ranks_exit_without_work():
    """Under torchrun the reference arm runs on rank 0 alone; the other ranks
    exit 0 at once and print nothing."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1", MASTER_PORT="29555")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       capture_output=True, text=True, env=env, cwd=ROOT, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""


def test_reference_arm_line_on_the_grid_workload():
    """bench.py --impl reference on rank 0 prints one JSON line with the
    metric, unit and config of the GPU arm, its CPU baseline and a
    zero-copy e2e (the 4,096-vertex grid workload keeps it to seconds)."""
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "grid64",
                        "--steps", "2", "--warmup", "3"], capture_output=True, text=True, env=env, cwd=ROOT,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    sys.path.insert(0, ROOT)
    import bench
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC and line["unit"] == bench.UNIT
    assert line["value"] > 0 and line["higher_is_better"] is True
    assert line["config"]["workload"].startswith("grid64")
    # the same config object as the GPU arm's line (bench.workload_config)
    from batchlayoutcode_gb300 import graphs as G
    g, _ = G.cached_workload("grid64")
    args = type("A", (), {"workload": "grid64"})()
    assert line["config"] == bench.workload_config(args, bench.WORKLOADS["grid64"], g)
    assert set(line["config"]) == {"workload", "vertices", "edges", "step", "l2"}
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": bench.UNIT, "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
