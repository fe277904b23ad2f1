"""bench.py's host logic on the CPU: the replica reduction of a multi-GPU run (two gloo ranks),
and the reference arm's contract (rank 0 alone prints; the implicit workloads have no CPU arm)."""
import json
import os
import socket
import subprocess
import sys

import pytest

import conftest

ROOT = conftest.ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        seconds = 1.0 + 2.0 * rank                      # rank 1 is the slowest
        t = bench.max_over_ranks(seconds, world, "cpu")
        rate = bench.job_throughput(1000, world, t)
        with open(os.path.join(out_dir, f"r{rank}.json"), "w") as f:
            json.dump({"t": t, "rate": rate}, f)
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks(tmp_path):
    """Every rank gets the slowest rank's time; the job's rate counts all ranks' units."""
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    for rank in range(world):
        r = json.loads((tmp_path / f"r{rank}.json").read_text())
        assert r["t"] == 3.0
        assert r["rate"] == pytest.approx(1000 * world / 3.0, rel=1e-15)


def test_single_rank_reduction_is_identity():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(2.5, 1, "cpu") == 2.5
    assert bench.job_throughput(10, 1, 2.0) == 5.0


def _bench(args, env_extra=None, timeout=600):
    env = dict(os.environ)
    env.update(env_extra or {})
    return subprocess.run([sys.executable, str(ROOT / "bench.py"), *args], capture_output=True, text=True,
                          timeout=timeout, cwd=str(ROOT), env=env)


def test_reference_arm_other_ranks_exit_quietly():
    r = _bench(["--impl", "reference", "--gpus", "2"], {"RANK": "1", "LOCAL_RANK": "1", "WORLD_SIZE": "2"})
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""


@pytest.mark.parametrize("workload", ["flatplate-implicit", "ffbox3d-implicit", "kdif3d", "adjoint3d"])
def test_reference_arm_unavailable_for_gpu_only_comparisons(workload):
    r = _bench(["--impl", "reference", "--workload", workload])
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unavailable"]


def test_reference_arm_line_small_box():
    """The reference arm's JSON line on a 4^3x5 box: the oracle timed on the host cores."""
    r = _bench(["--impl", "reference", "--n", "4", "--steps", "2", "--warmup", "1"], {"OMP_NUM_THREADS": "2"})
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["metric"] and line["unit"] == "cell-updates/s" and line["value"] > 0
    assert line["steps"] == 2 and line["warmup"] == 1 and line["higher_is_better"] is True
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] == 2 and cb["value"] == line["value"] and cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["config"]["cells"] == 5 * 4 ** 3
