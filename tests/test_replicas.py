"""Multi-rank logic of bench.py on CPU (gloo, world size 2).

The path does not shard: N GPUs run N independent replicas, synchronised by
barriers, timed by the slowest rank, and the whole-job value counts every
replica.  These tests run the same helpers as two gloo ranks.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)

import bench  # noqa: E402


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    w, r, local, pg = bench.dist_setup()
    bench.barrier(pg)
    ms = bench.max_over_ranks(pg, 10.0 * (rank + 1))
    val = bench.job_value(w, 1000, 4, ms)
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as fh:
        json.dump({"world": w, "rank": r, "ms": ms, "value": val}, fh)
    pg.destroy_process_group()


def test_max_over_ranks_and_job_value_gloo(tmp_path):
    import torch.multiprocessing as mp

    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(2)]
    for r, d in enumerate(res):
        assert d["world"] == 2 and d["rank"] == r
        assert d["ms"] == 20.0                      # slowest rank
        # 2 replicas x 1000 prisms x 4 steps in 20 ms
        assert d["value"] == pytest.approx(2 * 1000 * 4 / 0.020 / 1e6)


def test_job_value_single_rank():
    assert bench.job_value(1, 6291456, 5, 1000.0) == pytest.approx(6291456 * 5 / 1e6)


def test_reference_arm_two_ranks_rank0_only():
    """Under torchrun with 2 ranks the CPU reference arm runs on rank 0 alone,
    prints one JSON line, and both ranks exit 0."""
    pytest.importorskip("torch")
    env = dict(os.environ, OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py", "--impl", "reference",
           "--gpus", "2", "--workload", "config0", "--steps", "1", "--warmup", "0"]
    r = subprocess.run(cmd, cwd=REPO, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2
    assert d["value"] > 0 and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["cpu_baseline"]["kind"] == "port"


def test_reference_arm_loads_only_the_oracle():
    """The CPU arm builds its workload from the oracle's own synthetic inputs
    and never maps the product library."""
    code = ("import sys, argparse, bench\n"
            "a = argparse.Namespace(gpus=1, steps=1, warmup=1, workload='config0', ref_threads=2)\n"
            "bench.run_reference(a)\n"
            "maps = open('/proc/self/maps').read()\n"
            "print('LOADED', 'libnsmpgpu' in maps, 'nsmp_gb300' in sys.modules, 'libnsmp_oracle' in maps)\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=REPO, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    last = [l for l in r.stdout.splitlines() if l.startswith("LOADED")][0]
    assert last == "LOADED False False True", last
    d = json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][0])
    assert d["steps"] == 1 and d["warmup"] == 1
    assert len(d["bicgstab_iters_per_stage_timed"]) == 1 and len(d["bicgstab_iters_per_stage_timed"][0]) == 3
