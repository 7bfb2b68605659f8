"""The multi-GPU form of the bench is replicas only (one independent run per
rank, no data-path collective): the host logic that combines the ranks'
lines, and the reference arm under torch.distributed.run, on gloo ranks on
the CPU."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    # rank r: time per step 2 + r ms, throughput 1000 * (r + 1) particle-steps/s
    res = {"value": 1000.0 * (rank + 1), "ms_per_step": 2.0 + rank, "config": {"workload": "w"}}
    out = bench.combine_replicas(res, world)
    q.put((rank, out))
    dist.destroy_process_group()


def test_combine_replicas_takes_the_slowest_rank_and_sums_the_work():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(2):
        out = got[r]
        assert out["ms_per_step"] == 3.0
        # work of both ranks (1000*2 + 2000*3 particle-steps per ms) over the slowest time
        assert out["value"] == pytest.approx((1000.0 * 2.0 + 2000.0 * 3.0) / 3.0, abs=0.05)
        assert out["n_gpus"] == 2 and out["config"]["parallelism"] == "replicas x2"


def test_reference_arm_under_torchrun_prints_one_line():
    """bench.py --impl reference on two ranks: rank 0 runs the CPU reference
    (the oracle) and prints one JSON line; rank 1 exits 0 without work."""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--workload", "probe-20", "--steps", "1", "--warmup", "3"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["cpu_baseline"]["kind"] == "port"
    st = d["cpu_baseline"]["stage_s_per_step"]
    assert set(st) == {"distributor", "poisson", "efield", "accelerator", "move", "update", "injector"}
    assert d["cpu_baseline"]["particle_stages_value"] > d["value"] > 0


def test_cpu_baseline_reports_all_cores_and_one_thread():
    """The CPU baseline of the bench line: all host threads on full steps, and
    one thread (Poisson in full, particle stages on a subsample), with the
    stage times of each."""
    sys.path.insert(0, ROOT)
    import argparse

    import bench
    args = argparse.Namespace(n_side=20, n_per=20000, workload="probe-20")
    cb = bench.cpu_baseline(args, budget=4.0)
    assert cb["kind"] == "port" and cb["value"] == cb["all_cores"]["value"] > 0
    for leg in (cb["all_cores"], cb["single_thread"]):
        assert leg["particle_stages_value"] > leg["value"] > 0
        assert set(leg["stage_s_per_step"]) == set(bench.CPU_STAGES)
    assert cb["single_thread"]["cores"] == 1 and cb["all_cores"]["cores"] == (os.cpu_count() or 1)
