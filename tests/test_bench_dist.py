"""bench.py's multi-rank bookkeeping on CPU ranks (gloo, world size 2):
the timed region is the slowest rank's, and the value is the whole-job sum
over replicas."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = 100.0 + 50.0 * rank
    m = bench.max_over_ranks(ms)
    v = bench.whole_job_value(1e6, 10, world, m)
    out[rank] = (m, v)
    dist.destroy_process_group()


def test_max_over_ranks_and_whole_job_value():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    mgr = mp.Manager()
    out = mgr.dict()
    port = _free_port()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    assert out[0][0] == out[1][0] == 150.0
    assert abs(out[0][1] - 2 * 1e6 * 3 * 10 / 0.150 / 1e9) < 1e-12


@pytest.mark.parametrize("workload", ["headline", "timings"])
def test_reference_arm_json_line(workload):
    """The reference arm times the oracle port on host cores (no GPU): one JSON line with
    the contract's keys, its own value repeated as e2e with no host-device bytes."""
    import json
    import subprocess
    env = dict(os.environ, OMP_NUM_THREADS="2")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", workload,
                        "--steps", "1", "--warmup", "3", "--cpu-sample-n", "12"],
                       capture_output=True, text=True, timeout=600, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == "Gcell-updates/s"
    assert line["e2e"]["value"] == line["value"] and line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert ("timing-run" in line["config"]["workload"]) == (workload == "timings")
