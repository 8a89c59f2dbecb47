"""bench.py under torchrun with N > 1 (replicas, no collective on the data
path), run as world-size-2 gloo processes on CPU: the barrier, the maximum of
a per-rank time, the whole-job throughput from it, which rank reports, and
the reference arm's non-zero ranks exiting without work."""
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


WORKER = r"""
import os, sys, time
sys.path.insert(0, {root!r})
import bench
rep = bench.Replicas("gloo")
rank = rep.rank
t = 0.010 * (rank + 1)                       # rank 1 is the slow one
time.sleep(0.05 * rank)                      # ranks reach the barrier at different times
rep.barrier()
m = rep.max(t)
v = bench.job_throughput(rep.ws, 1000, m)
print(f"rank={{rank}} ws={{rep.ws}} max={{m!r}} value={{v!r}} reports={{rep.reports}}", flush=True)
rep.close()
"""


def test_two_replicas_agree_on_the_slowest_time():
    port = _free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, WORLD_SIZE="2", RANK=str(r), LOCAL_RANK=str(r), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", WORKER.format(root=ROOT)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
    outs = [p.communicate(timeout=300)[0] for p in procs]
    assert all(p.returncode == 0 for p in procs), outs
    lines = [next(l for l in o.splitlines() if l.startswith("rank=")) for o in outs]
    for r, line in enumerate(lines):
        f = dict(kv.split("=") for kv in line.split())
        assert int(f["rank"]) == r and int(f["ws"]) == 2
        assert float(f["max"]) == pytest.approx(0.020)
        assert float(f["value"]) == pytest.approx(2 * 1000 / 0.020)  # all ranks' units over the slowest time
        assert f["reports"] == ("True" if r == 0 else "False")


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, WORLD_SIZE="2", RANK="1", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1", MASTER_PORT="29999")
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "3"],
                       env=env, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert p.returncode == 0, p.stderr[-2000:]
    assert not [l for l in p.stdout.splitlines() if l.startswith("{")]
