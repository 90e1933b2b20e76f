"""The multi-GPU form of the benchmark is N independent replicas of the solve (the path
has one domain and no data-path collective): the ranks meet only at a host barrier
around the timed region and in the max over ranks of the time.  Here two gloo ranks on
CPU exercise that coordination as bench.py uses it under torchrun."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RANK_SCRIPT = r"""
import sys
sys.path.insert(0, {root!r})
import bench
d = bench.Dist()
assert (d.ws, d.rank, d.local) == (2, {rank}, {rank}), (d.ws, d.rank, d.local)
d.barrier()
print("max", d.max(float({rank} + 1) * 0.25), flush=True)
d.barrier()
d.close()
"""


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_replicas_meet_at_the_barrier_and_report_the_max():
    pytest.importorskip("torch.distributed")
    port = free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2",
                   RANK=str(rank), LOCAL_RANK=str(rank))
        procs.append(subprocess.Popen([sys.executable, "-c", RANK_SCRIPT.format(root=ROOT, rank=rank)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        try:
            o, e = p.communicate(timeout=120)
        except subprocess.TimeoutExpired:
            for q in procs:
                q.kill()
            raise
        assert p.returncode == 0, e
        outs.append(o)
    # each rank sees the max over both ranks (0.25 and 0.5)
    assert all("max 0.5" in o for o in outs), outs


def test_single_process_needs_no_process_group():
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    script = (f"import sys; sys.path.insert(0, {ROOT!r}); import bench; d = bench.Dist(); "
              "assert d.pg is None and d.max(1.5) == 1.5; d.barrier(); d.close(); print('ok')")
    r = subprocess.run([sys.executable, "-c", script], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "ok" in r.stdout, r.stderr
