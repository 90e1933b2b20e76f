"""bench.py --impl reference on CPU: the reference arm's JSON line (one complete solve
by the oracle's C restatement on the host cores, timed in K chunks of consecutive
iterations), on a small grid so that it runs in seconds, and its behaviour under two
ranks (rank 0 alone prints, the other exits 0 quietly)."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CMD = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--size", "24", "--steps", "3",
       "--warmup", "0", "--cpu-threads", "2"]


def single_env():
    return {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}


def test_reference_arm_prints_the_contract_line():
    r = subprocess.run(CMD, env=single_env(), capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["n_gpus"] == 1 and d["higher_is_better"] is False
    # the K steps are chunks of one complete solve: together they are its measured time
    assert d["steps"] == 3 and d["value"] > 0
    assert abs(d["ms_per_step"] * d["steps"] - 1e3 * d["value"]) < 1e-6 * 1e3 * d["value"]
    cfg = d["config"]
    assert len(cfg["chunk_seconds"]) == 3 and abs(sum(cfg["chunk_seconds"]) - d["value"]) < 1e-2
    assert cfg["iterations"] > 3 and cfg["err_iter"] < 1e-10
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] == 2
    assert d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_under_two_ranks_prints_once():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    procs = []
    for rank in range(2):
        env = dict(single_env(), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", RANK=str(rank),
                   LOCAL_RANK=str(rank))
        procs.append(subprocess.Popen(CMD, env=env, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        try:
            o, e = p.communicate(timeout=300)
        except subprocess.TimeoutExpired:
            for q in procs:
                q.kill()
            raise
        assert p.returncode == 0, e
        outs.append([ln for ln in o.splitlines() if ln.startswith("{")])
    assert len(outs[0]) == 1 and outs[1] == [], outs
    assert json.loads(outs[0][0])["n_gpus"] == 2
