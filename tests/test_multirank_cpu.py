"""The bench's multi-rank host logic on CPU: two gloo ranks (world_size 2).

The hot path does not shard, so N GPUs run N replicas; what N > 1 adds is
host-side: the barrier around the timed region, the max over ranks of the
elapsed time, and rank 0 alone printing the JSON line (the reference arm runs
on rank 0 only, the other ranks exit 0 without work).
"""

from __future__ import annotations

import json
import os
import socket
import subprocess
import sys
from pathlib import Path

REPO = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _cpu_env(**extra) -> dict:
    env = dict(os.environ)
    env["CUDA_VISIBLE_DEVICES"] = ""  # gloo, whatever the host has
    env["MASTER_ADDR"] = "127.0.0.1"
    env.update({k: str(v) for k, v in extra.items()})
    return env


_RANK_SCRIPT = """
import json, sys
sys.path.insert(0, {repo!r})
import bench
d = bench.Dist(2)
d.barrier()
m = d.max(float(d.rank) + 0.5)
d.barrier()
print(json.dumps({{"rank": d.rank, "world": d.world, "max": m}}), flush=True)
d.close()
"""


def test_dist_barrier_and_max_over_two_ranks():
    port = _free_port()
    script = _RANK_SCRIPT.format(repo=str(REPO))
    procs = [
        subprocess.Popen([sys.executable, "-c", script], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                         env=_cpu_env(RANK=r, LOCAL_RANK=r, WORLD_SIZE=2, MASTER_PORT=port))
        for r in range(2)
    ]
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=120)
        assert p.returncode == 0, err[-2000:]
        outs.append(json.loads(out.strip().splitlines()[-1]))
    assert sorted(o["rank"] for o in outs) == [0, 1]
    assert all(o["world"] == 2 and o["max"] == 1.5 for o in outs)


def test_reference_arm_prints_once_under_two_ranks():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), str(REPO / "bench.py"), "--impl", "reference", "--gpus", "2",
           "--config", "cfg1", "--steps", "1", "--warmup", "3"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=str(REPO), env=_cpu_env())
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    res = json.loads(lines[0])
    assert res["impl"] == "reference" and res["n_gpus"] == 2 and res["value"] > 0
    assert res["higher_is_better"] is True and res["e2e"]["h2d_bytes_per_step"] == 0
