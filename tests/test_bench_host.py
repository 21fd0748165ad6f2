"""bench.py's host logic (no device): the clock sampler's summary of the timed region, and the
reference arm's JSON line carrying the contract's keys."""

from __future__ import annotations

import json
import subprocess
import sys
import time
from pathlib import Path

import bench

REPO = Path(__file__).resolve().parents[1]


class _Done:
    """Stands in for the nvidia-smi process the sampler stops."""

    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0

    def kill(self):
        pass


def _stamp(t: float) -> str:
    return time.strftime("%Y/%m/%d %H:%M:%S", time.localtime(int(t))) + f".{int(round((t % 1) * 1000)):03d}"


def _sampler(tmp_path, rows) -> bench.ClockSampler:
    path = tmp_path / "clocks.csv"
    path.write_text("".join(
        f"{_stamp(t)}, 0, {sm}, 2070, 800.00, 0x0000000000000000, {hw}, Not Active, Not Active, {cap}\n"
        for t, sm, hw, cap in rows))
    s = bench.ClockSampler(0)
    s.path = path
    s.fh = open(path, "a")
    s.proc = _Done()
    return s


def test_clock_summary_keeps_only_the_timed_region(tmp_path):
    t0 = float(int(time.time()) - 100)
    rows = [(t0 - 1.0, 1200, "Active", "Not Active"),  # before: a slowdown that must not count
            (t0 + 0.2, 2070, "Not Active", "Active"),
            (t0 + 0.4, 2040, "Not Active", "Not Active"),
            (t0 + 0.6, 2055, "Not Active", "Not Active"),
            (t0 + 3.0, 900, "Active", "Not Active")]  # after
    out = _sampler(tmp_path, rows).stop(t0, t0 + 1.0)
    assert out["sampled"] == "timed region" and out["samples"] == 3
    assert out["sm_mhz"] == 2055.0 and out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == ["sw_power_cap"]


def test_clock_summary_falls_back_to_the_nearest_samples(tmp_path):
    t0 = float(int(time.time()) - 100)
    rows = [(t0 - 5.0, 2070, "Not Active", "Not Active"), (t0 + 5.0, 2070, "Not Active", "Not Active")]
    out = _sampler(tmp_path, rows).stop(t0, t0 + 1.0)
    assert out["sampled"].startswith("nearest") and out["samples"] == 2 and out["reasons"] == []
    empty = _sampler(tmp_path, []).stop(t0, t0 + 1.0)
    assert empty["sm_mhz"] is None and empty["reasons"] == ["no samples"]


def test_reference_arm_line_has_the_contract_keys():
    cmd = [sys.executable, str(REPO / "bench.py"), "--impl", "reference", "--config", "cfg1", "--steps", "1",
           "--warmup", "3"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=str(REPO))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    res = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "e2e", "cpu_baseline", "impl"):
        assert key in res, key
    assert res["n_gpus"] == 1 and res["steps"] == 1 and res["warmup"] == 3
    assert res["cpu_baseline"]["kind"] in ("port", "reference") and res["cpu_baseline"]["cores"] >= 1
    assert res["e2e"]["value"] == res["value"] and res["e2e"]["d2h_bytes_per_step"] == 0
    assert "workload" in res["config"]
