"""bench.py's JSON contract through its CPU arm (--impl reference runs the oracle on the host
cores, no GPU): one line with the required keys, the reference arm's own fields, and no output
from ranks other than 0; and the parser behind the line's `clocks` key."""
import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def run(args, env=None):
    e = dict(os.environ)
    e.update(env or {})
    return subprocess.run([sys.executable, str(ROOT / "bench.py"), *args], cwd=ROOT, env=e,
                          capture_output=True, text=True, timeout=600)


def test_reference_arm_line():
    r = run(["--impl", "reference", "--steps", "2", "--warmup", "3", "--cells", "65536"])
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config", "impl",
                "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["steps"] == 2 and d["warmup"] == 3
    assert d["value"] > 0 and d["higher_is_better"] is True and d["dtype"] == "f64"
    assert d["config"]["cells"] == 65536 and "65536" in d["config"]["workload"]
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_are_silent():
    r = run(["--impl", "reference", "--steps", "1", "--warmup", "3", "--cells", "4096"],
            env={"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""


def test_warmup_below_three_is_refused():
    r = run(["--impl", "reference", "--steps", "1", "--warmup", "2", "--cells", "4096"])
    assert r.returncode != 0 and "warmup" in r.stderr


def test_clock_summary_parses_the_sampler_output():
    """The `clocks` key of the bench line: median SM clock under load, the maximum, and the
    throttle reasons seen Active, from nvidia-smi's csv rows (no GPU needed: the rows are given)."""
    sys.path.insert(0, str(ROOT))
    import bench
    s = bench.ClockSampler(0)
    s.out = "\n".join([
        "0, 1965, 2070, 812.35, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "0, 1980, 2070, 1011.20, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
        "0, 2070, 2070, 900.00, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "0, [N/A], 2070, 0, 0x0, Not Active, Not Active, Not Active, Not Active",  # unreadable
        "garbage",
    ])
    assert s.summary() == {"sm_mhz": 1980.0, "sm_max_mhz": 2070.0, "samples": 3,
                           "reasons": ["sw_power_cap"]}
    s.out = ""
    assert s.summary() is None
