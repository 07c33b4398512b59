"""The reference arm of bench.py keeps the benchmark line's contract on the
CPU: one JSON line with this arm's metric, unit and config (the same
`workload_config` object at every world size), a cpu_baseline describing
its own run and an e2e block without copies, at least three warm-up steps;
ranks other than 0 exit 0 without work or output."""
import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _run(extra_env, n=16):
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    env.update(extra_env)
    return subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--n", str(n),
                           "--steps", "1", "--warmup", "1"], capture_output=True, text=True, env=env,
                          cwd=ROOT, timeout=600)


def test_reference_arm_line():
    sys.path.insert(0, str(ROOT))
    import bench
    for env, replicas in (({}, 1), ({"RANK": "0", "WORLD_SIZE": "2"}, 2)):
        r = _run(env)
        assert r.returncode == 0, r.stderr
        lines = [x for x in r.stdout.splitlines() if x.startswith("{")]
        assert len(lines) == 1
        d = json.loads(lines[0])
        assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
        assert d["higher_is_better"] is True and d["value"] > 0 and d["steps"] == 1
        assert d["warmup"] == 3  # raised to the minimum of three warm-up steps
        c = d["config"]
        assert c == bench.workload_config(16, c["nparts"], 100.0 * 16 / 64, 2, False, replicas)
        assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
        assert d["cpu_baseline"]["cores"] >= 1
        assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                            "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_exit_quietly():
    r = _run({"RANK": "1", "WORLD_SIZE": "2"})
    assert r.returncode == 0 and r.stdout.strip() == ""
