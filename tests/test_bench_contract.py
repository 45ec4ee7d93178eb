"""bench.py's reference arm on CPU: one JSON line with the contract's keys."""

import json
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_reference_arm_prints_one_contract_line(capsys):
    sys.path.insert(0, str(ROOT))
    import bench

    class Args:
        workload = "short_reads_100k"
        steps = 1
        warmup = 0
        gpus = 1

    bench.run_reference(Args, 0, 1)
    lines = [line for line in capsys.readouterr().out.splitlines() if line.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference"
    assert d["config"]["workload"] == "short_reads_100k"
    assert d["config"]["records"] == 100_000
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["cpu_baseline"]["kind"] == "port" and d["value"] > 0
