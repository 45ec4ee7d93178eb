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


def test_issue_model_of_the_inflate():
    """The inflate's issue roofline from the committed capture record: at the
    capture's own size and time it reproduces the capture's issue rate."""
    sys.path.insert(0, str(ROOT))
    import bench

    rec = json.loads((ROOT / "profiles" / "inflate_issue.json").read_text())

    class Tuning:
        warps_per_cta = 4

    class Eng:
        tuning = Tuning()

    class Frt:
        @staticmethod
        def inflate_ctas_per_sm(t):
            return 8

    m = bench.issue_model(Frt, Eng, rec["inflated_bytes_per_launch"], 15.83)
    peak = rec["sms"] * rec["schedulers_per_sm"] * rec["sm_clock_hz"]
    want = rec["warp_instructions_per_launch"] / 15.83e-3 / peak
    assert abs(m["frac"] - want) < 1e-3 and 0.5 < m["frac"] < 1.0
    assert m["chain"]["warps_in_flight"] == 152 * 4 * 8
    assert 50 < m["instructions_per_symbol"] < 60
