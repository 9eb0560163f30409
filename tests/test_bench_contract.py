"""The reference arm of bench.py prints the one JSON line its callers parse.

`python bench.py --impl reference` times the C oracle on the host cores over
a bounded sample of the 1.6 M-particle workload (no GPU is involved), so the
line's contract is checked here: the shared keys, the end-to-end record with
no host-device copies, and a CPU baseline that states its sample.
"""

import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_reference_arm_prints_one_contract_line():
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "3"],
                         cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [line for line in out.stdout.splitlines() if line.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["config"] == {"workload": "block_1p6M_8knives"}
    for key in ("metric", "unit", "n_gpus", "dtype", "data", "vs_baseline"):
        assert key in d, key
    assert d["steps"] == 1 and d["warmup"] == 3 and d["higher_is_better"] is True
    assert d["value"] > 0 and d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                                            "d2h_bytes_per_step": 0}
    base = d["cpu_baseline"]
    assert base["value"] == d["value"] and base["kind"] == "port" and base["cores"] >= 1
    assert base["sample"].startswith("1 substeps of the full 1600000-particle workload after 3 untimed substeps")
