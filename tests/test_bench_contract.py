"""bench.py's reference arm (the CPU port of the reference assembly, timed on the
host cores) keeps the one-JSON-line contract; it runs without a GPU."""
import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _reference_line(workload: str) -> dict:
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--workload", workload,
                          "--steps", "1", "--warmup", "0"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1, out.stdout[-2000:]
    return json.loads(lines[0])


@pytest.mark.parametrize("workload", ["neohookean", "j2", "poisson"])
def test_reference_arm_line(workload):
    d = _reference_line(workload)
    assert d["impl"] == "reference"
    for key in ("metric", "unit", "dtype", "data", "scaling"):
        assert isinstance(d[key], str) and d[key]
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["n_gpus"] == 1 and d["steps"] == 1 and d["warmup"] == 0
    assert d["higher_is_better"] is True and d["vs_baseline"] is None
    assert isinstance(d["config"]["workload"], str)
    cpu = d["cpu_baseline"]
    assert cpu["value"] == d["value"] and cpu["unit"] == d["unit"]
    assert cpu["kind"] in ("port", "reference") and cpu["cores"] >= 1 and cpu["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


@pytest.mark.parametrize("workload", ["j2mlp", "batched", "action", "symbolic"])
def test_reference_arm_unavailable_line(workload):
    d = _reference_line(workload)
    assert d["impl"] == "reference" and isinstance(d["unavailable"], str) and d["unavailable"]
