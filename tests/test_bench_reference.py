"""The reference arm of bench.py on CPU: `--impl reference` times the
reference's own colour sweep (SPPARKS built from its sources by
oracle/ref/Makefile, natively on this host) on the host cores and prints one
JSON line with the keys the benchmark contract asks for.  Where the reference
cannot be built, the arm times the oracle port and says so."""

import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_reference_arm_prints_one_contract_line():
    env = dict(os.environ)
    env.pop("RANK", None)
    res = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "3"], cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [l for l in res.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference"
    assert line["steps"] == 1 and line["warmup"] == 3 and line["n_gpus"] == 1
    assert line["value"] > 0 and line["unit"] == "site-updates/s" and line["higher_is_better"] is True
    cb = line["cpu_baseline"]
    import oracle

    built = oracle.reference_binary("runner_plain") is not None
    assert cb["kind"] == ("reference" if built else "port")
    assert cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    assert "workload" in line["config"]
