"""The bench's reference arm prints the contract's JSON line without a GPU:
the unmodified reference (baseline/_ref) on its numpy path when it is
installed, and the oracle's CPU restatement of that path otherwise or with
--ref-port."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STOCK = os.path.isdir(os.path.join(ROOT, "baseline", "_ref", "pyatmosphere"))


@pytest.mark.parametrize("port", [False, True], ids=["default", "ref-port"])
def test_reference_arm_prints_one_contract_line(port):
    env = dict(os.environ, WORLD_SIZE="1", RANK="0", LOCAL_RANK="0")
    cmd = [sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"]
    r = subprocess.run(cmd + (["--ref-port"] if port else []),
                       cwd=ROOT, capture_output=True, text=True, timeout=900, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["cpu_baseline"]["kind"] == ("reference" if STOCK and not port else "port")
    assert d["cpu_baseline"]["cores"] >= 1
    assert "2048" in d["config"]["workload"]
