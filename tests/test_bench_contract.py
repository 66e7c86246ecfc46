"""The reference arm of bench.py (the reference's CPU correlator path, run as
the oracle port on the host cores): one JSON line with the bench contract's
keys, the same `config` keys as the GPU arm, and an e2e object with no
host-device traffic.  CPU only: a one-rotation-per-core sample."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.timeout(600)
def test_reference_arm_prints_one_contract_line():
    res = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0", "--cpu-rot-per-core", "1"],
                         cwd=ROOT, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [ln for ln in res.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "rotations/s" and d["higher_is_better"]
    sys.path.insert(0, ROOT)
    import bench
    from powerfit_gb300 import synth
    cfg = synth.CONFIGS["lcc128_filtered"]
    assert set(d["config"]) == set(bench.workload_config("lcc128_filtered", cfg, cfg["shape"], 1, 1, "").keys())
    assert d["config"]["workload"] == "lcc128_filtered" and d["config"]["grid"] == [128, 128, 128]
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
