"""bench.py's reference arm (the CPU oracle on the benchmark scene) runs on the
CPU and prints one JSON line with the keys the benchmark contract asks for."""
import json
import os
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.slow
def test_reference_arm_prints_contract_line(built):
    out = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "1", "--cpu-budget", "5"], capture_output=True, text=True, timeout=600,
                         cwd=REPO)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "impl", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["warmup"] >= 1 and d["steps"] >= 1
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["config"]["fluid_particles"] == 1048576
    # the same workload description as the GPU arm, and no CUDA library in the process
    for k in ("workload", "phases", "h", "d", "dt", "box", "eos", "schedule", "seed"):
        assert k in d["config"], k
    assert d["config"]["schedule"].startswith("fused")
    libs = d["repo_libraries_loaded"]
    assert libs is not None and any("liboracle" in x for x in libs), libs
    assert not any("libsphmp" in x for x in libs), libs
