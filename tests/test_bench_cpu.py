"""The bench's reference arm on the CPU: one JSON line with the contract's keys, the same
`config` dict the GPU arm prints for the same mesh, a cpu_baseline describing the run and
an e2e object without host-device copies.  Run on a small mesh (8^3 macro elements)."""

import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402


def test_reference_arm_json_line():
    env = dict(os.environ, OMP_NUM_THREADS="2")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "1",
                        "--nx", "8"], capture_output=True, text=True, env=env, cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["config"] == bench.config_dict(bench.workload_config(8))
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0 == d["e2e"]["d2h_bytes_per_step"]


def test_stencil_fma_count():
    # 27 taps at the (L-1)^3 inside nodes, 18 on faces, 12 on edges, 8 at corners = (3L+1)^3
    for L in range(1, 17):
        assert bench.stencil_fma_per_element(L) == (3 * L + 1) ** 3
    assert bench.stencil_fma_per_element(4) == 2197
