"""bench.py pieces that run without a GPU: the reference arm (the oracle on the host) and the
algorithmic byte model of the solve."""

import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_json_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--config", "cube",
                          "--steps", "2", "--warmup", "1"], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert out.returncode == 0, out.stderr
    lines = [l for l in out.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "tet-element-steps/s" and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] == 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["steps"] == 2


def test_byte_model_matches_formula():
    sys.path.insert(0, ROOT)
    import bench

    nnz, N = 30865689, 270641
    n = 3 * N
    assert bench.bytes_per_iteration(nnz, N, 4) == nnz * 4 + (nnz // 9) * 4 + 4 * (N + 1) + 40 * n
    assert bench.bytes_per_refresh(nnz, N, 4) == nnz * 4 + (nnz // 9) * 4 + 4 * (N + 1) + 24 * n
