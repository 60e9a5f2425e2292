"""bench.py on the CPU: the roofline arithmetic of its JSON line (bound unit,
fractions, algorithmic flop and byte models) and the reference arm, which
times the reference's CPU path on the host and prints one JSON line with the
contract's keys."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_flop_and_byte_models():
    # 24 n^3 per matrix plus 20 n^2 per QR sweep; read A, write V and the eigenvalues
    assert bench.fp64_flops(16, 0, 1) == 24.0 * 16 ** 3
    assert bench.fp64_flops(16, 53, 2) == 2 * 24.0 * 16 ** 3 + 20.0 * 256 * 53
    assert bench.hbm_bytes(16, 1) == 32.0 * 256 + 16.0 * 16
    assert bench.r4(1.234567) == 1.235 and bench.r4(7) == 7


def test_roofline_picks_the_slowest_unit(monkeypatch):
    monkeypatch.setattr(bench, "PEAKS", {"fp64": 1.0e12, "fp32": 64.0e12, "bf16": 2.0e15, "hbm": 8.0e12})
    rl = bench.roofline(2.0, fp64=1.0e12, fp32=8.0e12, hbm=1.0e12)
    # fp64: 0.5e12 / 1e12 = 0.5; fp32: 4e12 / 64e12 = 0.0625; hbm: 0.5e12 / 8e12 = 0.0625
    assert rl["bound"] == "fp64" and rl["unit"] == "TFLOP/s"
    assert rl["frac"] == pytest.approx(0.5) and rl["achieved"] == pytest.approx(0.5) and rl["peak"] == 1.0
    assert set(rl["fracs"]) == {"fp64", "fp32", "hbm"}
    rl = bench.roofline(1.0, fp64=1.0e9, hbm=4.0e12)
    assert rl["bound"] == "hbm" and rl["unit"] == "GB/s" and rl["frac"] == pytest.approx(0.5)


def test_reference_arm_json_line():
    """`bench.py --impl reference` on a small host sample: one JSON line with the
    reference arm's keys (the compiled reference when it was built here, else
    the oracle's restatement)."""
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--ref-sample", "4096"], capture_output=True, text=True, timeout=600,
                       cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "eigensolves/s"
    assert d["higher_is_better"] is True and d["steps"] == 1
    assert d["cpu_baseline"]["kind"] in ("reference", "port") and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["config"]["n"] == 16
