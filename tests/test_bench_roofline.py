"""bench.py's adjoint roofline on the host: the measured bf16 peak when its file is
present, the fallback figure when it is not."""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_adjoint_roofline_uses_the_measured_peak(monkeypatch, tmp_path):
    (tmp_path / "MEASURED_PEAKS.json").write_text(json.dumps({"bf16_tflops": 2000.0}))
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    r = bench.adjoint_roofline(1000.0, 2500.0)
    assert r["bound"] == "tensor" and r["unit"] == "TFLOP/s" and r["kernel"] == "adjoint_tc_kernel"
    assert r["peak"] == 2000.0 and r["frac"] == 0.5 and "MEASURED_PEAKS.json" in r["peak_source"]
    assert r["frac_of_mma_loop_rate"] == 0.4


def test_adjoint_roofline_falls_back_without_measured_peaks(monkeypatch, tmp_path):
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    r = bench.adjoint_roofline(950.0, 0.0)
    assert r["peak"] == 1900.0 and r["frac"] == 0.5 and "fallback" in r["peak_source"]
    assert r["frac_of_mma_loop_rate"] is None


def test_adjoint_roofline_reports_the_algorithmic_fp32_fraction(monkeypatch, tmp_path):
    (tmp_path / "MEASURED_PEAKS.json").write_text(json.dumps({"bf16_tflops": 2000.0}))
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    r = bench.adjoint_roofline(1200.0, 2400.0, 400.0)
    assert r["frac"] == 0.6 and r["frac_of_mma_loop_rate"] == 0.5
    assert r["algorithmic_fp32"]["achieved"] == 400.0
    assert r["algorithmic_fp32"]["frac"] == 0.2 and r["algorithmic_fp32"]["frac_of_mma_loop_rate"] == round(400 / 2400, 4)
