"""Host-side pieces of the bench's JSON line, checked without a GPU: the roofline
object picks the kernel kind with the most event time, divides its algorithmic
work per launch by its time per launch, and takes its denominator from the
right peak."""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402


def test_roofline_fp64_gemm_dominant():
    # kind -> (launches, total ms, total work); gemm_f64 has the most time
    prof = {"gemm_f64": (100, 50.0, 4.0e10), "permute": (10, 5.0, 1.0e9), "qr": (20, 10.0, 0.0),
            "gemm_tc": (0, 0.0, 0.0)}
    r = bench.roofline(prof, 2, fp64_peak=1.1)
    assert r["kernel"] == "gemm_f64" and r["bound"] == "fp64" and r["unit"] == "TFLOP/s"
    # 4e8 flop per launch in 0.5 ms -> 0.8 TFLOP/s
    assert r["achieved"] == pytest.approx(0.8)
    assert r["peak"] == 1.1 and r["frac"] == pytest.approx(0.8 / 1.1)
    assert r["launches_per_step"] == 50 and r["traffic"] == pytest.approx(14.10e6)


def test_roofline_hbm_and_tensor_kinds():
    r = bench.roofline({"permute": (4, 2.0, 8.0e9)}, 1)
    assert r["bound"] == "hbm" and r["unit"] == "GB/s"
    assert r["achieved"] == pytest.approx(2.0e9 / 0.5e-3 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"])
    t = bench.roofline({"gemm_tc": (2, 1.0, 2.0e11)}, 1)
    assert t["bound"] == "tensor" and t["achieved"] == pytest.approx(1.0e11 / 0.5e-3 / 1e12)
    assert bench.roofline({"permute": (0, 0.0, 0.0)}, 1) is None
