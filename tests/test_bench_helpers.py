"""Host-side helpers of bench.py (CPU): the roofline fractions added to the secondary
configurations of the JSON line."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_roofline_fractions_of_secondary_configurations():
    line = {
        "mixed": {"config": {}, "plain_fp64": {"ms": 1.0, "tflops": 1.1}, "bf16": {"tflops": 19.0},
                  "fp16": {"tflops": 95.0}},
        "batched": {"config": {}, "fp64": {"tflops": 0.5}, "fp32": {"tflops": 3.3},
                    "tuned": {"tflops": 3.5, "mode": "fp32"}, "cpu_baseline": {"value": 1.0}},
        "batched_mixed": {"config": {}, "plain_fp64_per_matrix": {"tflops": 0.2}, "fp16": {"tflops": 18.7},
                          "bf16": {"tflops": 15.9}, "fp8": {"tflops": 11.0},
                          "tuned": {"tflops": 19.0, "prec": "fp16"}},
        "config_small": {"gpu": {"tflops": 0.17}, "cpu_baseline": {"value": 0.4}},
        "potri": {"gpu": {"tflops": 0.67}},
    }
    bench.add_roofline_fractions(line, 1.1, 1928.0)
    assert abs(line["mixed"]["plain_fp64"]["frac_of_peak"] - 1.0) < 1e-12
    assert abs(line["mixed"]["fp16"]["frac_of_peak"] - 95.0 / 1928.0) < 1e-12
    assert abs(line["batched_mixed"]["fp8"]["frac_of_peak"] - 11.0 / 3856.0) < 1e-12
    assert abs(line["potri"]["gpu"]["frac_of_peak"] - 0.67 / 1.1) < 1e-12
    assert abs(line["batched_mixed"]["tuned"]["frac_of_peak"] - 19.0 / 1928.0) < 1e-12
    assert "frac_of_peak" not in line["batched"]["fp32"]           # CUDA-core FP32: no tensor roofline
    assert "frac_of_peak" not in line["batched"]["tuned"]
    assert "frac_of_peak" not in line["batched"]["cpu_baseline"]
    assert line["peaks"]["fp8_tflops"] == 3856.0


def test_measured_bf16_peak_has_a_source():
    peak, src = bench.measured_bf16_peak()
    assert peak > 100.0 and isinstance(src, str) and src


def test_tensor_roofline_counts_the_update_tasks():
    """One emulated update task issues 2 passes x 28 plane pairs x 2 chunks x 4 MMAs of 128 x 64 x 16."""
    assert bench.EMU_TASK_FLOPS == 2 * 28 * 2 * 4 * 2 * 128 * 64 * 16
    r = bench.tensor_roofline(256, 256, 1e-3, 1906.1, "test")  # 2 blocks: one SYRK, no GEMM
    assert r["update_tasks"] == 1 and r["flops_per_launch"] == bench.EMU_TASK_FLOPS
    r = bench.tensor_roofline(32768, 512, 1.0, 1906.1, "test")  # 256 blocks
    assert r["update_tasks"] == 256 * 255 // 2 + 256 * 255 * 254 // 6
    assert abs(r["frac"] - r["achieved"] / 1906.1) < 1e-12 and r["bound"] == "tensor"
