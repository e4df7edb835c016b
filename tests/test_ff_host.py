"""Float-float helpers of the mixed-precision ACCD kernel (csrc/ff.cuh), checked
on the host: the header is compiled with the device intrinsics mapped to IEEE
single-precision host operations, and the integer split of FP64 values, the
sums, products and fused multiply-adds are compared with long double results.

Bars: split relative error <= 2^-46 (24 + 23 significant bits kept); sum and
fused multiply-add absolute error <= 2^-45 / 2^-44 of the operand magnitudes;
product relative error <= 2^-44; zero and FP64 subnormals map to zero.
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_ff_arithmetic_bounds(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "ff_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", os.path.join(HERE, "native", "ff_check.cpp"),
                    "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    rows = {}
    for line in out.stdout.splitlines():
        name, v, bound = line.split()
        rows[name] = (float(v), float(bound))
    assert set(rows) == {"split_rel", "sub_abs_over_magnitudes", "mul_rel", "fma_abs_over_magnitudes",
                         "special_value_failures"}
    for name, (v, bound) in rows.items():
        assert v <= bound, (name, v, bound)
    assert out.returncode == 0
