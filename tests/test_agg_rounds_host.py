"""Partition of the aggregates over the PCG kernel's blocks (csrc/agg_rounds.h),
on the host.

The aggregate block-Jacobi phase of the solver relies on it: every aggregate in
exactly one round of one block, every round within the shared-memory staging
(rows) and the round table (aggregates), and every aggregate's column items
within the kernel's shared slots.  Checked on seeded layouts (dense aggregates
of 1..32 vertices mixed with packs of isolated vertices, 1 to 4000 blocks, the
FP32 and FP64 limits); the blocks' costs stay within one aggregate of the mean.
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_aggregate_partition_invariants(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "agg_rounds_check")
    subprocess.run([cxx, "-O2", "-std=c++17", os.path.join(HERE, "native", "agg_rounds_check.cpp"), "-o", exe],
                   check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout[-4000:] + out.stderr
    assert "failures 0" in out.stdout
