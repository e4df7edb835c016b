"""Certified FP32 distance-type decisions (csrc/cert.cuh) against the FP64
classifiers (csrc/geom.cuh), on the host.

The FP64 ACCD kernel decides each step's point-triangle / edge-edge distance
type and its gap test with FP32 midpoint-radius enclosures of the FP64
operation sequence and falls back to FP64 when an enclosure straddles a
threshold.  Bar: over 1.6M random and constructed boundary configurations no
certain decision differs from the FP64 one (any difference would break the
kernel's bit-exactness); random configurations are decided (not deferred) for
at least 99% of point-triangle and 70% of edge-edge cases (the edge-edge set
deliberately holds a quarter of near-parallel pairs).
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_certified_types_agree_with_fp64(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "cert_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", os.path.join(HERE, "native", "cert_check.cpp"),
                    "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    rows = {}
    for line in out.stdout.splitlines():
        name, v, bound = line.split()
        rows[name] = (float(v), float(bound))
    for k in ("pt_random", "pt_boundary", "ee_random", "ee_boundary", "gap"):
        assert rows[k + "_wrong"][0] == 0, (k, out.stderr)
    for name, (v, bound) in rows.items():
        assert v <= bound, (name, v, bound)
    assert out.returncode == 0, out.stderr
