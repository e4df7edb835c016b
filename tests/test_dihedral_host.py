"""Hinge-bending Hessian forms (csrc/elements.cuh), on the host.

The mixed-precision bending kernel forms the Hessian of the dihedral angle in
FP32 (dihedral_hess_t<float>) from FP64 edge vectors; the FP64 kernel keeps
dihedral_hess.  Bars over 20000 seeded cloth-like hinges (edges 1e-3..1e-1 m,
angles up to ~170 degrees), relative Frobenius error against dihedral_hess:
the template in FP64 1e-11 (the same expressions), in FP32 2e-3; dihedral_hess
against central differences of dihedral_grad 1e-5.
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_dihedral_hessian_forms(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "dihedral_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", os.path.join(HERE, "native", "dihedral_check.cpp"),
                    "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    for line in out.stdout.splitlines():
        name, v, bound = line.split()
        assert float(v) <= float(bound), line
    assert out.returncode == 0, out.stdout + out.stderr
