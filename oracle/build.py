"""Build recipe for the CPU oracle (test infrastructure only).

``build_oracle()`` compiles this directory's C++ restatement into
``oracle/liboracle.so`` (OpenMP, ``-ffp-contract=off``: the oracle's explicit
``fma`` calls are the only fused operations).

``build_ref()`` compiles pieces of the reference itself into
``oracle/_ref/libcipc_ref.so`` when the Codim-IPC sources are available.  The
reference as a whole needs Eigen, Boost, SuiteSparse and Kokkos and cannot be
built here, but its symbolic-toolbox derivative routines (``g_PT``, ``H_PT``,
``g_EE``, ``H_EE``, ``g_PE3D``, ``H_PE3D``, ``g_EECN2``, ``H_EECN2``, the rod's
``g_MS``/``H_MS``/``g_RB``/``H_RB``), its contact barrier functions and its
strain-limiting barrier (``f/g/h_sl_u``, ``f/g/h_sl_l`` of INEXT.h), friction
mollifier (``f0_SF``, ``f1_SF_Div_RelDXNorm``, ``f2_SF_Term``), edge-edge
mollifier (``EEM``, ``g_EEM``, ``H_EEM``) and dihedral-angle derivatives
(``g_DA``, ``H_DA``) are plain scalar C++.  They are cut out of the headers where
they lie and piped straight into g++ (nothing is written to disk but the .so),
so the oracle's own derivation can be pinned against them.
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("CIPC_REFERENCE_ROOT", "/root/reference")


def build_oracle(force=False):
    out = os.path.join(HERE, "liboracle.so")
    srcs = [os.path.join(HERE, f) for f in ("oracle_math.cpp", "oracle_api.cpp", "oracle_shell.cpp", "oracle_learned.cpp", "oracle_rod.cpp", "oracle_sl.cpp", "oracle_tet.cpp")]
    srcs = [s for s in srcs if os.path.exists(s)]
    deps = srcs + [os.path.join(HERE, f) for f in os.listdir(HERE) if f.endswith(".h")]
    if not force and os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        return out
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-o", out] + srcs
    subprocess.check_call(cmd)
    return out


# (file, function name, kind) — kind "tmplT": `template <class T> void f(...) {...}`
_REF_FUNCS = [
    ("Library/Math/Distance/POINT_EDGE.h", "g_PE3D"),
    ("Library/Math/Distance/POINT_EDGE.h", "H_PE3D"),
    ("Library/Math/Distance/POINT_TRIANGLE.h", "g_PT"),
    ("Library/Math/Distance/POINT_TRIANGLE.h", "H_PT"),
    ("Library/Math/Distance/EDGE_EDGE.h", "g_EE"),
    ("Library/Math/Distance/EDGE_EDGE.h", "H_EE"),
    ("Library/Math/Distance/EDGE_EDGE_MOLLIFIER.h", "g_EECN2"),
    ("Library/Math/Distance/EDGE_EDGE_MOLLIFIER.h", "H_EECN2"),
    ("Library/Math/BARRIER.h", "Barrier"),
    ("Library/Math/BARRIER.h", "Barrier_Gradient"),
    ("Library/Math/BARRIER.h", "Barrier_Hessian"),
    ("Library/FEM/Shell/Rod/MASS_SPRING_DERIVATIVES.h", "g_MS"),
    ("Library/FEM/Shell/Rod/MASS_SPRING_DERIVATIVES.h", "H_MS"),
    ("Library/FEM/Shell/Rod/ROD_BENDING_DERIVATIVES.h", "g_RB"),
    ("Library/FEM/Shell/Rod/ROD_BENDING_DERIVATIVES.h", "H_RB"),
    ("Library/FEM/Shell/INEXT.h", "f_sl_u"),
    ("Library/FEM/Shell/INEXT.h", "g_sl_u"),
    ("Library/FEM/Shell/INEXT.h", "h_sl_u"),
    ("Library/FEM/Shell/INEXT.h", "f_sl_l"),
    ("Library/FEM/Shell/INEXT.h", "g_sl_l"),
    ("Library/FEM/Shell/INEXT.h", "h_sl_l"),
    ("Library/FEM/FRICTION_UTILS.h", "f0_SF"),
    ("Library/FEM/FRICTION_UTILS.h", "f1_SF_Div_RelDXNorm"),
    ("Library/FEM/FRICTION_UTILS.h", "f2_SF_Term"),
    ("Library/Math/DIHEDRAL_ANGLE.h", "g_DA"),
    ("Library/Math/DIHEDRAL_ANGLE.h", "H_DA"),
    ("Library/Math/Distance/EDGE_EDGE_MOLLIFIER.h", "EEM"),
    ("Library/Math/Distance/EDGE_EDGE_MOLLIFIER.h", "g_EEM"),
    ("Library/Math/Distance/EDGE_EDGE_MOLLIFIER.h", "H_EEM"),
]


def _extract(text, name):
    """Return `template <...> ... name(...) { ... }` cut from text by brace matching."""
    m = re.search(r"template\s*<[^>]*>\s*(?:inline\s+)?(?:void|T)\s+" + re.escape(name) + r"\s*\(", text)
    if not m:
        raise RuntimeError("function %s not found" % name)
    start = m.start()
    i = text.index("{", m.end())
    depth = 0
    for j in range(i, len(text)):
        if text[j] == "{":
            depth += 1
        elif text[j] == "}":
            depth -= 1
            if depth == 0:
                return text[start:j + 1]
    raise RuntimeError("unbalanced braces in %s" % name)


def build_ref(force=False):
    """Compile the reference's scalar derivative/barrier routines (see module doc)."""
    if not os.path.isdir(REF_ROOT):
        return None
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    out = os.path.join(outdir, "libcipc_ref.so")
    if os.path.exists(out) and not force:
        return out
    parts = ["#include <cmath>\n#include <algorithm>\nusing std::pow; using std::sqrt; using std::log;\n"
             "namespace ref {\n"]
    cache = {}
    for f, name in _REF_FUNCS:
        if f not in cache:
            with open(os.path.join(REF_ROOT, f)) as fh:
                cache[f] = fh.read()
        parts.append(_extract(cache[f], name) + "\n")
    parts.append("}\n")
    args12 = ", ".join("x[%d]" % k for k in range(12))
    args9 = ", ".join("x[%d]" % k for k in range(9))
    args6 = ", ".join("x[%d]" % k for k in range(6))
    parts.append('extern "C" {\n'
                 "void ref_g_PT(const double* x, double* g) { ref::g_PT<double>(%s, g); }\n"
                 "void ref_H_PT(const double* x, double* H) { ref::H_PT<double>(%s, H); }\n"
                 "void ref_g_EE(const double* x, double* g) { ref::g_EE<double>(%s, g); }\n"
                 "void ref_H_EE(const double* x, double* H) { ref::H_EE<double>(%s, H); }\n"
                 "void ref_g_PE3D(const double* x, double* g) { ref::g_PE3D<double>(%s, g); }\n"
                 "void ref_H_PE3D(const double* x, double* H) { ref::H_PE3D<double>(%s, H); }\n"
                 "void ref_g_EECN2(const double* x, double* g) { ref::g_EECN2<double>(%s, g); }\n"
                 "void ref_H_EECN2(const double* x, double* H) { ref::H_EECN2<double>(%s, H); }\n"
                 "void ref_barrier(double d, double dHat, double kappa, double* out) {\n"
                 "  double k[3] = {kappa, 0, 0};\n"
                 "  ref::Barrier<false>(d, dHat, k, out[0]);\n"
                 "  ref::Barrier_Gradient<false>(d, dHat, k, out[1]);\n"
                 "  ref::Barrier_Hessian<false>(d, dHat, k, out[2]); }\n"
                 "void ref_barrier_elastic(double d, double dHat, double kappa, double* out) {\n"
                 "  double k[3] = {kappa, 0, 0};\n"
                 "  ref::Barrier<true>(d, dHat, k, out[0]);\n"
                 "  ref::Barrier_Gradient<true>(d, dHat, k, out[1]);\n"
                 "  ref::Barrier_Hessian<true>(d, dHat, k, out[2]); }\n"
                 "void ref_g_MS(double k, double l, const double* x, double* g) { ref::g_MS<double>(k, l, %s, g); }\n"
                 "void ref_H_MS(double k, double l, const double* x, double* H) { ref::H_MS<double>(k, l, %s, H); }\n"
                 "void ref_g_RB(const double* x, double* g) { ref::g_RB<double>(%s, g); }\n"
                 "void ref_H_RB(const double* x, double* H) { ref::H_RB<double>(%s, H); }\n"
                 "void ref_sl(double s, double slim, double shat, double* out) {\n"
                 "  out[0] = ref::f_sl_u<double>(s, slim, shat); out[1] = ref::g_sl_u<double>(s, slim, shat);\n"
                 "  out[2] = ref::h_sl_u<double>(s, slim, shat); out[3] = ref::f_sl_l<double>(s, slim, shat);\n"
                 "  out[4] = ref::g_sl_l<double>(s, slim, shat); out[5] = ref::h_sl_l<double>(s, slim, shat); }\n"
                 "void ref_g_DA(const double* x, double* g) { ref::g_DA<double>(%s, g); }\n"
                 "void ref_H_DA(const double* x, double* H) { ref::H_DA<double>(%s, H); }\n"
                 "void ref_eem(double c, double eps, double* out) {\n"
                 "  ref::EEM<double>(c, eps, out[0]); ref::g_EEM<double>(c, eps, out[1]);\n"
                 "  ref::H_EEM<double>(c, eps, out[2]); }\n"
                 "void ref_friction(double x2, double eh, double* out) {\n"
                 "  ref::f0_SF<double>(x2, eh, out[0]); ref::f1_SF_Div_RelDXNorm<double>(x2, eh, out[1]);\n"
                 "  ref::f2_SF_Term<double>(x2, eh, out[2]); }\n"
                 "}\n" % (args12, args12, args12, args12, args9, args9, args12, args12, args6, args6, args9, args9,
                           args12, args12))
    src = "".join(parts)
    cmd = ["g++", "-O1", "-std=c++17", "-fPIC", "-shared", "-x", "c++", "-", "-o", out]
    subprocess.run(cmd, input=src.encode(), check=True)
    return out


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
