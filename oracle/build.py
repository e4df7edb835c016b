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
import platform
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


# The reference's distance-type, distance and ACCD routines, in the order they
# depend on each other: (file, function, text its signature must contain).
_REF_CCD_FUNCS = [
    ("Library/Math/Distance/POINT_POINT.h", "Point_Point_Distance", ""),
    ("Library/Math/Distance/POINT_EDGE.h", "Point_Edge_Distance", ""),
    ("Library/Math/Distance/POINT_TRIANGLE.h", "Point_Triangle_Distance", ""),
    ("Library/Math/Distance/EDGE_EDGE.h", "Edge_Edge_Distance", ""),
    ("Library/Math/Distance/DISTANCE_TYPE.h", "Point_Edge_Distance_Type", ""),
    ("Library/Math/Distance/DISTANCE_TYPE.h", "Point_Triangle_Distance_Type", ""),
    ("Library/Math/Distance/DISTANCE_TYPE.h", "Edge_Edge_Distance_Type", ""),
    ("Library/Math/Distance/DISTANCE_UNCLASSIFIED.h", "Point_Triangle_Distance_Unclassified", ""),
    ("Library/Math/Distance/DISTANCE_UNCLASSIFIED.h", "Edge_Edge_Distance_Unclassified", ""),
    ("Library/Math/Distance/DISTANCE_UNCLASSIFIED.h", "Point_Edge_Distance_Unclassified", ""),
    ("Library/Math/Distance/CCD.h", "Point_Triangle_CCD", ""),
    ("Library/Math/Distance/CCD.h", "Edge_Edge_CCD", ""),
    ("Library/Math/Distance/CCD.h", "Point_Edge_CCD", "Matrix<T, 3, 1>"),
    ("Library/Math/Distance/CCD.h", "Point_Point_CCD", ""),
]

# flags of the reference's own build: build.py configures CMAKE_BUILD_TYPE=Release
# (-O3 -DNDEBUG) and CMakeLists.txt:20 adds -mfma -mbmi2 -mavx2 (x86 only).  The
# vectorizer is turned off: GCC vectorizes the shim's small loops in some call
# sites and not others (in the point-edge ACCD it then fuses one norm's products
# in the other order), which says nothing about how real Eigen's code would be
# vectorized; with it off the compiled reference is one consistent contraction
# policy, the one the oracle and the CUDA kernels follow.
_REF_FLAGS_X86 = ["-O3", "-DNDEBUG", "-mfma", "-mbmi2", "-mavx2", "-fno-tree-vectorize"]


def _extract_def(text, name, must):
    """`template <...> <ret> name(...) {...}` whose signature contains `must`."""
    for m in re.finditer(r"template\s*<[^>]*>\s*(?:inline\s+)?(?:void|T|int|bool)\s+" + re.escape(name) + r"\s*\(",
                         text):
        i = text.index("{", m.end())
        if must and must not in text[m.end():i]:
            continue
        depth = 0
        j = i
        while j < len(text):
            if text.startswith("//", j):  # braces in comments do not count
                j = text.index("\n", j)
                continue
            if text.startswith("/*", j):
                j = text.index("*/", j) + 2
                continue
            if text[j] == "{":
                depth += 1
            elif text[j] == "}":
                depth -= 1
                if depth == 0:
                    return text[m.start():j + 1]
            j += 1
    raise RuntimeError("function %s not found" % name)


def build_ref_ccd(force=False):
    """Compile the reference's own distance-type classification, unclassified
    distances and additive CCD (DISTANCE_TYPE.h, DISTANCE_UNCLASSIFIED.h,
    POINT_*.h, EDGE_EDGE.h, CCD.h:279-483) against oracle/eigen_shim.h with the
    reference's build flags into oracle/_ref/libcipc_ref_ccd.so (x86 hosts; the
    functions are cut out of the headers and piped into g++, nothing else is
    written).  Returns None when the sources or an x86 compiler are absent."""
    if not os.path.isdir(REF_ROOT) or platform.machine() not in ("x86_64", "AMD64"):
        return None
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    out = os.path.join(outdir, "libcipc_ref_ccd.so")
    shim = os.path.join(HERE, "eigen_shim.h")
    if os.path.exists(out) and not force and os.path.getmtime(out) >= os.path.getmtime(shim):
        return out
    parts = ['#include "%s"\n#include <cstdint>\nnamespace ref {\n' % shim]
    cache = {}
    for f, name, must in _REF_CCD_FUNCS:
        if f not in cache:
            with open(os.path.join(REF_ROOT, f)) as fh:
                cache[f] = fh.read()
        parts.append(_extract_def(cache[f], name, must) + "\n")
    parts.append("}\n")
    parts.append(r"""
typedef Eigen::Matrix<double, 3, 1> V3;
static V3 v3(const double* p) { V3 r; r.a[0] = p[0]; r.a[1] = p[1]; r.a[2] = p[2]; return r; }
extern "C" {
int refc_pt_type(const double* x) { return ref::Point_Triangle_Distance_Type(v3(x), v3(x + 3), v3(x + 6), v3(x + 9)); }
int refc_ee_type(const double* x) { return ref::Edge_Edge_Distance_Type(v3(x), v3(x + 3), v3(x + 6), v3(x + 9)); }
int refc_pe_type(const double* x) { double r; return ref::Point_Edge_Distance_Type<double, 3>(v3(x), v3(x + 3), v3(x + 6), r); }
double refc_pt_d2(const double* x) { double d; ref::Point_Triangle_Distance_Unclassified(v3(x), v3(x + 3), v3(x + 6), v3(x + 9), d); return d; }
double refc_ee_d2(const double* x) { double d; ref::Edge_Edge_Distance_Unclassified(v3(x), v3(x + 3), v3(x + 6), v3(x + 9), d); return d; }
double refc_pe_d2(const double* x) { double d; ref::Point_Edge_Distance_Unclassified(v3(x), v3(x + 3), v3(x + 6), d); return d; }
// ACCD over pairs (type 0 PP, 1 PE, 2 PT, 3 EE; four vertex indices each); a
// miss reports toc_in, as the C ABI does (the reference leaves toc undefined then)
void refc_ccd_pairs(int64_t n, const uint8_t* type, const int32_t* idx, const double* x, const double* dx,
                    double eta, double th, double toc_in, double* toc_out, uint8_t* hit)
{
    for (int64_t i = 0; i < n; ++i) {
        const int32_t* id = idx + 4 * i;
        double toc = toc_in;
        bool h = false;
        switch (type[i]) {
            case 0: h = ref::Point_Point_CCD(v3(x + 3 * id[0]), v3(x + 3 * id[1]), v3(dx + 3 * id[0]), v3(dx + 3 * id[1]), eta, th, toc); break;
            case 1: h = ref::Point_Edge_CCD(v3(x + 3 * id[0]), v3(x + 3 * id[1]), v3(x + 3 * id[2]), v3(dx + 3 * id[0]), v3(dx + 3 * id[1]), v3(dx + 3 * id[2]), eta, th, toc); break;
            case 2: h = ref::Point_Triangle_CCD(v3(x + 3 * id[0]), v3(x + 3 * id[1]), v3(x + 3 * id[2]), v3(x + 3 * id[3]), v3(dx + 3 * id[0]), v3(dx + 3 * id[1]), v3(dx + 3 * id[2]), v3(dx + 3 * id[3]), eta, th, toc); break;
            default: h = ref::Edge_Edge_CCD(v3(x + 3 * id[0]), v3(x + 3 * id[1]), v3(x + 3 * id[2]), v3(x + 3 * id[3]), v3(dx + 3 * id[0]), v3(dx + 3 * id[1]), v3(dx + 3 * id[2]), v3(dx + 3 * id[3]), eta, th, toc); break;
        }
        hit[i] = h ? 1 : 0;
        toc_out[i] = h ? toc : toc_in;
    }
}
}
""")
    src = "".join(parts)
    cmd = ["g++", "-std=c++17", "-fPIC", "-shared"] + _REF_FLAGS_X86 + ["-x", "c++", "-", "-o", out]
    subprocess.run(cmd, input=src.encode(), check=True)
    return out


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
    print(build_ref_ccd(force="--force" in sys.argv))
