"""The C-ABI library loads and exports every entry point declared in include/cipc.h."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = []
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            with open(os.path.join(ROOT, "include", h)) as f:
                src = f.read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names += re.findall(r"\b(cipc_\w+)\s*\(", src)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    import build_lib
    import cipc_ffi
    build_lib.build()
    L = ctypes.CDLL(cipc_ffi.LIB_PATH)
    declared = _declared()
    assert len(declared) >= 6
    for name in declared:
        assert hasattr(L, name), name
    # the Python binding declares a signature for every entry point
    assert set(declared) <= set(cipc_ffi.exported_symbols())


def _prototypes():
    """name -> (return type, [parameter types]) of every cipc_* prototype in include/*.h."""
    out = {}
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h"):
            continue
        with open(os.path.join(ROOT, "include", h)) as f:
            src = re.sub(r"/\*.*?\*/", "", f.read(), flags=re.S)
        for m in re.finditer(r"([\w\s\*]+?)\b(cipc_\w+)\s*\(([^;{]*?)\)\s*;", src):
            params = [p.strip() for p in m.group(3).split(",") if p.strip() and p.strip() != "void"]
            out[m.group(2)] = (m.group(1).split()[-1], params)
    return out


def _kind_c(decl):
    """Coarse ABI class of a C parameter declaration."""
    if "*" in decl:
        return "ptr"
    t = decl.replace("const", "").split()[0]
    return {"int64_t": "i64", "uint64_t": "i64", "int": "i32", "int32_t": "i32", "uint32_t": "i32",
            "double": "f64", "float": "f32"}.get(t, t)


def _kind_ctypes(t):
    if t in (ctypes.c_int64, ctypes.c_longlong, ctypes.c_uint64, ctypes.c_ulonglong):
        return "i64"
    if t in (ctypes.c_int, ctypes.c_int32, ctypes.c_uint32):
        return "i32"
    if t is ctypes.c_double:
        return "f64"
    if t is ctypes.c_float:
        return "f32"
    return "ptr"  # c_void_p, c_char_p and POINTER(...)


def test_ctypes_signatures_match_header():
    # a drift between include/cipc.h and the ctypes table would pass arguments in
    # the wrong registers without any error; compare count and kind of every one
    import cipc_ffi
    protos = _prototypes()
    assert set(_declared()) <= set(protos)
    for name, (_, params) in protos.items():
        args = cipc_ffi._SIGS[name][1]
        assert len(args) == len(params), (name, params, args)
        for decl, t in zip(params, args):
            assert _kind_c(decl) == _kind_ctypes(t), (name, decl, t)


def test_struct_layouts_match_header(tmp_path):
    # the ctypes mirrors of the ABI structs must have the C compiler's field
    # offsets and sizes: a C program built against include/cipc.h prints them
    import shutil
    import subprocess

    import cipc_ffi
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        import pytest
        pytest.skip("no C compiler")
    structs = {"cipc_step_params": cipc_ffi.StepParams, "cipc_step_stats": cipc_ffi.StepStats,
               "cipc_codim_desc": cipc_ffi.CodimDesc, "cipc_tet_desc": cipc_ffi.TetDesc}
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "cipc.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append('printf("%s sizeof %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in py._fields_:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines += ["return 0; }"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = str(tmp_path / "layout")
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", exe], check=True)
    got = {}
    for line in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.splitlines():
        cname, field, v = line.split()
        got[(cname, field)] = int(v)
    for cname, py in structs.items():
        assert got[(cname, "sizeof")] == ctypes.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)


def test_host_only_entry_points():
    import cipc_ffi
    assert cipc_ffi.lib().cipc_version().startswith(b"cipc-gb300")
    assert cipc_ffi.lib().cipc_status_string(0) == b"ok"
    # reference constraint codes (IPC.h:571-661)
    assert list(cipc_ffi.encode_reference_constraint(2, [5, 1, 2, 3])) == [-6, 1, 2, 3]
    assert list(cipc_ffi.encode_reference_constraint(1, [5, 1, 2, -1], multiplicity=2)) == [-6, 1, 2, -2]
    assert list(cipc_ffi.encode_reference_constraint(0, [5, 1, -1, -1])) == [-6, 1, -1, -1]
    assert list(cipc_ffi.encode_reference_constraint(3, [5, 1, 2, 3], mollified=True)) == [5, 1, -3, 3]


def test_argument_validation_without_gpu():
    import cipc_ffi
    t = np.zeros(1, np.uint8)
    idx = np.zeros((1, 4), np.int32)
    x = np.zeros((2, 3))
    toc = np.zeros(1)
    hit = np.zeros(1, np.uint8)
    # invalid eta is rejected before any device work
    try:
        cipc_ffi.ccd_pairs(t, idx, x, x, toc, hit, eta=1.5)
        raise AssertionError("expected an error")
    except cipc_ffi.CipcError as e:
        assert e.status == cipc_ffi.CIPC_ERR_INVALID_ARG
    # empty input is a no-op
    e0 = np.zeros(0, np.uint8)
    st, ov = cipc_ffi.ccd_pairs(e0, np.zeros((0, 4), np.int32), x, x, np.zeros(0), np.zeros(0, np.uint8))
    assert st == 0 and ov == 0


def test_noalloc_argument_validation_without_gpu():
    """Slot and argument checks of cipc_ccd_pairs_noalloc run before any device work."""
    import cipc_ffi
    t = np.zeros(1, np.uint8)
    idx = np.zeros((1, 4), np.int32)
    x = np.zeros((2, 3))
    toc = np.zeros(1)
    hit = np.zeros(1, np.uint8)
    L = cipc_ffi.lib()

    def raw(n, eta=0.1, precision=0, slot=0):
        # straight through the C ABI: the binding itself refuses host buffers for a device call
        return L.cipc_ccd_pairs_noalloc(n, t.ctypes.data, idx.ctypes.data, 2, x.ctypes.data, x.ctypes.data, eta,
                                        0.0, 1.0, precision, slot, toc.ctypes.data, hit.ctypes.data, None, None)

    for kw in (dict(slot=-1), dict(slot=cipc_ffi.NOALLOC_SLOTS), dict(eta=0.0), dict(precision=7)):
        assert raw(1, **kw) == cipc_ffi.CIPC_ERR_INVALID_ARG, kw
    assert raw(0, slot=cipc_ffi.NOALLOC_SLOTS - 1) == cipc_ffi.CIPC_OK


def test_binding_checks_pair_buffers():
    """The Python binding rejects buffers of the wrong dtype, shape or placement
    before they reach a kernel (a float32 vertex array or an (n, 2) index array
    would otherwise be read past its end on the device)."""
    import cipc_ffi
    n, nv = 3, 8
    t = np.zeros(n, np.uint8)
    idx = np.zeros((n, 4), np.int32)
    x = np.zeros((nv, 3))
    toc = np.zeros(n)
    hit = np.zeros(n, np.uint8)
    bad = [dict(x=x.astype(np.float32)), dict(idx=np.zeros((n, 2), np.int32)), dict(dx=np.zeros((nv - 1, 3))),
           dict(toc_out=np.zeros(n, np.float32)), dict(hit=np.zeros(n + 1, np.uint8)),
           dict(type_=np.zeros(n, np.int32)), dict(x=np.zeros((nv, 3))[:, :2].copy())]
    for b in bad:
        args = dict(type_=t, idx=idx, x=x, dx=x, toc_out=toc, hit=hit)
        args.update(b)
        with pytest.raises((TypeError, ValueError)):
            cipc_ffi.ccd_pairs(**args)
    # host arrays are refused by the device-memory entry points
    for fn in (cipc_ffi.ccd_pairs_async, cipc_ffi.ccd_pairs_noalloc):
        with pytest.raises(ValueError):
            fn(t, idx, x, x, toc, hit)
    with pytest.raises(ValueError):
        cipc_ffi.ccd_pairs(t, idx, x, x, toc, hit, mem=cipc_ffi.MEM_DEVICE)
    E = np.zeros(n)
    g = np.zeros((n, 12))
    with pytest.raises(TypeError):  # FP64 needs a double Hessian
        cipc_ffi.barrier_pairs(t, idx, x, x, E, g, np.zeros((n, 78), np.float32), 1e-4, 1e-7, 1.0, True,
                               cipc_ffi.FP64)
    with pytest.raises(ValueError):
        cipc_ffi.barrier_pairs(t, idx, x, x, E, np.zeros((n, 9)), np.zeros((n, 78), np.float32), 1e-4, 1e-7, 1.0,
                               True, cipc_ffi.MIXED)


def test_fails_loudly_without_gpu_or_library():
    """The product path has no CPU fallback: without a CUDA device a compute call
    returns CIPC_ERR_NO_DEVICE, and without the built library the binding raises."""
    import subprocess
    import sys

    import cipc_ffi
    if cipc_ffi.lib().cipc_device_count() == 0:
        t = np.zeros(1, np.uint8)
        idx = np.array([[0, 1, -1, -1]], np.int32)
        x = np.zeros((2, 3))
        try:
            cipc_ffi.ccd_pairs(t, idx, x, x + 1.0, np.zeros(1), np.zeros(1, np.uint8))
            raise AssertionError("expected an error without a device")
        except cipc_ffi.CipcError as e:
            assert e.status == cipc_ffi.CIPC_ERR_NO_DEVICE
    code = ("import sys; sys.path.insert(0, %r); import cipc_ffi\n"
            "cipc_ffi.LIB_PATH = '/nonexistent/libcipc.so'; cipc_ffi._lib = None\n"
            "try:\n    cipc_ffi.lib()\nexcept ImportError as e:\n    print('raised', e)\n"
            % os.path.join(ROOT, "codim-ipc_gb300"))
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120)
    assert out.stdout.startswith("raised"), out.stdout + out.stderr
