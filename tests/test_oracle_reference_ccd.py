"""The oracle's distance-type decisions, unclassified distances and additive
CCD pinned bit for bit to the reference's own source.

tests/golden/reference_ccd.npz holds outputs of the reference's
Point_Triangle_Distance_Type / Edge_Edge_Distance_Type / Point_Edge_Distance_Type
(DISTANCE_TYPE.h:11-164), *_Distance_Unclassified (DISTANCE_UNCLASSIFIED.h) and
Point_Triangle_CCD / Edge_Edge_CCD / Point_Edge_CCD / Point_Point_CCD
(CCD.h:279-483), compiled from the Codim-IPC sources against oracle/eigen_shim.h
with the reference's build flags (-O3 -mfma, GCC's contraction; vectorizer off)
by tests/golden/make_golden_ccd.py.  Bar: every type, every squared distance,
every hit/miss decision and every time of impact bit-identical (the stated
contraction policy is the one the oracle and the CUDA kernels follow).  Where
the compiled reference itself is present (oracle/_ref), 100k more seeded pairs
are compared directly.  The GPU test holds the FP64 kernel to the same fixture.
"""
import ctypes
import os

import numpy as np
import pytest

import workloads

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLD = os.path.join(HERE, "golden", "reference_ccd.npz")
REF_SO = os.path.join(ROOT, "oracle", "_ref", "libcipc_ref_ccd.so")


def _bits(a):
    return np.ascontiguousarray(a, np.float64).view(np.uint64)


def test_types_and_distances_match_reference(orc):
    d = np.load(GOLD)
    cfg = d["cfg"]
    for i in range(cfg.shape[0]):
        x = np.ascontiguousarray(cfg[i])
        assert orc.pt_type(x) == d["pt_type"][i], i
        assert orc.ee_type(x) == d["ee_type"][i], i
        assert orc.pe_type(x[:9]) == d["pe_type"][i], i
    pt = np.array([orc.d2(5, np.ascontiguousarray(c)) for c in cfg])
    ee = np.array([orc.d2(6, np.ascontiguousarray(c)) for c in cfg])
    pe = np.array([orc.d2(7, np.ascontiguousarray(c[:9])) for c in cfg])
    assert np.array_equal(_bits(pt), _bits(d["pt_d2"]))
    assert np.array_equal(_bits(ee), _bits(d["ee_d2"]))
    assert np.array_equal(_bits(pe), _bits(d["pe_d2"]))
    # every region of both classifiers is exercised
    assert set(np.unique(d["pt_type"])) == set(range(7))
    assert set(np.unique(d["ee_type"])) == set(range(9))


@pytest.mark.parametrize("batch", ["b0", "b1", "b2"])
def test_accd_matches_reference(orc, batch):
    d = np.load(GOLD)
    eta, th, toc_in = d[batch + "_params"]
    toc, hit, _, ov = orc.ccd_pairs(d[batch + "_type"], d[batch + "_idx"], d[batch + "_x"], d[batch + "_dx"], eta,
                                    th, toc_in)
    assert ov == 0
    assert 0 < d[batch + "_hit"].sum() < d[batch + "_hit"].size
    assert np.array_equal(hit, d[batch + "_hit"])
    assert np.array_equal(_bits(toc), _bits(d[batch + "_toc"]))


@pytest.mark.skipif(not os.path.exists(REF_SO), reason="compiled reference (oracle/_ref) not present")
def test_accd_matches_compiled_reference_at_scale(orc):
    R = ctypes.CDLL(REF_SO)
    P = ctypes.c_void_p
    R.refc_ccd_pairs.argtypes = [ctypes.c_int64, P, P, P, P, ctypes.c_double, ctypes.c_double, ctypes.c_double, P, P]
    for seed, kw, th in ((31, {}, 1e-7), (32, dict(mix=(0.25, 0.25, 0.25, 0.25), sep_range=(1e-5, 1e-1)), 5e-6)):
        w = workloads.contact_pairs(100_000, seed=seed, **kw)
        n = w["type"].shape[0]
        toc = np.zeros(n)
        hit = np.zeros(n, np.uint8)
        R.refc_ccd_pairs(n, w["type"].ctypes.data, w["idx"].ctypes.data, w["x"].ctypes.data, w["dx"].ctypes.data,
                         0.1, th, 1.0, toc.ctypes.data, hit.ctypes.data)
        toc_o, hit_o, _, ov = orc.ccd_pairs(w["type"], w["idx"], w["x"], w["dx"], 0.1, th, 1.0)
        assert ov == 0
        assert np.array_equal(hit_o, hit)
        assert np.array_equal(_bits(toc_o), _bits(toc))


@pytest.mark.gpu
@pytest.mark.parametrize("batch", ["b0", "b1", "b2"])
def test_gpu_accd_matches_reference(cuda, batch):
    import cipc_ffi as F
    d = np.load(GOLD)
    eta, th, toc_in = d[batch + "_params"]
    n = d[batch + "_type"].shape[0]
    toc = np.zeros(n)
    hit = np.zeros(n, np.uint8)
    st, ov = F.ccd_pairs(np.ascontiguousarray(d[batch + "_type"]), np.ascontiguousarray(d[batch + "_idx"]),
                         np.ascontiguousarray(d[batch + "_x"]), np.ascontiguousarray(d[batch + "_dx"]), toc, hit,
                         eta=eta, thickness=th, toc_in=toc_in, precision=F.FP64)
    assert st == 0 and ov == 0
    assert np.array_equal(hit, d[batch + "_hit"])
    assert np.array_equal(_bits(toc), _bits(d[batch + "_toc"]))
