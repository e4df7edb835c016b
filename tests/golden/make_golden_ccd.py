"""Generates tests/golden/reference_ccd.npz from the reference's own code.

The reference's distance-type classification, unclassified distances and
additive CCD (Library/Math/Distance/DISTANCE_TYPE.h, DISTANCE_UNCLASSIFIED.h,
POINT_*.h, EDGE_EDGE.h, CCD.h:279-483) are compiled from the Codim-IPC sources
against oracle/eigen_shim.h with the reference's build flags
(``oracle/build.py:build_ref_ccd``); this script evaluates them on seeded inputs
and stores inputs and outputs, so that the oracle (and through it the CUDA
kernels) can be checked bit for bit on machines without the reference.

Inputs (small, so the fixture stays a few hundred KB):
  * ``cfg``: 3000 vertex quadruples -- 1000 uniform in the unit cube, 1000 with
    the point (resp. second edge) placed near the triangle plane (first edge) at
    separations 1e-9..1e-2 and barycentrics in [-0.3, 1.3], 1000 at scales
    1e-6..1e3 translated by up to 1e3 -- with their point-triangle and edge-edge
    types and unclassified squared distances, and the point-edge type and
    distance of their first three vertices;
  * three CCD batches of the contact-kernel benchmark generator: 2000 pairs
    (40/40/10/10, separations 1e-6..1e-2, xi 1e-7, step fraction 1), 2000
    balanced pairs (xi 5e-6, separations 1e-5..1e-1, displacement 1.5 x the
    separation) and 1000 pairs with step fraction 0.37 (displacement 3 x the
    separation); hit and time of impact
    per pair (a miss reports the step fraction, as the C ABI does).
Run:  python tests/golden/make_golden_ccd.py
"""
import ctypes
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path[:0] = [ROOT, os.path.join(ROOT, "codim-ipc_gb300")]
from oracle import build as ob  # noqa: E402
import workloads  # noqa: E402


def configs(rng):
    out = []
    out.append(rng.random((1000, 12)))
    near = np.empty((1000, 12))
    for i in range(1000):
        t0, t1, t2 = rng.random(3), rng.random(3), rng.random(3)
        n = np.cross(t1 - t0, t2 - t0)
        n /= np.linalg.norm(n)
        a, b = rng.uniform(-0.3, 1.3, 2)
        p = t0 + a * (t1 - t0) + b * (t2 - t0) + (10 ** rng.uniform(-9, -2)) * rng.choice([-1, 1]) * n
        near[i] = np.concatenate([p, t0, t1, t2]) if i % 2 == 0 else np.concatenate([t0, t1, p, p + (t2 - t0)])
    out.append(near)
    sc = rng.random((1000, 12)) * (10 ** rng.uniform(-6, 3, (1000, 1))) + rng.uniform(-1e3, 1e3, (1000, 1))
    out.append(sc)
    return np.ascontiguousarray(np.concatenate(out))


def main():
    path = ob.build_ref_ccd()
    if path is None:
        raise SystemExit("reference sources or an x86 compiler not available")
    L = ctypes.CDLL(path)
    P = ctypes.c_void_p
    for n in ("refc_pt_type", "refc_ee_type", "refc_pe_type"):
        getattr(L, n).argtypes = [P]
        getattr(L, n).restype = ctypes.c_int
    for n in ("refc_pt_d2", "refc_ee_d2", "refc_pe_d2"):
        getattr(L, n).argtypes = [P]
        getattr(L, n).restype = ctypes.c_double
    L.refc_ccd_pairs.argtypes = [ctypes.c_int64, P, P, P, P, ctypes.c_double, ctypes.c_double, ctypes.c_double, P, P]
    rng = np.random.default_rng(20240611)
    cfg = configs(rng)
    m = cfg.shape[0]
    res = {k: np.zeros(m, np.int32) for k in ("pt_type", "ee_type", "pe_type")}
    res.update({k: np.zeros(m) for k in ("pt_d2", "ee_d2", "pe_d2")})
    for i in range(m):
        x = np.ascontiguousarray(cfg[i])
        q = x.ctypes.data
        res["pt_type"][i] = L.refc_pt_type(q)
        res["ee_type"][i] = L.refc_ee_type(q)
        res["pe_type"][i] = L.refc_pe_type(q)
        res["pt_d2"][i] = L.refc_pt_d2(q)
        res["ee_d2"][i] = L.refc_ee_d2(q)
        res["pe_d2"][i] = L.refc_pe_d2(q)
    data = dict(cfg=cfg, **res)
    cases = [("b0", dict(n=2000, seed=101), 1e-7, 1.0),
             ("b1", dict(n=2000, seed=102, mix=(0.25, 0.25, 0.25, 0.25), sep_range=(1e-5, 1e-1), disp_scale=1.5),
              5e-6, 1.0),
             ("b2", dict(n=1000, seed=103, disp_scale=3.0), 1e-7, 0.37)]
    for name, kw, th, toc_in in cases:
        n = kw.pop("n")
        w = workloads.contact_pairs(n, **kw)
        # keep only the vertices the pairs use, renumbered, so the fixture stays small
        used = np.unique(w["idx"][w["idx"] >= 0])
        remap = -np.ones(w["x"].shape[0], np.int64)
        remap[used] = np.arange(used.size)
        idx = np.where(w["idx"] >= 0, remap[np.maximum(w["idx"], 0)], -1).astype(np.int32)
        x = np.ascontiguousarray(w["x"][used])
        dx = np.ascontiguousarray(w["dx"][used])
        t = np.ascontiguousarray(w["type"])
        idx = np.ascontiguousarray(idx)
        toc = np.zeros(n)
        hit = np.zeros(n, np.uint8)
        L.refc_ccd_pairs(n, t.ctypes.data, idx.ctypes.data, x.ctypes.data, dx.ctypes.data, 0.1, th, toc_in,
                         toc.ctypes.data, hit.ctypes.data)
        data.update({name + "_type": t, name + "_idx": idx, name + "_x": x, name + "_dx": dx, name + "_toc": toc,
                     name + "_hit": hit, name + "_params": np.array([0.1, th, toc_in])})
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_ccd.npz")
    np.savez_compressed(out, **data)
    print(out, {k: v.shape for k, v in data.items() if k.endswith("_hit")})


if __name__ == "__main__":
    main()
