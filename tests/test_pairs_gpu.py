"""GPU contact-pair kernels against the CPU oracle, through the C ABI.

Bars (stated per test):
  * CCD, FP64 variant: hit/miss decisions and times of impact bit-identical,
    also over the full 10M-pair benchmark workload.
  * CCD, mixed variant: decisions may differ only for pairs within FP32 rounding
    of a region boundary (<= 1e-4 of pairs); times agree to 1e-5 relative at the
    99.9th percentile, the rest within one conservative step, also for a scene
    translated far from the origin.
  * CCD, both variants: bit-identical answers when positions, displacements and
    xi are scaled by 2^-40 or 2^40.
  * Barrier: energy and gradient (FP64 in both variants) to 1e-9 relative;
    projected Hessian to 1e-8 (FP64 variant) / 2e-4 (mixed, FP32 Hessian) of the
    pair's largest entry.
"""
import numpy as np
import pytest

import cipc_ffi as F
import workloads

pytestmark = pytest.mark.gpu

ETA, TH = 0.1, 1e-7


def _gpu_ccd(w, precision, toc_in=1.0, th=TH, eta=ETA):
    n = w["type"].shape[0]
    toc = np.zeros(n)
    hit = np.zeros(n, np.uint8)
    st, ov = F.ccd_pairs(w["type"], w["idx"], w["x"], w["dx"], toc, hit, eta=eta, thickness=th, toc_in=toc_in,
                         precision=precision)
    return toc, hit, st, ov


@pytest.mark.parametrize("seed,toc_in", [(1, 1.0), (2, 0.37)])
def test_ccd_fp64_bit_exact(cuda, orc, seed, toc_in):
    w = workloads.contact_pairs(200_000, seed=seed)
    toc_o, hit_o, it_o, ov_o = orc.ccd_pairs(w["type"], w["idx"], w["x"], w["dx"], ETA, TH, toc_in)
    toc_g, hit_g, st, ov = _gpu_ccd(w, F.FP64, toc_in)
    assert st == 0 and ov == 0 and ov_o == 0
    assert 0 < hit_o.sum() < hit_o.size
    assert np.array_equal(hit_g, hit_o)
    assert np.array_equal(toc_g.view(np.uint64), toc_o.view(np.uint64))


def test_ccd_fp64_bit_exact_all_types_balanced(cuda, orc):
    w = workloads.contact_pairs(100_000, seed=7, mix=(0.25, 0.25, 0.25, 0.25), sep_range=(1e-5, 1e-1),
                                disp_scale=1.5)
    for th in (0.0, 5e-6):
        toc_o, hit_o, _, _ = orc.ccd_pairs(w["type"], w["idx"], w["x"], w["dx"], ETA, th, 1.0)
        toc_g, hit_g, st, _ = _gpu_ccd(w, F.FP64, th=th)
        for t in range(4):
            m = w["type"] == t
            assert hit_o[m].sum() > 0
        assert np.array_equal(hit_g, hit_o)
        assert np.array_equal(toc_g.view(np.uint64), toc_o.view(np.uint64))


def test_ccd_mixed_against_fp64_oracle(cuda, orc):
    w = workloads.contact_pairs(200_000, seed=3)
    toc_o, hit_o, _, _ = orc.ccd_pairs(w["type"], w["idx"], w["x"], w["dx"], ETA, TH, 1.0)
    toc_g, hit_g, st, ov = _gpu_ccd(w, F.MIXED)
    mism = (hit_g != hit_o).mean()
    assert mism <= 1e-4, mism
    both = (hit_g == 1) & (hit_o == 1)
    rel = np.abs(toc_g[both] - toc_o[both]) / toc_o[both]
    # FP32 stopping tests can end ACCD one conservative step apart for a few pairs
    assert np.quantile(rel, 0.999) <= 1e-5, np.quantile(rel, 0.999)
    assert rel.max() <= 1e-2, rel.max()


def test_ccd_mixed_translated_scene(cuda, orc):
    # the same pairs 1000 units from the origin: the mixed kernel forms its pair
    # differences in FP64, so the bars of the untranslated case still hold
    w = workloads.contact_pairs(200_000, seed=9)
    wt = dict(w, x=w["x"] + np.array([1000.0, -750.0, 500.0]))
    toc_o, hit_o, _, _ = orc.ccd_pairs(wt["type"], wt["idx"], wt["x"], wt["dx"], ETA, TH, 1.0)
    toc_g, hit_g, st, ov = _gpu_ccd(wt, F.MIXED)
    assert st == 0 and ov == 0 and 0 < hit_o.sum() < hit_o.size
    assert (hit_g != hit_o).mean() <= 1e-4
    both = (hit_g == 1) & (hit_o == 1)
    rel = np.abs(toc_g[both] - toc_o[both]) / toc_o[both]
    assert np.quantile(rel, 0.999) <= 1e-5, np.quantile(rel, 0.999)
    # a pair whose FP32 stopping test lands the other side of the threshold ends
    # one conservative step (up to ~(1 - eta) of the remaining gap) apart
    assert (rel > 1e-5).mean() <= 1e-3 and rel.max() <= 0.5, rel.max()


@pytest.mark.parametrize("precision", [F.FP64, F.MIXED])
def test_ccd_scale_invariant(cuda, precision):
    # ACCD's steps and stopping test are invariant under a common scaling of
    # positions, displacements and xi; by a power of two every rounding scales
    # exactly, so the answers must be bit-identical (the mixed kernel's float-float
    # split and per-pair rescaling included) at scales far from the unit cube
    w = workloads.contact_pairs(100_000, seed=8, mix=(0.25, 0.25, 0.25, 0.25))
    toc0, hit0, st, _ = _gpu_ccd(w, precision)
    assert st == 0 and 0 < hit0.sum() < hit0.size
    for k in (-40, 40):
        ws = dict(w, x=w["x"] * 2.0 ** k, dx=w["dx"] * 2.0 ** k)
        toc, hit, st, _ = _gpu_ccd(ws, precision, th=TH * 2.0 ** k)
        assert st == 0
        assert np.array_equal(hit, hit0), k
        assert np.array_equal(toc.view(np.uint64), toc0.view(np.uint64)), k


@pytest.mark.parametrize("precision", [F.FP64, F.MIXED])
def test_ccd_page_locked_host_buffers(cuda, precision):
    """Host buffers in page-locked memory are read and written in place by the
    kernel (no staging); results are bit-identical to the staged pageable call."""
    import torch
    w = workloads.contact_pairs(300_000, seed=14)
    n = w["type"].shape[0]
    pin = {k: torch.from_numpy(np.ascontiguousarray(w[k])).pin_memory().numpy() for k in ("type", "idx", "x", "dx")}
    toc_p = torch.full((n,), -1.0, dtype=torch.float64).pin_memory().numpy()
    hit_p = torch.full((n,), 7, dtype=torch.uint8).pin_memory().numpy()
    st, ov = F.ccd_pairs(pin["type"], pin["idx"], pin["x"], pin["dx"], toc_p, hit_p, eta=ETA, thickness=TH,
                         precision=precision)
    toc_h, hit_h, st_h, ov_h = _gpu_ccd(w, precision)
    assert st == st_h == 0 and ov == ov_h == 0
    assert np.array_equal(hit_p, hit_h) and 0 < hit_p.sum() < n
    assert np.array_equal(toc_p.view(np.uint64), toc_h.view(np.uint64))
    # a bad index is still caught and reported
    pin["idx"][5, 1] = w["x"].shape[0] + 2
    with pytest.raises(F.CipcError) as ei:
        F.ccd_pairs(pin["type"], pin["idx"], pin["x"], pin["dx"], toc_p, hit_p, eta=ETA, thickness=TH)
    assert ei.value.status == F.CIPC_ERR_INDEX_RANGE


def test_ccd_device_memory_matches_host(cuda):
    import torch
    w = workloads.contact_pairs(50_000, seed=4)
    toc_h, hit_h, _, _ = _gpu_ccd(w, F.FP64)
    dev = {k: torch.from_numpy(np.ascontiguousarray(w[k])).to(cuda) for k in ("type", "idx", "x", "dx")}
    toc = torch.zeros(w["type"].shape[0], dtype=torch.float64, device=cuda)
    hit = torch.zeros(w["type"].shape[0], dtype=torch.uint8, device=cuda)
    st, ov = F.ccd_pairs(dev["type"], dev["idx"], dev["x"], dev["dx"], toc, hit, eta=ETA, thickness=TH,
                         precision=F.FP64, mem=F.MEM_DEVICE, stream=torch.cuda.current_stream())
    assert st == 0 and ov == 0
    assert np.array_equal(toc.cpu().numpy().view(np.uint64), toc_h.view(np.uint64))
    assert np.array_equal(hit.cpu().numpy(), hit_h)


def test_ccd_edge_cases(cuda, orc):
    # zero displacement: no hit, toc = toc_in; a bad index is reported, never read
    w = workloads.contact_pairs(1000, seed=5)
    w0 = dict(w)
    w0["dx"] = np.zeros_like(w["dx"])
    toc, hit, st, _ = _gpu_ccd(w0, F.FP64, toc_in=0.8)
    assert not hit.any() and np.all(toc == 0.8)
    bad = dict(w)
    bad["idx"] = w["idx"].copy()
    bad["idx"][10, 2] = w["x"].shape[0] + 5
    n = bad["type"].shape[0]
    with pytest.raises(F.CipcError) as ei:
        F.ccd_pairs(bad["type"], bad["idx"], bad["x"], bad["dx"], np.zeros(n), np.zeros(n, np.uint8))
    assert ei.value.status == F.CIPC_ERR_INDEX_RANGE
    # one pair of each type, the smallest possible inputs
    for t in range(4):
        m = np.where(w["type"] == t)[0][:1]
        if m.size == 0:
            continue
        sub = dict(type=w["type"][m], idx=w["idx"][m], x=w["x"], dx=w["dx"])
        toc_o, hit_o, _, _ = orc.ccd_pairs(sub["type"], sub["idx"], sub["x"], sub["dx"], ETA, TH, 1.0)
        toc_g, hit_g, _, _ = _gpu_ccd(sub, F.FP64)
        assert np.array_equal(toc_g.view(np.uint64), toc_o.view(np.uint64)) and np.array_equal(hit_g, hit_o)


def _barrier_case(n, seed, mix=(0.1, 0.1, 0.4, 0.4)):
    w = workloads.contact_pairs(n, seed=seed, mix=mix)
    return w


def _gpu_barrier(w, x_rest, precision, dhat2=1e-4, xi=TH, kappa=1.0):
    n = w["type"].shape[0]
    E = np.zeros(n)
    g = np.zeros((n, 12))
    H = np.zeros((n, 78), np.float64 if precision == F.FP64 else np.float32)
    st, bad = F.barrier_pairs(w["type"], w["idx"], w["x"], x_rest, E, g, H, dhat2, xi, kappa, True, precision)
    return E, g, H, st, bad


@pytest.mark.parametrize("precision,htol", [(F.FP64, 1e-8), (F.MIXED, 2e-4)])
def test_barrier_against_oracle(cuda, orc, precision, htol):
    w = _barrier_case(20_000, 8, mix=(0.25, 0.25, 0.25, 0.25))
    E_o, g_o, H_o, bad_o = orc.barrier_pairs(w["type"], w["idx"], w["x"], w["x"], 1e-4, TH, 1.0)
    E_g, g_g, H_g, st, bad = _gpu_barrier(w, w["x"], precision)
    assert bad == bad_o == 0
    assert np.all(np.abs(E_g - E_o) <= 1e-9 * np.abs(E_o) + 1e-300)
    gs = np.abs(g_o).max(1, keepdims=True)
    assert np.all(np.abs(g_g - g_o) <= 1e-9 * gs + 1e-300)
    hs = np.abs(H_o).max(1, keepdims=True)
    err = np.abs(H_g.astype(np.float64) - H_o) / np.maximum(hs, 1e-300)
    assert err.max() <= htol, err.max()


def test_barrier_mollified_edge_edge(cuda, orc):
    """Nearly parallel edges take the mollified product-rule branch."""
    rng = np.random.default_rng(9)
    m = 2000
    ea0 = rng.random((m, 3))
    d = rng.standard_normal((m, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    ea1 = ea0 + 0.3 * d
    nrm = np.cross(d, rng.standard_normal((m, 3)))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    sep = 10 ** rng.uniform(-5, -2.5, m)
    tilt = rng.standard_normal((m, 3)) * 1e-3
    eb0 = ea0 + 0.05 * d + sep[:, None] * nrm
    eb1 = eb0 + 0.3 * d + tilt
    x = np.concatenate([ea0, ea1, eb0, eb1])
    idx = np.stack([np.arange(m), m + np.arange(m), 2 * m + np.arange(m), 3 * m + np.arange(m)], 1).astype(np.int32)
    w = dict(type=np.full(m, 3, np.uint8), idx=idx, x=x)
    # rest shape: perpendicular edges so eps_x is large and every pair is mollified
    x_rest = x.copy()
    x_rest[3 * m:] = x_rest[2 * m:3 * m] + 0.3 * nrm
    E_o, g_o, H_o, _ = orc.barrier_pairs(w["type"], idx, x, x_rest, 1e-4, 0.0, 1.0)
    for precision, htol in ((F.FP64, 1e-8), (F.MIXED, 2e-4)):
        E_g, g_g, H_g, st, bad = _gpu_barrier(w, x_rest, precision, xi=0.0)
        act = E_o != 0
        assert act.sum() > m // 2
        assert np.all(np.abs(E_g - E_o) <= 1e-9 * np.abs(E_o) + 1e-300)
        gs = np.abs(g_o).max(1, keepdims=True)
        assert np.all(np.abs(g_g - g_o) <= 1e-8 * gs + 1e-300)
        hs = np.abs(H_o).max(1, keepdims=True)
        err = np.abs(H_g.astype(np.float64) - H_o) / np.maximum(hs, 1e-300)
        assert err.max() <= htol, err.max()


def test_barrier_nonpositive_reported(cuda, orc):
    w = _barrier_case(2000, 10)
    # thickness above some separations: those pairs have s <= 0
    E_o, g_o, H_o, bad_o = orc.barrier_pairs(w["type"], w["idx"], w["x"], w["x"], 1e-4, 1e-5, 1.0)
    assert bad_o > 0
    n = w["type"].shape[0]
    E = np.zeros(n)
    g = np.zeros((n, 12))
    H = np.zeros((n, 78))
    st, bad = F.barrier_pairs(w["type"], w["idx"], w["x"], w["x"], E, g, H, 1e-4, 1e-5, 1.0, True, F.FP64)
    assert st == F.CIPC_ERR_NONPOSITIVE_DISTANCE and bad == bad_o


def test_ccd_fp64_bit_exact_benchmark_workload(cuda, orc):
    """The timed path of the contact-kernel benchmark at its full size: 10M seeded
    pairs (40/40/10/10, separations 1e-6..1e-2), device-memory FP64 kernel (with
    its certified FP32 type decisions), against the CPU oracle: hit/miss and the
    bits of every time of impact identical."""
    import torch
    w = workloads.contact_pairs(10_000_000, seed=0)
    toc_o, hit_o, _, ov_o = orc.ccd_pairs(w["type"], w["idx"], w["x"], w["dx"], ETA, TH, 1.0)
    dev = {k: torch.from_numpy(np.ascontiguousarray(w[k])).to(cuda) for k in ("type", "idx", "x", "dx")}
    n = w["type"].shape[0]
    toc = torch.empty(n, dtype=torch.float64, device=cuda)
    hit = torch.empty(n, dtype=torch.uint8, device=cuda)
    st, ov = F.ccd_pairs(dev["type"], dev["idx"], dev["x"], dev["dx"], toc, hit, eta=ETA, thickness=TH,
                         precision=F.FP64, mem=F.MEM_DEVICE)
    assert st == 0 and ov == 0 and ov_o == 0
    assert np.array_equal(hit.cpu().numpy(), hit_o)
    assert np.array_equal(toc.cpu().numpy().view(np.uint64), toc_o.view(np.uint64))


def test_ccd_mixed_direction_of_differences(cuda, orc):
    """The mixed kernel is neither bit-exact nor guaranteed conservative (the
    header says so); its differences from FP64 are counted by direction on 1M
    pairs and stay rare: unsafe misses (mixed no-hit where FP64 hits) below 2e-5
    of the pairs, times later than FP64's by more than 1e-5 relative below 1e-4."""
    w = workloads.contact_pairs(1_000_000, seed=13)
    toc_o, hit_o, _, _ = orc.ccd_pairs(w["type"], w["idx"], w["x"], w["dx"], ETA, TH, 1.0)
    toc_g, hit_g, st, ov = _gpu_ccd(w, F.MIXED)
    n = hit_o.size
    unsafe = int(((hit_g == 0) & (hit_o == 1)).sum())
    both = (hit_g == 1) & (hit_o == 1)
    late = int((toc_g[both] > toc_o[both] * (1 + 1e-5)).sum())
    assert unsafe <= 2e-5 * n and late <= 1e-4 * n, (unsafe, late)


def test_full_size_properties(cuda):
    """10M pairs (the benchmark size): FP64 vs mixed agreement and determinism."""
    import torch
    w = workloads.contact_pairs(10_000_000, seed=0)
    dev = {k: torch.from_numpy(np.ascontiguousarray(w[k])).to(cuda) for k in ("type", "idx", "x", "dx")}
    n = w["type"].shape[0]
    outs = []
    for precision in (F.FP64, F.MIXED, F.MIXED):
        toc = torch.empty(n, dtype=torch.float64, device=cuda)
        hit = torch.empty(n, dtype=torch.uint8, device=cuda)
        st, ov = F.ccd_pairs(dev["type"], dev["idx"], dev["x"], dev["dx"], toc, hit, eta=ETA, thickness=TH,
                             precision=precision, mem=F.MEM_DEVICE)
        assert st == 0 and ov == 0
        outs.append((toc.cpu().numpy(), hit.cpu().numpy()))
    (t64, h64), (tm, hm), (tm2, hm2) = outs
    assert np.array_equal(tm.view(np.uint64), tm2.view(np.uint64)) and np.array_equal(hm, hm2)
    assert (h64 != hm).mean() <= 1e-4
    assert np.all((t64 > 0) & (t64 <= 1.0))
    both = (h64 == 1) & (hm == 1)
    rel = np.abs(tm[both] - t64[both]) / t64[both]
    assert np.quantile(rel, 0.999) <= 1e-5, np.quantile(rel, 0.999)
    # a pair that stops one ACCD step earlier/later keeps a conservative time
    assert rel.max() <= 0.9, rel.max()
