"""cipc_ccd_pairs_noalloc against cipc_ccd_pairs (device memory).

The no-allocation entry point runs the same kernels with its counters in a
scratch array compiled into the library; its outputs must be bit-identical to
the allocating entry point's on the same pairs, on two calls in a row (the
second call proves the slot was zeroed again), and its counters must report a
bad pair in one call without leaking into the next.  This file is collected
last so that it also runs after every other GPU test in the same process.
"""
import os
import re

import numpy as np
import pytest

import cipc_ffi as F
import workloads as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_noalloc_source_has_no_allocation_calls():
    """The no-allocation translation unit names no allocating CUDA call outside comments."""
    with open(os.path.join(ROOT, "codim-ipc_gb300", "csrc", "capi_noalloc.cu")) as f:
        src = f.read()
    code = re.sub(r"//[^\n]*", "", re.sub(r"/\*.*?\*/", "", src, flags=re.S))
    for name in ("cudaMalloc", "cudaFree", "cudaHostAlloc", "cudaMallocHost", "cudaMallocManaged", "new ",
                 "malloc(", "std::vector"):
        assert name not in code, name


def _device_pairs(cuda, n, seed):
    import torch
    w = W.contact_pairs(n, seed=seed)
    return {k: torch.from_numpy(np.ascontiguousarray(w[k])).to(cuda) for k in ("type", "idx", "x", "dx")}


def _outputs(cuda, n):
    import torch
    return torch.full((n,), -1.0, dtype=torch.float64, device=cuda), torch.full((n,), 7, dtype=torch.uint8,
                                                                                 device=cuda)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [F.FP64, F.MIXED])
def test_noalloc_matches_allocating_entry_point(cuda, precision):
    import torch
    n = 200_000
    d = _device_pairs(cuda, n, seed=11)
    stream = torch.cuda.current_stream()
    toc_r, hit_r = _outputs(cuda, n)
    st, ov_r = F.ccd_pairs(d["type"], d["idx"], d["x"], d["dx"], toc_r, hit_r, precision=precision,
                           mem=F.MEM_DEVICE, stream=stream)
    for call in range(2):
        toc, hit = _outputs(cuda, n)
        st, ov = F.ccd_pairs_noalloc(d["type"], d["idx"], d["x"], d["dx"], toc, hit, precision=precision, slot=3,
                                     stream=stream)
        torch.cuda.synchronize()
        assert ov == ov_r, call
        assert torch.equal(hit, hit_r), call
        assert torch.equal(toc, toc_r), call
    assert int(hit_r.sum()) > 0


@pytest.mark.gpu
def test_noalloc_counters_reset_between_calls(cuda):
    """A pair with an out-of-range vertex (caught by the kernel's own index check,
    not evaluated) makes one call report CIPC_ERR_INDEX_RANGE; the next call on
    the same slot with valid pairs reports success."""
    import torch
    n = 4096
    d = _device_pairs(cuda, n, seed=5)
    nv = int(d["x"].shape[0])
    bad_idx = d["idx"].clone()
    bad_idx[17, 0] = nv + 3
    toc, hit = _outputs(cuda, n)
    st, _ = F.ccd_pairs_noalloc(d["type"], bad_idx, d["x"], d["dx"], toc, hit, slot=0,
                                allow=(F.CIPC_ERR_INDEX_RANGE,))
    assert st == F.CIPC_ERR_INDEX_RANGE
    toc_r, hit_r = _outputs(cuda, n)
    F.ccd_pairs(d["type"], d["idx"], d["x"], d["dx"], toc_r, hit_r, mem=F.MEM_DEVICE)
    for call in range(2):
        toc, hit = _outputs(cuda, n)
        st, ov = F.ccd_pairs_noalloc(d["type"], d["idx"], d["x"], d["dx"], toc, hit, slot=0)
        torch.cuda.synchronize()
        assert st == F.CIPC_OK and ov == 0
        assert torch.equal(toc, toc_r) and torch.equal(hit, hit_r)
    # enqueue-only form (no counts read back) gives the same outputs
    toc, hit = _outputs(cuda, n)
    F.ccd_pairs_noalloc(d["type"], d["idx"], d["x"], d["dx"], toc, hit, slot=F.NOALLOC_SLOTS - 1, counts=False)
    torch.cuda.synchronize()
    assert torch.equal(toc, toc_r) and torch.equal(hit, hit_r)


def _default_pool_stats(device_index):
    """(used, reserved, used high-water mark) of the device's default stream-ordered
    memory pool, read through the driver API (the pool every cudaMallocAsync on
    that device draws from unless the caller set another)."""
    import ctypes
    cu = ctypes.CDLL("libcuda.so.1")
    dev = ctypes.c_int()
    assert cu.cuDeviceGet(ctypes.byref(dev), device_index) == 0
    pool = ctypes.c_void_p()
    assert cu.cuDeviceGetDefaultMemPool(ctypes.byref(pool), dev) == 0
    out = []
    for attr in (7, 5, 8):  # CU_MEMPOOL_ATTR_USED_MEM_CURRENT, _RESERVED_MEM_CURRENT, _USED_MEM_HIGH
        v = ctypes.c_uint64()
        assert cu.cuMemPoolGetAttribute(pool, attr, ctypes.byref(v)) == 0
        out.append(v.value)
    return out, cu, pool


@pytest.mark.gpu
def test_noalloc_calls_leave_device_memory_untouched(cuda):
    """At run time, not only in the source: after a first call (which may load
    the kernels), repeated calls change neither torch's allocated memory nor the
    default pool's used and reserved bytes, and the pool's high-water mark (reset
    before the calls) does not rise."""
    import ctypes

    import torch
    n = 100_000
    d = _device_pairs(cuda, n, seed=21)
    toc, hit = _outputs(cuda, n)
    F.ccd_pairs_noalloc(d["type"], d["idx"], d["x"], d["dx"], toc, hit, slot=1)
    torch.cuda.synchronize()
    (used0, res0, _), cu, pool = _default_pool_stats(cuda.index or 0)
    zero = ctypes.c_uint64(0)
    assert cu.cuMemPoolSetAttribute(pool, 8, ctypes.byref(zero)) == 0  # reset the high-water mark
    alloc0 = torch.cuda.memory_allocated(cuda)
    for _ in range(3):
        F.ccd_pairs_noalloc(d["type"], d["idx"], d["x"], d["dx"], toc, hit, slot=1)
        F.ccd_pairs_noalloc(d["type"], d["idx"], d["x"], d["dx"], toc, hit, slot=2, counts=False)
    torch.cuda.synchronize()
    (used1, res1, high1), _, _ = _default_pool_stats(cuda.index or 0)
    assert torch.cuda.memory_allocated(cuda) == alloc0
    assert used1 == used0 and res1 == res0
    assert high1 <= used0
