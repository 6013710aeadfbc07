"""pcs_scan_distance_noalloc: the distance kernel for callers that cannot
let a library allocate device memory (a host framework's own caching
allocator, a fixed device-memory budget, real-time loops).  It must give
exactly what pcs_scan_distance and the oracle give, reset the histograms it
consumed, refuse sizes beyond its fixed scratch, work on back-to-back calls
that reuse the shared scratch, and take no device memory once its first call
on the device has loaded it.  Buffers here come from torch, i.e. from the
caller."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(rng, count, R, B):
    hist = rng.poisson(0.8, (count, R, B)).astype(np.uint32)
    ref = np.cumsum(np.cumsum(rng.poisson(0.8, (R, B)), 0), 1).astype(np.uint32)
    return hist, ref


def _call(pcs, torch, hist, ref):
    count, R, B = hist.shape
    d_hist = torch.from_numpy(hist.view(np.int32).copy()).cuda()
    d_ref = torch.from_numpy(ref.view(np.int32).copy()).cuda()
    d_dist = torch.full((count,), -1.0, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    st = pcs.lib().pcs_scan_distance_noalloc(C.c_void_p(d_hist.data_ptr()), C.c_void_p(d_ref.data_ptr()), R, B,
                                             count, C.c_void_p(d_dist.data_ptr()), None)
    torch.cuda.synchronize()
    return st, d_hist.cpu().numpy(), d_dist.cpu().numpy()


def test_noalloc_matches_allocating_entry_point(pcs, ctx, oracle):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(31)
    # two calls in a row with different shapes: the second must not see the
    # first call's descriptors or transposed histogram
    for count, R, B in [(5, 301, 128), (3, 201, 100)]:
        hist, ref = _case(rng, count, R, B)
        want = pcs.scan_distance(ctx, hist, ref)["dist_f32"]
        st, hist_after, got = _call(pcs, torch, hist, ref)
        assert st == 0, pcs.lib().pcs_last_error()
        assert got.tobytes() == want.tobytes()
        for q in range(count):
            assert got[q] == np.float32(oracle.distance_kdist(hist[q], ref)[0]), (R, B, q)
        assert not hist_after.any()


def test_noalloc_takes_no_device_memory(pcs, ctx):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(32)
    hist, ref = _case(rng, 4, 301, 128)
    count, R, B = hist.shape
    d_hist = torch.from_numpy(hist.view(np.int32).copy()).cuda()
    d_ref = torch.from_numpy(ref.view(np.int32).copy()).cuda()
    d_dist = torch.zeros(count, dtype=torch.float32, device="cuda")
    args = (C.c_void_p(d_hist.data_ptr()), C.c_void_p(d_ref.data_ptr()), R, B, count, C.c_void_p(d_dist.data_ptr()),
            None)
    assert pcs.lib().pcs_scan_distance_noalloc(*args) == 0  # loads the module and looks its array up
    torch.cuda.synchronize()
    free0, alloc0 = torch.cuda.mem_get_info()[0], torch.cuda.memory_allocated()
    for _ in range(3):
        assert pcs.lib().pcs_scan_distance_noalloc(*args) == 0, pcs.lib().pcs_last_error()
    torch.cuda.synchronize()
    assert torch.cuda.memory_allocated() == alloc0
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_rejects_sizes_beyond_its_scratch(pcs, ctx):
    torch = pytest.importorskip("torch")
    d = torch.zeros(16, dtype=torch.int32, device="cuda")
    p = C.c_void_p(d.data_ptr())
    st = pcs.lib().pcs_scan_distance_noalloc(p, p, 2048, 1024, 1, p, None)
    assert st == pcs._lib.ERR_INVALID_ARGUMENT
    assert b"exceeds the allocation-free limit" in pcs.lib().pcs_last_error()
    st = pcs.lib().pcs_scan_distance_noalloc(p, p, 2, 2, 5000, p, None)
    assert st == pcs._lib.ERR_INVALID_ARGUMENT
