"""pma_edt_noalloc, the allocation-free EDT entry point, against pma_edt through the C ABI.

The file name puts it last in collection order: it has to pass both in a fresh process,
where its first call performs the per-device set-up, and after every other GPU test.
"""
import ctypes

import numpy as np
import pytest

from porousmediaanalysis_gb300 import capi, synth

pytestmark = pytest.mark.gpu

SENTINEL = np.uint64(0xA5A5A5A5A5A5A5A5)


def _dims(t):
    sz, sx, sy = t.shape
    return capi.Dims(sx, sy, sz)


def _vp(t):
    return ctypes.c_void_p(t.data_ptr())


def _volumes(torch):
    """(SZ, SX, SY) uint8 volumes on cuda:0: overlapping spheres, and a nearly empty box whose
    distances exceed the 2048 histogram bins a block keeps in shared memory."""
    union = synth.sphere_union((72, 80, 88), count=60, rmin=4.0, rmax=9.0, seed=11)
    rng = np.random.default_rng(5)
    sparse = np.zeros((120, 128, 112), np.uint8)
    pts = rng.integers(0, sparse.size, 10)
    sparse.reshape(-1)[pts] = 1
    return [torch.from_numpy(np.ascontiguousarray(v.astype(np.uint8))).cuda() for v in (union, sparse)]


def _edt_ctx(lib, ctx, solid, hist_cap, torch):
    edt2 = torch.empty(solid.shape, dtype=torch.int32, device=solid.device)
    st = capi.EdtStats()
    hist = np.full(max(hist_cap, 1), SENTINEL, np.uint64)
    capi.check(lib.pma_edt(ctx.handle, _vp(solid), _dims(solid), _vp(edt2), ctypes.byref(st),
                           hist.ctypes.data_as(ctypes.c_void_p) if hist_cap else None, hist_cap))
    return edt2, (st.max_edt2, st.hist_len), hist


def _edt_noalloc(lib, solid, edt2, hist_cap, stream):
    st = capi.EdtStats()
    hist = np.full(max(hist_cap, 1), SENTINEL, np.uint64)
    status = lib.pma_edt_noalloc(_vp(solid), _dims(solid), _vp(edt2), ctypes.byref(st),
                                 hist.ctypes.data_as(ctypes.c_void_p) if hist_cap else None,
                                 hist_cap, ctypes.c_void_p(stream))
    return status, (st.max_edt2, st.hist_len), hist


def test_two_calls_in_a_row_match_pma_edt(pma_lib, ctx):
    torch = pytest.importorskip("torch")
    vols = _volumes(torch)
    outs = [torch.full(v.shape, -1, dtype=torch.int32, device="cuda") for v in vols]
    stream = torch.cuda.current_stream().cuda_stream
    caps = [4096, 8192]
    got = []
    for v, o, cap in zip(vols, outs, caps):  # two calls in a row, no other work between
        status, stats, hist = _edt_noalloc(pma_lib, v, o, cap, stream)
        assert status == capi.PMA_OK, capi.last_error()
        got.append((stats, hist))
    for v, o, cap, (stats, hist) in zip(vols, outs, caps, got):
        e_ref, s_ref, h_ref = _edt_ctx(pma_lib, ctx, v, cap, torch)
        torch.cuda.synchronize()
        assert torch.equal(o, e_ref)
        assert stats == s_ref
        assert np.array_equal(hist, h_ref)
    assert got[1][0][0] > 2048  # the second volume uses the global histogram bins


def test_repeated_calls_other_streams_and_truncated_histogram(pma_lib, ctx):
    torch = pytest.importorskip("torch")
    solid = _volumes(torch)[1]
    e_ref, s_ref, h_ref = _edt_ctx(pma_lib, ctx, solid, 100, torch)
    side = torch.cuda.Stream()
    for stream in (side.cuda_stream, 0, side.cuda_stream):
        out = torch.full(solid.shape, -1, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        status, stats, hist = _edt_noalloc(pma_lib, solid, out, 100, stream)
        assert status == capi.PMA_OK, capi.last_error()
        torch.cuda.synchronize()
        assert torch.equal(out, e_ref)
        assert stats == s_ref
        assert np.array_equal(hist, h_ref)


def test_no_device_memory_taken_after_setup(pma_lib):
    torch = pytest.importorskip("torch")
    solid = _volumes(torch)[0]
    out = torch.empty(solid.shape, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    assert _edt_noalloc(pma_lib, solid, out, 64, stream)[0] == capi.PMA_OK
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert _edt_noalloc(pma_lib, solid, out, 64, stream)[0] == capi.PMA_OK
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before


def test_rejects_volumes_beyond_the_scratch(pma_lib):
    torch = pytest.importorskip("torch")
    # smallest extent 1025 needs 512^2 + 1 bins, one more than the fixed scratch holds;
    # the buffers are real so that nothing runs out of bounds even if the check did not fire
    solid = torch.zeros((1025, 1025, 1025), dtype=torch.uint8, device="cuda")
    out = torch.empty((1025, 1025, 1025), dtype=torch.int32, device="cuda")
    status, _, _ = _edt_noalloc(pma_lib, solid, out, 0, torch.cuda.current_stream().cuda_stream)
    assert capi.STATUS[status] == "PMA_ERR_LIMIT"
    assert "1024" in capi.last_error()
    del solid, out
    torch.cuda.empty_cache()
