"""kgb_dissimilarity_inplace_device: the allocation-free, device-pointer form of
the co-label proximity.  Checked against kgb_dissimilarity_inplace (host
buffers) on the same inputs, on two calls in a row; results must be equal
bit for bit (tolerance 0: both run the same integer counts and the same
double-rounded arithmetic)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(seed, n, K, runs):
    rng = np.random.default_rng(seed)
    gidx = rng.integers(1, n + 1, (n, K)).astype(np.int32)
    gidx[rng.random((n, K)) < 0.03] = -1
    gdist = np.sort(rng.random((n, K), dtype=np.float32) * 4.0, axis=1)
    res = rng.integers(0, 7, (runs, n)).astype(np.int32)
    return gidx, gdist, res


def _device_call(lib, torch, gidx, gdist, res):
    n, K = gidx.shape
    runs = res.shape[0]
    di = torch.from_numpy(gidx).cuda()
    dd = torch.from_numpy(gdist).cuda()
    dr = torch.from_numpy(res).cuda()
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    rc = lib.kgb_dissimilarity_inplace_device(
        ctypes.c_void_p(di.data_ptr()), ctypes.c_void_p(dd.data_ptr()), n, K,
        ctypes.c_void_p(dr.data_ptr()), runs, torch.cuda.current_device(),
        ctypes.c_void_p(stream.cuda_stream))
    free_after = torch.cuda.mem_get_info()[0]
    return rc, di.cpu().numpy(), dd.cpu().numpy(), free_before, free_after


def test_device_noalloc_matches_host_entry(kg):
    torch = pytest.importorskip("torch")
    from kodama_gb300 import _native
    lib = _native.load()
    cases = [_case(31, 3000, 20, 40), _case(32, 5000, 30, 100)]
    for call, (gidx, gdist, res) in enumerate(cases):
        want_i, want_d = gidx.copy(), gdist.copy()
        kg.KODAMADissimilarityInPlace(want_i, want_d, res)
        rc, got_i, got_d, free_before, free_after = _device_call(lib, torch, gidx, gdist, res)
        _native.check(rc)
        assert np.array_equal(got_i, want_i), f"call {call}: indices differ"
        assert np.array_equal(got_d.view(np.uint32), want_d.view(np.uint32)), f"call {call}: distances differ"
        if call > 0:
            # after the per-device set-up, a call takes no device memory
            assert free_after == free_before


def test_device_noalloc_rejects(kg):
    torch = pytest.importorskip("torch")
    from kodama_gb300 import _native
    lib = _native.load()
    # beyond the static scratch: rejected on the host, nothing launched
    rc = lib.kgb_dissimilarity_inplace_device(
        ctypes.c_void_p(16), ctypes.c_void_p(16), 50000, 10, ctypes.c_void_p(16), 100, 0, None)
    assert rc == _native.KGB_EINVAL
    buf = ctypes.create_string_buffer(512)
    lib.kgb_last_error(buf, 512)
    assert b"exceeds the static scratch" in buf.value
    # a zero-based index is rejected by the device check and leaves the graph as it was
    gidx, gdist, res = _case(33, 500, 8, 10)
    gidx[7, 3] = 0
    rc, got_i, got_d, _, _ = _device_call(lib, torch, gidx, gdist, res)
    assert rc == _native.KGB_EINVAL
    assert np.array_equal(got_i, gidx) and np.array_equal(got_d, gdist)
