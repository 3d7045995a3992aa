"""fg_sort_pairs_noalloc -- the sort entry point for callers that cannot
allocate device memory while they sort (hosts whose memory pool owns the whole
GPU, step loops that must not wait on cudaMalloc/cudaFree).  It keeps its
scratch in a fixed array inside the library instead of allocating.

Checked through the C ABI against the existing entry point fgc_sort_pairs
(same keys, same values, bit for bit -- integer work, so the tolerance is
exact equality) on two calls in a row, so the second call runs on scratch
that still holds the first call's data.  Also checks that sizes above the
1,048,576-pair maximum are refused with a clear error.  Collected last so a
failure here leaves every other test already run; it passes alone in a fresh
process and after the rest of the suite."""
import ctypes

import numpy as np
import pytest

from fluidgrid_gb300 import _ffi, build

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

MAX_PAIRS = 1 << 20


@pytest.fixture(scope="module")
def L():
    build.build()
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return _ffi.load()


def _dev(a):
    t = torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()
    torch.cuda.synchronize()
    return t


def _host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy().view(np.uint32)


def test_noalloc_sort_matches_existing_entry_point_two_calls(L):
    rng = np.random.default_rng(2024)
    cases = [(MAX_PAIRS, 21), (300001, 32)]  # second call: different size and key width
    for n, bits in cases:
        keys = rng.integers(0, 1 << bits, n, dtype=np.uint64).astype(np.uint32)
        keys[: n // 4] = keys[n // 2]  # long runs of equal keys: stability matters
        vals = rng.permutation(n).astype(np.uint32)
        ka, va = _dev(keys), _dev(vals)
        kb, vb = _dev(keys), _dev(vals)
        L.fgc_sort_pairs(ctypes.c_void_p(ka.data_ptr()), ctypes.c_void_p(va.data_ptr()), bits, n)
        assert L.fgc_last_status() == 0
        assert L.fg_device_synchronize() == 0
        st = L.fg_sort_pairs_noalloc(ctypes.c_void_p(kb.data_ptr()), ctypes.c_void_p(vb.data_ptr()), bits, n, None)
        assert st == 0, L.fg_last_error()
        assert L.fg_device_synchronize() == 0
        k_ref, v_ref = _host(ka), _host(va)
        k_got, v_got = _host(kb), _host(vb)
        assert np.array_equal(k_got, k_ref)
        assert np.array_equal(v_got, v_ref)
        assert np.all(np.diff(k_got.astype(np.int64)) >= 0)


def test_noalloc_sort_rejects_sizes_above_maximum(L):
    k = _dev(np.zeros(4, np.uint32))
    st = L.fg_sort_pairs_noalloc(ctypes.c_void_p(k.data_ptr()), ctypes.c_void_p(k.data_ptr()), 8, MAX_PAIRS + 1,
                                 None)
    assert _ffi.STATUS[st] == "FG_E_INVALID"
    assert b"1048576" in L.fg_last_error()
