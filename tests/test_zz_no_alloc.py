"""The allocation-free sort entry point, msc_sort_pairs_device_noalloc.

It exists for callers that cannot allocate device memory while they run (a
host that reserves its whole device budget up front, or a latency-critical loop
that cannot take cudaFree's device synchronisation).  It must give exactly the
same pairs as the allocating entry point, msc_sort_pairs_device, on two calls
in a row that share its static scratch.  This file sorts last so that a run
stopping at the first failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sort_on_device(fn, torch, keys, vals, bits):
    k = torch.from_numpy(keys.view(np.int32)).cuda()
    v = torch.from_numpy(vals.view(np.int32)).cuda()
    torch.cuda.synchronize()
    rc = fn(C.c_void_p(k.data_ptr()), C.c_void_p(v.data_ptr()), keys.shape[0], bits, None)
    torch.cuda.synchronize()
    return rc, k.cpu().numpy().view(np.uint32), v.cpu().numpy().view(np.uint32)


def test_noalloc_sort_matches_allocating_sort_twice(built):
    torch = pytest.importorskip("torch")
    mscgpu, _ = built
    lib = mscgpu.load_library()
    rng = np.random.default_rng(2024)
    # two calls in a row: a full-size one, then a smaller one with fewer key bits
    for n, bits in ((1 << 20, 32), (300007, 22)):
        keys = rng.integers(0, 1 << 32, size=n, dtype=np.uint64).astype(np.uint32)
        keys[::5] = keys[0]  # repeated keys exercise stability
        vals = rng.permutation(n).astype(np.uint32)
        rc_a, ka, va = _sort_on_device(lib.msc_sort_pairs_device_noalloc, torch, keys, vals, bits)
        rc_b, kb, vb = _sort_on_device(lib.msc_sort_pairs_device, torch, keys, vals, bits)
        assert rc_a == 0 and rc_b == 0
        assert np.array_equal(ka, kb)
        assert np.array_equal(va, vb)
        # and directly against a stable CPU sort of the same pairs on the low `bits` bits
        masked = keys & np.uint32((1 << bits) - 1) if bits < 32 else keys
        order = np.argsort(masked, kind="stable")
        assert np.array_equal(va, vals[order])
        assert np.array_equal(ka, keys[order])


def test_noalloc_sort_rejects_more_than_its_maximum(built):
    torch = pytest.importorskip("torch")
    mscgpu, _ = built
    lib = mscgpu.load_library()
    n = (1 << 20) + 1
    k = torch.zeros(n, dtype=torch.int32, device="cuda")
    v = torch.zeros(n, dtype=torch.int32, device="cuda")
    rc = lib.msc_sort_pairs_device_noalloc(C.c_void_p(k.data_ptr()), C.c_void_p(v.data_ptr()), n, 32, None)
    assert rc == -1
    assert b"exceeds the maximum" in lib.msc_last_error(None)
