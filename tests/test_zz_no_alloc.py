"""The allocation-free key/value sort, checked against the allocating sorter.

Some callers of this library may not call cudaMalloc: an engine callback that owns the whole
device-memory budget, or code running while other streams are in flight (allocation can synchronise
the device).  gs_sort_key_value_noalloc serves them with its scratch in a fixed device array inside
the library.  This file calls it through the C ABI and
compares its result with gs_sorter_sort_key_value_indirect on the same inputs, on consecutive calls
(the shared array keeps each call's leftovers), plus the rejection of a size beyond its maximum.
It is collected last so that a failure here never hides the result of another test.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _inputs(rng, n):
    keys = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    keys[: n // 4] = keys[n // 4: 2 * (n // 4)]  # duplicates exercise stability
    keys[-(n // 8):] &= np.uint32(0xFF)          # and a cluster of small keys
    return keys, np.arange(n, dtype=np.uint32)


def test_noalloc_sort_matches_the_sorter_on_consecutive_calls(cuda):
    import torch
    from vkgs_gb300 import Sorter
    from vkgs_gb300 import _lib as L

    lib = L.load()
    max_count = L.GS_SORT_NOALLOC_MAX_COUNT
    rng = np.random.default_rng(2024)
    stream = torch.cuda.current_stream()
    sorter = Sorter()
    for n, count in [(300_000, 299_123), (max_count, max_count), (4097, 4097)]:
        keys, vals = _inputs(rng, n)
        k_new = torch.from_numpy(keys.view(np.int32)).cuda()
        v_new = torch.from_numpy(vals.view(np.int32)).cuda()
        k_ref, v_ref = k_new.clone(), v_new.clone()
        cnt = torch.tensor([count], dtype=torch.int32, device="cuda")
        err = torch.zeros(1, dtype=torch.int32, device="cuda")
        st = lib.gs_sort_key_value_noalloc(ctypes.c_void_p(stream.cuda_stream), n, _ptr(cnt), _ptr(k_new),
                                           _ptr(v_new), _ptr(err))
        assert st == L.GS_SUCCESS
        sorter.sort_key_value(k_ref, v_ref, count=count)
        sorter.check()
        torch.cuda.synchronize()
        assert int(err.item()) == 0
        np.testing.assert_array_equal(k_new.cpu().numpy(), k_ref.cpu().numpy())
        np.testing.assert_array_equal(v_new.cpu().numpy(), v_ref.cpu().numpy())
        order = np.argsort(keys[:count], kind="stable")
        np.testing.assert_array_equal(k_new.cpu().numpy().view(np.uint32)[:count], keys[:count][order])


def test_noalloc_sort_rejects_sizes_beyond_its_maximum(cuda):
    import torch
    from vkgs_gb300 import _lib as L

    lib = L.load()
    k = torch.zeros(8, dtype=torch.int32, device="cuda")
    cnt = torch.tensor([8], dtype=torch.int32, device="cuda")
    st = lib.gs_sort_key_value_noalloc(None, L.GS_SORT_NOALLOC_MAX_COUNT + 1, _ptr(cnt), _ptr(k), _ptr(k), None)
    assert st == L.GS_ERROR_CAPACITY
    assert lib.gs_sort_key_value_noalloc(None, 8, None, _ptr(k), _ptr(k), None) == L.GS_ERROR_INVALID_ARGUMENT


def test_noalloc_sort_takes_no_device_memory(cuda):
    """What the entry point exists for: after the first call on the device (which looks up the fixed
    array's address), its calls take no device memory -- free device memory is the same before and
    after three calls on fresh keys -- and each result equals the allocating sorter's."""
    import torch
    from vkgs_gb300 import Sorter
    from vkgs_gb300 import _lib as L

    lib = L.load()
    n = 200_000
    rng = np.random.default_rng(77)
    k_buf = torch.empty(n, dtype=torch.int32, device="cuda")
    v_buf = torch.empty(n, dtype=torch.int32, device="cuda")
    cnt = torch.tensor([n], dtype=torch.int32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    sorter = Sorter()
    stream = torch.cuda.current_stream()

    def call():
        return lib.gs_sort_key_value_noalloc(ctypes.c_void_p(stream.cuda_stream), n, _ptr(cnt), _ptr(k_buf),
                                             _ptr(v_buf), _ptr(err))

    def load(keys, vals):
        k_buf.copy_(torch.from_numpy(keys.view(np.int32)))
        v_buf.copy_(torch.from_numpy(vals.view(np.int32)))

    inputs = [_inputs(rng, n) for _ in range(3)]
    wants = []
    for keys, vals in inputs:
        k_ref = torch.from_numpy(keys.view(np.int32)).cuda()
        v_ref = torch.from_numpy(vals.view(np.int32)).cuda()
        sorter.sort_key_value(k_ref, v_ref, count=n)
        sorter.check()
        wants.append((k_ref, v_ref))
    load(*inputs[0])
    assert call() == L.GS_SUCCESS  # the first call on this device does the set-up
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for kv, (k_ref, v_ref) in zip(inputs, wants):
        load(*kv)
        assert call() == L.GS_SUCCESS
        torch.cuda.synchronize()
        assert torch.equal(k_buf, k_ref) and torch.equal(v_buf, v_ref)
    assert torch.cuda.mem_get_info()[0] == free0
    assert int(err.item()) == 0
