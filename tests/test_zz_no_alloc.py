"""lpma_shuffle_static (the shuffle that allocates nothing) against lpma_shuffle.

Both go through the C ABI.  The result is integer data, so the tolerance is
zero: the two entry points must give the same keys in the same order, on
two calls in a row (the second call reuses the scratch the first one left).
"""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


def _lib():
    from lpma_gb300 import _abi
    return _abi, _abi.load()


def _keys(n, seed):
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    k = torch.randint(0, 1 << 62, (n,), dtype=torch.int64, device="cuda", generator=g)
    if n >= 8:
        k[n // 2:n // 2 + n // 8] = k[:n // 8]  # repeated keys too
    return k


@pytest.mark.parametrize("n", [2, 1000, 2048, 2049, 40000, 65536])
def test_static_shuffle_equals_shuffle_twice_in_a_row(n):
    import torch
    _abi, L = _lib()
    keys = _keys(n, 7 + n)
    want = keys.clone()
    _abi.check(L.lpma_shuffle(99, ctypes.c_void_p(want.data_ptr()), n, None), "lpma_shuffle")
    for _ in range(2):
        got = keys.clone()
        _abi.check(L.lpma_shuffle_static(99, ctypes.c_void_p(got.data_ptr()), n, None), "lpma_shuffle_static")
        torch.cuda.synchronize()
        assert torch.equal(got, want)
    # a permutation of the input
    assert torch.equal(torch.sort(want).values, torch.sort(keys).values)


def test_static_shuffle_rejects_sizes_above_its_scratch():
    import torch
    _abi, L = _lib()
    n = _abi.SHUFFLE_STATIC_MAX_KEYS + 1
    keys = _keys(n, 3)
    before = keys.clone()
    st = L.lpma_shuffle_static(1, ctypes.c_void_p(keys.data_ptr()), n, None)
    torch.cuda.synchronize()
    assert _abi.STATUS_NAMES[st] == "LPMA_ERR_SCRATCH_LIMIT"
    assert L.lpma_status_string(st) == b"n exceeds the fixed scratch of this entry point"
    assert torch.equal(keys, before)


def test_static_shuffle_trivial_sizes():
    import torch
    _abi, L = _lib()
    one = _keys(1, 5)
    before = one.clone()
    _abi.check(L.lpma_shuffle_static(4, ctypes.c_void_p(one.data_ptr()), 1, None), "n=1")
    _abi.check(L.lpma_shuffle_static(4, None, 0, None), "n=0")
    torch.cuda.synchronize()
    assert torch.equal(one, before)


def test_static_shuffle_null_keys_rejected_before_size():
    _abi, L = _lib()
    for n in (5, _abi.SHUFFLE_STATIC_MAX_KEYS + 1):
        st = L.lpma_shuffle_static(4, None, n, None)
        assert _abi.STATUS_NAMES[st] == "LPMA_ERR_INVALID_ARGUMENT", (n, st)


def test_static_shuffle_on_a_caller_stream_holds_device_memory_constant():
    """Two back-to-back calls on the caller's own (non-default) stream, with
    only that stream synchronised: both results equal lpma_shuffle's, and the
    device's free memory is the same after the warm calls as before them (a
    scratch buffer taken from cudaMalloc or a stream-ordered pool would leave
    it lower)."""
    import torch
    _abi, L = _lib()
    n = 50000
    a, b = _keys(n, 11), _keys(n, 12)
    wa, wb = a.clone(), b.clone()
    _abi.check(L.lpma_shuffle(5, ctypes.c_void_p(wa.data_ptr()), n, None), "lpma_shuffle")
    _abi.check(L.lpma_shuffle(6, ctypes.c_void_p(wb.data_ptr()), n, None), "lpma_shuffle")
    torch.cuda.synchronize()
    ga, gb = a.clone(), b.clone()
    warm = a.clone()
    _abi.check(L.lpma_shuffle_static(5, ctypes.c_void_p(warm.data_ptr()), n, None), "warm-up")
    s = torch.cuda.Stream()
    sp = ctypes.c_void_p(s.cuda_stream)
    torch.cuda.synchronize()  # the inputs above are ready before the stream reads them
    free_before = torch.cuda.mem_get_info()[0]
    _abi.check(L.lpma_shuffle_static(5, ctypes.c_void_p(ga.data_ptr()), n, sp), "first")
    _abi.check(L.lpma_shuffle_static(6, ctypes.c_void_p(gb.data_ptr()), n, sp), "second")
    s.synchronize()
    free_after = torch.cuda.mem_get_info()[0]
    assert torch.equal(ga, wa) and torch.equal(gb, wb)
    assert free_after == free_before, (free_before, free_after)
