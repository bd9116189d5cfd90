"""The executor grain cut-overs' settings through the C ABI, without a GPU:
values outside the executors' ranges are refused and 0, 0 restores the
defaults (windows of up to 4 segments to the 8-lane-group executor, up to
32 to the shared-memory one)."""
import ctypes

import pytest


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__
    __graft_entry__._load_builder().build()
    from lpma_gb300 import _abi
    return _abi.load()


def get(L, b):
    g, s = ctypes.c_uint32(), ctypes.c_uint32()
    assert L.lpma_grain_get(b, ctypes.byref(g), ctypes.byref(s)) == 0
    return g.value, s.value


def test_grain_settings_validated_and_reset(lib):
    L = lib
    b = 13
    assert get(L, b) == (4, 32)
    for bad in ((40, 2, 8), (b, 5, 32), (b, 4, 2), (b, 0, 8), (b, 2, 33), (b, 3, 0)):
        assert L.lpma_grain_set(*bad) != 0, bad
        assert get(L, b) == (4, 32)
    try:
        assert L.lpma_grain_set(b, 2, 16) == 0
        assert get(L, b) == (2, 16)
        assert get(L, b + 1) == (4, 32)  # one bucket only
        assert L.lpma_grain_set(b, 1, 1) == 0  # every multi-segment window to the tile grain
        assert get(L, b) == (1, 1)
    finally:
        assert L.lpma_grain_set(b, 0, 0) == 0
    assert get(L, b) == (4, 32)
    g, s = ctypes.c_uint32(), ctypes.c_uint32()
    assert L.lpma_grain_get(33, ctypes.byref(g), ctypes.byref(s)) != 0
