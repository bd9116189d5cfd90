"""lpma_memory_reserve: the update memory pool grows by the requested bytes
and keeps them; a request the device cannot hold is refused with
LPMA_ERR_OUT_OF_MEMORY and leaves the engine usable."""
import ctypes

import numpy as np
import pytest

from test_gpu_parity import _dev, assert_same

pytestmark = pytest.mark.gpu


def test_reserve_then_update(engine, oracle):
    from lpma_gb300 import _abi, rpma
    rpma.memory_reserve(1 << 30)
    rpma.memory_reserve(0)
    L = _abi.load()
    st = L.lpma_memory_reserve(ctypes.c_uint64(1 << 42), None)  # 4 TB: more than any GB300 holds
    assert _abi.STATUS_NAMES[st] == "LPMA_ERR_OUT_OF_MEMORY"
    V = 1 << 12
    e = oracle.shuffle(oracle.rmat_edges(5, 12, 16), 6)
    g, o = engine.Lpma(V), oracle.OracleLpma(V)
    for a in range(0, e.size, 20000):
        g.update(ins=_dev(e[a:a + 20000]))
        o.update(ins=e[a:a + 20000])
    assert_same(g, o, "after the reservations")
    g.close()
