"""The bounded grid-barrier wait of the cooperative batch sort, made to give up.

The cooperative sort's CTAs meet at grid barriers; every wait polls a
bounded number of times, then records a timeout and goes on, so the kernel
always ends.  Here the test setting of the barrier (lpma_debug_sort_barrier)
makes every wait aim at an arrival count that never comes, with a short
poll limit: no CTA hangs, nothing is written out of range (the sort's
scatter is bounds-checked), the update returns LPMA_ERR_TIMEOUT with the
structure unchanged, and the same handle takes the same batch correctly
once the setting is cleared.  Nothing here faults or hangs the GPU: the
failure is a wait that runs out by design.
"""
import ctypes

import numpy as np
import pytest

from test_gpu_parity import _dev, assert_csr, assert_same

pytestmark = pytest.mark.gpu

LPMA_ERR_TIMEOUT = 7


def test_sort_barrier_give_up_returns_timeout_and_keeps_handle(engine, oracle):
    from lpma_gb300 import LpmaError, _abi, rpma
    L = _abi.load()
    V = 1 << 14
    e = oracle.shuffle(oracle.rmat_edges(17, 14, 16), 5)
    half = e.size // 2
    g, o = engine.Lpma(V), oracle.OracleLpma(V)
    d = _dev(e)
    g.update(ins=d[:half])
    o.update(ins=e[:half])
    n = 20000                      # bucket 2^15, forced onto the cooperative sort
    bucket = int(n - 1).bit_length()
    rpma.tune_set(bucket, "cooperative")
    try:
        _abi.check(L.lpma_debug_sort_barrier(256, 1), "lpma_debug_sort_barrier")
        for attempt in range(2):  # the first call captures the front, the second replays it
            with pytest.raises(LpmaError) as ei:
                g.update(ins=d[half:half + n])
            assert ei.value.status == LPMA_ERR_TIMEOUT, ei.value
            assert_same(g, o, "after give-up %d" % attempt)
    finally:
        L.lpma_debug_sort_barrier(0, 0)
        rpma.tune_set(bucket, 0)
    # the handle is usable: the same batch through the cooperative sort again
    rpma.tune_set(bucket, "cooperative")
    try:
        sg = g.update(ins=d[half:half + n])
    finally:
        rpma.tune_set(bucket, 0)
    so = o.update(ins=e[half:half + n])
    assert sg["n_ins_applied"] == so["n_ins_applied"] and sg["sort_passes"] > 0
    assert_same(g, o, "after recovery")
    assert_csr(g, o)
    g.close()
