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


def test_executor_copy_wait_give_up_is_reported_on_the_next_call(engine, oracle):
    """The bounded wait of the 5..32-segment executor for its bulk copies into
    shared memory, made to give up (lpma_debug_exec_wait): the warp records
    ERR_TIMEOUT in the handle's sticky word, waits (bounded) for its copies
    in flight and stops.  The call that launched it returns normally (its
    status was published before the executors ran); the next call on the
    handle reports LPMA_ERR_TIMEOUT.  Nothing faults or hangs: the wait
    that runs out is a bounded one, and the copies land before the warp
    leaves."""
    import torch
    from lpma_gb300 import LpmaError, _abi
    L = _abi.load()
    V = 1 << 12
    e = oracle.shuffle(oracle.rmat_edges(3, 12, 8), 4)
    half = e.size // 2
    g, o = engine.Lpma(V), oracle.OracleLpma(V)
    g.update(ins=_dev(e[:half]))
    o.update(ins=e[:half])
    # 120 new edges of one low-degree source: one window of 15 segments
    src = 4000
    keys = np.array([(src << 42) | (d << 20) for d in range(100, 220)], dtype=np.uint64)
    so = o.update(ins=keys)
    assert so["win_slots"][4] == 480
    _abi.check(L.lpma_debug_exec_wait(1), "lpma_debug_exec_wait")
    try:
        sg = g.update(ins=_dev(keys))
        torch.cuda.synchronize()
    finally:
        L.lpma_debug_exec_wait(0)
    assert sg["n_ins_applied"] == 120 and sg["windows_small"] - sg["windows_single"] == 1
    with pytest.raises(LpmaError) as ei:
        g.update(ins=_dev(keys[:1]))
    assert ei.value.status == LPMA_ERR_TIMEOUT, ei.value
    g.close()
