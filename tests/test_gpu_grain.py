"""Executor grain cut-overs (lpma_grain_set, lpma_autotune_grain) against the
oracle.

The cut-overs decide which executor rewrites a window, never the layout:
under every setting, including one that sends every window of two or more
segments through the tile grain (gather / spread), an insert / delete
stream gives the oracle's layout slot for slot.  The tuner inserts and
deletes the caller's batch of absent keys on the caller's own handle: the
oracle replays the same rounds and the layouts stay equal; a batch holding
a stored key is refused with nothing changed.
"""
import numpy as np
import pytest

from test_gpu_parity import _dev, assert_csr, assert_same

pytestmark = pytest.mark.gpu


def set_all(rpma, g, s):
    for b in range(0, 33):
        rpma.grain_set(b, g, s)


@pytest.mark.parametrize("cut", [(1, 1), (1, 32), (2, 8), (3, 5), (4, 16)])
def test_layout_independent_of_cut_overs(engine, oracle, cut):
    from lpma_gb300 import rpma
    V = 1 << 12
    e = oracle.shuffle(oracle.rmat_edges(31, 12, 16), 7)
    half = e.size // 2
    g, o = engine.Lpma(V), oracle.OracleLpma(V)
    d = _dev(e)
    g.update(ins=d[:half])
    o.update(ins=e[:half])
    set_all(rpma, *cut)
    try:
        rng = np.random.default_rng(cut[0] * 100 + cut[1])
        pos = half
        for i in range(10):
            b = int(rng.integers(50, 4000))
            if i % 2 == 0 and pos < e.size:
                sg, so = g.update(ins=d[pos:pos + b]), o.update(ins=e[pos:pos + b])
                pos += b
            else:
                dels = rng.choice(e[:pos], size=min(b, pos), replace=False)
                sg, so = g.update(dels=_dev(dels)), o.update(dels=dels)
            for k in ("n_ins_applied", "n_del_applied", "root_executed", "overflow", "rebuilt"):
                assert sg[k] == so[k], (cut, i, k)
            assert_same(g, o, "cut %s batch %d" % (cut, i))
        assert_csr(g, o)
    finally:
        set_all(rpma, 0, 0)
    g.close()


def test_autotune_grain_keeps_the_set(engine, oracle):
    from lpma_gb300 import LpmaError, rpma
    V = 1 << 13
    e = oracle.shuffle(oracle.rmat_edges(33, 13, 16), 8)
    half = e.size // 2
    g, o = engine.Lpma(V), oracle.OracleLpma(V)
    g.update(ins=_dev(e[:half]))
    o.update(ins=e[:half])
    batch = e[half:half + 3000]
    bucket = int(batch.size - 1).bit_length()
    reps = 2
    try:
        res = rpma.autotune_grain(g, _dev(batch), reps=reps)
        assert len(res) == 6 and all(r["us"] > 0 for r in res)
        chosen = rpma.grain_get(bucket)
        assert chosen in [(r["max_segs_group"], r["max_segs_shared"]) for r in res]
        # the oracle replays the tuner's rounds: insert and delete, one
        # warm-up and `reps` timed per setting
        for _ in range(6 * (reps + 1)):
            o.update(ins=batch)
            o.update(dels=batch)
        assert_same(g, o, "after the tuner")
        # a batch with a stored key is refused before anything changes
        bad = np.concatenate([batch[:100], e[:1]])
        with pytest.raises(LpmaError):
            rpma.autotune_grain(g, _dev(bad), reps=1)
        assert_same(g, o, "after the refused batch")
        sg, so = g.update(ins=_dev(batch)), o.update(ins=batch)
        assert sg["n_ins_applied"] == so["n_ins_applied"] == batch.size
        assert_same(g, o, "the chosen setting in use")
    finally:
        rpma.grain_set(bucket, 0, 0)
    g.close()
