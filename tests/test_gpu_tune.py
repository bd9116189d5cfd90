"""The batch-sort autotuner and every sort tier it can pick.

All tiers must give the same stable order, so an update sorted with any of
them leaves the same layout: each tier is forced for the bucket of the
batch size under test, and the layout is compared slot for slot with the
oracle after every batch (integer data, no tolerance).
"""
import numpy as np
import pytest

from test_gpu_parity import _dev, assert_same

pytestmark = pytest.mark.gpu

TIERS = ("small", "block", "tile_merge", "cooperative", "multi_pass")


def _bucket(n):
    return max(0, int(n - 1).bit_length())


def _expected_passes(keys, tier):
    """Digit passes of the batch sort: one per byte where the keys differ,
    or for the cooperative sort one per 9-bit window, each starting at the
    lowest differing bit the earlier windows left uncovered."""
    if keys.size < 2:
        return 0
    diff = int(np.bitwise_and.reduce(keys)) ^ int(np.bitwise_or.reduce(keys))
    if tier != "cooperative":
        return sum(1 for b in range(8) if (diff >> (8 * b)) & 0xFF)
    n = 0
    while diff:
        low = (diff & -diff).bit_length() - 1
        diff = (diff >> (low + 9)) << (low + 9)
        n += 1
    return n


@pytest.fixture
def reset_table(engine):
    from lpma_gb300 import rpma
    yield rpma
    for b in range(33):
        for conc in (False, True):
            rpma.tune_set(b, 0, concurrent=conc)


def test_autotune_reports_and_sets(engine, reset_table):
    from lpma_gb300 import _abi
    rp = reset_table
    rows = rp.autotune(1 << 17)
    assert len(rows) == 2 * (17 - 11 + 1)
    L = _abi.load()
    import ctypes
    for r in rows:
        assert r["tier"] in r["us"], r  # the chosen tier was timed
        assert r["us"][r["tier"]] <= min(r["us"].values()) + 0.1  # the fastest (times reported to 0.1 us)
        if not r["concurrent"] and r["keys"] > 2048:
            assert "cooperative" in r["us"]
        if r["concurrent"]:
            assert "cooperative" not in r["us"]
        t = ctypes.c_uint32()
        _abi.check(L.lpma_tune_get(_bucket(r["keys"]), int(r["concurrent"]), ctypes.byref(t)), "lpma_tune_get")
        assert _abi.SORT_TIERS[t.value] == r["tier"]


@pytest.mark.parametrize("n,tiers", [
    (1500, ("small", "block", "tile_merge")),
    (6000, ("block", "tile_merge", "cooperative", "multi_pass")),
    (40000, ("tile_merge", "cooperative", "multi_pass")),
])
def test_every_tier_gives_the_same_layout(engine, oracle, reset_table, n, tiers):
    rp = reset_table
    V = 1 << 13
    keys = oracle.shuffle(oracle.rmat_edges(31, 13, 16), 5)
    rng = np.random.default_rng(n)
    for tier in tiers:
        rp.tune_set(_bucket(n), tier)
        g, o = engine.Lpma(V), oracle.OracleLpma(V)
        g.update(ins=_dev(keys[:20000]))
        o.update(ins=keys[:20000])
        pos = 20000
        for step in range(3):
            ins = keys[pos:pos + (n if step != 1 else 0)]
            pos += ins.size
            k, _ = o.export_sorted()
            live = k[((k >> np.uint64(20)) & np.uint64(0x3FFFFF)) != np.uint64(0x3FFFFE)]
            nd = n if step == 1 else n // 3
            dels = rng.choice(live, size=min(nd, live.size), replace=False)
            if step == 2:  # the batch holds n keys in all
                ins = ins[:n - dels.size]
            st = g.update(ins=_dev(ins), dels=_dev(dels))
            o.update(ins=ins, dels=dels)
            assert_same(g, o, "tier %s, batch of %d, step %d" % (tier, ins.size + dels.size, step))
            assert st["sort_passes"] == _expected_passes(np.concatenate([ins, dels]), tier), (tier, st["sort_passes"])
        g.close()
        rp.tune_set(_bucket(n), 0)
