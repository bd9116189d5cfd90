"""Randomised soak against the oracle.

A long stream of update batches per graph: sizes log-uniform over 1..50K
keys, insert/delete mixes drawn per batch, inserts of fresh keys plus
re-inserts of stored keys (upserts) and duplicates inside the batch, random
values, deletes of stored keys plus absent keys and one key the same batch
inserts (applied delete-first).  One graph grows from empty (overflow,
one-level growth, eager level-up, root windows, a rebuild), one shrinks from
a bulk load (root windows and rebuilds down).  After every batch the
physical layout, the sentinel slots, the height, the item count and the
resize path taken must equal the oracle's; the CSR view at the end.
"""
import numpy as np
import pytest

from test_gpu_parity import _dev, _dev8, assert_csr, assert_same

pytestmark = pytest.mark.gpu

PATH_FLAGS = ("overflow", "levelup_path", "rebuilt", "eager_levelup", "root_executed", "fill_empty", "levelup")


def _live(o):
    k, _ = o.export_sorted()
    return k[((k >> np.uint64(20)) & np.uint64(0x3FFFFF)) != np.uint64(0x3FFFFE)]


@pytest.mark.parametrize("V,seed,bulk_frac,del_lo,del_hi,expect", [
    (1 << 14, 11, 0.0, 0.0, 0.3, ("levelup_path", "eager_levelup", "rebuilt")),
    (1 << 13, 12, 0.9, 0.5, 1.0, ("rebuilt", "root_executed")),
])
def test_random_stream(engine, oracle, V, seed, bulk_frac, del_lo, del_hi, expect):
    scale = int(V).bit_length() - 1
    pool = oracle.shuffle(oracle.rmat_edges(seed, scale, 16), seed + 1)
    rng = np.random.default_rng(seed)
    g, o = engine.Lpma(V), oracle.OracleLpma(V)
    pos = int(bulk_frac * pool.size)
    if pos:
        g.update(ins=_dev(pool[:pos]))
        o.update(ins=pool[:pos])
        assert_same(g, o, "bulk")
    seen = set()
    for step in range(60):
        n = int(np.exp(rng.uniform(0, np.log(50000))))
        n_del = int(round(n * rng.uniform(del_lo, del_hi)))
        n_ins = n - n_del
        if pos + n_ins <= pool.size:
            fresh = pool[pos:pos + n_ins]
            pos += fresh.size
        else:
            fresh = rng.choice(pool, size=n_ins, replace=False) if n_ins else pool[:0]
        live = _live(o)
        ups = rng.choice(live, size=min(live.size, n_ins // 20), replace=False) if live.size else live
        dup = rng.choice(fresh, size=fresh.size // 10, replace=True) if fresh.size else fresh
        ins = np.concatenate([fresh, ups, dup]).astype(np.uint64)
        vals = rng.integers(1, 255, ins.size).astype(np.uint8)
        dsel = rng.choice(live, size=min(live.size, n_del), replace=False) if live.size else live
        absent = pool[-3:] if pos < pool.size - 3 else pool[:0]
        dels = np.concatenate([dsel, absent, ins[:1]]).astype(np.uint64)
        sg = g.update(ins=_dev(ins), ins_vals=_dev8(vals), dels=_dev(dels))
        so = o.update(ins=ins, ins_vals=vals, dels=dels)
        where = "step %d (%d inserts, %d deletes)" % (step, ins.size, dels.size)
        assert_same(g, o, where)
        for key in PATH_FLAGS + ("n_ins_applied", "n_del_applied"):
            assert sg[key] == so[key], "%s: %s %d vs %d" % (where, key, sg[key], so[key])
            if key in PATH_FLAGS and sg[key]:
                seen.add(key)
    assert set(expect) <= seen, seen
    assert_csr(g, o)
    g.close()
