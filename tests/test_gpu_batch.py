"""lpma_update_batch (the update of many graphs in one call) against
per-graph lpma_update and the CPU oracle.

Each graph has a twin updated one call at a time and an oracle copy; after
every round the batched graph's physical layout (every slot's key and
value, the sentinel slots, the height) must equal both, bit for bit, and
its per-graph stats must equal the twin's.  The rounds mix batch sizes that
take every sort tier of the shared front (one key, in-register block sort,
chunked per-graph radix sort) with batches the call hands to lpma_update
(an expiry threshold, more keys than one CTA sorts).
"""
import numpy as np
import pytest

from test_gpu_parity import _dev, _dev8, assert_same

pytestmark = pytest.mark.gpu

# every stat but sort_passes, which counts the passes of the sort that ran
# (the shared tile-merge sort here, possibly the cooperative one for the twin)
STAT_KEYS = ("height_before", "height_after", "n_ins_applied", "n_upserts", "n_del_applied", "n_noop",
             "root_executed", "eager_levelup", "overflow", "rebuilt", "levelup_path", "fill_empty", "levelup",
             "windows_single", "windows_small", "windows_big", "slots_rewritten", "slots_small", "num_items")


class _Twin:
    """One graph three ways: batched, per-graph, oracle."""

    def __init__(self, engine, oracle, V, seed, ef, with_vals=False, timed=False):
        self.V, self.with_vals, self.timed = V, with_vals, timed
        scale = max(1, int(V).bit_length() - 1)
        e = oracle.rmat_edges(seed, scale, ef)
        self.pool = oracle.shuffle(e, seed + 1)
        if timed:  # keys arrive in timestamp order, 97 per tick
            self.pool = self.pool | (np.arange(e.size, dtype=np.uint64) // np.uint64(97) + np.uint64(1))
        self.pos = 0
        self.rng = np.random.default_rng(seed)
        self.g, self.g2, self.o = engine.Lpma(V), engine.Lpma(V), oracle.OracleLpma(V)

    def next_batch(self, n_ins, n_del, expire=False):
        ins = self.pool[self.pos:self.pos + n_ins]
        self.pos += ins.size
        # expiry threshold: a few ticks before the batch's oldest insert (an
        # insert older than the threshold is an invalid key)
        thres = max(1, int(ins[0] & np.uint64(0xFFFFF)) - 3) if expire and ins.size else 0
        k, _ = self.o.export_sorted()
        live = k[((k >> np.uint64(20)) & np.uint64(0x3FFFFF)) != np.uint64(0x3FFFFE)]
        dels = self.rng.choice(live, size=min(n_del, live.size), replace=False) if live.size else live
        if n_del and self.rng.random() < 0.5:  # absent deletes and a delete of a key inserted in the same batch
            dels = np.concatenate([dels, self.pool[-3:], ins[:2]])
        vals = (self.rng.integers(1, 255, ins.size)).astype(np.uint8) if self.with_vals else None
        return ins, vals, dels, thres

    def device_batch(self, b):
        ins, vals, dels, thres = b
        d = {"ins": _dev(ins), "dels": _dev(dels), "thres": thres}
        if vals is not None:
            d["ins_vals"] = _dev8(vals)
        return d

    def apply_twin_and_oracle(self, b, d):
        ins, vals, dels, thres = b
        s2 = self.g2.update(ins=d["ins"], ins_vals=d.get("ins_vals"), dels=d["dels"], thres=thres)
        self.o.update(ins=ins, ins_vals=vals, dels=dels, thres=thres)
        return s2

    def check(self, stats, s2, where):
        assert_same(self.g, self.o, where)
        k1, v1, s1, h1 = self.g.layout()
        k2, v2, s2_, h2 = self.g2.layout()
        assert h1 == h2 and np.array_equal(k1, k2) and np.array_equal(v1, v2) and np.array_equal(s1, s2_), where
        for key in STAT_KEYS:
            assert stats[key] == s2[key], "%s: stat %s %d vs %d" % (where, key, stats[key], s2[key])

    def close(self):
        self.g.close()
        self.g2.close()


def _round(engine, twins, batches):
    B = engine.Batcher()
    devs = [t.device_batch(b) for t, b in zip(twins, batches)]
    stats, status = B.update([t.g for t in twins], devs)
    assert all(s == 0 for s in status), status
    for i, (t, b, d) in enumerate(zip(twins, batches, devs)):
        s2 = t.apply_twin_and_oracle(b, d)
        yield t, stats[i], s2
    B.close()


def test_batched_rounds_match_per_graph_and_oracle(engine, oracle):
    twins = [
        _Twin(engine, oracle, 1 << 6, 1, 8),
        _Twin(engine, oracle, 1 << 9, 2, 16, with_vals=True),
        _Twin(engine, oracle, 1 << 10, 3, 16),
        _Twin(engine, oracle, 1 << 11, 4, 16),
        _Twin(engine, oracle, 1 << 12, 5, 16, with_vals=True),
        _Twin(engine, oracle, 1 << 12, 6, 16, timed=True),
        _Twin(engine, oracle, 1 << 13, 7, 16),
        _Twin(engine, oracle, 1 << 15, 8, 16),
    ]
    # (n_ins, n_del) per graph per round; round 0 loads, the largest load
    # (2^18 keys) and the expiry rounds of the timed graph take lpma_update
    plan = [
        [(300, 0), (4000, 0), (9000, 0), (20000, 0), (30000, 0), (8000, 0), (60000, 0), (1 << 18, 0)],
        [(1, 0), (100, 50), (3000, 1000), (5000, 5000), (9000, 200), (2000, 100), (40000, 20000), (90000, 40000)],
        [(0, 0), (10, 200), (8192, 0), (1, 1), (700, 3000), (500, 0), (200, 60000), (0, 70000)],
        [(50, 25), (2000, 100), (4000, 4000), (6000, 3000), (9000, 9000), (300, 20), (30000, 100), (120000, 10000)],
    ]
    for r, sizes in enumerate(plan):
        batches = []
        for t, (ni, nd) in zip(twins, sizes):
            batches.append(t.next_batch(ni, nd, expire=t.timed and r >= 2))
        for t, stats, s2 in _round(engine, twins, batches):
            t.check(stats, s2, "round %d, V=%d" % (r, t.V))
    for t in twins:
        t.close()


def test_many_small_graphs_over_rounds(engine, oracle):
    """64 graphs with batches of 64..2048 keys for 6 rounds: level-ups,
    root windows and small-tree rebuilds happen inside the batched call."""
    rng = np.random.default_rng(3)
    twins = [_Twin(engine, oracle, 1 << int(rng.integers(6, 12)), 100 + i, 16, with_vals=bool(i % 3 == 0))
             for i in range(64)]
    for r in range(6):
        batches = [t.next_batch(int(rng.integers(64, 2048)), int(rng.integers(0, 1024)) if r else 0)
                   for t in twins]
        for t, stats, s2 in _round(engine, twins, batches):
            t.check(stats, s2, "round %d, V=%d" % (r, t.V))
    for t in twins:
        t.close()


def test_batch_errors_are_per_graph(engine, oracle):
    """A rejected batch leaves its graph unchanged and the others apply; a
    graph named twice gets INVALID_ARGUMENT for its second entry."""
    from lpma_gb300 import _abi
    a = _Twin(engine, oracle, 1 << 10, 11, 8)
    b = _Twin(engine, oracle, 1 << 10, 12, 8)
    B = engine.Batcher()
    ba, bb = a.next_batch(2000, 0), b.next_batch(2000, 0)
    da, db = a.device_batch(ba), b.device_batch(bb)
    B.update([a.g, b.g], [da, db])
    a.apply_twin_and_oracle(ba, da)
    b.apply_twin_and_oracle(bb, db)
    bad = {"ins": _dev(np.array([(a.V + 5) << 42], np.uint64))}  # source out of range
    ba2 = b.next_batch(500, 100)
    db2 = b.device_batch(ba2)
    stats, status = B.update([a.g, b.g, b.g], [bad, db2, db2], raise_on_error=False)
    assert _abi.STATUS_NAMES[status[0]] == "LPMA_ERR_INVALID_KEY"
    assert status[1] == 0
    assert _abi.STATUS_NAMES[status[2]] == "LPMA_ERR_INVALID_ARGUMENT"
    s2 = b.apply_twin_and_oracle(ba2, db2)
    b.check(stats[1], s2, "after a batch next to a rejected one")
    assert_same(a.g, a.o, "rejected graph unchanged")
    # the graph whose batch was rejected still updates
    ba3 = a.next_batch(300, 300)
    da3 = a.device_batch(ba3)
    stats, status = B.update([a.g], [da3])
    s2 = a.apply_twin_and_oracle(ba3, da3)
    a.check(stats[0], s2, "after the rejection")
    # an empty call
    assert B.update([], []) == ([], [])
    B.close()
    a.close()
    b.close()
