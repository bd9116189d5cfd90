"""Bit-exact checks on the stream the throughput figure is measured on.

Workload: directed R-MAT, scale 21 (2,097,152 vertices), edge factor 16,
(a, b, c, d) = (.57, .19, .19, .05), seed 1, self loops and duplicates
removed, shuffled with seed 1001; the first half S is bulk-loaded.  Inserts
are drawn from the cyclic sequence U ++ S and deletes from S ++ U (U = the
unloaded half), alternating, exactly as bench.py drives the engine: 22
batches each of 1,024, 10,240 and 102,400 keys, then 56 batches of
1,048,576 keys (warm-up, timed, profiled and end-to-end steps of the bench).

Checks, all exact (integer data):
* after the bulk load and after each of the first four 1M batches, the whole
  physical layout (every slot's key and value), the height and the sentinel
  slots equal the CPU oracle's (oracle/lpma_oracle.c, which runs the
  reference's level-by-level loop);
* after every 1M batch (and at the end of each smaller batch size), the
  sorted key set (export_sorted) and the sentinel-inclusive CSR view
  (to_csr: row_offset, col_index, values) equal those built from the
  sorted-merge CSR rebuild of the same stream (oracle CsrBaseline), the
  reference's own check of its update path (test_update_rpma.cu:131-165:
  the stored keys, sentinels skipped, equal the sorted input).
"""
import time

import numpy as np
import pytest

from test_gpu_parity import _dev, assert_same

pytestmark = pytest.mark.gpu

SCALE, EF, SEED = 21, 16, 1
NBR_END = 0x3FFFFE
DST_AND_TIME_END = 0x000003FFFFEFFFFF


def expected_views(edges, V):
    """The sorted key set with sentinels and the sentinel-inclusive CSR of a
    sorted edge array: row v holds its edges (col = dst) then its sentinel
    (col = v), values 1 for edges and 0xFF for sentinels."""
    n = edges.size
    src = (edges >> np.uint64(42)).astype(np.int64)
    dst = ((edges >> np.uint64(20)) & np.uint64(0x3FFFFF)).astype(np.uint32)
    plain = np.searchsorted(src, np.arange(V + 1)).astype(np.int64)
    ro = (plain + np.arange(V + 1)).astype(np.uint32)
    keys = np.empty(n + V, np.uint64)
    col = np.empty(n + V, np.uint32)
    vals = np.empty(n + V, np.uint8)
    pos = np.arange(n, dtype=np.int64) + src  # edge i of row v sits after v sentinels
    spos = plain[1:] + np.arange(V)           # sentinel of v closes its row
    keys[pos] = edges
    keys[spos] = (np.arange(V, dtype=np.uint64) << np.uint64(42)) + np.uint64(DST_AND_TIME_END)
    col[pos] = dst
    col[spos] = np.arange(V, dtype=np.uint32)
    vals[pos] = 1
    vals[spos] = 0xFF
    return keys, ro, col, vals


def check_views(g, base, V, where):
    keys, ro, col, vals = expected_views(base.edges(), V)
    gk, gv = g.export_sorted()
    assert gk.size == keys.size, "%s: %d keys stored, %d expected" % (where, gk.size, keys.size)
    assert np.array_equal(gk, keys), "%s: sorted key set differs" % where
    gro, gci, gva = g.to_csr()
    assert np.array_equal(gro, ro), "%s: row_offset differs" % where
    assert np.array_equal(gci, col), "%s: col_index differs" % where
    assert np.array_equal(gva, vals), "%s: CSR values differ" % where


def test_scale21_stream_matches_reference_checks(engine, oracle):
    t0 = time.time()
    V = 1 << SCALE
    e = oracle.shuffle(oracle.rmat_edges(SEED, SCALE, EF), SEED + 1000)
    half = e.size // 2
    S, U = e[:half], e[half:]
    ins_seq, del_seq = np.concatenate([U, S]), np.concatenate([S, U])
    d_ins, d_del = _dev(ins_seq), _dev(del_seq)
    n = ins_seq.size
    cur = {"ins": 0, "del": 0}

    def nxt(kind, B):
        a = cur[kind] % n
        cur[kind] += B
        seq = d_ins if kind == "ins" else d_del
        host = ins_seq if kind == "ins" else del_seq
        if a + B <= n:
            return seq[a:a + B], host[a:a + B]
        import torch
        return torch.cat([seq[a:], seq[:a + B - n]]), np.concatenate([host[a:], host[:a + B - n]])

    g = engine.Lpma(V)
    o = oracle.OracleLpma(V)
    base = oracle.CsrBaseline(V, threads=16)
    g.build(_dev(S))
    o.update(ins=S)
    base.load(S)
    assert_same(g, o, "bulk load")
    check_views(g, base, V, "bulk load")
    follow = True  # the oracle follows the stream until the layout checks are done
    kinds = ("ins", "del")
    events = {}

    def step(kind, B, where, layout):
        nonlocal follow
        dev, host = nxt(kind, B)
        sg = g.update(ins=dev) if kind == "ins" else g.update(dels=dev)
        if follow:
            so = o.update(ins=host) if kind == "ins" else o.update(dels=host)
            for k in ("n_ins_applied", "n_del_applied", "root_executed", "overflow", "rebuilt", "levelup"):
                assert sg[k] == so[k], "%s: %s %d vs %d" % (where, k, sg[k], so[k])
        (base.insert if kind == "ins" else base.delete)(host)
        assert sg["n_ins_applied"] == (B if kind == "ins" else 0) and sg["n_del_applied"] == (B if kind == "del" else 0)
        for k in ("root_executed", "eager_levelup", "rebuilt", "levelup_path", "fill_empty"):
            if sg[k]:
                events[k] = events.get(k, 0) + 1
        if layout:
            assert_same(g, o, where)

    # the bench's per-batch-size sweep: 2 + 20 batches at each size
    for B in (1024, 10240, 102400):
        for i in range(22):
            step(kinds[i % 2], B, "sweep %d #%d" % (B, i), False)
        check_views(g, base, V, "after the %d-key batches" % B)
    # 1M batches: warm-up 4, timed 20, profiled 10, end-to-end 2 + 20
    for i in range(56):
        first = i < 4
        step(kinds[i % 2], 1 << 20, "1M batch %d" % i, first)
        if i == 3:
            follow = False
            o.close()
        check_views(g, base, V, "1M batch %d" % i)
    print("scale-21 stream: %d vertices, %d edges, height %d, events %s, %.0f s"
          % (V, e.size, g.height, events, time.time() - t0))
    g.close()
