"""GPU read paths through the C ABI against their CPU restatements.

The structure is built and updated on the device and, in lockstep, in the
oracle; the read results (neighbour lists with time windows, edge-query
counts, BFS hop counts) must equal the restatements over the oracle's key
set exactly.  PageRank is float64 with atomic accumulation on the device,
whose summation order varies: relative tolerance 1e-10.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

INT_MAX = 2**31 - 1


def _dev(a, dtype=np.uint64):
    import torch
    a = np.ascontiguousarray(a, dtype=dtype)
    view = {np.uint64: np.int64, np.uint32: np.int32}.get(dtype, dtype)
    return torch.from_numpy(a.view(view)).cuda()


def _timed_stream(oracle, seed, scale, ef):
    """R-MAT keys with timestamps 0..999 (several keys per (src, dst) pair)."""
    e = oracle.rmat_edges(seed, scale, ef)
    rng = np.random.default_rng(seed)
    t = rng.integers(0, 1000, e.size).astype(np.uint64)
    extra = e[rng.random(e.size) < 0.2] | rng.integers(0, 1000, 1).astype(np.uint64)
    keys = np.unique(np.concatenate([e | t, extra]))
    return oracle.shuffle(keys, seed + 7)


def _pair(engine, oracle, V, keys, n_bulk, batches):
    g, o = engine.Lpma(V), oracle.OracleLpma(V)
    g.update(ins=_dev(keys[:n_bulk]))
    o.update(ins=keys[:n_bulk])
    pos = n_bulk
    rng = np.random.default_rng(1)
    for b in batches:
        ins = keys[pos:pos + b]
        pos += b
        k, _ = o.export_sorted()
        live = k[((k >> np.uint64(20)) & np.uint64(0x3FFFFF)) != np.uint64(0x3FFFFE)]
        dels = rng.choice(live, size=min(b // 2, live.size), replace=False) if live.size else live
        g.update(ins=_dev(ins), dels=_dev(dels))
        o.update(ins=ins, dels=dels)
    return g, o


@pytest.fixture(scope="module")
def graph(engine, oracle):
    V = 1 << 12
    keys = _timed_stream(oracle, 11, 12, 16)
    g, o = _pair(engine, oracle, V, keys, keys.size // 2, [3000, 700, 5000, 64])
    yield g, o, V
    g.close()


def test_neighbor_queries_match(graph, oracle):
    import torch
    g, o, V = graph
    k, v = o.export_sorted()
    src = (k >> np.uint64(42)).astype(np.int64)
    hubs = np.argsort(-np.bincount(src, minlength=V))[:8]
    rng = np.random.default_rng(5)
    srcs = np.concatenate([[0, V - 1, V, V + 10], hubs, rng.integers(0, V, 500), [hubs[0], hubs[0]]]).astype(np.uint32)
    lb = rng.integers(0, 800, srcs.size).astype(np.uint64)
    ub = lb + rng.integers(0, 400, srcs.size).astype(np.uint64)
    wins = (lb << np.uint64(32)) | ub
    wins[:12] = 0xFFFFFFFF  # every timestamp
    offs, nb, nv = g.query_neighbors(_dev(srcs, np.uint32), _dev(wins))
    eo, en, ev = oracle.neighbors(k, v, srcs, wins, V)
    assert np.array_equal(offs.cpu().numpy().astype(np.int64), eo)
    assert np.array_equal(nb.cpu().numpy().astype(np.int64), en)
    assert np.array_equal(nv.cpu().numpy(), ev)
    # an empty query batch, and sizing without an output buffer
    offs0, nb0, _ = g.query_neighbors(torch.zeros(0, dtype=torch.int32, device="cuda"))
    assert offs0.cpu().tolist() == [0] and nb0.numel() == 0


def test_edge_queries_match(graph, oracle):
    g, o, V = graph
    k, _ = o.export_sorted()
    live = k[((k >> np.uint64(20)) & np.uint64(0x3FFFFF)) != np.uint64(0x3FFFFE)]
    rng = np.random.default_rng(9)
    present = rng.choice(live, 400, replace=False)
    absent = (rng.integers(0, V, 400).astype(np.uint64) << np.uint64(42)) | \
             (rng.integers(0, V, 400).astype(np.uint64) << np.uint64(20)) | rng.integers(0, 1000, 400).astype(np.uint64)
    odd = np.array([(V + 3) << 42, (5 << 42) | (0x3FFFFE << 20), 0], np.uint64)
    q = np.concatenate([present, absent, odd])
    for window in (0, 50, 100000, 0xFFFFF):
        got = g.edge_query(_dev(q), window).cpu().numpy().astype(np.int64)
        assert np.array_equal(got, oracle.edge_query_counts(k, q, window)), window
    # any-time existence (check_edge_kernel): t = window = 0xFFFFF
    qa = (q & ~np.uint64(0xFFFFF)) | np.uint64(0xFFFFF)
    got = g.edge_query(_dev(qa), 0xFFFFF).cpu().numpy().astype(np.int64)
    assert np.array_equal(got, oracle.edge_query_counts(k, qa, 0xFFFFF))


@pytest.mark.parametrize("sources,depth", [([0], 0), ([1, 2, 3, 1], 0), ([5], 2), (list(range(0, 4096, 4)), 2)])
def test_bfs_matches(graph, oracle, sources, depth):
    g, o, V = graph
    k, _ = o.export_sorted()
    dist, levels, reached = g.bfs(_dev(np.array(sources), np.uint32), depth)
    want = oracle.bfs(k, V, sources, depth)
    got = dist.cpu().numpy().astype(np.int64)
    assert np.array_equal(got, want)
    assert reached == int((want != INT_MAX).sum())


def test_pagerank_matches(graph, oracle):
    g, o, V = graph
    k, _ = o.export_sorted()
    for alpha, iters in ((0.85, 20), (0.9, 5)):
        got = g.pagerank(alpha, iters).cpu().numpy()
        want = oracle.pagerank(k, V, alpha, iters)
        np.testing.assert_allclose(got, want, rtol=1e-10, atol=0)
        assert abs(got.sum() - 1.0) < 1e-9


@pytest.mark.parametrize("V,n", [(1, 0), (7, 30), (100, 2000), (3000, 40000)])
def test_reads_after_growth(engine, oracle, V, n):
    """Small trees right after level-ups (empty leaves between full segments)."""
    rng = np.random.default_rng(V)
    src = rng.integers(0, V, n).astype(np.uint64)
    dst = rng.integers(0, V, n).astype(np.uint64)
    keys = np.unique((src << np.uint64(42)) | (dst << np.uint64(20)) | rng.integers(0, 50, n).astype(np.uint64))
    keys = oracle.shuffle(keys, 3)
    g, o = engine.Lpma(V), oracle.OracleLpma(V)
    for a in range(0, keys.size, max(1, keys.size // 5)):
        b = keys[a:a + max(1, keys.size // 5)]
        g.update(ins=_dev(b))
        o.update(ins=b)
        k, v = o.export_sorted()
        srcs = np.arange(V, dtype=np.uint32)
        offs, nb, nv = g.query_neighbors(_dev(srcs, np.uint32))
        eo, en, ev = oracle.neighbors(k, v, srcs, np.full(V, 0xFFFFFFFF, np.uint64), V)
        assert np.array_equal(offs.cpu().numpy().astype(np.int64), eo)
        assert np.array_equal(nb.cpu().numpy().astype(np.int64), en)
        dist, _, _ = g.bfs(_dev(np.array([0]), np.uint32))
        assert np.array_equal(dist.cpu().numpy().astype(np.int64), oracle.bfs(k, V, [0]))
    g.close()
