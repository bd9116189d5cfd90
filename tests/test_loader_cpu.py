"""Edgelist / timestamp / query file readers (host code of the C ABI; no GPU).

Formats of the reference's drivers: README.md:9-20 ("N E" then E lines
"src dst"), read_edgelist_and_timestamps (test.cu:191-221: one timestamp
per edge), read_queries (test.cu:223-241: "Q" then "src lb ub" lines).
"""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def rp():
    import __graft_entry__
    __graft_entry__._load_builder().build()
    from lpma_gb300 import rpma
    return rpma


def test_edgelist_roundtrip(rp, tmp_path):
    rng = np.random.default_rng(0)
    V, E = 1000, 5000
    src, dst = rng.integers(0, V, E), rng.integers(0, V, E)
    lines = ["%d %d" % (V, E)] + ["%d\t%d" % (s, d) for s, d in zip(src, dst)]
    p = tmp_path / "g.edgelist"
    p.write_text("\n".join(lines) + "\n")
    keys, n = rp.read_edgelist(str(p))
    assert n == V
    want = (src.astype(np.uint64) << np.uint64(42)) | (dst.astype(np.uint64) << np.uint64(20))
    assert np.array_equal(keys, want)
    t = rng.integers(0, 1 << 20, E)
    tp = tmp_path / "g.timestamps"
    tp.write_text("\n".join(str(x) for x in t) + "\n")
    keys_t, _ = rp.read_edgelist(str(p), str(tp))
    assert np.array_equal(keys_t, want | t.astype(np.uint64))


def test_queries_roundtrip(rp, tmp_path):
    p = tmp_path / "g.query"
    p.write_text("3\n0 0 10\n7 5 4294967295\n2 100 200\n")
    srcs, wins = rp.read_queries(str(p))
    assert srcs.tolist() == [0, 7, 2]
    assert wins.tolist() == [10, (5 << 32) | 0xFFFFFFFF, (100 << 32) | 200]


@pytest.mark.parametrize("body", ["3 2\n0 1\n", "3 2\n0 1\n1 3\n", "3 2\n0 x\n1 2\n", "", "3"])
def test_malformed_edgelists_are_rejected(rp, tmp_path, body):
    from lpma_gb300._abi import LpmaError
    p = tmp_path / "bad.edgelist"
    p.write_text(body)
    with pytest.raises(LpmaError) as ei:
        rp.read_edgelist(str(p))
    assert ei.value.status == 10  # LPMA_ERR_IO


def test_missing_file_and_bad_timestamps(rp, tmp_path):
    from lpma_gb300._abi import LpmaError
    with pytest.raises(LpmaError):
        rp.read_edgelist(str(tmp_path / "none.edgelist"))
    p = tmp_path / "g.edgelist"
    p.write_text("4 2\n0 1\n2 3\n")
    tp = tmp_path / "g.timestamps"
    tp.write_text("5\n%d\n" % (1 << 20))
    with pytest.raises(LpmaError):
        rp.read_edgelist(str(p), str(tp))


def test_sizing_call_reports_counts(rp, tmp_path):
    import ctypes
    from lpma_gb300 import _abi
    p = tmp_path / "g.edgelist"
    p.write_text("10 3\n0 1\n2 3\n4 5\n")
    L = _abi.load()
    V, E = ctypes.c_uint32(), ctypes.c_size_t()
    rc = L.lpma_read_edgelist(str(p).encode(), None, None, 0, ctypes.byref(V), ctypes.byref(E))
    assert rc == 8 and V.value == 10 and E.value == 3  # LPMA_ERR_BUFFER_TOO_SMALL with the sizes
