"""The benchmark's edge streams (host logic, no GPU): the insert and delete
sequences are cyclic, so any step count yields full batches in order."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def test_stream_is_cyclic():
    import torch
    import bench
    n, B = 10, 4
    ins_seq = torch.arange(n, dtype=torch.int64)
    del_seq = torch.arange(100, 100 + n, dtype=torch.int64)
    st = bench.Stream(ins_seq, del_seq)
    got = [st.next("ins", B).tolist() for _ in range(4)]
    assert got == [[0, 1, 2, 3], [4, 5, 6, 7], [8, 9, 0, 1], [2, 3, 4, 5]]
    assert st.next("del", B).tolist() == [100, 101, 102, 103]


def test_cpu_baseline_batches_wrap():
    import bench
    from oracle import pyoracle as O
    e = O.shuffle(O.rmat_edges(3, 10, 8), 4)
    r = bench.cpu_baseline((e, e.size // 2), 3000, 12, 2)  # 12 batches of 3000 > the 8K-edge stream
    assert len(r["lat"]) == 12 and r["value"] > 0


class _OracleAsEngine:
    """The oracle behind the two calls the bench's check makes."""

    def __init__(self, o):
        self.o = o

    def export_sorted(self):
        return self.o.export_sorted()

    def to_csr(self):
        return self.o.csr()


def test_set_check_follows_the_stream_and_catches_a_wrong_set():
    import torch
    import bench
    from oracle import pyoracle as O
    V = 1 << 10
    e = O.shuffle(O.rmat_edges(5, 10, 8), 6)
    half = e.size // 2
    S = torch.from_numpy(e[:half].view(np.int64))
    o = O.OracleLpma(V)
    o.update(ins=e[:half])
    chk = bench.SetCheck(S, V)
    B = 500
    st = bench.Stream(torch.from_numpy(np.concatenate([e[half:], e[:half]]).view(np.int64)),
                      torch.from_numpy(np.concatenate([e[:half], e[half:]]).view(np.int64)))
    for i in range(6):
        kind = "ins" if i % 2 == 0 else "del"
        x = st.next(kind, B)
        s = o.update(ins=x.numpy().view(np.uint64)) if kind == "ins" else o.update(dels=x.numpy().view(np.uint64))
        chk.batch(kind, x, s, B)
    chk.point(_OracleAsEngine(o), "six batches")
    assert chk.summary()["ok"], chk.summary()
    # a key the stream never deleted goes missing: count and checksums catch it
    o.update(dels=e[half - 1:half])
    chk.point(_OracleAsEngine(o), "one key lost")
    p = chk.summary()["points"][-1]
    assert not chk.summary()["ok"] and not p["count"] and not p["checksums"]


def test_rebalance_roofline_classes_and_big_fallback():
    """18 bytes per rewritten slot over each class's kernel time; with no big
    window among the profiled steps the big class comes from the profiled
    scratch batches, and the line names that source."""
    import bench
    st = {"windows_single": 1000, "slots_small": 32 * 1000 + 640, "slots_rewritten": 32 * 1000 + 640}
    res = {"prof": {"exec_single": (2, 0.02), "exec_small": (2, 0.004)}, "pstats": [st, st]}
    rb = bench.rebalance_roofline(res, 1000.0, "test")
    assert rb["single"]["bytes_per_step"] == 18 * 32000 and rb["small"]["bytes_per_step"] == 18 * 640
    assert abs(rb["single"]["ms_per_step"] - 0.01) < 1e-12 and rb["big"]["frac"] == 0.0
    assert "source" not in rb["big"]
    big = {"windows_single": 10, "slots_small": 320, "slots_rewritten": 320 + (1 << 20)}
    res["big_alt"] = {"prof": {"exec_gather": (1, 0.2), "exec_spread": (1, 0.1)}, "pstats": [st, big],
                      "source": "scratch"}
    rb = bench.rebalance_roofline(res, 1000.0, "test")
    assert rb["big"]["source"] == "scratch"
    want = 18 * (big["slots_rewritten"] - big["slots_small"]) / 2
    assert rb["big"]["bytes_per_step"] == want and abs(rb["big"]["ms_per_step"] - 0.15) < 1e-12
