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
