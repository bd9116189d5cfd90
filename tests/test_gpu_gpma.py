"""GPMA mode (LPMA_FLAG_GPMA, the flat array of gpma.cuh) against the oracle.

Bit-exact after every batch: every slot's key and value of the flat array,
the sentinel slots (row_offset[v + 1], the view analytics read), the
segment length and height, and the live key set, compared with the CPU
restatement of update_gpma (oracle/lpma_oracle.c, ogpma_*).  Covers the
first state, insert streams through the level loop, deletes as tombstones
that stay until their window is rebalanced, upserts, a tombstoned key
inserted again, repeated keys in a batch, resizes up and down, the
whole-array path for batches of 5,000,000 new keys and more, the host entry
point and rejected batches.
"""
import numpy as np
import pytest

from test_gpu_parity import _dev, _dev8

pytestmark = pytest.mark.gpu


def gkeys(e):
    """src << 32 | dst from leveled keys src << 42 | dst << 20."""
    return ((e >> np.uint64(42)) << np.uint64(32)) | ((e >> np.uint64(20)) & np.uint64(0x3FFFFF))


def make(engine, oracle, V):
    return engine.Lpma(V, config=engine.gpma_config()), oracle.OracleGpma(V)


def assert_same(g, o, where=""):
    gk, gv, gs, gh = g.layout()
    ok_, ov, oro = o.layout()
    size, seg, h = o.geometry()
    (_, _, _), (gsize, gseg, gh2) = g.gpma_view()
    assert (gsize, gseg, gh) == (size, seg, h) and gh2 == h, "%s: geometry %s vs %s" % (where, (gsize, gseg, gh),
                                                                                        (size, seg, h))
    if not np.array_equal(gk, ok_):
        bad = np.nonzero(gk != ok_)[0]
        raise AssertionError("%s: %d key slots differ, first at %d: %x vs %x" % (where, bad.size, bad[0], gk[bad[0]],
                                                                                ok_[bad[0]]))
    assert np.array_equal(gv, ov), "%s: values differ" % where
    assert np.array_equal(gs, oro[1:]), "%s: sentinel slots differ" % where
    k, v = g.export_sorted()
    ok2, ov2 = o.export_sorted()
    assert np.array_equal(k, ok2) and np.array_equal(v, ov2), "%s: live keys differ" % where
    assert g.num_items == ok2.size


@pytest.mark.parametrize("V", [1, 2, 5, 30, 62, 63, 64, 100, 1000, 4096])
def test_gpma_create(engine, oracle, V):
    g, o = make(engine, oracle, V)
    assert_same(g, o, "create V=%d" % V)
    g.close()


@pytest.mark.parametrize("batch", [1, 9, 300, 3000])
def test_gpma_insert_delete_stream(engine, oracle, batch):
    V = 1 << 11
    e = gkeys(oracle.shuffle(oracle.rmat_edges(13 + batch, 11, 16), 4))
    g, o = make(engine, oracle, V)
    d = _dev(e)
    half = e.size // 2
    g.update(ins=d[:half])
    o.update(ins=e[:half])
    assert_same(g, o, "bulk")
    rng = np.random.default_rng(batch)
    pos = half
    for i in range(min(14, (e.size - half) // batch)):
        sg = g.update(ins=d[pos:pos + batch])
        so = o.update(ins=e[pos:pos + batch])
        pos += batch
        for k in ("n_ins_applied", "n_upserts", "rebuilt", "overflow", "root_executed"):
            assert sg[k] == so[k], "ins %d: %s %d vs %d" % (i, k, sg[k], so[k])
        assert_same(g, o, "ins %d" % i)
        dels = rng.choice(e[:pos], size=max(1, batch // 2), replace=False)
        sg = g.update(dels=_dev(dels))
        so = o.update(dels=dels)
        assert sg["n_del_applied"] == so["n_del_applied"] and sg["n_noop"] == so["n_noop"]
        assert_same(g, o, "del %d" % i)
    g.close()


def test_gpma_tombstones_upserts_and_returns(engine, oracle):
    """Deletes leave tombstones in place; inserting a tombstoned key brings
    it back in place; upserts overwrite values; repeated keys in a batch and
    a key inserted and deleted in one batch follow the set rules."""
    V = 1 << 10
    e = gkeys(oracle.shuffle(oracle.rmat_edges(5, 10, 8), 6))
    g, o = make(engine, oracle, V)
    vals = (np.arange(e.size) % 200 + 1).astype(np.uint8)
    g.update(ins=_dev(e[:4000]), ins_vals=_dev8(vals[:4000]))
    o.update(ins=e[:4000], ins_vals=vals[:4000])
    assert_same(g, o, "bulk")
    g.update(dels=_dev(e[:1500]))
    o.update(dels=e[:1500])
    assert_same(g, o, "tombstones")
    ins = np.concatenate([e[1000:1200], e[3000:3100], e[4000:4100], e[4050:4080]])  # back, upserts, new, repeats
    iv = (np.arange(ins.size) % 250 + 3).astype(np.uint8)
    dels = np.concatenate([e[2000:2050], e[4100:4110], e[4000:4010], e[100:110]])  # present, absent, inserted, tombstoned
    sg = g.update(ins=_dev(ins), ins_vals=_dev8(iv), dels=_dev(dels))
    so = o.update(ins=ins, ins_vals=iv, dels=dels)
    for k in ("n_ins_applied", "n_upserts", "n_del_applied", "n_noop"):
        assert sg[k] == so[k], (k, sg[k], so[k])
    assert_same(g, o, "mixed")
    g.update()
    assert_same(g, o, "empty batch")
    g.close()


def test_gpma_grow_and_shrink(engine, oracle):
    """Heavy deletes, then inserts that reach the root: resizes down (the
    root fails its lower bound) and up again."""
    V = 1 << 12
    e = gkeys(oracle.shuffle(oracle.rmat_edges(21, 12, 16), 4))
    g, o = make(engine, oracle, V)
    nb = int(e.size * 0.6)
    g.update(ins=_dev(e[:nb]))
    o.update(ins=e[:nb])
    assert_same(g, o, "bulk")
    sizes = [o.geometry()[0]]
    g.update(dels=_dev(e[:int(nb * 0.95)]))
    o.update(dels=e[:int(nb * 0.95)])
    assert_same(g, o, "tombstones")
    resized = 0
    # new keys (tombstoned ones would come back in place and move nothing)
    for i, a in enumerate(range(nb, e.size, 2500)):
        ins = e[a:a + 2500]
        sg = g.update(ins=_dev(ins))
        so = o.update(ins=ins)
        assert sg["rebuilt"] == so["rebuilt"]
        resized += sg["rebuilt"]
        assert_same(g, o, "reinsert %d" % i)
        sizes.append(o.geometry()[0])
    assert min(sizes) < sizes[0] and resized > 0, sizes
    g.close()


def test_gpma_significant_insert(engine, oracle):
    """A batch of 5,000,000 new keys or more respreads the whole array at
    the resize rule's size (significant_insert, gpma.cuh:720-744)."""
    V = 1 << 20
    e = gkeys(oracle.shuffle(oracle.rmat_edges(2, 20, 8), 3))
    assert e.size > 5_100_000
    g, o = make(engine, oracle, V)
    d = _dev(e)
    g.update(ins=d[:100000])
    o.update(ins=e[:100000])
    sg = g.update(ins=d[100000:5_150_000])
    so = o.update(ins=e[100000:5_150_000])
    assert sg["rebuilt"] == so["rebuilt"] == 1 and sg["n_ins_applied"] == so["n_ins_applied"]
    assert_same(g, o, "significant insert")
    sg = g.update(ins=d[5_150_000:5_160_000])
    o.update(ins=e[5_150_000:5_160_000])
    assert_same(g, o, "after")
    g.close()


def test_gpma_host_entry_and_rejections(engine, oracle):
    from lpma_gb300 import LpmaError
    V = 1 << 10
    e = gkeys(oracle.shuffle(oracle.rmat_edges(8, 10, 8), 2))
    g, o = make(engine, oracle, V)
    g.update(ins=e[:3000])  # numpy: lpma_update_host
    o.update(ins=e[:3000])
    assert_same(g, o, "host entry")
    bad = [np.array([(V + 1) << 32], np.uint64), np.array([(3 << 32) | 0xFFFFFFFF], np.uint64),
           np.array([(2 << 32) | (V + 7)], np.uint64)]
    for b in bad:
        with pytest.raises(LpmaError):
            g.update(ins=_dev(b))
        with pytest.raises(LpmaError):
            g.update(dels=_dev(b))
        assert_same(g, o, "after rejected %x" % int(b[0]))
    with pytest.raises(LpmaError):
        g.update(ins=_dev(e[3000:3001]), ins_vals=_dev8(np.array([0xFF], np.uint8)))
    with pytest.raises(LpmaError):
        g.to_csr()
    assert_same(g, o, "end")
    g.close()
