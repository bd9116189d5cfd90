"""Oracle behaviour on the CPU: the reference's own result checks and the
batch semantics of the delete extension.

Checks taken from the reference's drivers: the stored key set equals the
sorted input with sentinels set apart (test_update_rpma.cu:131-165), every
row of the CSR view holds the vertex's sorted neighbours and is closed by
its sentinel (test_csr.cu:14-39).
"""
import numpy as np
import pytest

SENT_LOW = np.uint64(0x000003FFFFEFFFFF)


def _set(keys):
    return set(int(x) for x in keys)


def check_against_set(o, ref, V):
    from oracle.pyoracle import sentinel_key
    k, v = o.export_sorted()
    assert np.all(k[1:] > k[:-1])
    edges = k[(k & np.uint64(0x000003FFFFFFFFFF)) != SENT_LOW]
    assert _set(edges) == ref
    assert _set(k[(k & np.uint64(0x000003FFFFFFFFFF)) == SENT_LOW]) == {sentinel_key(x) for x in range(V)}
    # CSR view: rows sorted by dst, sentinel closes each row
    ro, ci, vals = o.csr()
    ks = np.array(sorted(ref), dtype=np.uint64)
    src = (ks >> np.uint64(42)).astype(np.int64)
    dst = ((ks >> np.uint64(20)) & np.uint64(0x3FFFFF)).astype(np.int64)
    cnt = np.bincount(src, minlength=V)
    assert np.array_equal(np.diff(ro.astype(np.int64)) - 1, cnt)
    assert np.array_equal(ci[ro[1:].astype(np.int64) - 1], np.arange(V))
    assert np.all(vals[ro[1:].astype(np.int64) - 1] == 0xFF)
    keep = np.ones(ci.size, bool)
    keep[ro[1:].astype(np.int64) - 1] = False
    assert np.array_equal(ci[keep].astype(np.int64), dst)


def test_insert_stream_config1_shape(oracle):
    V = 1 << 12
    e = oracle.shuffle(oracle.rmat_edges(1, 12, 16), 101)
    o = oracle.OracleLpma(V)
    half = e.size // 2
    o.update(ins=e[:half])
    ref = _set(e[:half])
    batches = [e[i:i + 1024] for i in range(half, e.size, 1024)]
    for b in batches:
        o.update(ins=b)
        ref |= _set(b)
    check_against_set(o, ref, V)
    for b in reversed(batches):
        o.update(dels=b)
        ref -= _set(b)
    check_against_set(o, ref, V)


def test_batch_semantics(oracle):
    V = 256
    e = oracle.shuffle(oracle.rmat_edges(4, 8, 8), 3)
    o = oracle.OracleLpma(V)
    st = o.update(ins=e[:500], ins_vals=np.full(500, 7, np.uint8))
    assert st["n_ins_applied"] == 500
    # duplicates in a batch collapse; the last insert gives the value
    ins = np.concatenate([e[500:510], e[500:510]])
    vals = np.concatenate([np.full(10, 3, np.uint8), np.full(10, 9, np.uint8)])
    st = o.update(ins=ins, ins_vals=vals)
    assert st["n_ins_applied"] == 10 and st["n_noop"] == 10
    k, v = o.export_sorted()
    pos = np.searchsorted(k, np.sort(e[500:510]))
    assert np.all(v[pos] == 9)
    # insert of a present key overwrites its value in place
    st = o.update(ins=e[:3], ins_vals=np.array([11, 12, 13], np.uint8))
    assert st["n_upserts"] == 3 and st["n_ins_applied"] == 0
    # delete of an absent key is a no-op; insert + delete of a key leaves it present
    st = o.update(ins=e[600:601], dels=np.concatenate([e[600:601], e[700:701]]))
    assert st["n_ins_applied"] == 1 and st["n_del_applied"] == 0 and st["n_noop"] == 2
    assert int(e[600]) in _set(o.export_sorted()[0])


def test_rejected_inputs_change_nothing(oracle):
    V = 128
    o = oracle.OracleLpma(V)
    e = oracle.shuffle(oracle.rmat_edges(5, 7, 8), 1)
    o.update(ins=e[:300])
    before = o.layout()
    bad = [dict(ins=np.array([(V + 1) << 42], np.uint64)),
           dict(dels=np.array([(3 << 42) + 0x000003FFFFEFFFFF], np.uint64)),
           dict(ins=e[300:301], ins_vals=np.array([0xFF], np.uint8)),
           dict(ins=e[300:301] | np.uint64(5), thres=6)]
    for kw in bad:
        with pytest.raises(ValueError):
            o.update(**kw)
        after = o.layout()
        assert np.array_equal(before[0], after[0]) and np.array_equal(before[1], after[1])


def test_deletes_shrink_the_tree(oracle):
    V = 1 << 11
    e = oracle.shuffle(oracle.rmat_edges(9, 11, 16), 2)
    o = oracle.OracleLpma(V)
    o.update(ins=e)
    h0 = o.height
    ref = _set(e)
    for i in range(0, int(e.size * 0.9), 2048):
        o.update(dels=e[i:i + 2048])
        ref -= _set(e[i:i + 2048])
    assert o.height < h0
    check_against_set(o, ref, V)


def test_timestamp_expiry(oracle):
    V = 512
    e = oracle.shuffle(oracle.rmat_edges(6, 9, 16), 8)
    t = (np.arange(e.size) // 400).astype(np.uint64) + np.uint64(1)
    keys = e | t
    o = oracle.OracleLpma(V)
    for i in range(0, keys.size, 400):
        thres = max(0, int(t[i]) - 3)
        o.update(ins=keys[i:i + 400], thres=thres)
    k, _ = o.export_sorted()
    assert np.all(k[1:] > k[:-1])


def test_cpu_baseline_matches_numpy(oracle):
    V = 1 << 12
    e = oracle.shuffle(oracle.rmat_edges(2, 12, 16), 5)
    for threads in (1, 4):
        c = oracle.CsrBaseline(V, threads=threads)
        half = e.size // 2
        c.load(e[:half])
        cur = np.sort(e[:half])
        for i in range(half, e.size, 3000):
            c.insert(e[i:i + 3000])
            cur = np.union1d(cur, e[i:i + 3000])
            assert np.array_equal(c.edges(), cur)
        c.delete(e[:2000])
        cur = np.setdiff1d(cur, e[:2000])
        assert np.array_equal(c.edges(), cur)
        ro = c.row_offset()
        src = (cur >> np.uint64(42)).astype(np.int64)
        assert np.array_equal(np.diff(ro.astype(np.int64)), np.bincount(src, minlength=V))
        c.close()


@pytest.mark.parametrize("V", [13, 20, 53, 96, 97, 1000])
def test_create_sizes(oracle, V):
    o = oracle.OracleLpma(V)
    check_against_set(o, set(), V)
