"""GPU parity: the CUDA engine, called through the C ABI, against the CPU oracle.

Bit-exact: after every batch the physical layout (keys and values of every
slot of the reference's level arrays laid end to end), the sentinel slots
(the reference's csr_idx/csr_lane), the height and the CSR view must equal
the oracle's.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint64).view(np.int64)).cuda()


def _dev8(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint8)).cuda()


def assert_same(g, o, where=""):
    gk, gv, gs, gh = g.layout()
    ok_, ov = o.layout()
    assert gh == o.height, "%s: height %d vs oracle %d" % (where, gh, o.height)
    if not np.array_equal(gk, ok_):
        bad = np.nonzero(gk != ok_)[0]
        raise AssertionError("%s: %d key slots differ, first at %d: %x vs %x" % (where, bad.size, bad[0], gk[bad[0]],
                                                                                ok_[bad[0]]))
    assert np.array_equal(gv, ov), "%s: values differ" % where
    assert np.array_equal(gs, o.sentinel_slots()), "%s: sentinel slots differ" % where
    assert g.num_items == o.num_items(), where


def assert_csr(g, o):
    ro, ci, va = g.to_csr()
    oro, oci, ova = o.csr()
    assert np.array_equal(ro, oro)
    assert np.array_equal(ci, oci)
    assert np.array_equal(va, ova)
    k, v = g.export_sorted()
    ok_, ov = o.export_sorted()
    assert np.array_equal(k, ok_) and np.array_equal(v, ov)


def test_generator_and_shuffle_match_cpu(engine, oracle):
    import torch
    scale, ef = 14, 16
    out = torch.empty((1 << scale) * ef, dtype=torch.int64, device="cuda")
    n = engine.gen_rmat_device(3, scale, ef, out)
    ref = oracle.rmat_edges(3, scale, ef)
    got = out[:n].cpu().numpy().view(np.uint64)
    assert n == ref.size and np.array_equal(got, ref)
    engine.shuffle_device(9, out[:n])
    assert np.array_equal(out[:n].cpu().numpy().view(np.uint64), oracle.shuffle(ref, 9))


@pytest.mark.parametrize("V", [1, 5, 13, 20, 33, 52, 53, 96, 97, 200, 4096])
def test_create_small_graphs(engine, oracle, V):
    g = engine.Lpma(V)
    o = oracle.OracleLpma(V)
    assert_same(g, o, "create V=%d" % V)
    assert_csr(g, o)


def _stream(oracle, seed, scale, ef, batch):
    e = oracle.shuffle(oracle.rmat_edges(seed, scale, ef), seed + 100)
    half = e.size // 2
    b = [(i, min(i + batch, e.size)) for i in range(half, e.size, batch)]
    return e, half, b


def test_config1_insert_then_delete_reverse(engine, oracle):
    """Scale-16 R-MAT, 50% bulk, batches of 16,384 inserted then deleted in reverse."""
    V = 1 << 16
    e, half, batches = _stream(oracle, 1, 16, 16, 16384)
    g, o = engine.Lpma(V), oracle.OracleLpma(V)
    d = _dev(e)
    g.update(ins=d[:half])
    o.update(ins=e[:half])
    assert_same(g, o, "bulk")
    for a, b in batches:
        sg = g.update(ins=d[a:b])
        so = o.update(ins=e[a:b])
        assert sg["n_ins_applied"] == so["n_ins_applied"]
        assert_same(g, o, "insert %d" % a)
    assert_csr(g, o)
    for a, b in reversed(batches):
        g.update(dels=d[a:b])
        o.update(dels=e[a:b])
        assert_same(g, o, "delete %d" % a)
    assert_csr(g, o)


@pytest.mark.parametrize("batch", [1, 7, 100, 1000, 5000, 30000])
def test_mixed_batches_scale14(engine, oracle, batch):
    V = 1 << 14
    e, half, batches = _stream(oracle, 5 + batch, 14, 16, batch)
    g, o = engine.Lpma(V), oracle.OracleLpma(V)
    d = _dev(e)
    g.update(ins=d[:half])
    o.update(ins=e[:half])
    rng = np.random.default_rng(batch)
    stored = half
    for i, (a, b) in enumerate(batches[:12]):
        g.update(ins=d[a:b])
        o.update(ins=e[a:b])
        assert_same(g, o, "ins %d" % i)
        # delete a random sample of what is stored, plus some absent keys
        k = rng.choice(stored, size=min(b - a, stored), replace=False)
        dels = np.concatenate([e[k], e[-3:]])
        g.update(dels=_dev(dels))
        o.update(dels=dels)
        assert_same(g, o, "del %d" % i)
    assert_csr(g, o)


def test_bulk_then_heavy_deletes_halving(engine, oracle):
    V = 1 << 13
    e = oracle.shuffle(oracle.rmat_edges(21, 13, 16), 4)
    g, o = engine.Lpma(V), oracle.OracleLpma(V)
    g.update(ins=_dev(e))
    o.update(ins=e)
    heights = [o.height]
    lowered = 0
    for i in range(0, int(e.size * 0.95), 4096):
        sg = g.update(dels=_dev(e[i:i + 4096]))
        so = o.update(dels=e[i:i + 4096])
        assert_same(g, o, "del %d" % i)
        # update_rpma's return value: true after any overflow, also when the
        # rebuild it triggers lowers the height
        for key in ("levelup", "overflow", "rebuilt", "root_executed"):
            assert sg[key] == so[key], "del %d: %s %d vs %d" % (i, key, sg[key], so[key])
        if sg["height_after"] < sg["height_before"]:
            assert sg["rebuilt"] and sg["levelup"], sg
            lowered += 1
        heights.append(o.height)
    assert heights[-1] < heights[0] and lowered > 0
    assert_csr(g, o)


def test_batch_semantics(engine, oracle):
    """Duplicates, upserts, insert+delete of one key, absent deletes, values."""
    V = 1 << 10
    e = oracle.shuffle(oracle.rmat_edges(8, 10, 8), 2)
    g, o = engine.Lpma(V), oracle.OracleLpma(V)
    vals = (np.arange(e.size) % 200 + 1).astype(np.uint8)
    g.update(ins=_dev(e[:3000]), ins_vals=_dev8(vals[:3000]))
    o.update(ins=e[:3000], ins_vals=vals[:3000])
    assert_same(g, o, "bulk")
    ins = np.concatenate([e[2990:3100], e[3000:3050], e[100:120]])  # dups + upserts
    iv = (np.arange(ins.size) % 250 + 2).astype(np.uint8)
    dels = np.concatenate([e[50:70], e[3100:3110], e[110:115]])      # present, absent, also inserted
    sg = g.update(ins=_dev(ins), ins_vals=_dev8(iv), dels=_dev(dels))
    so = o.update(ins=ins, ins_vals=iv, dels=dels)
    for k in ("n_ins_applied", "n_upserts", "n_del_applied", "n_noop"):
        assert sg[k] == so[k], k
    assert_same(g, o, "mixed")
    assert_csr(g, o)
    # empty batch
    g.update()
    assert_same(g, o, "empty")


def test_invalid_keys_rejected_without_change(engine, oracle):
    from lpma_gb300 import LpmaError
    V = 1 << 10
    e = oracle.shuffle(oracle.rmat_edges(8, 10, 8), 2)
    g, o = engine.Lpma(V), oracle.OracleLpma(V)
    g.update(ins=_dev(e[:2000]))
    o.update(ins=e[:2000])
    bad = [
        dict(ins=np.array([(1 << 64) - 1], np.uint64)),                       # KEY_NONE
        dict(ins=np.array([(V + 5) << 42], np.uint64)),                       # src out of range
        dict(ins=np.array([(3 << 42) | ((V + 1) << 20)], np.uint64)),         # dst out of range
        dict(dels=np.array([(7 << 42) + 0x000003FFFFEFFFFF], np.uint64)),      # sentinel delete
        dict(ins=e[2000:2001], ins_vals=np.array([0xFF], np.uint8)),          # tombstone value
    ]
    for kw in bad:
        dkw = {k: (_dev8(v) if k == "ins_vals" else _dev(v)) for k, v in kw.items()}
        with pytest.raises(LpmaError):
            g.update(**dkw)
        assert_same(g, o, "after rejected %s" % list(kw))


def test_host_entry_point_and_pair32(engine, oracle):
    V = 1 << 12
    e = oracle.shuffle(oracle.rmat_edges(4, 12, 8), 3)
    g, o = engine.Lpma(V), oracle.OracleLpma(V)
    g.update(ins=e[:5000])          # numpy -> lpma_update_host
    o.update(ins=e[:5000])
    assert_same(g, o, "host path")
    cfg = engine.default_config(key_format=1)
    g2 = engine.Lpma(V, config=cfg)
    pairs = ((e >> np.uint64(42)) << np.uint64(32)) | ((e >> np.uint64(20)) & np.uint64(0x3FFFFF))
    g2.update(ins=_dev(pairs[:5000]))
    k1, _ = g.export_sorted()
    k2, _ = g2.export_sorted()
    assert np.array_equal(k1, k2)


def test_host_batches_back_to_back(engine, oracle):
    """lpma_update_host calls in a row through one reused host buffer: each
    call's copy runs on the handle's copy stream while the previous call's
    executors may still run, and the buffer is overwritten as soon as the
    call returns.  Sizes grow past the staging capacity twice."""
    V = 1 << 12
    e = oracle.shuffle(oracle.rmat_edges(21, 12, 16), 4)
    import torch
    g, o = engine.Lpma(V), oracle.OracleLpma(V)
    pinned = torch.empty(e.size, dtype=torch.int64, pin_memory=True)  # asynchronous copies
    buf = pinned.numpy().view(np.uint64)
    rng = np.random.default_rng(2)
    pos = 0
    for i, n in enumerate([700, 3000, 64, 9000, 1, 20000, 500, 40000]):
        ins = e[pos:pos + n]
        pos += ins.size
        k, _ = o.export_sorted()
        live = k[((k >> np.uint64(20)) & np.uint64(0x3FFFFF)) != np.uint64(0x3FFFFE)]
        dels = rng.choice(live, size=min(n // 3, live.size), replace=False) if live.size else live
        if i % 2:
            buf[:ins.size] = ins
            g.update(ins=buf[:ins.size], dels=dels)
        else:
            buf[:dels.size] = dels
            g.update(ins=ins, dels=buf[:dels.size])
        buf[:] = np.uint64(0xFFFFFFFFFFFFFFFF)  # the call has returned: its copy must be done
        o.update(ins=ins, dels=dels)
        assert_same(g, o, "host batch %d" % i)
    assert_csr(g, o)
    g.close()


def test_timestamp_expiry(engine, oracle):
    V = 1 << 10
    e = oracle.shuffle(oracle.rmat_edges(6, 10, 16), 8)
    t = (np.arange(e.size) // 500).astype(np.uint64) + np.uint64(1)
    keys = e | t
    g, o = engine.Lpma(V), oracle.OracleLpma(V)
    for i in range(0, keys.size, 500):
        thres = max(0, int(t[i]) - 4)
        g.update(ins=_dev(keys[i:i + 500]), thres=thres)
        o.update(ins=keys[i:i + 500], thres=thres)
        assert_same(g, o, "ts batch %d" % i)
    assert_csr(g, o)


@pytest.mark.parametrize("batch", [1024, 10240, 102400])
def test_scale18_stream(engine, oracle, batch):
    """Larger tree: root rebalances, eager level-ups and rebuilds along the stream."""
    V = 1 << 18
    e, half, batches = _stream(oracle, 31, 18, 16, batch)
    g, o = engine.Lpma(V), oracle.OracleLpma(V)
    d = _dev(e)
    g.update(ins=d[:half])
    o.update(ins=e[:half])
    assert_same(g, o, "bulk")
    events = set()
    for i, (a, b) in enumerate(batches[:6]):
        s1 = g.update(ins=d[a:b])
        o.update(ins=e[a:b])
        assert_same(g, o, "ins %d" % i)
        s2 = g.update(dels=d[a:(a + b) // 2])
        o.update(dels=e[a:(a + b) // 2])
        assert_same(g, o, "del %d" % i)
        for s in (s1, s2):
            assert s["levelup"] == int(bool(s["root_executed"] or s["overflow"])), s
            for k in ("root_executed", "eager_levelup", "rebuilt", "levelup_path", "fill_empty"):
                if s[k]:
                    events.add(k)
    assert_csr(g, o)


PATH_FLAGS = ("overflow", "levelup_path", "rebuilt", "eager_levelup", "root_executed", "fill_empty", "levelup")


@pytest.mark.parametrize("V,frac,dfrac,path", [
    (1 << 10, 0.8, 0.0, "levelup_path"),  # an overflow absorbed by one new level
    (1 << 10, 0.8, 0.1, "levelup_path"),  # the same with deletes pending in the batch
    (1 << 12, 0.8, 0.05, "fill_empty"),   # the level-up leaves an empty leaf: full respread
    (1 << 12, 0.2, 0.1, "rebuilt"),       # an overflow that needs a rebuild
])
def test_overflow_paths(engine, oracle, V, frac, dfrac, path):
    """Growing batches (each frac of what was inserted so far, plus deletes
    of dfrac of the stored edges) drive the root window past its capacity.
    The updates no window absorbed stay pending across the level-up; the
    path each batch takes and the layout after it match the oracle."""
    scale = int(V).bit_length() - 1
    e = oracle.shuffle(oracle.rmat_edges(41, scale, 16), 3)
    g, o = engine.Lpma(V), oracle.OracleLpma(V)
    rng = np.random.default_rng(7)
    pos = e.size // 8
    g.update(ins=_dev(e[:pos]))
    o.update(ins=e[:pos])
    seen = set()
    for i in range(6):
        n = max(1, int(frac * pos))
        if pos + n > e.size:
            break
        k, _ = o.export_sorted()
        live = k[((k >> np.uint64(20)) & np.uint64(0x3FFFFF)) != np.uint64(0x3FFFFE)]
        dels = rng.choice(live, size=int(dfrac * live.size), replace=False) if dfrac else np.empty(0, np.uint64)
        sg = g.update(ins=_dev(e[pos:pos + n]), dels=_dev(dels))
        so = o.update(ins=e[pos:pos + n], dels=dels)
        pos += n
        assert_same(g, o, "batch %d" % i)
        for key in PATH_FLAGS:
            assert bool(sg[key]) == bool(so[key]), "batch %d: %s %d vs %d" % (i, key, sg[key], so[key])
            if sg[key]:
                seen.add(key)
    assert path in seen and "overflow" in seen, seen
    assert_csr(g, o)
    g.close()


def test_cached_front_survives_buffer_moves(engine, oracle):
    """A repeated batch shape replays a captured front; batch buffers that
    grow in between, and a sort-mode change, must not leave a stale one."""
    V = 1 << 11
    e = oracle.shuffle(oracle.rmat_edges(31, 11, 16), 4)
    g, o = engine.Lpma(V), oracle.OracleLpma(V)
    d = _dev(e)
    pos = 0
    plan = [100, 100, 100, 5000, 100, 100, 9000, 100, 100]
    for i, b in enumerate(plan):
        if i == 7:
            g.set_flags(1)
        if i == 8:
            g.set_flags(0)
        g.update(ins=d[pos:pos + b])
        o.update(ins=e[pos:pos + b])
        pos += b
        assert_same(g, o, "step %d (batch %d)" % (i, b))
    g.close()


def test_shrink_then_grow_with_poisoned_buffers(engine, oracle, monkeypatch):
    """Heights move down and up again through rebuilds, an eager level-up and
    the one-level growth path, with every new device buffer filled with
    garbage (LPMA_POISON=1): no kernel may read a count, key or flag that
    no kernel wrote (the last window of a level once read one count past
    the last segment)."""
    monkeypatch.setenv("LPMA_POISON", "1")
    V = 1 << 12
    e = oracle.shuffle(oracle.rmat_edges(26, 12, 16), 27)
    half = e.size // 2
    g, o = engine.Lpma(V), oracle.OracleLpma(V)
    d = _dev(e)
    g.update(ins=d[:half])
    o.update(ins=e[:half])
    assert_same(g, o, "bulk")
    steps = [("del", 0, int(half * 0.95)), ("del", int(half * 0.95), int(half * 0.955)),
             ("del", int(half * 0.955), int(half * 0.985)), ("ins", half, e.size), ("ins", 0, int(half * 0.3))]
    for kind, a, b in steps:
        if kind == "del":
            g.update(dels=d[a:b])
            o.update(dels=e[a:b])
        else:
            g.update(ins=d[a:b])
            o.update(ins=e[a:b])
        assert_same(g, o, "%s %d:%d" % (kind, a, b))
    assert_csr(g, o)
    g.close()


def _skew_stream(oracle, seed, scale, ef, batch, n_batches, bulk_frac=0.25, hub_frac=0.9):
    """Config-3 shape: half uniform (Erdos-Renyi) and half R-MAT (.7, .1, .1)
    edges; a quarter preloaded; batches of batch/2 inserts (hub_frac of them
    with a source among the top 1% out-degrees) and batch/2 deletes of
    stored edges."""
    er = oracle.rmat_edges(seed, scale, ef, a=0.25, b=0.25, c=0.25)
    rm = oracle.rmat_edges(seed + 1, scale, ef, a=0.7, b=0.1, c=0.1)
    e = oracle.shuffle(np.union1d(er, rm), seed + 2)
    src = (e >> np.uint64(42)).astype(np.int64)
    deg = np.bincount(src, minlength=1 << scale)
    hubs = np.zeros(1 << scale, bool)
    hubs[np.argsort(-deg)[:max(1, (1 << scale) // 100)]] = True
    nb = int(e.size * bulk_frac)
    bulk, pool = e[:nb], e[nb:]
    is_hub = hubs[(pool >> np.uint64(42)).astype(np.int64)]
    hub_pool, cold_pool = pool[is_hub], pool[~is_hub]
    rng = np.random.default_rng(seed)
    stored = set(bulk.tolist())
    batches, ph, pc = [], 0, 0
    for _ in range(n_batches):
        nh = int(batch // 2 * hub_frac)
        nc = batch // 2 - nh
        ins = np.concatenate([hub_pool[ph:ph + nh], cold_pool[pc:pc + nc]])
        ph, pc = ph + nh, pc + nc
        dels = rng.choice(np.array(sorted(stored), np.uint64), size=min(batch // 2, len(stored)), replace=False)
        stored = (stored - set(dels.tolist())) | set(ins.tolist())
        batches.append((ins, dels))
    return bulk, batches


@pytest.mark.parametrize("scale,batch", [(11, 2048), (13, 8192)])
def test_skewed_mixed_batches(engine, oracle, scale, batch):
    """Hub-heavy inserts with uniform deletes force windows up to the root,
    level-ups and shrinking rebuilds: slot-for-slot parity after each batch."""
    V = 1 << scale
    bulk, batches = _skew_stream(oracle, 40 + scale, scale, 16, batch, 8)
    g, o = engine.Lpma(V), oracle.OracleLpma(V)
    g.update(ins=_dev(bulk))
    o.update(ins=bulk)
    assert_same(g, o, "bulk")
    big = 0
    for i, (ins, dels) in enumerate(batches):
        sg = g.update(ins=_dev(ins), dels=_dev(dels))
        so = o.update(ins=ins, dels=dels)
        assert sg["n_ins_applied"] == so["n_ins_applied"] and sg["n_del_applied"] == so["n_del_applied"]
        big += sg["windows_big"] + sg["rebuilt"] + sg["levelup_path"] + sg["root_executed"]
        assert_same(g, o, "skewed batch %d" % i)
    assert big > 0  # the stress reached the big-window / resize paths
    assert_csr(g, o)
    g.close()
