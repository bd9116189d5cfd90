"""The oracle against the reference's own code, compiled for the host.

oracle/ref_host.py copies functions of the reference's update path
verbatim out of rpma.cuh / gpma.cuh and compiles them with g++ (CUDA
qualifiers defined away, kernels run as one thread).  Each step of the
oracle that has such a counterpart is compared with it exactly, on many
inputs: the index macros and fls / lls, the density table, the skip state
machine, the resize height rule, the locate descent (locate_leaf_kernel
and locate_leaf_kernel_mixed) over layouts of seeded update streams, and
the even redistribution of redispatch_kernel (slots, values and the
csr_idx / csr_lane of every sentinel).

Runs where the reference sources are present (this is where the fixtures
in tests/golden are generated); skipped elsewhere.  The committed fixtures
carry the same checks to machines without the reference
(tests/test_oracle_golden.py).
"""
import numpy as np
import pytest

KEY_NONE = np.uint64(0xFFFFFFFFFFFFFFFF)


@pytest.fixture(scope="module")
def ref():
    from oracle import ref_host
    try:
        ref_host.build()
    except ref_host.RefUnavailable as e:
        pytest.skip("reference pieces unavailable: %s" % e)
    return ref_host


def test_index_macros_and_bit_scans(ref, oracle):
    L, O = ref.lib(), oracle.lib()
    rng = np.random.default_rng(1)
    xs = list(range(1, 70)) + [int(x) for x in rng.integers(1, 1 << 32, 2000)] + [0xFFFFFFFF, 1 << 31]
    for x in xs:
        assert L.ref_fls(x) == int(x).bit_length()
        assert L.ref_lls(x) == (x & -x).bit_length()
    for H in range(0, 12):
        n = 32 * ((2 << H) - 1)
        lins = range(n) if n <= 4096 else rng.integers(0, n, 4096)
        for lin in lins:
            lin = int(lin)
            i = L.ref_get_idx(lin, H)
            ln = L.ref_get_lane(lin, i, H)
            assert O.opma_get_idx(lin, H) == i
            assert O.opma_get_lane(lin, i, H) == ln
            assert O.opma_get_linear_idx(i, ln, H) == L.ref_get_linear_idx(i, ln, H)


def test_density_skip_and_resize_rules(ref, oracle):
    import ctypes
    O = oracle.lib()
    lo, up = ref.density()
    olo, oup = np.zeros(26, np.uint32), np.zeros(26, np.uint32)
    O.opma_density_table(olo.ctypes.data_as(ctypes.c_void_p), oup.ctypes.data_as(ctypes.c_void_p), 26)
    assert np.array_equal(lo, olo) and np.array_equal(up, oup)
    for H in range(0, 25):
        want = ref.skip_table(H, H + 2)  # the reference evaluates levels 0 .. H+1
        got = np.zeros(H + 2, np.uint8)
        O.opma_skip_table(H, got.ctypes.data_as(ctypes.c_void_p), H + 2)
        assert np.array_equal(want, got), H
    rng = np.random.default_rng(2)
    L = ref.lib()
    for _ in range(3000):
        H = int(rng.integers(0, 21))
        comp = int(rng.integers(0, 32 * (2 << min(H + 2, 21))))
        upd = int(rng.integers(0, 1 << int(rng.integers(0, 22))))
        root = int(rng.integers(0, 2))
        assert L.ref_resize_height(H, comp, upd, root) == O.opma_resize_height(comp + upd, root)


def _streams(oracle):
    """Layouts of seeded streams: inserts, deletes (tombstones until their
    window runs), heights 0 to about 10."""
    out = []
    for seed, scale, ef, batch in [(3, 4, 4, 7), (5, 8, 8, 300), (7, 10, 8, 2000), (9, 12, 16, 9000)]:
        V = 1 << scale
        e = oracle.shuffle(oracle.rmat_edges(seed, scale, ef), seed + 1)
        o = oracle.OracleLpma(V)
        out.append((o, e, "create"))
        rng = np.random.default_rng(seed)
        pos = 0
        while pos < e.size:
            o.update(ins=e[pos:pos + batch])
            pos += batch
            k, _ = o.export_sorted()
            if k.size > V and rng.random() < 0.5:
                o.update(dels=rng.choice(e[:pos], size=min(pos, batch // 3 + 1), replace=False))
            out.append((o, e, "after %d" % pos))
            yield o, e, pos
    return out


def test_locate_matches_reference_descent(ref, oracle):
    rng = np.random.default_rng(4)
    cases = 0
    for o, e, pos in _streams(oracle):
        k, _ = o.layout()
        H = o.height
        stored, _ = o.export_sorted()
        q = np.concatenate([e[:pos], stored, rng.integers(0, 1 << 63, 500, dtype=np.uint64),
                            stored[:50] + np.uint64(1), stored[-50:] - np.uint64(1),
                            np.array([0, 1 << 62], np.uint64)])
        want = ref.locate(k, H, q)
        assert np.array_equal(want, ref.locate_mixed(k, H, q))
        got = o.locate(q)
        bad = np.nonzero(want != got)[0]
        assert bad.size == 0, "H=%d: %d keys located differently, first %x: %d vs %d" % (
            H, bad.size, q[bad[0]], want[bad[0]], got[bad[0]])
        cases += 1
    assert cases > 10


def test_redistribution_matches_reference(ref, oracle):
    rng = np.random.default_rng(5)
    V = 1 << 12
    for _ in range(400):
        H = int(rng.integers(0, 9))
        nslots = 32 * ((2 << H) - 1)
        level = int(rng.integers(0, H + 2))
        width = 32 << level
        node = int(rng.integers(0, (nslots + 32) // width)) * width
        if node + width >= 32 << (H + 1):  # the last window of a level is clipped by one segment
            width -= 32
        if width <= 0:
            continue
        m = int(rng.integers(0, width + 1))
        src = np.sort(rng.integers(0, V, m)).astype(np.uint64)
        items = np.sort((src << np.uint64(42)) | rng.integers(0, 1 << 42, m, dtype=np.uint64))
        items = np.unique(items)
        if items.size and rng.random() < 0.5:  # some sentinels among them
            sel = rng.random(items.size) < 0.2
            items[sel] = ((items[sel] >> np.uint64(42)) << np.uint64(42)) + np.uint64(0x000003FFFFEFFFFF)
            items = np.unique(items)
        m = items.size
        vals = rng.integers(1, 250, m).astype(np.uint8)
        keys = rng.integers(0, 1 << 63, nslots, dtype=np.uint64)
        hv = rng.integers(0, 256, nslots).astype(np.uint8)
        # the reference's callers clear the window's keys first (level_memset_kernel)
        phys = np.array([_phys(L_, H) for L_ in range(node, node + width)], np.int64)
        keys[phys] = KEY_NONE
        rk, rv, ci, cl = ref.redispatch(keys, hv, H, node, width, items, vals, V)
        ok_, ov = keys.copy(), hv.copy()
        sent = np.full(V, 0xFFFFFFFF, np.uint32)
        oracle.redistribute_window(H, V, node, width, items, vals, ok_, ov, sent)
        assert np.array_equal(rk, ok_) and np.array_equal(rv, ov), (H, node, width, m)
        for v in range(V):
            if ci[v + 1] != 0xFFFFFFFF:
                assert sent[v] == 32 * ((1 << int(ci[v + 1])) - 1) + int(cl[v + 1]), v
            else:
                assert sent[v] == 0xFFFFFFFF


def _phys(L, H):
    s1 = (L >> 5) + 1
    t = (s1 & -s1).bit_length() - 1
    return 32 * ((1 << (H - t)) - 1) + 32 * (s1 >> (t + 1)) + (L & 31)


# ---------------------------------------------------------------- GPMA (gpma.cuh)
def _gpma_keys(e):
    """src << 32 | dst form of leveled keys src << 42 | dst << 20."""
    return ((e >> np.uint64(42)) << np.uint64(32)) | ((e >> np.uint64(20)) & np.uint64(0x3FFFFF))


def test_gpma_size_rule_and_density(ref, oracle):
    for m in list(range(0, 300)) + [1000, 4095, 4096, 4097, 65537, 1 << 20, 5_000_000, 33_554_432, 33_554_433]:
        assert ref.gpma_size(m) == oracle.gpma_size_rule(m), m
    for seg, h in [(2, 1), (4, 2), (4, 4), (8, 7), (8, 11), (16, 12), (16, 21), (32, 25)]:
        lo, up = ref.gpma_density(seg, h)
        olo, oup = oracle.gpma_density(seg, h)
        assert np.array_equal(lo, olo) and np.array_equal(up, oup), (seg, h)


def _gpma_states(oracle):
    """GPMA oracles along seeded streams with tombstones: (oracle, edges, ops)
    where replaying ops on a new oracle gives the same state."""
    for seed, scale, ef, batch in [(3, 5, 4, 11), (5, 8, 8, 300), (7, 11, 8, 2500)]:
        V = 1 << scale
        e = _gpma_keys(oracle.shuffle(oracle.rmat_edges(seed, scale, ef), seed + 1))
        rng = np.random.default_rng(seed)
        a = oracle.OracleGpma(V)
        ops = []
        yield a, e, list(ops)
        pos = 0
        while pos < e.size:
            ops.append(("ins", e[pos:pos + batch]))
            pos += batch
            if rng.random() < 0.6:
                ops.append(("del", rng.choice(e[:pos], size=min(pos, batch // 2 + 1), replace=False)))
            for kind, keys in ops[-2:] if ops[-1][0] == "del" else ops[-1:]:
                a.update(ins=keys) if kind == "ins" else a.update(dels=keys)
            yield a, e, list(ops)


def _replay(oracle, V, ops):
    b = oracle.OracleGpma(V)
    for kind, keys in ops:
        b.update(ins=keys) if kind == "ins" else b.update(dels=keys)
    return b


def test_gpma_locate_and_handle_del_mod(ref, oracle):
    """locate_leaf_kernel with handle_del_mod (gpma.cuh:162-200): the stop
    segment of every update, and what it does in place (upsert, tombstone,
    a tombstoned key brought back), on the oracle's layouts."""
    rng = np.random.default_rng(8)
    n_cases = 0
    for a, e, ops in _gpma_states(oracle):
        keys, vals, _ = a.layout()
        size, seg, h = a.geometry()
        q = np.unique(np.concatenate([e[rng.integers(0, e.size, 200)], rng.integers(0, 1 << 40, 50, dtype=np.uint64)]))
        qv = rng.integers(1, 255, q.size).astype(np.uint8)
        qv[rng.random(q.size) < 0.3] = 0xFF  # deletes
        leaf_ref, vals_ref = ref.gpma_locate(keys, vals, seg, h, q, qv)
        b = _replay(oracle, a.V, ops)
        assert np.array_equal(b.layout()[0], keys)
        leaf_o = b.resolve_only(q, qv)
        assert np.array_equal(leaf_ref, leaf_o), (seg, h, len(ops))
        _, vals_o, _ = b.layout()
        occupied = keys != np.uint64(0xFFFFFFFFFFFFFFFF)
        assert np.array_equal(vals_ref[occupied], vals_o[occupied])
        n_cases += 1
    assert n_cases > 10


def test_gpma_redistribution(ref, oracle):
    rng = np.random.default_rng(9)
    V = 256
    for _ in range(300):
        size = 1 << int(rng.integers(2, 12))
        _, seg, h = oracle.gpma_size_rule(size)
        level = int(rng.integers(0, h + 1))
        width = seg << level
        node = int(rng.integers(0, size // width)) * width
        m = int(rng.integers(0, width + 1))
        items = np.unique((rng.integers(0, V, m).astype(np.uint64) << np.uint64(32)) |
                          rng.integers(0, V, m).astype(np.uint64))
        sel = rng.random(items.size) < 0.2
        items[sel] |= np.uint64(0xFFFFFFFF)
        items = np.unique(items)
        iv = rng.integers(1, 250, items.size).astype(np.uint8)
        keys = np.sort(rng.integers(0, 1 << 62, size, dtype=np.uint64))
        vals = rng.integers(0, 256, size).astype(np.uint8)
        keys[node:node + width] = np.uint64(0xFFFFFFFFFFFFFFFF)  # the callers clear the window first
        ro = np.zeros(V + 1, np.uint32)
        rk, rv, rro = ref.gpma_redispatch(keys, vals, node, width, seg, items, iv, ro)
        ok, ov, oro = keys.copy(), vals.copy(), ro.copy()
        oracle.gpma_spread_window(V, seg, node, width, items, iv, ok, ov, oro)
        assert np.array_equal(rk, ok) and np.array_equal(rv, ov) and np.array_equal(rro, oro), (size, seg, level)
