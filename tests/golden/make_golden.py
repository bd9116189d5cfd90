"""Generate the layout-stream fixture of tests/golden from a second restatement.

Run from the repository root:

    python tests/golden/make_golden.py [--reference <reference checkout>]

What it writes (JSON, committed):

* small_streams.json -- layouts produced by a pure-Python restatement of the
  reference's insert path (init_csr_rpma + update_rpma, rpma.cuh:1301-1823),
  written slot for slot from the reference with its per-level arrays, for
  a few seeded small insert-only streams.  Each snapshot stores the height,
  a SHA-256 of the layout (keys and values of every slot, level arrays laid
  end to end) and, for the last snapshot of a stream, the full layout.

The whole update loop of the reference does not compile here, so these
layouts are "parity unpinned": they pin the C oracle (oracle/lpma_oracle.c)
to a second, independent restatement (different language, the reference's
own per-level data structure and locate/rebalance code paths).  The
restatement's index macros, density table and skip rule are first checked
against index_algebra.json and tables.json, which the reference's own code
produced (tests/golden/make_ref_golden.py).  With --reference, the macro
definitions are also looked up in the reference header.
"""
import hashlib
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
M32 = 0xFFFFFFFF
KEY_NONE = (1 << 64) - 1
TIME_MASK = 0xFFFFF
DST_AND_TIME_MASK = 0x000003FFFFFFFFFF
DST_AND_TIME_END = 0x000003FFFFEFFFFF
SRC_SHIFT = 42


# ----------------------------------------------------------------- rpma.cuh:98-134
def lls(x):
    r = 1
    if not (x & 0x0000FFFF):
        x >>= 16
        r += 16
    if not (x & 0x000000FF):
        x >>= 8
        r += 8
    if not (x & 0x0000000F):
        x >>= 4
        r += 4
    if not (x & 0x00000003):
        x >>= 2
        r += 2
    if not (x & 0x00000001):
        x >>= 1
        r += 1
    return r


def fls(x):
    r = 32
    if not x:
        return 0
    if not (x & 0xFFFF0000):
        x = (x << 16) & M32
        r -= 16
    if not (x & 0xFF000000):
        x = (x << 8) & M32
        r -= 8
    if not (x & 0xF0000000):
        x = (x << 4) & M32
        r -= 4
    if not (x & 0xC0000000):
        x = (x << 2) & M32
        r -= 2
    if not (x & 0x80000000):
        x = (x << 1) & M32
        r -= 1
    return r


def GET_IDX(L, H):
    return (H + 1 - lls(((L >> 5) + 1) & M32)) & M32


def GET_LANE(L, I, H):
    return ((((((L >> 5) + 1) >> (H - I)) - 1) >> 1) << 5) + (L % 32)


def GET_LINEAR_IDX(I, lane, H):
    return ((32 << (H - I)) - 32 + ((lane >> 5) << (H - I + 1) << 5)) & M32


# ----------------------------------------------------------------- tables
def density_tables(n=26):
    lower, upper = [], []
    ll = 32
    for _ in range(n):
        lower.append(int(0.42 * ll))  # SIZE_TYPE conversion truncates
        upper.append(ll)
        ll <<= 1
    return lower, upper


def skip_table(H, n=27):
    out, skip = [], False
    for level in range(n):
        if level == 4 or level == H // 3:
            skip = True
        if level == ((H // 3 - 1) & M32) or level == H + 1:
            skip = False
        out.append(1 if skip else 0)
    return out


def redistribute_counts(f, m):
    c = [0] * f
    for i in range(m):
        c[(f * i) // m] += 1
    return c


# ----------------------------------------------------------------- the reference insert path
class RefRPMA:
    """rpma.cuh's RPMA with its per-level arrays (levels_key_ptr_array)."""

    def __init__(self, row_num):
        # init_rpma, rpma.cuh:1764-1795
        self.H = 0
        self.seg = 32
        self.keys = [[KEY_NONE] * 32]
        self.vals = [[0] * 32]
        self.lower, self.upper = density_tables(26)
        self.row_num = row_num
        self.csr_idx = [0] * (row_num + 1)
        self.csr_lane = [0] * (row_num + 1)
        # init_csr_rpma, rpma.cuh:1808-1824
        rows = [(v << SRC_SHIFT) + DST_AND_TIME_END for v in range(row_num)]
        self.update(rows, [0] * row_num)

    # locate_leaf_kernel, rpma.cuh:281-315
    def locate(self, key):
        idx, lane = 0, 0
        while idx < self.H and self.keys[idx][lane] != KEY_NONE:
            if self.keys[idx][lane] > key:
                idx += 1
                lane <<= 1
                continue
            l, r = 0, self.seg - 1
            while l < r:
                mid = (l + r + 1) >> 1
                if self.keys[idx][lane + mid] == KEY_NONE:
                    r = mid - 1
                else:
                    l = mid
            if key > self.keys[idx][lane + l]:
                idx += 1
                lane = (lane << 1) + self.seg
            else:
                break
        return GET_LINEAR_IDX(idx, lane, self.H)

    def slot(self, L):
        i = GET_IDX(L, self.H)
        return i, GET_LANE(L, i, self.H)

    def compact(self, start, width, thres=0):
        ks, vs = [], []
        for L in range(start, start + width):
            i, ln = self.slot(L)
            k = self.keys[i][ln]
            if not (k == KEY_NONE or (k & TIME_MASK) < thres):
                ks.append(k)
                vs.append(self.vals[i][ln])
        return ks, vs

    # block_redispatch_merge_kernel / redispatch_kernel, rpma.cuh:661-695, 954-984
    def redispatch(self, mk, mv, start, width):
        frac, deno = width // self.seg, len(mk)
        for L in range(start, start + width):
            i, ln = self.slot(L)
            self.keys[i][ln] = KEY_NONE
        for t in range(deno):
            seg_idx = (frac * t) // deno
            seg_lane = ((frac * t) % deno) // frac
            L = seg_idx * self.seg + seg_lane + start
            i, ln = self.slot(L)
            self.keys[i][ln] = mk[t]
            self.vals[i][ln] = mv[t]
            if (mk[t] & DST_AND_TIME_MASK) == DST_AND_TIME_END:
                row = mk[t] >> SRC_SHIFT
                self.csr_idx[row + 1] = i
                self.csr_lane[row + 1] = ln

    # alloc_or_del_levels, rpma.cuh:1396-1415
    def alloc_or_del(self, h):
        for i in range(self.H + 1, h + 1):
            self.keys.append([KEY_NONE] * (self.seg << i))
            self.vals.append([0] * (self.seg << i))
        del self.keys[h + 1:]
        del self.vals[h + 1:]
        self.H = h

    def count_items(self, thres=0):
        n = 0
        for i in range(self.H + 1):
            n += sum(1 for k in self.keys[i] if k != KEY_NONE and (k & TIME_MASK) >= thres)
        return n

    # resize_rpma, rpma.cuh:1301-1354
    def resize(self, update_size, reach_root):
        merge = self.count_items() + update_size
        h = 0
        while self.seg * ((2 << h) - 1) < merge:
            h += 1
        if reach_root:
            h += 1
        return h

    # one level loop, rpma.cuh:1611-1657 (first) and 1686-1703 (second)
    def level_loop(self, upd, use_skip, eager):
        skip = False
        level = 0
        while level <= self.H + 1 and upd:
            H = self.H
            if use_skip:
                if level == 4 or level == H // 3:
                    skip = True
                if level == ((H // 3 - 1) & M32) or level == H + 1:
                    skip = False
            width = self.seg << level
            lower, upper = self.lower[level], self.upper[level]
            applied = [False] * len(upd)
            i = 0
            while i < len(upd):
                node = upd[i][0]
                j = i
                while j < len(upd) and upd[j][0] == node:
                    j += 1
                ww, up, ok = width, upper, True
                if node + ww >= (self.seg << (H + 1)):
                    ww -= self.seg
                    up -= self.seg
                    if ww == 0:
                        ok = False
                if ok and width > 1024 and skip:
                    ok = False
                if ok:
                    ak, av = self.compact(node, ww)
                    m = len(ak) + (j - i)
                    if lower <= m <= up:
                        # mergesmallk: stable merge, ties take the stored key
                        bk = [upd[t][1] for t in range(i, j)]
                        bv = [upd[t][2] for t in range(i, j)]
                        mk, mv, x, y = [], [], 0, 0
                        while x < len(ak) or y < len(bk):
                            if y >= len(bk) or (x < len(ak) and ak[x] <= bk[y]):
                                mk.append(ak[x])
                                mv.append(av[x])
                                x += 1
                            else:
                                mk.append(bk[y])
                                mv.append(bv[y])
                                y += 1
                        self.redispatch(mk, mv, node, ww)
                        for t in range(i, j):
                            applied[t] = True
                i = j
            upd = [(u[0] & ~(32 << level), u[1], u[2]) for t, u in enumerate(upd) if not applied[t]]
            if eager and level == H + 1 and not upd:
                self.alloc_or_del(self.resize(0, True))
            level += 1
        return upd

    # rebuild_rpma, rpma.cuh:1417-1472
    def rebuild(self, h, upd):
        ak, av = self.compact(0, self.seg * ((2 << self.H) - 1))
        pairs = sorted(zip(ak + [u[1] for u in upd], av + [u[2] for u in upd]), key=lambda p: p[0])
        self.alloc_or_del(h)
        n = self.seg * ((2 << h) - 1)
        for i in range(h + 1):
            self.keys[i] = [KEY_NONE] * (self.seg << i)
        self.redispatch([p[0] for p in pairs], [p[1] for p in pairs], 0, n)

    # fill_empty_segs, rpma.cuh:1474-1530
    def fill_empty(self):
        lv = self.keys[self.H - 1]
        empty = any(all(lv[s * 32 + t] == KEY_NONE for t in range(32)) for s in range(len(lv) // 32))
        if empty:
            n = self.seg * ((2 << self.H) - 1)
            ak, av = self.compact(0, n)
            self.redispatch(ak, av, 0, n)

    # update_rpma, rpma.cuh:1549-1718 (thres = 0, no edge queries)
    def update(self, keys, vals):
        pairs = sorted(zip(keys, vals), key=lambda p: p[0])
        upd = [(self.locate(k), k, v) for k, v in pairs]
        upd = self.level_loop(upd, True, True)
        if upd:
            orig = self.H
            h = self.resize(len(upd), False)
            if h < orig or h - orig > 1:
                self.rebuild(h, upd)
            elif h - orig == 1:
                self.alloc_or_del(h)
                upd = [(self.locate(u[1]), u[1], u[2]) for u in upd]
                upd = self.level_loop(upd, False, False)
                assert not upd
                if self.H > 0:
                    self.fill_empty()
            else:
                raise AssertionError("reference asserts here (rpma.cuh:1710)")

    def layout(self):
        ks, vs = [], []
        for i in range(self.H + 1):
            ks.extend(self.keys[i])
            vs.extend(0 if k == KEY_NONE else v for k, v in zip(self.keys[i], self.vals[i]))
        return ks, vs

    def sentinel_slots(self):
        out = []
        for v in range(self.row_num):
            i, ln = self.csr_idx[v + 1], self.csr_lane[v + 1]
            out.append(32 * ((1 << i) - 1) + ln)
        return out


def digest(keys, vals):
    h = hashlib.sha256()
    h.update(b"".join(int(k).to_bytes(8, "little") for k in keys))
    h.update(bytes(vals))
    return h.hexdigest()


# ----------------------------------------------------------------- streams
def mix64(z):
    z = (z + 0x9E3779B97F4A7C15) & ((1 << 64) - 1)
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & ((1 << 64) - 1)
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & ((1 << 64) - 1)
    return z ^ (z >> 31)


def small_stream(seed, V, n_edges):
    """Distinct non-loop edges, seeded: src, dst uniform below V."""
    seen, out, c = set(), [], 0
    while len(out) < n_edges:
        r = mix64(seed * 1000003 + c)
        c += 1
        s, d = (r >> 32) % V, (r & 0xFFFFFFFF) % V
        k = (s << 42) | (d << 20)
        if s != d and k not in seen:
            seen.add(k)
            out.append(k)
    return out


STREAMS = [
    # (seed, vertices, edges, batch sizes in order)
    (1, 64, 400, [200, 30, 30, 50, 90]),
    (2, 100, 700, [350, 100, 100, 150]),
    (3, 200, 1500, [64] * 8 + [900]),
    (4, 53, 300, [13, 13, 40, 100, 134]),
    (5, 300, 2400, [1200, 400, 400, 400]),
]


def streams_fixture():
    out = []
    for seed, V, n, batches in STREAMS:
        edges = small_stream(seed, V, n)
        p = RefRPMA(V)
        snaps = []
        k, v = p.layout()
        snaps.append({"after": "create", "height": p.H, "sha256": digest(k, v),
                      "sentinel_sha256": hashlib.sha256(str(p.sentinel_slots()).encode()).hexdigest()})
        pos = 0
        for b in batches:
            keys = edges[pos:pos + b]
            pos += b
            p.update(keys, [1] * len(keys))
            k, v = p.layout()
            snaps.append({"after": "insert %d" % b, "height": p.H, "sha256": digest(k, v),
                          "sentinel_sha256": hashlib.sha256(str(p.sentinel_slots()).encode()).hexdigest()})
        k, v = p.layout()
        out.append({"seed": seed, "vertices": V, "edges": [str(e) for e in edges], "batches": batches,
                    "snapshots": snaps, "final_keys": [str(x) for x in k], "final_vals": v,
                    "final_sentinel_slots": p.sentinel_slots()})
    return out


def check_macros_against_reference_text(reference_dir):
    """The restated macros are those of the reference header, verbatim in form."""
    if not reference_dir:
        return
    path = os.path.join(reference_dir, "rpma.cuh")
    if not os.path.exists(path):
        return
    src = open(path).read()
    for name in ("GET_IDX", "GET_LANE", "GET_LINEAR_IDX"):
        assert re.search(r"#define\s+%s\(" % name, src), name


def main(argv):
    import argparse
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--reference", default=os.environ.get("LPMA_REFERENCE_DIR"),
                    help="checkout of the reference, for the macro self-check (optional)")
    args = ap.parse_args(argv)
    check_macros_against_reference_text(args.reference)
    # cross-check of this restatement against the fixtures that the
    # reference's own code produced (tests/golden/make_ref_golden.py)
    with open(os.path.join(HERE, "index_algebra.json")) as f:
        for block in json.load(f)["blocks"]:
            H = block["height"]
            for lin, idx, lane, back in block["rows"]:
                assert GET_IDX(lin, H) == idx and GET_LANE(lin, idx, H) == lane
    with open(os.path.join(HERE, "tables.json")) as f:
        t = json.load(f)
    lower, upper = density_tables(26)
    assert lower == t["lower"] and upper == t["upper"]
    assert all(skip_table(int(H)) == v for H, v in t["skip"].items())
    with open(os.path.join(HERE, "small_streams.json"), "w") as f:
        json.dump(streams_fixture(), f, separators=(",", ":"))
    print("small_streams.json written to", HERE)


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
