"""ctypes binding of the CPU oracle (oracle/lpma_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of ``bench.py``.  The product package never
imports this module.

Parity status of the restatement: its single steps (index macros, density,
skip rule, resize height, locate, redistribution) are pinned to the
reference's own code compiled for the host (oracle/ref_host.py); whole-batch
layouts are "partially unpinned" (the reference's update loop does not build
under CUDA 13), pinned by the reference's result checks and a second
restatement (tests/golden).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liblpma_oracle.so")
SRC = os.path.join(HERE, "lpma_oracle.c")

KEY_NONE = (1 << 64) - 1
SRC_SHIFT = 42
DST_SHIFT = 20
DST_AND_TIME_END = 0x000003FFFFEFFFFF
NBR_END = 0x3FFFFE


def build(force=False):
    """Compile the oracle with gcc (plain C, pthreads)."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        subprocess.check_call(["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-o", LIB, SRC, "-lpthread"])
    return LIB


class OPmaStats(ctypes.Structure):
    _fields_ = [
        ("height_before", ctypes.c_uint32), ("height_after", ctypes.c_uint32),
        ("n_ins_applied", ctypes.c_uint32), ("n_upserts", ctypes.c_uint32),
        ("n_del_applied", ctypes.c_uint32), ("n_noop", ctypes.c_uint32),
        ("root_executed", ctypes.c_uint32), ("eager_levelup", ctypes.c_uint32),
        ("overflow", ctypes.c_uint32), ("rebuilt", ctypes.c_uint32),
        ("levelup_path", ctypes.c_uint32), ("fill_empty", ctypes.c_uint32),
        ("levelup", ctypes.c_uint32),
        ("win_count", ctypes.c_uint64 * 32), ("win_slots", ctypes.c_uint64 * 32),
    ]

    def as_dict(self):
        d = {f: getattr(self, f) for f, _ in self._fields_[:13]}
        d["win_count"] = list(self.win_count)
        d["win_slots"] = list(self.win_slots)
        return d


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        P, U32, U64, SZ, I = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_size_t, ctypes.c_int
        sig = {
            "opma_create": (P, [U32, I]),
            "opma_destroy": (None, [P]),
            "opma_update": (I, [P, P, P, SZ, P, SZ, U32, P]),
            "opma_height": (U32, [P]),
            "opma_num_slots": (U64, [P]),
            "opma_num_items": (U64, [P]),
            "opma_layout": (I, [P, P, P, SZ]),
            "opma_sentinel_slots": (I, [P, P, SZ]),
            "opma_export_sorted": (ctypes.c_int64, [P, P, P, SZ]),
            "opma_csr": (ctypes.c_int64, [P, P, P, P, SZ]),
            "opma_get_idx": (U32, [U32, U32]),
            "opma_get_lane": (U32, [U32, U32, U32]),
            "opma_get_linear_idx": (U32, [U32, U32, U32]),
            "opma_density_table": (None, [P, P, I]),
            "opma_skip_table": (None, [U32, P, I]),
            "opma_redistribute_counts": (None, [U64, U64, P]),
            "opma_locate_keys": (I, [P, P, SZ, P]),
            "opma_redistribute_window": (I, [U32, U32, U64, U64, P, P, U64, P, P, P]),
            "opma_resize_height": (U32, [U64, I]),
            "ogpma_create": (P, [U32, ctypes.c_double]),
            "ogpma_destroy": (None, [P]),
            "ogpma_update": (I, [P, P, P, SZ, P, SZ, P]),
            "ogpma_size": (U64, [P, P, P]),
            "ogpma_layout": (I, [P, P, P, SZ, P]),
            "ogpma_export_sorted": (ctypes.c_int64, [P, P, P, SZ]),
            "ogpma_size_rule": (None, [U64, P, P, P]),
            "ogpma_density": (None, [U32, U32, ctypes.c_double, P, P]),
            "ogpma_locate_keys": (I, [P, P, SZ, P]),
            "ogpma_resolve_only": (I, [P, P, P, SZ, P]),
            "ogpma_spread_window": (I, [U32, U32, U64, U64, P, P, U64, P, P, P]),
            "opma_mix64": (U64, [U64]),
            "opma_rmat_raw": (None, [U64, U32, U64, U32, U32, U32, P]),
            "opma_dedup": (U64, [P, U64]),
            "opma_shuffle": (None, [U64, P, U64]),
            "ocsr_create": (P, [U32, I]),
            "ocsr_destroy": (None, [P]),
            "ocsr_load": (I, [P, P, U64]),
            "ocsr_insert": (I, [P, P, U64]),
            "ocsr_delete": (I, [P, P, U64]),
            "ocsr_num_edges": (U64, [P]),
            "ocsr_edges": (P, [P]),
            "ocsr_row_offset": (P, [P]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


class OracleLpma:
    """The reference update path restated on the CPU (one instance = one graph)."""

    def __init__(self, num_vertices, skip_rule=True):
        self.V = int(num_vertices)
        self.h = lib().opma_create(self.V, 1 if skip_rule else 0)
        if not self.h:
            raise RuntimeError("opma_create failed (num_vertices=%d)" % self.V)

    def close(self):
        if self.h:
            lib().opma_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def update(self, ins=None, ins_vals=None, dels=None, thres=0):
        ins = np.ascontiguousarray(ins if ins is not None else np.zeros(0, np.uint64), dtype=np.uint64)
        dels = np.ascontiguousarray(dels if dels is not None else np.zeros(0, np.uint64), dtype=np.uint64)
        iv = None if ins_vals is None else np.ascontiguousarray(ins_vals, dtype=np.uint8)
        st = OPmaStats()
        rc = lib().opma_update(self.h, _ptr(ins), _ptr(iv), ins.size, _ptr(dels), dels.size, int(thres),
                               ctypes.byref(st))
        if rc != 0:
            raise ValueError("opma_update failed rc=%d" % rc)
        return st.as_dict()

    @property
    def height(self):
        return lib().opma_height(self.h)

    def num_slots(self):
        return lib().opma_num_slots(self.h)

    def num_items(self):
        return lib().opma_num_items(self.h)

    def layout(self):
        n = self.num_slots()
        k = np.empty(n, np.uint64)
        v = np.empty(n, np.uint8)
        assert lib().opma_layout(self.h, _ptr(k), _ptr(v), n) == 0
        return k, v

    def sentinel_slots(self):
        out = np.empty(self.V, np.uint32)
        assert lib().opma_sentinel_slots(self.h, _ptr(out), self.V) == 0
        return out

    def export_sorted(self):
        n = self.num_items()
        k = np.empty(n, np.uint64)
        v = np.empty(n, np.uint8)
        got = lib().opma_export_sorted(self.h, _ptr(k), _ptr(v), n)
        assert got == n
        return k, v

    def locate(self, keys):
        """Stop segment of each key (linear slot index of its first lane)."""
        keys = np.ascontiguousarray(keys, dtype=np.uint64)
        out = np.zeros(keys.size, np.uint32)
        assert lib().opma_locate_keys(self.h, _ptr(keys), keys.size, _ptr(out)) == 0
        return out

    def csr(self):
        n = self.num_items()
        ro = np.zeros(self.V + 1, np.uint32)
        ci = np.empty(n, np.uint32)
        vals = np.empty(n, np.uint8)
        got = lib().opma_csr(self.h, _ptr(ro), _ptr(ci), _ptr(vals), n)
        assert got == n
        return ro, ci, vals


GPMA_KEY_MAX = 0xFFFFFFFFFFFFFFFE
GPMA_DENSITY_LOWER = 0.15


def gpma_sentinel_key(v):
    return (int(v) << 32) | 0xFFFFFFFF


class OracleGpma:
    """update_gpma (gpma.cuh:747-816) restated on the CPU: one flat array,
    keys src << 32 | dst, deletes tombstone in place."""

    def __init__(self, num_vertices, density_lower=GPMA_DENSITY_LOWER):
        self.V = int(num_vertices)
        self.h = lib().ogpma_create(self.V, float(density_lower))
        if not self.h:
            raise RuntimeError("ogpma_create failed (num_vertices=%d)" % self.V)

    def close(self):
        if self.h:
            lib().ogpma_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def update(self, ins=None, ins_vals=None, dels=None):
        ins = np.ascontiguousarray(ins if ins is not None else np.zeros(0, np.uint64), dtype=np.uint64)
        dels = np.ascontiguousarray(dels if dels is not None else np.zeros(0, np.uint64), dtype=np.uint64)
        iv = None if ins_vals is None else np.ascontiguousarray(ins_vals, dtype=np.uint8)
        st = OPmaStats()
        rc = lib().ogpma_update(self.h, _ptr(ins), _ptr(iv), ins.size, _ptr(dels), dels.size, ctypes.byref(st))
        if rc != 0:
            raise ValueError("ogpma_update failed rc=%d" % rc)
        return st.as_dict()

    def geometry(self):
        seg, hh = ctypes.c_uint32(), ctypes.c_uint32()
        size = lib().ogpma_size(self.h, ctypes.byref(seg), ctypes.byref(hh))
        return size, seg.value, hh.value

    def layout(self):
        """(keys, values, row_offset) of the flat array; empty slots key ~0, value 0."""
        size, _, _ = self.geometry()
        k = np.empty(size, np.uint64)
        v = np.empty(size, np.uint8)
        ro = np.empty(self.V + 1, np.uint32)
        assert lib().ogpma_layout(self.h, _ptr(k), _ptr(v), size, _ptr(ro)) == 0
        return k, v, ro

    def export_sorted(self):
        size, _, _ = self.geometry()
        k = np.empty(size, np.uint64)
        v = np.empty(size, np.uint8)
        n = lib().ogpma_export_sorted(self.h, _ptr(k), _ptr(v), size)
        return k[:n].copy(), v[:n].copy()

    def locate(self, keys):
        keys = np.ascontiguousarray(keys, dtype=np.uint64)
        out = np.zeros(keys.size, np.uint32)
        assert lib().ogpma_locate_keys(self.h, _ptr(keys), keys.size, _ptr(out)) == 0
        return out

    def resolve_only(self, keys, vals):
        keys = np.ascontiguousarray(keys, dtype=np.uint64)
        vals = np.ascontiguousarray(vals, dtype=np.uint8)
        out = np.zeros(keys.size, np.uint32)
        assert lib().ogpma_resolve_only(self.h, _ptr(keys), _ptr(vals), keys.size, _ptr(out)) == 0
        return out


class CsrBaseline:
    """Sorted-merge CSR rebuild per batch on the host cores (the CPU baseline)."""

    def __init__(self, num_vertices, threads=1):
        self.V = int(num_vertices)
        self.h = lib().ocsr_create(self.V, int(threads))

    def close(self):
        if self.h:
            lib().ocsr_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def load(self, keys):
        keys = np.ascontiguousarray(keys, dtype=np.uint64)
        assert lib().ocsr_load(self.h, _ptr(keys), keys.size) == 0

    def insert(self, keys):
        keys = np.ascontiguousarray(keys, dtype=np.uint64)
        assert lib().ocsr_insert(self.h, _ptr(keys), keys.size) == 0

    def delete(self, keys):
        keys = np.ascontiguousarray(keys, dtype=np.uint64)
        assert lib().ocsr_delete(self.h, _ptr(keys), keys.size) == 0

    def edges(self):
        n = lib().ocsr_num_edges(self.h)
        p = lib().ocsr_edges(self.h)
        if n == 0:
            return np.zeros(0, np.uint64)
        return np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_uint64)), shape=(n,)).copy()

    def row_offset(self):
        p = lib().ocsr_row_offset(self.h)
        return np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_uint32)), shape=(self.V + 1,)).copy()


# ---------------------------------------------------------------- workloads
RMAT_A, RMAT_B, RMAT_C = 0.57, 0.19, 0.19


def rmat_thresholds(a=RMAT_A, b=RMAT_B, c=RMAT_C):
    """Integer quadrant thresholds: floor(p * 2^32) in IEEE double."""
    return int(a * 4294967296.0), int((a + b) * 4294967296.0), int((a + b + c) * 4294967296.0)


def rmat_edges(seed, scale, edge_factor, a=RMAT_A, b=RMAT_B, c=RMAT_C):
    """Seeded R-MAT keys (src<<42|dst<<20), self loops and duplicates removed, sorted."""
    n = (1 << scale) * edge_factor
    out = np.empty(n, np.uint64)
    ta, tab, tabc = rmat_thresholds(a, b, c)
    lib().opma_rmat_raw(seed, scale, n, ta, tab, tabc, _ptr(out))
    m = lib().opma_dedup(_ptr(out), n)
    return out[:m].copy()


def shuffle(keys, seed):
    keys = np.ascontiguousarray(keys, dtype=np.uint64).copy()
    lib().opma_shuffle(seed, _ptr(keys), keys.size)
    return keys


def sentinel_key(v):
    return (int(v) << SRC_SHIFT) + DST_AND_TIME_END


# ---------------------------------------------------------------- read paths
# Restatements of the reference's read paths over a sorted key set (the
# oracle's export_sorted()): what the device read kernels must return.

TIME_MASK = 0xFFFFF
NBR_END = 0x3FFFFE


def _split(keys):
    keys = np.asarray(keys, dtype=np.uint64)
    src = (keys >> np.uint64(SRC_SHIFT)).astype(np.int64)
    dst = ((keys >> np.uint64(20)) & np.uint64(0x3FFFFF)).astype(np.int64)
    t = (keys & np.uint64(TIME_MASK)).astype(np.int64)
    return src, dst, t


def neighbors(keys, vals, srcs, windows, V):
    """query_rpma (rpma.cuh:1827-2036) with the result check of test.cu:16-42:
    for query i, the dst of every key of srcs[i] with lb <= t <= ub
    (windows[i] = lb << 32 | ub), in key order; lists in query order."""
    keys = np.asarray(keys, dtype=np.uint64)
    vals = np.asarray(vals, dtype=np.uint8)
    src, dst, t = _split(keys)
    live = dst != NBR_END
    src, dst, t, vv = src[live], dst[live], t[live], vals[live]
    starts = np.searchsorted(src, np.arange(V + 1))
    offs, nb, nv = [0], [], []
    for s, w in zip(np.asarray(srcs, dtype=np.int64), np.asarray(windows, dtype=np.uint64)):
        lb, ub = int(w) >> 32, int(w) & 0xFFFFFFFF
        if s >= V:
            offs.append(offs[-1])
            continue
        a, b = starts[s], starts[s + 1]
        m = (t[a:b] >= lb) & (t[a:b] <= ub)
        nb.append(dst[a:b][m])
        nv.append(vv[a:b][m])
        offs.append(offs[-1] + int(m.sum()))
    cat = (lambda xs, dt: np.concatenate(xs).astype(dt) if xs else np.zeros(0, dt))
    return np.array(offs, np.int64), cat(nb, np.int64), cat(nv, np.uint8)


def edge_query_counts(keys, queries, window):
    """Edge query counts (test.cu:46-62): stored keys (src, dst, t') with
    t - window <= t' <= t for each query key (src, dst, t)."""
    keys = np.asarray(keys, dtype=np.uint64)
    q = np.asarray(queries, dtype=np.uint64)
    pre = q & ~np.uint64(TIME_MASK)
    t = (q & np.uint64(TIME_MASK)).astype(np.int64)
    lb = np.maximum(t - int(window), 0).astype(np.uint64)
    lo = np.searchsorted(keys, pre | lb, side="left")
    hi = np.searchsorted(keys, pre | t.astype(np.uint64), side="right")
    src, dst, _ = _split(q)
    return np.where(dst >= NBR_END, 0, hi - lo).astype(np.int64)


def bfs(keys, V, sources, max_depth=0):
    """Directed BFS hop counts from the sources over the stored edges
    (nvGRAPH BFS of test.cu:168-183 / test_algos.cu:136-186); 2^31-1 where
    unreached; at most max_depth levels (0: no bound)."""
    src, dst, _ = _split(keys)
    live = dst != NBR_END
    src, dst = src[live], dst[live]
    starts = np.searchsorted(src, np.arange(V + 1))
    INF = 2**31 - 1
    dist = np.full(V, INF, np.int64)
    front = np.unique(np.asarray([s for s in sources if s < V], dtype=np.int64))
    dist[front] = 0
    level = 0
    while front.size and (max_depth == 0 or level < max_depth):
        nxt = np.concatenate([dst[starts[u]:starts[u + 1]] for u in front]) if front.size else np.zeros(0, np.int64)
        nxt = np.unique(nxt)
        nxt = nxt[dist[nxt] == INF]
        dist[nxt] = level + 1
        front = nxt
        level += 1
    return dist


def pagerank(keys, V, alpha, iterations):
    """Power-iteration PageRank in float64 (test_algos.cu:44-90 runs nvGRAPH's):
    rank = (1-alpha)/V + alpha (sum over u->v of rank[u]/outdeg(u) + dangling/V)."""
    src, dst, _ = _split(keys)
    live = dst != NBR_END
    src, dst = src[live], dst[live]
    deg = np.bincount(src, minlength=V).astype(np.float64)
    rank = np.full(V, 1.0 / V)
    for _ in range(iterations):
        contrib = np.where(deg > 0, rank / np.maximum(deg, 1), 0.0)
        dangling = rank[deg == 0].sum()
        acc = np.bincount(dst, weights=contrib[src], minlength=V)
        rank = (1 - alpha) / V + alpha * (acc + dangling / V)
    return rank


def redistribute_window(H, V, node, width, items, item_vals, keys, vals, sent):
    """The oracle's even redistribution of sorted items over one window of
    a heap layout (keys / vals / sent are updated in place)."""
    items = np.ascontiguousarray(items, dtype=np.uint64)
    iv = np.ascontiguousarray(item_vals, dtype=np.uint8)
    rc = lib().opma_redistribute_window(H, V, node, width, _ptr(items), _ptr(iv), items.size, _ptr(keys), _ptr(vals),
                                        _ptr(sent))
    assert rc == 0


def gpma_size_rule(merge):
    size, seg, h = ctypes.c_uint64(), ctypes.c_uint32(), ctypes.c_uint32()
    lib().ogpma_size_rule(merge, ctypes.byref(size), ctypes.byref(seg), ctypes.byref(h))
    return size.value, seg.value, h.value


def gpma_density(seg, h, dlow=GPMA_DENSITY_LOWER):
    lo, up = np.zeros(h + 1, np.uint32), np.zeros(h + 1, np.uint32)
    lib().ogpma_density(seg, h, float(dlow), _ptr(lo), _ptr(up))
    return lo, up


def gpma_spread_window(V, seg, node, width, items, item_vals, keys, vals, row_offset):
    items = np.ascontiguousarray(items, dtype=np.uint64)
    iv = np.ascontiguousarray(item_vals, dtype=np.uint8)
    rc = lib().ogpma_spread_window(V, seg, node, width, _ptr(items), _ptr(iv), items.size, _ptr(keys), _ptr(vals),
                                   _ptr(row_offset))
    assert rc == 0
