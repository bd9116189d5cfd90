"""Host-side mirror of the reference's LPMA interface over the C ABI.

Names follow rpma.cuh: ``init_csr_rpma`` (rpma.cuh:1808), ``update_rpma``
(rpma.cuh:1549), ``to_csr_rpma`` (rpma.cuh:2250), ``get_data_rpma``
(rpma.cuh:1735), ``destroy_rpma`` (rpma.cuh:1720).  Inputs may be torch CUDA
tensors (device path, ``lpma_update``) or numpy arrays (host path,
``lpma_update_host``).  Every call goes to the CUDA library; there is no CPU
implementation behind this module.
"""
import ctypes

import numpy as np

from . import _abi
from ._abi import LpmaConfig, LpmaError, LpmaStats, check

SRC_SHIFT = 42
DST_SHIFT = 20
DST_AND_TIME_END = 0x000003FFFFEFFFFF
NBR_END = 0x3FFFFE
KEY_NONE = (1 << 64) - 1


def pack_key(src, dst, t=0):
    """src << 42 | dst << 20 | t (rpma.cuh:43-50, test_update_rpma.cu:189)."""
    return (int(src) << SRC_SHIFT) | (int(dst) << DST_SHIFT) | int(t)


def sentinel_key(v):
    return (int(v) << SRC_SHIFT) + DST_AND_TIME_END


def default_config(**kw):
    cfg = LpmaConfig()
    check(_abi.load().lpma_config_default(ctypes.byref(cfg)), "lpma_config_default")
    for k, v in kw.items():
        setattr(cfg, k, v)
    return cfg


def gpma_config(**kw):
    """The configuration of a GPMA-mode handle (gpma.cuh's flat array): flags
    LPMA_FLAG_GPMA, density 0.15 / 1.0, keys src << 32 | dst."""
    cfg = LpmaConfig()
    check(_abi.load().lpma_config_gpma(ctypes.byref(cfg)), "lpma_config_gpma")
    for k, v in kw.items():
        setattr(cfg, k, v)
    return cfg


def gpma_key(src, dst):
    """src << 32 | dst, the GPMA key layout (gpma.cuh)."""
    return (int(src) << 32) | int(dst)


_torch = None
_raw_stream = None


def _stream_ptr(stream):
    global _torch, _raw_stream
    if stream is None:
        if _torch is None:
            try:
                import torch
                _torch = torch if torch.cuda.is_available() else False
            except ImportError:
                _torch = False
            if _torch:
                # the current stream's handle without building a Stream object
                # (a few microseconds a call, which a 1K-edge update notices)
                get_raw = getattr(_torch._C, "_cuda_getCurrentRawStream", None)
                get_dev = getattr(_torch._C, "_cuda_getDevice", None)
                if get_raw is not None and get_dev is not None:
                    _raw_stream = lambda: get_raw(get_dev())  # noqa: E731
        if _raw_stream is not None:
            return _raw_stream()
        if _torch:
            return _torch.cuda.current_stream().cuda_stream
        return None
    if isinstance(stream, int):
        return ctypes.c_void_p(stream)
    return ctypes.c_void_p(stream.cuda_stream)


def _is_cuda_tensor(x):
    return hasattr(x, "is_cuda") and x.is_cuda


_SAME_BITS = {"uint64": ("torch.uint64", "torch.int64"), "uint8": ("torch.uint8", "torch.int8")}
_OK_DTYPES = {}


def _dev(x, dtype_name):
    if x is None:
        return None, 0
    ok = _OK_DTYPES.get((x.dtype, dtype_name))
    if ok is None:
        ok = _OK_DTYPES[(x.dtype, dtype_name)] = str(x.dtype) in _SAME_BITS[dtype_name]
    if not ok:
        raise TypeError("expected a torch.%s tensor, got %s" % (dtype_name, x.dtype))
    if not x.is_contiguous():
        raise ValueError("device inputs must be contiguous")
    return x.data_ptr(), x.numel()


def _host(x, dtype):
    if x is None:
        return None, None, 0
    a = np.ascontiguousarray(x, dtype=dtype)
    return a, a.ctypes.data_as(ctypes.c_void_p), a.size


class Lpma:
    """One dynamic graph held as a leveled PMA on the current CUDA device."""

    def __init__(self, num_vertices, config=None, stream=None):
        self._L = _abi.load()
        self.num_vertices = int(num_vertices)
        self.stream = stream
        h = ctypes.c_void_p()
        cfg = config if config is not None else default_config()
        check(self._L.lpma_create(ctypes.byref(cfg), self.num_vertices, _stream_ptr(stream), ctypes.byref(h)),
              "lpma_create")
        self._h = h
        self.gpma = bool(cfg.flags & 2)

    # -------------------------------------------------------------- updates
    def build(self, keys, values=None):
        """Bulk load (one update of all edges)."""
        return self.update(ins=keys, ins_vals=values)

    def update(self, ins=None, ins_vals=None, dels=None, thres=0):
        """update_rpma with deletes; returns the call's LpmaStats (indexable like a dict)."""
        st = LpmaStats()
        sp = _stream_ptr(self.stream)
        if _is_cuda_tensor(ins) or _is_cuda_tensor(dels):
            pi, ni = _dev(ins, "uint64") if ins is not None else (None, 0)
            pv, _ = _dev(ins_vals, "uint8") if ins_vals is not None else (None, 0)
            pd, nd = _dev(dels, "uint64") if dels is not None else (None, 0)
            rc = self._L.lpma_update(self._h, pi, pv, ni, pd, nd, thres, sp, ctypes.byref(st))
        else:
            ai, pi, ni = _host(ins, np.uint64)
            av, pv, _ = _host(ins_vals, np.uint8)
            ad, pd, nd = _host(dels, np.uint64)
            rc = self._L.lpma_update_host(self._h, pi, pv, ni, pd, nd, int(thres), sp, ctypes.byref(st))
            del ai, av, ad
        check(rc, "lpma_update")
        return st

    # -------------------------------------------------------------- views
    def info(self):
        H, n, V = ctypes.c_uint32(), ctypes.c_uint64(), ctypes.c_uint32()
        check(self._L.lpma_info(self._h, ctypes.byref(H), ctypes.byref(n), ctypes.byref(V)), "lpma_info")
        return {"height": H.value, "num_items": n.value, "num_vertices": V.value}

    @property
    def height(self):
        return self.info()["height"]

    @property
    def num_items(self):
        return self.info()["num_items"]

    def csr_view(self):
        """Device pointers (row_offset, col_index, values) and nnz, owned by the handle."""
        ro, ci, va, nnz = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_size_t()
        check(self._L.lpma_csr_view(self._h, ctypes.byref(ro), ctypes.byref(ci), ctypes.byref(va),
                                    ctypes.byref(nnz), _stream_ptr(self.stream)), "lpma_csr_view")
        return ro.value, ci.value, va.value, nnz.value

    def to_csr(self):
        """to_csr_rpma: numpy (row_offset, col_index, values)."""
        n = self.num_items
        ro = np.empty(self.num_vertices + 1, np.uint32)
        ci = np.empty(max(n, 1), np.uint32)
        va = np.empty(max(n, 1), np.uint8)
        nnz = ctypes.c_size_t()
        check(self._L.lpma_to_csr(self._h, ro.ctypes.data_as(ctypes.c_void_p), ci.ctypes.data_as(ctypes.c_void_p),
                                  va.ctypes.data_as(ctypes.c_void_p), ci.size, ctypes.byref(nnz),
                                  _stream_ptr(self.stream)), "lpma_to_csr")
        return ro, ci[:nnz.value], va[:nnz.value]

    def export_sorted(self):
        """get_data_rpma: numpy (keys, values) in sorted order."""
        n = self.num_items
        k = np.empty(max(n, 1), np.uint64)
        v = np.empty(max(n, 1), np.uint8)
        got = ctypes.c_size_t()
        check(self._L.lpma_export_sorted(self._h, k.ctypes.data_as(ctypes.c_void_p),
                                         v.ctypes.data_as(ctypes.c_void_p), k.size, ctypes.byref(got),
                                         _stream_ptr(self.stream)), "lpma_export_sorted")
        return k[:got.value], v[:got.value]

    def gpma_view(self):
        """GPMA handles: device pointers (row_offset, keys, values) and the
        geometry (size, segment_length, height)."""
        ro, k, v = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        size, seg, h = ctypes.c_uint64(), ctypes.c_uint32(), ctypes.c_uint32()
        check(self._L.lpma_gpma_view(self._h, ctypes.byref(ro), ctypes.byref(k), ctypes.byref(v), ctypes.byref(size),
                                     ctypes.byref(seg), ctypes.byref(h)), "lpma_gpma_view")
        return (ro.value, k.value, v.value), (size.value, seg.value, h.value)

    def layout(self):
        """(keys, values, sentinel_slots, height) of the physical layout: the
        heap-order level arrays, or for a GPMA handle the flat array."""
        H = self.height
        ns = self.gpma_view()[1][0] if self.gpma else 32 * ((2 << H) - 1)
        k = np.empty(ns, np.uint64)
        v = np.empty(ns, np.uint8)
        sent = np.empty(self.num_vertices, np.uint32)
        h = ctypes.c_uint32()
        check(self._L.lpma_export_layout(self._h, k.ctypes.data_as(ctypes.c_void_p), v.ctypes.data_as(ctypes.c_void_p),
                                         ns, sent.ctypes.data_as(ctypes.c_void_p), sent.size, ctypes.byref(h),
                                         _stream_ptr(self.stream)), "lpma_export_layout")
        return k, v, sent, h.value

    def set_flags(self, flags):
        """LPMA_FLAG_* bits (1: calls may run concurrently with other handles')."""
        check(self._L.lpma_set_flags(self._h, int(flags)), "lpma_set_flags")

    # -------------------------------------------------------------- read paths
    def query_neighbors(self, srcs, windows=None):
        """query_rpma: neighbour lists of srcs (torch CUDA uint32/int32) with time
        windows (torch CUDA int64, lb << 32 | ub; default every timestamp).
        Returns torch tensors (offsets [n+1] int32, nbrs int32, values uint8)."""
        import torch
        n = srcs.numel()
        dev = srcs.device
        srcs = srcs.to(torch.int32).contiguous()
        if windows is None:
            windows = torch.full((n,), 0xFFFFFFFF, dtype=torch.int64, device=dev)
        windows = windows.to(torch.int64).contiguous()
        offsets = torch.empty(n + 1, dtype=torch.int32, device=dev)
        total = ctypes.c_size_t()
        sp = _stream_ptr(self.stream)
        check(self._L.lpma_query_neighbors(self._h, srcs.data_ptr(), windows.data_ptr(), n, offsets.data_ptr(), None,
                                           None, 0, ctypes.byref(total), sp), "lpma_query_neighbors")
        nbrs = torch.empty(max(total.value, 1), dtype=torch.int32, device=dev)
        vals = torch.empty(max(total.value, 1), dtype=torch.uint8, device=dev)
        check(self._L.lpma_query_neighbors(self._h, srcs.data_ptr(), windows.data_ptr(), n, offsets.data_ptr(),
                                           nbrs.data_ptr(), vals.data_ptr(), nbrs.numel(), ctypes.byref(total), sp),
              "lpma_query_neighbors")
        return offsets, nbrs[:total.value], vals[:total.value]

    def edge_query(self, keys, window=0xFFFFF):
        """Count of stored keys (src, dst, t') with t - window <= t' <= t per query key (torch CUDA int64)."""
        import torch
        keys = keys.to(torch.int64).contiguous()
        res = torch.empty(keys.numel(), dtype=torch.int32, device=keys.device)
        check(self._L.lpma_edge_query(self._h, keys.data_ptr(), keys.numel(), int(window), res.data_ptr(),
                                      _stream_ptr(self.stream)), "lpma_edge_query")
        return res

    def bfs(self, sources, max_depth=0):
        """Directed BFS hop counts (torch int32 [V], INT32_MAX when unreached), levels, vertices reached."""
        import torch
        sources = sources.to(torch.int32).contiguous()
        dist = torch.empty(self.num_vertices, dtype=torch.int32, device=sources.device)
        lv, reached = ctypes.c_uint32(), ctypes.c_uint64()
        check(self._L.lpma_bfs(self._h, sources.data_ptr(), sources.numel(), int(max_depth), dist.data_ptr(),
                               ctypes.byref(lv), ctypes.byref(reached), _stream_ptr(self.stream)), "lpma_bfs")
        return dist, lv.value, reached.value

    def pagerank(self, alpha=0.85, iterations=20, device="cuda"):
        """PageRank ranks (torch float64 [V]) after `iterations` power iterations."""
        import torch
        rank = torch.empty(self.num_vertices, dtype=torch.float64, device=device)
        check(self._L.lpma_pagerank(self._h, float(alpha), int(iterations), rank.data_ptr(), _stream_ptr(self.stream)),
              "lpma_pagerank")
        return rank

    def close(self):
        if getattr(self, "_h", None):
            self._L.lpma_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------ reference-named API
def init_csr_rpma(row_num, config=None, stream=None):
    return Lpma(row_num, config=config, stream=stream)


def update_rpma(rpma, keys, values=None, thres=0, del_keys=None):
    """update_rpma (rpma.cuh:1549-1718): returns the reference's bool, true
    when the updates reached the root level (absorbed there or overflowed)."""
    return bool(rpma.update(ins=keys, ins_vals=values, dels=del_keys, thres=thres)["levelup"])


def to_csr_rpma(rpma):
    ro, ci, _ = rpma.to_csr()
    return ro, ci


def get_data_rpma(rpma):
    return rpma.export_sorted()


def destroy_rpma(rpma):
    rpma.close()


# ------------------------------------------------------ workload generator
class Pool:
    """Worker pool over many resident graphs (lpma_pool_*): submit update,
    neighbour, BFS and edge-query requests; different graphs run
    concurrently, one graph's requests run in submission order.  Inputs and
    outputs are torch CUDA tensors, kept alive by the request until done."""

    def __init__(self, workers=8, hbm_budget_bytes=0):
        self._L = _abi.load()
        p = ctypes.c_void_p()
        check(self._L.lpma_pool_create(int(workers), int(hbm_budget_bytes), ctypes.byref(p)), "lpma_pool_create")
        self._p = p

    def _submit(self, req, keep):
        req._keep = keep
        check(self._L.lpma_pool_submit(self._p, ctypes.byref(req)), "lpma_pool_submit")
        return req

    def update(self, graph, ins=None, dels=None, ins_vals=None, thres=0):
        r = _abi.LpmaRequest()
        r.kind, r.graph, r.thres = _abi.REQ_UPDATE, graph._h, int(thres)
        if ins is not None:
            r.keys0, r.n0 = _dev(ins, "uint64")
        if ins_vals is not None:
            r.vals0 = _dev(ins_vals, "uint8")[0]
        if dels is not None:
            r.keys1, r.n1 = _dev(dels, "uint64")
        return self._submit(r, (ins, dels, ins_vals))

    def neighbors(self, graph, srcs, windows, offsets, nbrs, vals):
        r = _abi.LpmaRequest()
        r.kind, r.graph = _abi.REQ_NEIGHBORS, graph._h
        r.vertices, r.windows, r.nv = srcs.data_ptr(), windows.data_ptr(), srcs.numel()
        r.out_u32, r.out_nbrs, r.out_vals, r.cap = offsets.data_ptr(), nbrs.data_ptr(), vals.data_ptr(), nbrs.numel()
        return self._submit(r, (srcs, windows, offsets, nbrs, vals))

    def bfs(self, graph, sources, dist, max_depth=0):
        r = _abi.LpmaRequest()
        r.kind, r.graph, r.max_depth = _abi.REQ_BFS, graph._h, int(max_depth)
        r.vertices, r.nv, r.out_dist = sources.data_ptr(), sources.numel(), dist.data_ptr()
        return self._submit(r, (sources, dist))

    def update_many(self, graphs, batches, kinds):
        """One update request per (graph, device batch, "ins" | "del"),
        submitted in one call; returns the request array (keep it alive
        until drained)."""
        n = len(graphs)
        reqs = (_abi.LpmaRequest * n)()
        for i, (g, x, k) in enumerate(zip(graphs, batches, kinds)):
            r = reqs[i]
            r.kind, r.graph = _abi.REQ_UPDATE, g._h
            ptr, cnt = x.data_ptr(), x.numel()
            if k == "ins":
                r.keys0, r.n0 = ptr, cnt
            else:
                r.keys1, r.n1 = ptr, cnt
        reqs._keep = batches
        check(self._L.lpma_pool_submit_many(self._p, reqs, n), "lpma_pool_submit_many")
        return reqs

    def wait(self, req):
        return self._L.lpma_pool_wait(self._p, ctypes.byref(req))

    def drain(self):
        check(self._L.lpma_pool_drain(self._p), "lpma_pool_drain")

    def close(self):
        if getattr(self, "_p", None):
            self._L.lpma_pool_destroy(self._p)
            self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batcher:
    """Updates of many graphs in one call (lpma_update_batch): the update
    fronts of all graphs share their launches, then each graph runs its own
    executors.  Each graph appears at most once per call; batches are torch
    CUDA tensors."""

    def __init__(self):
        self._L = _abi.load()
        b = ctypes.c_void_p()
        check(self._L.lpma_batcher_create(ctypes.byref(b)), "lpma_batcher_create")
        self._b = b

    def update(self, graphs, batches, stream=None, raise_on_error=True):
        """graphs: Lpma objects; batches: per graph a dict with any of ins,
        ins_vals, dels, thres (or an (ins, dels) pair).  Returns (stats,
        statuses), one entry per graph."""
        n = len(graphs)
        items = (_abi.LpmaBatch * n)()
        hs = (ctypes.c_void_p * n)()
        keep = []
        for i, (g, b) in enumerate(zip(graphs, batches)):
            if not isinstance(b, dict):
                b = {"ins": b[0], "dels": b[1]}
            hs[i] = g._h.value
            it = items[i]
            if b.get("ins") is not None:
                it.ins, it.n_ins = _dev(b["ins"], "uint64")
            if b.get("ins_vals") is not None:
                it.ins_vals = _dev(b["ins_vals"], "uint8")[0]
            if b.get("dels") is not None:
                it.dels, it.n_del = _dev(b["dels"], "uint64")
            it.thres = int(b.get("thres", 0))
            keep.append(b)
        stats = (LpmaStats * n)()
        status = (ctypes.c_int * n)()
        rc = self._L.lpma_update_batch(self._b, hs, items, n, _stream_ptr(stream), stats, status)
        if raise_on_error:
            check(rc, "lpma_update_batch")
        return list(stats), list(status)

    def close(self):
        if getattr(self, "_b", None):
            self._L.lpma_batcher_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune(max_keys=1 << 20, stream=None):
    """Time every usable batch-sort tier per batch-size bucket and keep the
    fastest (lpma_autotune).  Returns one dict per (bucket, sort mode)."""
    L = _abi.load()
    cap = 2 * 32
    ents = (_abi.LpmaTuneEntry * cap)()
    n = ctypes.c_size_t()
    check(L.lpma_autotune(int(max_keys), _stream_ptr(stream), ents, cap, ctypes.byref(n)), "lpma_autotune")
    out = []
    for e in ents[:n.value]:
        out.append({"keys": 1 << e.log2_keys, "concurrent": bool(e.concurrent),
                    "tier": _abi.SORT_TIERS.get(e.tier, e.tier),
                    "us": {_abi.SORT_TIERS[t]: round(e.us[t], 1) for t in _abi.SORT_TIERS if e.us[t] > 0}})
    return out


def tune_set(log2_keys, tier, concurrent=False):
    """Override one autotuner entry (tier name or number; 0 / None = built-in cutovers)."""
    if isinstance(tier, str):
        tier = {v: k for k, v in _abi.SORT_TIERS.items()}[tier]
    check(_abi.load().lpma_tune_set(int(log2_keys), 1 if concurrent else 0, int(tier or 0)), "lpma_tune_set")


def grain_set(log2_keys, max_segs_group=0, max_segs_shared=0):
    """Executor cut-overs of one batch-size bucket (0, 0: the defaults 4 and 32)."""
    check(_abi.load().lpma_grain_set(int(log2_keys), int(max_segs_group), int(max_segs_shared)), "lpma_grain_set")


def grain_get(log2_keys):
    g, sh = ctypes.c_uint32(), ctypes.c_uint32()
    check(_abi.load().lpma_grain_get(int(log2_keys), ctypes.byref(g), ctypes.byref(sh)), "lpma_grain_get")
    return g.value, sh.value


def autotune_grain(g, keys, reps=3):
    """lpma_autotune_grain on handle g with a device batch of absent keys;
    returns one dict per setting timed (the fastest is kept for the batch's
    bucket)."""
    cap = 8
    out = (_abi.LpmaGrainTime * cap)()
    n = ctypes.c_size_t()
    p, nk = _dev(keys, "uint64")
    check(_abi.load().lpma_autotune_grain(g._h, p, nk, int(reps), _stream_ptr(g.stream), out, cap, ctypes.byref(n)),
          "lpma_autotune_grain")
    return [{"max_segs_group": e.max_segs_group, "max_segs_shared": e.max_segs_shared,
             "us": round(e.us_median, 1)} for e in out[:n.value]]


def memory_bytes(g):
    b = ctypes.c_uint64()
    check(_abi.load().lpma_memory_bytes(g._h, ctypes.byref(b)), "lpma_memory_bytes")
    return b.value


def memory_reserve(nbytes, stream=None):
    """Grow the update memory pool by nbytes (lpma_memory_reserve), so that
    graphs growing under load do not map new device memory then."""
    check(_abi.load().lpma_memory_reserve(int(nbytes), _stream_ptr(stream)), "lpma_memory_reserve")


def query_rpma(rpma, srcs, constraints=None):
    """query_rpma (rpma.cuh:1974-2036): (offsets, nbrs, values), lists in the callers' query order."""
    return rpma.query_neighbors(srcs, constraints)


def edge_query_rpma(rpma, keys, window=0xFFFFF):
    """Edge query (rpma.cuh:2040-2066, result check test.cu:46-62)."""
    return rpma.edge_query(keys, window)


def read_edgelist(path, timestamps_path=None):
    """read_edgelist / read_edgelist_and_timestamps: (numpy uint64 keys, num_vertices)."""
    L = _abi.load()
    V, E = ctypes.c_uint32(), ctypes.c_size_t()
    tp = timestamps_path.encode() if timestamps_path else None
    rc = L.lpma_read_edgelist(path.encode(), tp, None, 0, ctypes.byref(V), ctypes.byref(E))
    if rc not in (0, 8):
        check(rc, "lpma_read_edgelist")
    keys = np.empty(max(E.value, 1), np.uint64)
    check(L.lpma_read_edgelist(path.encode(), tp, keys.ctypes.data_as(ctypes.c_void_p), keys.size, ctypes.byref(V),
                               ctypes.byref(E)), "lpma_read_edgelist")
    return keys[:E.value], V.value


def read_queries(path):
    """read_queries: (numpy uint32 srcs, numpy uint64 windows lb << 32 | ub)."""
    L = _abi.load()
    Q = ctypes.c_size_t()
    rc = L.lpma_read_queries(path.encode(), None, None, 0, ctypes.byref(Q))
    if rc not in (0, 8):
        check(rc, "lpma_read_queries")
    srcs = np.empty(max(Q.value, 1), np.uint32)
    wins = np.empty(max(Q.value, 1), np.uint64)
    check(L.lpma_read_queries(path.encode(), srcs.ctypes.data_as(ctypes.c_void_p), wins.ctypes.data_as(ctypes.c_void_p),
                              srcs.size, ctypes.byref(Q)), "lpma_read_queries")
    return srcs[:Q.value], wins[:Q.value]


def rmat_thresholds(a=0.57, b=0.19, c=0.19):
    """Integer quadrant thresholds floor(p * 2^32) (IEEE double)."""
    return int(a * 4294967296.0), int((a + b) * 4294967296.0), int((a + b + c) * 4294967296.0)


def gen_rmat_device(seed, scale, edge_factor, out, a=0.57, b=0.19, c=0.19, stream=None):
    """R-MAT keys on the device into the torch uint64 tensor `out`; returns the deduplicated count."""
    L = _abi.load()
    ta, tab, tabc = rmat_thresholds(a, b, c)
    n = ctypes.c_size_t()
    check(L.lpma_gen_rmat(seed, scale, edge_factor, ta, tab, tabc, ctypes.c_void_p(out.data_ptr()), out.numel(),
                          ctypes.byref(n), _stream_ptr(stream)), "lpma_gen_rmat")
    return n.value


def shuffle_device(seed, keys, stream=None):
    L = _abi.load()
    check(L.lpma_shuffle(seed, ctypes.c_void_p(keys.data_ptr()), keys.numel(), _stream_ptr(stream)), "lpma_shuffle")


def kernel_launches():
    return _abi.load().lpma_kernel_launches()


def profile_enable(on=True):
    _abi.load().lpma_prof_enable(1 if on else 0)


def profile_report():
    """{kernel name: (launches, total ms)} since the last report (synchronises)."""
    L = _abi.load()
    buf = ctypes.create_string_buffer(1 << 16)
    L.lpma_prof_report(buf, len(buf))
    out = {}
    for line in buf.value.decode().splitlines():
        name, cnt, ms = line.split()
        out[name] = (int(cnt), float(ms))
    return out


__all__ = ["Lpma", "LpmaError", "default_config", "init_csr_rpma", "update_rpma", "to_csr_rpma", "get_data_rpma",
           "destroy_rpma", "pack_key", "sentinel_key", "gen_rmat_device", "shuffle_device", "kernel_launches",
           "profile_enable", "profile_report"]
