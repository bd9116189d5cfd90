"""ctypes binding of the CPU oracle (oracle/lpma_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()``
and by the CPU-baseline leg of ``bench.py``.  The product package never
imports this module.

Parity status of the restatement: layout "parity unpinned" (the reference
does not build under CUDA 13); pinned by the reference's known-answer checks
held in tests/golden.
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
        ("win_count", ctypes.c_uint64 * 32), ("win_slots", ctypes.c_uint64 * 32),
    ]

    def as_dict(self):
        d = {f: getattr(self, f) for f, _ in self._fields_[:12]}
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

    def csr(self):
        n = self.num_items()
        ro = np.zeros(self.V + 1, np.uint32)
        ci = np.empty(n, np.uint32)
        vals = np.empty(n, np.uint8)
        got = lib().opma_csr(self.h, _ptr(ro), _ptr(ci), _ptr(vals), n)
        assert got == n
        return ro, ci, vals


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
