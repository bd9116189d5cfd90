"""ctypes declarations of the C ABI in include/lpma.h.

The shared library is built in-tree (lpma_gb300/_lpma.so, see build.py).  If
it is missing, importing the package raises: there is no CPU fallback.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lpma.so")

LPMA_OK = 0
STATUS_NAMES = {
    0: "LPMA_OK", 1: "LPMA_ERR_INVALID_ARGUMENT", 2: "LPMA_ERR_INVALID_KEY", 3: "LPMA_ERR_OUT_OF_MEMORY",
    4: "LPMA_ERR_CUDA", 5: "LPMA_ERR_CAPACITY", 6: "LPMA_ERR_INTERNAL", 7: "LPMA_ERR_TIMEOUT",
    8: "LPMA_ERR_BUFFER_TOO_SMALL", 9: "LPMA_ERR_SCRATCH_LIMIT", 10: "LPMA_ERR_IO",
}
KEY_PACKED, KEY_PAIR32 = 0, 1
FLAG_CONCURRENT = 1
MAX_HEIGHT = 24

# every entry point include/lpma.h declares
EXPORTS = [
    "lpma_config_default", "lpma_create", "lpma_build", "lpma_update", "lpma_update_host", "lpma_csr_view",
    "lpma_to_csr", "lpma_export_sorted", "lpma_export_layout", "lpma_info", "lpma_destroy", "lpma_status_string",
    "lpma_gen_rmat", "lpma_shuffle", "lpma_kernel_launches", "lpma_prof_enable", "lpma_prof_report",
    "lpma_shuffle_static", "lpma_query_neighbors", "lpma_edge_query", "lpma_bfs", "lpma_pagerank",
    "lpma_read_edgelist", "lpma_read_queries", "lpma_memory_bytes", "lpma_pool_create", "lpma_pool_submit",
    "lpma_pool_wait", "lpma_pool_drain", "lpma_pool_destroy", "lpma_set_flags", "lpma_error_detail", "lpma_pool_submit_many",
    "lpma_batcher_create", "lpma_batcher_destroy", "lpma_update_batch",
    "lpma_autotune", "lpma_tune_set", "lpma_tune_get", "lpma_memory_reserve", "lpma_debug_sort_barrier",
    "lpma_debug_exec_wait",
    "lpma_config_gpma", "lpma_gpma_view", "lpma_grain_set", "lpma_grain_get", "lpma_autotune_grain",
]
SORT_TIERS = {1: "small", 2: "block", 3: "tile_merge", 4: "cooperative", 5: "multi_pass"}
REQ_UPDATE, REQ_NEIGHBORS, REQ_BFS, REQ_EDGE_QUERY = 0, 1, 2, 3
SHUFFLE_STATIC_MAX_KEYS = 65536


class LpmaConfig(ctypes.Structure):
    _fields_ = [("segment_length", ctypes.c_uint32), ("key_format", ctypes.c_uint32),
                ("skip_rule", ctypes.c_uint32), ("flags", ctypes.c_uint32),
                ("density_lower_root", ctypes.c_double), ("density_upper_root", ctypes.c_double)]


class LpmaStats(ctypes.Structure):
    _fields_ = [("height_before", ctypes.c_uint32), ("height_after", ctypes.c_uint32),
                ("n_ins_applied", ctypes.c_uint32), ("n_upserts", ctypes.c_uint32),
                ("n_del_applied", ctypes.c_uint32), ("n_noop", ctypes.c_uint32),
                ("root_executed", ctypes.c_uint32), ("eager_levelup", ctypes.c_uint32),
                ("overflow", ctypes.c_uint32), ("rebuilt", ctypes.c_uint32),
                ("levelup_path", ctypes.c_uint32), ("fill_empty", ctypes.c_uint32),
                ("windows_single", ctypes.c_uint64), ("windows_small", ctypes.c_uint64),
                ("windows_big", ctypes.c_uint64),
                ("slots_rewritten", ctypes.c_uint64), ("slots_small", ctypes.c_uint64),
                ("num_items", ctypes.c_uint64),
                ("h2d_bytes", ctypes.c_uint64), ("d2h_bytes", ctypes.c_uint64),
                ("sort_passes", ctypes.c_uint32), ("levelup", ctypes.c_uint32)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}

    def __getitem__(self, name):
        return getattr(self, name)


class LpmaRequest(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_uint32), ("host_inputs", ctypes.c_uint32), ("graph", ctypes.c_void_p),
                ("keys0", ctypes.c_void_p), ("vals0", ctypes.c_void_p), ("n0", ctypes.c_size_t),
                ("keys1", ctypes.c_void_p), ("n1", ctypes.c_size_t),
                ("vertices", ctypes.c_void_p), ("windows", ctypes.c_void_p), ("nv", ctypes.c_size_t),
                ("thres", ctypes.c_uint32), ("max_depth", ctypes.c_uint32),
                ("out_u32", ctypes.c_void_p), ("out_nbrs", ctypes.c_void_p), ("out_vals", ctypes.c_void_p),
                ("out_dist", ctypes.c_void_p), ("cap", ctypes.c_size_t),
                ("status", ctypes.c_int), ("levels", ctypes.c_uint32), ("reached", ctypes.c_uint64),
                ("stats", LpmaStats),
                ("t_submit_ns", ctypes.c_uint64), ("t_start_ns", ctypes.c_uint64), ("t_end_ns", ctypes.c_uint64),
                ("t_call_ns", ctypes.c_uint64), ("pool_growth_bytes", ctypes.c_uint64), ("device_ms", ctypes.c_float),
                ("done", ctypes.c_uint32)]


class LpmaBatch(ctypes.Structure):
    _fields_ = [("ins", ctypes.c_void_p), ("ins_vals", ctypes.c_void_p), ("n_ins", ctypes.c_size_t),
                ("dels", ctypes.c_void_p), ("n_del", ctypes.c_size_t),
                ("thres", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class LpmaTuneEntry(ctypes.Structure):
    _fields_ = [("log2_keys", ctypes.c_uint32), ("concurrent", ctypes.c_uint32), ("tier", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32), ("us", ctypes.c_float * 6)]


class LpmaGrainTime(ctypes.Structure):
    _fields_ = [("max_segs_group", ctypes.c_uint32), ("max_segs_shared", ctypes.c_uint32),
                ("us_median", ctypes.c_float), ("reserved", ctypes.c_uint32)]


class LpmaError(RuntimeError):
    def __init__(self, status, where=""):
        self.status = status
        super().__init__("%s: %s" % (where, STATUS_NAMES.get(status, status)))


_lib = None


def load():
    """Load the engine library; raises ImportError when it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("lpma_gb300/_lpma.so is missing: build it with `python -m lpma_gb300.build` "
                          "(or __graft_entry__.build()); the engine has no CPU fallback")
    L = ctypes.CDLL(LIB_PATH)
    P, SZ, U32, U64, I = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int
    sig = {
        "lpma_config_default": [P],
        "lpma_create": [P, U32, P, P],
        "lpma_build": [P, P, P, SZ, P],
        "lpma_update": [P, P, P, SZ, P, SZ, U32, P, P],
        "lpma_update_host": [P, P, P, SZ, P, SZ, U32, P, P],
        "lpma_csr_view": [P, P, P, P, P, P],
        "lpma_to_csr": [P, P, P, P, SZ, P, P],
        "lpma_export_sorted": [P, P, P, SZ, P, P],
        "lpma_export_layout": [P, P, P, SZ, P, SZ, P, P],
        "lpma_info": [P, P, P, P],
        "lpma_destroy": [P],
        "lpma_gen_rmat": [U64, U32, U32, U32, U32, U32, P, SZ, P, P],
        "lpma_shuffle": [U64, P, SZ, P],
        "lpma_shuffle_static": [U64, P, SZ, P],
        "lpma_query_neighbors": [P, P, P, SZ, P, P, P, SZ, P, P],
        "lpma_edge_query": [P, P, SZ, U32, P, P],
        "lpma_bfs": [P, P, SZ, U32, P, P, P, P],
        "lpma_pagerank": [P, ctypes.c_double, U32, P, P],
        "lpma_read_edgelist": [ctypes.c_char_p, ctypes.c_char_p, P, SZ, P, P],
        "lpma_read_queries": [ctypes.c_char_p, P, P, SZ, P],
        "lpma_memory_bytes": [P, P],
        "lpma_memory_reserve": [U64, P],
        "lpma_set_flags": [P, U32],
        "lpma_error_detail": [P, P],
        "lpma_pool_create": [U32, U64, P],
        "lpma_pool_submit": [P, P],
        "lpma_pool_submit_many": [P, P, SZ],
        "lpma_pool_wait": [P, P],
        "lpma_pool_drain": [P],
        "lpma_pool_destroy": [P],
        "lpma_batcher_create": [P],
        "lpma_batcher_destroy": [P],
        "lpma_update_batch": [P, P, P, SZ, P, P, P],
        "lpma_autotune": [U32, P, P, SZ, P],
        "lpma_tune_set": [U32, U32, U32],
        "lpma_tune_get": [U32, U32, P],
        "lpma_grain_set": [U32, U32, U32],
        "lpma_grain_get": [U32, P, P],
        "lpma_autotune_grain": [P, P, SZ, U32, P, P, SZ, P],
        "lpma_debug_sort_barrier": [U32, I],
        "lpma_debug_exec_wait": [I],
        "lpma_config_gpma": [P],
        "lpma_gpma_view": [P, P, P, P, P, P, P],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = I
    L.lpma_status_string.argtypes = [I]
    L.lpma_status_string.restype = ctypes.c_char_p
    L.lpma_prof_enable.argtypes = [I]
    L.lpma_prof_enable.restype = I
    L.lpma_prof_report.argtypes = [ctypes.c_char_p, SZ]
    L.lpma_prof_report.restype = SZ
    L.lpma_kernel_launches.argtypes = []
    L.lpma_kernel_launches.restype = U64
    _lib = L
    return L


def check(status, where):
    if status != LPMA_OK:
        raise LpmaError(status, where)
