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


_torch = None


def _stream_ptr(stream):
    global _torch
    if stream is None:
        if _torch is None:
            try:
                import torch
                _torch = torch if torch.cuda.is_available() else False
            except ImportError:
                _torch = False
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

    def layout(self):
        """(keys, values, sentinel_slots, height) of the physical heap-order layout."""
        H = self.height
        ns = 32 * ((2 << H) - 1)
        k = np.empty(ns, np.uint64)
        v = np.empty(ns, np.uint8)
        sent = np.empty(self.num_vertices, np.uint32)
        h = ctypes.c_uint32()
        check(self._L.lpma_export_layout(self._h, k.ctypes.data_as(ctypes.c_void_p), v.ctypes.data_as(ctypes.c_void_p),
                                         ns, sent.ctypes.data_as(ctypes.c_void_p), sent.size, ctypes.byref(h),
                                         _stream_ptr(self.stream)), "lpma_export_layout")
        return k, v, sent, h.value

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
    return rpma.update(ins=keys, ins_vals=values, dels=del_keys, thres=thres)


def to_csr_rpma(rpma):
    ro, ci, _ = rpma.to_csr()
    return ro, ci


def get_data_rpma(rpma):
    return rpma.export_sorted()


def destroy_rpma(rpma):
    rpma.close()


# ------------------------------------------------------ workload generator
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
