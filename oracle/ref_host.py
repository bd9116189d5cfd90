"""Pieces of the reference compiled for the host, to pin the oracle.

TEST INFRASTRUCTURE ONLY: used by tests/ and tests/golden/make_ref_golden.py
to check the oracle (oracle/lpma_oracle.c) against the reference's own code.
The product never loads it.

The reference (pkumod/LPMA) does not build under CUDA 13 as a whole
(device-side cudaDeviceSynchronize of CUDA Dynamic Parallelism 1 and the
removed __shfl_down).  Several of its functions on the update path are
plain integer code, though, and compile for the host unchanged once the
CUDA qualifiers are defined away and a kernel is run as a single thread
(blockDim = gridDim = 1, so its grid-stride loop covers every item):

  rpma.cuh  typedefs and key constants (:21-50); class RPMA, fls, lls,
            GET_IDX / GET_LANE / GET_LINEAR_IDX (:60-134);
            recalculate_density (:136-168); locate_leaf_kernel (:253-315) and
            locate_leaf_kernel_mixed (:318-413);
            redispatch_kernel (:953-983); the height rule of resize_rpma
            (:1311-1312, :1340-1352); the skip state machine of update_rpma
            (:1614-1619)
  gpma.cuh  typedefs and constants (:17-34); class GPMA (:39-64); fls
            (:66-82); recalculate_density (:102-131); handle_del_mod and
            locate_leaf_kernel (:162-200); redispatch_kernel (:428-452); the
            size rule of resize_gpma (:706-711)

This recipe copies that text, verbatim, out of the reference where it
lies (LPMA_REFERENCE_DIR, default /root/reference) into generated
translation units under oracle/_ref/ (git-ignored), adds a prelude of
shims and extern "C" wrappers, and compiles them with g++ into
oracle/_ref/libref_host.so.  Nothing of the reference's text is committed.
"""
import ctypes
import hashlib
import os
import re
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT, "libref_host.so")
DEFAULT_REF = "/root/reference"


class RefUnavailable(RuntimeError):
    pass


def reference_dir():
    return os.environ.get("LPMA_REFERENCE_DIR", DEFAULT_REF)


# ------------------------------------------------------------------ extraction
def _lines(src):
    return src.split("\n")


def region(src, start_re, end_re):
    """Lines from the one line matching start_re through the first line at
    or after it matching end_re (both inclusive)."""
    ls = _lines(src)
    starts = [i for i, l in enumerate(ls) if re.search(start_re, l)]
    if len(starts) != 1:
        raise RefUnavailable("anchor %r found %d times" % (start_re, len(starts)))
    for j in range(starts[0], len(ls)):
        if re.search(end_re, ls[j]):
            return "\n".join(ls[starts[0]:j + 1])
    raise RefUnavailable("end anchor %r not found" % end_re)


def function(src, signature, qualifier_lines=1):
    """A whole function definition: the line holding `signature` (plus the
    qualifier lines just above it, e.g. __global__) through its closing
    brace."""
    i = src.find(signature)
    if i < 0 or src.find(signature, i + 1) >= 0:
        raise RefUnavailable("function %r not found exactly once" % signature)
    line_start = src.rfind("\n", 0, i) + 1
    begin = line_start
    for _ in range(qualifier_lines):
        prev = src.rfind("\n", 0, begin - 1) + 1
        if prev >= begin - 1:
            break
        begin = prev
    j = src.find("{", i)
    depth = 0
    k = j
    while k < len(src):
        two = src[k:k + 2]
        if two == "//":  # braces inside comments do not count
            k = src.find("\n", k)
            if k < 0:
                break
            continue
        if two == "/*":
            k = src.find("*/", k) + 2
            continue
        if src[k] in "\"'":  # nor inside string or character literals
            q = src[k]
            k += 1
            while k < len(src) and src[k] != q:
                k += 2 if src[k] == "\\" else 1
        elif src[k] == "{":
            depth += 1
        elif src[k] == "}":
            depth -= 1
            if depth == 0:
                return src[begin:k + 1]
        k += 1
    raise RefUnavailable("unbalanced braces in %r" % signature)


def statement(src, text):
    """The one line holding `text`."""
    hits = [l for l in _lines(src) if text in l]
    if len(hits) != 1:
        raise RefUnavailable("statement %r found %d times" % (text, len(hits)))
    return hits[0]


PRELUDE = r"""
// generated by oracle/ref_host.py -- host shims for code of the reference
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
namespace thrust {
template <typename T> using device_vector = std::vector<T>;
template <typename T> using host_vector = std::vector<T>;
}
#define __host__
#define __device__
#define __global__
#define __forceinline__ inline
#define __inline__ inline
#define __shared__ static
#define cErr(x) ((void)(x))
static inline int cudaDeviceSynchronize() { return 0; }
struct RefDim3 { unsigned x, y, z; };
static const RefDim3 threadIdx = {0, 0, 0}, blockIdx = {0, 0, 0}, blockDim = {1, 1, 1}, gridDim = {1, 1, 1};
static inline void __syncthreads() {}
using std::min;
using std::max;
"""


def rpma_unit(src):
    parts = [
        region(src, r"^typedef unsigned long long KEY_TYPE;", r"^const SIZE_TYPE NBR_END"),
        region(src, r"^class RPMA \{", r"^#define GET_LINEAR_IDX"),
        function(src, "void recalculate_density(RPMA &rpma)"),
        function(src, "void locate_leaf_kernel(KEY_PTR key_ptrs[]"),
        function(src, "void locate_leaf_kernel_mixed(KEY_PTR key_ptrs[]"),
        function(src, "void redispatch_kernel(KEY_TYPE *tmp_keys"),
    ]
    resize = function(src, "int resize_rpma(RPMA &rpma")
    height_rule = "\n".join([
        statement(resize, "SIZE_TYPE updated_tree_height = 0;"),
        statement(resize, "SIZE_TYPE tree_size = rpma.segment_length * ((2 << updated_tree_height) - 1);"),
        region(resize, r"SIZE_TYPE merge_size = compacted_size \+ update_size;", r"^\s*return updated_tree_height;"),
    ])
    upd = function(src, "bool update_rpma(RPMA &rpma")
    skip = region(upd, r"if\(level==4\|\|level==rpma.tree_height/3\)\{", r"skip=false;")
    skip += "\n\t\t}"
    wrappers = r"""
// ---- wrappers (not reference text) ----
static SIZE_TYPE ref_resize_height_body(RPMA &rpma, SIZE_TYPE compacted_size, SIZE_TYPE update_size, bool reach_root) {
%s
}
extern "C" {
uint32_t ref_fls(uint32_t x) { return fls(x); }
uint32_t ref_lls(uint32_t x) { return lls(x); }
uint32_t ref_get_idx(uint32_t L, uint32_t H) { SIZE_TYPE LINEAR = L, HEIGHT = H; return GET_IDX(LINEAR, HEIGHT); }
uint32_t ref_get_lane(uint32_t L, uint32_t I, uint32_t H) {
    SIZE_TYPE LINEAR = L, IDX = I, HEIGHT = H; return GET_LANE(LINEAR, IDX, HEIGHT);
}
uint32_t ref_get_linear_idx(uint32_t I, uint32_t lane, uint32_t H) {
    SIZE_TYPE IDX = I, LANE = lane, HEIGHT = H; return GET_LINEAR_IDX(IDX, LANE, HEIGHT);
}
void ref_density(uint32_t *lower, uint32_t *upper) {
    RPMA r; r.segment_length = 32; r.tree_height = 0;
    recalculate_density(r);
    for (int i = 0; i < 26; i++) { lower[i] = r.lower_element[i]; upper[i] = r.upper_element[i]; }
}
uint32_t ref_resize_height(uint32_t H, uint32_t compacted_size, uint32_t update_size, int reach_root) {
    RPMA r; r.segment_length = 32; r.tree_height = H;
    return ref_resize_height_body(r, compacted_size, update_size, reach_root != 0);
}
void ref_skip_table(uint32_t H, uint8_t *out, int n) {
    RPMA rpma; rpma.segment_length = 32; rpma.tree_height = H;
    bool skip = false;
    for (SIZE_TYPE level = 0; level < (SIZE_TYPE)n; ++level) {
%s
        out[level] = skip ? 1 : 0;
    }
}
// heap layout: level i at slot 32 * (2^i - 1)
void ref_locate(const uint64_t *heap_keys, uint32_t H, const uint64_t *keys, uint32_t n, uint32_t *leaf) {
    KEY_PTR kp[26]; VALUE_PTR vp[26];
    std::vector<VALUE_TYPE> dummy_vals(32ull * ((2ull << H) - 1));
    for (int i = 0; i < 26; i++) {
        uint64_t base = 32ull * ((1ull << (i <= (int)H ? i : 0)) - 1);
        kp[i] = (KEY_TYPE *)heap_keys + base;
        vp[i] = dummy_vals.data() + base;
    }
    std::vector<KEY_TYPE> k((const KEY_TYPE *)keys, (const KEY_TYPE *)keys + n);
    std::vector<VALUE_TYPE> v(n, 1);
    locate_leaf_kernel(kp, vp, 32, H, k.data(), v.data(), n, leaf);
}
// the first loop's locate (update keys only, no edge queries)
void ref_locate_mixed(const uint64_t *heap_keys, uint32_t H, const uint64_t *keys, uint32_t n, uint32_t *leaf) {
    KEY_PTR kp[26]; VALUE_PTR vp[26];
    std::vector<VALUE_TYPE> dummy_vals(32ull * ((2ull << H) - 1));
    for (int i = 0; i < 26; i++) {
        uint64_t base = 32ull * ((1ull << (i <= (int)H ? i : 0)) - 1);
        kp[i] = (KEY_TYPE *)heap_keys + base;
        vp[i] = dummy_vals.data() + base;
    }
    std::vector<KEY_TYPE> k((const KEY_TYPE *)keys, (const KEY_TYPE *)keys + n);
    std::vector<VALUE_TYPE> v(n, 1);
    KEY_TYPE no_query = 0;
    VALUE_TYPE no_flag = 0;
    locate_leaf_kernel_mixed(kp, vp, 32, H, k.data(), v.data(), &no_query, &no_flag, n, 0, leaf);
}
// items (sorted) spread over the window [node, node + width) of a heap layout
void ref_redispatch(uint64_t *heap_keys, uint8_t *heap_vals, uint32_t H, uint32_t node, uint32_t width,
                    const uint64_t *items, const uint8_t *item_vals, uint32_t m, uint32_t *csr_idx, uint32_t *csr_lane) {
    KEY_PTR kp[26]; VALUE_PTR vp[26];
    for (int i = 0; i < 26; i++) {
        uint64_t base = 32ull * ((1ull << (i <= (int)H ? i : 0)) - 1);
        kp[i] = (KEY_TYPE *)heap_keys + base; vp[i] = heap_vals + base;
    }
    std::vector<KEY_TYPE> k((const KEY_TYPE *)items, (const KEY_TYPE *)items + m);
    std::vector<VALUE_TYPE> v(item_vals, item_vals + m);
    redispatch_kernel(k.data(), v.data(), kp, vp, width, 32, m, node, H, csr_idx, csr_lane);
}
}
""" % (height_rule, skip)
    return PRELUDE + "\n".join(parts) + wrappers


def gpma_unit(src):
    parts = [
        region(src, r"^typedef unsigned long long KEY_TYPE;", r"^const KEY_TYPE COL_IDX_NONE"),
        region(src, r"^class GPMA \{", r"^\};"),
        function(src, "SIZE_TYPE fls(SIZE_TYPE x)", qualifier_lines=1),
        function(src, "void recalculate_density(GPMA &gpma)"),
        function(src, "SIZE_TYPE handle_del_mod(KEY_TYPE *keys", qualifier_lines=0),
        function(src, "void locate_leaf_kernel(KEY_TYPE *keys"),
        function(src, "void redispatch_kernel(KEY_TYPE *tmp_keys"),
    ]
    rg = function(src, "int resize_gpma(GPMA &gpma")
    size_rule = region(rg, r"SIZE_TYPE tree_size = 4;", r"gpma.tree_height = fls\(tree_size / gpma.segment_length\) - 1;")
    wrappers = r"""
// ---- wrappers (not reference text) ----
static SIZE_TYPE ref_gpma_size_body(GPMA &gpma, SIZE_TYPE merge_size) {
%s
    return tree_size;
}
extern "C" {
uint32_t ref_gpma_fls(uint32_t x) { return fls(x); }
// tree size, segment length and height for merge_size items
void ref_gpma_size(uint32_t merge_size, uint32_t *tree_size, uint32_t *seg_length, uint32_t *height) {
    GPMA g;
    *tree_size = ref_gpma_size_body(g, merge_size);
    *seg_length = g.segment_length;
    *height = g.tree_height;
}
// density table of a GPMA of the given segment length and height
void ref_gpma_density(uint32_t seg_length, uint32_t height, uint32_t *lower, uint32_t *upper) {
    GPMA g; g.segment_length = seg_length; g.tree_height = height;
    recalculate_density(g);
    for (uint32_t i = 0; i <= height; i++) { lower[i] = g.lower_element[i]; upper[i] = g.upper_element[i]; }
}
// locate + handle_del_mod over a flat array (vals updated in place, as the kernel does)
void ref_gpma_locate(const uint64_t *keys, uint8_t *vals, uint32_t tree_size, uint32_t seg_length, uint32_t height,
                     const uint64_t *upd, const uint8_t *upd_vals, uint32_t n, uint32_t *leaf) {
    std::vector<KEY_TYPE> k((const KEY_TYPE *)upd, (const KEY_TYPE *)upd + n);
    std::vector<VALUE_TYPE> v((const VALUE_TYPE *)upd_vals, (const VALUE_TYPE *)upd_vals + n);
    locate_leaf_kernel((KEY_TYPE *)keys, (VALUE_TYPE *)vals, tree_size, seg_length, height, k.data(),
                       v.data(), n, leaf);
}
// items (sorted) spread over [node, node + width) of a flat array
void ref_gpma_redispatch(uint64_t *keys, uint8_t *vals, uint32_t node, uint32_t width, uint32_t seg_length,
                         const uint64_t *items, const uint8_t *item_vals, uint32_t m, uint32_t *row_offset) {
    std::vector<KEY_TYPE> k((const KEY_TYPE *)items, (const KEY_TYPE *)items + m);
    std::vector<VALUE_TYPE> v((const VALUE_TYPE *)item_vals, (const VALUE_TYPE *)item_vals + m);
    redispatch_kernel(k.data(), v.data(), (KEY_TYPE *)keys + node, (VALUE_TYPE *)vals + node, width, seg_length, m, row_offset,
                      node);
}
}
""" % size_rule
    return PRELUDE + "\n".join(parts) + wrappers


def build(force=False):
    """Generate and compile oracle/_ref/libref_host.so; RefUnavailable when
    the reference or g++ is missing or the text no longer matches."""
    ref = reference_dir()
    rp, gp = os.path.join(ref, "rpma.cuh"), os.path.join(ref, "gpma.cuh")
    if not (os.path.exists(rp) and os.path.exists(gp)):
        raise RefUnavailable("reference sources not found under %s" % ref)
    rsrc, gsrc = open(rp).read(), open(gp).read()
    units = {"ref_rpma.cpp": rpma_unit(rsrc), "ref_gpma.cpp": gpma_unit(gsrc)}
    digest = hashlib.sha256("".join(units[k] for k in sorted(units)).encode()).hexdigest()
    os.makedirs(OUT, exist_ok=True)
    stamp = os.path.join(OUT, "sha256")
    if not force and os.path.exists(LIB) and os.path.exists(stamp) and open(stamp).read() == digest:
        return LIB
    for name, text in units.items():
        with open(os.path.join(OUT, name), "w") as f:
            f.write(text)
    cmd = ["g++", "-std=c++17", "-O1", "-fPIC", "-shared", "-w", "-o", LIB] + \
          [os.path.join(OUT, n) for n in sorted(units)]
    try:
        subprocess.check_output(cmd, stderr=subprocess.STDOUT)
    except (OSError, subprocess.CalledProcessError) as e:
        raise RefUnavailable("g++ failed on the extracted reference text: %s" % getattr(e, "output", e))
    with open(stamp, "w") as f:
        f.write(digest)
    return LIB


def source_digest():
    """SHA-256 of the generated translation units (the fixtures record it)."""
    build()
    return open(os.path.join(OUT, "sha256")).read()


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(build())
        P, U32, I = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int
        sig = {
            "ref_fls": (U32, [U32]), "ref_lls": (U32, [U32]),
            "ref_get_idx": (U32, [U32, U32]), "ref_get_lane": (U32, [U32, U32, U32]),
            "ref_get_linear_idx": (U32, [U32, U32, U32]),
            "ref_density": (None, [P, P]),
            "ref_resize_height": (U32, [U32, U32, U32, I]),
            "ref_skip_table": (None, [U32, P, I]),
            "ref_locate": (None, [P, U32, P, U32, P]),
            "ref_locate_mixed": (None, [P, U32, P, U32, P]),
            "ref_redispatch": (None, [P, P, U32, U32, U32, P, P, U32, P, P]),
            "ref_gpma_fls": (U32, [U32]),
            "ref_gpma_size": (None, [U32, P, P, P]),
            "ref_gpma_density": (None, [U32, U32, P, P]),
            "ref_gpma_locate": (None, [P, P, U32, U32, U32, P, P, U32, P]),
            "ref_gpma_redispatch": (None, [P, P, U32, U32, U32, P, P, U32, P]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def density():
    lo, up = np.zeros(26, np.uint32), np.zeros(26, np.uint32)
    lib().ref_density(_p(lo), _p(up))
    return lo, up


def skip_table(H, n):
    out = np.zeros(n, np.uint8)
    lib().ref_skip_table(H, _p(out), n)
    return out


def locate(heap_keys, H, keys):
    heap_keys = np.ascontiguousarray(heap_keys, np.uint64)
    keys = np.ascontiguousarray(keys, np.uint64)
    out = np.zeros(keys.size, np.uint32)
    lib().ref_locate(_p(heap_keys), H, _p(keys), keys.size, _p(out))
    return out


def locate_mixed(heap_keys, H, keys):
    heap_keys = np.ascontiguousarray(heap_keys, np.uint64)
    keys = np.ascontiguousarray(keys, np.uint64)
    out = np.zeros(keys.size, np.uint32)
    lib().ref_locate_mixed(_p(heap_keys), H, _p(keys), keys.size, _p(out))
    return out


def redispatch(heap_keys, heap_vals, H, node, width, items, item_vals, V):
    """Spreads items over the window (keys of the window must already be
    KEY_NONE, as the reference's callers leave them); returns the new layout
    and the (csr_idx, csr_lane) rows it wrote (others stay 0xFFFFFFFF)."""
    k = np.ascontiguousarray(heap_keys, np.uint64).copy()
    v = np.ascontiguousarray(heap_vals, np.uint8).copy()
    items = np.ascontiguousarray(items, np.uint64)
    iv = np.ascontiguousarray(item_vals, np.uint8)
    ci = np.full(V + 1, 0xFFFFFFFF, np.uint32)
    cl = np.full(V + 1, 0xFFFFFFFF, np.uint32)
    lib().ref_redispatch(_p(k), _p(v), H, node, width, _p(items), _p(iv), items.size, _p(ci), _p(cl))
    return k, v, ci, cl


def gpma_size(merge_size):
    t, s, h = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
    lib().ref_gpma_size(merge_size, ctypes.byref(t), ctypes.byref(s), ctypes.byref(h))
    return t.value, s.value, h.value


def gpma_density(seg_length, height):
    lo, up = np.zeros(height + 1, np.uint32), np.zeros(height + 1, np.uint32)
    lib().ref_gpma_density(seg_length, height, _p(lo), _p(up))
    return lo, up


def gpma_locate(keys, vals, seg_length, height, upd, upd_vals):
    keys = np.ascontiguousarray(keys, np.uint64)
    v = np.ascontiguousarray(vals, np.uint8).copy()
    upd = np.ascontiguousarray(upd, np.uint64)
    uv = np.ascontiguousarray(upd_vals, np.uint8)
    leaf = np.zeros(upd.size, np.uint32)
    lib().ref_gpma_locate(_p(keys), _p(v), keys.size, seg_length, height, _p(upd), _p(uv), upd.size, _p(leaf))
    return leaf, v


def gpma_redispatch(keys, vals, node, width, seg_length, items, item_vals, row_offset):
    k = np.ascontiguousarray(keys, np.uint64).copy()
    v = np.ascontiguousarray(vals, np.uint8).copy()
    ro = np.ascontiguousarray(row_offset, np.uint32).copy()
    items = np.ascontiguousarray(items, np.uint64)
    iv = np.ascontiguousarray(item_vals, np.uint8)
    lib().ref_gpma_redispatch(_p(k), _p(v), node, width, seg_length, _p(items), _p(iv), items.size, _p(ro))
    return k, v, ro
