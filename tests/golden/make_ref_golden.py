"""Generate golden vectors of tests/golden from the reference's own code.

The reference's integer functions on the update path are compiled for the
host by oracle/ref_host.py (verbatim text of rpma.cuh / gpma.cuh, CUDA
qualifiers defined away, kernels run as one thread).  This script runs
them and writes what they return:

* index_algebra.json -- GET_IDX / GET_LANE / GET_LINEAR_IDX (rpma.cuh:132-134)
  over every slot of trees of height 0..6;
* tables.json -- recalculate_density (rpma.cuh:136-168), the skip state
  machine of update_rpma (rpma.cuh:1614-1619), fls (rpma.cuh:98-113) and
  per-segment counts of redispatch_kernel's even spread (rpma.cuh:953-983);
* ref_vectors.json -- the resize height rule (rpma.cuh:1340-1352) on a grid,
  locate_leaf_kernel (rpma.cuh:253-315) over the layouts of seeded streams
  (the queries and the stop segment the reference finds), redispatch_kernel
  slot placements, GPMA's size rule (gpma.cuh:706-711) and density table
  (gpma.cuh:102-131), and GPMA's locate_leaf_kernel with handle_del_mod
  (gpma.cuh:162-200: stop slot and in-place value changes) over the layouts
  of seeded GPMA streams.

Each file records the SHA-256 of the generated translation units it came
from.  Run from the repository root, with the reference where
oracle/ref_host.py finds it (LPMA_REFERENCE_DIR):

    python tests/golden/make_ref_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import pyoracle as O  # noqa: E402
from oracle import ref_host as R  # noqa: E402

# streams whose layouts the locate vectors are taken on: step j inserts
# e[(j-1)*batch : j*batch]; every even step also deletes the first third
# of the batch inserted two steps before
LOCATE_STREAMS = [
    {"seed": 3, "scale": 5, "ef": 4, "batch": 9, "steps": [1, 4, 8]},
    {"seed": 5, "scale": 8, "ef": 8, "batch": 300, "steps": [1, 2, 5]},
    {"seed": 7, "scale": 10, "ef": 8, "batch": 1500, "steps": [2, 3, 5]},
]


def stream_states(spec):
    """(step, oracle) after each step of a locate stream (the oracle is reused)."""
    V = 1 << spec["scale"]
    e = O.shuffle(O.rmat_edges(spec["seed"], spec["scale"], spec["ef"]), spec["seed"] + 1)
    o = O.OracleLpma(V)
    b = spec["batch"]
    for j in range(1, max(spec["steps"]) + 1):
        o.update(ins=e[(j - 1) * b:j * b])
        if j % 2 == 0:
            o.update(dels=e[(j - 2) * b:(j - 2) * b + b // 3])
        if j in spec["steps"]:
            yield j, o, e


# GPMA streams (keys src << 32 | dst): step j inserts e[(j-1)*batch : j*batch]
# and, on even steps, deletes the first half of the batch two steps before
GPMA_STREAMS = [
    {"seed": 3, "scale": 5, "ef": 4, "batch": 11, "steps": [1, 3, 6]},
    {"seed": 5, "scale": 9, "ef": 8, "batch": 700, "steps": [2, 4, 5]},
]


def gpma_keys(e):
    return ((e >> np.uint64(42)) << np.uint64(32)) | ((e >> np.uint64(20)) & np.uint64(0x3FFFFF))


def gpma_stream_states(spec):
    V = 1 << spec["scale"]
    e = gpma_keys(O.shuffle(O.rmat_edges(spec["seed"], spec["scale"], spec["ef"]), spec["seed"] + 1))
    o = O.OracleGpma(V)
    b = spec["batch"]
    for j in range(1, max(spec["steps"]) + 1):
        o.update(ins=e[(j - 1) * b:j * b])
        if j % 2 == 0:
            o.update(dels=e[(j - 2) * b:(j - 2) * b + b // 2])
        if j in spec["steps"]:
            yield j, o, e


def locate_queries(o, e, seed, n=600):
    rng = np.random.default_rng(seed)
    stored, _ = o.export_sorted()
    pick = stored[rng.integers(0, stored.size, n // 3)]
    return np.concatenate([pick, pick + np.uint64(1), e[rng.integers(0, e.size, n // 3)],
                           rng.integers(0, 1 << 63, n - 3 * (n // 3), dtype=np.uint64)])


def phys(L, H):
    s1 = (L >> 5) + 1
    t = (s1 & -s1).bit_length() - 1
    return 32 * ((1 << (H - t)) - 1) + 32 * (s1 >> (t + 1)) + (L & 31)


def main():
    out = os.environ.get("LPMA_GOLDEN_OUT", HERE)
    R.build()
    digest = R.source_digest()
    prov = {"generator": "tests/golden/make_ref_golden.py via oracle/ref_host.py",
            "source": "reference rpma.cuh / gpma.cuh functions compiled for the host",
            "units_sha256": digest}
    L = R.lib()

    blocks = []
    for H in range(0, 7):
        n = 32 * ((2 << H) - 1)
        rows = []
        for lin in range(n):
            i = L.ref_get_idx(lin, H)
            ln = L.ref_get_lane(lin, i, H)
            rows.append([lin, i, ln, L.ref_get_linear_idx(i, ln, H) + (ln % 32)])
        blocks.append({"height": H, "rows": rows})
    with open(os.path.join(out, "index_algebra.json"), "w") as f:
        json.dump({"provenance": prov, "blocks": blocks}, f, separators=(",", ":"))

    lo, up = R.density()
    red = []
    for f_ in (1, 2, 3, 4, 7, 8, 16, 31, 32):
        for m in (1, 2, 5, 13, 31, 32, 33, 100, 32 * f_):
            if m > 32 * f_:
                continue
            width = 32 * f_
            H = max(0, (f_ - 1).bit_length())  # a tree tall enough for a window of f segments at node 0
            while 32 * ((2 << H) - 1) < width:
                H += 1
            nslots = 32 * ((2 << H) - 1)
            items = np.arange(1, m + 1, dtype=np.uint64) << np.uint64(20)
            keys = np.full(nslots, 0xFFFFFFFFFFFFFFFF, np.uint64)
            rk, _, _, _ = R.redispatch(keys, np.zeros(nslots, np.uint8), H, 0, width, items, np.ones(m, np.uint8), 4)
            counts = [int(sum(rk[phys(32 * s + l, H)] != np.uint64(0xFFFFFFFFFFFFFFFF) for l in range(32)))
                      for s in range(f_)]
            red.append({"f": f_, "m": m, "counts": counts})
    tables = {"provenance": prov, "lower": lo.tolist(), "upper": up.tolist(),
              "skip": {str(H): R.skip_table(H, 27).tolist() for H in range(0, 25)},
              "fls": {str(x): int(L.ref_fls(x)) for x in [0, 1, 2, 3, 4, 5, 31, 32, 33, 1000, 65535, 65536, 2 ** 31]},
              "redistribute": red}
    with open(os.path.join(out, "tables.json"), "w") as f:
        json.dump(tables, f, separators=(",", ":"))

    rng = np.random.default_rng(11)
    resize = []
    for _ in range(400):
        H = int(rng.integers(0, 21))
        comp = int(rng.integers(0, 32 * (2 << min(H + 2, 21))))
        upd = int(rng.integers(0, 1 << int(rng.integers(0, 22))))
        root = int(rng.integers(0, 2))
        resize.append([H, comp, upd, root, int(L.ref_resize_height(H, comp, upd, root))])

    locate = []
    for spec in LOCATE_STREAMS:
        for j, o, e in stream_states(spec):
            k, _ = o.layout()
            q = locate_queries(o, e, 100 * spec["seed"] + j)
            leaf = R.locate(k, o.height, q)
            assert np.array_equal(leaf, R.locate_mixed(k, o.height, q))
            locate.append({"stream": {x: spec[x] for x in ("seed", "scale", "ef", "batch")}, "step": j,
                           "height": o.height, "queries": [str(int(x)) for x in q], "leaf": leaf.tolist()})

    spread = []
    for c in range(80):
        H = int(rng.integers(0, 6))
        nslots = 32 * ((2 << H) - 1)
        level = int(rng.integers(0, H + 2))
        width = 32 << level
        node = int(rng.integers(0, (nslots + 32) // width)) * width
        if node + width >= 32 << (H + 1):
            width -= 32
        if width <= 0:
            continue
        m = int(rng.integers(0, width + 1))
        V = 64
        src = np.sort(rng.integers(0, V, m)).astype(np.uint64)
        items = np.unique((src << np.uint64(42)) | rng.integers(0, 1 << 42, m, dtype=np.uint64))
        sel = rng.random(items.size) < 0.15
        items[sel] = ((items[sel] >> np.uint64(42)) << np.uint64(42)) + np.uint64(0x000003FFFFEFFFFF)
        items = np.unique(items)
        vals = rng.integers(1, 250, items.size).astype(np.uint8)
        keys = np.full(nslots, 0xFFFFFFFFFFFFFFFF, np.uint64)
        rk, rv, ci, cl = R.redispatch(keys, np.zeros(nslots, np.uint8), H, node, width, items, vals, V)
        where = {int(x): i for i, x in enumerate(rk) if x != np.uint64(0xFFFFFFFFFFFFFFFF)}
        slots = [where[int(x)] for x in items]
        sent = [[v, int(ci[v + 1]), int(cl[v + 1])] for v in range(V) if ci[v + 1] != 0xFFFFFFFF]
        spread.append({"height": H, "node": node, "width": width, "items": [str(int(x)) for x in items],
                       "vals": vals.tolist(), "slots": slots, "sentinels": sent})

    gpma_locate = []
    for spec in GPMA_STREAMS:
        for j, o, e in gpma_stream_states(spec):
            keys, vals, _ = o.layout()
            size, seg, h = o.geometry()
            qrng = np.random.default_rng(1000 * spec["seed"] + j)
            q = np.unique(np.concatenate([e[qrng.integers(0, e.size, 150)],
                                          qrng.integers(0, 1 << 40, 30, dtype=np.uint64)]))
            qv = qrng.integers(1, 255, q.size).astype(np.uint8)
            qv[qrng.random(q.size) < 0.3] = 0xFF
            leaf, v2 = R.gpma_locate(keys, vals, seg, h, q, qv)
            occ = keys != np.uint64(0xFFFFFFFFFFFFFFFF)
            gpma_locate.append({"stream": {x: spec[x] for x in ("seed", "scale", "ef", "batch")}, "step": j,
                                "geometry": [size, seg, h], "queries": [str(int(x)) for x in q],
                                "qvals": qv.tolist(), "leaf": leaf.tolist(),
                                "vals_after": [int(x) for x in v2[occ]]})

    gpma_size = [[m] + list(R.gpma_size(m)) for m in list(range(0, 70)) + [100, 127, 128, 129, 1000, 4096, 4097,
                                                                            100000, 5_000_000, 33_554_433]]
    gpma_density = []
    for seg, h in [(2, 1), (4, 3), (8, 10), (16, 15), (16, 21), (32, 26)]:
        lo_, up_ = R.gpma_density(seg, h)
        gpma_density.append({"segment_length": seg, "height": h, "lower": lo_.tolist(), "upper": up_.tolist()})
    with open(os.path.join(out, "ref_vectors.json"), "w") as f:
        json.dump({"provenance": prov, "resize_height": resize, "locate": locate, "redistribute": spread,
                   "gpma_size": gpma_size, "gpma_density": gpma_density, "gpma_locate": gpma_locate}, f,
                  separators=(",", ":"))
    print("wrote index_algebra.json, tables.json, ref_vectors.json from units %s" % digest[:16])


if __name__ == "__main__":
    main()
