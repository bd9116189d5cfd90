/*
 * CPU oracle for the LPMA batched edge-update path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: tests/, the smoke
 * check and the CPU-baseline leg of bench.py load it to compute the expected
 * layout and results.  The product (lpma_gb300) never links or calls it.
 *
 * Parity status: the reference (pkumod/LPMA) does not compile with CUDA 13
 * as a whole (device-side cudaDeviceSynchronize / CDP1 and the removed
 * __shfl_down).  Its integer functions on the update path do compile for
 * the host (oracle/ref_host.py): the index macros, fls / lls, the density
 * table, the skip state machine, the resize height rule, the locate descent
 * and the even redistribution.  Each of these steps of this restatement is
 * pinned to that compiled reference code, live (tests/test_oracle_reference.py)
 * and through fixtures it generated (tests/golden).  The whole-batch control
 * flow (level loop, window choice, merge, resize paths) is pinned only by the
 * reference's own result checks (sorted key set, per-row adjacency closed by
 * the sentinel) and by a second restatement in Python: for whole layouts the
 * parity is "partially unpinned".
 */
#ifndef LPMA_ORACLE_H
#define LPMA_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct OPma OPma;

typedef struct {
    /* what the update call did, for tests and for the byte model */
    uint32_t height_before, height_after;
    uint32_t n_ins_applied;     /* inserts that were new keys */
    uint32_t n_upserts;         /* inserts whose key was present: value overwritten */
    uint32_t n_del_applied;     /* deletes whose key was present */
    uint32_t n_noop;            /* deletes of absent keys + in-batch duplicates */
    uint32_t root_executed;     /* a level H+1 window absorbed updates */
    uint32_t eager_levelup;     /* a level was added after the root absorbed */
    uint32_t overflow;          /* updates left after the root */
    uint32_t rebuilt;           /* full rebuild happened (resize to new height) */
    uint32_t levelup_path;      /* overflow handled by adding one level + second loop */
    uint32_t fill_empty;        /* fill_empty_segs redistributed the array */
    uint32_t levelup;           /* update_rpma's return value: the level H+1 loop step absorbed the
                                   remaining updates (rpma.cuh:1646-1653) or updates overflowed (:1662-1668) */
    uint64_t win_count[32];     /* executed windows per level (reference order) */
    uint64_t win_slots[32];     /* slots covered by executed windows per level */
} OPmaStats;

/* init_csr_rpma (rpma.cuh:1808-1824): empty height-0 array, then V sentinels */
OPma *opma_create(uint32_t num_vertices, int skip_rule);
void opma_destroy(OPma *p);

/* update_rpma (rpma.cuh:1549-1718) with delete/dedup extension.
 * ins_vals may be NULL (value 1, as test_update_rpma.cu:72). */
int opma_update(OPma *p, const uint64_t *ins, const uint8_t *ins_vals, size_t n_ins,
                const uint64_t *del, size_t n_del, uint32_t thres, OPmaStats *st);

uint32_t opma_height(const OPma *p);
uint64_t opma_num_slots(const OPma *p);        /* 32 * (2^(H+1) - 1) */
uint64_t opma_num_items(const OPma *p);        /* physically present keys */

/* physical layout in heap (level-concatenated) order, as the reference's
 * per-level arrays laid end to end; empty slots have key ~0 */
int opma_layout(const OPma *p, uint64_t *keys, uint8_t *vals, size_t cap);
/* sentinel slot of vertex v (physical index), the csr_idx/csr_lane pair */
int opma_sentinel_slots(const OPma *p, uint32_t *out, size_t cap);

/* get_data_rpma (rpma.cuh:1735-1761): all present keys in sorted order */
int64_t opma_export_sorted(const OPma *p, uint64_t *keys, uint8_t *vals, size_t cap);

/* to_csr_rpma (rpma.cuh:2249-2295): row_offset (V+1), col_index, values */
int64_t opma_csr(const OPma *p, uint32_t *row_offset, uint32_t *col_index,
                 uint8_t *values, size_t cap);

/* index algebra (rpma.cuh:98-134) and thresholds (rpma.cuh:137-168), for
 * the known-answer tests */
uint32_t opma_get_idx(uint32_t linear, uint32_t height);
uint32_t opma_get_lane(uint32_t linear, uint32_t idx, uint32_t height);
uint32_t opma_get_linear_idx(uint32_t idx, uint32_t lane, uint32_t height);
void opma_density_table(uint32_t *lower, uint32_t *upper, int n);
/* the reference's skip state machine (rpma.cuh:1609-1619) for one height:
 * out[level] = 1 when big-grain windows at that level are skipped */
void opma_skip_table(uint32_t height, uint8_t *out, int n);
/* segment count of one destination segment under even redistribution
 * (rpma.cuh:677-679): item i -> segment floor(f*i/m) */
void opma_redistribute_counts(uint64_t f, uint64_t m, uint32_t *counts);

/* ---- test hooks: single steps of the restatement, compared with the
 * reference's own functions compiled for the host (oracle/ref_host.py) ----
 * opma_locate_keys: the stop segment of each key (linear slot of its first
 * lane), locate_leaf_kernel rpma.cuh:253-315.  opma_redistribute_window:
 * m sorted items spread over [node, node + width) of a heap layout of
 * height H, sentinel slots into sent (redispatch_kernel rpma.cuh:953-983).
 * opma_resize_height: resize_rpma's height rule (rpma.cuh:1340-1352). */
int opma_locate_keys(const OPma *p, const uint64_t *keys, size_t n, uint32_t *out);
int opma_redistribute_window(uint32_t H, uint32_t V, uint64_t node, uint64_t width, const uint64_t *mk,
                             const uint8_t *mv, uint64_t m, uint64_t *keys, uint8_t *vals, uint32_t *sent);
uint32_t opma_resize_height(uint64_t count, int reach_root);

/* ---- GPMA (gpma.cuh): the flat packed memory array ----
 * Keys src << 32 | dst, sentinel v << 32 | 0xFFFFFFFF, two KEY_MAX guards.
 * ogpma_create: init_csr_gpma (gpma.cuh:836-847); ogpma_update: update_gpma
 * (gpma.cuh:747-816) with deletes as VALUE_NONE updates; density_lower is
 * density_lower_thres_root (0.15, gpma.cuh:52). */
typedef struct OGpma OGpma;
OGpma *ogpma_create(uint32_t num_vertices, double density_lower);
void ogpma_destroy(OGpma *g);
int ogpma_update(OGpma *g, const uint64_t *ins, const uint8_t *ins_vals, size_t n_ins, const uint64_t *del,
                 size_t n_del, OPmaStats *st);
uint64_t ogpma_size(const OGpma *g, uint32_t *seg, uint32_t *height);
int ogpma_layout(const OGpma *g, uint64_t *keys, uint8_t *vals, size_t cap, uint32_t *row_offset);
int64_t ogpma_export_sorted(const OGpma *g, uint64_t *keys, uint8_t *vals, size_t cap);
void ogpma_size_rule(uint64_t merge, uint64_t *size, uint32_t *seg, uint32_t *height);
void ogpma_density(uint32_t seg, uint32_t height, double density_lower, uint32_t *lower, uint32_t *upper);
int ogpma_locate_keys(const OGpma *g, const uint64_t *keys, size_t n, uint32_t *out);
int ogpma_resolve_only(OGpma *g, const uint64_t *keys, const uint8_t *vals, size_t n, uint32_t *leaf);
int ogpma_spread_window(uint32_t V, uint32_t seg, uint64_t node, uint64_t width, const uint64_t *mk, const uint8_t *mv,
                        uint64_t m, uint64_t *keys, uint8_t *vals, uint32_t *row_offset);

/* ---- synthetic workload generators (identical integer arithmetic to the
 * device generator in lpma_gb300/csrc/gen.cu) ---- */
uint64_t opma_mix64(uint64_t z);
/* raw R-MAT keys (src<<42 | dst<<20), before self-loop removal/dedup */
void opma_rmat_raw(uint64_t seed, uint32_t scale, uint64_t n_edges,
                   uint32_t ta, uint32_t tab, uint32_t tabc, uint64_t *out);
/* remove self loops, sort, dedup; returns the new count */
uint64_t opma_dedup(uint64_t *keys, uint64_t n);
/* order by (mix64(seed ^ key), key) */
void opma_shuffle(uint64_t seed, uint64_t *keys, uint64_t n);

/* ---- CPU baseline: sorted-merge CSR rebuild per batch ---- */
typedef struct OCsr OCsr;
OCsr *ocsr_create(uint32_t num_vertices, int threads);
void ocsr_destroy(OCsr *c);
int ocsr_load(OCsr *c, const uint64_t *keys, uint64_t n);
int ocsr_insert(OCsr *c, const uint64_t *keys, uint64_t n);
int ocsr_delete(OCsr *c, const uint64_t *keys, uint64_t n);
uint64_t ocsr_num_edges(const OCsr *c);
const uint64_t *ocsr_edges(const OCsr *c);
const uint32_t *ocsr_row_offset(const OCsr *c);

#ifdef __cplusplus
}
#endif
#endif
