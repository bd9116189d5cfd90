/*
 * lpma.h -- C ABI of the GB300 LPMA (leveled packed memory array) engine.
 *
 * Drop-in boundary for the batched edge-update path of pkumod/LPMA.  Every
 * entry point takes plain pointers and sizes, returns an lpma_status_t and
 * never prints.  Device pointers are borrowed for the duration of the call
 * and read only.  Calls on one handle are ordered on the stream passed in;
 * different handles are independent.  (An update also runs part of its work
 * on a stream of the handle's own, forked from and joined back into the
 * caller's stream, so later work on that stream still follows all of it.)
 * Every call that returns a count or a host buffer synchronises with its
 * stream before returning.
 *
 * Key layout (reference rpma.cuh:43-50): a 64-bit key is
 *     src << 42 | dst << 20 | t
 * with src, dst < num_vertices <= 0x3FFFFE and t a 20-bit timestamp.  Every
 * vertex v owns a sentinel key v << 42 | 0x3FFFFEFFFFF that closes its row.
 * With LPMA_KEY_PAIR32 the caller passes src << 32 | dst instead and the
 * engine repacks it with t = 0.
 */
#ifndef LPMA_H
#define LPMA_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define LPMA_API __attribute__((visibility("default")))
#else
#define LPMA_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* same object as cudaStream_t; 0 is the legacy default stream */
typedef struct CUstream_st *lpma_stream_t;

typedef struct LpmaHandle LpmaHandle;

typedef enum {
    LPMA_OK = 0,
    LPMA_ERR_INVALID_ARGUMENT = 1, /* null handle/pointer, bad config */
    LPMA_ERR_INVALID_KEY = 2,      /* key out of range, sentinel delete, value 0xFF, expired insert */
    LPMA_ERR_OUT_OF_MEMORY = 3,
    LPMA_ERR_CUDA = 4,             /* a CUDA runtime call failed */
    LPMA_ERR_CAPACITY = 5,         /* tree height would exceed LPMA_MAX_HEIGHT */
    LPMA_ERR_INTERNAL = 6,         /* a device-side consistency check failed */
    LPMA_ERR_TIMEOUT = 7,          /* a bounded device-side wait gave up */
    LPMA_ERR_BUFFER_TOO_SMALL = 8,
    LPMA_ERR_SCRATCH_LIMIT = 9,    /* n above the fixed scratch of lpma_shuffle_static */
    LPMA_ERR_IO = 10               /* a file is missing, unreadable or malformed */
} lpma_status_t;

enum { LPMA_KEY_PACKED = 0, LPMA_KEY_PAIR32 = 1 };
/* LPMA_FLAG_CONCURRENT: the handle's calls may run while other handles'
 * calls run on other streams (a worker pool).  Its batch sort then uses
 * ordinary launches instead of the one cooperative launch, because two
 * cooperative grids that each hold part of the GPU could wait on each
 * other. */
/* LPMA_FLAG_GPMA: the handle stores the flat packed memory array of the
 * reference's gpma.cuh instead of the leveled tree of rpma.cuh (see
 * lpma_config_gpma). */
enum { LPMA_FLAG_CONCURRENT = 1, LPMA_FLAG_GPMA = 2 };
enum { LPMA_MAX_HEIGHT = 24 };

typedef struct {
    uint32_t segment_length;   /* slots per segment; 32 (rpma.cuh:1769) */
    uint32_t key_format;       /* LPMA_KEY_PACKED or LPMA_KEY_PAIR32 */
    uint32_t skip_rule;        /* 1: the reference's big-grain skip state machine (rpma.cuh:1609-1619) */
    uint32_t flags;            /* LPMA_FLAG_* */
    double density_lower_root; /* 0.42 (rpma.cuh:77) */
    double density_upper_root; /* 1.0 (rpma.cuh:78) */
} LpmaConfig;

typedef struct {
    uint32_t height_before, height_after;
    uint32_t n_ins_applied;    /* inserts of new keys */
    uint32_t n_upserts;        /* inserts of present keys: value overwritten in place */
    uint32_t n_del_applied;    /* deletes of present keys */
    uint32_t n_noop;           /* absent-key deletes and in-batch duplicates */
    uint32_t root_executed;    /* the whole-array window absorbed updates */
    uint32_t eager_levelup;    /* a level was added after the root absorbed */
    uint32_t overflow;         /* updates were left after the root */
    uint32_t rebuilt;          /* full rebuild at a new height */
    uint32_t levelup_path;     /* overflow absorbed by adding one level */
    uint32_t fill_empty;       /* an empty segment forced a full redistribution */
    uint64_t windows_single;   /* single-segment rebalance windows executed */
    uint64_t windows_small;    /* rebalance windows of <= 32 segments executed (incl. single) */
    uint64_t windows_big;      /* larger windows (tile grain) executed */
    uint64_t slots_rewritten;  /* slots covered by executed windows (incl. rebuild) */
    uint64_t slots_small;      /* of which in windows of <= 32 segments */
    uint64_t num_items;        /* keys stored after the call, sentinels included */
    uint64_t h2d_bytes;        /* host->device bytes the call copied (inputs, control) */
    uint64_t d2h_bytes;        /* device->host bytes the call copied (status blocks) */
    uint32_t sort_passes;      /* digit passes the batch sort ran: one per byte that varies over the batch,
                                  or, for the cooperative sort, one per 9-bit digit window */
    uint32_t levelup;          /* update_rpma's return value (rpma.cuh:1646-1653, 1662-1668): 1 when updates
                                  reached the root level, i.e. the root window absorbed them (root_executed,
                                  whether or not a level was added) or they overflowed it (overflow, whatever
                                  the new height, a lower one after a rebuild included) */
} LpmaStats;

/* defaults that reproduce the reference: 32 / 0.42 / 1.0 / skip rule on */
LPMA_API lpma_status_t lpma_config_default(LpmaConfig *cfg);

/* ---- GPMA mode (gpma.cuh) ----
 * A handle created with lpma_config_gpma's configuration (flags =
 * LPMA_FLAG_GPMA) holds the reference's flat GPMA instead of the leveled
 * array: one array of size slots (a power of two) cut into segments of
 * 2^(fls(fls(size)) - 1) slots, density bounds trunc(density_lower_root *
 * len) and len per level (0.15 / 1.0, gpma.cuh:52-55), a copying resize to
 * the smallest power of two that holds the items (resize_gpma,
 * gpma.cuh:694-718) and a whole-array respread for batches of 5,000,000 new
 * keys or more (significant_insert, gpma.cuh:720-744).  Keys are
 * src << 32 | dst with src, dst < num_vertices <= 0xFFFFFFFE; the sentinel
 * of vertex v is v << 32 | 0xFFFFFFFF (value 1) and two guards of key
 * 0xFFFFFFFFFFFFFFFE (value 1) stay at the end (init_csr_gpma / init_gpma,
 * gpma.cuh:818-847).  lpma_update inserts (values default 1) and deletes
 * (handle_del_mod, gpma.cuh:162-175: a present key is tombstoned in place,
 * value 0xFF, and leaves at the next rebalance of its window; inserting a
 * tombstoned key brings it back in place); thres must be 0.  The first
 * state after lpma_create is the one update_gpma's resize path gives for
 * the sentinels and guards (the reference's first update reads past its
 * 4-slot initial array).  lpma_export_sorted returns the live keys
 * (sentinels included, guards and tombstones left out), lpma_export_layout
 * the flat array with sentinel_slots[v] = row_offset[v + 1], lpma_info the
 * tree height.  The CSR view, the read paths, lpma_set_flags and the
 * batched update return LPMA_ERR_INVALID_ARGUMENT for these handles. */
LPMA_API lpma_status_t lpma_config_gpma(LpmaConfig *cfg);

/* The GPMA view analytics read (gpma.cuh:341-344, 471-474): device
 * pointers, valid until the next update, to row_offset (num_vertices + 1
 * entries; row_offset[0] = 0 and row_offset[v + 1] is the slot of v's
 * sentinel, so row v's keys lie in slots row_offset[v] .. row_offset[v + 1]
 * skipping empty slots, value-0xFF tombstones and, for v > 0, the slot
 * row_offset[v] itself), the key and value arrays (*size slots), and the
 * segment length and height.  LPMA_ERR_INVALID_ARGUMENT for a leveled
 * handle. */
LPMA_API lpma_status_t lpma_gpma_view(LpmaHandle *h, const uint32_t **row_offset, const uint64_t **keys,
                                      const uint8_t **values, uint64_t *size, uint32_t *segment_length,
                                      uint32_t *height);

/* Replaces init_csr_rpma(RPMA&, SIZE_TYPE row_num) (rpma.cuh:1808-1824):
 * empty height-0 array, then the num_vertices sentinel keys inserted through
 * the update path. */
LPMA_API lpma_status_t lpma_create(const LpmaConfig *cfg, uint32_t num_vertices, lpma_stream_t stream,
                          LpmaHandle **out);

/* Bulk load = one update of all edges, the pattern of test_csr.cu:49-55 and
 * init_csr_rpma's update_rpma(row_wall) (rpma.cuh:1823).  d_vals may be NULL
 * (every value 1, test_update_rpma.cu:72). */
LPMA_API lpma_status_t lpma_build(LpmaHandle *h, const uint64_t *d_keys, const uint8_t *d_vals, size_t n,
                         lpma_stream_t stream);

/* Replaces bool update_rpma(RPMA&, DEV_VEC_KEY& keys, DEV_VEC_VALUE& values,
 * DEV_VEC_KEY& edgequery, DEV_VEC_VALUE& flag, SIZE_TYPE thres)
 * (rpma.cuh:1549-1718), extended with deletes (GPMA semantics,
 * gpma.cuh:162-175).  The batch is a set of updates: an insert of a present
 * key overwrites its value, a delete of an absent key is a no-op, a key
 * both inserted and deleted in one batch ends up present.  Keys with
 * t < thres are expired (removed at the next rebalance of their window, as
 * in the reference); inserting a key with t < thres is rejected.  The
 * inputs are not modified (the reference sorts them in place).  stats may
 * be NULL; it is filled when the call returns. */
LPMA_API lpma_status_t lpma_update(LpmaHandle *h, const uint64_t *d_ins, const uint8_t *d_ins_vals, size_t n_ins,
                          const uint64_t *d_del, size_t n_del, uint32_t thres, lpma_stream_t stream,
                          LpmaStats *stats);

/* Same as lpma_update with host buffers: copies in, updates, fills stats.
 * The end-to-end entry point for callers without device memory. */
LPMA_API lpma_status_t lpma_update_host(LpmaHandle *h, const uint64_t *h_ins, const uint8_t *h_ins_vals, size_t n_ins,
                               const uint64_t *h_del, size_t n_del, uint32_t thres, lpma_stream_t stream,
                               LpmaStats *stats);

/* Replaces to_csr_rpma(RPMA&, DEV_VEC_SIZE& row_offset, DEV_VEC_SIZE& col_index)
 * (rpma.cuh:2249-2295).  Device arrays owned by the handle, valid until the
 * next mutating call: row_offset has num_vertices + 1 entries with one extra
 * slot per row for its sentinel (row length = row_offset[v+1] -
 * row_offset[v] - 1, col_index[row_offset[v+1] - 1] == v); col_index has
 * *nnz entries (dst for edges, src for sentinels); values has the stored
 * value for edges and 0xFF for sentinels. */
LPMA_API lpma_status_t lpma_csr_view(LpmaHandle *h, const uint32_t **row_offset, const uint32_t **col_index,
                            const uint8_t **values, size_t *nnz, lpma_stream_t stream);

/* Copy-out form of to_csr_rpma, which fills caller-owned vectors: writes the
 * same three arrays into caller buffers (host or device memory; cap is the
 * capacity of col_index and values, row_offset needs num_vertices + 1).
 * *nnz receives the entry count.  Synchronises with the stream. */
LPMA_API lpma_status_t lpma_to_csr(LpmaHandle *h, uint32_t *row_offset, uint32_t *col_index, uint8_t *values,
                                   size_t cap, size_t *nnz, lpma_stream_t stream);

/* Replaces get_data_rpma(RPMA&, KEY_PTR&, VALUE_PTR&) (rpma.cuh:1735-1761):
 * every stored key (sentinels included) in sorted order into caller host
 * buffers of capacity cap; *n receives the count.  h_vals may be NULL. */
LPMA_API lpma_status_t lpma_export_sorted(LpmaHandle *h, uint64_t *h_keys, uint8_t *h_vals, size_t cap, size_t *n,
                                 lpma_stream_t stream);

/* Physical layout for parity checks: the reference's level arrays laid end
 * to end (level i at slot 32*(2^i - 1)), empty slots ~0, values of empty
 * slots 0.  *height receives the tree height; the slot count is
 * 32*(2^(height+1) - 1).  Also the per-vertex sentinel slots (the
 * reference's csr_idx/csr_lane pair as one physical slot index). */
LPMA_API lpma_status_t lpma_export_layout(LpmaHandle *h, uint64_t *h_keys, uint8_t *h_vals, size_t cap_slots,
                                 uint32_t *sentinel_slots, size_t cap_vertices, uint32_t *height,
                                 lpma_stream_t stream);

LPMA_API lpma_status_t lpma_info(const LpmaHandle *h, uint32_t *height, uint64_t *num_items, uint32_t *num_vertices);

/* Replaces destroy_rpma (rpma.cuh:1720-1732). */
LPMA_API lpma_status_t lpma_destroy(LpmaHandle *h);

LPMA_API const char *lpma_status_string(lpma_status_t s);

/* ---- read paths: they read the structure in place (no CSR view is built)
 * and order after earlier work on `stream` (use the update stream). ---- */

/* Replaces query_rpma(RPMA&, DEV_VEC_SIZE& srcs, DEV_VEC_KEY& constraints,
 * offset, len, edgelist, v_list) (rpma.cuh:1974-2036): for query i, the
 * neighbours of d_srcs[i] whose timestamp t has lb <= t <= ub, where
 * d_windows[i] = lb << 32 | ub, in key order (dst ascending, then t).
 * d_offsets (n + 1 device entries) receives the start of each list (its
 * last entry the total), d_nbrs / d_vals (device, cap entries) the neighbour
 * ids and values, *total the number of neighbours.  With d_nbrs NULL only
 * the offsets and the total are produced; with total > cap the call returns
 * LPMA_ERR_BUFFER_TOO_SMALL after the offsets.  The reference sorts the
 * caller's queries and returns the lists in that order with sentinel markers
 * between them; here the lists follow the caller's order and hold
 * neighbours only.  A query with src >= V gets an empty list.  Synchronises
 * the stream once, to read the total. */
LPMA_API lpma_status_t lpma_query_neighbors(LpmaHandle *h, const uint32_t *d_srcs, const uint64_t *d_windows, size_t n,
                                            uint32_t *d_offsets, uint32_t *d_nbrs, uint8_t *d_vals, size_t cap,
                                            size_t *total, lpma_stream_t stream);

/* Edge query (check_edge_kernel rpma.cuh:2040-2066; result check
 * test.cu:46-62): d_counts[i] = number of stored keys (src, dst, t') for
 * query key (src, dst, t) with t - window <= t' <= t.  window = t = 0xFFFFF
 * counts every timestamp, as check_edge_kernel (which ignores time) does.
 * src >= V or dst >= 0x3FFFFE counts 0.  Asynchronous. */
LPMA_API lpma_status_t lpma_edge_query(LpmaHandle *h, const uint64_t *d_keys, size_t n, uint32_t window,
                                       uint32_t *d_counts, lpma_stream_t stream);

/* Directed BFS over the stored edges from d_sources, the analytics step of
 * test.cu:168-183 (nvGRAPH BFS over the exported CSR): d_dist (V int32,
 * device) receives hop counts from the nearest source, INT32_MAX where
 * unreached (nvGRAPH's convention).  max_depth bounds the levels (0: no
 * bound; 2 for a 2-hop BFS from many seeds).  levels / reached (may be
 * NULL) receive the levels expanded and the vertices reached.  Synchronises
 * once per level. */
LPMA_API lpma_status_t lpma_bfs(LpmaHandle *h, const uint32_t *d_sources, size_t n_sources, uint32_t max_depth,
                                int32_t *d_dist, uint32_t *levels, uint64_t *reached, lpma_stream_t stream);

/* PageRank over the stored edges (test_algos.cu:44-90 runs nvGRAPH's on the
 * CSR), in f64: from rank = 1/V, `iterations` times
 *   rank[v] = (1 - alpha)/V + alpha * (sum over edges u->v of rank[u]/outdeg(u) + dangling/V)
 * where dangling sums the rank of vertices without out-edges.  d_rank: V
 * doubles on the device.  Asynchronous. */
LPMA_API lpma_status_t lpma_pagerank(LpmaHandle *h, double alpha, uint32_t iterations, double *d_rank,
                                     lpma_stream_t stream);

/* After LPMA_ERR_INTERNAL: the device check that failed (1 multi-segment
 * window size, 2 big-window item count, 3 single-segment window size, 4/5
 * big-window staging bounds), 0 when none. */
LPMA_API lpma_status_t lpma_error_detail(const LpmaHandle *h, uint32_t *site);

/* Change the handle's LPMA_FLAG_* bits; no call on the handle may be in
 * flight. */
LPMA_API lpma_status_t lpma_set_flags(LpmaHandle *h, uint32_t flags);

/* ---- one update per graph for many graphs at once ----
 * The update batches of many graphs go through shared launches: one launch
 * per step of the update front (status reset, pack, sort, locate, compact,
 * plan) covers every graph, instead of a dozen launches per graph.  Each
 * graph then goes on as after its own front (window executors, root,
 * overflow, resize), so each graph ends exactly as lpma_update would leave
 * it.  Batches with an expiry threshold, above 131,072 keys, or whose
 * first level loop allows windows of 2^9+ segments take lpma_update inside
 * the call.  A graph may appear once per call; its buffers are the handle's
 * own, the batcher keeps the shared tables between calls.  stats and
 * status (NULL or n entries) receive each graph's result; the return value
 * is the first error, or LPMA_OK.  Synchronises the stream once.  (No
 * counterpart in the reference: its drivers update one graph at a time.) */
typedef struct LpmaBatcher LpmaBatcher;
typedef struct {
    const uint64_t *ins;       /* device */
    const uint8_t *ins_vals;   /* device, may be NULL */
    size_t n_ins;
    const uint64_t *del;       /* device */
    size_t n_del;
    uint32_t thres;
    uint32_t reserved;
} LpmaBatch;
LPMA_API lpma_status_t lpma_batcher_create(LpmaBatcher **out);
LPMA_API lpma_status_t lpma_batcher_destroy(LpmaBatcher *b);
LPMA_API lpma_status_t lpma_update_batch(LpmaBatcher *b, LpmaHandle *const *graphs, const LpmaBatch *batches,
                                         size_t n, lpma_stream_t stream, LpmaStats *stats, lpma_status_t *status);

/* ---- autotuner: the batch-sort algorithm per batch-size bucket ----
 * The update front sorts each batch with one of five algorithms ("tiers"):
 * 1 one CTA through shared memory (<= 2048 keys), 2 tiles of 2048 keys
 * sorted by all-pairs rank over many CTAs, then placed by binary searches
 * across the tiles (<= 16384), 3 register-sorted tiles plus
 * merge-path rounds (<= 2^24), 4 one cooperative launch for all digit
 * passes (handles without LPMA_FLAG_CONCURRENT), 5 three launches per digit
 * pass.  All give the same order.  lpma_autotune times every usable tier on
 * seeded batches of 2^b keys for b = 11 .. ceil(log2 max_keys), for both
 * sort modes (concurrent 0: cooperative launches allowed, 1: not), keeps
 * the fastest in a process-wide table that later update calls read, and
 * reports one entry per (b, mode) (median microseconds per tier; 0 where a
 * tier does not apply).  lpma_tune_set / lpma_tune_get read or override one
 * entry (tier 0: the built-in cutovers).  Batches of 2^(b-1)+1 .. 2^b keys
 * use entry b.  (The reference's cut-over is fixed: rebalance_batch,
 * rpma.cuh:1214-1256.) */
typedef struct {
    uint32_t log2_keys;
    uint32_t concurrent;
    uint32_t tier;
    uint32_t reserved;
    float us[6];
} LpmaTuneEntry;
/* Test setting of the cooperative batch sort's grid barrier on the current
 * device, for tests of its give-up path: every barrier wait of that sort
 * polls at most poll_limit times (0 restores the built-in limit of 2^22)
 * and, with unreachable set, waits for an arrival count that never comes,
 * so every wait gives up.  A sort whose wait gave up leaves the structure
 * unchanged and its update returns LPMA_ERR_TIMEOUT; the handle stays
 * usable.  Synchronous; no update may be in flight on the device. */
LPMA_API lpma_status_t lpma_debug_sort_barrier(uint32_t poll_limit, int unreachable);

/* Test setting of the executor of 5..32-segment windows on the current
 * device, for tests of its give-up path: with give_up set, the bounded wait
 * for a window's bulk copies into shared memory gives up at once; the warp
 * then records LPMA_ERR_TIMEOUT in the handle's sticky error word, waits
 * (bounded) for its copies in flight and stops, so the next call on that
 * handle returns LPMA_ERR_TIMEOUT.  0 restores the normal wait.
 * Synchronous; no update may be in flight on the device. */
LPMA_API lpma_status_t lpma_debug_exec_wait(int give_up);

LPMA_API lpma_status_t lpma_autotune(uint32_t max_keys, lpma_stream_t stream, LpmaTuneEntry *out, size_t cap,
                                     size_t *n_out);
LPMA_API lpma_status_t lpma_tune_set(uint32_t log2_keys, uint32_t concurrent, uint32_t tier);
LPMA_API lpma_status_t lpma_tune_get(uint32_t log2_keys, uint32_t concurrent, uint32_t *tier);

/* ---- executor grain cut-overs per batch-size bucket ----
 * After planning, every maximal window goes to one of four executors by its
 * segment count: 1 segment, up to max_segs_group (8-lane-group executor,
 * 1..4, default 4), up to max_segs_shared (shared-memory executor,
 * max_segs_group..32, default 32), larger (the tile grain: gather and
 * spread through the alternate array).  The reference fixes its cut-over
 * at 1024 slots (rebalance_batch, rpma.cuh:1214-1256).  No setting changes
 * the layout an update produces, only its speed.  Entry log2_keys serves
 * batches of 2^(log2_keys-1)+1 .. 2^log2_keys keys, process-wide, for
 * lpma_update and lpma_update_host on leveled handles (lpma_update_batch
 * and GPMA handles keep the defaults); lpma_grain_set(b, 0, 0) restores the
 * defaults, lpma_grain_get reports the values in effect. */
typedef struct {
    uint32_t max_segs_group;
    uint32_t max_segs_shared;
    float us_median; /* one insert plus one delete of the batch, CUDA events on the stream */
    uint32_t reserved;
} LpmaGrainTime;
LPMA_API lpma_status_t lpma_grain_set(uint32_t log2_keys, uint32_t max_segs_group, uint32_t max_segs_shared);
LPMA_API lpma_status_t lpma_grain_get(uint32_t log2_keys, uint32_t *max_segs_group, uint32_t *max_segs_shared);
/* Times six grain settings ({4, 2} x {32, 16, 8}) on the caller's own leveled
 * handle: rounds of lpma_update inserting the n device keys and lpma_update
 * deleting them again, the settings taking turns (one warm-up round each,
 * then `reps` timed), and keeps the fastest in the entry of n's bucket when
 * it is at least 3% faster than the defaults (else the defaults).  The
 * settings only differ where the handle's windows do: tune on a handle in
 * the state the updates will meet.  The keys must be absent
 * from the handle: a batch holding a stored key is refused
 * (LPMA_ERR_INVALID_ARGUMENT) before anything changes.  Afterwards the
 * handle stores the same set (its layout is another valid one of it).
 * Writes one LpmaGrainTime per setting timed to out (up to cap) and their
 * count to *n_out.  Blocks the calling thread; not for GPMA handles. */
LPMA_API lpma_status_t lpma_autotune_grain(LpmaHandle *h, const uint64_t *d_keys, size_t n, uint32_t reps,
                                           lpma_stream_t stream, LpmaGrainTime *out, size_t cap, size_t *n_out);

/* Device bytes the handle holds (structure, scratch, views). */
LPMA_API lpma_status_t lpma_memory_bytes(const LpmaHandle *h, uint64_t *bytes);

/* Grow the current device's update memory pool (the stream-ordered pool the
 * handles' capacity and batch buffers come from) to hold at least `bytes`
 * more: the bytes are allocated on `stream` and freed again, and the pool
 * keeps them.  A server calls this before taking traffic, so that a graph
 * growing a level under load is served from memory the pool already holds
 * instead of mapping new memory then.  Synchronous; LPMA_ERR_OUT_OF_MEMORY
 * if the device cannot provide them. */
LPMA_API lpma_status_t lpma_memory_reserve(uint64_t bytes, lpma_stream_t stream);

/* ---- request pool: many resident graphs, batched or served ----
 * Worker threads, each with its own stream, run submitted requests.
 * Requests on different graphs run concurrently; requests on one graph run
 * one at a time in submission order.  A request is admitted while the
 * resident graphs plus the scratch of the requests in flight fit
 * hbm_budget_bytes (0: no budget; one request is always admitted when none
 * runs).  Graphs given to a pool should be created with
 * LPMA_FLAG_CONCURRENT.  The caller owns each LpmaRequest and keeps it
 * valid until done is set; its timestamps are host steady-clock
 * nanoseconds.  (The reference has no counterpart: its drivers update one
 * graph at a time.) */
typedef struct LpmaPool LpmaPool;
enum { LPMA_REQ_UPDATE = 0, LPMA_REQ_NEIGHBORS = 1, LPMA_REQ_BFS = 2, LPMA_REQ_EDGE_QUERY = 3 };
typedef struct {
    uint32_t kind;              /* LPMA_REQ_* */
    uint32_t host_inputs;       /* update: 1 when keys0/vals0/keys1 are host memory */
    LpmaHandle *graph;
    const uint64_t *keys0;      /* update: inserts; edge query: query keys */
    const uint8_t *vals0;       /* update: insert values (NULL: 1) */
    size_t n0;
    const uint64_t *keys1;      /* update: deletes */
    size_t n1;
    const uint32_t *vertices;   /* neighbours: query sources; BFS: sources */
    const uint64_t *windows;    /* neighbours: lb << 32 | ub per query */
    size_t nv;
    uint32_t thres;             /* update: expiry threshold; edge query: window */
    uint32_t max_depth;         /* BFS */
    uint32_t *out_u32;          /* neighbours: offsets (nv + 1); edge query: counts */
    uint32_t *out_nbrs;         /* neighbours */
    uint8_t *out_vals;          /* neighbours */
    int32_t *out_dist;          /* BFS: V entries */
    size_t cap;                 /* neighbours: capacity of out_nbrs / out_vals */
    /* filled by the pool */
    lpma_status_t status;
    uint32_t levels;            /* BFS */
    uint64_t reached;           /* BFS: vertices reached; neighbours: total */
    LpmaStats stats;            /* update */
    uint64_t t_submit_ns, t_start_ns, t_end_ns;
    /* where a request's service time went: t_call_ns is when the library
     * call returned (its host part, launches and host waits inside the call
     * included); device_ms the interval between two events recorded on the
     * worker's stream before and after the request's work (GPU time plus
     * any gap while the host had not yet launched); pool_growth_bytes how
     * much the update memory pool's reserved memory grew meanwhile (new
     * device memory mapped during the request) */
    uint64_t t_call_ns;
    uint64_t pool_growth_bytes;
    float device_ms;
    volatile uint32_t done;
} LpmaRequest;

LPMA_API lpma_status_t lpma_pool_create(uint32_t n_workers, uint64_t hbm_budget_bytes, LpmaPool **out);
LPMA_API lpma_status_t lpma_pool_submit(LpmaPool *p, LpmaRequest *req);
/* Submits reqs[0..n) (a contiguous array the caller keeps valid until all
 * are done) in array order, under one lock. */
LPMA_API lpma_status_t lpma_pool_submit_many(LpmaPool *p, LpmaRequest *reqs, size_t n);
LPMA_API lpma_status_t lpma_pool_wait(LpmaPool *p, LpmaRequest *req);
LPMA_API lpma_status_t lpma_pool_drain(LpmaPool *p);
LPMA_API lpma_status_t lpma_pool_destroy(LpmaPool *p);

/* ---- edgelist files (README.md:9-20) ---- */

/* read_edgelist (test_update_rpma.cu:175-192) and
 * read_edgelist_and_timestamps (test.cu:191-221): "N E" then E lines
 * "src dst"; timestamps_path (may be NULL) holds E timestamps, one per
 * edge.  Writes keys src << 42 | dst << 20 | t into h_keys (host).  With
 * cap < E it returns LPMA_ERR_BUFFER_TOO_SMALL after setting *num_vertices
 * and *num_edges (h_keys may then be NULL).  LPMA_ERR_IO for a missing or
 * malformed file, an id >= N, an id >= 0x3FFFFE or a timestamp >= 2^20. */
LPMA_API lpma_status_t lpma_read_edgelist(const char *path, const char *timestamps_path, uint64_t *h_keys, size_t cap,
                                          uint32_t *num_vertices, size_t *num_edges);

/* read_queries (test.cu:223-241): "Q" then Q lines "src lb ub"; writes
 * h_srcs[i] = src and h_windows[i] = lb << 32 | ub (host).  Sizing and
 * errors as lpma_read_edgelist. */
LPMA_API lpma_status_t lpma_read_queries(const char *path, uint32_t *h_srcs, uint64_t *h_windows, size_t cap,
                                         size_t *num_queries);

/* ---- synthetic workload (device generator; the same integer arithmetic
 * as the CPU workload generator used by the tests) ---- */

/* Seeded R-MAT keys src << 42 | dst << 20 with thresholds floor(p * 2^32):
 * writes 2^scale * edge_factor raw edges into d_out (capacity cap), removes
 * self loops and duplicates, sorts; *n_out receives the count. */
LPMA_API lpma_status_t lpma_gen_rmat(uint64_t seed, uint32_t scale, uint32_t edge_factor, uint32_t ta, uint32_t tab,
                            uint32_t tabc, uint64_t *d_out, size_t cap, size_t *n_out, lpma_stream_t stream);

/* Reorders d_keys by (mix64(seed ^ key), key). */
LPMA_API lpma_status_t lpma_shuffle(uint64_t seed, uint64_t *d_keys, size_t n, lpma_stream_t stream);

/* ---- shuffle without allocation (no counterpart in the reference) ----
 *
 * Same result as lpma_shuffle, bit for bit, for n <= LPMA_SHUFFLE_STATIC_MAX_KEYS,
 * but it allocates nothing: no cudaMalloc, no cudaFree, no allocating
 * library call.  It is meant for callers that must not allocate or free
 * device memory while they run -- a serving loop that has handed the whole
 * HBM budget to resident graphs and cannot risk an out-of-memory failure in
 * mid-request, or a latency-critical path where cudaFree's implicit device
 * synchronisation would stall every stream.
 *
 * Its scratch is one fixed device array inside the library,
 * LPMA_SHUFFLE_STATIC_SCRATCH_BYTES long (about 2.5 MB), enough for
 * LPMA_SHUFFLE_STATIC_MAX_KEYS keys.  A larger n returns
 * LPMA_ERR_SCRATCH_LIMIT before anything is launched, with d_keys untouched.
 * No part of the scratch has to hold zeros on entry: the call clears what it
 * counts in and writes every other byte before reading it.
 *
 * The first call on each device does a one-time set-up with that device
 * current (it looks up the array's device address and sets kernel
 * attributes); make that first call before any stream capture begins.
 *
 * Every call in the process shares the one array per device, so calls whose
 * GPU work overlaps -- on different streams, or from different threads --
 * race on it and give wrong results.  Issue them on one stream, or order
 * them.  The call is asynchronous on `stream`.  While per-kernel profiling
 * (lpma_prof_enable) is on, the profiler creates CUDA events for this call's
 * launches too; keep it off where nothing may be allocated. */
enum { LPMA_SHUFFLE_STATIC_MAX_KEYS = 65536, LPMA_SHUFFLE_STATIC_SCRATCH_BYTES = 2621440 };
LPMA_API lpma_status_t lpma_shuffle_static(uint64_t seed, uint64_t *d_keys, size_t n, lpma_stream_t stream);

/* Per-kernel timing for profiling: while enabled, each kernel launch is
 * bracketed by CUDA events on its stream.  lpma_prof_report writes one line
 * "name launches total_ms" per kernel name into buf, clears the record and
 * returns the full report length. */
LPMA_API lpma_status_t lpma_prof_enable(int on);
LPMA_API size_t lpma_prof_report(char *buf, size_t cap);

/* Number of kernels this library launched since load (a counter for benches). */
LPMA_API uint64_t lpma_kernel_launches(void);

#ifdef __cplusplus
}
#endif
#endif
