// Launchers for the update-path and view kernels (definitions in update.cu
// and view.cu).  Host orchestration lives in abi.cu.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "lpma_common.cuh"
#include "prims.cuh"

namespace lpma {

struct UpdList {  // compacted, key-sorted update list
    uint64_t *key;
    uint8_t *val;
    uint8_t *kind;
    uint32_t *seg;  // linear segment located for the key
    uint32_t *ip;   // exclusive count of inserts before each entry (n+1 entries)
};

struct Geo {  // one tree geometry in HBM
    uint64_t *keys;
    uint8_t *vals;
    uint32_t H;
};

// validate + pack both input arrays into one key/payload array; payload bits
// 0-7 = value, bit 8 = delete.  Also clears the planner bitmap (bitmap_words
// 32-bit words) for the call's first plan, the locate's chunk-group totals
// (sup_words words) and the cooperative sort's barrier counter (sort_bar,
// may be null), and prefetches the first pf_segs entries of the segment
// bounds (fl) and counts (cnt) into L2.
void launch_pack(const uint64_t *ins, const uint8_t *ins_vals, uint32_t n_ins, const uint64_t *del,
                 uint32_t n_del, uint32_t V, uint32_t thres, uint32_t key_format, int internal,
                 uint64_t *keys_out, uint16_t *pay_out, DevStatus *st, uint32_t *bitmap, uint32_t bitmap_words,
                 const ulonglong2 *fl, const uint8_t *cnt, uint64_t pf_segs, uint32_t *sup, uint32_t sup_words,
                 uint32_t *sort_bar, cudaStream_t s);

// words of the locate's chunk-group totals for n keys (an (nn, inserts)
// pair per 64 chunks of 256 keys)
inline uint32_t sup_words_for(uint64_t n) { return 2 * (uint32_t)((n + 256 * 64 - 1) / (256 * 64)) + 2; }

// the pack kernel's entry (graph replays update its input pointers)
const void *pack_kernel_fn();

// per-segment live counts (key present and t >= thres) + their total
void launch_live_counts(const uint64_t *keys, uint32_t H, uint32_t thres, uint8_t *cnt_live, DevStatus *st,
                        cudaStream_t s);

// collapse duplicates, locate every key, membership test against its
// segment, upsert/tombstone in place; per-256-block counts of kept entries
// and inserts, and their totals per 64 blocks added into sup (cleared by
// the pack).  The sorted batch is (k0, p0) or (k1, p1), as sort_pairs_dev
// left it.
void launch_resolve_locate(const uint64_t *k0, const uint16_t *p0, const uint64_t *k1, const uint16_t *p1, uint32_t n,
                           SortMask mask, Geo g, const ulonglong2 *fl, uint32_t thres, uint8_t *kind, uint32_t *seg,
                           uint32_t *blk_nn, uint32_t *blk_ins, uint32_t *sup, DevStatus *st, cudaStream_t s);

// the update list: each 256-block's offsets from the group totals and the
// block counts before it; the last block writes n_u, n_ins, n_del and the
// end of ip
void launch_compact(const uint64_t *k0, const uint16_t *p0, const uint64_t *k1, const uint16_t *p1, SortMask mask,
                    const uint8_t *kind, const uint32_t *seg, uint32_t n, uint32_t *blk_nn, uint32_t *blk_ins,
                    const uint32_t *sup, UpdList u, DevStatus *st, cudaStream_t s);

// locate only (second loop after a level-up): u.seg from u.key
void launch_relocate(UpdList u, uint32_t n, Geo g, const ulonglong2 *fl, cudaStream_t s);

// keep only updates flagged pending; rebuilds ip
void launch_compact_pending(const UpdList in, const uint8_t *pend, uint32_t n, UpdList out, uint32_t *blk_nn,
                            uint32_t *blk_ins, DevStatus *st, cudaStream_t s);

// test setting of the 5..32-segment executor's bulk-copy wait (its first
// wait per window gives up at once when give_up is set), current device
cudaError_t set_exec_wait_debug(uint32_t give_up);

// count-only planner: per segment with updates, the first level whose
// window passes the density test; maximal windows go to small/big lists.
// pub: when set, the planner's last CTA writes the status block into this
// pinned host mirror and then sets its `published` word.
void launch_plan(const UpdList u, uint32_t n_cap, const uint8_t *cnt, const uint32_t *P, int use_P,
                 uint64_t total_live, const unsigned long long *total_live_dev, uint32_t H, const Tables &tb,
                 uint32_t *bitmap, Window *cand, Window *single, Window *small4, Window *small, Window *big,
                 uint8_t *pend, DevStatus *st, cudaStream_t s, DevStatus *pub = nullptr);

// in-place executors for windows of <= 32 segments: the single-segment
// list (DevStatus::n_single), and in one launch the windows of 2..4
// segments (n_small4) and of 5..32 segments (n_small).  guarded: launched
// before the host has read the plan (the caps an upper bound), the executor
// does nothing when the plan overflowed or the batch was rejected.
void launch_exec_single(const Window *w, uint32_t n_cap, Geo g, uint8_t *cnt, ulonglong2 *fl, uint32_t *sent,
                        uint32_t V, const UpdList u, uint32_t thres, DevStatus *st, cudaStream_t s,
                        bool guarded = false);
void launch_exec_multi(const Window *w4, uint32_t cap4, const Window *w32, uint32_t cap32, Geo g, uint8_t *cnt,
                       ulonglong2 *fl, uint32_t *sent, uint32_t V, const UpdList u, uint32_t thres, DevStatus *st,
                       cudaStream_t s, bool guarded = false);

// adds to *count how many of the n keys (key_format as lpma_update's) the
// tree stores, live or tombstoned; read only
void launch_count_present(const uint64_t *keys, uint32_t n, uint32_t key_format, Geo g, const ulonglong2 *fl,
                          uint32_t *count, cudaStream_t s);

// per-segment counts for the tile grain: qi/qd from the update list
void launch_seg_update_counts(const UpdList u, uint32_t n_cap, uint32_t *qi, uint32_t *qd, const DevStatus *st,
                              cudaStream_t s);
// PQ / US: exclusive prefixes over the segments of q = kept + ins - del and
// qn = ins + del, the totals at [nseg]; tmp holds ceil(nseg / 2048) words
void launch_tile_prefix(const uint8_t *cnt, const uint8_t *cnt_live, const uint32_t *qi, const uint32_t *qd,
                        uint64_t nseg, uint32_t *PQ, uint32_t *US, uint64_t *tmp, cudaStream_t s);
inline size_t tile_prefix_tmp_words(uint64_t nseg) { return (size_t)((nseg + 2047) / 2048) + 1; }

struct TileJob {      // one window of more than 32 segments, or a rebuild
    uint32_t sa, sf;  // source linear segment range
    uint32_t da, df;  // destination linear segment range
    uint32_t m;       // items
    uint32_t stile0;  // first 32-segment source tile of this job
    uint32_t dtile0;  // first 32-segment destination tile of this job
    uint32_t pad;
};
// big windows and rebuilds: gather the merged items into M (rank order),
// then spread them over the destination geometry
void launch_exec_big(const TileJob *jobs, uint32_t njobs, uint32_t stiles, uint32_t dtiles, Geo src,
                     const uint32_t *PQ, const uint32_t *US, const UpdList u, uint32_t n_upd, uint32_t thres,
                     uint64_t *Mk, uint8_t *Mv, uint64_t m_cap, Geo dst, uint8_t *cnt_d, ulonglong2 *fl_d,
                     uint32_t *sent, uint32_t V, DevStatus *st, cudaStream_t s);

// The big windows (n, count known on the host) as tile jobs in order of
// their first segment, built on the device: the window list is sorted by
// position in the scratch arrays, then one CTA scans the tile counts.
void launch_big_jobs(const Window *wbig, uint32_t n, uint64_t *kscratch, uint64_t *kscratch2, uint16_t *pscratch,
                     uint16_t *pscratch2, SortScratch &ss, TileJob *jobs, cudaStream_t s);

// one job written from the kernel argument (no host staging, no implicit
// synchronisation of a pageable copy)
void launch_set_job(TileJob *jobs, const TileJob &j, cudaStream_t s);

// new level: cnt re-index (old s -> 2s+1), empty leaves
void launch_levelup_cnt(const uint8_t *cnt_old, uint8_t *cnt_new, uint32_t H_old, cudaStream_t s);
void launch_check_empty_level(const uint8_t *cnt, uint32_t H, DevStatus *st, cudaStream_t s);
void launch_sum_cnt(const uint8_t *cnt, uint64_t nseg, DevStatus *st, cudaStream_t s);

// view
void launch_csr_fill(Geo g, const uint8_t *cnt, const uint32_t *P, uint32_t *row_offset, uint32_t *col_index,
                     uint8_t *values, uint64_t *export_keys, uint8_t *export_vals, cudaStream_t s);

// generators
void launch_sentinels(uint32_t V, uint64_t *keys, uint8_t *vals, cudaStream_t s);
void launch_rmat(uint64_t seed, uint32_t scale, uint64_t n, uint32_t ta, uint32_t tab, uint32_t tabc, uint64_t *out,
                 cudaStream_t s);
void launch_hash_keys(uint64_t seed, const uint64_t *keys, uint64_t *hash, uint64_t n, cudaStream_t s);
void launch_unique_flags(const uint64_t *keys, uint64_t n, uint32_t *flags, cudaStream_t s);
void launch_scatter_flags(const uint64_t *keys, const uint32_t *pos, const uint32_t *flags, uint64_t n,
                          uint64_t *out, cudaStream_t s);


// ---- read paths over the PMA (query.cu)
void launch_nbr_count(const uint32_t *srcs, const uint64_t *windows, uint32_t n, Geo g, const uint8_t *cnt,
                      const uint32_t *sent, uint32_t V, uint32_t *qcnt, cudaStream_t s);
void launch_nbr_fill(const uint32_t *srcs, const uint64_t *windows, uint32_t n, Geo g, const uint8_t *cnt,
                     const uint32_t *sent, uint32_t V, const uint32_t *offsets, uint32_t *nbrs, uint8_t *vals,
                     cudaStream_t s);
void launch_edge_query(const uint64_t *q, uint32_t n, uint32_t window, Geo g, const uint8_t *cnt,
                       const ulonglong2 *fl, const uint32_t *sent, uint32_t V, uint32_t *res, cudaStream_t s);
void launch_bfs_init(const uint32_t *sources, uint32_t n, uint32_t V, int32_t *dist, uint32_t *frontier,
                     uint32_t *count, cudaStream_t s);
void launch_bfs_expand(const uint32_t *frontier, const uint32_t *nf, uint32_t nf_host, int32_t level, Geo g,
                       const uint8_t *cnt, const uint32_t *sent, int32_t *dist, uint32_t *next, uint32_t *next_count,
                       cudaStream_t s);
void launch_outdeg(Geo g, const uint8_t *cnt, uint32_t *deg, cudaStream_t s);
void launch_fill_f64(double *p, uint64_t n, double x, cudaStream_t s);
void launch_pr_iteration(Geo g, const uint8_t *cnt, const uint32_t *deg, uint32_t V, double alpha, double *rank,
                         double *contrib, double *acc, double *dangling, cudaStream_t s);


// ---- batched update of many graphs (forest launches): one launch per front
// phase over all graphs; block b of a launch works for graph g with
// boff[g] <= b < boff[g + 1] (boff: one table per phase).
struct ForestGraph {
    Geo g;
    const ulonglong2 *fl;
    uint8_t *cnt;
    uint32_t V;
    uint32_t key_format;
    const uint64_t *ins;
    const uint8_t *ins_vals;
    const uint64_t *del;
    uint32_t n_ins, n_del;
    uint64_t *bk0;  // packed batch (pack output, sort input)
    uint16_t *bp0;
    const uint64_t *sk;  // sorted batch: (bk0, bp0) or the second buffer pair
    const uint16_t *sp;
    uint8_t *kind;
    uint32_t *seg, *blk_nn, *blk_ins;
    uint32_t *sup;  // the locate's per-64-block totals (cleared by phase 0)
    uint32_t sup_words;
    UpdList u;
    uint32_t *bitmap;
    uint64_t bitmap_words;
    Window *cand, *wsingle, *wsmall4, *wsmall, *wbig;
    uint8_t *pend;
    Tables tb;
    unsigned long long total_items;
    DevStatus *st;
};
// The common executors of many graphs in one launch each (lpma_update_batch):
// per graph its geometry and the window lists of the single, 4-segment and
// 32-segment executors with their host-known counts.
struct ForestExec {
    Geo g;
    uint8_t *cnt;
    ulonglong2 *fl;
    uint32_t *sent;
    uint32_t V;
    uint32_t n[3];
    const Window *w[3];
    UpdList u;
    DevStatus *st;
};
// kind 0: single-segment windows, 1: up to 4 segments, 2: up to 32
void launch_forest_exec(int kind, const ForestExec *E, const uint32_t *boff, uint32_t ngraphs, uint32_t nblocks,
                        cudaStream_t s);
// CTAs the executor of `kind` gets for n windows (as in lpma_update)
uint32_t exec_ctas(int kind, uint32_t n);
// phases: 0 reset statuses, planner bitmaps and the locate's group totals,
// 1 pack, 2 resolve + locate, 3 compact, 4 plan, 5 maximal windows, 6 status
// copy into out[g]
void launch_forest_phase(int phase, const ForestGraph *F, const uint32_t *boff, uint32_t ngraphs,
                         uint32_t nblocks, DevStatus *out, cudaStream_t s);

}  // namespace lpma
