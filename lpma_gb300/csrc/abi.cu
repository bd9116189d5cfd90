// Host orchestration and the extern "C" boundary of the GB300 LPMA engine.
//
// One update call (reference update_rpma, rpma.cuh:1549-1718):
//   1. pack + validate the batch (a bad key turns the rest of the front
//      into a no-op, so the structure does not change)
//   2. radix sort, resolve + locate + membership, compaction
//   3. count-only plan of the first level loop (skip rule on), the status
//      block published by the planner's last CTA into the pinned host
//      mirror, then the windows of up to 32 segments executed (guarded on
//      the device: nothing happens when the plan overflowed); steps 1-3
//      replay as one CUDA graph and the host waits for the published
//      status only (the one synchronisation of a call without overflow)
//   4. no overflow: execute the bigger maximal windows; if the root took
//      updates, the eager level-up of rpma.cuh:1646-1653
//      overflow (rpma.cuh:1662-1712): resize to h; h == H+1 executes the
//      first loop, adds a level, re-locates the pending updates and runs a
//      second plan with every level allowed, then fill_empty_segs; any
//      other h rebuilds from the pre-batch array plus every update.
#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

#include "gpma.cuh"
#include "kernels.cuh"
#include "lpma.h"
#include "prims.cuh"

using namespace lpma;

namespace lpma {
uint64_t launch_count();
void prof_enable(int on);
size_t prof_report(char *buf, size_t cap);
}

namespace {

// Arrays whose size follows the tree capacity (height Hc).
struct Cap {
    uint32_t Hc = 0;
    uint64_t *keys = nullptr, *keys_alt = nullptr;
    uint8_t *vals = nullptr, *vals_alt = nullptr;
    uint8_t *cnt = nullptr, *cnt_alt = nullptr, *cnt_live = nullptr;
    ulonglong2 *fl = nullptr;
    uint32_t *segP = nullptr, *PQ = nullptr, *US = nullptr, *qi = nullptr, *qd = nullptr;
    uint32_t *bitmap = nullptr;
    uint32_t *scan_tmp = nullptr;
    uint64_t *ts_tmp = nullptr;  // block totals of the big windows' prefix scan
    void *arena = nullptr;  // one stream-ordered allocation holding all of the above
};

// Replays of the front as a CUDA graph, one per batch shape and buffer set.
// Only the pack kernel's input pointers change between replays.
struct FrontGraph {
    uint64_t key[12];
    uint64_t stamp;
    uint64_t launches;  // kernels in the graph, for the launch counter
    cudaGraph_t graph;
    cudaGraphExec_t exec;
    cudaGraphNode_t pack;
    cudaKernelNodeParams pack_params;
};

}  // namespace

struct LpmaHandle {
    LpmaConfig cfg{};
    uint32_t V = 0;
    uint32_t H = 0;
    uint64_t total = 0;        // keys physically present
    uint32_t min_t = 0xFFFFF;  // lower bound of the stored timestamps
    lpma_status_t sticky = LPMA_OK;
    Cap c;
    uint32_t *sent = nullptr;
    DevStatus *dst = nullptr;
    DevStatus *hst = nullptr;   // pinned mirror
    DevStatus *hst_dev = nullptr;  // its device address: the front's planner publishes the status there
    DevStatus *hinit = nullptr; // pinned reset template
    // batch scratch
    size_t bcap = 0;
    uint64_t *bk0 = nullptr, *bk1 = nullptr;
    uint16_t *bp0 = nullptr, *bp1 = nullptr;
    uint8_t *kind = nullptr, *pend = nullptr;
    uint32_t *seg = nullptr, *blk_nn = nullptr, *blk_ins = nullptr;
    uint32_t *sup = nullptr;  // the locate's (kept, insert) totals per 64 blocks of 256 keys
    UpdList u{}, u2{};
    Window *cand = nullptr, *wsingle = nullptr, *wsmall4 = nullptr, *wsmall = nullptr, *wbig = nullptr;
    SortScratch sort{};
    uint32_t *sort_err = nullptr;
    TileJob *jobs_d = nullptr;
    void *arena = nullptr;  // batch scratch: every per-key buffer of an update
    size_t jobs_cap = 0;
    // host-copy staging (lpma_update_host)
    // host-batch staging, two buffer sets: the copy of one call runs on
    // copy_stream while the previous call's executors still run
    uint64_t *stage_ins[2] = {nullptr, nullptr}, *stage_del[2] = {nullptr, nullptr};
    uint8_t *stage_vals[2] = {nullptr, nullptr};
    size_t stage_cap = 0;
    int stage_next = 0;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t stage_free[2] = {nullptr, nullptr};  // after the last call that read the set
    cudaEvent_t copy_done = nullptr;
    // view / export
    uint32_t *row_offset = nullptr, *col_index = nullptr;
    uint8_t *view_vals = nullptr;
    uint64_t *exp_keys = nullptr;
    uint8_t *exp_vals = nullptr;
    size_t view_cap = 0, exp_cap = 0;
    bool view_valid = false;
    uint64_t h2d = 0, d2h = 0;  // bytes copied by the current call
    cudaStream_t cap_stream = nullptr;  // private stream for graph capture
    cudaEvent_t front_ev = nullptr;     // recorded after the front's planner (and its status copy, if any)
    cudaEvent_t front_ev_blk = nullptr; // the same, waited on without spinning (concurrent handles)
    // recorded after the last work of each call that returns with work in
    // flight, on the call's stream: lpma_destroy waits for it, not the device
    cudaEvent_t done_ev = nullptr;
    bool done_recorded = false;
    // LPMA_FLAG_GPMA: the flat array of gpma.cuh (gpma.cu) instead of the
    // leveled tree; the leveled fields above stay unused
    GpmaState *gp = nullptr;
    // the front's 4- and 32-segment executors run on side_stream, beside the
    // single-segment one: fork after the planner, join after them
    cudaStream_t side_stream = nullptr;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    std::vector<FrontGraph> graphs;
    uint64_t graph_clock = 0;
    bool host_staged = false;    // h2d already holds the staged input bytes
    // read paths (neighbour query, BFS, PageRank)
    uint32_t *q_cnt = nullptr, *q_tmp = nullptr;
    size_t q_cap = 0;
    uint32_t *bfs_a = nullptr, *bfs_b = nullptr, *bfs_cnt = nullptr;
    uint32_t *pr_deg = nullptr;
    double *pr_contrib = nullptr, *pr_acc = nullptr, *pr_dangling = nullptr;
    uint32_t *pin_word = nullptr;  // pinned: totals read back by the read paths
    uint64_t recent_shapes[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // front shapes seen, for the capture policy
    uint32_t recent_pos = 0;
    // Bumped whenever a buffer the front reads or writes is (re)allocated:
    // cached front graphs hold raw pointers to every such buffer, so they
    // are all dropped when one moves.  (The sort mode is part of their key.)
    uint64_t buf_gen = 1, graph_gen = 0;
    // the last front sorted with the cooperative sort's 9-bit digits (for
    // the pass count in the stats)
    bool front_sort_wide = false;
};

namespace {

#define CK(x)                                         \
    do {                                              \
        cudaError_t e_ = (x);                         \
        if (e_ != cudaSuccess) return cuda_fail(e_);  \
    } while (0)
#define CKS(x)                                 \
    do {                                       \
        lpma_status_t s_ = (x);                \
        if (s_ != LPMA_OK) return s_;          \
    } while (0)

lpma_status_t cuda_fail(cudaError_t e) {
    (void)e;
    return e == cudaErrorMemoryAllocation ? LPMA_ERR_OUT_OF_MEMORY : LPMA_ERR_CUDA;
}

// LPMA_POISON=1 fills every new buffer with 0xA5 bytes: a debugging aid
// that makes a read of memory no kernel wrote show up deterministically.
bool poison_enabled() {
    const char *e = getenv("LPMA_POISON");  // read per allocation: tests switch it
    return e && e[0] == '1';
}

// LPMA_POISON_ONLY=<text> restricts the poisoning to buffers whose name
// contains <text>.
bool poison_this(const char *name) {
    if (!poison_enabled()) return false;
    const char *only = getenv("LPMA_POISON_ONLY");
    return !only || !only[0] || strstr(name, only) != nullptr;
}

// Device buffers of handles and batchers come from the stream-ordered pool
// (allocated on the calling thread's default stream, which is synchronised
// before the buffer is used, so any stream may use it).  A buffer replaced
// in mid-life is freed with dfree (cudaFree: it waits for the device, so no
// kernel still reads it); a handle that is destroyed after waiting for its
// own work frees its buffers with dfree_async, which does not wait for the
// other handles' streams.
template <typename T>
cudaError_t dalloc_named(const char *name, T **p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = pool_alloc((void **)p, count * sizeof(T), cudaStreamPerThread);
    if (e == cudaSuccess && poison_this(name)) e = cudaMemsetAsync(*p, 0xA5, count * sizeof(T), cudaStreamPerThread);
    if (e == cudaSuccess) e = cudaStreamSynchronize(cudaStreamPerThread);
    return e;
}
#define dalloc(p, n) dalloc_named(#p, p, n)
template <typename T>
void dfree(T *&p) {
    if (p) cudaFree((void *)p);
    p = nullptr;
}
template <typename T>
void dfree_async(T *&p) {
    if (p) cudaFreeAsync((void *)p, cudaStreamPerThread);
    p = nullptr;
}

// Small page-locked host buffers (status mirrors, read-back words, the
// batcher's tables) are kept on a free list when released instead of being
// handed to cudaFreeHost, which waits for the whole device.
std::mutex g_pinned_mu;
std::vector<std::pair<size_t, void *>> g_pinned_free;

template <typename T>
cudaError_t pinned_alloc(T **p, size_t bytes) {
    {
        std::lock_guard<std::mutex> lk(g_pinned_mu);
        for (size_t i = 0; i < g_pinned_free.size(); i++)
            if (g_pinned_free[i].first == bytes) {
                *p = (T *)g_pinned_free[i].second;
                g_pinned_free[i] = g_pinned_free.back();
                g_pinned_free.pop_back();
                return cudaSuccess;
            }
    }
    return cudaMallocHost((void **)p, bytes);
}
template <typename T>
void pinned_release(T *&p, size_t bytes) {
    if (p) {
        std::lock_guard<std::mutex> lk(g_pinned_mu);
        g_pinned_free.emplace_back(bytes, (void *)p);
    }
    p = nullptr;
}

uint32_t min_height(uint64_t cnt) {
    uint32_t h = 0;
    while (nslots_of(h) < cnt) h++;
    return h;
}

uint64_t bitmap_words(uint32_t H) { return ((1ull << (H + 2)) + 31) / 32 + 1; }

// Stream-ordered memory pool of the structure and batch arenas: the memory
// stays cached in the process, so a batch that outgrows its buffers or a
// tree that outgrows its capacity costs no device-wide synchronisation (a
// cudaFree would stall every stream, the other graphs of a batched update
// included).
cudaMemPool_t batch_pool() {
    static std::mutex mu;
    static cudaMemPool_t pools[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lk(mu);
    if (!pools[dev]) {
        cudaMemPoolProps p{};
        p.allocType = cudaMemAllocationTypePinned;
        p.location.type = cudaMemLocationTypeDevice;
        p.location.id = dev;
        if (cudaMemPoolCreate(&pools[dev], &p) != cudaSuccess) {
            pools[dev] = nullptr;
            return nullptr;
        }
        uint64_t keep = ~0ull;
        cudaMemPoolSetAttribute(pools[dev], cudaMemPoolAttrReleaseThreshold, &keep);
    }
    return pools[dev];
}

}  // namespace

uint64_t lpma::pool_reserved_bytes() {
    cudaMemPool_t pool = batch_pool();
    uint64_t v = 0;
    if (pool) cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &v);
    return v;
}

cudaError_t lpma::pool_alloc(void **p, size_t bytes, cudaStream_t s) {
    cudaMemPool_t pool = batch_pool();
    return pool ? cudaMallocFromPoolAsync(p, bytes, pool, s) : cudaMallocAsync(p, bytes, s);
}

namespace {

// Executor grain cut-overs per batch-size bucket (entry b: batches of
// 2^(b-1)+1 .. 2^b keys): cut_group | cut_shared << 8, 0 for the defaults
// (4 and 32 segments).  Process-wide, like the sort tier table.
std::atomic<uint32_t> g_grain[33];

uint32_t grain_bucket(size_t n) {
    const uint32_t b = n <= 1 ? 0u : 64u - (uint32_t)__builtin_clzll((unsigned long long)(n - 1));
    return b > 32 ? 32u : b;
}

uint32_t grain_word(size_t n) { return g_grain[grain_bucket(n)].load(std::memory_order_relaxed); }

void set_grain(Tables &tb, size_t n) {
    const uint32_t w = grain_word(n);
    tb.cut_group = w & 0xFFu;
    tb.cut_shared = (w >> 8) & 0xFFu;
}

// Releases the capacity's arena in stream order (s = nullptr: at once, with
// a device synchronisation).
void free_cap(Cap &c, cudaStream_t s, bool now = false) {
    if (c.arena) {
        if (now)
            cudaFree(c.arena);
        else
            cudaFreeAsync(c.arena, s);
    }
    c = Cap{};
}

// One arena per capacity, from the stream-ordered pool, on stream s.
cudaError_t alloc_cap(Cap &c, uint32_t Hc, cudaStream_t s) {
    const uint64_t ns = nslots_of(Hc), nseg = nseg_of(Hc);
    c = Cap{};
    c.Hc = Hc;
    size_t off = 0;
    std::vector<std::pair<void **, size_t>> parts;
    auto part = [&](auto **p, size_t count) {
        parts.emplace_back(reinterpret_cast<void **>(p), off);
        off += (count * sizeof(**p) + 255) & ~size_t(255);
    };
    part(&c.keys, ns), part(&c.keys_alt, ns), part(&c.vals, ns), part(&c.vals_alt, ns);
    part(&c.cnt, nseg + 64), part(&c.cnt_alt, nseg + 64), part(&c.cnt_live, nseg + 64);
    part(&c.fl, nseg);
    part(&c.segP, nseg + 2), part(&c.PQ, nseg + 2);
    part(&c.US, nseg + 2), part(&c.qi, nseg + 2), part(&c.qd, nseg + 2);
    part(&c.bitmap, bitmap_words(Hc)), part(&c.scan_tmp, scan_tmp_words((uint32_t)nseg + 2) + 64);
    part(&c.ts_tmp, tile_prefix_tmp_words(nseg));
    cudaError_t e = pool_alloc(&c.arena, off, s);
    if (e != cudaSuccess) {
        c = Cap{};
        return e;
    }
    for (auto &pp : parts) *pp.first = static_cast<char *>(c.arena) + pp.second;
    if (poison_this("cap") && (e = cudaMemsetAsync(c.arena, 0xA5, off, s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(c.cnt, 0, nseg + 64, s)) != cudaSuccess) return e;
    return cudaMemsetAsync(c.cnt_live, 0, nseg + 64, s);
}

// Grow the capacity to hold height h, keeping the current tree (prefix copy:
// the heap layout of height H is a prefix of any larger one).
lpma_status_t grow_to(LpmaHandle *h, uint32_t hneed, cudaStream_t s) {
    if (hneed <= h->c.Hc) return LPMA_OK;
    if (hneed > LPMA_MAX_HEIGHT) return LPMA_ERR_CAPACITY;
    uint32_t Hc = std::min<uint32_t>(hneed + 1, LPMA_MAX_HEIGHT);
    Cap n;
    CK(alloc_cap(n, Hc, s));
    Cap &o = h->c;
    if (o.keys) {
        CK(cudaMemcpyAsync(n.keys, o.keys, nslots_of(h->H) * 8, cudaMemcpyDeviceToDevice, s));
        CK(cudaMemcpyAsync(n.vals, o.vals, nslots_of(h->H), cudaMemcpyDeviceToDevice, s));
        CK(cudaMemcpyAsync(n.cnt, o.cnt, nseg_of(h->H), cudaMemcpyDeviceToDevice, s));
        CK(cudaMemcpyAsync(n.fl, o.fl, nseg_of(h->H) * sizeof(ulonglong2), cudaMemcpyDeviceToDevice, s));
    }
    free_cap(o, s);  // in stream order, after the copies
    h->c = n;
    h->buf_gen++;
    return LPMA_OK;
}

// Batch scratch for n update keys: capacity the next power of two (a graph's
// buffers move O(log n) times), all arrays carved from one arena allocated
// on the call's stream; the old arena is released in stream order.
lpma_status_t ensure_batch(LpmaHandle *h, size_t n, cudaStream_t s) {
    if (n <= h->bcap) return LPMA_OK;
    h->buf_gen++;
    size_t cap = 4096;
    while (cap < n) cap <<= 1;
    const size_t nb = cap / 256 + 4;
    const size_t status_words = sort_status_words_wide((uint32_t)cap);
    size_t off = 0;
    std::vector<std::pair<void **, size_t>> parts;
    auto part = [&](auto **p, size_t count) {
        parts.emplace_back(reinterpret_cast<void **>(p), off);
        off += (count * sizeof(**p) + 255) & ~size_t(255);
    };
    part(&h->bk0, cap), part(&h->bk1, cap), part(&h->bp0, cap), part(&h->bp1, cap);
    part(&h->kind, cap), part(&h->pend, cap), part(&h->seg, cap), part(&h->blk_nn, nb), part(&h->blk_ins, nb);
    part(&h->sup, sup_words_for(cap));
    for (UpdList *u : {&h->u, &h->u2})
        part(&u->key, cap), part(&u->val, cap), part(&u->kind, cap), part(&u->seg, cap), part(&u->ip, cap + 1);
    part(&h->cand, cap), part(&h->wsingle, cap), part(&h->wsmall4, cap), part(&h->wsmall, cap), part(&h->wbig, cap);
    part(&h->sort.status, status_words);
    h->bcap = 0;
    if (h->arena) {
        CK(cudaFreeAsync(h->arena, s));
        h->arena = nullptr;
    }
    cudaMemPool_t pool = batch_pool();
    if (pool) {
        CK(cudaMallocFromPoolAsync(&h->arena, off, pool, s));
    } else {
        CK(cudaMallocAsync(&h->arena, off, s));
    }
    if (poison_this("batch")) CK(cudaMemsetAsync(h->arena, 0xA5, off, s));
    for (auto &pp : parts) *pp.first = static_cast<char *>(h->arena) + pp.second;
    h->sort.status_words = status_words;
    h->bcap = cap;
    return LPMA_OK;
}

// a handle that shares the GPU with concurrent callers waits without spinning
inline bool blocking_waits(const LpmaHandle *h) { return (h->cfg.flags & LPMA_FLAG_CONCURRENT) != 0; }
// The front's status reaches the host through the planner's publish into
// the pinned mirror (polled), unless the handle's waits must sleep.
inline bool front_publishes(const LpmaHandle *h) { return h->hst_dev != nullptr && !blocking_waits(h); }

lpma_status_t sync_status(LpmaHandle *h, cudaStream_t s) {
    CK(cudaMemcpyAsync(h->hst, h->dst, sizeof(DevStatus), cudaMemcpyDeviceToHost, s));
    h->d2h += sizeof(DevStatus);
    CK(host_wait(s, blocking_waits(h)));
    CK(cudaGetLastError());
    const uint32_t e = h->hst->error | h->hst->sticky;
    if (e & ERR_TIMEOUT) return LPMA_ERR_TIMEOUT;
    if (e & ERR_INTERNAL) return LPMA_ERR_INTERNAL;
    return LPMA_OK;
}

cudaError_t reset_plan_counters(LpmaHandle *h, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(&h->dst->n_cand, 0, offsetof(DevStatus, empty_found) - offsetof(DevStatus, n_cand), s);
    if (e) return e;
    return cudaMemsetAsync(&h->dst->slots_small, 0, 2 * sizeof(unsigned long long), s);
}

Tables make_tables(const LpmaHandle *h, uint32_t H, bool first_loop) {
    Tables tb{};
    uint64_t len = 32;
    for (int i = 0; i < 32; i++) {
        double d = h->cfg.density_lower_root * (double)len;  // recalculate_density, rpma.cuh:164
        tb.lower[i] = (uint32_t)d;
        len <<= 1;
    }
    int skip = 0;
    for (uint32_t l = 0; l <= H + 1 && l < 32; l++) {
        bool allowed = true;
        if (first_loop && h->cfg.skip_rule) {
            if (l == 4 || l == H / 3) skip = 1;  // rpma.cuh:1614-1619
            if (l == (uint32_t)(H / 3 - 1u) || l == H + 1) skip = 0;
            allowed = (32ull << l) <= 1024 || !skip;
        }
        if (allowed) tb.allowed |= 1u << l;
    }
    return tb;
}

bool needs_prefix(const Tables &tb, uint32_t H) {
    for (uint32_t l = 9; l <= H; l++)
        if ((tb.allowed >> l) & 1u) return true;
    return false;
}

// fresh: the plan counters and the bitmap are already clear (the call's
// first plan), so no memset sits between the front's kernels
lpma_status_t run_plan(LpmaHandle *h, const UpdList &u, uint32_t n_cap, bool thres_active, uint64_t total_live,
                       const Tables &tb, cudaStream_t s, const unsigned long long *total_live_dev = nullptr,
                       bool fresh = false, DevStatus *pub = nullptr) {
    const uint32_t H = h->H;
    const uint64_t nseg = nseg_of(H);
    if (!fresh) {
        CK(cudaMemsetAsync(h->c.bitmap, 0, bitmap_words(H) * 4, s));
        CK(reset_plan_counters(h, s));
    }
    const uint8_t *cntp = thres_active ? h->c.cnt_live : h->c.cnt;
    const bool useP = needs_prefix(tb, H);
    if (useP) CK(scan_u8_to_u32(cntp, h->c.segP, (uint32_t)nseg, h->c.segP + nseg, h->c.scan_tmp, s));
    launch_plan(u, n_cap, cntp, h->c.segP, useP ? 1 : 0, total_live, total_live_dev, H, tb, h->c.bitmap, h->cand,
                h->wsingle, h->wsmall4, h->wsmall, h->wbig, h->pend, h->dst, s, pub);
    CK(cudaGetLastError());
    return LPMA_OK;
}

// Per-segment prefix arrays for the tile grain over the current geometry.
lpma_status_t tile_prep(LpmaHandle *h, const UpdList &u, uint32_t n_list, bool thres_active, cudaStream_t s) {
    const uint64_t nseg = nseg_of(h->H);
    CK(cudaMemsetAsync(h->c.qi, 0, (nseg + 2) * 4, s));
    CK(cudaMemsetAsync(h->c.qd, 0, (nseg + 2) * 4, s));
    launch_seg_update_counts(u, n_list, h->c.qi, h->c.qd, h->dst, s);
    launch_tile_prefix(h->c.cnt, thres_active ? h->c.cnt_live : nullptr, h->c.qi, h->c.qd, nseg, h->c.PQ, h->c.US,
                       h->c.ts_tmp, s);
    CK(cudaGetLastError());
    return LPMA_OK;
}

// Execute the planned maximal windows (status already synced).
// small_done: the single / 4 / 32-segment windows were already launched
// (the shared executors of a batched update).
lpma_status_t exec_plan(LpmaHandle *h, const UpdList &u, uint32_t n_list, uint32_t thres, bool thres_active,
                        cudaStream_t s, LpmaStats *st, bool small_done = false) {
    const uint32_t n_single = h->hst->n_single, n_small4 = h->hst->n_small4, n_small = h->hst->n_small,
                   n_big = h->hst->n_big;
    Geo g{h->c.keys, h->c.vals, h->H};
    if (!small_done) {
        launch_exec_single(h->wsingle, n_single, g, h->c.cnt, h->c.fl, h->sent, h->V, u, thres, h->dst, s);
        launch_exec_multi(h->wsmall4, n_small4, h->wsmall, n_small, g, h->c.cnt, h->c.fl, h->sent, h->V, u, thres,
                          h->dst, s);
    }
    st->windows_single += n_single;
    st->windows_small += n_single + n_small4 + n_small;
    st->slots_rewritten += h->hst->slots_small;
    st->slots_small += h->hst->slots_small;
    if (n_big) {
        // the job list is built on the device (windows sorted by position,
        // tile prefix); the tile count came with the status read-back, so
        // the big windows need no host round trip
        if (n_big > h->jobs_cap) {
            CK(cudaStreamSynchronize(s));  // the old list may still be read
            dfree(h->jobs_d);
            h->jobs_cap = n_big * 2;
            CK(dalloc(&h->jobs_d, h->jobs_cap));
        }
        CKS(tile_prep(h, u, n_list, thres_active, s));
        launch_big_jobs(h->wbig, n_big, h->bk1, h->bk0, h->bp1, h->bp0, h->sort, h->jobs_d, s);
        const uint32_t tiles = h->hst->big_tiles;
        launch_exec_big(h->jobs_d, n_big, tiles, tiles, g, h->c.PQ, h->c.US, u, n_list,
                        thres_active ? thres : 0, h->c.keys_alt, h->c.vals_alt, nslots_of(h->c.Hc), g, h->c.cnt,
                        h->c.fl, h->sent, h->V, h->dst, s);
        CK(cudaGetLastError());
        st->windows_big += n_big;
        st->slots_rewritten += h->hst->slots_big;
    }
    return LPMA_OK;
}

// Add one leaf level (alloc_or_del_levels, rpma.cuh:1396-1415): new empty
// slots at the end of the heap layout, linear counts re-indexed.
lpma_status_t level_up(LpmaHandle *h, cudaStream_t s) {
    const uint32_t H = h->H;
    CKS(grow_to(h, H + 1, s));
    CK(cudaMemsetAsync(h->c.keys + nslots_of(H), 0xFF, (nslots_of(H + 1) - nslots_of(H)) * 8, s));
    CK(cudaMemsetAsync(h->c.vals + nslots_of(H), 0, nslots_of(H + 1) - nslots_of(H), s));
    CK(cudaMemsetAsync(h->c.fl + nseg_of(H), 0xFF, (nseg_of(H + 1) - nseg_of(H)) * sizeof(ulonglong2), s));
    launch_levelup_cnt(h->c.cnt, h->c.cnt_alt, H, s);
    std::swap(h->c.cnt, h->c.cnt_alt);
    h->H = H + 1;
    CK(cudaGetLastError());
    return LPMA_OK;
}

// Rebuild at height hh (rebuild_rpma, rpma.cuh:1417-1472): every kept key of
// the current array plus the list's inserts, spread over the new array.
lpma_status_t rebuild(LpmaHandle *h, uint32_t hh, const UpdList &u, uint32_t n_list, uint64_t m, uint32_t thres,
                      bool thres_active, cudaStream_t s, LpmaStats *st) {
    if (hh > LPMA_MAX_HEIGHT) return LPMA_ERR_CAPACITY;
    const uint32_t H = h->H;
    CKS(tile_prep(h, u, n_list, thres_active, s));
    Cap fresh;
    const bool grow = hh > h->c.Hc;
    if (grow) CK(alloc_cap(fresh, std::min<uint32_t>(hh + 1, LPMA_MAX_HEIGHT), s));
    // gather into the alternate buffer, spread into the main buffer (of the
    // new capacity when the tree outgrows the current one)
    Geo src{h->c.keys, h->c.vals, H};
    Geo dst = grow ? Geo{fresh.keys, fresh.vals, hh} : Geo{h->c.keys, h->c.vals, hh};
    uint64_t *Mk = grow ? fresh.keys_alt : h->c.keys_alt;
    uint8_t *Mv = grow ? fresh.vals_alt : h->c.vals_alt;
    uint8_t *cnt_d = grow ? fresh.cnt : h->c.cnt;
    ulonglong2 *fl_d = grow ? fresh.fl : h->c.fl;
    const uint32_t sf = (uint32_t)nseg_of(H), df = (uint32_t)nseg_of(hh);
    if (!h->jobs_d) {
        CK(dalloc(&h->jobs_d, 64));
        h->jobs_cap = 64;
    }
    launch_set_job(h->jobs_d, TileJob{0, sf, 0, df, (uint32_t)m, 0, 0, 0}, s);
    const uint64_t m_cap = nslots_of(grow ? fresh.Hc : h->c.Hc);
    launch_exec_big(h->jobs_d, 1, (sf + 31) / 32, (df + 31) / 32, src, h->c.PQ, h->c.US, u, n_list,
                    thres_active ? thres : 0, Mk, Mv, m_cap, dst, cnt_d, fl_d, h->sent, h->V, h->dst, s);
    CK(cudaGetLastError());
    if (grow) {
        free_cap(h->c, s);  // in stream order, after the gather read it
        h->c = fresh;
        h->buf_gen++;
    } else if (hh < H) {
        CK(cudaMemsetAsync(h->c.cnt + nseg_of(hh), 0, nseg_of(H) - nseg_of(hh) + 64, s));
    }
    h->H = hh;
    st->rebuilt = 1;
    st->slots_rewritten += nslots_of(hh);
    return LPMA_OK;
}

// Segments whose bounds and counts the pack kernel prefetches into L2: all
// of them when the batch is large against the tree (the locate then touches
// most of the deep levels), none for a small batch.
uint64_t prefetch_segs(const LpmaHandle *h, size_t n) {
    const uint64_t nseg = nseg_of(h->H);
    return (h->c.fl && h->c.cnt && (uint64_t)n * 8 >= nseg) ? nseg : 0;
}

// Everything of an update call up to the host round trip: status reset,
// pack, sort, resolve + locate, compaction, plan and the status read-back.
lpma_status_t enqueue_front(LpmaHandle *h, cudaStream_t s, const uint64_t *ins, const uint8_t *ins_vals,
                            size_t n_ins, const uint64_t *del, size_t n_del, uint32_t thres, bool thres_active,
                            bool internal) {
    const size_t n = n_ins + n_del;
    CK(cudaMemcpyAsync(h->dst, h->hinit, offsetof(DevStatus, sticky), cudaMemcpyHostToDevice, s));
    // the engine's own sentinel keys are always in the packed layout
    const uint32_t key_format = internal ? (uint32_t)LPMA_KEY_PACKED : h->cfg.key_format;
    launch_pack(ins, ins_vals, (uint32_t)n_ins, del, (uint32_t)n_del, h->V, thres, key_format, internal ? 1 : 0,
                h->bk0, h->bp0, h->dst, h->c.bitmap, (uint32_t)bitmap_words(h->H), h->c.fl, h->c.cnt,
                prefetch_segs(h, n), h->sup, sup_words_for(n), h->sort.bar, s);
    if (thres_active) launch_live_counts(h->c.keys, h->H, thres, h->c.cnt_live, h->dst, s);
    // sort (digit bytes decided on the device), resolve + locate, compact
    const SortTier tier = sort_tier_for_update((uint32_t)n, h->sort);
    const SortMask mask = update_sort_mask(&h->dst->key_and, tier, (uint32_t)n, h->sort);
    h->sort.bar_cleared = h->sort.bar != nullptr;  // by k_pack
    const cudaError_t se = sort_pairs_dev<uint16_t>(h->bk0, h->bp0, h->bk1, h->bp1, (uint32_t)n, mask, h->sort, s, tier);
    h->sort.bar_cleared = false;
    CK(se);
    Geo g{h->c.keys, h->c.vals, h->H};
    launch_resolve_locate(h->bk0, h->bp0, h->bk1, h->bp1, (uint32_t)n, mask, g, h->c.fl, thres, h->kind, h->seg,
                          h->blk_nn, h->blk_ins, h->sup, h->dst, s);
    launch_compact(h->bk0, h->bp0, h->bk1, h->bp1, mask, h->kind, h->seg, (uint32_t)n, h->blk_nn, h->blk_ins, h->sup,
                   h->u, h->dst, s);
    // plan the first loop
    Tables tb = make_tables(h, h->H, true);
    set_grain(tb, n);
    // the status reset cleared the plan counters and k_pack the bitmap
    const bool pub = front_publishes(h);
    CKS(run_plan(h, h->u, (uint32_t)n, thres_active, 0, tb, s,
                 thres_active ? &h->dst->live_total : &h->dst->total_items, true, pub ? h->hst_dev : nullptr));
    // The status read-back and the first loop's single / 4 / 32-segment
    // windows follow without a host round trip: the executors read their
    // counts on the device and do nothing when the plan overflowed, so they
    // run while the host decides what else the call needs.  The read-back is
    // the planner's publish into the pinned mirror (the host polls its flag;
    // the front's event, recorded after the planner, backs the poll), or,
    // for a handle whose waits sleep, a copy with a blocking event after it.
    // The copy, the event and the 4- and 32-segment executors (one launch)
    // run on a second stream (a parallel branch of the captured graph): the
    // single-segment executor follows the planner directly, as its
    // programmatic dependent, and the windows of the three are disjoint.
    // The join makes everything after them on s wait for all.  The
    // in-library profiler times each kernel alone, so it keeps them on one
    // stream.
    Geo ge{h->c.keys, h->c.vals, h->H};
    const bool fork = !prof_enabled();
    cudaStream_t side = fork ? h->side_stream : s;
    if (fork) {
        CK(cudaEventRecord(h->fork_ev, s));
        CK(cudaStreamWaitEvent(side, h->fork_ev, 0));
    }
    if (!pub) CK(cudaMemcpyAsync(h->hst, h->dst, sizeof(DevStatus), cudaMemcpyDeviceToHost, side));
    // an event record node when the front is being captured into a graph
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    CK(cudaStreamIsCapturing(s, &cs));
    CK(cudaEventRecordWithFlags(blocking_waits(h) ? h->front_ev_blk : h->front_ev, side,
                                cs == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : cudaEventRecordDefault));
    launch_exec_multi(h->wsmall4, (uint32_t)n, h->wsmall, (uint32_t)n, ge, h->c.cnt, h->c.fl, h->sent, h->V, h->u,
                      thres, h->dst, side, true);
    if (fork) CK(cudaEventRecord(h->join_ev, side));
    launch_exec_single(h->wsingle, (uint32_t)n, ge, h->c.cnt, h->c.fl, h->sent, h->V, h->u, thres, h->dst, s, true);
    if (fork) CK(cudaStreamWaitEvent(s, h->join_ev, 0));
    return LPMA_OK;
}

bool graphs_enabled() {
    static int on = -1;
    if (on < 0) {
        const char *e = getenv("LPMA_NO_GRAPH");
        on = (e && e[0] == '1') ? 0 : 1;
    }
    return on == 1;
}

lpma_status_t run_front(LpmaHandle *h, cudaStream_t s, const uint64_t *ins, const uint8_t *ins_vals, size_t n_ins,
                        const uint64_t *del, size_t n_del, uint32_t thres, bool thres_active, bool internal) {
    const size_t n = n_ins + n_del;
    h->h2d += offsetof(DevStatus, sticky);
    h->d2h += sizeof(DevStatus);
    // the planner of this front sets it again (no GPU write to the mirror
    // is pending: the last front's was waited for)
    if (front_publishes(h)) __atomic_store_n(&h->hst->published, 0u, __ATOMIC_RELEASE);
    // the stored-key count reaches the planner through the status reset copy,
    // so that it is not a kernel argument of a cached graph
    h->hinit->total_items = h->total;
    h->front_sort_wide = update_sort_mask(nullptr, sort_tier_for_update((uint32_t)n, h->sort), (uint32_t)n, h->sort).wide;
    if (internal || prof_enabled() || !graphs_enabled()) {
        CKS(enqueue_front(h, s, ins, ins_vals, n_ins, del, n_del, thres, thres_active, internal));
    } else {
        const uint64_t key[12] = {n_ins, n_del, h->H, thres,
                                  (uint64_t)thres_active | ((uint64_t)(ins_vals != nullptr) << 1) |
                                      ((uint64_t)(h->sort.bar != nullptr) << 2) |
                                      ((uint64_t)sort_tier_for_update((uint32_t)n, h->sort) << 3) |
                                      ((uint64_t)grain_word(n) << 16),
                                  (uint64_t)h->c.keys, (uint64_t)h->c.vals, (uint64_t)h->c.cnt, (uint64_t)h->c.fl,
                                  (uint64_t)h->bk0, (uint64_t)h->c.cnt_live, (uint64_t)h->c.bitmap};
        if (h->graph_gen != h->buf_gen) {
            for (FrontGraph &f : h->graphs) {
                cudaGraphExecDestroy(f.exec);
                cudaGraphDestroy(f.graph);
            }
            h->graphs.clear();
            h->graph_gen = h->buf_gen;
        }
        FrontGraph *fg = nullptr;
        for (FrontGraph &f : h->graphs)
            if (!memcmp(f.key, key, sizeof(key))) fg = &f;
        if (!fg) {
            // capture a shape only when it repeats: a stream of varying batch
            // sizes would otherwise pay a capture and instantiation per call
            uint64_t hk = 1469598103934665603ull;
            for (uint64_t w : key) hk = (hk ^ w) * 1099511628211ull;
            bool seen = false;
            for (uint64_t x : h->recent_shapes) seen |= x == hk;
            if (!seen) {
                h->recent_shapes[h->recent_pos++ % 8] = hk;
                return enqueue_front(h, s, ins, ins_vals, n_ins, del, n_del, thres, thres_active, internal);
            }
        }
        if (!fg) {
            if (h->graphs.size() >= 16) {
                auto lru = std::min_element(h->graphs.begin(), h->graphs.end(),
                                            [](const FrontGraph &a, const FrontGraph &b) { return a.stamp < b.stamp; });
                cudaGraphExecDestroy(lru->exec);
                cudaGraphDestroy(lru->graph);
                h->graphs.erase(lru);
            }
            FrontGraph f{};
            memcpy(f.key, key, sizeof(key));
            const uint64_t l0 = launch_count();
            CK(cudaStreamBeginCapture(h->cap_stream, cudaStreamCaptureModeThreadLocal));
            lpma_status_t r = enqueue_front(h, h->cap_stream, ins, ins_vals, n_ins, del, n_del, thres, thres_active,
                                            internal);
            cudaGraph_t gr = nullptr;
            cudaError_t ce = cudaStreamEndCapture(h->cap_stream, &gr);
            if (r != LPMA_OK) return r;
            CK(ce);
            f.graph = gr;
            f.launches = launch_count() - l0;
            CK(cudaGraphInstantiate(&f.exec, gr, 0));
            size_t nn = 0;
            CK(cudaGraphGetNodes(gr, nullptr, &nn));
            std::vector<cudaGraphNode_t> nodes(nn);
            CK(cudaGraphGetNodes(gr, nodes.data(), &nn));
            for (cudaGraphNode_t nd : nodes) {
                cudaGraphNodeType t;
                CK(cudaGraphNodeGetType(nd, &t));
                if (t != cudaGraphNodeTypeKernel) continue;
                cudaKernelNodeParams kp;
                CK(cudaGraphKernelNodeGetParams(nd, &kp));
                if (kp.func == pack_kernel_fn()) {
                    f.pack = nd;
                    f.pack_params = kp;
                }
            }
            if (!f.pack) return LPMA_ERR_INTERNAL;
            h->graphs.push_back(f);
            fg = &h->graphs.back();
            note_launch(-(int)f.launches);  // counted again on each replay
        }
        fg->stamp = ++h->graph_clock;
        // k_pack(ins, ins_vals, n_ins, del, n_del, V, thres, key_format, internal, keys_out, pay_out, st, bitmap,
        //        bitmap_words, fl, cnt, pf_segs, sup, sup_words, sort_bar)
        const uint64_t *a_ins = ins, *a_del = del;
        const uint8_t *a_vals = ins_vals;
        uint32_t a_nins = (uint32_t)n_ins, a_ndel = (uint32_t)n_del, a_V = h->V, a_thres = thres,
                 a_fmt = h->cfg.key_format;
        int a_internal = 0;
        uint64_t *a_ko = h->bk0;
        uint16_t *a_po = h->bp0;
        DevStatus *a_st = h->dst;
        uint32_t *a_bm = h->c.bitmap;
        uint32_t a_bmw = (uint32_t)bitmap_words(h->H);
        const ulonglong2 *a_fl = h->c.fl;
        const uint8_t *a_cnt = h->c.cnt;
        uint64_t a_pf = prefetch_segs(h, n);
        uint32_t *a_sup = h->sup;
        uint32_t a_supw = sup_words_for(n);
        uint32_t *a_bar = h->sort.bar;
        void *args[] = {&a_ins, &a_vals, &a_nins, &a_del, &a_ndel, &a_V, &a_thres, &a_fmt, &a_internal, &a_ko, &a_po, &a_st,
                        &a_bm, &a_bmw, &a_fl, &a_cnt, &a_pf, &a_sup, &a_supw, &a_bar};
        cudaKernelNodeParams kp = fg->pack_params;
        kp.kernelParams = args;
        kp.extra = nullptr;
        CK(cudaGraphExecKernelNodeSetParams(fg->exec, fg->pack, &kp));
        CK(cudaGraphLaunch(fg->exec, s));
        note_launch((int)fg->launches);
    }
    return LPMA_OK;
}

// The handle's last work is on stream s: lpma_destroy waits for this event.
void mark_done(LpmaHandle *h, cudaStream_t s) {
    if (h->done_ev && cudaEventRecord(h->done_ev, s) == cudaSuccess) h->done_recorded = true;
}

// Polls the mirror's `published` word (set by the planner's last CTA after
// the status words).  The front's event completes after the planner too:
// queried now and then, it ends the wait with the error of a failed kernel,
// or, should the word not be seen once the planner has finished, the status
// is copied back instead.
cudaError_t wait_published(LpmaHandle *h) {
    for (uint32_t spin = 1;; spin++) {
        if (__atomic_load_n(&h->hst->published, __ATOMIC_ACQUIRE)) return cudaSuccess;
        if (spin % 64) continue;
        const cudaError_t q = cudaEventQuery(h->front_ev);
        if (q == cudaErrorNotReady) continue;
        if (q != cudaSuccess) return q;
        if (__atomic_load_n(&h->hst->published, __ATOMIC_ACQUIRE)) return cudaSuccess;
        const cudaError_t e = cudaMemcpyAsync(h->hst, h->dst, sizeof(DevStatus), cudaMemcpyDeviceToHost, h->side_stream);
        return e ? e : cudaStreamSynchronize(h->side_stream);
    }
}

lpma_status_t wait_front(LpmaHandle *h, cudaStream_t) {
    CK(front_publishes(h) ? wait_published(h)
                          : blocking_waits(h) ? event_wait(h->front_ev_blk) : cudaEventSynchronize(h->front_ev));
    CK(cudaGetLastError());
    const uint32_t e = h->hst->error | h->hst->sticky;
    if (e & ERR_TIMEOUT) return LPMA_ERR_TIMEOUT;
    if (e & ERR_INTERNAL) return LPMA_ERR_INTERNAL;
    return LPMA_OK;
}

// Everything after the front's status read-back (rs is the read-back's
// verdict, h->hst holds the status block): the window executors, the
// root / overflow / resize paths and the stats.  Shared by lpma_update and
// the graphs of a batched update.  small_done: the first loop's single / 4 /
// 32-segment executors already ran (in lpma_update's front, guarded, or in
// the shared launches of a batched update).
lpma_status_t finish_update(LpmaHandle *h, lpma_status_t rs, size_t n, uint32_t thres, bool thres_active,
                            cudaStream_t s, LpmaStats &st, LpmaStats *out, bool small_done = false) {
    // a sort that gave up a bounded wait turned the front into a no-op:
    // nothing changed, so the handle stays usable
    if (rs == LPMA_ERR_TIMEOUT && h->hst->sticky == 0) return rs;
    if (rs != LPMA_OK) return h->sticky = rs;
    if (h->hst->error & ERR_KEY) return LPMA_ERR_INVALID_KEY;
    {
        // the digit passes the sort made: one per differing byte, or with
        // 9-bit digits one per window (the greedy plan of the sort itself)
        uint64_t diff = h->hst->key_and ^ h->hst->key_or;
        if (h->front_sort_wide) {
            while (diff) {
                const int b = __builtin_ctzll(diff);
                diff = b + WIDE_DIGIT_BITS >= 64 ? 0ull : (diff >> (b + WIDE_DIGIT_BITS)) << (b + WIDE_DIGIT_BITS);
                st.sort_passes++;
            }
        } else {
            for (int b = 0; b < 8; b++) st.sort_passes += ((diff >> (8 * b)) & 0xFF) ? 1u : 0u;
        }
    }
    const uint32_t min_t_ins = h->hst->min_t_ins;
    const int64_t live_before = thres_active ? (int64_t)h->hst->live_total : (int64_t)h->total;
    const uint32_t n_u = h->hst->n_u, n_new = h->hst->n_ins, n_gone = h->hst->n_del;
    st.n_ins_applied = n_new;
    st.n_del_applied = n_gone;
    st.n_upserts = h->hst->n_upsert;
    st.n_noop = h->hst->n_noop;
    const int64_t live_after = live_before - n_gone + n_new;

    lpma_status_t r = LPMA_OK;
    if (n_u > 0 && !h->hst->ovf) {
        const bool root = h->hst->root != 0;
        r = exec_plan(h, h->u, (uint32_t)n, thres, thres_active, s, &st, small_done);
        if (r == LPMA_OK && root) {
            st.root_executed = 1;
            st.levelup = 1;  // update_rpma returns true once the root absorbed (rpma.cuh:1646-1653)
            if (min_height((uint64_t)live_after) + 1 > h->H) {  // eager level-up
                r = level_up(h, s);
                st.eager_levelup = 1;
            }
        }
    } else if (n_u > 0) {
        st.overflow = 1;
        st.levelup = 1;  // and after any overflow, whatever the new height (rpma.cuh:1662-1668)
        const uint32_t hh = min_height((uint64_t)live_after);
        if (hh == h->H + 1) {
            st.levelup_path = 1;
            r = exec_plan(h, h->u, (uint32_t)n, thres, thres_active, s, &st);
            if (r == LPMA_OK) r = level_up(h, s);
            if (r == LPMA_OK) {
                launch_compact_pending(h->u, h->pend, n_u, h->u2, h->blk_nn, h->blk_ins, h->dst, s);
                r = sync_status(h, s);
            }
            if (r == LPMA_OK) {
                const uint32_t n2 = h->hst->n_u, i2 = h->hst->n_ins, d2 = h->hst->n_del;
                const int64_t live_mid = live_before - (int64_t)(n_gone - d2) + (int64_t)(n_new - i2);
                Geo g2{h->c.keys, h->c.vals, h->H};
                launch_relocate(h->u2, n2, g2, h->c.fl, s);
                if (thres_active) {
                    CK(cudaMemsetAsync(&h->dst->live_total, 0, 8, s));
                    launch_live_counts(h->c.keys, h->H, thres, h->c.cnt_live, h->dst, s);
                }
                Tables tb2 = make_tables(h, h->H, false);
                set_grain(tb2, n);
                r = run_plan(h, h->u2, n2, thres_active, (uint64_t)live_mid, tb2, s);
                if (r == LPMA_OK) r = sync_status(h, s);
                if (r == LPMA_OK && h->hst->ovf) {
                    // the reference asserts here (rpma.cuh:1704); rebuild instead
                    r = rebuild(h, min_height((uint64_t)live_after), h->u2, n2, (uint64_t)live_after, thres,
                                thres_active, s, &st);
                } else if (r == LPMA_OK) {
                    r = exec_plan(h, h->u2, n2, thres, thres_active, s, &st);
                    if (r == LPMA_OK && h->H > 0) {  // fill_empty_segs, rpma.cuh:1474-1530
                        CK(cudaMemsetAsync(&h->dst->empty_found, 0, 4, s));
                        launch_check_empty_level(h->c.cnt, h->H, h->dst, s);
                        r = sync_status(h, s);
                        if (r == LPMA_OK && h->hst->empty_found) {
                            if (thres_active) launch_live_counts(h->c.keys, h->H, thres, h->c.cnt_live, h->dst, s);
                            r = rebuild(h, h->H, h->u2, 0, (uint64_t)live_after, thres, thres_active, s, &st);
                            st.rebuilt = 0;
                            st.fill_empty = 1;
                        }
                    }
                }
            }
        } else {
            // h < H, h > H+1 (and h == H, where the reference asserts): rebuild
            r = rebuild(h, hh, h->u, (uint32_t)n, (uint64_t)live_after, thres, thres_active, s, &st);
        }
    }
    if (r != LPMA_OK) return h->sticky = r;
    if (thres_active) {
        // executed windows dropped expired keys: recount what is stored
        CK(cudaMemsetAsync(&h->dst->cnt_total, 0, 8, s));
        launch_sum_cnt(h->c.cnt, nseg_of(h->H), h->dst, s);
        rs = sync_status(h, s);
        if (rs != LPMA_OK) return h->sticky = rs;
    }
    // the common path returns here (big windows may still run on the stream)
    h->total = thres_active ? h->hst->cnt_total : (uint64_t)live_after;
    if (n_new && min_t_ins < h->min_t) h->min_t = min_t_ins;
    st.height_after = h->H;
    st.num_items = h->total;
    st.h2d_bytes = h->h2d;
    st.d2h_bytes = h->d2h;
    if (out) *out = st;
    mark_done(h, s);
    return LPMA_OK;
}

lpma_status_t do_update(LpmaHandle *h, const uint64_t *ins, const uint8_t *ins_vals, size_t n_ins,
                        const uint64_t *del, size_t n_del, uint32_t thres, cudaStream_t s, LpmaStats *out,
                        bool internal) {
    if (h->sticky != LPMA_OK) return h->sticky;
    if (!internal && !h->host_staged) h->h2d = 0;
    h->host_staged = false;
    h->d2h = 0;
    LpmaStats st{};
    st.height_before = h->H;
    const size_t n = n_ins + n_del;
    if ((n_ins && !ins) || (n_del && !del)) return LPMA_ERR_INVALID_ARGUMENT;
    if (n == 0) {
        st.height_after = h->H;
        st.num_items = h->total;
        if (out) *out = st;
        return LPMA_OK;
    }
    if (n >= (1u << 30)) return LPMA_ERR_INVALID_ARGUMENT;
    if (thres > 0xFFFFF) return LPMA_ERR_INVALID_ARGUMENT;
    if (min_height(h->total + n_ins) > LPMA_MAX_HEIGHT) return LPMA_ERR_CAPACITY;
    CKS(ensure_batch(h, n, s));
    h->view_valid = false;
    const bool thres_active = thres > h->min_t;

    // pack, sort, resolve + locate, compact, plan (one CUDA graph when the
    // batch shape repeats), then the one host round trip of the common path;
    // a rejected batch turns every kernel after k_pack into a no-op
    CKS(run_front(h, s, ins, ins_vals, n_ins, del, n_del, thres, thres_active, internal));
    return finish_update(h, wait_front(h, s), n, thres, thres_active, s, st, out, true);
}

}  // namespace

// ====================================================================== C ABI
// Host threads that finish the graphs of a batched update that need more
// than the shared executors (big windows, overflow, resize: paths with host
// round trips), each on its own stream so that their round trips overlap.
struct BatchWorkers {
    std::mutex mu;
    std::condition_variable cv, done_cv;
    std::vector<std::thread> th;
    std::vector<cudaStream_t> st;
    std::vector<cudaEvent_t> ev;
    std::vector<uint8_t> used;
    std::function<void(size_t, cudaStream_t)> fn;
    std::atomic<size_t> next{0};
    size_t n = 0;
    uint64_t gen = 0;
    int busy = 0;
    bool stop = false;

    cudaError_t start(int nthreads) {
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e) return e;
        st.assign(nthreads, nullptr);
        ev.assign(nthreads, nullptr);
        used.assign(nthreads, 0);
        for (int w = 0; w < nthreads; w++) {
            if ((e = cudaStreamCreateWithFlags(&st[w], cudaStreamNonBlocking)) ||
                (e = cudaEventCreateWithFlags(&ev[w], cudaEventDisableTiming)))
                return e;
        }
        for (int w = 0; w < nthreads; w++) th.emplace_back([this, w, dev] { loop(w, dev); });
        return cudaSuccess;
    }

    void loop(int w, int dev) {
        cudaSetDevice(dev);
        uint64_t seen = 0;
        for (;;) {
            {
                std::unique_lock<std::mutex> lk(mu);
                cv.wait(lk, [&] { return stop || gen != seen; });
                if (stop) return;
                seen = gen;
            }
            bool any = false;
            for (size_t i; (i = next.fetch_add(1)) < n;) {
                fn(i, st[w]);
                any = true;
            }
            if (any) cudaEventRecord(ev[w], st[w]);
            std::lock_guard<std::mutex> lk(mu);
            used[w] = any;
            if (--busy == 0) done_cv.notify_all();
        }
    }

    // runs fn(i, stream) for i < count on the workers and the calling thread
    // (which uses s); afterwards s waits for the workers' streams
    void run(size_t count, cudaStream_t s, std::function<void(size_t, cudaStream_t)> f) {
        {
            std::lock_guard<std::mutex> lk(mu);
            fn = std::move(f);
            n = count;
            next = 0;
            busy = (int)th.size();
            gen++;
        }
        cv.notify_all();
        for (size_t i; (i = next.fetch_add(1)) < count;) fn(i, s);
        std::unique_lock<std::mutex> lk(mu);
        done_cv.wait(lk, [&] { return busy == 0; });
        for (size_t w = 0; w < th.size(); w++)
            if (used[w]) cudaStreamWaitEvent(s, ev[w], 0);
    }

    ~BatchWorkers() {
        {
            std::lock_guard<std::mutex> lk(mu);
            stop = true;
        }
        cv.notify_all();
        for (std::thread &t : th) t.join();
        for (cudaStream_t x : st)
            if (x) cudaStreamDestroy(x);
        for (cudaEvent_t x : ev)
            if (x) cudaEventDestroy(x);
    }
};

// Device and pinned tables of a batched update (lpma_update_batch), kept
// between calls.
struct LpmaBatcher {
    size_t cap_g = 0;
    ForestGraph *dF = nullptr, *hF = nullptr;
    uint32_t *dB = nullptr, *hB = nullptr;  // block offsets: FOREST_TABLES tables of G + 1
    ForestSortJob *dJ = nullptr, *hJ = nullptr;
    DevStatus *dS = nullptr, *hS = nullptr;
    ForestExec *dE = nullptr, *hE = nullptr;
    uint32_t *dX = nullptr, *hX = nullptr;  // executor block offsets: 3 tables of G + 1
    cudaEvent_t done = nullptr;             // after the last shared executor of the previous call
    // the shared 4- and 32-segment executors run on side beside the
    // single-segment one (disjoint windows)
    cudaStream_t side = nullptr;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    bool pending = false;
    BatchWorkers *workers = nullptr;
};

namespace {

// block-offset tables of a batched update: pack, resolve, compact, plan,
// maximal windows, then the sort's tile launch and merge rounds
constexpr int FOREST_TABLES = 6 + (int)FOREST_MERGE_ROUNDS_MAX;

// final: the batcher's work is known to be done, so the device buffers go
// back to the pool without a device-wide synchronisation
void batcher_free(LpmaBatcher *b, bool final = false) {
    if (final) {
        dfree_async(b->dF), dfree_async(b->dB), dfree_async(b->dJ), dfree_async(b->dS), dfree_async(b->dE),
            dfree_async(b->dX);
    } else {
        dfree(b->dF), dfree(b->dB), dfree(b->dJ), dfree(b->dS), dfree(b->dE), dfree(b->dX);
    }
    const size_t c = b->cap_g;
    pinned_release(b->hF, c * sizeof(ForestGraph));
    pinned_release(b->hB, FOREST_TABLES * (c + 1) * sizeof(uint32_t));
    pinned_release(b->hJ, c * sizeof(ForestSortJob));
    pinned_release(b->hS, c * sizeof(DevStatus));
    pinned_release(b->hE, c * sizeof(ForestExec));
    pinned_release(b->hX, 3 * (c + 1) * sizeof(uint32_t));
    b->cap_g = 0;
}

lpma_status_t batcher_reserve(LpmaBatcher *b, size_t G) {
    if (G <= b->cap_g) return LPMA_OK;
    batcher_free(b);
    const size_t c = std::max<size_t>(G, 64);
    CK(dalloc(&b->dF, c));
    CK(dalloc(&b->dB, FOREST_TABLES * (c + 1)));
    CK(dalloc(&b->dJ, c));
    CK(dalloc(&b->dS, c));
    CK(pinned_alloc(&b->hF, c * sizeof(ForestGraph)));
    CK(pinned_alloc(&b->hB, FOREST_TABLES * (c + 1) * sizeof(uint32_t)));
    CK(pinned_alloc(&b->hJ, c * sizeof(ForestSortJob)));
    CK(pinned_alloc(&b->hS, c * sizeof(DevStatus)));
    CK(dalloc(&b->dE, c));
    CK(dalloc(&b->dX, 3 * (c + 1)));
    CK(pinned_alloc(&b->hE, c * sizeof(ForestExec)));
    CK(pinned_alloc(&b->hX, 3 * (c + 1) * sizeof(uint32_t)));
    b->cap_g = c;
    return LPMA_OK;
}

}  // namespace

extern "C" {

lpma_status_t lpma_config_default(LpmaConfig *cfg) {
    if (!cfg) return LPMA_ERR_INVALID_ARGUMENT;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->segment_length = 32;
    cfg->key_format = LPMA_KEY_PACKED;
    cfg->skip_rule = 1;
    cfg->density_lower_root = 0.42;
    cfg->density_upper_root = 1.0;
    return LPMA_OK;
}

lpma_status_t lpma_config_gpma(LpmaConfig *cfg) {
    if (!cfg) return LPMA_ERR_INVALID_ARGUMENT;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->segment_length = 0;  // 2^(fls(fls(size)) - 1), from the size
    cfg->key_format = LPMA_KEY_PAIR32;
    cfg->flags = LPMA_FLAG_GPMA;
    cfg->density_lower_root = 0.15;  // gpma.cuh:52
    cfg->density_upper_root = 1.0;
    return LPMA_OK;
}

lpma_status_t lpma_gpma_view(LpmaHandle *h, const uint32_t **row_offset, const uint64_t **keys, const uint8_t **values,
                             uint64_t *size, uint32_t *segment_length, uint32_t *height) {
    if (!h || !h->gp) return LPMA_ERR_INVALID_ARGUMENT;
    gpma_view(h->gp, row_offset, keys, values);
    return gpma_geometry(h->gp, size, segment_length, height, nullptr);
}

lpma_status_t lpma_destroy(LpmaHandle *h) {
    if (!h) return LPMA_ERR_INVALID_ARGUMENT;
    if (h->gp) {
        gpma_destroy(h->gp);
        delete h;
        return LPMA_OK;
    }
    // wait for this handle's own work only: its last call's stream (the
    // event recorded after that call's last launch) and its private streams;
    // then every buffer goes back to the stream-ordered pool without a
    // device-wide synchronisation, so other handles' streams keep running
    if (h->done_recorded) cudaEventSynchronize(h->done_ev);
    for (cudaStream_t st : {h->side_stream, h->cap_stream, h->copy_stream})
        if (st) cudaStreamSynchronize(st);
    for (FrontGraph &f : h->graphs) {
        cudaGraphExecDestroy(f.exec);
        cudaGraphDestroy(f.graph);
    }
    h->graphs.clear();
    if (h->cap_stream) cudaStreamDestroy(h->cap_stream);
    if (h->side_stream) cudaStreamDestroy(h->side_stream);
    if (h->fork_ev) cudaEventDestroy(h->fork_ev);
    if (h->join_ev) cudaEventDestroy(h->join_ev);
    if (h->front_ev) cudaEventDestroy(h->front_ev);
    if (h->front_ev_blk) cudaEventDestroy(h->front_ev_blk);
    free_cap(h->c, cudaStreamPerThread);
    dfree_async(h->sent), dfree_async(h->dst);
    pinned_release(h->hst, sizeof(DevStatus));
    pinned_release(h->hinit, sizeof(DevStatus));
    if (h->arena) cudaFreeAsync(h->arena, cudaStreamPerThread);  // the batch scratch
    h->arena = nullptr;
    dfree_async(h->sort.hist), dfree_async(h->sort.counters), dfree_async(h->sort_err);
    dfree_async(h->jobs_d);
    for (int b = 0; b < 2; b++) {
        dfree_async(h->stage_ins[b]), dfree_async(h->stage_del[b]), dfree_async(h->stage_vals[b]);
        if (h->stage_free[b]) cudaEventDestroy(h->stage_free[b]);
    }
    if (h->copy_done) cudaEventDestroy(h->copy_done);
    if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
    dfree_async(h->row_offset), dfree_async(h->col_index), dfree_async(h->view_vals), dfree_async(h->exp_keys),
        dfree_async(h->exp_vals);
    dfree_async(h->q_cnt), dfree_async(h->q_tmp), dfree_async(h->bfs_a), dfree_async(h->bfs_b),
        dfree_async(h->bfs_cnt);
    dfree_async(h->pr_deg), dfree_async(h->pr_contrib), dfree_async(h->pr_acc), dfree_async(h->pr_dangling);
    if (h->done_ev) cudaEventDestroy(h->done_ev);
    pinned_release(h->pin_word, 2 * sizeof(uint32_t));
    delete h;
    return LPMA_OK;
}

lpma_status_t lpma_create(const LpmaConfig *cfg, uint32_t num_vertices, lpma_stream_t stream, LpmaHandle **out) {
    if (!out) return LPMA_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    LpmaConfig c;
    if (cfg)
        c = *cfg;
    else
        lpma_config_default(&c);
    if (c.flags & LPMA_FLAG_GPMA) {
        // the flat array of gpma.cuh: keys src << 32 | dst, vertex ids below
        // 2^32 - 1 (the sentinel's column is all ones), segment length from
        // the size, no expiry, no concurrent mode
        if ((c.flags & ~(uint32_t)LPMA_FLAG_GPMA) || !(c.density_lower_root >= 0.0 && c.density_lower_root <= 1.0) ||
            c.density_upper_root != 1.0 || num_vertices == 0 || num_vertices > 0xFFFFFFFEu)
            return LPMA_ERR_INVALID_ARGUMENT;
        LpmaHandle *h = new LpmaHandle();
        h->cfg = c;
        h->V = num_vertices;
        const lpma_status_t r = gpma_create(num_vertices, c.density_lower_root, (cudaStream_t)stream, &h->gp);
        if (r != LPMA_OK) {
            delete h;
            return r;
        }
        *out = h;
        return LPMA_OK;
    }
    if (c.segment_length != 32 || c.key_format > 1 || !(c.density_lower_root >= 0.0 && c.density_lower_root <= 1.0) ||
        c.density_upper_root != 1.0)
        return LPMA_ERR_INVALID_ARGUMENT;
    if (num_vertices == 0 || num_vertices > NBR_END) return LPMA_ERR_INVALID_ARGUMENT;
    cudaStream_t s = (cudaStream_t)stream;
    LpmaHandle *h = new LpmaHandle();
    h->cfg = c;
    h->V = num_vertices;
    auto fail = [&](lpma_status_t r) {
        lpma_destroy(h);
        return r;
    };
    if (dalloc(&h->dst, 1) || pinned_alloc(&h->hst, sizeof(DevStatus)) ||
        pinned_alloc(&h->hinit, sizeof(DevStatus)) || dalloc(&h->sent, num_vertices) ||
        dalloc(&h->sort.hist, 8 * 256) || dalloc(&h->sort.counters, 16) || dalloc(&h->sort_err, 1))
        return fail(LPMA_ERR_OUT_OF_MEMORY);
    // batches up to coop_sort_max_keys() sort in one cooperative launch,
    // unless the handle shares the GPU with concurrent calls
    h->sort.bar = (c.flags & LPMA_FLAG_CONCURRENT) ? nullptr : h->sort.counters;
    h->sort.err = &h->dst->error;
    if (cudaHostGetDevicePointer((void **)&h->hst_dev, h->hst, 0) != cudaSuccess) {
        h->hst_dev = nullptr;  // the status then comes back by a copy
        cudaGetLastError();
    }
    std::memset(h->hinit, 0, sizeof(DevStatus));
    h->hinit->min_t_ins = 0xFFFFFFFFu;
    h->hinit->key_and = ~0ull;
    h->hinit->err_info[0] = 0xFFFFFFFFu;
    if (alloc_cap(h->c, std::min<uint32_t>(min_height(num_vertices) + 1, LPMA_MAX_HEIGHT), s) != cudaSuccess)
        return fail(LPMA_ERR_OUT_OF_MEMORY);
    // empty height-0 tree (init_rpma, rpma.cuh:1764-1795)
    h->H = 0;
    if (cudaStreamCreateWithFlags(&h->cap_stream, cudaStreamNonBlocking) ||
        cudaStreamCreateWithFlags(&h->side_stream, cudaStreamNonBlocking) ||
        cudaEventCreateWithFlags(&h->fork_ev, cudaEventDisableTiming) ||
        cudaEventCreateWithFlags(&h->join_ev, cudaEventDisableTiming) ||
        cudaEventCreateWithFlags(&h->front_ev, cudaEventDisableTiming) ||
        cudaEventCreateWithFlags(&h->front_ev_blk, cudaEventDisableTiming | cudaEventBlockingSync) ||
        cudaEventCreateWithFlags(&h->done_ev, cudaEventDisableTiming) || sort_prepare())
        return fail(LPMA_ERR_CUDA);
    if (cudaMemsetAsync(h->dst, 0, sizeof(DevStatus), s) || cudaMemsetAsync(h->c.keys, 0xFF, 32 * 8, s) ||
        cudaMemsetAsync(h->c.vals, 0, 32, s) ||
        cudaMemsetAsync(h->c.fl, 0xFF, sizeof(ulonglong2), s) || cudaMemsetAsync(h->sent, 0, 4ull * num_vertices, s))
        return fail(LPMA_ERR_CUDA);
    // the sentinels through the update path (init_csr_rpma, rpma.cuh:1819-1823)
    uint64_t *sk = nullptr;
    uint8_t *sv = nullptr;
    if (dalloc(&sk, num_vertices) || dalloc(&sv, num_vertices)) return fail(LPMA_ERR_OUT_OF_MEMORY);
    launch_sentinels(num_vertices, sk, sv, s);
    lpma_status_t r = do_update(h, sk, sv, num_vertices, nullptr, 0, 0, s, nullptr, true);
    cudaStreamSynchronize(s);
    dfree_async(sk);
    dfree_async(sv);
    if (r != LPMA_OK) return fail(r);
    h->min_t = 0xFFFFF;
    *out = h;
    return LPMA_OK;
}

lpma_status_t lpma_build(LpmaHandle *h, const uint64_t *d_keys, const uint8_t *d_vals, size_t n, lpma_stream_t stream) {
    if (!h) return LPMA_ERR_INVALID_ARGUMENT;
    if (h->gp) return gpma_update(h->gp, d_keys, d_vals, n, nullptr, 0, (cudaStream_t)stream, nullptr);
    return do_update(h, d_keys, d_vals, n, nullptr, 0, 0, (cudaStream_t)stream, nullptr, false);
}

lpma_status_t lpma_update(LpmaHandle *h, const uint64_t *d_ins, const uint8_t *d_ins_vals, size_t n_ins,
                          const uint64_t *d_del, size_t n_del, uint32_t thres, lpma_stream_t stream, LpmaStats *stats) {
    if (!h) return LPMA_ERR_INVALID_ARGUMENT;
    if (h->gp) {
        if (thres) return LPMA_ERR_INVALID_ARGUMENT;  // GPMA keys carry no timestamp
        return gpma_update(h->gp, d_ins, d_ins_vals, n_ins, d_del, n_del, (cudaStream_t)stream, stats);
    }
    return do_update(h, d_ins, d_ins_vals, n_ins, d_del, n_del, thres, (cudaStream_t)stream, stats, false);
}

lpma_status_t lpma_update_host(LpmaHandle *h, const uint64_t *h_ins, const uint8_t *h_ins_vals, size_t n_ins,
                               const uint64_t *h_del, size_t n_del, uint32_t thres, lpma_stream_t stream,
                               LpmaStats *stats) {
    if (!h) return LPMA_ERR_INVALID_ARGUMENT;
    if ((n_ins && !h_ins) || (n_del && !h_del)) return LPMA_ERR_INVALID_ARGUMENT;
    if (h->gp) {
        if (thres) return LPMA_ERR_INVALID_ARGUMENT;
        cudaStream_t s = (cudaStream_t)stream;
        uint64_t *di = nullptr, *dd = nullptr;
        uint8_t *dv = nullptr;
        if (pool_alloc((void **)&di, n_ins * 8 + 8, s) || pool_alloc((void **)&dd, n_del * 8 + 8, s) ||
            pool_alloc((void **)&dv, n_ins + 8, s))
            return LPMA_ERR_OUT_OF_MEMORY;
        lpma_status_t r = LPMA_OK;
        if ((n_ins && cudaMemcpyAsync(di, h_ins, n_ins * 8, cudaMemcpyHostToDevice, s)) ||
            (n_ins && h_ins_vals && cudaMemcpyAsync(dv, h_ins_vals, n_ins, cudaMemcpyHostToDevice, s)) ||
            (n_del && cudaMemcpyAsync(dd, h_del, n_del * 8, cudaMemcpyHostToDevice, s)))
            r = LPMA_ERR_CUDA;
        if (r == LPMA_OK) r = gpma_update(h->gp, di, h_ins_vals ? dv : nullptr, n_ins, dd, n_del, s, stats);
        cudaFreeAsync(di, s), cudaFreeAsync(dd, s), cudaFreeAsync(dv, s);
        if (stats) stats->h2d_bytes = n_ins * 8 + (h_ins_vals ? n_ins : 0) + n_del * 8;
        cudaStreamSynchronize(s);
        return r;
    }
    cudaStream_t s = (cudaStream_t)stream;
    if (h->sticky != LPMA_OK) return h->sticky;
    if (!h->copy_stream) {
        if (cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking) ||
            cudaEventCreateWithFlags(&h->copy_done, cudaEventDisableTiming) ||
            cudaEventCreateWithFlags(&h->stage_free[0], cudaEventDisableTiming) ||
            cudaEventCreateWithFlags(&h->stage_free[1], cudaEventDisableTiming))
            return LPMA_ERR_CUDA;
    }
    const size_t need = std::max(n_ins, n_del);
    if (need > h->stage_cap) {
        // no copy or front may still use the old sets
        if (cudaStreamSynchronize(s) || cudaStreamSynchronize(h->copy_stream)) return LPMA_ERR_CUDA;
        for (int b = 0; b < 2; b++) dfree(h->stage_ins[b]), dfree(h->stage_del[b]), dfree(h->stage_vals[b]);
        h->stage_cap = 0;
        size_t cap = need + need / 4;
        for (int b = 0; b < 2; b++)
            if (dalloc(&h->stage_ins[b], cap) || dalloc(&h->stage_del[b], cap) || dalloc(&h->stage_vals[b], cap))
                return LPMA_ERR_OUT_OF_MEMORY;
        h->stage_cap = cap;
    }
    // the copy waits only for the call before last (the one that read this
    // set); the front waits for the copy
    const int b = h->stage_next;
    h->stage_next ^= 1;
    cudaStream_t c = h->copy_stream;
    CK(cudaStreamWaitEvent(c, h->stage_free[b], 0));
    if (n_ins && cudaMemcpyAsync(h->stage_ins[b], h_ins, n_ins * 8, cudaMemcpyHostToDevice, c)) return LPMA_ERR_CUDA;
    if (n_ins && h_ins_vals && cudaMemcpyAsync(h->stage_vals[b], h_ins_vals, n_ins, cudaMemcpyHostToDevice, c))
        return LPMA_ERR_CUDA;
    if (n_del && cudaMemcpyAsync(h->stage_del[b], h_del, n_del * 8, cudaMemcpyHostToDevice, c)) return LPMA_ERR_CUDA;
    CK(cudaEventRecord(h->copy_done, c));
    CK(cudaStreamWaitEvent(s, h->copy_done, 0));
    h->h2d = n_ins * 8 + (h_ins_vals ? n_ins : 0) + n_del * 8;
    h->host_staged = true;
    const lpma_status_t r = do_update(h, h->stage_ins[b], h_ins_vals ? h->stage_vals[b] : nullptr, n_ins,
                                      h->stage_del[b], n_del, thres, s, stats, false);
    CK(cudaEventRecord(h->stage_free[b], s));
    // a call that ended before its front ran has not waited for the copy;
    // the caller may reuse the host batch once the call returns
    if (r != LPMA_OK) cudaEventSynchronize(h->copy_done);
    return r;
}

static lpma_status_t fill_view(LpmaHandle *h, cudaStream_t s, bool csr, bool exp) {
    const uint64_t nseg = nseg_of(h->H);
    const size_t nnz = h->total;
    if (csr && nnz + 1 > h->view_cap) {
        dfree(h->row_offset), dfree(h->col_index), dfree(h->view_vals);
        h->view_cap = 0;
        if (dalloc(&h->row_offset, h->V + 1) || dalloc(&h->col_index, nnz + 1) || dalloc(&h->view_vals, nnz + 1))
            return LPMA_ERR_OUT_OF_MEMORY;
        h->view_cap = nnz + 1;
    }
    if (exp && nnz + 1 > h->exp_cap) {
        dfree(h->exp_keys), dfree(h->exp_vals);
        h->exp_cap = 0;
        if (dalloc(&h->exp_keys, nnz + 1) || dalloc(&h->exp_vals, nnz + 1)) return LPMA_ERR_OUT_OF_MEMORY;
        h->exp_cap = nnz + 1;
    }
    CK(scan_u8_to_u32(h->c.cnt, h->c.segP, (uint32_t)nseg, h->c.segP + nseg, h->c.scan_tmp, s));
    if (csr) CK(cudaMemsetAsync(h->row_offset, 0, 4ull * (h->V + 1), s));
    Geo g{h->c.keys, h->c.vals, h->H};
    launch_csr_fill(g, h->c.cnt, h->c.segP, csr ? h->row_offset : nullptr, csr ? h->col_index : nullptr,
                    csr ? h->view_vals : nullptr, exp ? h->exp_keys : nullptr, exp ? h->exp_vals : nullptr, s);
    CK(cudaGetLastError());
    return LPMA_OK;
}

lpma_status_t lpma_csr_view(LpmaHandle *h, const uint32_t **row_offset, const uint32_t **col_index,
                            const uint8_t **values, size_t *nnz, lpma_stream_t stream) {
    if (!h || !row_offset || !col_index || !nnz) return LPMA_ERR_INVALID_ARGUMENT;
    if (h->gp) return LPMA_ERR_INVALID_ARGUMENT;  // not offered for the flat GPMA layout
    if (h->sticky != LPMA_OK) return h->sticky;
    cudaStream_t s = (cudaStream_t)stream;
    if (!h->view_valid) {
        CKS(fill_view(h, s, true, false));
        h->view_valid = true;
        mark_done(h, s);
    }
    *row_offset = h->row_offset;
    *col_index = h->col_index;
    if (values) *values = h->view_vals;
    *nnz = h->total;
    return LPMA_OK;
}

lpma_status_t lpma_to_csr(LpmaHandle *h, uint32_t *row_offset, uint32_t *col_index, uint8_t *values, size_t cap,
                          size_t *nnz, lpma_stream_t stream) {
    if (!h || !nnz) return LPMA_ERR_INVALID_ARGUMENT;
    if (h->gp) return LPMA_ERR_INVALID_ARGUMENT;  // not offered for the flat GPMA layout
    const uint32_t *ro, *ci;
    const uint8_t *va;
    size_t n;
    lpma_status_t r = lpma_csr_view(h, &ro, &ci, &va, &n, stream);
    if (r != LPMA_OK) return r;
    *nnz = n;
    if (!row_offset && !col_index && !values) return LPMA_OK;
    if ((col_index || values) && cap < n) return LPMA_ERR_BUFFER_TOO_SMALL;
    cudaStream_t s = (cudaStream_t)stream;
    if (row_offset) CK(cudaMemcpyAsync(row_offset, ro, 4ull * (h->V + 1), cudaMemcpyDefault, s));
    if (col_index) CK(cudaMemcpyAsync(col_index, ci, 4 * n, cudaMemcpyDefault, s));
    if (values) CK(cudaMemcpyAsync(values, va, n, cudaMemcpyDefault, s));
    CK(cudaStreamSynchronize(s));
    return LPMA_OK;
}

lpma_status_t lpma_export_sorted(LpmaHandle *h, uint64_t *h_keys, uint8_t *h_vals, size_t cap, size_t *n,
                                 lpma_stream_t stream) {
    if (!h || !n) return LPMA_ERR_INVALID_ARGUMENT;
    if (h->gp) {
        uint64_t items = 0;
        gpma_geometry(h->gp, nullptr, nullptr, nullptr, &items);
        *n = items;
        if (!h_keys) return LPMA_OK;
        return gpma_export_sorted(h->gp, h_keys, h_vals, cap, n, (cudaStream_t)stream);
    }
    if (h->sticky != LPMA_OK) return h->sticky;
    *n = h->total;
    if (!h_keys) return LPMA_OK;
    if (cap < h->total) return LPMA_ERR_BUFFER_TOO_SMALL;
    cudaStream_t s = (cudaStream_t)stream;
    CKS(fill_view(h, s, false, true));
    CK(cudaMemcpyAsync(h_keys, h->exp_keys, h->total * 8, cudaMemcpyDeviceToHost, s));
    if (h_vals) CK(cudaMemcpyAsync(h_vals, h->exp_vals, h->total, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return LPMA_OK;
}

lpma_status_t lpma_export_layout(LpmaHandle *h, uint64_t *h_keys, uint8_t *h_vals, size_t cap_slots,
                                 uint32_t *sentinel_slots, size_t cap_vertices, uint32_t *height,
                                 lpma_stream_t stream) {
    if (!h) return LPMA_ERR_INVALID_ARGUMENT;
    if (h->gp) {
        // the flat array; sentinel_slots[v] = row_offset[v + 1], the slot of v's sentinel
        uint64_t size = 0;
        uint32_t hh = 0;
        gpma_geometry(h->gp, &size, nullptr, &hh, nullptr);
        if (height) *height = hh;
        if (sentinel_slots && cap_vertices < h->V) return LPMA_ERR_BUFFER_TOO_SMALL;
        std::vector<uint32_t> ro(sentinel_slots ? (size_t)h->V + 1 : 0);
        const lpma_status_t r = gpma_export_layout(h->gp, h_keys, h_vals, h_keys ? cap_slots : size,
                                                   sentinel_slots ? ro.data() : nullptr, ro.size(), (cudaStream_t)stream);
        if (r == LPMA_OK && sentinel_slots) std::memcpy(sentinel_slots, ro.data() + 1, 4ull * h->V);
        return r;
    }
    if (h->sticky != LPMA_OK) return h->sticky;
    if (height) *height = h->H;
    const uint64_t ns = nslots_of(h->H);
    cudaStream_t s = (cudaStream_t)stream;
    if (h_keys) {
        if (cap_slots < ns) return LPMA_ERR_BUFFER_TOO_SMALL;
        CK(cudaMemcpyAsync(h_keys, h->c.keys, ns * 8, cudaMemcpyDeviceToHost, s));
        if (h_vals) CK(cudaMemcpyAsync(h_vals, h->c.vals, ns, cudaMemcpyDeviceToHost, s));
    }
    if (sentinel_slots) {
        if (cap_vertices < h->V) return LPMA_ERR_BUFFER_TOO_SMALL;
        CK(cudaMemcpyAsync(sentinel_slots, h->sent, 4ull * h->V, cudaMemcpyDeviceToHost, s));
    }
    CK(cudaStreamSynchronize(s));
    if (h_keys && h_vals)
        for (uint64_t i = 0; i < ns; i++)
            if (h_keys[i] == KEY_NONE) h_vals[i] = 0;
    return LPMA_OK;
}

lpma_status_t lpma_info(const LpmaHandle *h, uint32_t *height, uint64_t *num_items, uint32_t *num_vertices) {
    if (!h) return LPMA_ERR_INVALID_ARGUMENT;
    if (h->gp) {
        if (num_vertices) *num_vertices = h->V;
        return gpma_geometry(h->gp, nullptr, nullptr, height, num_items);
    }
    if (height) *height = h->H;
    if (num_items) *num_items = h->total;
    if (num_vertices) *num_vertices = h->V;
    return LPMA_OK;
}

lpma_status_t lpma_query_neighbors(LpmaHandle *h, const uint32_t *d_srcs, const uint64_t *d_windows, size_t n,
                                   uint32_t *d_offsets, uint32_t *d_nbrs, uint8_t *d_vals, size_t cap, size_t *total,
                                   lpma_stream_t stream) {
    if (!h || !total || (n && (!d_srcs || !d_windows)) || !d_offsets || (d_nbrs && !d_vals))
        return LPMA_ERR_INVALID_ARGUMENT;
    if (h->gp) return LPMA_ERR_INVALID_ARGUMENT;  // not offered for the flat GPMA layout
    if (n >= (1u << 30)) return LPMA_ERR_INVALID_ARGUMENT;
    if (h->sticky != LPMA_OK) return h->sticky;
    cudaStream_t s = (cudaStream_t)stream;
    if (!h->pin_word) CK(pinned_alloc(&h->pin_word, 2 * sizeof(uint32_t)));
    if (n > h->q_cap) {
        dfree(h->q_cnt), dfree(h->q_tmp);
        h->q_cap = 0;
        const size_t c = std::max<size_t>(n, 1024);
        CK(dalloc(&h->q_cnt, c));
        CK(dalloc(&h->q_tmp, scan_tmp_words((uint32_t)c) + 64));
        h->q_cap = c;
    }
    Geo g{h->c.keys, h->c.vals, h->H};
    if (n) {
        launch_nbr_count(d_srcs, d_windows, (uint32_t)n, g, h->c.cnt, h->sent, h->V, h->q_cnt, s);
        CK(scan_u32(h->q_cnt, d_offsets, (uint32_t)n, d_offsets + n, h->q_tmp, s));
    } else {
        CK(cudaMemsetAsync(d_offsets, 0, sizeof(uint32_t), s));
    }
    CK(cudaMemcpyAsync(h->pin_word, d_offsets + n, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    CK(host_wait(s, blocking_waits(h)));
    *total = h->pin_word[0];
    if (!d_nbrs || !n) return LPMA_OK;
    if (*total > cap) return LPMA_ERR_BUFFER_TOO_SMALL;
    launch_nbr_fill(d_srcs, d_windows, (uint32_t)n, g, h->c.cnt, h->sent, h->V, d_offsets, d_nbrs, d_vals, s);
    CK(cudaGetLastError());
    mark_done(h, s);
    return LPMA_OK;
}

lpma_status_t lpma_edge_query(LpmaHandle *h, const uint64_t *d_keys, size_t n, uint32_t window, uint32_t *d_counts,
                              lpma_stream_t stream) {
    if (!h || (n && (!d_keys || !d_counts)) || n >= (1u << 31)) return LPMA_ERR_INVALID_ARGUMENT;
    if (h->gp) return LPMA_ERR_INVALID_ARGUMENT;  // not offered for the flat GPMA layout
    if (h->sticky != LPMA_OK) return h->sticky;
    if (!n) return LPMA_OK;
    launch_edge_query(d_keys, (uint32_t)n, window, Geo{h->c.keys, h->c.vals, h->H}, h->c.cnt, h->c.fl, h->sent, h->V,
                      d_counts, (cudaStream_t)stream);
    CK(cudaGetLastError());
    mark_done(h, (cudaStream_t)stream);
    return LPMA_OK;
}

lpma_status_t lpma_bfs(LpmaHandle *h, const uint32_t *d_sources, size_t n_sources, uint32_t max_depth, int32_t *d_dist,
                       uint32_t *levels, uint64_t *reached, lpma_stream_t stream) {
    if (!h || !d_dist || (n_sources && !d_sources) || n_sources >= (1u << 31)) return LPMA_ERR_INVALID_ARGUMENT;
    if (h->gp) return LPMA_ERR_INVALID_ARGUMENT;  // not offered for the flat GPMA layout
    if (h->sticky != LPMA_OK) return h->sticky;
    cudaStream_t s = (cudaStream_t)stream;
    if (!h->pin_word) CK(pinned_alloc(&h->pin_word, 2 * sizeof(uint32_t)));
    if (!h->bfs_a) {
        CK(dalloc(&h->bfs_a, h->V));
        CK(dalloc(&h->bfs_b, h->V));
        CK(dalloc(&h->bfs_cnt, 2));
    }
    CK(cudaMemsetAsync(h->bfs_cnt, 0, 2 * sizeof(uint32_t), s));
    launch_bfs_init(d_sources, (uint32_t)n_sources, h->V, d_dist, h->bfs_a, h->bfs_cnt, s);
    CK(cudaMemcpyAsync(h->pin_word, h->bfs_cnt, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    CK(host_wait(s, blocking_waits(h)));
    uint32_t nf = h->pin_word[0], lv = 0;
    uint64_t total = nf;
    uint32_t *cur = h->bfs_a, *nxt = h->bfs_b;
    const Geo g{h->c.keys, h->c.vals, h->H};
    while (nf > 0 && (max_depth == 0 || lv < max_depth)) {
        CK(cudaMemsetAsync(h->bfs_cnt + 1, 0, sizeof(uint32_t), s));
        launch_bfs_expand(cur, h->bfs_cnt, nf, (int32_t)lv, g, h->c.cnt, h->sent, d_dist, nxt, h->bfs_cnt + 1, s);
        CK(cudaMemcpyAsync(h->bfs_cnt, h->bfs_cnt + 1, sizeof(uint32_t), cudaMemcpyDeviceToDevice, s));
        CK(cudaMemcpyAsync(h->pin_word, h->bfs_cnt + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        CK(host_wait(s, blocking_waits(h)));
        nf = h->pin_word[0];
        total += nf;
        lv++;
        std::swap(cur, nxt);
    }
    if (levels) *levels = lv;
    if (reached) *reached = total;
    return LPMA_OK;
}

lpma_status_t lpma_pagerank(LpmaHandle *h, double alpha, uint32_t iterations, double *d_rank, lpma_stream_t stream) {
    if (!h || !d_rank || !(alpha >= 0.0 && alpha <= 1.0)) return LPMA_ERR_INVALID_ARGUMENT;
    if (h->gp) return LPMA_ERR_INVALID_ARGUMENT;  // not offered for the flat GPMA layout
    if (h->sticky != LPMA_OK) return h->sticky;
    cudaStream_t s = (cudaStream_t)stream;
    if (!h->pr_deg) {
        CK(dalloc(&h->pr_deg, h->V));
        CK(dalloc(&h->pr_contrib, h->V));
        CK(dalloc(&h->pr_acc, h->V));
        CK(dalloc(&h->pr_dangling, 1));
    }
    const Geo g{h->c.keys, h->c.vals, h->H};
    CK(cudaMemsetAsync(h->pr_deg, 0, sizeof(uint32_t) * h->V, s));
    CK(cudaMemsetAsync(h->pr_acc, 0, sizeof(double) * h->V, s));
    launch_outdeg(g, h->c.cnt, h->pr_deg, s);
    launch_fill_f64(d_rank, h->V, 1.0 / (double)h->V, s);
    for (uint32_t it = 0; it < iterations; it++)
        launch_pr_iteration(g, h->c.cnt, h->pr_deg, h->V, alpha, d_rank, h->pr_contrib, h->pr_acc, h->pr_dangling, s);
    CK(cudaGetLastError());
    mark_done(h, s);
    return LPMA_OK;
}

lpma_status_t lpma_error_detail(const LpmaHandle *h, uint32_t *site) {
    if (!h || !site) return LPMA_ERR_INVALID_ARGUMENT;
    *site = h->hst ? h->hst->sticky_site : 0u;
    return LPMA_OK;
}

lpma_status_t lpma_set_flags(LpmaHandle *h, uint32_t flags) {
    if (!h || (flags & ~(uint32_t)LPMA_FLAG_CONCURRENT)) return LPMA_ERR_INVALID_ARGUMENT;
    if (h->gp) return LPMA_ERR_INVALID_ARGUMENT;  // the layout is fixed at creation
    h->cfg.flags = flags;
    h->sort.bar = (flags & LPMA_FLAG_CONCURRENT) ? nullptr : h->sort.counters;
    return LPMA_OK;  // cached fronts are keyed by the sort mode
}

lpma_status_t lpma_memory_reserve(uint64_t bytes, lpma_stream_t stream) {
    cudaMemPool_t pool = batch_pool();
    if (!pool) return LPMA_ERR_CUDA;
    if (bytes == 0) return LPMA_OK;
    cudaStream_t s = (cudaStream_t)stream;
    void *p = nullptr;
    const cudaError_t e = cudaMallocFromPoolAsync(&p, (size_t)bytes, pool, s);
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return LPMA_ERR_OUT_OF_MEMORY;
    }
    CK(e);
    CK(cudaFreeAsync(p, s));
    CK(cudaStreamSynchronize(s));
    return LPMA_OK;
}

lpma_status_t lpma_memory_bytes(const LpmaHandle *h, uint64_t *bytes) {
    if (!h || !bytes) return LPMA_ERR_INVALID_ARGUMENT;
    if (h->gp) {
        *bytes = gpma_memory_bytes(h->gp);
        return LPMA_OK;
    }
    uint64_t b = 0;
    if (h->c.Hc || h->c.keys) {
        const uint64_t ns = nslots_of(h->c.Hc), nseg = nseg_of(h->c.Hc);
        b += 18 * ns + nseg * (4 + 16 + 7 * 4) + bitmap_words(h->c.Hc) * 4;
    }
    b += 4ull * h->V + h->bcap * 64ull + h->view_cap * 9ull + h->exp_cap * 9ull + h->stage_cap * 34ull;
    if (h->bfs_a) b += 8ull * h->V;
    if (h->pr_deg) b += 20ull * h->V;
    b += h->q_cap * 8ull;
    *bytes = b;
    return LPMA_OK;
}

lpma_status_t lpma_batcher_create(LpmaBatcher **out) {
    if (!out) return LPMA_ERR_INVALID_ARGUMENT;
    *out = new LpmaBatcher();
    return LPMA_OK;
}

lpma_status_t lpma_batcher_destroy(LpmaBatcher *b) {
    if (!b) return LPMA_ERR_INVALID_ARGUMENT;
    // wait for the batcher's own work: the shared executors of its last call
    // (the done event), its side stream and its worker threads' streams
    if (b->pending && b->done) cudaEventSynchronize(b->done);
    if (b->side) cudaStreamSynchronize(b->side);
    if (b->workers)
        for (cudaStream_t x : b->workers->st)
            if (x) cudaStreamSynchronize(x);
    delete b->workers;
    batcher_free(b, true);
    if (b->done) cudaEventDestroy(b->done);
    if (b->fork_ev) cudaEventDestroy(b->fork_ev);
    if (b->join_ev) cudaEventDestroy(b->join_ev);
    if (b->side) cudaStreamDestroy(b->side);
    delete b;
    return LPMA_OK;
}

lpma_status_t lpma_update_batch(LpmaBatcher *b, LpmaHandle *const *graphs, const LpmaBatch *items, size_t n,
                                lpma_stream_t stream, LpmaStats *stats, lpma_status_t *status) {
    if (!b || (n && (!graphs || !items)) || n > (1u << 20)) return LPMA_ERR_INVALID_ARGUMENT;
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<lpma_status_t> res(n, LPMA_OK);
    std::vector<LpmaStats> sts(n);
    std::vector<size_t> forest, plain;
    std::vector<LpmaHandle *> seen;
    seen.reserve(n);
    for (size_t i = 0; i < n; i++) {
        LpmaHandle *h = graphs[i];
        const LpmaBatch &it = items[i];
        sts[i] = LpmaStats{};
        if (!h || h->gp || (it.n_ins && !it.ins) || (it.n_del && !it.del)) {  // leveled graphs only
            res[i] = LPMA_ERR_INVALID_ARGUMENT;
            continue;
        }
        if (std::find(seen.begin(), seen.end(), h) != seen.end()) {  // one batch per graph per call
            res[i] = LPMA_ERR_INVALID_ARGUMENT;
            continue;
        }
        seen.push_back(h);
        if (h->sticky != LPMA_OK) {
            res[i] = h->sticky;
            continue;
        }
        const size_t m = it.n_ins + it.n_del;
        sts[i].height_before = sts[i].height_after = h->H;
        sts[i].num_items = h->total;
        if (m == 0) continue;
        // the shared launches take batches without expiry that one CTA sorts
        // and whose first level loop plans from segment counts alone
        if (it.thres == 0 && m <= FOREST_SORT_MAX && !needs_prefix(make_tables(h, h->H, true), h->H) &&
            min_height(h->total + it.n_ins) <= LPMA_MAX_HEIGHT)
            forest.push_back(i);
        else
            plain.push_back(i);
    }
    lpma_status_t r = LPMA_OK;
    const uint32_t G = (uint32_t)forest.size();
    if (G) {
        // the previous call's shared executors read the tables rewritten below
        if (b->pending) {
            CK(cudaEventSynchronize(b->done));
            b->pending = false;
        }
        if ((r = batcher_reserve(b, G)) != LPMA_OK) return r;
        uint32_t *boff = b->hB, nblk[FOREST_TABLES] = {}, rounds = 0;
        std::vector<size_t> ready;
        for (uint32_t k = 0; k < G; k++) {
            const size_t i = forest[k];
            LpmaHandle *h = graphs[i];
            const LpmaBatch &it = items[i];
            const size_t m = it.n_ins + it.n_del;
            if ((res[i] = ensure_batch(h, m, s)) != LPMA_OK) return res[i];
        }
        for (uint32_t k = 0; k < G; k++) {
            const size_t i = forest[k];
            LpmaHandle *h = graphs[i];
            const LpmaBatch &it = items[i];
            const uint32_t m = (uint32_t)(it.n_ins + it.n_del);
            h->view_valid = false;
            h->h2d = sizeof(ForestGraph);
            h->d2h = sizeof(DevStatus);
            ForestGraph &f = b->hF[k];
            f = ForestGraph{};
            f.g = Geo{h->c.keys, h->c.vals, h->H};
            f.fl = h->c.fl;
            f.cnt = h->c.cnt;
            f.V = h->V;
            f.key_format = h->cfg.key_format;
            f.ins = it.ins, f.ins_vals = it.ins_vals, f.del = it.del;
            f.n_ins = (uint32_t)it.n_ins, f.n_del = (uint32_t)it.n_del;
            f.bk0 = h->bk0, f.bp0 = h->bp0, f.kind = h->kind, f.seg = h->seg;
            f.blk_nn = h->blk_nn, f.blk_ins = h->blk_ins, f.u = h->u;
            f.bitmap = h->c.bitmap, f.bitmap_words = bitmap_words(h->H);
            f.sup = h->sup, f.sup_words = sup_words_for(m);
            f.cand = h->cand, f.wsingle = h->wsingle, f.wsmall4 = h->wsmall4, f.wsmall = h->wsmall, f.wbig = h->wbig;
            f.pend = h->pend;
            f.tb = make_tables(h, h->H, true);
            f.total_items = h->total;
            f.st = h->dst;
            b->hJ[k] = ForestSortJob{h->bk0, h->bk1, h->bp0, h->bp1, &h->dst->key_and, m, tm_tile_forest(m)};
            const uint32_t rk = forest_sort_rounds(m);
            rounds = std::max(rounds, rk);
            f.sk = (rk & 1) ? h->bk1 : h->bk0;
            f.sp = (rk & 1) ? h->bp1 : h->bp0;
            const uint32_t chunks = (m + 255) / 256;
            // pack strides over its keys; resolve stages the top of the tree
            // once per CTA, so each of its CTAs takes 8 or more chunks
            uint32_t per[FOREST_TABLES] = {std::min<uint32_t>(chunks, 64),
                                           std::min<uint32_t>(chunks, std::max<uint32_t>(8, (chunks + 7) / 8)),
                                           chunks, chunks, chunks, m > 1 ? forest_sort_tiles(m) : 0};
            for (uint32_t r = 0; r < rk; r++) per[6 + r] = forest_merge_ctas(m);
            for (int ph = 0; ph < FOREST_TABLES; ph++) {
                boff[ph * (G + 1) + k] = nblk[ph];
                nblk[ph] += per[ph];
            }
        }
        for (int ph = 0; ph < FOREST_TABLES; ph++) boff[ph * (G + 1) + G] = nblk[ph];
        CK(cudaMemcpyAsync(b->dF, b->hF, G * sizeof(ForestGraph), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(b->dB, b->hB, FOREST_TABLES * (G + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(b->dJ, b->hJ, G * sizeof(ForestSortJob), cudaMemcpyHostToDevice, s));
        const uint32_t *B = b->dB;
        launch_forest_phase(0, b->dF, nullptr, G, G, nullptr, s);
        launch_forest_phase(1, b->dF, B, G, nblk[0], nullptr, s);
        CK(forest_sort(b->dJ, G, B + 5 * (G + 1), nblk + 5, rounds, s));
        launch_forest_phase(2, b->dF, B + (G + 1), G, nblk[1], nullptr, s);
        launch_forest_phase(3, b->dF, B + 2 * (G + 1), G, nblk[2], nullptr, s);
        launch_forest_phase(4, b->dF, B + 3 * (G + 1), G, nblk[3], nullptr, s);
        launch_forest_phase(5, b->dF, B + 4 * (G + 1), G, nblk[4], nullptr, s);
        launch_forest_phase(6, b->dF, nullptr, G, G, b->dS, s);
        CK(cudaMemcpyAsync(b->hS, b->dS, G * sizeof(DevStatus), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        CK(cudaGetLastError());
        // graphs whose first loop needs only the common executors (no
        // error, no overflow, no window of 2^6+ segments): one launch per
        // executor over all of them
        std::vector<uint8_t> shared(G, 0);
        uint32_t GS = 0, xblk[3] = {0, 0, 0};
        uint32_t *xoff = b->hX;
        for (uint32_t k = 0; k < G; k++) {
            const DevStatus &d = b->hS[k];
            if ((d.error | d.sticky) || d.n_u == 0 || d.ovf || d.n_big) continue;
            LpmaHandle *h = graphs[forest[k]];
            shared[k] = 1;
            ForestExec &e = b->hE[GS];
            e = ForestExec{};
            e.g = Geo{h->c.keys, h->c.vals, h->H};
            e.cnt = h->c.cnt, e.fl = h->c.fl, e.sent = h->sent, e.V = h->V;
            e.n[0] = d.n_single, e.n[1] = d.n_small4, e.n[2] = d.n_small;
            e.w[0] = h->wsingle, e.w[1] = h->wsmall4, e.w[2] = h->wsmall;
            e.u = h->u;
            e.st = h->dst;
            for (int kind = 0; kind < 3; kind++) {
                xoff[kind * (G + 1) + GS] = xblk[kind];
                xblk[kind] += exec_ctas(kind, e.n[kind]);
            }
            GS++;
        }
        if (GS) {
            for (int kind = 0; kind < 3; kind++) {
                xoff[kind * (G + 1) + GS] = xblk[kind];
                if (kind) memmove(xoff + kind * (GS + 1), xoff + kind * (G + 1), (GS + 1) * sizeof(uint32_t));
            }
            CK(cudaMemcpyAsync(b->dE, b->hE, GS * sizeof(ForestExec), cudaMemcpyHostToDevice, s));
            CK(cudaMemcpyAsync(b->dX, b->hX, 3 * (GS + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
            if (!b->side) {
                CK(cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking));
                CK(cudaEventCreateWithFlags(&b->fork_ev, cudaEventDisableTiming));
                CK(cudaEventCreateWithFlags(&b->join_ev, cudaEventDisableTiming));
            }
            // one stream while the in-library profiler times each kernel
            const bool fork = !prof_enabled();
            cudaStream_t side = fork ? b->side : s;
            if (fork) {
                CK(cudaEventRecord(b->fork_ev, s));
                CK(cudaStreamWaitEvent(side, b->fork_ev, 0));
            }
            for (int kind = 1; kind < 3; kind++)
                launch_forest_exec(kind, b->dE, b->dX + kind * (GS + 1), GS, xblk[kind], side);
            if (fork) CK(cudaEventRecord(b->join_ev, side));
            launch_forest_exec(0, b->dE, b->dX, GS, xblk[0], s);
            if (fork) CK(cudaStreamWaitEvent(s, b->join_ev, 0));
            if (!b->done) CK(cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming));
            CK(cudaEventRecord(b->done, s));
            b->pending = true;
        }
        // each graph goes on as after its own front: first those of the
        // shared executors (host work, maybe an eager level-up), then the
        // rest, whose paths wait on the device, on several host threads
        std::vector<uint32_t> rest;
        auto finish = [&](uint32_t k, cudaStream_t st) {
            const size_t i = forest[k];
            LpmaHandle *h = graphs[i];
            memcpy(h->hst, &b->hS[k], sizeof(DevStatus));
            const uint32_t e = h->hst->error | h->hst->sticky;
            const lpma_status_t rs = (e & ERR_TIMEOUT) ? LPMA_ERR_TIMEOUT
                                                       : ((e & ERR_INTERNAL) ? LPMA_ERR_INTERNAL : LPMA_OK);
            sts[i].height_before = h->H;
            h->front_sort_wide = false;  // the shared tile-merge sort
            res[i] = finish_update(h, rs, items[i].n_ins + items[i].n_del, 0, false, st, sts[i], &sts[i],
                                   shared[k] != 0);
        };
        for (uint32_t k = 0; k < G; k++) {
            if (shared[k])
                finish(k, s);
            else
                rest.push_back(k);
        }
        if (rest.size() > 1 && !prof_enabled()) {
            if (!b->workers) {
                b->workers = new BatchWorkers();
                const unsigned hw = std::thread::hardware_concurrency();
                CK(b->workers->start((int)std::max(1u, std::min(7u, hw > 1 ? hw - 1 : 1u))));
            }
            b->workers->run(rest.size(), s, [&](size_t j, cudaStream_t st) { finish(rest[j], st); });
        } else {
            for (uint32_t k : rest) finish(k, s);
        }
    }
    for (size_t i : plain) {
        const LpmaBatch &it = items[i];
        res[i] = do_update(graphs[i], it.ins, it.ins_vals, it.n_ins, it.del, it.n_del, it.thres, s, &sts[i], false);
    }
    for (size_t i = 0; i < n; i++) {
        if (stats) stats[i] = sts[i];
        if (status) status[i] = res[i];
        if (r == LPMA_OK && res[i] != LPMA_OK) r = res[i];
    }
    return r;
}

const char *lpma_status_string(lpma_status_t s) {
    switch (s) {
        case LPMA_OK: return "ok";
        case LPMA_ERR_INVALID_ARGUMENT: return "invalid argument";
        case LPMA_ERR_INVALID_KEY: return "invalid key in batch";
        case LPMA_ERR_OUT_OF_MEMORY: return "out of device memory";
        case LPMA_ERR_CUDA: return "CUDA runtime error";
        case LPMA_ERR_CAPACITY: return "tree height limit exceeded";
        case LPMA_ERR_INTERNAL: return "internal consistency check failed";
        case LPMA_ERR_TIMEOUT: return "bounded device wait gave up";
        case LPMA_ERR_BUFFER_TOO_SMALL: return "buffer too small";
        case LPMA_ERR_SCRATCH_LIMIT: return "n exceeds the fixed scratch of this entry point";
        case LPMA_ERR_IO: return "file missing, unreadable or malformed";
    }
    return "unknown status";
}

uint64_t lpma_kernel_launches(void) { return lpma::launch_count(); }

lpma_status_t lpma_prof_enable(int on) {
    lpma::prof_enable(on);
    return LPMA_OK;
}

size_t lpma_prof_report(char *buf, size_t cap) { return lpma::prof_report(buf, cap); }

lpma_status_t lpma_gen_rmat(uint64_t seed, uint32_t scale, uint32_t edge_factor, uint32_t ta, uint32_t tab,
                            uint32_t tabc, uint64_t *d_out, size_t cap, size_t *n_out, lpma_stream_t stream) {
    if (!d_out || !n_out || scale == 0 || scale > 22) return LPMA_ERR_INVALID_ARGUMENT;
    const uint64_t n = (1ull << scale) * edge_factor;
    if (n >= (1ull << 30)) return LPMA_ERR_INVALID_ARGUMENT;
    if (cap < n) return LPMA_ERR_BUFFER_TOO_SMALL;
    cudaStream_t s = (cudaStream_t)stream;
    uint64_t *tmp = nullptr;
    uint16_t *p0 = nullptr, *p1 = nullptr;
    uint32_t *flags = nullptr, *pos = nullptr, *total = nullptr, *stmp = nullptr, *err = nullptr;
    SortScratch ss;
    ss.status_words = sort_status_words((uint32_t)n);
    lpma_status_t r = LPMA_OK;
    if (dalloc(&tmp, n) || dalloc(&p0, n) || dalloc(&p1, n) || dalloc(&flags, n) || dalloc(&pos, n) ||
        dalloc(&total, 1) || dalloc(&stmp, scan_tmp_words((uint32_t)n) + 64) || dalloc(&err, 1) ||
        dalloc(&ss.status, ss.status_words) || dalloc(&ss.hist, 8 * 256) || dalloc(&ss.counters, 16)) {
        r = LPMA_ERR_OUT_OF_MEMORY;
    } else {
        cudaMemsetAsync(p0, 0, n * 2, s);
        cudaMemsetAsync(err, 0, 4, s);
        launch_rmat(seed, scale, n, ta, tab, tabc, d_out, s);
        int which = 0;
        cudaError_t e = sort_pairs<uint16_t>(d_out, p0, tmp, p1, (uint32_t)n, ~0ull, ss, err, s, &which);
        uint64_t *sorted = which ? tmp : d_out;
        uint64_t *other = which ? d_out : tmp;
        if (!e) {
            launch_unique_flags(sorted, n, flags, s);
            e = scan_u32(flags, pos, (uint32_t)n, total, stmp, s);
        }
        if (!e) {
            launch_scatter_flags(sorted, pos, flags, n, other, s);
            if (other != d_out) e = cudaMemcpyAsync(d_out, other, n * 8, cudaMemcpyDeviceToDevice, s);
        }
        uint32_t tot = 0, herr = 0;
        if (!e) e = cudaMemcpyAsync(&tot, total, 4, cudaMemcpyDeviceToHost, s);
        if (!e) e = cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, s);
        if (!e) e = cudaStreamSynchronize(s);
        if (e)
            r = cuda_fail(e);
        else if (herr)
            r = LPMA_ERR_TIMEOUT;
        *n_out = tot;
    }
    cudaStreamSynchronize(s);
    dfree(tmp), dfree(p0), dfree(p1), dfree(flags), dfree(pos), dfree(total), dfree(stmp), dfree(err);
    dfree(ss.status), dfree(ss.hist), dfree(ss.counters);
    return r;
}

lpma_status_t lpma_debug_sort_barrier(uint32_t poll_limit, int unreachable) {
    CK(set_barrier_debug(poll_limit, unreachable ? 1u : 0u));
    return LPMA_OK;
}

lpma_status_t lpma_debug_exec_wait(int give_up) {
    CK(set_exec_wait_debug(give_up ? 1u : 0u));
    return LPMA_OK;
}

lpma_status_t lpma_tune_set(uint32_t log2_keys, uint32_t concurrent, uint32_t tier) {
    if (log2_keys > 32 || tier >= TIER_COUNT) return LPMA_ERR_INVALID_ARGUMENT;
    sort_tier_set(log2_keys, concurrent ? 1 : 0, (SortTier)tier);
    return LPMA_OK;
}

lpma_status_t lpma_tune_get(uint32_t log2_keys, uint32_t concurrent, uint32_t *tier) {
    if (log2_keys > 32 || !tier) return LPMA_ERR_INVALID_ARGUMENT;
    *tier = (uint32_t)sort_tier_get(log2_keys, concurrent ? 1 : 0);
    return LPMA_OK;
}

lpma_status_t lpma_grain_set(uint32_t log2_keys, uint32_t max_segs_group, uint32_t max_segs_shared) {
    if (log2_keys > 32) return LPMA_ERR_INVALID_ARGUMENT;
    if (max_segs_group == 0 && max_segs_shared == 0) {
        g_grain[log2_keys].store(0, std::memory_order_relaxed);
        return LPMA_OK;
    }
    if (max_segs_group < 1 || max_segs_group > CUT_GROUP_MAX || max_segs_shared < max_segs_group ||
        max_segs_shared > SMALL_WIN_SEGS)
        return LPMA_ERR_INVALID_ARGUMENT;
    g_grain[log2_keys].store(max_segs_group | (max_segs_shared << 8), std::memory_order_relaxed);
    return LPMA_OK;
}

lpma_status_t lpma_grain_get(uint32_t log2_keys, uint32_t *max_segs_group, uint32_t *max_segs_shared) {
    if (log2_keys > 32 || !max_segs_group || !max_segs_shared) return LPMA_ERR_INVALID_ARGUMENT;
    const uint32_t w = g_grain[log2_keys].load(std::memory_order_relaxed);
    *max_segs_group = (w & 0xFFu) ? (w & 0xFFu) : CUT_GROUP_DEFAULT;
    *max_segs_shared = ((w >> 8) & 0xFFu) ? ((w >> 8) & 0xFFu) : SMALL_WIN_SEGS;
    return LPMA_OK;
}

// Times the update of the caller's own handle under each candidate grain
// setting: the batch of absent keys inserted and deleted again (the stored
// set is the same afterwards; the layout is a valid one of it), and keeps
// the fastest for the batch's bucket.  Keys already stored are refused
// before anything changes.
lpma_status_t lpma_autotune_grain(LpmaHandle *h, const uint64_t *d_keys, size_t n, uint32_t reps,
                                  lpma_stream_t stream, LpmaGrainTime *out, size_t cap, size_t *n_out) {
    if (!h || h->gp || !d_keys || !n || n > 0xFFFFFFFFu || !reps || reps > 1000) return LPMA_ERR_INVALID_ARGUMENT;
    if (h->sticky != LPMA_OK) return h->sticky;
    cudaStream_t s = (cudaStream_t)stream;
    {
        uint32_t *cnt_d = nullptr;
        CK(dalloc(&cnt_d, 1));
        uint32_t present = 0;
        cudaError_t e = cudaMemsetAsync(cnt_d, 0, 4, s);
        if (!e) {
            Geo g{h->c.keys, h->c.vals, h->H};
            launch_count_present(d_keys, (uint32_t)n, h->cfg.key_format, g, h->c.fl, cnt_d, s);
            e = cudaGetLastError();
        }
        if (!e) e = cudaMemcpyAsync(&present, cnt_d, 4, cudaMemcpyDeviceToHost, s);
        if (!e) e = cudaStreamSynchronize(s);
        dfree(cnt_d);
        if (e) return LPMA_ERR_CUDA;
        if (present) return LPMA_ERR_INVALID_ARGUMENT;
    }
    static const uint32_t cand[6][2] = {{4, 32}, {2, 32}, {4, 16}, {2, 16}, {4, 8}, {2, 8}};
    const uint32_t b = grain_bucket(n);
    const uint32_t saved = g_grain[b].load(std::memory_order_relaxed);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) || cudaEventCreate(&e1)) {
        if (e0) cudaEventDestroy(e0);
        return LPMA_ERR_CUDA;
    }
    lpma_status_t r = LPMA_OK;
    // the settings take turns round by round (round 0 warms each up and
    // captures its front), so that a drift of the handle or the clocks
    // spreads over all of them
    std::vector<float> t[6];
    for (uint32_t rep = 0; rep <= reps && r == LPMA_OK; rep++) {
        for (int c = 0; c < 6 && r == LPMA_OK; c++) {
            g_grain[b].store(cand[c][0] | (cand[c][1] << 8), std::memory_order_relaxed);
            LpmaStats st{};
            if (cudaEventRecord(e0, s)) r = LPMA_ERR_CUDA;
            if (r == LPMA_OK) r = lpma_update(h, d_keys, nullptr, n, nullptr, 0, 0, stream, &st);
            if (r == LPMA_OK) r = lpma_update(h, nullptr, nullptr, 0, d_keys, n, 0, stream, &st);
            if (r == LPMA_OK && (cudaEventRecord(e1, s) || cudaEventSynchronize(e1))) r = LPMA_ERR_CUDA;
            float ms = 0.f;
            if (r == LPMA_OK && rep > 0 && !cudaEventElapsedTime(&ms, e0, e1)) t[c].push_back(ms * 1000.f);
        }
    }
    // a setting replaces the defaults (the first candidate) only when it is
    // at least 3% faster: the difference between settings is often within
    // the noise of a few rounds
    float med[6] = {0, 0, 0, 0, 0, 0};
    size_t nout = 0;
    int best = 0;
    for (int c = 0; c < 6 && r == LPMA_OK; c++) {
        std::sort(t[c].begin(), t[c].end());
        med[c] = t[c].empty() ? 0.f : t[c][t[c].size() / 2];
        if (out && nout < cap) out[nout] = LpmaGrainTime{cand[c][0], cand[c][1], med[c], 0u};
        nout++;
        if (med[c] > 0.f && med[c] < med[best]) best = c;
    }
    const uint32_t best_w = (best == 0 || med[best] > 0.97f * med[0]) ? 0u : (cand[best][0] | (cand[best][1] << 8));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    g_grain[b].store(r == LPMA_OK ? best_w : saved, std::memory_order_relaxed);
    if (n_out) *n_out = nout;
    return r;
}

// Times every usable sort tier on seeded batches of 2^b keys (the update
// path's key layout: 21-bit source and destination ids, six active digit
// bytes), for b = 11 .. ceil(log2 max_keys) and both sort modes, and keeps
// the fastest per (b, mode) in the process-wide table that update calls
// read.  All tiers give the same order, so this changes speed only.
lpma_status_t lpma_autotune(uint32_t max_keys, lpma_stream_t stream, LpmaTuneEntry *out, size_t cap,
                            size_t *n_out) {
    if (max_keys < 2048 || max_keys > (1u << 24)) return LPMA_ERR_INVALID_ARGUMENT;
    cudaStream_t s = (cudaStream_t)stream;
    CK(sort_prepare());
    uint32_t bmax = 11;
    while ((1u << bmax) < max_keys) bmax++;
    const uint32_t N = 1u << bmax;
    // seeded keys, their pristine copy and running AND / OR per prefix
    std::vector<uint64_t> hk(N);
    std::vector<uint16_t> hp(N);
    uint64_t x = 0x5EEDull;
    for (uint32_t i = 0; i < N; i++) {
        x += 0x9E3779B97F4A7C15ull;
        uint64_t z = x;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        hk[i] = ((z & 0x1FFFFFull) << 42) | (((z >> 21) & 0x1FFFFFull) << 20);
        hp[i] = (uint16_t)((i & 0xFF) | ((i & 1) << 8));
    }
    uint64_t *k0 = nullptr, *k1 = nullptr, *kp = nullptr;
    uint16_t *p0 = nullptr, *p1 = nullptr, *pp = nullptr;
    unsigned long long *andor = nullptr;
    uint32_t *err = nullptr;
    SortScratch sc;
    sc.status_words = sort_status_words_wide(N);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    lpma_status_t r = LPMA_OK;
    size_t nout = 0;
    auto cleanup = [&]() {
        cudaStreamSynchronize(s);
        dfree(k0), dfree(k1), dfree(kp), dfree(p0), dfree(p1), dfree(pp), dfree(andor), dfree(err);
        dfree(sc.status), dfree(sc.hist), dfree(sc.counters);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    };
    if (dalloc(&k0, N) || dalloc(&k1, N) || dalloc(&kp, N) || dalloc(&p0, N) || dalloc(&p1, N) || dalloc(&pp, N) ||
        dalloc(&andor, 2) || dalloc(&err, 1) || dalloc(&sc.status, sc.status_words) || dalloc(&sc.hist, 8 * 256) ||
        dalloc(&sc.counters, 16) || cudaEventCreate(&e0) || cudaEventCreate(&e1)) {
        cleanup();
        return LPMA_ERR_OUT_OF_MEMORY;
    }
    sc.err = err;
    if (cudaMemcpy(kp, hk.data(), N * 8ull, cudaMemcpyHostToDevice) ||
        cudaMemcpy(pp, hp.data(), N * 2ull, cudaMemcpyHostToDevice) || cudaMemset(err, 0, 4)) {
        cleanup();
        return LPMA_ERR_CUDA;
    }
    uint64_t a = ~0ull, o = 0;
    uint32_t done = 0;
    for (uint32_t b = 11; b <= bmax && r == LPMA_OK; b++) {
        const uint32_t n = 1u << b;
        for (; done < n; done++) a &= hk[done], o |= hk[done];
        const unsigned long long ao[2] = {a, o};
        if (cudaMemcpy(andor, ao, sizeof(ao), cudaMemcpyHostToDevice)) {
            r = LPMA_ERR_CUDA;
            break;
        }
        for (int conc = 0; conc < 2 && r == LPMA_OK; conc++) {
            sc.bar = conc ? nullptr : sc.counters;
            LpmaTuneEntry ent{};
            ent.log2_keys = b;
            ent.concurrent = (uint32_t)conc;
            float best = 0.f;
            uint32_t best_t = 0;
            for (uint32_t t = TIER_SMALL; t < TIER_COUNT; t++) {
                if (!sort_tier_usable((SortTier)t, n, sc)) continue;
                const SortMask m = update_sort_mask(andor, (SortTier)t, n, sc);
                float ts[6];
                for (int rep = 0; rep < 6; rep++) {  // one warm-up, five timed
                    cudaError_t ce = cudaMemcpyAsync(k0, kp, n * 8ull, cudaMemcpyDeviceToDevice, s);
                    if (!ce) ce = cudaMemcpyAsync(p0, pp, n * 2ull, cudaMemcpyDeviceToDevice, s);
                    if (!ce) ce = cudaEventRecord(e0, s);
                    if (!ce) ce = sort_pairs_dev<uint16_t>(k0, p0, k1, p1, n, m, sc, s, (SortTier)t);
                    if (!ce) ce = cudaEventRecord(e1, s);
                    if (!ce) ce = cudaEventSynchronize(e1);
                    float ms = 0.f;
                    if (!ce) ce = cudaEventElapsedTime(&ms, e0, e1);
                    if (ce) {
                        r = LPMA_ERR_CUDA;
                        break;
                    }
                    ts[rep] = ms * 1000.f;
                }
                if (r != LPMA_OK) break;
                std::sort(ts + 1, ts + 6);
                ent.us[t] = ts[3];
                if (!best_t || ts[3] < best) best = ts[3], best_t = t;
            }
            uint32_t herr = 0;
            if (r == LPMA_OK && (cudaMemcpy(&herr, err, 4, cudaMemcpyDeviceToHost) || herr)) r = LPMA_ERR_TIMEOUT;
            if (r != LPMA_OK) break;
            ent.tier = best_t;
            sort_tier_set(b, conc, (SortTier)best_t);
            if (out && nout < cap) out[nout] = ent;
            nout++;
        }
    }
    if (n_out) *n_out = nout;
    cleanup();
    return r;
}

lpma_status_t lpma_shuffle(uint64_t seed, uint64_t *d_keys, size_t n, lpma_stream_t stream) {
    if (!d_keys || n >= (1ull << 30)) return LPMA_ERR_INVALID_ARGUMENT;
    if (n < 2) return LPMA_OK;
    cudaStream_t s = (cudaStream_t)stream;
    uint64_t *tmp = nullptr, *hash = nullptr, *hash2 = nullptr, *pay2 = nullptr;
    uint16_t *p0 = nullptr, *p1 = nullptr;
    uint32_t *err = nullptr;
    SortScratch ss;
    ss.status_words = sort_status_words((uint32_t)n);
    lpma_status_t r = LPMA_OK;
    if (dalloc(&tmp, n) || dalloc(&hash, n) || dalloc(&hash2, n) || dalloc(&pay2, n) || dalloc(&p0, n) ||
        dalloc(&p1, n) || dalloc(&err, 1) || dalloc(&ss.status, ss.status_words) || dalloc(&ss.hist, 8 * 256) ||
        dalloc(&ss.counters, 16)) {
        r = LPMA_ERR_OUT_OF_MEMORY;
    } else {
        cudaMemsetAsync(p0, 0, n * 2, s);
        cudaMemsetAsync(err, 0, 4, s);
        int which = 0;
        // (hash, key) order: keys ascending, then a stable sort by hash
        cudaError_t e = sort_pairs<uint16_t>(d_keys, p0, tmp, p1, (uint32_t)n, ~0ull, ss, err, s, &which);
        uint64_t *sorted = which ? tmp : d_keys;
        if (!e) {
            launch_hash_keys(seed, sorted, hash, n, s);
            e = sort_pairs<uint64_t>(hash, sorted, hash2, pay2, (uint32_t)n, ~0ull, ss, err, s, &which);
        }
        uint64_t *res = which ? pay2 : sorted;
        if (!e && res != d_keys) e = cudaMemcpyAsync(d_keys, res, n * 8, cudaMemcpyDeviceToDevice, s);
        uint32_t herr = 0;
        if (!e) e = cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, s);
        if (!e) e = cudaStreamSynchronize(s);
        if (e)
            r = cuda_fail(e);
        else if (herr)
            r = LPMA_ERR_TIMEOUT;
    }
    cudaStreamSynchronize(s);
    dfree(tmp), dfree(hash), dfree(hash2), dfree(pay2), dfree(p0), dfree(p1), dfree(err);
    dfree(ss.status), dfree(ss.hist), dfree(ss.counters);
    return r;
}

}  // extern "C"
