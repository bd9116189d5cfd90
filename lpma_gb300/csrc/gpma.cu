// GPMA mode of the engine: the flat packed memory array of the reference's
// gpma.cuh, as a configuration of the update pipeline (LPMA_FLAG_GPMA).
//
// Layout in HBM: one array of `size` slots (a power of two), cut into
// 2^h segments of seg = 2^(fls(fls(size)) - 1) slots (resize_gpma,
// gpma.cuh:706-711); keys src << 32 | dst, the sentinel of row v is
// v << 32 | 0xFFFFFFFF, two KEY_MAX guards sit at the end; row_offset[v + 1]
// is the absolute slot of v's sentinel (gpma.cuh:341-344).  A delete
// tombstones a present key in place (value 0xFF) and takes no part in the
// density checks until a window that holds it is rebalanced
// (handle_del_mod, gpma.cuh:162-175).
//
// One update: pack + validate, the shared radix sort, resolve (locate by
// binary search over the first slot of each segment, membership scan of the
// segment, upsert / tombstone / a tombstoned key brought back in place),
// the pending inserts compacted into the update list, then the shared
// count-only planner and maximal-window filter (k_plan / k_plan_max, with
// the flat segment length and count) over per-segment live counts.  The
// maximal windows run on flat executors: single-segment windows one warp
// each, windows of up to 32 segments one CTA each in shared memory, bigger
// ones as gather / clear / merge-spread.
// When the root cannot take the batch, or a batch brings 5,000,000 new keys
// or more (significant_insert, gpma.cuh:720-744), the whole array is
// rebuilt at the resize rule's size (a copying resize, gpma.cuh:694-718).
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include "gpma.cuh"
#include "kernels.cuh"
#include "prims.cuh"

namespace lpma {
namespace {

constexpr int GTPB = 256;
constexpr uint32_t SIGNIFICANT = 5000000u;  // gpma.cuh:771
constexpr uint32_t SMALL_SLOTS = 32 * 32;   // windows of <= 32 segments of <= 32 slots

__device__ __forceinline__ bool g_sentinel(uint64_t k) { return (k & 0xFFFFFFFFull) == 0xFFFFFFFFull && k != KEY_NONE; }
__device__ __forceinline__ bool g_kept(uint64_t k, uint8_t v) { return k != KEY_NONE && v != VAL_TOMB; }

// per-segment u8 counts, changed by one with a word atomic (a count never
// leaves 0..32, so no carry or borrow crosses into a neighbour's byte)
__device__ __forceinline__ void cnt_add(uint8_t *cnt, uint64_t s, int d) {
    uint32_t *w = reinterpret_cast<uint32_t *>(cnt + (s & ~3ull));
    const uint32_t sh = 8u * (uint32_t)(s & 3u);
    if (d > 0)
        atomicAdd(w, 1u << sh);
    else
        atomicSub(w, 1u << sh);
}

// ------------------------------------------------------------------ pack
__global__ void __launch_bounds__(GTPB) k_gpma_pack(const uint64_t *__restrict__ ins, const uint8_t *__restrict__ ins_vals,
                                                     uint32_t n_ins, const uint64_t *__restrict__ del, uint32_t n_del,
                                                     uint32_t V, uint64_t *k_out, uint16_t *p_out, DevStatus *st) {
    const uint32_t i = blockIdx.x * GTPB + threadIdx.x;
    if (i >= n_ins + n_del) return;
    uint64_t key;
    uint16_t p;
    bool bad;
    if (i < n_ins) {
        key = ins[i];
        const uint8_t v = ins_vals ? ins_vals[i] : (uint8_t)1;
        bad = v == VAL_TOMB;
        p = v;
    } else {
        key = del[i - n_ins];
        bad = false;
        p = 0x100;
    }
    bad |= (key >> 32) >= V || (key & 0xFFFFFFFFull) >= V;
    if (bad) {
        atomicOr(&st->error, ERR_KEY);
        atomicMin(&st->err_info[0], i);
    }
    k_out[i] = key;
    p_out[i] = p;
}

// ------------------------------------------------------------------ resolve
// One thread per sorted key, on a persistent grid.  Repeated keys collapse
// as in the leveled path: the last insert of a key gives its value and an
// insert of a key also deleted in the batch wins (delete first).  flag[i] =
// 1 for a pending insert, seg_of[i] its located segment.  Counters: n_ins =
// tombstoned keys brought back, n_upsert, n_del, n_noop.
//
// The locate is locate_leaf_kernel's binary search over the segments' first
// slots (gpma.cuh:185-191), run over the leaders table (lead[s] = the key in
// segment s's first slot; 16 MB for 2M segments, so its deep levels are L2
// reads, not random DRAM lines of the slot array): depth d probes segment
// ps | (nseg >> (d + 1)).  Each CTA first stages the probes of the first
// GR_TOP depths in shared memory in heap order (node k at depth d =
// floor(log2 k) probes segment (k - 2^d) * (nseg >> d) + (nseg >> (d + 1))),
// so a key walks those depths there and only the deeper ones in the table.
constexpr uint32_t GR_TOP = 10;
__global__ void __launch_bounds__(GTPB) k_gpma_resolve(const uint64_t *__restrict__ sk, const uint16_t *__restrict__ sp,
                                                        uint32_t n, const uint64_t *__restrict__ keys, uint8_t *vals,
                                                        uint8_t *live, uint32_t seg, uint32_t seg_log, uint32_t h,
                                                        uint32_t *flag, uint32_t *seg_of, const uint64_t *__restrict__ lead,
                                                        DevStatus *st) {
    __shared__ uint64_t sel[1u << GR_TOP];
    const bool rejected = (st->error & (ERR_KEY | ERR_TIMEOUT)) != 0;  // invalid key, or the sort gave up a wait
    const uint64_t nseg = 1ull << h;
    const uint32_t ts = h < GR_TOP ? h : GR_TOP;
    if (!rejected)
        for (uint32_t k = 1 + threadIdx.x; k < (1u << ts); k += GTPB) {
            const uint32_t d = 31 - __clz(k);
            sel[k] = lead[(uint64_t)(k - (1u << d)) * (nseg >> d) + (nseg >> (d + 1))];
        }
    __syncthreads();
    uint32_t back = 0, ups = 0, dels = 0, noop = 0;
    for (uint32_t i = blockIdx.x * GTPB + threadIdx.x; i < n; i += gridDim.x * GTPB) {
        uint32_t f = 0;
        if (rejected) {
            flag[i] = 0;
            continue;
        }
        const uint64_t key = sk[i];
        const uint16_t p = sp[i];
        const bool is_del = (p >> 8) & 1;
        bool rep;
        if (is_del)
            rep = (i == 0 || sk[i - 1] != key);
        else
            rep = (i + 1 == n || sk[i + 1] != key || ((sp[i + 1] >> 8) & 1));
        if (rep) {
            uint32_t node = 1;
            for (uint32_t d = 0; d < ts; d++) node = 2 * node + (sel[node] <= key ? 1u : 0u);
            uint64_t ps = (uint64_t)(node - (1u << ts)) * (nseg >> ts);
            for (uint64_t bit = (nseg >> ts) >> 1; bit; bit >>= 1)
                if (lead[ps | bit] <= key) ps |= bit;
            const uint64_t prefix = ps << seg_log;
            // handle_del_mod: the first equal key of the segment
            int hit = -1;
            for (uint32_t l = 0; l < seg; l++)
                if (keys[prefix + l] == key) {
                    hit = (int)l;
                    break;
                }
            const uint64_t s = prefix >> seg_log;
            if (!is_del) {
                if (hit >= 0) {
                    const uint8_t old = vals[prefix + hit];
                    vals[prefix + hit] = (uint8_t)(p & 0xFF);
                    if (old == VAL_TOMB) {
                        cnt_add(live, s, +1);
                        back++;
                    } else {
                        ups++;
                    }
                } else {
                    f = 1;
                    seg_of[i] = (uint32_t)s;
                }
            } else if (hit >= 0 && vals[prefix + hit] != VAL_TOMB) {
                vals[prefix + hit] = VAL_TOMB;
                cnt_add(live, s, -1);
                dels++;
            } else {
                noop++;
            }
        } else {
            noop++;
        }
        flag[i] = f;
    }
    back = __reduce_add_sync(0xffffffffu, back);
    ups = __reduce_add_sync(0xffffffffu, ups);
    dels = __reduce_add_sync(0xffffffffu, dels);
    noop = __reduce_add_sync(0xffffffffu, noop);
    if ((threadIdx.x & 31) == 0) {
        if (back) atomicAdd(&st->n_ins, back);
        if (ups) atomicAdd(&st->n_upsert, ups);
        if (dels) atomicAdd(&st->n_del, dels);
        if (noop) atomicAdd(&st->n_noop, noop);
    }
}

// pending inserts into the update list (key order); ip is the identity
// (every entry is an insert)
__global__ void __launch_bounds__(GTPB) k_gpma_list(const uint64_t *__restrict__ sk, const uint16_t *__restrict__ sp,
                                                     const uint32_t *__restrict__ flag, const uint32_t *__restrict__ pos,
                                                     const uint32_t *__restrict__ seg_of, uint32_t n, UpdList u) {
    const uint32_t i = blockIdx.x * GTPB + threadIdx.x;
    if (i <= n) u.ip[i] = i;
    if (i < n && flag[i]) {
        const uint32_t x = pos[i];
        u.key[x] = sk[i];
        u.val[x] = (uint8_t)(sp[i] & 0xFF);
        u.kind[x] = KIND_INS;
        u.seg[x] = seg_of[i];
    }
}

// ------------------------------------------------------------------ spread helpers
// item r of m over f segments: segment f*r/m, lane (f*r % m)/f
// (redispatch_kernel, gpma.cuh:440-443)
__device__ __forceinline__ uint64_t spread_slot(uint64_t r, uint64_t m, uint64_t f, uint32_t seg) {
    const uint64_t fr = f * r;
    return (fr / m) * seg + (fr % m) / f;
}

// lead (optional): the segment leaders (the first slot's key of every
// segment), written here for the items that land in a first slot; the
// executors that pass none write the leaders of their windows themselves
__device__ __forceinline__ void put_item(uint64_t *keys, uint8_t *vals, uint32_t *row_offset, uint32_t V,
                                         uint64_t *lead, uint32_t seg, uint64_t slot, uint64_t k, uint8_t v) {
    keys[slot] = k;
    vals[slot] = v;
    if (lead && (slot & (seg - 1)) == 0) lead[slot >> (__ffs(seg) - 1)] = k;
    if (g_sentinel(k)) {
        const uint64_t row = k >> 32;
        if (row < V) row_offset[row + 1] = (uint32_t)slot;
    }
}

// number of entries of a[0..n) below key (strict) or at most key (!strict)
__device__ __forceinline__ uint32_t rank_in(const uint64_t *a, uint32_t n, uint64_t key, bool strict) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (strict ? a[mid] < key : a[mid] <= key)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// ------------------------------------------------------------------ single-segment windows
// Windows of one segment (at most 32 slots; most of the windows) take one
// warp each, one slot a lane, on a persistent grid: the kept items' ranks by
// ballot, each insert's merged rank by one ballot over the kept items and a
// count of the inserts below every kept item, kept items before inserts on
// equal keys as in k_gpma_exec_small; the segment is cleared and its items
// placed at their ranks (the even spread over one segment packs them from
// slot 0).  The warp reads every slot before it writes any.
__global__ void __launch_bounds__(GTPB, 8) k_gpma_exec_single(const Window *__restrict__ wins,
                                                            const uint32_t *__restrict__ n_win, uint32_t n_cap,
                                                            uint64_t *keys, uint8_t *vals, uint8_t *live,
                                                            uint32_t *row_offset, uint32_t V, uint32_t seg, UpdList u,
                                                            uint64_t *lead, DevStatus *st) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warps = gridDim.x * (GTPB / 32);
    const uint32_t nwin = min(*n_win, n_cap);
    for (uint32_t wi = blockIdx.x * (GTPB / 32) + (threadIdx.x >> 5); wi < nwin; wi += warps) {  // uniform per warp
        const Window w = wins[wi];
        const uint32_t W = w.f * seg;
        const uint64_t base = (uint64_t)w.a * seg;
        const uint32_t k = w.hi - w.lo;  // the window's pending inserts, in key order
        uint64_t key = KEY_NONE, b = KEY_NONE;
        uint8_t val = VAL_TOMB, bv = 0;
        if (lane < W && W <= 32) key = keys[base + lane], val = vals[base + lane];
        if (lane < k && k <= 32) b = u.key[w.lo + lane], bv = u.val[w.lo + lane];
        const bool kept = lane < W && g_kept(key, val);
        const uint32_t kb = __ballot_sync(0xffffffffu, kept);
        const uint32_t c = __popc(kb), kidx = __popc(kb & ((1u << lane) - 1));
        const uint32_t m = c + k;
        if (m != w.m || m > W || W > 32 || w.f != 1) {  // the plan's count and the slots disagree
            if (lane == 0) {
                atomicOr(&st->sticky, ERR_INTERNAL);
                atomicCAS(&st->sticky_site, 0u, 7u);
            }
            continue;
        }
        uint32_t below = 0, kept_le = 0;  // inserts below this lane's kept item; kept items <= this lane's insert
        for (uint32_t j = 0; j < k; j++) {
            const uint64_t bj = __shfl_sync(0xffffffffu, b, j);
            below += (kept && bj < key) ? 1u : 0u;
            const uint32_t le = __popc(__ballot_sync(0xffffffffu, kept && key <= bj));
            if (lane == j) kept_le = le;
        }
        __syncwarp();
        // the segment's leader: written only when the first slot's key
        // changes (an insert below the first key, or the first key gone)
        const uint64_t old0 = __shfl_sync(0xffffffffu, key, 0);
        if (lane < W) keys[base + lane] = KEY_NONE;
        __syncwarp();
        if (kept) put_item(keys, vals, row_offset, V, nullptr, seg, base + kidx + below, key, val);
        if (lane < k) put_item(keys, vals, row_offset, V, nullptr, seg, base + lane + kept_le, b, bv);
        if (kept && kidx + below == 0 && key != old0) lead[w.a] = key;
        if (lane < k && lane + kept_le == 0 && b != old0) lead[w.a] = b;
        if (lane == 0 && m == 0 && old0 != KEY_NONE) lead[w.a] = KEY_NONE;
        if (lane == 0) live[w.a] = (uint8_t)m;
    }
}

// ------------------------------------------------------------------ small windows
// One CTA per window of up to 32 segments: the window's kept items (A, in
// slot order) and its inserts (B, key order) merged by key, A before B on
// equal keys (the stable block sort of block_redispatch_kernel,
// gpma.cuh:309-313), then spread evenly over the window.
struct SmallSmem {
    uint64_t a[SMALL_SLOTS], b[SMALL_SLOTS], m[SMALL_SLOTS];
    uint8_t av[SMALL_SLOTS], bv[SMALL_SLOTS], mv[SMALL_SLOTS];
    uint32_t wsum[GTPB / 32];
};

__global__ void __launch_bounds__(GTPB) k_gpma_exec_small(const Window *__restrict__ wins, const uint32_t *__restrict__ n_win,
                                                           uint64_t *keys, uint8_t *vals, uint8_t *live,
                                                           uint32_t *row_offset, uint32_t V, uint32_t seg, UpdList u,
                                                           uint64_t *lead, DevStatus *st) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SmallSmem &S = *reinterpret_cast<SmallSmem *>(smem_raw);
    if (blockIdx.x >= *n_win) return;
    const Window w = wins[blockIdx.x];
    const uint64_t base = (uint64_t)w.a * seg;
    const uint32_t W = w.f * seg;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    // compact the kept slots, in slot order, four slots a thread
    uint32_t c_run = 0;
    for (uint32_t b0 = 0; b0 < W; b0 += GTPB * 4) {
        uint64_t kk[4];
        uint8_t vv[4];
        uint32_t keep = 0;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const uint32_t x = b0 + (uint32_t)tid * 4 + q;
            kk[q] = x < W ? keys[base + x] : KEY_NONE;
            vv[q] = x < W ? vals[base + x] : VAL_TOMB;
            keep |= (g_kept(kk[q], vv[q]) ? 1u : 0u) << q;
        }
        const uint32_t cnt = __popc(keep);
        uint32_t incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) S.wsum[wid] = incl;
        __syncthreads();
        uint32_t before = 0, total = 0;
        for (int ww = 0; ww < GTPB / 32; ww++) {
            if (ww < wid) before += S.wsum[ww];
            total += S.wsum[ww];
        }
        uint32_t at = c_run + before + incl - cnt;
#pragma unroll
        for (int q = 0; q < 4; q++)
            if ((keep >> q) & 1u) {
                S.a[at] = kk[q];
                S.av[at] = vv[q];
                at++;
            }
        c_run += total;
        __syncthreads();
    }
    const uint32_t c = c_run, k = w.hi - w.lo, m = c + k;
    if (m != w.m || m > W) {  // the plan's count and the slots disagree: leave the window alone
        if (tid == 0) {
            atomicOr(&st->sticky, ERR_INTERNAL);
            atomicCAS(&st->sticky_site, 0u, 7u);
        }
        return;
    }
    for (uint32_t j = tid; j < k; j += GTPB) {
        S.b[j] = u.key[w.lo + j];
        S.bv[j] = u.val[w.lo + j];
    }
    __syncthreads();
    for (uint32_t i = tid; i < c; i += GTPB) {
        const uint32_t r = i + rank_in(S.b, k, S.a[i], true);
        S.m[r] = S.a[i];
        S.mv[r] = S.av[i];
    }
    for (uint32_t j = tid; j < k; j += GTPB) {
        const uint32_t r = j + rank_in(S.a, c, S.b[j], false);
        S.m[r] = S.b[j];
        S.mv[r] = S.bv[j];
    }
    __syncthreads();
    for (uint32_t x = tid; x < W; x += GTPB) keys[base + x] = KEY_NONE;
    __syncthreads();
    for (uint32_t r = tid; r < m; r += GTPB)
        put_item(keys, vals, row_offset, V, nullptr, seg, base + spread_slot(r, m, w.f, seg), S.m[r], S.mv[r]);
    // segment d's first slot takes item first_rank(d), when it gets any
    for (uint32_t d = tid; d < w.f; d += GTPB) {
        const uint32_t r0 = (uint32_t)first_rank(d, m, w.f), r1 = (uint32_t)first_rank(d + 1, m, w.f);
        live[w.a + d] = (uint8_t)(r1 - r0);
        lead[w.a + d] = r1 > r0 ? S.m[r0] : KEY_NONE;
    }
}

// ------------------------------------------------------------------ big windows and rebuilds
// Gather: the kept items of source segments [sa, sa + sf) into A at their
// rank (P holds the exclusive prefix of the live counts, P[sa] the first);
// one warp per segment.
// A live count that disagrees with the slots would send a rank past cap: the
// write is skipped and ERR_INTERNAL set instead.
__global__ void __launch_bounds__(GTPB) k_gpma_gather(const uint64_t *__restrict__ keys, const uint8_t *__restrict__ vals,
                                                       const uint32_t *__restrict__ P, uint64_t sa, uint64_t sf,
                                                       uint32_t seg, uint64_t *Ak, uint8_t *Av, uint64_t cap,
                                                       DevStatus *st) {
    const uint64_t s = sa + ((uint64_t)blockIdx.x * GTPB + threadIdx.x) / 32;
    const uint32_t lane = threadIdx.x & 31;
    if (s >= sa + sf) return;
    const uint64_t x = s * seg + lane;
    const uint64_t k = lane < seg ? keys[x] : KEY_NONE;
    const uint8_t v = lane < seg ? vals[x] : VAL_TOMB;
    const bool keep = g_kept(k, v);
    const uint32_t bal = __ballot_sync(0xffffffffu, keep);
    if (lane == 0 && (uint32_t)__popc(bal) != P[s + 1] - P[s]) {
        atomicOr(&st->sticky, ERR_INTERNAL);
        atomicCAS(&st->sticky_site, 0u, 8u);
    }
    if (keep) {
        const uint64_t r = (uint64_t)(P[s] - P[sa]) + __popc(bal & ((1u << lane) - 1u));
        if (r < cap) {
            Ak[r] = k;
            Av[r] = v;
        }
    }
}

// Merge A (c items) with B (k inserts) by key, A first on equal keys, and
// spread the m = c + k items over the slots [base, base + f * seg).
__global__ void __launch_bounds__(GTPB) k_gpma_merge_spread(const uint64_t *__restrict__ Ak, const uint8_t *__restrict__ Av,
                                                             uint32_t c, const uint64_t *__restrict__ Bk,
                                                             const uint8_t *__restrict__ Bv, uint32_t k, uint64_t base,
                                                             uint64_t f, uint32_t seg, uint64_t *keys, uint8_t *vals,
                                                             uint32_t *row_offset, uint32_t V, uint64_t *lead) {
    const uint64_t t = (uint64_t)blockIdx.x * GTPB + threadIdx.x;
    const uint64_t m = (uint64_t)c + k;
    if (t < c) {
        const uint64_t r = t + rank_in(Bk, k, Ak[t], true);
        put_item(keys, vals, row_offset, V, lead, seg, base + spread_slot(r, m, f, seg), Ak[t], Av[t]);
    } else if (t < m) {
        const uint32_t j = (uint32_t)(t - c);
        const uint64_t r = j + rank_in(Ak, c, Bk[j], false);
        put_item(keys, vals, row_offset, V, lead, seg, base + spread_slot(r, m, f, seg), Bk[j], Bv[j]);
    }
}

// live count of every destination segment of an even spread of m items
__global__ void __launch_bounds__(GTPB) k_gpma_spread_counts(uint8_t *live, uint64_t a, uint64_t f, uint64_t m) {
    const uint64_t d = (uint64_t)blockIdx.x * GTPB + threadIdx.x;
    if (d < f) live[a + d] = (uint8_t)(first_rank(d + 1, m, f) - first_rank(d, m, f));
}

// the sentinels and the two KEY_MAX guards of a new array (value 1)
__global__ void __launch_bounds__(GTPB) k_gpma_init_items(uint32_t V, uint64_t *k, uint8_t *v) {
    const uint32_t i = blockIdx.x * GTPB + threadIdx.x;
    if (i < V) {
        k[i] = ((uint64_t)i << 32) | 0xFFFFFFFFull;
        v[i] = 1;
    } else if (i < V + 2) {
        k[i] = GPMA_KEY_MAX;
        v[i] = 1;
    }
}

// export: 1 for a live key (tombstones and guards left out)
__global__ void __launch_bounds__(GTPB) k_gpma_live_flags(const uint64_t *__restrict__ keys, const uint8_t *__restrict__ vals,
                                                           uint64_t size, uint32_t *flag) {
    const uint64_t i = (uint64_t)blockIdx.x * GTPB + threadIdx.x;
    if (i < size) flag[i] = (g_kept(keys[i], vals[i]) && keys[i] != GPMA_KEY_MAX) ? 1u : 0u;
}
__global__ void __launch_bounds__(GTPB) k_gpma_live_gather(const uint64_t *__restrict__ keys, const uint8_t *__restrict__ vals,
                                                            const uint32_t *__restrict__ flag, const uint32_t *__restrict__ pos,
                                                            uint64_t size, uint64_t *ok, uint8_t *ov, uint64_t cap) {
    const uint64_t i = (uint64_t)blockIdx.x * GTPB + threadIdx.x;
    if (i < size && flag[i] && pos[i] < cap) {
        ok[pos[i]] = keys[i];
        ov[pos[i]] = vals[i];
    }
}

uint32_t fls32(uint64_t x) { return x ? 64u - (uint32_t)__builtin_clzll(x) : 0u; }

// resize_gpma's size rule (gpma.cuh:706-711)
void size_rule(uint64_t merge, uint64_t *size, uint32_t *seg, uint32_t *h) {
    uint64_t t = 4;
    while ((double)t < (double)merge) t <<= 1;
    *size = t;
    *seg = 1u << (fls32(fls32(t)) - 1);
    *h = fls32(t / *seg) - 1;
}

inline unsigned nblk(uint64_t n) { return (unsigned)((n + GTPB - 1) / GTPB); }

// device memory from the engine's stream-ordered pool (cached in the
// process, no device-wide synchronisation to take or give back)
template <typename T>
cudaError_t salloc(T **p, size_t count, cudaStream_t s) {
    *p = nullptr;
    return pool_alloc((void **)p, (count ? count : 1) * sizeof(T), s);
}
template <typename T>
void sfree(T *&p, cudaStream_t s) {
    if (p) cudaFreeAsync((void *)p, s);
    p = nullptr;
}

}  // namespace

// ====================================================================== state
struct GpmaState {
    uint32_t V = 0;
    double dlow = 0.15;
    uint64_t size = 0;
    uint32_t seg = 0, h = 0;
    uint64_t live_total = 0;  // kept items, guards included
    uint64_t *keys = nullptr;
    uint8_t *vals = nullptr;
    uint8_t *live = nullptr;  // per segment (padded to 16 bytes)
    uint64_t *lead = nullptr; // per segment: the key in its first slot (the locate's search table)
    uint32_t *row = nullptr;  // V + 1
    DevStatus *dst = nullptr, *hst = nullptr;
    uint32_t sticky = 0;
};

namespace {

#define GCK(x)                                                                  \
    do {                                                                        \
        cudaError_t e_ = (x);                                                   \
        if (e_ != cudaSuccess)                                                  \
            return e_ == cudaErrorMemoryAllocation ? LPMA_ERR_OUT_OF_MEMORY : LPMA_ERR_CUDA; \
    } while (0)

uint64_t nseg_of_flat(const GpmaState *g) { return g->size / g->seg; }

// Everything kept in the array plus k sorted items (Bk, Bv) spread over a
// new array of the resize rule's size (the root after resize_gpma,
// significant_insert, and the first state).
lpma_status_t rebuild(GpmaState *g, const uint64_t *Bk, const uint8_t *Bv, uint32_t k, cudaStream_t s) {
    uint64_t c = 0;
    uint64_t *Ak = nullptr, *nk = nullptr, *nld = nullptr;
    uint8_t *Av = nullptr, *nv = nullptr, *nl = nullptr;
    uint32_t *P = nullptr, *tmp = nullptr;
    const uint64_t nseg_old = g->keys ? nseg_of_flat(g) : 0;
    if (nseg_old) {
        // the kept items: the sum of the live counts, as the gather ranks them
        uint32_t total = 0;
        GCK(salloc(&P, nseg_old + 1, s));
        GCK(salloc(&tmp, scan_tmp_words((uint32_t)nseg_old) + 64, s));
        GCK(scan_u8_to_u32(g->live, P, (uint32_t)nseg_old, P + nseg_old, tmp, s));
        GCK(cudaMemcpyAsync(&total, P + nseg_old, 4, cudaMemcpyDeviceToHost, s));
        GCK(cudaStreamSynchronize(s));
        if (total != g->live_total) return LPMA_ERR_INTERNAL;
        c = total;
    }
    uint64_t ns;
    uint32_t seg, h;
    size_rule(c + k, &ns, &seg, &h);
    const uint64_t nseg_new = ns / seg;
    GCK(salloc(&Ak, c, s));
    GCK(salloc(&Av, c, s));
    GCK(salloc(&nk, ns, s));
    GCK(salloc(&nv, ns, s));
    GCK(salloc(&nl, (nseg_new + 15) & ~15ull, s));
    GCK(salloc(&nld, nseg_new, s));
    if (c) {
        k_gpma_gather<<<nblk(nseg_old * 32), GTPB, 0, s>>>(g->keys, g->vals, P, 0, nseg_old, g->seg, Ak, Av, c, g->dst);
        note_launch();
    }
    GCK(cudaMemsetAsync(nk, 0xFF, ns * 8, s));
    GCK(cudaMemsetAsync(nv, 0, ns, s));
    GCK(cudaMemsetAsync(nl, 0, (nseg_new + 15) & ~15ull, s));
    GCK(cudaMemsetAsync(nld, 0xFF, nseg_new * 8, s));
    {
        ProfScope ps("gpma_merge_spread", s);
        k_gpma_merge_spread<<<nblk(c + k), GTPB, 0, s>>>(Ak, Av, (uint32_t)c, Bk, Bv, k, 0, nseg_new, seg, nk, nv,
                                                          g->row, g->V, nld);
        note_launch();
    }
    k_gpma_spread_counts<<<nblk(nseg_new), GTPB, 0, s>>>(nl, 0, nseg_new, c + k);
    note_launch();
    GCK(cudaGetLastError());
    sfree(Ak, s), sfree(Av, s), sfree(P, s), sfree(tmp, s);
    sfree(g->keys, s), sfree(g->vals, s), sfree(g->live, s), sfree(g->lead, s);
    g->keys = nk, g->vals = nv, g->live = nl, g->lead = nld;
    g->size = ns, g->seg = seg, g->h = h;
    g->live_total = c + k;
    return LPMA_OK;
}

// one window of more than 32 segments: gather its kept items, clear it,
// merge with its inserts and spread
lpma_status_t exec_big(GpmaState *g, const Window &w, const uint32_t *P, const UpdList &u, cudaStream_t s) {
    uint32_t P2[2];
    GCK(cudaMemcpyAsync(P2, P + w.a, 4, cudaMemcpyDeviceToHost, s));
    GCK(cudaMemcpyAsync(P2 + 1, P + w.a + w.f, 4, cudaMemcpyDeviceToHost, s));
    GCK(cudaStreamSynchronize(s));
    const uint32_t c = P2[1] - P2[0], k = w.hi - w.lo;
    if (c + k != w.m) return LPMA_ERR_INTERNAL;
    uint64_t *Ak = nullptr;
    uint8_t *Av = nullptr;
    GCK(salloc(&Ak, c, s));
    GCK(salloc(&Av, c, s));
    const uint64_t base = (uint64_t)w.a * g->seg, W = (uint64_t)w.f * g->seg;
    ProfScope ps("gpma_exec_big", s);
    k_gpma_gather<<<nblk((uint64_t)w.f * 32), GTPB, 0, s>>>(g->keys, g->vals, P, w.a, w.f, g->seg, Ak, Av, c, g->dst);
    GCK(cudaMemsetAsync(g->keys + base, 0xFF, W * 8, s));
    GCK(cudaMemsetAsync(g->lead + w.a, 0xFF, (uint64_t)w.f * 8, s));
    k_gpma_merge_spread<<<nblk((uint64_t)c + k), GTPB, 0, s>>>(Ak, Av, c, u.key + w.lo, u.val + w.lo, k, base, w.f,
                                                                g->seg, g->keys, g->vals, g->row, g->V, g->lead);
    k_gpma_spread_counts<<<nblk(w.f), GTPB, 0, s>>>(g->live, w.a, w.f, (uint64_t)c + k);
    note_launch(3);
    GCK(cudaGetLastError());
    sfree(Ak, s), sfree(Av, s);
    return LPMA_OK;
}

}  // namespace

lpma_status_t gpma_create(uint32_t V, double density_lower, cudaStream_t s, GpmaState **out) {
    *out = nullptr;
    if (V == 0 || V >= 0xFFFFFFFEu || !(density_lower >= 0.0 && density_lower <= 1.0)) return LPMA_ERR_INVALID_ARGUMENT;
    GpmaState *g = new GpmaState();
    g->V = V;
    g->dlow = density_lower;
    auto fail = [&](lpma_status_t r) {
        gpma_destroy(g);
        return r;
    };
    if (salloc(&g->row, (size_t)V + 1, s) || salloc(&g->dst, 1, s) || cudaMallocHost(&g->hst, sizeof(DevStatus)))
        return fail(LPMA_ERR_OUT_OF_MEMORY);
    if (cudaMemsetAsync(g->row, 0, 4ull * (V + 1), s)) return fail(LPMA_ERR_CUDA);
    uint64_t *k = nullptr;
    uint8_t *v = nullptr;
    if (salloc(&k, (size_t)V + 2, s) || salloc(&v, (size_t)V + 2, s)) return fail(LPMA_ERR_OUT_OF_MEMORY);
    k_gpma_init_items<<<nblk((uint64_t)V + 2), GTPB, 0, s>>>(V, k, v);
    note_launch();
    lpma_status_t r = rebuild(g, k, v, V + 2, s);
    sfree(k, s), sfree(v, s);
    if (r != LPMA_OK) return fail(r);
    if (cudaStreamSynchronize(s)) return fail(LPMA_ERR_CUDA);
    *out = g;
    return LPMA_OK;
}

void gpma_destroy(GpmaState *g) {
    if (!g) return;
    cudaStream_t s = cudaStreamPerThread;
    sfree(g->keys, s), sfree(g->vals, s), sfree(g->live, s), sfree(g->lead, s), sfree(g->row, s), sfree(g->dst, s);
    if (g->hst) cudaFreeHost(g->hst);
    delete g;
}

lpma_status_t gpma_update(GpmaState *g, const uint64_t *ins, const uint8_t *ins_vals, size_t n_ins, const uint64_t *del,
                          size_t n_del, cudaStream_t s, LpmaStats *out) {
    if (g->sticky) return LPMA_ERR_INTERNAL;
    LpmaStats st{};
    st.height_before = st.height_after = g->h;
    const size_t n = n_ins + n_del;
    if ((n_ins && !ins) || (n_del && !del)) return LPMA_ERR_INVALID_ARGUMENT;
    if (n >= (1u << 30)) return LPMA_ERR_INVALID_ARGUMENT;
    if (n == 0) {
        st.num_items = g->live_total - 2;
        if (out) *out = st;
        return LPMA_OK;
    }
    const uint32_t nn = (uint32_t)n;
    // batch buffers, stream-ordered
    uint64_t *k0 = nullptr, *k1 = nullptr;
    uint16_t *p0 = nullptr, *p1 = nullptr;
    uint32_t *flag = nullptr, *pos = nullptr, *seg_of = nullptr, *tmp = nullptr, *P = nullptr, *bitmap = nullptr;
    uint32_t *sort_status = nullptr, *sort_hist = nullptr, *sort_cnt = nullptr, *sort_bar = nullptr;
    UpdList u{};
    uint8_t *pend = nullptr;
    Window *wl = nullptr;
    const uint64_t nseg = nseg_of_flat(g);
    const uint32_t Hp = g->h - 1;  // the planner's root level is Hp + 1 = h
    const uint64_t bm_words = ((1ull << (Hp + 2)) + 31) / 32 + 1;
    const size_t scan_words = scan_tmp_words((uint32_t)std::max<uint64_t>(n, nseg)) + 64;
    lpma_status_t r = LPMA_OK;
    auto release = [&]() {
        sfree(k0, s), sfree(k1, s), sfree(p0, s), sfree(p1, s), sfree(flag, s), sfree(pos, s), sfree(seg_of, s);
        sfree(tmp, s), sfree(P, s), sfree(bitmap, s), sfree(sort_status, s), sfree(sort_hist, s), sfree(sort_cnt, s);
        sfree(sort_bar, s);
        sfree(u.key, s), sfree(u.val, s), sfree(u.kind, s), sfree(u.seg, s), sfree(u.ip, s), sfree(pend, s), sfree(wl, s);
    };
#define GCKR(x)                                                                               \
    do {                                                                                      \
        cudaError_t e_ = (x);                                                                 \
        if (e_ != cudaSuccess) {                                                              \
            release();                                                                        \
            return e_ == cudaErrorMemoryAllocation ? LPMA_ERR_OUT_OF_MEMORY : LPMA_ERR_CUDA; \
        }                                                                                     \
    } while (0)
    const size_t sw = sort_status_words_wide(nn);  // room for the cooperative sort's tile counts
    GCKR(salloc(&k0, n, s));
    GCKR(salloc(&k1, n, s));
    GCKR(salloc(&p0, n, s));
    GCKR(salloc(&p1, n, s));
    GCKR(salloc(&flag, n, s));
    GCKR(salloc(&pos, n + 1, s));
    GCKR(salloc(&seg_of, n, s));
    GCKR(salloc(&tmp, scan_words, s));
    GCKR(salloc(&P, nseg + 1, s));
    GCKR(salloc(&bitmap, bm_words, s));
    GCKR(salloc(&sort_status, sw, s));
    GCKR(salloc(&sort_hist, 8 * 256, s));
    GCKR(salloc(&sort_cnt, 16, s));
    GCKR(salloc(&sort_bar, 1, s));
    GCKR(salloc(&u.key, n, s));
    GCKR(salloc(&u.val, n, s));
    GCKR(salloc(&u.kind, n, s));
    GCKR(salloc(&u.seg, n, s));
    GCKR(salloc(&u.ip, n + 1, s));
    GCKR(salloc(&pend, n, s));
    GCKR(salloc(&wl, 5 * n, s));
    Window *cand = wl, *wsingle = wl + n, *wsmall4 = wl + 2 * n, *wsmall = wl + 3 * n, *wbig = wl + 4 * n;
    GCKR(cudaMemsetAsync(g->dst, 0, sizeof(DevStatus), s));
    GCKR(cudaMemsetAsync(&g->dst->err_info[0], 0xFF, 4, s));
    GCKR(cudaMemsetAsync(bitmap, 0, bm_words * 4, s));
    {
        ProfScope ps("gpma_pack", s);
        k_gpma_pack<<<nblk(n), GTPB, 0, s>>>(ins, ins_vals, (uint32_t)n_ins, del, (uint32_t)n_del, g->V, k0, p0, g->dst);
        note_launch();
    }
    // the bits where keys may differ: src and dst below V
    uint64_t vm = 1;
    while (vm < g->V) vm <<= 1;
    vm -= 1;
    SortScratch ss;
    ss.status = sort_status;
    ss.status_words = sw;
    ss.hist = sort_hist;
    ss.counters = sort_cnt;
    // the cooperative sort (its barrier word cleared by the sort; a wait
    // that gives up marks the status, and the resolve then changes nothing)
    ss.bar = sort_bar;
    ss.err = &g->dst->error;
    int which = 0;
    GCKR(sort_pairs<uint16_t>(k0, p0, k1, p1, nn, (vm << 32) | vm, ss, nullptr, s, &which));
    const uint64_t *sk = which ? k1 : k0;
    const uint16_t *sp = which ? p1 : p0;
    {
        ProfScope ps("gpma_resolve", s);
        k_gpma_resolve<<<std::min<uint32_t>(nblk(n), 152 * 8), GTPB, 0, s>>>(sk, sp, nn, g->keys, g->vals, g->live, g->seg,
                                                  (uint32_t)__builtin_ctz(g->seg), g->h, flag, seg_of, g->lead, g->dst);
        note_launch();
    }
    GCKR(scan_u32(flag, pos, nn, &g->dst->n_u, tmp, s));
    k_gpma_list<<<nblk(n + 1), GTPB, 0, s>>>(sk, sp, flag, pos, seg_of, nn, u);
    note_launch();
    // the shared planner over the live counts (after this batch's
    // tombstones and returns), with the flat geometry
    GCKR(scan_u8_to_u32(g->live, P, (uint32_t)nseg, P + nseg, tmp, s));
    GCKR(cudaMemcpyAsync(g->hst, g->dst, sizeof(DevStatus), cudaMemcpyDeviceToHost, s));
    GCKR(cudaStreamSynchronize(s));
    if (g->hst->error & ERR_KEY) {
        release();
        return LPMA_ERR_INVALID_KEY;
    }
    if (g->hst->error & ERR_TIMEOUT) {  // nothing changed
        release();
        return LPMA_ERR_TIMEOUT;
    }
    const uint32_t n_u = g->hst->n_u, back = g->hst->n_ins, dels = g->hst->n_del;
    st.n_ins_applied = n_u + back;
    st.n_upserts = g->hst->n_upsert;
    st.n_del_applied = dels;
    st.n_noop = g->hst->n_noop;
    const uint64_t live_now = g->live_total + back - dels;  // kept items before the new inserts
    g->live_total = live_now;
    bool whole = n_u >= SIGNIFICANT;
    if (n_u > 0 && !whole) {
        Tables tb{};
        uint32_t len = g->seg;
        for (uint32_t i = 0; i <= g->h && i < 32; i++) {
            tb.lower[i] = (uint32_t)(g->dlow * (double)len);  // recalculate_density, gpma.cuh:127
            len <<= 1;
        }
        tb.allowed = (g->h + 1 >= 32) ? 0xFFFFFFFFu : ((1u << (g->h + 1)) - 1u);
        tb.seg_len = g->seg;
        tb.nseg = nseg;
        launch_plan(u, n_u, g->live, P, g->h > 8, live_now, nullptr, Hp, tb, bitmap, cand, wsingle, wsmall4, wsmall,
                    wbig, pend, g->dst, s);
        GCKR(cudaGetLastError());
        GCKR(cudaMemcpyAsync(g->hst, g->dst, sizeof(DevStatus), cudaMemcpyDeviceToHost, s));
        GCKR(cudaStreamSynchronize(s));
        if (g->hst->ovf) {
            whole = true;
            st.overflow = 1;
        } else {
            const DevStatus hs = *g->hst;
            st.root_executed = hs.root ? 1u : 0u;
            st.windows_single = hs.n_single;
            st.windows_small = (uint64_t)hs.n_single + hs.n_small4 + hs.n_small;
            st.windows_big = hs.n_big;
            st.slots_small = hs.slots_small / 32 * g->seg;
            st.slots_rewritten = (hs.slots_small + hs.slots_big) / 32 * g->seg;
            const size_t smem = sizeof(SmallSmem);  // below 48 KB: no opt-in
            const uint32_t counts[3] = {hs.n_single, hs.n_small4, hs.n_small};
            const Window *lists[3] = {wsingle, wsmall4, wsmall};
            const uint32_t *dev_counts[3] = {&g->dst->n_single, &g->dst->n_small4, &g->dst->n_small};
            for (int c = 0; c < 3; c++) {
                if (!counts[c]) continue;
                const bool one = c == 0 && g->seg <= 32;  // single-segment windows: a warp each
                ProfScope ps(one ? "gpma_exec_single" : "gpma_exec_small", s);
                if (one) {
                    const uint32_t nb = std::min<uint32_t>((counts[0] + GTPB / 32 - 1) / (GTPB / 32), 152 * 8);
                    k_gpma_exec_single<<<nb, GTPB, 0, s>>>(lists[0], dev_counts[0], counts[0], g->keys, g->vals,
                                                            g->live, g->row, g->V, g->seg, u, g->lead, g->dst);
                } else {
                    k_gpma_exec_small<<<counts[c], GTPB, smem, s>>>(lists[c], dev_counts[c], g->keys, g->vals, g->live,
                                                                     g->row, g->V, g->seg, u, g->lead, g->dst);
                }
                note_launch();
            }
            GCKR(cudaGetLastError());
            if (hs.n_big) {
                std::vector<Window> big(hs.n_big);
                GCKR(cudaMemcpyAsync(big.data(), wbig, hs.n_big * sizeof(Window), cudaMemcpyDeviceToHost, s));
                GCKR(cudaStreamSynchronize(s));
                for (const Window &w : big) {
                    r = exec_big(g, w, P, u, s);
                    if (r != LPMA_OK) break;
                }
            }
            g->live_total = live_now + n_u;
        }
    }
    if (whole && r == LPMA_OK) {
        // resize_gpma + root rebalance, or significant_insert: every kept
        // item and every pending insert over a new array
        st.rebuilt = 1;
        st.root_executed = 1;
        st.slots_rewritten = 0;
        r = rebuild(g, u.key, u.val, n_u, s);
        st.slots_rewritten = g->size;
    }
    st.levelup = st.rebuilt;
    release();
#undef GCKR
    if (r != LPMA_OK) return r;
    GCK(cudaStreamSynchronize(s));
    GCK(cudaMemcpy(&g->sticky, &g->dst->sticky, 4, cudaMemcpyDeviceToHost));
    if (g->sticky) return LPMA_ERR_INTERNAL;
    st.height_after = g->h;
    st.num_items = g->live_total - 2;
    if (out) *out = st;
    return LPMA_OK;
}

lpma_status_t gpma_geometry(const GpmaState *g, uint64_t *size, uint32_t *seg, uint32_t *h, uint64_t *num_items) {
    if (size) *size = g->size;
    if (seg) *seg = g->seg;
    if (h) *h = g->h;
    if (num_items) *num_items = g->live_total - 2;
    return LPMA_OK;
}

lpma_status_t gpma_view(GpmaState *g, const uint32_t **row_offset, const uint64_t **keys, const uint8_t **vals) {
    if (row_offset) *row_offset = g->row;
    if (keys) *keys = g->keys;
    if (vals) *vals = g->vals;
    return LPMA_OK;
}

lpma_status_t gpma_export_layout(GpmaState *g, uint64_t *h_keys, uint8_t *h_vals, size_t cap_slots,
                                 uint32_t *row_offset, size_t cap_rows, cudaStream_t s) {
    if (cap_slots < g->size || (row_offset && cap_rows < (size_t)g->V + 1)) return LPMA_ERR_BUFFER_TOO_SMALL;
    if (h_keys) GCK(cudaMemcpyAsync(h_keys, g->keys, g->size * 8, cudaMemcpyDeviceToHost, s));
    if (h_vals) GCK(cudaMemcpyAsync(h_vals, g->vals, g->size, cudaMemcpyDeviceToHost, s));
    if (row_offset) GCK(cudaMemcpyAsync(row_offset, g->row, 4ull * (g->V + 1), cudaMemcpyDeviceToHost, s));
    GCK(cudaStreamSynchronize(s));
    if (h_keys && h_vals)
        for (uint64_t i = 0; i < g->size; i++)
            if (h_keys[i] == KEY_NONE) h_vals[i] = 0;  // empty slots read as value 0
    return LPMA_OK;
}

lpma_status_t gpma_export_sorted(GpmaState *g, uint64_t *h_keys, uint8_t *h_vals, size_t cap, size_t *n_out,
                                 cudaStream_t s) {
    const uint64_t n = g->live_total - 2;
    *n_out = n;
    if (cap < n) return LPMA_ERR_BUFFER_TOO_SMALL;
    uint32_t *flag = nullptr, *pos = nullptr, *tmp = nullptr;
    uint64_t *ok = nullptr;
    uint8_t *ov = nullptr;
    GCK(salloc(&flag, g->size, s));
    GCK(salloc(&pos, g->size + 1, s));
    GCK(salloc(&tmp, scan_tmp_words((uint32_t)g->size) + 64, s));
    GCK(salloc(&ok, n, s));
    GCK(salloc(&ov, n, s));
    k_gpma_live_flags<<<nblk(g->size), GTPB, 0, s>>>(g->keys, g->vals, g->size, flag);
    GCK(scan_u32(flag, pos, (uint32_t)g->size, pos + g->size, tmp, s));
    k_gpma_live_gather<<<nblk(g->size), GTPB, 0, s>>>(g->keys, g->vals, flag, pos, g->size, ok, ov, n);
    note_launch(2);
    GCK(cudaMemcpyAsync(h_keys, ok, n * 8, cudaMemcpyDeviceToHost, s));
    if (h_vals) GCK(cudaMemcpyAsync(h_vals, ov, n, cudaMemcpyDeviceToHost, s));
    sfree(flag, s), sfree(pos, s), sfree(tmp, s), sfree(ok, s), sfree(ov, s);
    GCK(cudaStreamSynchronize(s));
    return LPMA_OK;
}

uint64_t gpma_memory_bytes(const GpmaState *g) {
    return g->size * 9ull + 9ull * (g->size / std::max<uint32_t>(g->seg, 1)) + 4ull * (g->V + 1);
}

}  // namespace lpma
