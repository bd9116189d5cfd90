// Update-path kernels of the GB300 LPMA engine.
//
// One batch runs: pack/validate -> radix sort -> resolve+locate (dedup,
// tree descent, membership, in-place upsert / tombstone) -> compaction ->
// count-only planner -> one execution pass over the maximal windows.
//
// The planner replaces the reference's level loop (rpma.cuh:1611-1657),
// which per level rebalances every candidate window, compacts the update
// list, lifts node ids and run-length-encodes them again.  For a window W
// at level l the reference's merge size is compacted(W) + pending(W); since
// every sub-window executed below W absorbed exactly its own updates, this
// equals live(W) + inserts(W) - deletes(W) whatever happened below.  So the
// first level at which a segment's updates are absorbed is a pure function
// of per-segment counts, and the final layout is that of the maximal
// executed windows alone (each re-spreads its whole content), executed once.
#include <algorithm>

#include "kernels.cuh"
#include "prims.cuh"

namespace lpma {
namespace {

constexpr int TPB = 256;
// tree levels staged in shared memory by every CTA of the locate: 9 levels
// (511 heap entries = 8 KB of (first, last)) measured faster than 10 or 11
// (the staging of each persistent CTA costs more than a descent level) and
// than 8
constexpr int TOPL = 9;
constexpr int TOPN = (1 << TOPL) - 1;
constexpr int LSUM = 8;                // windows up to 2^8 segments sum counts directly
constexpr uint32_t SUP_CHUNKS = 64;     // chunks (of TPB keys) per group total of the locate

__device__ inline uint32_t warp_sum(uint32_t v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// smallest y in [0, y0] with seg[y] >= a, given seg[y0] >= a
__device__ inline uint32_t lb_back(const uint32_t *seg, uint32_t y, uint32_t a) {
    uint32_t step = 1;
    while (y > 0) {
        uint32_t t = y > step ? y - step : 0;
        if (seg[t] >= a) {
            y = t;
            step <<= 1;
            continue;
        }
        uint32_t L = t + 1, R = y;
        while (L < R) {
            uint32_t mid = (L + R) >> 1;
            if (seg[mid] >= a)
                R = mid;
            else
                L = mid + 1;
        }
        return L;
    }
    return 0;
}

// smallest y in [y0, n] with seg[y] >= b (n if none), given seg[y0-1] < b
__device__ inline uint32_t lb_fwd(const uint32_t *seg, uint32_t y, uint32_t n, uint64_t b) {
    if (y >= n || seg[y] >= b) return y;
    uint32_t low = y, step = 1;  // seg[low] < b
    while (true) {
        uint64_t t = (uint64_t)low + step;
        if (t >= n) {
            t = n;
        } else if (seg[t] < b) {
            low = (uint32_t)t;
            step <<= 1;
            continue;
        }
        uint32_t L = low + 1, R = (uint32_t)t;  // answer in [L, R]
        while (L < R) {
            uint32_t mid = (L + R) >> 1;
            if (seg[mid] >= b)
                R = mid;
            else
                L = mid + 1;
        }
        return L;
    }
}

// first index in [lo, hi) whose key is >= k
__device__ inline uint32_t lb_key(const uint64_t *key, uint32_t lo, uint32_t hi, uint64_t k) {
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (key[mid] < k)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// Descend the in-order segment tree (locate_leaf_kernel, rpma.cuh:281-310):
// stop at an empty node or at a leaf; go left when key < first, right when
// key > last, else stop.  (first, last) per heap segment; the top TOPL
// levels come from shared memory.
__device__ inline uint64_t descend(uint64_t key, const ulonglong2 *top, uint32_t ntop, const ulonglong2 *fl,
                                   uint32_t H, uint32_t *level_out) {
    uint64_t j = 0;
    uint32_t lvl = 0;
    while (lvl < H) {
        ulonglong2 f = j < ntop ? top[j] : fl[j];
        if (f.x == KEY_NONE) break;
        if (key < f.x)
            j = 2 * j + 1;
        else if (key > f.y)
            j = 2 * j + 2;
        else
            break;
        ++lvl;
    }
    *level_out = lvl;
    return j;
}

// ------------------------------------------------------------------ pack
__device__ __forceinline__ void k_pack_body(const uint64_t *__restrict__ ins, const uint8_t *__restrict__ ins_vals,
                                              uint32_t n_ins, const uint64_t *__restrict__ del, uint32_t n_del,
                                              uint32_t V, uint32_t thres, uint32_t key_format, int internal,
                                              uint64_t *__restrict__ keys_out, uint16_t *__restrict__ pay_out,
                                              DevStatus *st, uint32_t bid_, uint32_t nblk_) {
    const uint32_t n = n_ins + n_del;
    unsigned long long kand = ~0ull, kor = 0;
    uint32_t mint = 0xFFFFFFFFu, bad = 0xFFFFFFFFu;
    for (uint32_t i = bid_ * TPB + threadIdx.x; i < n; i += nblk_ * TPB) {
        uint64_t k;
        uint16_t pay;
        bool ok;
        const bool is_del = i >= n_ins;
        k = is_del ? del[i - n_ins] : ins[i];
        bool range_ok = true;
        if (key_format == 1) {  // src << 32 | dst
            uint64_t s = k >> 32, d = k & 0xFFFFFFFFull;
            range_ok = s < V && d < V;
            k = (s << SRC_SHIFT) | (d << DST_SHIFT);
        }
        const uint64_t src = k >> SRC_SHIFT, dst = (k & DST_MASK) >> DST_SHIFT;
        if (!is_del) {
            uint8_t v = ins_vals ? ins_vals[i] : (uint8_t)1;
            ok = range_ok && k != KEY_NONE && src < V && ((internal && is_sentinel(k)) || dst < V) && v != VAL_TOMB &&
                 (k & TIME_MASK) >= (uint64_t)thres;
            pay = v;
            mint = min(mint, (uint32_t)(k & TIME_MASK));
        } else {
            ok = range_ok && k != KEY_NONE && src < V && dst < V;
            pay = 0x100;
        }
        if (!ok) bad = min(bad, i);
        keys_out[i] = k;
        pay_out[i] = pay;
        kand &= k;
        kor |= k;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        kand &= __shfl_xor_sync(0xffffffffu, kand, o);
        kor |= __shfl_xor_sync(0xffffffffu, kor, o);
        mint = min(mint, __shfl_xor_sync(0xffffffffu, mint, o));
        bad = min(bad, __shfl_xor_sync(0xffffffffu, bad, o));
    }
    // one set of atomics per block: the status words are single addresses
    __shared__ unsigned long long s_and[TPB / 32], s_or[TPB / 32];
    __shared__ uint32_t s_min[TPB / 32], s_bad[TPB / 32];
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) s_and[w] = kand, s_or[w] = kor, s_min[w] = mint, s_bad[w] = bad;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int i = 1; i < TPB / 32; i++) {
            kand &= s_and[i];
            kor |= s_or[i];
            mint = min(mint, s_min[i]);
            bad = min(bad, s_bad[i]);
        }
        atomicAnd(&st->key_and, kand);
        atomicOr(&st->key_or, kor);
        if (mint != 0xFFFFFFFFu) atomicMin(&st->min_t_ins, mint);
        if (bad != 0xFFFFFFFFu) {
            atomicOr(&st->error, ERR_KEY);
            atomicMin(&st->err_info[0], bad);
        }
    }
}

// Bulk L2 prefetch of [p, p + bytes) (p 16-byte aligned), spread over the
// grid in 4 KB requests; bytes past the last multiple of 16 are left out.
__device__ __forceinline__ void l2_prefetch(const void *p, uint64_t bytes) {
    constexpr uint64_t CH = 4096;
    const uint64_t nch = (bytes + CH - 1) / CH;
    for (uint64_t c = (uint64_t)blockIdx.x * TPB + threadIdx.x; c < nch; c += (uint64_t)gridDim.x * TPB) {
        const uint64_t off = c * CH;
        const uint32_t len = (uint32_t)(umin64(CH, bytes - off) & ~15ull);
        if (len) asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"((const char *)p + off), "r"(len) : "memory");
    }
}

__global__ void __launch_bounds__(TPB) k_pack(const uint64_t *__restrict__ ins, const uint8_t *__restrict__ ins_vals,
                                              uint32_t n_ins, const uint64_t *__restrict__ del, uint32_t n_del,
                                              uint32_t V, uint32_t thres, uint32_t key_format, int internal,
                                              uint64_t *__restrict__ keys_out, uint16_t *__restrict__ pay_out,
                                              DevStatus *st, uint32_t *bitmap, uint32_t bitmap_words,
                                              const ulonglong2 *fl, const uint8_t *cnt, uint64_t pf_segs,
                                              uint32_t *sup, uint32_t sup_words, uint32_t *sort_bar) {
    // the planner bitmap and the locate's chunk-group totals of this call
    // start clear
    for (uint32_t i = blockIdx.x * TPB + threadIdx.x; i < bitmap_words; i += gridDim.x * TPB) bitmap[i] = 0;
    for (uint32_t i = blockIdx.x * TPB + threadIdx.x; i < sup_words; i += gridDim.x * TPB) sup[i] = 0;
    // the cooperative sort's barrier counter (the sort that follows)
    if (sort_bar && blockIdx.x == 0 && threadIdx.x == 0) *sort_bar = 0;
    k_pack_body(ins, ins_vals, n_ins, del, n_del, V, thres, key_format, internal, keys_out, pay_out, st, blockIdx.x, gridDim.x);
    // the segment bounds and counts that the locate and the planner read at
    // random come into L2 while the batch is sorted (the sort runs out of L2
    // and leaves DRAM idle); issued after the block's own accesses
    if (pf_segs) {
        l2_prefetch(fl, 16 * pf_segs);
        l2_prefetch(cnt, pf_segs);
    }
}

// ------------------------------------------------------------------ live counts
__global__ void __launch_bounds__(TPB) k_live_counts(const uint64_t *__restrict__ keys, uint32_t H, uint32_t thres,
                                                     uint8_t *cnt_live, DevStatus *st) {
    const uint64_t nseg = nseg_of(H);
    const int lane = threadIdx.x & 31;
    uint32_t acc = 0;
    for (uint64_t s = (blockIdx.x * (uint64_t)TPB + threadIdx.x) >> 5; s < nseg; s += (gridDim.x * (uint64_t)TPB) >> 5) {
        uint64_t j = heap_of_linear(s, H);
        uint64_t k = keys[32 * j + lane];
        uint32_t c = __popc(__ballot_sync(0xffffffffu, k != KEY_NONE && (k & TIME_MASK) >= (uint64_t)thres));
        if (lane == 0) cnt_live[s] = (uint8_t)c;
        acc += c;
    }
    if (lane == 0 && acc) atomicAdd(&st->live_total, (unsigned long long)acc);
}

// ------------------------------------------------------------------ resolve + locate
__device__ __forceinline__ void k_resolve_locate_body(const uint64_t *__restrict__ k0,
                                                        const uint16_t *__restrict__ p0,
                                                        const uint64_t *__restrict__ k1,
                                                        const uint16_t *__restrict__ p1, uint32_t n, SortMask mask,
                                                        Geo g, const ulonglong2 *__restrict__ fl, uint32_t thres,
                                                        uint8_t *kind, uint32_t *seg, uint32_t *blk_nn,
                                                        uint32_t *blk_ins, uint32_t *sup, DevStatus *st, uint32_t bid_,
                                                        uint32_t nblk_) {
    const bool odd = sort_result_odd(mask, n);
    const uint64_t *__restrict__ skey = odd ? k1 : k0;
    const uint16_t *__restrict__ spay = odd ? p1 : p0;
    // a rejected batch (validation in k_pack), or one whose sort gave up a
    // bounded wait, changes nothing
    const bool rejected = (st->error & (ERR_KEY | ERR_TIMEOUT)) != 0;
    // persistent grid: the top TOPL levels are staged once per CTA and the
    // CTA walks 256-entry chunks; chunk c writes its counts to blk_*[c]
    __shared__ ulonglong2 top[TOPN];
    const uint32_t H = g.H;
    const uint32_t ntop = (uint32_t)umin64(nseg_of(H), TOPN);
    for (uint32_t t = threadIdx.x; t < ntop; t += TPB) top[t] = fl[t];
    __syncthreads();
    const uint32_t nchunks = (n + TPB - 1) / TPB;
    uint32_t ups = 0, noop = 0;
    for (uint32_t chunk = bid_; chunk < nchunks; chunk += nblk_) {
        const uint32_t i = chunk * TPB + threadIdx.x;
        uint32_t kd = KIND_NOP, sg = 0;
        if (i < n && !rejected) {
            const uint64_t key = skey[i];
            const uint16_t p = spay[i];
            const bool is_del = (p >> 8) & 1;
            bool rep;
            if (is_del)
                rep = (i == 0 || skey[i - 1] != key);
            else
                rep = (i + 1 == n || skey[i + 1] != key || ((spay[i + 1] >> 8) & 1));
            if (rep) {
                uint32_t lvl;
                const uint64_t j = descend(key, top, ntop, fl, H, &lvl);
                sg = (uint32_t)linear_of_heap(j, lvl, H);
                // membership: the stop segment is sorted, NONE-padded (left packed)
                const uint64_t *sk = g.keys + 32 * j;
                uint32_t pos = 0;
#pragma unroll
                for (uint32_t step = 16; step; step >>= 1)
                    if (sk[pos + step - 1] < key) pos += step;
                const bool found = sk[pos] == key;
                const uint64_t slot = 32 * j + pos;
                if (!is_del) {
                    if (found) {
                        g.vals[slot] = (uint8_t)(p & 0xFF);  // upsert (handle_del_mod, gpma.cuh:162-175)
                        ups++;
                    } else {
                        kd = KIND_INS;
                    }
                } else {
                    if (found && (key & TIME_MASK) >= (uint64_t)thres) {
                        g.vals[slot] = VAL_TOMB;  // tombstone until its window executes
                        kd = KIND_DEL;
                    } else {
                        noop++;
                    }
                }
            } else {
                noop++;
            }
        }
        if (i < n) {
            kind[i] = (uint8_t)kd;
            seg[i] = sg;
        }
        const uint32_t c_nn = __syncthreads_count(kd != KIND_NOP);
        const uint32_t c_ins = __syncthreads_count(kd == KIND_INS);
        if (threadIdx.x == 0) {
            blk_nn[chunk] = c_nn;
            blk_ins[chunk] = c_ins;
            // totals per group of SUP_CHUNKS chunks, for the compaction's offsets
            if (sup && c_nn) {
                atomicAdd(&sup[2 * (chunk / SUP_CHUNKS)], c_nn);
                if (c_ins) atomicAdd(&sup[2 * (chunk / SUP_CHUNKS) + 1], c_ins);
            }
        }
    }
    ups = warp_sum(ups);
    noop = warp_sum(noop);
    if ((threadIdx.x & 31) == 0) {
        if (ups) atomicAdd(&st->n_upsert, ups);
        if (noop) atomicAdd(&st->n_noop, noop);
    }
}

__global__ void __launch_bounds__(TPB) k_resolve_locate(const uint64_t *__restrict__ k0,
                                                        const uint16_t *__restrict__ p0,
                                                        const uint64_t *__restrict__ k1,
                                                        const uint16_t *__restrict__ p1, uint32_t n, SortMask mask,
                                                        Geo g, const ulonglong2 *__restrict__ fl, uint32_t thres,
                                                        uint8_t *kind, uint32_t *seg, uint32_t *blk_nn,
                                                        uint32_t *blk_ins, uint32_t *sup, DevStatus *st) {
    griddep_wait();
    k_resolve_locate_body(k0, p0, k1, p1, n, mask, g, fl, thres, kind, seg, blk_nn, blk_ins, sup, st, blockIdx.x,
                          gridDim.x);
}

// exclusive scans of the two block-count arrays (one CTA); totals -> status
__device__ __forceinline__ void k_scan_pairs_body(uint32_t *a, uint32_t *b, uint32_t nb, uint32_t *ip,
                                                     DevStatus *st, uint32_t bid_, uint32_t nblk_) {
    // one pass per 8192 entries: each of the 1024 threads loads up to 8
    // consecutive pairs at once, the thread sums are scanned, then each
    // thread writes its run
    constexpr uint32_t PER = 8;
    __shared__ uint32_t wa[32], wb[32];
    __shared__ uint32_t ca, cb;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) ca = cb = 0;
    __syncthreads();
    for (uint32_t b0 = 0; b0 < nb; b0 += 1024 * PER) {
        const uint32_t cnt = nb - b0 < 1024 * PER ? nb - b0 : 1024 * PER;
        const uint32_t per = (cnt + 1023) / 1024;
        const uint32_t beg = b0 + threadIdx.x * per, end = b0 + cnt;
        uint32_t xa[PER], xb[PER], sa = 0, sb = 0;
#pragma unroll
        for (uint32_t q = 0; q < PER; q++) {
            const bool in = q < per && beg + q < end;
            xa[q] = in ? a[beg + q] : 0u;
            xb[q] = in ? b[beg + q] : 0u;
            sa += xa[q];
            sb += xb[q];
        }
        uint32_t va = sa, vb = sb;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t ya = __shfl_up_sync(0xffffffffu, va, o), yb = __shfl_up_sync(0xffffffffu, vb, o);
            if (lane >= o) va += ya, vb += yb;
        }
        if (lane == 31) wa[w] = va, wb[w] = vb;
        __syncthreads();
        if (w == 0) {
            uint32_t ta = wa[lane], tb = wb[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t ya = __shfl_up_sync(0xffffffffu, ta, o), yb = __shfl_up_sync(0xffffffffu, tb, o);
                if (lane >= o) ta += ya, tb += yb;
            }
            wa[lane] = ta;
            wb[lane] = tb;
        }
        __syncthreads();
        uint32_t ra = ca + (w ? wa[w - 1] : 0) + va - sa, rb = cb + (w ? wb[w - 1] : 0) + vb - sb;
#pragma unroll
        for (uint32_t q = 0; q < PER; q++) {
            if (q < per && beg + q < end) {
                a[beg + q] = ra;
                b[beg + q] = rb;
            }
            ra += xa[q];
            rb += xb[q];
        }
        __syncthreads();
        if (threadIdx.x == 0) ca += wa[31], cb += wb[31];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        st->n_u = ca;
        st->n_ins = cb;
        st->n_del = ca - cb;
        ip[ca] = cb;
    }
}

__global__ void __launch_bounds__(1024) k_scan_pairs(uint32_t *a, uint32_t *b, uint32_t nb, uint32_t *ip,
                                                     DevStatus *st) {
    griddep_wait();
    k_scan_pairs_body(a, b, nb, ip, st, blockIdx.x, gridDim.x);
}

__device__ inline uint32_t block_excl_scan(uint32_t x, uint32_t *wsum) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t v = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += y;
    }
    if (lane == 31) wsum[w] = v;
    __syncthreads();
    if (w == 0) {
        uint32_t s = lane < TPB / 32 ? wsum[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < TPB / 32) wsum[lane] = s;
    }
    __syncthreads();
    uint32_t r = (w ? wsum[w - 1] : 0) + v - x;
    __syncthreads();
    return r;
}

// The same over u64 values (fields packed in the word add independently as
// long as none of the block's sums overflows its field).
__device__ inline uint64_t block_excl_scan_u64(uint64_t x, uint64_t *wsum) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint64_t v = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint64_t y = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += y;
    }
    if (lane == 31) wsum[w] = v;
    __syncthreads();
    if (w == 0) {
        uint64_t t = lane < TPB / 32 ? wsum[lane] : 0;
#pragma unroll
        for (int o = 1; o < TPB / 32; o <<= 1) {
            const uint64_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < TPB / 32) wsum[lane] = t;
    }
    __syncthreads();
    const uint64_t r = (w ? wsum[w - 1] : 0) + v - x;
    __syncthreads();
    return r;
}

// How many of n keys the tree stores (live or tombstoned): the locate
// descent and the membership search of k_resolve_locate, read only.
__global__ void __launch_bounds__(TPB) k_count_present(const uint64_t *__restrict__ keys, uint32_t n,
                                                       uint32_t key_format, Geo g, const ulonglong2 *__restrict__ fl,
                                                       uint32_t *count) {
    uint32_t c = 0;
    for (uint32_t i = blockIdx.x * TPB + threadIdx.x; i < n; i += gridDim.x * TPB) {
        uint64_t key = keys[i];
        if (key_format == 1) key = ((key >> 32) << SRC_SHIFT) | ((key & 0xFFFFFFFFull) << DST_SHIFT);
        uint32_t lvl;
        const uint64_t j = descend(key, nullptr, 0, fl, g.H, &lvl);
        const uint64_t *sk = g.keys + 32 * j;
        uint32_t pos = 0;
#pragma unroll
        for (uint32_t step = 16; step; step >>= 1)
            if (sk[pos + step - 1] < key) pos += step;
        c += (pos < 32 && sk[pos] == key) ? 1u : 0u;
    }
    c = __reduce_add_sync(0xffffffffu, c);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, c);
}

__device__ __forceinline__ void k_compact_body(const uint64_t *__restrict__ k0, const uint16_t *__restrict__ p0,
                                                 const uint64_t *__restrict__ k1, const uint16_t *__restrict__ p1,
                                                 SortMask mask, const uint8_t *__restrict__ kind,
                                                 const uint32_t *__restrict__ seg, uint32_t n,
                                                 const uint32_t *blk_nn, const uint32_t *blk_ins,
                                                 const uint32_t *sup, UpdList u, DevStatus *st, uint32_t bid_,
                                                 uint32_t nblk_) {
    const bool odd = sort_result_odd(mask, n);
    const uint64_t *__restrict__ skey = odd ? k1 : k0;
    const uint16_t *__restrict__ spay = odd ? p1 : p0;
    __shared__ uint32_t wsum[TPB / 32];
    __shared__ uint64_t wsum64[TPB / 32];
    // this chunk's offsets: with sup, the counts of the chunks before it
    // (whole groups from the group totals, then the chunks of its own group;
    // nn in the low half of the sum, inserts in the high half); without, the
    // scanned chunk counts
    uint32_t base_nn, base_ins;
    if (sup) {
        const uint32_t grp = bid_ / SUP_CHUNKS;
        uint64_t acc = 0;
        for (uint32_t t = threadIdx.x; t < grp; t += TPB)
            acc += (uint64_t)sup[2 * t] | ((uint64_t)sup[2 * t + 1] << 32);
        for (uint32_t t = grp * SUP_CHUNKS + threadIdx.x; t < bid_; t += TPB)
            acc += (uint64_t)blk_nn[t] | ((uint64_t)blk_ins[t] << 32);
#pragma unroll
        for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if ((threadIdx.x & 31) == 0) wsum64[threadIdx.x >> 5] = acc;
        __syncthreads();
        acc = 0;
#pragma unroll
        for (int w = 0; w < TPB / 32; w++) acc += wsum64[w];
        base_nn = (uint32_t)acc, base_ins = (uint32_t)(acc >> 32);
    } else {
        base_nn = blk_nn[bid_], base_ins = blk_ins[bid_];
    }
    const uint32_t i = bid_ * TPB + threadIdx.x;
    const uint32_t kd = i < n ? kind[i] : KIND_NOP;
    // pack (kept, insert) flags into one scan word
    const uint32_t x = (kd != KIND_NOP ? 1u : 0u) | (kd == KIND_INS ? 1u << 16 : 0u);
    const uint32_t ex = block_excl_scan(x, wsum);
    if (kd != KIND_NOP) {
        const uint32_t pos = base_nn + (ex & 0xFFFF);
        u.key[pos] = skey[i];
        u.val[pos] = (uint8_t)(spay[i] & 0xFF);
        u.kind[pos] = (uint8_t)kd;
        u.seg[pos] = seg[i];
        u.ip[pos] = base_ins + (ex >> 16);
    }
    // the last chunk knows the totals: list length, inserts, the end of ip
    if (sup && bid_ == nblk_ - 1 && threadIdx.x == TPB - 1) {
        const uint32_t t = ex + x, nu = base_nn + (t & 0xFFFF), ni = base_ins + (t >> 16);
        st->n_u = nu;
        st->n_ins = ni;
        st->n_del = nu - ni;
        u.ip[nu] = ni;
    }
}

__global__ void __launch_bounds__(TPB) k_compact(const uint64_t *__restrict__ k0, const uint16_t *__restrict__ p0,
                                                 const uint64_t *__restrict__ k1, const uint16_t *__restrict__ p1,
                                                 SortMask mask, const uint8_t *__restrict__ kind,
                                                 const uint32_t *__restrict__ seg, uint32_t n,
                                                 const uint32_t *blk_nn, const uint32_t *blk_ins,
                                                 const uint32_t *sup, UpdList u, DevStatus *st) {
    griddep_wait();
    k_compact_body(k0, p0, k1, p1, mask, kind, seg, n, blk_nn, blk_ins, sup, u, st, blockIdx.x, gridDim.x);
}

// ------------------------------------------------------------------ relocate / pending
__global__ void __launch_bounds__(TPB) k_relocate(UpdList u, uint32_t n, Geo g, const ulonglong2 *__restrict__ fl) {
    __shared__ ulonglong2 top[TOPN];
    const uint32_t H = g.H;
    const uint32_t ntop = (uint32_t)umin64(nseg_of(H), TOPN);
    for (uint32_t t = threadIdx.x; t < ntop; t += TPB) top[t] = fl[t];
    __syncthreads();
    const uint32_t i = blockIdx.x * TPB + threadIdx.x;
    if (i >= n) return;
    uint32_t lvl;
    uint64_t j = descend(u.key[i], top, ntop, fl, H, &lvl);
    u.seg[i] = (uint32_t)linear_of_heap(j, lvl, H);
}

__global__ void __launch_bounds__(TPB) k_pending_counts(const uint8_t *__restrict__ kind, const uint8_t *__restrict__ pend,
                                                        uint32_t n, const DevStatus *st, uint32_t *blk_nn,
                                                        uint32_t *blk_ins) {
    const uint32_t nu = st->n_u;
    const uint32_t i = blockIdx.x * TPB + threadIdx.x;
    const bool keep = i < n && i < nu && pend[i];
    uint32_t c = __syncthreads_count(keep);
    uint32_t ci = __syncthreads_count(keep && kind[i] == KIND_INS);
    if (threadIdx.x == 0) {
        blk_nn[blockIdx.x] = c;
        blk_ins[blockIdx.x] = ci;
    }
}

__global__ void __launch_bounds__(TPB) k_pending_scatter(const UpdList in, const uint8_t *__restrict__ pend, uint32_t n,
                                                         uint32_t nu_old, const uint32_t *blk_nn,
                                                         const uint32_t *blk_ins, UpdList out) {
    __shared__ uint32_t wsum[TPB / 32];
    const uint32_t i = blockIdx.x * TPB + threadIdx.x;
    const bool keep = i < n && i < nu_old && pend[i];
    const uint32_t kd = keep ? in.kind[i] : KIND_NOP;
    const uint32_t x = (keep ? 1u : 0u) | (kd == KIND_INS ? 1u << 16 : 0u);
    const uint32_t ex = block_excl_scan(x, wsum);
    if (keep) {
        const uint32_t pos = blk_nn[blockIdx.x] + (ex & 0xFFFF);
        out.key[pos] = in.key[i];
        out.val[pos] = in.val[i];
        out.kind[pos] = (uint8_t)kd;
        out.seg[pos] = in.seg[i];
        out.ip[pos] = blk_ins[blockIdx.x] + (ex >> 16);
    }
}

// ------------------------------------------------------------------ planner
// Sum of the counts of the window [a, a + 2^l) clipped to nseg segments.
// The last window of a level reaches one entry past the last segment
// (a + 2^l = nseg + 1); that entry is not a segment and may hold a stale
// count from another height, so it is taken back out.
__device__ inline uint32_t sum_cnt(const uint8_t *cnt, uint64_t a, uint32_t l, uint64_t nseg) {
    uint32_t s = 0;
    if (l < 4) {
        for (uint32_t t = 0; t < (1u << l); t++)
            if (a + t < nseg) s += cnt[a + t];
        return s;
    }
    const uint4 *p = reinterpret_cast<const uint4 *>(cnt + a);
    for (uint32_t t = 0; t < (1u << (l - 4)); t++) {
        uint4 v = p[t];
        s = __dp4a(v.x, 0x01010101u, s);
        s = __dp4a(v.y, 0x01010101u, s);
        s = __dp4a(v.z, 0x01010101u, s);
        s = __dp4a(v.w, 0x01010101u, s);
    }
    if (a + (1ull << l) > nseg) s -= cnt[nseg];
    return s;
}

__device__ inline uint64_t bit_of(uint32_t H, uint32_t l, uint64_t widx) {
    return ((1ull << (H + 2)) - (1ull << (H + 2 - l))) + widx;
}

__device__ __forceinline__ void k_plan_body(const UpdList u, uint32_t n_cap, const uint8_t *__restrict__ cnt,
                                              const uint32_t *__restrict__ P, int use_P, uint64_t total_live_host,
                                              const unsigned long long *__restrict__ total_live_dev, uint32_t H,
                                              Tables tb, uint32_t *bitmap, Window *cand, uint8_t *pend,
                                              DevStatus *st, uint32_t bid_, uint32_t nblk_) {
    const uint64_t total_live = total_live_dev ? *total_live_dev : total_live_host;
    __shared__ uint32_t wsum[TPB / 32];
    __shared__ uint32_t base_s;
    __shared__ uint32_t s_lv, s_fl;  // executed levels; bit 0 an overflow, bit 1 a root window
    if (threadIdx.x == 0) s_lv = 0, s_fl = 0;
    __syncthreads();
    const uint32_t nu = st->n_u;
    const uint32_t x = bid_ * TPB + threadIdx.x;
    uint32_t s = 0;
    bool lead = false;
    if (x < nu && x < n_cap) {
        s = u.seg[x];
        lead = (x == 0 || u.seg[x - 1] != s);  // one thread per segment with updates
    }
    uint32_t e = EXEC_OVF, lo = x, hi = x;
    uint64_t wa = 0, wf = 0;
    int64_t wm = 0;
    bool own = false;
    if (lead) {
        const uint32_t hi0 = lb_fwd(u.seg, x, nu, (uint64_t)s + 1);
        const uint64_t nseg = tb.nseg ? tb.nseg : nseg_of(H);
        const uint64_t seg_len = tb.seg_len ? tb.seg_len : 32u;
        hi = hi0;
        for (uint32_t l = 0; l <= H + 1; l++) {
            if (!((tb.allowed >> l) & 1u)) continue;
            const uint64_t a = ((uint64_t)s >> l) << l;
            const uint64_t b = umin64(a + (1ull << l), nseg);
            lo = lb_back(u.seg, lo, (uint32_t)a);
            hi = lb_fwd(u.seg, hi, nu, b);
            int64_t live;
            if (l == H + 1)
                live = (int64_t)total_live;
            else if (l <= LSUM || !use_P)
                live = sum_cnt(cnt, a, l, nseg);
            else
                live = (int64_t)P[b] - (int64_t)P[a];
            const int64_t net = 2 * ((int64_t)u.ip[hi] - (int64_t)u.ip[lo]) - (int64_t)(hi - lo);
            const int64_t m = live + net;
            if (m >= (int64_t)tb.lower[l] && m <= (int64_t)(seg_len * (b - a))) {
                e = l;
                wa = a;
                wf = b - a;
                wm = m;
                break;
            }
        }
        // the run's pending mark (read on the overflow paths; the other
        // updates of the run copy it from here)
        pend[x] = (uint8_t)(e == EXEC_OVF);
        if (e == 0) {
            // a single-segment window has one leader, and the maximality
            // probe never reads level 0: no bitmap atomic on the common path
            own = true;
        } else if (e != EXEC_OVF) {
            const uint64_t bit = bit_of(H, e, (uint64_t)s >> e);
            const uint32_t mask = 1u << (bit & 31);
            own = !(atomicOr(&bitmap[bit >> 5], mask) & mask);
        }
    }
    // levels with an executed window (for the maximality test), overflow
    // and root flags: one block barrier for all three
    const uint32_t lv = __reduce_or_sync(0xffffffffu, (lead && e != EXEC_OVF) ? 1u << e : 0u);
    const uint32_t fg = __reduce_or_sync(0xffffffffu, (lead && e == EXEC_OVF ? 1u : 0u) | (lead && e == H + 1 ? 2u : 0u));
    if ((threadIdx.x & 31) == 0) {
        if (lv) atomicOr(&s_lv, lv);
        if (fg) atomicOr(&s_fl, fg);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (s_fl & 1u) atomicOr(&st->ovf, 1u);
        if (s_fl & 2u) atomicOr(&st->root, 1u);
        if (s_lv) atomicOr(&st->exec_levels, s_lv);
    }
    // block-aggregated append of the windows this block owns
    const uint32_t ex = block_excl_scan(own ? 1u : 0u, wsum);
    if (threadIdx.x == TPB - 1 && ex + (own ? 1u : 0u)) base_s = atomicAdd(&st->n_cand, ex + (own ? 1u : 0u));
    __syncthreads();
    if (own) cand[base_s + ex] = Window{(uint32_t)wa, (uint32_t)wf, (uint32_t)wm, e, lo, hi};
}

__global__ void __launch_bounds__(TPB) k_plan(const UpdList u, uint32_t n_cap, const uint8_t *__restrict__ cnt,
                                              const uint32_t *__restrict__ P, int use_P, uint64_t total_live_host,
                                              const unsigned long long *__restrict__ total_live_dev, uint32_t H,
                                              Tables tb, uint32_t *bitmap, Window *cand, uint8_t *pend,
                                              DevStatus *st) {
    griddep_wait();
    k_plan_body(u, n_cap, cnt, P, use_P, total_live_host, total_live_dev, H, tb, bitmap, cand, pend, st, blockIdx.x, gridDim.x);
}

// Keep the candidates not inside a larger executed window; sort them into
// single-segment, small (<= 32 segments) and big lists.
__device__ __forceinline__ void k_plan_max_body(const Window *__restrict__ cand, uint32_t n_cap, uint32_t H,
                                                  const uint32_t *__restrict__ bitmap, Window *single, Window *small4,
                                                  Window *small, Window *big, const UpdList u, uint8_t *pend,
                                                  DevStatus *st, uint32_t bid_, uint32_t nblk_,
                                                  uint32_t cut_group = CUT_GROUP_DEFAULT,
                                                  uint32_t cut_shared = SMALL_WIN_SEGS) {
    // updates of segments that no window absorbed stay pending (overflow):
    // each update copies the mark its run's first update (the planner's
    // leader) wrote.  The marks are read only on the overflow paths.
    if (st->ovf) {
        const uint32_t x = bid_ * TPB + threadIdx.x;
        if (x < st->n_u && x < n_cap) {
            const uint32_t s = u.seg[x];
            if (x > 0 && u.seg[x - 1] == s) pend[x] = pend[lb_back(u.seg, x, s)];
        }
    }
    __shared__ uint64_t wsum[TPB / 32];
    __shared__ uint32_t base_s[4];
    __shared__ unsigned long long sl[2][TPB / 32];
    const uint32_t c = bid_ * TPB + threadIdx.x;
    // classes: 0 single segment, 1 two to cut_group (4), 2 up to cut_shared (32),
    // 3 larger, 4 none
    uint32_t cls = 4;
    Window w{};
    if (c < st->n_cand && c < n_cap) {
        w = cand[c];
        cls = w.f == 1 ? 0 : (w.f <= cut_group ? 1 : (w.f <= cut_shared ? 2 : 3));
        // inside a larger executed window?  The ancestor words are loaded
        // without an early exit so that the loads are in flight together.
        uint32_t hit = 0;
        const uint32_t lv = st->exec_levels;
        const uint32_t ltop = lv ? min(H + 1, 31u - __clz(lv)) : 0u;  // the highest executed level
#pragma unroll 4
        for (uint32_t l = w.level + 1; l <= ltop; l++) {
            if (!((lv >> l) & 1u)) continue;  // no window of that level executes
            const uint64_t bit = bit_of(H, l, (uint64_t)w.a >> l);
            hit |= (bitmap[bit >> 5] >> (bit & 31)) & 1u;
        }
        if (hit) cls = 4;
    }
    // the four classes' positions in one scan: a 16-bit field each (at most
    // TPB per block), classes 0 and 1 in the low word, 2 and 3 in the high
    const uint32_t pa = cls < 2 ? 1u << (16 * cls) : 0u;
    const uint32_t pb = (cls == 2 || cls == 3) ? 1u << (16 * (cls - 2)) : 0u;
    const uint64_t exab = block_excl_scan_u64((uint64_t)pa | ((uint64_t)pb << 32), wsum);
    const uint32_t exa = (uint32_t)exab, exb = (uint32_t)(exab >> 32);
    // slots of disjoint maximal windows: a warp's sums stay below 2^32
    uint32_t s_small = cls <= 2 ? 32u * w.f : 0u, s_big = cls == 3 ? 32u * w.f : 0u;
    uint32_t t_big = cls == 3 ? (w.f + 31) / 32 : 0u;
    s_small = __reduce_add_sync(0xffffffffu, s_small);
    s_big = __reduce_add_sync(0xffffffffu, s_big);
    t_big = __reduce_add_sync(0xffffffffu, t_big);
    if ((threadIdx.x & 31) == 0 && t_big) atomicAdd(&st->big_tiles, t_big);
    if ((threadIdx.x & 31) == 0) sl[0][threadIdx.x >> 5] = s_small, sl[1][threadIdx.x >> 5] = s_big;
    if (threadIdx.x == TPB - 1) {
        // the status words share a cache line: only the lists this block
        // appends to take an atomic
        const uint32_t ta = exa + pa, tb = exb + pb;
        if (ta & 0xFFFFu) base_s[0] = atomicAdd(&st->n_single, ta & 0xFFFFu);
        if (ta >> 16) base_s[1] = atomicAdd(&st->n_small4, ta >> 16);
        if (tb & 0xFFFFu) base_s[2] = atomicAdd(&st->n_small, tb & 0xFFFFu);
        if (tb >> 16) base_s[3] = atomicAdd(&st->n_big, tb >> 16);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long a = 0, b = 0;
        for (int i = 0; i < TPB / 32; i++) a += sl[0][i], b += sl[1][i];
        if (a) atomicAdd(&st->slots_small, a);
        if (b) atomicAdd(&st->slots_big, b);
    }
    if (cls < 4) {
        const uint32_t ex = cls < 2 ? exa : exb;
        const uint32_t idx = base_s[cls] + ((ex >> (16 * (cls & 1))) & 0xFFFFu);
        (cls == 0 ? single : cls == 1 ? small4 : cls == 2 ? small : big)[idx] = w;
    }
}

// pub (optional): the handle's pinned host mirror of the status block.  The
// last CTA to finish (a counter in the status block) copies the status words
// there and then sets pub->published, so the host reads the front's verdict
// as soon as the plan is complete, without a copy node and an event behind it.
__global__ void __launch_bounds__(TPB) k_plan_max(const Window *__restrict__ cand, uint32_t n_cap, uint32_t H,
                                                  const uint32_t *__restrict__ bitmap, Window *single, Window *small4,
                                                  Window *small, Window *big, const UpdList u, uint8_t *pend,
                                                  DevStatus *st, uint32_t cut_group, uint32_t cut_shared,
                                                  DevStatus *pub) {
    griddep_wait();
    k_plan_max_body(cand, n_cap, H, bitmap, single, small4, small, big, u, pend, st, blockIdx.x, gridDim.x, cut_group,
                    cut_shared);
    if (pub == nullptr) return;  // uniform over the grid
    __shared__ uint32_t last;
    __threadfence();  // this CTA's status atomics before its count
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(&st->plan_done, 1u) == gridDim.x - 1 ? 1u : 0u;
    __syncthreads();
    if (!last) return;
    __threadfence();
    constexpr uint32_t W = offsetof(DevStatus, published) / 4;  // every word up to the flag
    const volatile uint32_t *src = reinterpret_cast<const volatile uint32_t *>(st);
    volatile uint32_t *dst = reinterpret_cast<volatile uint32_t *>(pub);
    for (uint32_t i = threadIdx.x; i < W; i += TPB) dst[i] = src[i];
    __threadfence_system();  // the words before the flag, for the host
    __syncthreads();
    if (threadIdx.x == 0) dst[W] = 1u;
}

// ------------------------------------------------------------------ multi-segment windows
// Both classes merge a window the same way: the window's inserts are staged
// in shared memory at their insert rank (the update list is in key order),
// the kept keys of the whole window are compacted in slot order, each
// insert finds its merged rank (insert index + kept keys below it, a binary
// search) and marks it in a bitmask, and every output slot takes its key by
// a popcount of the marks below its rank: a marked rank holds the insert of
// that index, any other the kept key of index rank - marks below.  This is
// the merge of the per-segment runs the reference performs
// (block_rebalancing_kernel, rpma.cuh:765-847); destination segment d then
// receives ranks [first_rank(d), first_rank(d + 1)) of the even spread.  In
// place: a window's slots are all read before any is written, and windows
// are disjoint.
//
// Windows of 2..4 segments (most of them) take one group of 8 lanes each, so
// a warp merges 4 windows at once: lane gl of the group loads slots
// 4gl..4gl+3 of every segment of its window together (16-byte loads), and
// the next window's record loads while this one merges.  The kept keys fill
// the group's 128-entry row of shared memory from the front and the inserts
// from the back (together they are the window's m <= 128 items).  When the
// list holds no more windows than the grid has warps, each window takes a
// warp instead (one round, a shorter chain).  Windows of 5..32 segments take
// one warp each with a 1024-entry row, 4 segments a round.

// kept_slot with the timestamp test compiled in only for calls that pass an
// expiry threshold (TH); without one every stored key with a live value is
// kept
template <bool TH>
__device__ __forceinline__ bool kept_t(uint64_t key, uint8_t val, uint32_t thres) {
    return TH ? kept_slot(key, val, thres) : (key != KEY_NONE && val != VAL_TOMB);
}

// first_rank(k, m, f) with a reciprocal inv = floor((2^64 - 1) / f): the
// high half of n * inv is floor(n / f) or one less (n = k * m + f - 1 <
// 2^58 here), so one check replaces a 64-bit division
__device__ __forceinline__ uint64_t first_rank_recip(uint64_t k, uint64_t m, uint64_t f, uint64_t inv) {
    const uint64_t n = k * m + f - 1;
    uint64_t q = __umul64hi(n, inv);
    if ((q + 1) * f <= n) q++;
    return q;
}

// first_rank for windows of <= 32 segments (k <= 32, m <= 1024): the
// product fits 32 bits, and a 32-bit division is far cheaper than the
// 64-bit one
__device__ __forceinline__ uint32_t first_rank32(uint32_t k, uint32_t m, uint32_t f) { return (k * m + f - 1) / f; }

constexpr int EM_TPB = 256;
constexpr int EM_GROUPS = EM_TPB / 8;

struct Multi4Smem {  // 2..4-segment windows, one row per group
    uint64_t k[EM_GROUPS][128];
    uint8_t v[EM_GROUPS][128];
    uint32_t im[EM_GROUPS][4];
};
struct MultiWarpSmem {  // a window per warp: 4 warps with rows of 1024, or 8 of 128
    uint64_t k[4 * 1024];
    uint8_t v[4 * 1024];
    uint32_t im[4 * 32];   // insert marks by merged rank
    uint32_t imc[4 * 32];  // marks in the words before
    uint64_t bar[4];       // the rows of 1024: one mbarrier per warp for the bulk copies
};

// Bulk copies (the TMA engine's untiled form) of global memory into shared
// memory, completing on an mbarrier of the issuing CTA.  Both addresses
// 16-byte aligned, sizes multiples of 16.
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init1(uint64_t *bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_to_smem(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t phase) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(phase)
        : "memory");
    return ok != 0;
}
// a bounded wait for the phase (each try suspends for at most a short,
// hardware-defined time): false when it did not complete
constexpr uint32_t MBAR_TRIES = 1u << 20;
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t phase, uint32_t tries = MBAR_TRIES) {
    for (uint32_t it = 0; it < tries; it++)
        if (mbar_try_wait(bar, phase)) return true;
    return false;
}

// Test setting of the 5..32-segment executor's bulk-copy wait
// (lpma_debug_exec_wait): when set, a window's first wait makes no try and
// so takes the give-up path; the wait that follows it, for the copies
// still in flight, keeps the full limit.  Read at run time, so captured
// update fronts follow it too.
__device__ uint32_t g_exec_wait_give_up = 0;
// generic-proxy accesses of shared memory before later bulk copies into it
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
constexpr size_t EM_SMEM = sizeof(Multi4Smem) > sizeof(MultiWarpSmem) ? sizeof(Multi4Smem) : sizeof(MultiWarpSmem);

template <bool TH>
__device__ __forceinline__ void k_exec_multi4_body(Multi4Smem &S, const Window *__restrict__ wins,
                                                   const uint32_t *__restrict__ n_win, uint32_t n_cap, Geo g,
                                                   uint8_t *cnt, ulonglong2 *fl, uint32_t *sent, uint32_t V,
                                                   const UpdList u, uint32_t thres, DevStatus *st, uint32_t bid_,
                                                   uint32_t nblk_) {
    const int lane = threadIdx.x & 31, gl = lane & 7, grp = threadIdx.x >> 3;
    uint64_t *K = S.k[grp];
    uint8_t *KV = S.v[grp];
    uint32_t *IM = S.im[grp];
    const uint32_t nwin = min(*n_win, n_cap);
    const uint32_t stride = nblk_ * EM_GROUPS;
    uint32_t wi = bid_ * EM_GROUPS + grp;
    Window Wn{};
    if (wi < nwin) Wn = wins[wi];
    for (; __any_sync(0xffffffffu, wi < nwin); wi += stride) {
        const bool active = wi < nwin;
        const Window W = Wn;
        if (wi + stride < nwin) Wn = wins[wi + stride];
        const uint32_t f = active ? min(W.f, 4u) : 0u;
        // segment rounds: as many as the warp's largest window needs
        const uint32_t fmax = __reduce_max_sync(0xffffffffu, f);
        // every segment's slots and the update bounds load together
        uint64_t k[4][4];
        uint32_t v4[4];
#pragma unroll
        for (int r = 0; r < 4; r++) {
            k[r][0] = k[r][1] = k[r][2] = k[r][3] = KEY_NONE;
            v4[r] = 0;
            if ((uint32_t)r < f) {
                const uint64_t j = heap_of_linear32(W.a + r, g.H);
                const ulonglong2 *kp = reinterpret_cast<const ulonglong2 *>(g.keys + 32 * j + 4 * gl);
                const ulonglong2 a = kp[0], b = kp[1];
                k[r][0] = a.x, k[r][1] = a.y, k[r][2] = b.x, k[r][3] = b.y;
                v4[r] = *reinterpret_cast<const uint32_t *>(g.vals + 32 * j + 4 * gl);
            }
        }
        const uint32_t ip0 = active ? u.ip[W.lo] : 0u;
        const uint32_t nins = active ? u.ip[W.hi] - ip0 : 0u;
        // inserts from the back of the row, rank r at 127 - r
        for (uint32_t x = W.lo + gl; active && nins && x < W.hi; x += 8) {
            const uint8_t kd = u.kind[x];
            const uint32_t r = u.ip[x] - ip0;
            const uint64_t y = u.key[x];
            const uint8_t yv = u.val[x];
            if (kd == KIND_INS && r < 128) {
                K[127 - r] = y;
                KV[127 - r] = yv;
            }
        }
        // kept keys from the front, in slot order
        uint32_t nk = 0;
#pragma unroll
        for (int r = 0; r < 4; r++) {
            if ((uint32_t)r >= fmax) break;
            uint32_t kmask = 0;
#pragma unroll
            for (int q = 0; q < 4; q++)
                if ((uint32_t)r < f && kept_t<TH>(k[r][q], (uint8_t)(v4[r] >> (8 * q)), thres)) kmask |= 1u << q;
            const uint32_t nl = __popc(kmask);
            uint32_t incl = nl;
#pragma unroll
            for (int o = 1; o < 8; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o, 8);
                if (gl >= o) incl += y;
            }
            const uint32_t base = nk + incl - nl;
#pragma unroll
            for (int q = 0; q < 4; q++)
                if ((kmask >> q) & 1u) {
                    const uint32_t c = base + __popc(kmask & ((1u << q) - 1));
                    if (c < 128) {
                        K[c] = k[r][q];
                        KV[c] = (uint8_t)(v4[r] >> (8 * q));
                    }
                }
            nk += __shfl_sync(0xffffffffu, incl, 7, 8);
        }
        if (gl < 4) IM[gl] = 0;
        __syncwarp();
        const uint32_t m = nk + nins;
        const bool ok = active && m == W.m && m <= 32u * W.f && W.f <= 4u && W.f >= 1u;
        // inserts: merged rank = insert index + kept keys below, marked
        for (uint32_t i = gl; ok && i < nins; i += 8) {
            const uint64_t y = K[127 - i];
            uint32_t L = 0, R = nk;
            while (L < R) {
                const uint32_t mid = (L + R) >> 1;
                if (K[mid] < y)
                    L = mid + 1;
                else
                    R = mid;
            }
            const uint32_t r = i + L;
            if (r < 128) atomicOr(&IM[r >> 5], 1u << (r & 31));
        }
        __syncwarp();
        if (active && !ok && gl == 0) {
            atomicOr(&st->sticky, ERR_INTERNAL);
            atomicCAS(&st->sticky_site, 0u, 1u);
        }
        const uint32_t w0 = IM[0], w1 = IM[1], w2 = IM[2], w3 = IM[3];
        const uint32_t c1 = __popc(w0), c2 = c1 + __popc(w1), c3 = c2 + __popc(w2);
        // row position of merged rank rk: an insert from the back, a kept key
        // from the front
        auto row_of = [&](uint32_t rk) -> uint32_t {
            const uint32_t wd = rk >> 5, bit = 1u << (rk & 31);
            const uint32_t w = wd == 0 ? w0 : wd == 1 ? w1 : wd == 2 ? w2 : w3;
            const uint32_t below = (wd == 0 ? 0u : wd == 1 ? c1 : wd == 2 ? c2 : c3) + __popc(w & (bit - 1));
            return ((w & bit) ? 127 - below : rk - below) & 127;
        };
        uint32_t f1 = 0;  // first rank of the segment after
#pragma unroll
        for (int r = 0; r < 4; r++) {
            if ((uint32_t)r >= fmax) break;
            if (!ok || (uint32_t)r >= f) continue;
            const uint32_t f0 = f1;
            f1 = first_rank32(r + 1, m, f);
            const uint32_t cnk = f1 - f0;
            const uint64_t j = heap_of_linear32(W.a + r, g.H);
            uint64_t o[4];
            uint32_t ovw = 0;
            // the marks of this lane's 4 ranks rb..rb+3, and the marks below rb
            const uint32_t rb = f0 + 4 * gl, wd = (rb >> 5) & 3, sh = rb & 31;
            const uint32_t wa = wd == 0 ? w0 : wd == 1 ? w1 : wd == 2 ? w2 : w3;
            const uint32_t wb = wd == 0 ? w1 : wd == 1 ? w2 : wd == 2 ? w3 : 0u;
            const uint32_t bits = (wa >> sh) | (sh ? wb << (32 - sh) : 0u);
            const uint32_t below0 = (wd == 0 ? 0u : wd == 1 ? c1 : wd == 2 ? c2 : c3) + __popc(wa & ((1u << sh) - 1));
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const uint32_t slot = 4 * gl + q;
                o[q] = KEY_NONE;
                if (slot < cnk) {
                    const uint32_t below = below0 + __popc(bits & ((1u << q) - 1));
                    const uint32_t at = (((bits >> q) & 1u) ? 127 - below : rb + q - below) & 127;
                    o[q] = K[at];
                    ovw |= (uint32_t)KV[at] << (8 * q);
                    if (is_sentinel(o[q])) {
                        const uint32_t row = (uint32_t)(o[q] >> SRC_SHIFT);
                        if (row < V) sent[row] = (uint32_t)(32 * j + slot);
                    }
                }
            }
            ulonglong2 *kp = reinterpret_cast<ulonglong2 *>(g.keys + 32 * j + 4 * gl);
            kp[0] = make_ulonglong2(o[0], o[1]);
            kp[1] = make_ulonglong2(o[2], o[3]);
            *reinterpret_cast<uint32_t *>(g.vals + 32 * j + 4 * gl) = ovw;
            if (gl == 0) {
                cnt[W.a + r] = (uint8_t)cnk;
                fl[j] = cnk ? make_ulonglong2(o[0], K[row_of(f1 - 1)]) : make_ulonglong2(KEY_NONE, KEY_NONE);
            }
        }
        __syncwarp();
    }
}

// A window of up to ROW / 32 segments on one warp: its 4 groups take 4
// segments a round (group q: segment 4r + q), so a window of <= 4 segments
// is one round.  The row holds the kept keys from the front and the inserts
// from the back.  Rows of 128 (windows of up to 4 segments): each lane
// loads its slots, the next round's while a round compacts.  Rows of 1024
// (5..32 segments): lane s first bulk-copies segment s's keys (256 B) and
// values (32 B) into the row at 32 s, so all of the window's loads are in
// flight at once (one mbarrier wait, bounded), and the kept keys are then
// compacted in place (a kept key only moves down, past slots already read);
// its inserts are written to the back of the row after the compaction.
template <uint32_t ROW, bool TH>
__device__ __forceinline__ void k_exec_multi_warp_body(uint64_t *K, uint8_t *KV, uint32_t *IM, uint32_t *IMC,
                                                       uint64_t *bar, const Window *__restrict__ wins,
                                                       const uint32_t *__restrict__ n_win, uint32_t n_cap, Geo g,
                                                       uint8_t *cnt, ulonglong2 *fl, uint32_t *sent, uint32_t V,
                                                       const UpdList u, uint32_t thres, DevStatus *st, uint32_t wid,
                                                       uint32_t nwarps) {
    constexpr uint32_t WORDS = ROW / 32, MAXF = ROW / 32;
    constexpr bool STAGED = ROW == 1024;
    const int lane = threadIdx.x & 31, gl = lane & 7, gq = lane >> 3;
    const uint32_t nwin = min(*n_win, n_cap);
    uint32_t phase = 0, tries = MBAR_TRIES;
    if (STAGED) {
        if (lane == 0) mbar_init1(bar);
        if (*reinterpret_cast<volatile uint32_t *>(&g_exec_wait_give_up)) tries = 0;
        __syncwarp();
    }
    for (uint32_t wi = wid; wi < nwin; wi += nwarps) {  // uniform over the warp
        const Window W = wins[wi];
        const uint32_t f = min(W.f, MAXF);
        const uint32_t rounds = (f + 3) / 4;
        if (STAGED) {
            // the row's earlier reads and writes come before the copies into it
            fence_proxy_async_smem();
            __syncwarp();
            if (lane == 0) mbar_expect_tx(bar, f * 288u);
            __syncwarp();
            if ((uint32_t)lane < f) {
                const uint64_t j = heap_of_linear32(W.a + lane, g.H);
                bulk_to_smem(K + 32 * lane, g.keys + 32 * j, 256u, bar);
                bulk_to_smem(KV + 32 * lane, g.vals + 32 * j, 32u, bar);
            }
        }
        auto load = [&](uint32_t r, uint64_t (&k)[4], uint32_t &v4) {
            const uint32_t sg = 4 * r + gq;
            k[0] = k[1] = k[2] = k[3] = KEY_NONE;
            v4 = 0;
            if (sg < f) {
                const uint64_t j = heap_of_linear32(W.a + sg, g.H);
                const ulonglong2 *kp = reinterpret_cast<const ulonglong2 *>(g.keys + 32 * j + 4 * gl);
                const ulonglong2 a = kp[0], b = kp[1];
                k[0] = a.x, k[1] = a.y, k[2] = b.x, k[3] = b.y;
                v4 = *reinterpret_cast<const uint32_t *>(g.vals + 32 * j + 4 * gl);
            }
        };
        uint64_t kn[4] = {KEY_NONE, KEY_NONE, KEY_NONE, KEY_NONE};
        uint32_t vn = 0;
        if (!STAGED) load(0, kn, vn);
        const uint32_t ip0 = u.ip[W.lo];
        const uint32_t nins = u.ip[W.hi] - ip0;
        // inserts go to the back of the row, rank r at ROW - 1 - r; a staged
        // row holds the slots until the compaction, so the window's first 32
        // updates wait in registers meanwhile
        uint64_t y0 = 0;
        uint32_t r0 = ~0u, yv0 = 0;
        for (uint32_t x = W.lo + lane; nins && x < (STAGED ? min(W.hi, W.lo + 32) : W.hi); x += 32) {
            const uint8_t kd = u.kind[x];
            const uint32_t r = u.ip[x] - ip0;
            const uint64_t y = u.key[x];
            const uint8_t yv = u.val[x];
            if (STAGED) {
                if (kd == KIND_INS) r0 = r, y0 = y, yv0 = yv;
            } else if (kd == KIND_INS && r < ROW) {
                K[ROW - 1 - r] = y;
                KV[ROW - 1 - r] = yv;
            }
        }
        if (STAGED) {
            const uint32_t ph = phase;
            phase ^= 1u;
            if (!__all_sync(0xffffffffu, mbar_wait_bounded(bar, ph, tries))) {
                // the copies did not land in time: report, let them finish
                // (bounded) before the row is left, and stop this warp
                if (lane == 0) {
                    atomicOr(&st->sticky, ERR_TIMEOUT);
                    atomicCAS(&st->sticky_site, 0u, 9u);
                }
                mbar_wait_bounded(bar, ph);
                return;
            }
        }
        // kept keys from the front, in slot order (lane order within a round)
        uint32_t nk = 0;
        for (uint32_t r = 0; r < rounds; r++) {
            uint64_t k[4] = {kn[0], kn[1], kn[2], kn[3]};
            uint32_t v4 = vn;
            if (STAGED) {
                const uint32_t sg = 4 * r + gq;
                if (sg < f) {
                    const ulonglong2 *kp = reinterpret_cast<const ulonglong2 *>(K + 32 * sg + 4 * gl);
                    const ulonglong2 a = kp[0], b = kp[1];
                    k[0] = a.x, k[1] = a.y, k[2] = b.x, k[3] = b.y;
                    v4 = *reinterpret_cast<const uint32_t *>(KV + 32 * sg + 4 * gl);
                } else {
                    k[0] = k[1] = k[2] = k[3] = KEY_NONE;
                    v4 = 0;
                }
                __syncwarp();  // the round's slots are read before kept keys move down over them
            } else if (r + 1 < rounds) {
                load(r + 1, kn, vn);
            }
            uint32_t kmask = 0;
#pragma unroll
            for (int q = 0; q < 4; q++)
                if (kept_t<TH>(k[q], (uint8_t)(v4 >> (8 * q)), thres)) kmask |= 1u << q;
            const uint32_t nl = __popc(kmask);
            uint32_t incl = nl;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += y;
            }
            const uint32_t base = nk + incl - nl;
#pragma unroll
            for (int q = 0; q < 4; q++)
                if ((kmask >> q) & 1u) {
                    const uint32_t c = base + __popc(kmask & ((1u << q) - 1));
                    if (c < ROW) {
                        K[c] = k[q];
                        KV[c] = (uint8_t)(v4 >> (8 * q));
                    }
                }
            nk += __shfl_sync(0xffffffffu, incl, 31);
        }
        if (STAGED) {
            __syncwarp();  // the kept keys are in place: the back of the row is free
            if (r0 < ROW) {
                K[ROW - 1 - r0] = y0;
                KV[ROW - 1 - r0] = (uint8_t)yv0;
            }
            for (uint32_t x = W.lo + 32 + lane; nins && x < W.hi; x += 32) {
                const uint32_t r = u.ip[x] - ip0;
                if (u.kind[x] == KIND_INS && r < ROW) {
                    K[ROW - 1 - r] = u.key[x];
                    KV[ROW - 1 - r] = u.val[x];
                }
            }
        }
        if ((uint32_t)lane < WORDS) IM[lane] = 0;
        __syncwarp();
        const uint32_t m = nk + nins;
        const bool ok = m == W.m && m <= 32u * W.f && W.f <= MAXF;
        // inserts: merged rank = insert index + kept keys below, marked
        for (uint32_t i = lane; ok && i < nins; i += 32) {
            const uint64_t y = K[ROW - 1 - i];
            uint32_t L = 0, R = nk;
            while (L < R) {
                const uint32_t mid = (L + R) >> 1;
                if (K[mid] < y)
                    L = mid + 1;
                else
                    R = mid;
            }
            const uint32_t r = i + L;
            if (r < ROW) atomicOr(&IM[r >> 5], 1u << (r & 31));
        }
        __syncwarp();
        {
            const uint32_t c = (uint32_t)lane < WORDS ? __popc(IM[lane]) : 0u;
            uint32_t x = c;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            if ((uint32_t)lane < WORDS) IMC[lane] = x - c;
        }
        __syncwarp();
        if (!ok) {
            if (lane == 0) {
                atomicOr(&st->sticky, ERR_INTERNAL);
                atomicCAS(&st->sticky_site, 0u, 1u);
            }
        } else {
            auto row_of = [&](uint32_t rk) -> uint32_t {
                const uint32_t w = IM[rk >> 5], bit = 1u << (rk & 31);
                const uint32_t below = IMC[rk >> 5] + __popc(w & (bit - 1));
                return ((w & bit) ? ROW - 1 - below : rk - below) & (ROW - 1);
            };
            for (uint32_t r = 0; r < rounds; r++) {
                const uint32_t sg = 4 * r + gq;
                if (sg >= f) continue;
                const uint32_t f0 = first_rank32(sg, m, f), f1 = first_rank32(sg + 1, m, f);
                const uint32_t cnk = f1 - f0;
                const uint64_t j = heap_of_linear32(W.a + sg, g.H);
                uint64_t o[4];
                uint32_t ovw = 0;
                const uint32_t rb = f0 + 4 * gl, wd = (rb >> 5) & (WORDS - 1), sh = rb & 31;
                const uint32_t wa = IM[wd], wb = wd + 1 < WORDS ? IM[wd + 1] : 0u;
                const uint32_t bits = (wa >> sh) | (sh ? wb << (32 - sh) : 0u);
                const uint32_t below0 = IMC[wd] + __popc(wa & ((1u << sh) - 1));
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const uint32_t slot = 4 * gl + q;
                    o[q] = KEY_NONE;
                    if (slot < cnk) {
                        const uint32_t below = below0 + __popc(bits & ((1u << q) - 1));
                        const uint32_t at = (((bits >> q) & 1u) ? ROW - 1 - below : rb + q - below) & (ROW - 1);
                        o[q] = K[at];
                        ovw |= (uint32_t)KV[at] << (8 * q);
                        if (is_sentinel(o[q])) {
                            const uint32_t row = (uint32_t)(o[q] >> SRC_SHIFT);
                            if (row < V) sent[row] = (uint32_t)(32 * j + slot);
                        }
                    }
                }
                ulonglong2 *kp = reinterpret_cast<ulonglong2 *>(g.keys + 32 * j + 4 * gl);
                kp[0] = make_ulonglong2(o[0], o[1]);
                kp[1] = make_ulonglong2(o[2], o[3]);
                *reinterpret_cast<uint32_t *>(g.vals + 32 * j + 4 * gl) = ovw;
                if (gl == 0) {
                    cnt[W.a + sg] = (uint8_t)cnk;
                    fl[j] = cnk ? make_ulonglong2(o[0], K[row_of(f1 - 1)]) : make_ulonglong2(KEY_NONE, KEY_NONE);
                }
            }
        }
        __syncwarp();
    }
}

// The 2..4-segment list: one window per 8-lane group (4 per warp) when the
// list holds more windows than the grid has warps, else one per warp (a
// single round, the shorter chain when few windows run).
template <bool TH>
__device__ __forceinline__ void exec_multi4(unsigned char *smem, const Window *__restrict__ w4,
                                            const uint32_t *__restrict__ n4, uint32_t cap4, Geo g, uint8_t *cnt,
                                            ulonglong2 *fl, uint32_t *sent, uint32_t V, const UpdList u,
                                            uint32_t thres, DevStatus *st, uint32_t bid_, uint32_t nblk_) {
    const uint32_t warps = nblk_ * (EM_TPB / 32);
    if (min(*n4, cap4) > warps) {
        k_exec_multi4_body<TH>(*reinterpret_cast<Multi4Smem *>(smem), w4, n4, cap4, g, cnt, fl, sent, V, u, thres, st,
                           bid_, nblk_);
    } else {
        MultiWarpSmem &S = *reinterpret_cast<MultiWarpSmem *>(smem);
        const uint32_t w = threadIdx.x >> 5;
        k_exec_multi_warp_body<128, TH>(S.k + 128 * w, S.v + 128 * w, S.im + 4 * w, S.imc + 4 * w, nullptr, w4, n4, cap4,
                                        g, cnt, fl, sent, V, u, thres, st, bid_ * (EM_TPB / 32) + w, warps);
    }
}

// The 5..32-segment list: one window per warp, 4 warps a block (rows of
// 1024 entries).
template <bool TH>
__device__ __forceinline__ void exec_multi32(unsigned char *smem, const Window *__restrict__ w32,
                                             const uint32_t *__restrict__ n32, uint32_t cap32, Geo g, uint8_t *cnt,
                                             ulonglong2 *fl, uint32_t *sent, uint32_t V, const UpdList u,
                                             uint32_t thres, DevStatus *st, uint32_t bid_, uint32_t nblk_) {
    const uint32_t w = threadIdx.x >> 5;
    if (w >= 4) return;
    MultiWarpSmem &S = *reinterpret_cast<MultiWarpSmem *>(smem);
    k_exec_multi_warp_body<1024, TH>(S.k + 1024 * w, S.v + 1024 * w, S.im + 32 * w, S.imc + 32 * w, S.bar + w, w32, n32,
                                     cap32, g, cnt, fl, sent, V, u, thres, st, bid_ * 4 + w, nblk_ * 4);
}

// a plan that overflowed or a rejected batch: the guarded executors skip
__device__ __forceinline__ bool plan_void(const DevStatus *st) { return (st->ovf | st->error) != 0; }

// Both multi-segment classes in one launch: the first gridDim.x - nb4
// blocks run the 5..32-segment windows one CTA each, the last nb4 blocks
// the 2..4-segment windows one 8-lane group each.
template <bool TH>
__global__ void __launch_bounds__(EM_TPB, 4) k_exec_multi(const Window *__restrict__ w4, const uint32_t *__restrict__ n4,
                                                       uint32_t cap4, uint32_t nb4, const Window *__restrict__ w32,
                                                       const uint32_t *__restrict__ n32, uint32_t cap32, Geo g,
                                                       uint8_t *cnt, ulonglong2 *fl, uint32_t *sent, uint32_t V,
                                                       const UpdList u, uint32_t thres, DevStatus *st, int guarded) {
    __shared__ __align__(16) unsigned char smem[EM_SMEM];
    griddep_wait();
    if (guarded && plan_void(st)) return;
    const uint32_t nb32 = gridDim.x - nb4;
    if (blockIdx.x < nb32)
        exec_multi32<TH>(smem, w32, n32, cap32, g, cnt, fl, sent, V, u, thres, st, blockIdx.x, nb32);
    else
        exec_multi4<TH>(smem, w4, n4, cap4, g, cnt, fl, sent, V, u, thres, st, blockIdx.x - nb32, nb4);
}

// ------------------------------------------------------------------ single-segment windows
// The level-0 windows (one segment, about 94% of the executed windows) get a
// group of 8 lanes each, so a warp keeps 4 windows in flight.  Lane gl of a
// group moves slots 4gl..4gl+3 with two 16-byte key loads/stores and one
// 4-byte value load/store.  The window's kept keys are compacted into shared
// memory; an insert's merged slot is (inserts before it) + (kept keys below
// it, a binary search), and the inserts mark their slots in a 32-bit mask.
// Every output slot then reads its key without a search: a marked slot takes
// the insert whose index is the count of marks below it, any other slot the
// kept key whose index is the count of unmarked slots below it.  576 bytes of
// shared memory per group.
constexpr int ES_TPB = 256;
constexpr int ES_GROUPS = ES_TPB / 8;

template <bool TH>
__device__ __forceinline__ void k_exec_single_body(const Window *__restrict__ wins,
                                                        const uint32_t *__restrict__ n_win, uint32_t n_cap, Geo g,
                                                        uint8_t *cnt, ulonglong2 *fl, uint32_t *sent, uint32_t V,
                                                        const UpdList u, uint32_t thres, DevStatus *st, uint32_t bid_, uint32_t nblk_) {
    __shared__ uint64_t kk[ES_GROUPS][32];  // kept keys of the window, compacted
    __shared__ uint64_t ik[ES_GROUPS][32];  // insert keys of the window, in key order
    __shared__ uint8_t kv[ES_GROUPS][32];   // their values
    __shared__ uint8_t iv[ES_GROUPS][32];
    const int lane = threadIdx.x & 31, gl = lane & 7, grp = threadIdx.x >> 3;
    const uint32_t nwin = min(*n_win, n_cap);
    const uint32_t stride = nblk_ * ES_GROUPS;
    // software pipeline: the segment slots and update bounds of the next
    // window are loaded while the current one is merged, and the window
    // record two ahead (its segment address is known when its slots load)
    uint32_t wi = bid_ * ES_GROUPS + grp;
    Window Wn{}, Wnn{};
    uint64_t jn = 0;
    ulonglong2 na = make_ulonglong2(KEY_NONE, KEY_NONE), nb = na;
    uint32_t nv4 = 0, nip0 = 0, nip1 = 0;
    if (wi < nwin) {
        Wn = wins[wi];
        jn = heap_of_linear32(Wn.a, g.H);
        const ulonglong2 *kp = reinterpret_cast<const ulonglong2 *>(g.keys + 32 * jn + 4 * gl);
        na = kp[0], nb = kp[1];
        nv4 = *reinterpret_cast<const uint32_t *>(g.vals + 32 * jn + 4 * gl);
        nip0 = u.ip[Wn.lo], nip1 = u.ip[Wn.hi];
    }
    if (wi + stride < nwin) Wnn = wins[wi + stride];
    for (; __any_sync(0xffffffffu, wi < nwin); wi += stride) {
        const bool active = wi < nwin;
        const Window W = Wn;
        const uint64_t j = jn;
        const ulonglong2 a = na, b = nb;
        const uint32_t v4 = nv4, ip0c = nip0, ip1c = nip1;
        if (wi + stride < nwin) {
            Wn = Wnn;
            jn = heap_of_linear32(Wn.a, g.H);
            const ulonglong2 *kp = reinterpret_cast<const ulonglong2 *>(g.keys + 32 * jn + 4 * gl);
            na = kp[0], nb = kp[1];
            nv4 = *reinterpret_cast<const uint32_t *>(g.vals + 32 * jn + 4 * gl);
            nip0 = u.ip[Wn.lo], nip1 = u.ip[Wn.hi];
            if (wi + 2 * stride < nwin) Wnn = wins[wi + 2 * stride];
        }
        uint64_t k[4];
        uint32_t kmask = 0;
        k[0] = a.x, k[1] = a.y, k[2] = b.x, k[3] = b.y;
#pragma unroll
        for (int q = 0; q < 4; q++)
            if (active && kept_t<TH>(k[q], (uint8_t)(v4 >> (8 * q)), thres)) kmask |= 1u << q;
        // exclusive prefix of kept counts across the group
        const uint32_t nl = __popc(kmask);
        uint32_t incl = nl;
#pragma unroll
        for (int o = 1; o < 8; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o, 8);
            if (gl >= o) incl += y;
        }
        const uint32_t kbase = incl - nl;
        const uint32_t nk = __shfl_sync(0xffffffffu, incl, 7, 8);
        // kept keys and values, compacted in order
#pragma unroll
        for (int q = 0; q < 4; q++)
            if ((kmask >> q) & 1u) {
                const uint32_t x = kbase + __popc(kmask & ((1u << q) - 1));
                kk[grp][x] = k[q];
                kv[grp][x] = (uint8_t)(v4 >> (8 * q));
            }
        __syncwarp();
        // updates of the window, 8 per round (usually one round)
        const uint32_t lo = W.lo, hi = active ? W.hi : W.lo;
        const uint32_t ip0 = active ? ip0c : 0;
        const uint32_t nins = active ? ip1c - ip0 : 0;
        // deletes were applied as tombstones by the locate: a window without
        // inserts needs no pass over its updates
        const uint32_t rounds = __reduce_max_sync(0xffffffffu, nins ? (hi - lo + 7) / 8 : 0u);
        uint32_t imask = 0;
        for (uint32_t r = 0; r < rounds; r++) {
            const uint32_t x = lo + 8 * r + gl;
            // the update's fields load together (not behind the kind test)
            uint8_t kd = KIND_NOP, yv = 0;
            uint64_t yk = 0;
            uint32_t yip = 0;
            if (x < hi) kd = u.kind[x], yk = u.key[x], yip = u.ip[x], yv = u.val[x];
            if (kd == KIND_INS) {
                const uint32_t ri = yip - ip0;
                uint32_t L = 0, R = nk;
                while (L < R) {
                    const uint32_t mid = (L + R) >> 1;
                    if (kk[grp][mid] < yk)
                        L = mid + 1;
                    else
                        R = mid;
                }
                if (ri < 32) {
                    ik[grp][ri] = yk;
                    iv[grp][ri] = yv;
                }
                if (ri + L < 32) imask |= 1u << (ri + L);
            }
        }
        if (rounds) {  // warp-uniform: the group's marks in every lane
            imask |= __shfl_xor_sync(0xffffffffu, imask, 1, 8);
            imask |= __shfl_xor_sync(0xffffffffu, imask, 2, 8);
            imask |= __shfl_xor_sync(0xffffffffu, imask, 4, 8);
        }
        __syncwarp();
        const uint32_t m = nk + nins;
        const bool ok = active && m == W.m && m <= 32;
        if (active && !ok && gl == 0) {
            atomicOr(&st->sticky, ERR_INTERNAL);
            atomicCAS(&st->sticky_site, 0u, 3u);
        }
        if (ok) {
            uint64_t o[4];
            uint32_t ov = 0;
            // marks of this lane's slots 4gl..4gl+3 and the marks below them
            const uint32_t bits = imask >> (4 * gl), below0 = __popc(imask & ((1u << (4 * gl)) - 1));
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const uint32_t slot = 4 * gl + q;
                o[q] = KEY_NONE;
                if (slot < m) {
                    const uint32_t below = below0 + __popc(bits & ((1u << q) - 1));
                    if ((bits >> q) & 1u) {
                        o[q] = ik[grp][below];
                        ov |= (uint32_t)iv[grp][below] << (8 * q);
                    } else {
                        o[q] = kk[grp][slot - below];
                        ov |= (uint32_t)kv[grp][slot - below] << (8 * q);
                    }
                    if (is_sentinel(o[q])) {
                        const uint32_t row = (uint32_t)(o[q] >> SRC_SHIFT);
                        if (row < V) sent[row] = (uint32_t)(32 * j + slot);
                    }
                }
            }
            ulonglong2 *kp = reinterpret_cast<ulonglong2 *>(g.keys + 32 * j + 4 * gl);
            kp[0] = make_ulonglong2(o[0], o[1]);
            kp[1] = make_ulonglong2(o[2], o[3]);
            *reinterpret_cast<uint32_t *>(g.vals + 32 * j + 4 * gl) = ov;
            if (gl == 0) {
                cnt[W.a] = (uint8_t)m;
                // the last slot holds the last insert or the last kept key
                const uint64_t last = m ? (((imask >> (m - 1)) & 1u) ? ik[grp][nins - 1] : kk[grp][nk - 1]) : KEY_NONE;
                fl[j] = make_ulonglong2(o[0], last);
            }
        }
        __syncwarp();
    }
}

template <bool TH>
__global__ void __launch_bounds__(ES_TPB, 4) k_exec_single(const Window *__restrict__ wins,
                                                        const uint32_t *__restrict__ n_win, uint32_t n_cap, Geo g,
                                                        uint8_t *cnt, ulonglong2 *fl, uint32_t *sent, uint32_t V,
                                                        const UpdList u, uint32_t thres, DevStatus *st,
                                                        int guarded) {
    griddep_wait();
    if (guarded && plan_void(st)) return;
    k_exec_single_body<TH>(wins, n_win, n_cap, g, cnt, fl, sent, V, u, thres, st, blockIdx.x, gridDim.x);
}

// ------------------------------------------------------------------ tile grain
__global__ void __launch_bounds__(TPB) k_seg_update_counts(const UpdList u, uint32_t n_cap, uint32_t *qi, uint32_t *qd,
                                                           const DevStatus *st) {
    const uint32_t nu = st->n_u;
    const uint32_t x = blockIdx.x * TPB + threadIdx.x;
    if (x >= nu || x >= n_cap) return;
    const uint32_t s = u.seg[x];
    if (x > 0 && u.seg[x - 1] == s) return;
    const uint32_t hi0 = lb_fwd(u.seg, x, nu, (uint64_t)s + 1);
    const uint32_t ins = u.ip[hi0] - u.ip[x];
    qi[s] = ins;
    qd[s] = (hi0 - x) - ins;
}

// The big windows' prefixes: for every segment s, q = live(s) - deletes(s)
// + inserts(s) (its items after the update) and qn = inserts(s) +
// deletes(s) (its updates), and their exclusive prefixes PQ (the window
// rank base of its items) and US (its first update), PQ[nseg] and
// US[nseg] the totals.  The pairs are computed where they are read and
// scanned packed in one u64 (each sum stays below 2^32): a reduce, a top
// and a down pass.
constexpr uint32_t TS_IPT = 8, TS_TILE = TPB * TS_IPT;

__device__ __forceinline__ uint64_t seg_pair(const uint8_t *__restrict__ cnt, const uint8_t *__restrict__ cnt_live,
                                             const uint32_t *__restrict__ qi, const uint32_t *__restrict__ qd,
                                             uint64_t s) {
    const uint32_t c = cnt_live ? cnt_live[s] : cnt[s];
    const uint32_t i = qi[s], d = qd[s];
    return (uint64_t)(c - d + i) | ((uint64_t)(i + d) << 32);
}

__global__ void __launch_bounds__(TPB) k_ts_reduce(const uint8_t *__restrict__ cnt, const uint8_t *__restrict__ cnt_live,
                                                   const uint32_t *__restrict__ qi, const uint32_t *__restrict__ qd,
                                                   uint64_t nseg, uint64_t *tmp) {
    __shared__ uint64_t wsum[TPB / 32];
    const uint64_t base = (uint64_t)blockIdx.x * TS_TILE;
    uint64_t v = 0;
#pragma unroll
    for (uint32_t i = 0; i < TS_IPT; i++) {
        const uint64_t p = base + (uint64_t)i * TPB + threadIdx.x;
        if (p < nseg) v += seg_pair(cnt, cnt_live, qi, qd, p);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint64_t t = 0;
        for (int w = 0; w < TPB / 32; w++) t += wsum[w];
        tmp[blockIdx.x] = t;
    }
}

// one CTA: the block totals to exclusive offsets, and the two totals
__global__ void __launch_bounds__(1024) k_ts_top(uint64_t *tmp, uint32_t nb, uint32_t *pq_total, uint32_t *us_total) {
    __shared__ uint64_t ws[32];
    __shared__ uint64_t carry;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint32_t b0 = 0; b0 < nb; b0 += 1024) {
        const uint32_t i = b0 + threadIdx.x;
        const uint64_t x = i < nb ? tmp[i] : 0;
        uint64_t v = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint64_t y = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += y;
        }
        if (lane == 31) ws[w] = v;
        __syncthreads();
        if (w == 0) {
            uint64_t t = ws[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint64_t y = __shfl_up_sync(0xffffffffu, t, o);
                if (lane >= o) t += y;
            }
            ws[lane] = t;
        }
        __syncthreads();
        if (i < nb) tmp[i] = carry + (w ? ws[w - 1] : 0) + v - x;
        __syncthreads();
        if (threadIdx.x == 0) carry += ws[31];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        *pq_total = (uint32_t)carry;
        *us_total = (uint32_t)(carry >> 32);
    }
}

__global__ void __launch_bounds__(TPB) k_ts_down(const uint8_t *__restrict__ cnt, const uint8_t *__restrict__ cnt_live,
                                                 const uint32_t *__restrict__ qi, const uint32_t *__restrict__ qd,
                                                 uint64_t nseg, const uint64_t *__restrict__ tmp, uint32_t *PQ,
                                                 uint32_t *US) {
    __shared__ uint64_t wsum[TPB / 32];
    const uint64_t base = (uint64_t)blockIdx.x * TS_TILE + (uint64_t)threadIdx.x * TS_IPT;
    uint64_t x[TS_IPT];
    uint64_t v = 0;
#pragma unroll
    for (uint32_t i = 0; i < TS_IPT; i++) {
        const uint64_t p = base + i;
        x[i] = p < nseg ? seg_pair(cnt, cnt_live, qi, qd, p) : 0;
        v += x[i];
    }
    uint64_t off = block_excl_scan_u64(v, wsum) + tmp[blockIdx.x];
#pragma unroll
    for (uint32_t i = 0; i < TS_IPT; i++) {
        const uint64_t p = base + i;
        if (p < nseg) {
            PQ[p] = (uint32_t)off;
            US[p] = (uint32_t)(off >> 32);
        }
        off += x[i];
    }
}

// Windows larger than 32 segments (root, level >= 6, rebuild) run in two
// fully parallel phases.  Gather: one 8-lane group per source segment merges
// its kept slots with the inserts located into it and writes them, in
// window rank order, to a contiguous sequence M (the alternate buffer) at
// PQ[s] + rank.  Spread: one 8-lane group per destination segment takes its
// items [first_rank(k), first_rank(k+1)) from M.  Every source slot is read
// before any destination slot is written (two launches), so the windows are
// rewritten in place.
__device__ inline uint32_t find_job(const TileJob *jobs, uint32_t njobs, uint32_t tile, bool dst) {
    uint32_t L = 0, R = njobs - 1;  // last job whose first tile <= tile
    while (L < R) {
        const uint32_t mid = (L + R + 1) >> 1;
        if ((dst ? jobs[mid].dtile0 : jobs[mid].stile0) <= tile)
            L = mid;
        else
            R = mid - 1;
    }
    return L;
}

constexpr int GT_TPB = 256;  // 32 groups of 8 lanes: one 32-segment tile per CTA
constexpr uint32_t GT_LOCAL = 8;  // updates of a segment the group merges in registers

template <bool TH>
__global__ void __launch_bounds__(GT_TPB) k_gather(const TileJob *__restrict__ jobs, uint32_t njobs, uint32_t ntiles,
                                                   Geo src, const uint32_t *__restrict__ PQ,
                                                   const uint32_t *__restrict__ US, const UpdList u, uint32_t thres,
                                                   uint64_t *__restrict__ Mk, uint8_t *__restrict__ Mv, uint64_t m_cap,
                                                   DevStatus *st) {
    const int lane = threadIdx.x & 31, gl = lane & 7, grp = threadIdx.x >> 3;
    for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const TileJob J = jobs[find_job(jobs, njobs, tile, false)];
        const uint32_t s = J.sa + 32 * (tile - J.stile0) + grp;
        const bool active = s < J.sa + J.sf;
        uint64_t k[4] = {KEY_NONE, KEY_NONE, KEY_NONE, KEY_NONE};
        uint8_t v[4] = {0, 0, 0, 0};
        uint32_t kmask = 0, us = 0, ue = 0;
        uint64_t base = 0;
        if (active) {
            const uint64_t j = heap_of_linear(s, src.H);
            const ulonglong2 *kp = reinterpret_cast<const ulonglong2 *>(src.keys + 32 * j + 4 * gl);
            const ulonglong2 a = kp[0], b = kp[1];
            const uint32_t v4 = *reinterpret_cast<const uint32_t *>(src.vals + 32 * j + 4 * gl);
            k[0] = a.x, k[1] = a.y, k[2] = b.x, k[3] = b.y;
#pragma unroll
            for (int q = 0; q < 4; q++) {
                v[q] = (uint8_t)(v4 >> (8 * q));
                if (kept_t<TH>(k[q], v[q], thres)) kmask |= 1u << q;
            }
            us = US[s];
            ue = US[s + 1];
            base = PQ[s];
        }
        const uint32_t nl = __popc(kmask);
        uint32_t incl = nl;
#pragma unroll
        for (int o = 1; o < 8; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o, 8);
            if (gl >= o) incl += y;
        }
        const uint32_t kbase = incl - nl;
        const uint32_t nupd = ue - us;
        // a segment with few updates (nearly all of them in a root window)
        // merges them in registers: lane gl holds update us + gl
        const bool local = active && nupd <= GT_LOCAL;
        uint64_t y = KEY_NONE;
        uint32_t yip = 0;
        uint8_t yv = 0;
        bool yins = false;
        if (local && (uint32_t)gl < nupd) {
            const uint32_t x = us + gl;
            yins = u.kind[x] == KIND_INS;
            y = u.key[x];
            yip = u.ip[x];
            yv = u.val[x];
        }
        // ip of the segment's first update (every lane takes part in the shuffle)
        const uint32_t ip0 = __shfl_sync(0xffffffffu, yip, lane & ~7);
        uint32_t below[4] = {0, 0, 0, 0};
        uint32_t my_kept_below = 0;  // for this lane's insert: kept slots of the segment below it
        // as many rounds as the warp's busiest local segment has updates
        const uint32_t tmax = __reduce_max_sync(0xffffffffu, local ? nupd : 0u);
        if (tmax) {
            for (uint32_t t = 0; t < tmax; t++) {
                const uint64_t yt = __shfl_sync(0xffffffffu, y, (lane & ~7) + t);
                const bool it = __shfl_sync(0xffffffffu, (int)yins, (lane & ~7) + t) != 0;
                // the kept keys above insert t count it below them
#pragma unroll
                for (int q = 0; q < 4; q++) below[q] += (it && yt < k[q]) ? 1u : 0u;
                // kept slots below insert t, summed over the group
                uint32_t c = 0;
#pragma unroll
                for (int q = 0; q < 4; q++) c += (((kmask >> q) & 1u) && k[q] < yt) ? 1u : 0u;
                c += __shfl_xor_sync(0xffffffffu, c, 1, 8);
                c += __shfl_xor_sync(0xffffffffu, c, 2, 8);
                c += __shfl_xor_sync(0xffffffffu, c, 4, 8);
                if ((uint32_t)gl == t) my_kept_below = c;
            }
        }
        // kept slots: rank = kept before + inserts of this segment below the key
#pragma unroll
        for (int q = 0; q < 4; q++) {
            if ((kmask >> q) & 1u) {
                uint32_t bl;
                if (local)
                    bl = below[q];
                else
                    bl = ue > us ? u.ip[lb_key(u.key, us, ue, k[q])] - u.ip[us] : 0u;
                const uint64_t r = base + kbase + __popc(kmask & ((1u << q) - 1)) + bl;
                if (r < m_cap) {
                    Mk[r] = k[q];
                    Mv[r] = v[q];
                } else {  // only if the update list broke its sortedness invariant
                    atomicOr(&st->sticky, ERR_INTERNAL);
                    atomicCAS(&st->sticky_site, 0u, 4u);
                }
            }
        }
        // this lane's insert of a local segment: inserts before it + kept below
        if (local && yins) {
            const uint64_t r = base + (yip - ip0) + my_kept_below;
            if (r < m_cap) {
                Mk[r] = y;
                Mv[r] = yv;
            } else {
                atomicOr(&st->sticky, ERR_INTERNAL);
                atomicCAS(&st->sticky_site, 0u, 4u);
            }
        }
        __syncwarp();
    }
}

// The inserts of big windows in segments with more than GT_LOCAL updates,
// one thread each (a segment may carry millions of them when a bulk load
// lands in a near-empty tree): rank = segment base
// + inserts of the segment before it + kept slots of the segment below it.
// Slots below it that are not kept are the tombstones of the segment's
// deletes before it in the sorted update list, plus expired keys.
__global__ void __launch_bounds__(TPB) k_gather_ins(const TileJob *__restrict__ jobs, uint32_t njobs, Geo src,
                                                    const uint32_t *__restrict__ PQ,
                                                    const uint32_t *__restrict__ US, const UpdList u,
                                                    DevStatus *st, uint32_t n_cap, uint32_t thres,
                                                    uint64_t *__restrict__ Mk, uint8_t *__restrict__ Mv,
                                                    uint64_t m_cap) {
    const uint32_t nu = min(st->n_u, n_cap);
    for (uint32_t x = blockIdx.x * TPB + threadIdx.x; x < nu; x += gridDim.x * TPB) {
        if (u.kind[x] != KIND_INS) continue;
        const uint32_t s = u.seg[x];
        uint32_t L = 0, R = njobs - 1;  // last job starting at or before s
        while (L < R) {
            const uint32_t mid = (L + R + 1) >> 1;
            if (jobs[mid].sa <= s)
                L = mid;
            else
                R = mid - 1;
        }
        if (s < jobs[L].sa || s >= jobs[L].sa + jobs[L].sf) continue;  // a small window took it
        const uint32_t us = US[s];
        if (US[s + 1] - us <= GT_LOCAL) continue;  // k_gather merged this segment's updates
        const uint64_t y = u.key[x];
        const uint32_t ri = u.ip[x] - u.ip[us];
        const uint32_t tomb_below = (x - us) - ri;
        const uint64_t *sk = src.keys + 32 * heap_of_linear(s, src.H);
        uint32_t pos = 0;  // slots below y (the segment is sorted, NONE-padded)
#pragma unroll
        for (uint32_t step = 16; step; step >>= 1)
            if (sk[pos + step - 1] < y) pos += step;
        if (sk[pos] < y) pos++;
        uint32_t expired_below = 0;
        if (thres) {
            const uint8_t *sv = src.vals + (sk - src.keys);
            for (uint32_t t = 0; t < pos; t++)
                expired_below += (sv[t] != VAL_TOMB && (sk[t] & TIME_MASK) < (uint64_t)thres) ? 1u : 0u;
        }
        const uint64_t r = (uint64_t)PQ[s] + ri + (pos - tomb_below - expired_below);
        if (r < m_cap) {
            Mk[r] = y;
            Mv[r] = u.val[x];
        } else {  // only if the update list broke its sortedness invariant
            atomicOr(&st->sticky, ERR_INTERNAL);
            atomicCAS(&st->sticky_site, 0u, 5u);
        }
    }
}

__global__ void __launch_bounds__(GT_TPB) k_spread(const TileJob *__restrict__ jobs, uint32_t njobs, uint32_t ntiles,
                                                   Geo dst, const uint64_t *__restrict__ Mk,
                                                   const uint8_t *__restrict__ Mv, uint64_t m_cap,
                                                   const uint32_t *__restrict__ PQ, uint8_t *cnt_d, ulonglong2 *fl_d,
                                                   uint32_t *sent, uint32_t V, DevStatus *st) {
    const int lane = threadIdx.x & 31, gl = lane & 7, grp = threadIdx.x >> 3;
    for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const TileJob J = jobs[find_job(jobs, njobs, tile, true)];
        const uint64_t inv = ~0ull / J.df;  // the same for every thread of the tile
        const uint64_t k = 32ull * (tile - J.dtile0) + grp;
        if (k >= J.df) continue;
        const uint64_t mb = PQ[J.sa];
        if (k == 0 && gl == 0 && PQ[J.sa + J.sf] - mb != J.m) {  // the gather must account for m items
            atomicOr(&st->sticky, ERR_INTERNAL);
            atomicCAS(&st->sticky_site, 0u, 2u);
        }
        if (mb + J.m > m_cap) continue;  // reported above; never read past M
        const uint64_t ds = J.da + k;
        const uint64_t j = heap_of_linear(ds, dst.H);
        const uint64_t f0 = first_rank_recip(k, J.m, J.df, inv), f1 = first_rank_recip(k + 1, J.m, J.df, inv);
        const uint32_t nk = (uint32_t)(f1 - f0);
        uint64_t o[4];
        uint32_t ov = 0;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const uint32_t slot = 4 * gl + q;
            o[q] = KEY_NONE;
            if (slot < nk) {
                o[q] = Mk[mb + f0 + slot];
                ov |= (uint32_t)Mv[mb + f0 + slot] << (8 * q);
                if (is_sentinel(o[q])) {
                    const uint32_t row = (uint32_t)(o[q] >> SRC_SHIFT);
                    if (row < V) sent[row] = (uint32_t)(32 * j + slot);
                }
            }
        }
        ulonglong2 *kp = reinterpret_cast<ulonglong2 *>(dst.keys + 32 * j + 4 * gl);
        kp[0] = make_ulonglong2(o[0], o[1]);
        kp[1] = make_ulonglong2(o[2], o[3]);
        *reinterpret_cast<uint32_t *>(dst.vals + 32 * j + 4 * gl) = ov;
        if (gl == 0) {
            cnt_d[ds] = (uint8_t)nk;
            fl_d[j] = nk ? make_ulonglong2(Mk[mb + f0], Mk[mb + f1 - 1]) : make_ulonglong2(KEY_NONE, KEY_NONE);
        }
    }
}

// ------------------------------------------------------------------ levels
__global__ void __launch_bounds__(TPB) k_levelup_cnt(const uint8_t *__restrict__ cnt_old, uint8_t *cnt_new,
                                                     uint32_t H_old) {
    const uint64_t nn = nseg_of(H_old + 1);
    for (uint64_t s = blockIdx.x * (uint64_t)TPB + threadIdx.x; s < nn + 64; s += gridDim.x * (uint64_t)TPB)
        cnt_new[s] = (s < nn && (s & 1)) ? cnt_old[s >> 1] : (uint8_t)0;
}

__global__ void __launch_bounds__(TPB) k_check_empty_level(const uint8_t *__restrict__ cnt, uint32_t H, DevStatus *st) {
    const uint64_t nseg = nseg_of(H);
    for (uint64_t t = blockIdx.x * (uint64_t)TPB + threadIdx.x; 4 * t + 1 < nseg; t += gridDim.x * (uint64_t)TPB)
        if (cnt[4 * t + 1] == 0) st->empty_found = 1;
}

__global__ void __launch_bounds__(TPB) k_sum_cnt(const uint8_t *__restrict__ cnt, uint64_t nseg, DevStatus *st) {
    uint32_t acc = 0;
    for (uint64_t s = blockIdx.x * (uint64_t)TPB + threadIdx.x; s < nseg; s += gridDim.x * (uint64_t)TPB) acc += cnt[s];
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0 && acc) atomicAdd(&st->cnt_total, (unsigned long long)acc);
}

inline uint32_t grid_for(uint64_t n, uint32_t per_block, uint32_t cap = 152 * 16) {
    uint64_t g = (n + per_block - 1) / per_block;
    if (g == 0) g = 1;
    return (uint32_t)(g < cap ? g : cap);
}

}  // namespace

// ------------------------------------------------------------------ launchers
const void *pack_kernel_fn() { return reinterpret_cast<const void *>(&k_pack); }

void launch_pack(const uint64_t *ins, const uint8_t *ins_vals, uint32_t n_ins, const uint64_t *del, uint32_t n_del,
                 uint32_t V, uint32_t thres, uint32_t key_format, int internal, uint64_t *keys_out, uint16_t *pay_out,
                 DevStatus *st, uint32_t *bitmap, uint32_t bitmap_words, const ulonglong2 *fl, const uint8_t *cnt,
                 uint64_t pf_segs, uint32_t *sup, uint32_t sup_words, uint32_t *sort_bar, cudaStream_t s) {
    ProfScope ps_("pack", s);
    // enough blocks for the planner bitmap's clear too (16 words a thread)
    const uint32_t nb = std::max(grid_for(n_ins + n_del, TPB), grid_for(bitmap_words, TPB * 16, 152 * 4));
    k_pack<<<nb, TPB, 0, s>>>(ins, ins_vals, n_ins, del, n_del, V, thres, key_format, internal,
                                                        keys_out, pay_out, st, bitmap, bitmap_words, fl, cnt, pf_segs,
                                                        sup, sup_words, sort_bar);
    note_launch();
}

void launch_live_counts(const uint64_t *keys, uint32_t H, uint32_t thres, uint8_t *cnt_live, DevStatus *st,
                        cudaStream_t s) {
    ProfScope ps_("live_counts", s);
    k_live_counts<<<grid_for(nseg_of(H), TPB / 32), TPB, 0, s>>>(keys, H, thres, cnt_live, st);
    note_launch();
}

void launch_resolve_locate(const uint64_t *k0, const uint16_t *p0, const uint64_t *k1, const uint16_t *p1, uint32_t n,
                           SortMask mask, Geo g, const ulonglong2 *fl, uint32_t thres, uint8_t *kind, uint32_t *seg,
                           uint32_t *blk_nn, uint32_t *blk_ins, uint32_t *sup, DevStatus *st, cudaStream_t s) {
    ProfScope ps_("resolve_locate", s);
    const uint32_t nb = (n + TPB - 1) / TPB;
    launch_pdl(k_resolve_locate, dim3(nb < 152 * 8 ? nb : 152 * 8), dim3(TPB), 0, s, k0, p0, k1, p1, n, mask, g, fl,
               thres, kind, seg, blk_nn, blk_ins, sup, st);
    note_launch();
}

void launch_compact(const uint64_t *k0, const uint16_t *p0, const uint64_t *k1, const uint16_t *p1, SortMask mask,
                    const uint8_t *kind, const uint32_t *seg, uint32_t n, uint32_t *blk_nn, uint32_t *blk_ins,
                    const uint32_t *sup, UpdList u, DevStatus *st, cudaStream_t s) {
    ProfScope ps_("compact", s);
    const uint32_t nb = (n + TPB - 1) / TPB;
    launch_pdl(k_compact, dim3(nb), dim3(TPB), 0, s, k0, p0, k1, p1, mask, kind, seg, n, blk_nn, blk_ins, sup, u, st);
    note_launch();
}

void launch_relocate(UpdList u, uint32_t n, Geo g, const ulonglong2 *fl, cudaStream_t s) {
    ProfScope ps_("relocate", s);
    if (!n) return;
    k_relocate<<<(n + TPB - 1) / TPB, TPB, 0, s>>>(u, n, g, fl);
    note_launch();
}

void launch_compact_pending(const UpdList in, const uint8_t *pend, uint32_t n, UpdList out, uint32_t *blk_nn,
                            uint32_t *blk_ins, DevStatus *st, cudaStream_t s) {
    ProfScope ps_("compact_pending", s);
    // n = old compacted count (known on the host at this point)
    const uint32_t nb = (n + TPB - 1) / TPB;
    if (!nb) return;
    k_pending_counts<<<nb, TPB, 0, s>>>(in.kind, pend, n, st, blk_nn, blk_ins);
    k_scan_pairs<<<1, 1024, 0, s>>>(blk_nn, blk_ins, nb, out.ip, st);
    k_pending_scatter<<<nb, TPB, 0, s>>>(in, pend, n, n, blk_nn, blk_ins, out);
    note_launch(3);
}

void launch_plan(const UpdList u, uint32_t n_cap, const uint8_t *cnt, const uint32_t *P, int use_P,
                 uint64_t total_live, const unsigned long long *total_live_dev, uint32_t H, const Tables &tb,
                 uint32_t *bitmap, Window *cand, Window *single, Window *small4, Window *small, Window *big,
                 uint8_t *pend, DevStatus *st, cudaStream_t s, DevStatus *pub) {
    ProfScope ps_("plan", s);
    const uint32_t nb = (n_cap + TPB - 1) / TPB;
    if (!nb) return;
    launch_pdl(k_plan, dim3(nb), dim3(TPB), 0, s, u, n_cap, cnt, P, use_P, total_live, total_live_dev, H, tb, bitmap,
               cand, pend, st);
    launch_pdl(k_plan_max, dim3(nb), dim3(TPB), 0, s, cand, n_cap, H, bitmap, single, small4, small, big, u, pend, st,
               tb.cut_group ? tb.cut_group : CUT_GROUP_DEFAULT, tb.cut_shared ? tb.cut_shared : SMALL_WIN_SEGS, pub);
    note_launch(2);
}

void launch_exec_single(const Window *w, uint32_t n_cap, Geo g, uint8_t *cnt, ulonglong2 *fl, uint32_t *sent,
                        uint32_t V, const UpdList u, uint32_t thres, DevStatus *st, cudaStream_t s, bool guarded) {
    if (!n_cap) return;
    ProfScope ps_("exec_single", s);
    // one wave of resident blocks (4 a SM at 64 registers), each looping over
    // its windows: a second, partial wave would leave SMs idle at the end
    launch_pdl(thres ? k_exec_single<true> : k_exec_single<false>, dim3(grid_for(n_cap, ES_GROUPS, 152 * 4)),
               dim3(ES_TPB), 0, s, w, &st->n_single, n_cap, g, cnt, fl, sent, V, u, thres, st, guarded ? 1 : 0);
    note_launch();
}

void launch_exec_multi(const Window *w4, uint32_t cap4, const Window *w32, uint32_t cap32, Geo g, uint8_t *cnt,
                       ulonglong2 *fl, uint32_t *sent, uint32_t V, const UpdList u, uint32_t thres, DevStatus *st,
                       cudaStream_t s, bool guarded) {
    const uint32_t nb4 = cap4 ? grid_for(cap4, EM_GROUPS, 152 * 8) : 0, nb32 = cap32 ? grid_for(cap32, 4, 152 * 8) : 0;
    if (!nb4 && !nb32) return;
    ProfScope ps_("exec_small", s);
    launch_pdl(thres ? k_exec_multi<true> : k_exec_multi<false>, dim3(nb4 + nb32), dim3(EM_TPB), 0, s, w4,
               &st->n_small4, cap4, nb4, w32, &st->n_small, cap32, g, cnt, fl, sent, V, u, thres, st,
               guarded ? 1 : 0);
    note_launch();
}

void launch_count_present(const uint64_t *keys, uint32_t n, uint32_t key_format, Geo g, const ulonglong2 *fl,
                          uint32_t *count, cudaStream_t s) {
    if (!n) return;
    k_count_present<<<grid_for(n, TPB, 152 * 8), TPB, 0, s>>>(keys, n, key_format, g, fl, count);
    note_launch();
}

void launch_seg_update_counts(const UpdList u, uint32_t n_cap, uint32_t *qi, uint32_t *qd, const DevStatus *st,
                              cudaStream_t s) {
    ProfScope ps_("seg_counts", s);
    if (!n_cap) return;
    k_seg_update_counts<<<(n_cap + TPB - 1) / TPB, TPB, 0, s>>>(u, n_cap, qi, qd, st);
    note_launch();
}

void launch_tile_prefix(const uint8_t *cnt, const uint8_t *cnt_live, const uint32_t *qi, const uint32_t *qd,
                        uint64_t nseg, uint32_t *PQ, uint32_t *US, uint64_t *tmp, cudaStream_t s) {
    ProfScope ps_("scan", s);
    const uint32_t nb = (uint32_t)((nseg + TS_TILE - 1) / TS_TILE);
    if (!nb) {
        k_ts_top<<<1, 1024, 0, s>>>(tmp, 0, PQ + nseg, US + nseg);
        note_launch();
        return;
    }
    k_ts_reduce<<<nb, TPB, 0, s>>>(cnt, cnt_live, qi, qd, nseg, tmp);
    k_ts_top<<<1, 1024, 0, s>>>(tmp, nb, PQ + nseg, US + nseg);
    k_ts_down<<<nb, TPB, 0, s>>>(cnt, cnt_live, qi, qd, nseg, tmp, PQ, US);
    note_launch(3);
}

void launch_exec_big(const TileJob *jobs, uint32_t njobs, uint32_t stiles, uint32_t dtiles, Geo src,
                     const uint32_t *PQ, const uint32_t *US, const UpdList u, uint32_t n_upd, uint32_t thres,
                     uint64_t *Mk, uint8_t *Mv, uint64_t m_cap, Geo dst, uint8_t *cnt_d, ulonglong2 *fl_d,
                     uint32_t *sent, uint32_t V, DevStatus *st, cudaStream_t s) {
    if (!njobs) return;
    {
        ProfScope ps_("exec_gather", s);
        (thres ? k_gather<true> : k_gather<false>)<<<grid_for(stiles, 1, 152 * 8), GT_TPB, 0, s>>>(
            jobs, njobs, stiles, src, PQ, US, u, thres, Mk, Mv, m_cap, st);
        if (n_upd)
            k_gather_ins<<<grid_for(n_upd, TPB), TPB, 0, s>>>(jobs, njobs, src, PQ, US, u, st, n_upd, thres, Mk, Mv,
                                                              m_cap);
    }
    {
        ProfScope ps_("exec_spread", s);
        k_spread<<<grid_for(dtiles, 1, 152 * 8), GT_TPB, 0, s>>>(jobs, njobs, dtiles, dst, Mk, Mv, m_cap, PQ, cnt_d,
                                                                 fl_d, sent, V, st);
    }
    note_launch(n_upd ? 3 : 2);
}

namespace {
// big windows -> (first segment, index) pairs for the sort by position
__global__ void __launch_bounds__(TPB) k_big_keys(const Window *__restrict__ w, uint32_t n, uint64_t *keys,
                                                  uint16_t *pay) {
    for (uint32_t i = blockIdx.x * TPB + threadIdx.x; i < n; i += gridDim.x * TPB) {
        // the window index rides in the key's low half (a < 2^32), so the
        // sort payload is unused
        keys[i] = ((uint64_t)w[i].a << 32) | i;
        pay[i] = 0;
    }
}

// sorted big windows -> tile jobs: one CTA, a chunk of windows per thread
__global__ void __launch_bounds__(1024) k_big_jobs(const uint64_t *__restrict__ sorted, const Window *__restrict__ w,
                                                   uint32_t n, TileJob *jobs) {
    __shared__ uint32_t wsum[32];
    __shared__ uint32_t carry;
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint32_t b0 = 0; b0 < n; b0 += 1024) {
        const uint32_t i = b0 + threadIdx.x;
        Window W{};
        uint32_t t = 0;
        if (i < n) {
            W = w[(uint32_t)sorted[i]];
            t = (W.f + 31) / 32;
        }
        uint32_t v = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += y;
        }
        if (lane == 31) wsum[wp] = v;
        __syncthreads();
        if (wp == 0) {
            uint32_t x = wsum[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            wsum[lane] = x;
        }
        __syncthreads();
        const uint32_t ex = carry + (wp ? wsum[wp - 1] : 0) + v - t;
        if (i < n) jobs[i] = TileJob{W.a, W.f, W.a, W.f, W.m, ex, ex, 0};
        __syncthreads();
        if (threadIdx.x == 0) carry += wsum[31];
        __syncthreads();
    }
}
}  // namespace

namespace {
__global__ void k_set_job(TileJob *jobs, TileJob j) { jobs[0] = j; }
}  // namespace

void launch_set_job(TileJob *jobs, const TileJob &j, cudaStream_t s) {
    k_set_job<<<1, 1, 0, s>>>(jobs, j);
    note_launch();
}

void launch_big_jobs(const Window *wbig, uint32_t n, uint64_t *kscratch, uint64_t *kscratch2, uint16_t *pscratch,
                     uint16_t *pscratch2, SortScratch &ss, TileJob *jobs, cudaStream_t s) {
    ProfScope ps_("big_jobs", s);
    k_big_keys<<<grid_for(n, TPB), TPB, 0, s>>>(wbig, n, kscratch, pscratch);
    // first segments are unique: sorting (a << 32 | index) by its upper four
    // bytes orders the windows; four passes leave ping-pong tiers in place
    const SortTier t = sort_tier_for_update(n, ss);
    sort_pairs_dev<uint16_t>(kscratch, pscratch, kscratch2, pscratch2, n,
                             SortMask{nullptr, 0xF0u, sort_tier_in_place(t) ? 0u : 1u}, ss, s, t);
    k_big_jobs<<<1, 1024, 0, s>>>(kscratch, wbig, n, jobs);
    note_launch(3);
}

void launch_levelup_cnt(const uint8_t *cnt_old, uint8_t *cnt_new, uint32_t H_old, cudaStream_t s) {
    ProfScope ps_("levelup_cnt", s);
    k_levelup_cnt<<<grid_for(nseg_of(H_old + 1) + 64, TPB), TPB, 0, s>>>(cnt_old, cnt_new, H_old);
    note_launch();
}

void launch_check_empty_level(const uint8_t *cnt, uint32_t H, DevStatus *st, cudaStream_t s) {
    ProfScope ps_("check_empty", s);
    k_check_empty_level<<<grid_for(nseg_of(H) / 4 + 1, TPB), TPB, 0, s>>>(cnt, H, st);
    note_launch();
}

void launch_sum_cnt(const uint8_t *cnt, uint64_t nseg, DevStatus *st, cudaStream_t s) {
    ProfScope ps_("sum_cnt", s);
    k_sum_cnt<<<grid_for(nseg, TPB), TPB, 0, s>>>(cnt, nseg, st);
    note_launch();
}

// ------------------------------------------------------------------ forest launches
namespace {

// per-call status reset (the single-graph front copies a host template) and
// the planner bitmap; one block per graph
__global__ void __launch_bounds__(TPB) k_forest_reset(const ForestGraph *__restrict__ F) {
    const ForestGraph &f = F[blockIdx.x];
    uint32_t *w = reinterpret_cast<uint32_t *>(f.st);
    constexpr uint32_t NW = offsetof(DevStatus, sticky) / 4;
    for (uint32_t i = threadIdx.x; i < NW; i += TPB) w[i] = 0;
    for (uint64_t i = threadIdx.x; i < f.bitmap_words; i += TPB) f.bitmap[i] = 0;
    for (uint32_t i = threadIdx.x; i < f.sup_words; i += TPB) f.sup[i] = 0;
    __syncthreads();
    if (threadIdx.x == 0) {
        f.st->min_t_ins = 0xFFFFFFFFu;
        f.st->key_and = ~0ull;
        f.st->err_info[0] = 0xFFFFFFFFu;
        f.st->total_items = f.total_items;
    }
}

__global__ void __launch_bounds__(TPB) k_forest_pack(const ForestGraph *__restrict__ F, const uint32_t *boff,
                                                     uint32_t G) {
    const uint32_t g = forest_job_of(boff, G, blockIdx.x);
    const ForestGraph &f = F[g];
    k_pack_body(f.ins, f.ins_vals, f.n_ins, f.del, f.n_del, f.V, 0, f.key_format, 0, f.bk0, f.bp0, f.st,
                blockIdx.x - boff[g], boff[g + 1] - boff[g]);
}

// the sorted batch is (f.sk, f.sp), wherever the forest sort left it:
// parity mask {nullptr, 0}
__global__ void __launch_bounds__(TPB) k_forest_resolve(const ForestGraph *__restrict__ F, const uint32_t *boff,
                                                        uint32_t G) {
    const uint32_t g = forest_job_of(boff, G, blockIdx.x);
    const ForestGraph &f = F[g];
    k_resolve_locate_body(f.sk, f.sp, f.sk, f.sp, f.n_ins + f.n_del, SortMask{nullptr, 0u, 0u}, f.g, f.fl, 0, f.kind,
                          f.seg, f.blk_nn, f.blk_ins, f.sup, f.st, blockIdx.x - boff[g], boff[g + 1] - boff[g]);
}

__global__ void __launch_bounds__(TPB) k_forest_compact(const ForestGraph *__restrict__ F, const uint32_t *boff,
                                                        uint32_t G) {
    const uint32_t g = forest_job_of(boff, G, blockIdx.x);
    const ForestGraph &f = F[g];
    k_compact_body(f.sk, f.sp, f.sk, f.sp, SortMask{nullptr, 0u, 0u}, f.kind, f.seg, f.n_ins + f.n_del, f.blk_nn,
                   f.blk_ins, f.sup, f.u, f.st, blockIdx.x - boff[g], boff[g + 1] - boff[g]);
}

__global__ void __launch_bounds__(TPB) k_forest_plan(const ForestGraph *__restrict__ F, const uint32_t *boff,
                                                     uint32_t G) {
    const uint32_t g = forest_job_of(boff, G, blockIdx.x);
    const ForestGraph &f = F[g];
    k_plan_body(f.u, f.n_ins + f.n_del, f.cnt, nullptr, 0, 0, &f.st->total_items, f.g.H, f.tb, f.bitmap, f.cand,
                f.pend, f.st, blockIdx.x - boff[g], boff[g + 1] - boff[g]);
}

__global__ void __launch_bounds__(TPB) k_forest_plan_max(const ForestGraph *__restrict__ F, const uint32_t *boff,
                                                         uint32_t G) {
    const uint32_t g = forest_job_of(boff, G, blockIdx.x);
    const ForestGraph &f = F[g];
    k_plan_max_body(f.cand, f.n_ins + f.n_del, f.g.H, f.bitmap, f.wsingle, f.wsmall4, f.wsmall, f.wbig, f.u, f.pend,
                    f.st, blockIdx.x - boff[g], boff[g + 1] - boff[g]);
}

__global__ void __launch_bounds__(ES_TPB, 4) k_forest_exec_single(const ForestExec *__restrict__ E,
                                                                   const uint32_t *boff, uint32_t G) {
    const uint32_t g = forest_job_of(boff, G, blockIdx.x);
    const ForestExec &e = E[g];
    k_exec_single_body<false>(e.w[0], &e.st->n_single, e.n[0], e.g, e.cnt, e.fl, e.sent, e.V, e.u, 0, e.st,
                       blockIdx.x - boff[g], boff[g + 1] - boff[g]);
}

template <int GS>
__global__ void __launch_bounds__(EM_TPB, 4) k_forest_exec_multi(const ForestExec *__restrict__ E, const uint32_t *boff,
                                                                 uint32_t G) {
    constexpr int K = GS == 4 ? 1 : 2;
    __shared__ __align__(16) unsigned char smem[EM_SMEM];
    const uint32_t g = forest_job_of(boff, G, blockIdx.x);
    const ForestExec &e = E[g];
    if (GS == 4)
        exec_multi4<false>(smem, e.w[K], &e.st->n_small4, e.n[K], e.g, e.cnt, e.fl, e.sent, e.V, e.u, 0, e.st,
                    blockIdx.x - boff[g], boff[g + 1] - boff[g]);
    else
        exec_multi32<false>(smem, e.w[K], &e.st->n_small, e.n[K], e.g, e.cnt, e.fl, e.sent, e.V, e.u, 0, e.st,
                     blockIdx.x - boff[g], boff[g + 1] - boff[g]);
}

__global__ void __launch_bounds__(64) k_forest_status(const ForestGraph *__restrict__ F, DevStatus *out) {
    const uint32_t *src = reinterpret_cast<const uint32_t *>(F[blockIdx.x].st);
    uint32_t *dst = reinterpret_cast<uint32_t *>(out + blockIdx.x);
    for (uint32_t i = threadIdx.x; i < sizeof(DevStatus) / 4; i += 64) dst[i] = src[i];
}

}  // namespace

cudaError_t set_exec_wait_debug(uint32_t give_up) {
    return cudaMemcpyToSymbol(g_exec_wait_give_up, &give_up, sizeof(uint32_t));
}

uint32_t exec_ctas(int kind, uint32_t n) {
    if (!n) return 0;
    return grid_for(n, kind == 0 ? ES_GROUPS : (kind == 1 ? EM_GROUPS : 4), 152 * 8);
}

void launch_forest_exec(int kind, const ForestExec *E, const uint32_t *boff, uint32_t G, uint32_t nblocks,
                        cudaStream_t s) {
    if (!G || !nblocks) return;
    if (kind == 0) {
        ProfScope ps_("forest_exec_single", s);
        k_forest_exec_single<<<nblocks, ES_TPB, 0, s>>>(E, boff, G);
    } else if (kind == 1) {
        ProfScope ps_("forest_exec_small4", s);
        k_forest_exec_multi<4><<<nblocks, EM_TPB, 0, s>>>(E, boff, G);
    } else {
        ProfScope ps_("forest_exec_small32", s);
        k_forest_exec_multi<32><<<nblocks, EM_TPB, 0, s>>>(E, boff, G);
    }
    note_launch();
}

void launch_forest_phase(int phase, const ForestGraph *F, const uint32_t *boff, uint32_t G, uint32_t nblocks,
                         DevStatus *out, cudaStream_t s) {
    if (!G || (phase >= 1 && phase <= 5 && !nblocks)) return;
    static const char *const names[7] = {"forest_reset", "forest_pack",     "forest_resolve", "forest_compact",
                                         "forest_plan",  "forest_plan_max", "forest_status"};
    ProfScope ps_(names[phase % 7], s);
    switch (phase) {
        case 0: k_forest_reset<<<G, TPB, 0, s>>>(F); break;
        case 1: k_forest_pack<<<nblocks, TPB, 0, s>>>(F, boff, G); break;
        case 2: k_forest_resolve<<<nblocks, TPB, 0, s>>>(F, boff, G); break;
        case 3: k_forest_compact<<<nblocks, TPB, 0, s>>>(F, boff, G); break;
        case 4: k_forest_plan<<<nblocks, TPB, 0, s>>>(F, boff, G); break;
        case 5: k_forest_plan_max<<<nblocks, TPB, 0, s>>>(F, boff, G); break;
        case 6: k_forest_status<<<G, 64, 0, s>>>(F, out); break;
    }
    note_launch();
}

}  // namespace lpma
