// Radix sort and scan primitives (hand-written, sm_103a).
//
// Sort: LSD radix sort on 8-bit digits, reduce-then-scan per digit pass:
// k_upsweep counts the digits of every 2048-key tile, k_dscan turns the
// (digit, tile) counts into exclusive global offsets (digit-major, one warp
// per digit, digit bases from a histogram of all eight digits taken once
// per sort), k_downsweep ranks each tile's keys stably with
// __match_any_sync and scatters them.  No CTA waits on another.  Bytes that
// are equal across all keys are skipped.  Batches of at most one tile are
// sorted by one CTA in shared memory in a single launch.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "lpma_common.cuh"
#include "per_device.h"
#include "prims.cuh"

namespace lpma {

static std::atomic<uint64_t> g_launches{0};
void note_launch(int k) { g_launches += (uint64_t)k; }
uint64_t launch_count() { return g_launches.load(); }

struct ProfRec {
    const char *name;
    cudaEvent_t a, b;
};
static std::vector<ProfRec> g_prof;
static std::vector<cudaEvent_t> g_event_pool;
static bool g_prof_on = false;
static std::mutex g_prof_mu;

static cudaEvent_t pool_event() {
    if (!g_event_pool.empty()) {
        cudaEvent_t e = g_event_pool.back();
        g_event_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}

bool prof_enabled() { return g_prof_on; }

cudaError_t host_wait(cudaStream_t s, bool blocking) {
    if (!blocking) return cudaStreamSynchronize(s);
    thread_local cudaEvent_t ev = nullptr;
    thread_local int ev_dev = -1;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e) return e;
    if (!ev || ev_dev != dev) {
        if ((e = cudaEventCreateWithFlags(&ev, cudaEventBlockingSync | cudaEventDisableTiming))) return e;
        ev_dev = dev;
    }
    if ((e = cudaEventRecord(ev, s))) return e;
    return event_wait(ev);
}

cudaError_t event_wait(cudaEvent_t ev) {
    // short waits end in the spin; long ones sleep (the event was created
    // with cudaEventBlockingSync)
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        const cudaError_t q = cudaEventQuery(ev);
        if (q != cudaErrorNotReady) return q;
        if (std::chrono::steady_clock::now() - t0 > std::chrono::microseconds(40)) break;
    }
    return cudaEventSynchronize(ev);
}

// one thread spins for `cycles` SM clocks (bounded by construction)
__global__ void k_prof_delay(long long cycles) {
    if (threadIdx.x) return;
    const long long t0 = clock64();
    while (clock64() - t0 < cycles) {
    }
}

ProfScope::ProfScope(const char *name, cudaStream_t st) : idx(-1), s(st) {
    if (!g_prof_on) return;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    k_prof_delay<<<1, 32, 0, s>>>(60000);  // about 30 us at 2 GHz
    ProfRec r{name, pool_event(), pool_event()};
    cudaEventRecord(r.a, s);
    g_prof.push_back(r);
    idx = (int)g_prof.size() - 1;
}
ProfScope::~ProfScope() {
    if (idx < 0) return;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    cudaEventRecord(g_prof[idx].b, s);
}

void prof_enable(int on) {
    std::lock_guard<std::mutex> lk(g_prof_mu);
    g_prof_on = on != 0;
}

// "name launches total_ms" per kernel name, in order of first appearance;
// clears the record.  Synchronises with the recorded events.
size_t prof_report(char *buf, size_t cap) {
    std::lock_guard<std::mutex> lk(g_prof_mu);
    std::vector<std::string> names;
    std::vector<double> tot;
    std::vector<long> cnt;
    for (ProfRec &r : g_prof) {
        cudaEventSynchronize(r.b);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, r.a, r.b);
        size_t k = 0;
        while (k < names.size() && names[k] != r.name) k++;
        if (k == names.size()) {
            names.push_back(r.name);
            tot.push_back(0.0);
            cnt.push_back(0);
        }
        tot[k] += ms;
        cnt[k] += 1;
        g_event_pool.push_back(r.a);
        g_event_pool.push_back(r.b);
    }
    g_prof.clear();
    std::string out;
    char line[256];
    for (size_t k = 0; k < names.size(); k++) {
        snprintf(line, sizeof(line), "%s %ld %.6f\n", names[k].c_str(), cnt[k], tot[k]);
        out += line;
    }
    if (buf && cap) {
        size_t n = out.size() < cap - 1 ? out.size() : cap - 1;
        memcpy(buf, out.data(), n);
        buf[n] = 0;
    }
    return out.size();
}

namespace {

// Block-wide exclusive scan of one value per thread (blockDim == 256).
__device__ inline uint32_t block_excl_scan_256(uint32_t x, uint32_t *wsum /*[8]*/, uint32_t *total) {
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
        uint32_t s = lane < 8 ? wsum[lane] : 0;
#pragma unroll
        for (int o = 1; o < 8; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < 8) wsum[lane] = s;  // inclusive warp sums
    }
    __syncthreads();
    uint32_t base = w ? wsum[w - 1] : 0;
    if (total) *total = wsum[7];
    uint32_t r = base + v - x;
    __syncthreads();
    return r;
}

// The same over u64 values (two independent u32 scans in the halves, as
// long as neither half's total reaches 2^32).
__device__ inline uint64_t block_excl_scan_256_u64(uint64_t x, uint64_t *wsum /*[8]*/, uint64_t *total) {
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
        uint64_t s = lane < 8 ? wsum[lane] : 0;
#pragma unroll
        for (int o = 1; o < 8; o <<= 1) {
            const uint64_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < 8) wsum[lane] = s;
    }
    __syncthreads();
    const uint64_t base = w ? wsum[w - 1] : 0;
    if (total) *total = wsum[7];
    const uint64_t r = base + v - x;
    __syncthreads();
    return r;
}

// Rank the IPT keys each lane holds among the keys of its warp with the same
// digit.  Keys of warp w are at tile positions w*32*IPT + i*32 + lane, so
// the rank order is the input order.  whist[2^RB] is this warp's digit
// counter row (zeroed by the caller); on return it holds the warp's counts.
// The lanes that share a digit are found with RB ballots (one per digit
// bit), which issue far faster than a match instruction; the lowest of them
// adds the group's size to the warp's counter and shares the old value.
// Counter updates of one warp land in program order, so ranks are stable.
template <int IPT, int RB = 8>
__device__ inline void warp_rank(const uint64_t (&k)[IPT], uint32_t valid_mask, int sh, uint32_t *whist,
                                 uint32_t (&rank)[IPT], int rounds = IPT) {
    const uint32_t lt = lanemask_lt();
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int i = 0; i < IPT; i++) {
        if (i >= rounds) break;  // warp-uniform: no valid key in rounds >= rounds
        const bool valid = (valid_mask >> i) & 1u;
        const uint32_t d = (uint32_t)((k[i] >> sh) & ((1u << RB) - 1));
        uint32_t peers = __ballot_sync(0xffffffffu, valid);
#pragma unroll
        for (int b = 0; b < RB; b++) {
            const bool bit = (d >> b) & 1u;
            const uint32_t bal = __ballot_sync(0xffffffffu, bit);
            peers &= bit ? bal : ~bal;
        }
        const int leader = __ffs(peers) - 1;
        uint32_t base = 0;
        if (valid && lane == leader) base = atomicAdd(&whist[d], (uint32_t)__popc(peers));
        base = __shfl_sync(0xffffffffu, base, leader & 31);
        rank[i] = base + __popc(peers & lt);
    }
    __syncwarp();
}

// ---------------------------------------------------------------- histogram
__global__ void __launch_bounds__(256) k_hist(const uint64_t *__restrict__ keys, uint32_t n, uint32_t *hist) {
    __shared__ uint32_t h[8][256];
    for (int i = threadIdx.x; i < 8 * 256; i += 256) (&h[0][0])[i] = 0;
    __syncthreads();
    for (uint32_t i = blockIdx.x * 256 + threadIdx.x; i < n; i += gridDim.x * 256) {
        const uint64_t k = keys[i];
#pragma unroll
        for (int b = 0; b < 8; b++) atomicAdd(&h[b][(k >> (8 * b)) & 0xFF], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 8 * 256; i += 256) {
        uint32_t c = (&h[0][0])[i];
        if (c) atomicAdd(&hist[i], c);
    }
}

// ---------------------------------------------------------------- one pass
__global__ void __launch_bounds__(SORT_TPB) k_upsweep(const uint64_t *__restrict__ k0, const uint64_t *__restrict__ k1,
                                                      uint32_t n, int byte, SortMask mask, uint32_t *counts,
                                                      uint32_t T) {
    const uint32_t act = active_bytes(mask);
    if (!((act >> byte) & 1u)) return;
    const uint64_t *keys = (__popc(act & ((1u << byte) - 1)) & 1) ? k1 : k0;
    const int sh = 8 * byte;
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const uint64_t base = (uint64_t)blockIdx.x * SORT_TILE;
#pragma unroll
    for (int i = 0; i < SORT_IPT; i++) {
        const uint64_t p = base + (uint64_t)i * SORT_TPB + threadIdx.x;
        if (p < n) atomicAdd(&h[(keys[p] >> sh) & 0xFF], 1u);
    }
    __syncthreads();
    counts[(size_t)threadIdx.x * T + blockIdx.x] = h[threadIdx.x];
}

// one warp per digit: offs[d][t] = base(d) + sum of counts[d][t' < t]
__global__ void __launch_bounds__(256) k_dscan(const uint32_t *__restrict__ counts, uint32_t T,
                                               const uint32_t *__restrict__ hist, uint32_t *offs, int byte,
                                               SortMask mask) {
    if (!((active_bytes(mask) >> byte) & 1u)) return;
    __shared__ uint32_t gd[256];
    __shared__ uint32_t wsum[8];
    gd[threadIdx.x] = block_excl_scan_256(hist[threadIdx.x], wsum, nullptr);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const uint32_t d = blockIdx.x * 8 + (threadIdx.x >> 5);
    uint32_t run = gd[d];
    const uint32_t *c = counts + (size_t)d * T;
    uint32_t *o = offs + (size_t)d * T;
    for (uint32_t t0 = 0; t0 < T; t0 += 32) {
        const uint32_t t = t0 + lane;
        const uint32_t x = t < T ? c[t] : 0;
        uint32_t v = x;
#pragma unroll
        for (int k = 1; k < 32; k <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, v, k);
            if (lane >= k) v += y;
        }
        if (t < T) o[t] = run + v - x;
        run += __shfl_sync(0xffffffffu, v, 31);
    }
}

template <typename V>
struct PassSmem {
    uint64_t k[SORT_TILE];
    V v[SORT_TILE];
    uint32_t whist[8][256];
    uint32_t gbase[256];
    uint32_t ldig[256];
    uint32_t wsum[8];
};

template <typename V>
__global__ void __launch_bounds__(SORT_TPB) k_downsweep(uint64_t *k0, V *v0, uint64_t *k1, V *v1, uint32_t n, int byte,
                                                        SortMask mask, const uint32_t *__restrict__ offs, uint32_t T) {
    const uint32_t act = active_bytes(mask);
    if (!((act >> byte) & 1u)) return;
    const bool odd = __popc(act & ((1u << byte) - 1)) & 1;
    const uint64_t *__restrict__ ki = odd ? k1 : k0;
    const V *__restrict__ vi = odd ? v1 : v0;
    uint64_t *__restrict__ ko = odd ? k0 : k1;
    V *__restrict__ vo = odd ? v0 : v1;
    const int sh = 8 * byte;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    PassSmem<V> &S = *reinterpret_cast<PassSmem<V> *>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const uint32_t tile = blockIdx.x;
    for (int i = tid; i < 8 * 256; i += SORT_TPB) (&S.whist[0][0])[i] = 0;
    S.gbase[tid] = offs[(size_t)tid * T + tile];
    __syncthreads();
    const uint64_t base = (uint64_t)tile * SORT_TILE;
    uint64_t k[SORT_IPT];
    V v[SORT_IPT];
    uint32_t vmask = 0;
#pragma unroll
    for (int i = 0; i < SORT_IPT; i++) {
        const uint64_t p = base + (uint64_t)w * 32 * SORT_IPT + i * 32 + lane;
        if (p < n) {
            k[i] = ki[p];
            v[i] = vi[p];
            vmask |= 1u << i;
        } else {
            k[i] = ~0ull;
            v[i] = V(0);
        }
    }
    uint32_t rank[SORT_IPT];
    warp_rank<SORT_IPT>(k, vmask, sh, S.whist[w], rank);
    __syncthreads();
    // per digit (thread tid == digit): warp-exclusive offsets and tile count
    uint32_t tcount = 0;
#pragma unroll
    for (int ww = 0; ww < 8; ww++) {
        const uint32_t c = S.whist[ww][tid];
        S.whist[ww][tid] = tcount;
        tcount += c;
    }
    S.ldig[tid] = block_excl_scan_256(tcount, S.wsum, nullptr);
    __syncthreads();
#pragma unroll
    for (int i = 0; i < SORT_IPT; i++) {
        if ((vmask >> i) & 1u) {
            const uint32_t d = (uint32_t)((k[i] >> sh) & 0xFF);
            const uint32_t pos = S.ldig[d] + S.whist[w][d] + rank[i];
            S.k[pos] = k[i];
            S.v[pos] = v[i];
        }
    }
    __syncthreads();
    const uint32_t nvalid = (uint32_t)umin64(SORT_TILE, n - base);
    for (uint32_t p = tid; p < nvalid; p += SORT_TPB) {
        const uint64_t kk = S.k[p];
        const uint32_t d = (uint32_t)((kk >> sh) & 0xFF);
        const uint32_t g = S.gbase[d] + (p - S.ldig[d]);
        ko[g] = kk;
        vo[g] = S.v[p];
    }
}

// ---------------------------------------------------------------- cooperative sort
// All digit passes of one sort in one cooperative launch: CTA t owns tile t
// (COOP_TILE keys) in every pass.  A pass is: load the tile, rank it by the
// pass digit, publish the tile's digit counts; grid barrier (the tile is
// reordered in shared memory while the CTA waits); CTAs scan the count
// columns (one digit each); grid barrier; every CTA adds its column offsets
// to the global digit bases and writes its reordered tile out; grid
// barrier before the next pass reads.  The
// three grid barriers replace the reduce-then-scan sort's three launches
// per digit and its separate histogram pass.  Every barrier wait is bounded:
// after BAR_SPIN_LIMIT polls the CTA records ERR_TIMEOUT and goes on, so
// the kernel always ends.

constexpr uint32_t BAR_SPIN_LIMIT = 1u << 22;

// Test setting of the grid barrier (lpma_debug_sort_barrier): a poll limit
// in place of BAR_SPIN_LIMIT (0: the default) and, when unreachable is set,
// a target that no arrival count reaches, so that every wait runs out and
// takes the give-up path.  Read by the waiting thread at run time, so
// captured update fronts follow it too.
__device__ uint32_t g_bar_poll_limit = 0;
__device__ uint32_t g_bar_unreachable = 0;

__device__ __forceinline__ uint32_t ld_acquire_gpu(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Split grid barrier.  Arrive: after the CTA's barrier, one release add
// (it orders every write the CTA made before it, at GPU scope).  Wait: one
// thread polls with acquire loads, then the CTA's barrier passes the order
// on.  Work that needs no other CTA's data can run between the two.
__device__ __forceinline__ void grid_arrive(uint32_t *bar) {
    __syncthreads();
    if (threadIdx.x == 0) asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(bar) : "memory");
}

__device__ __forceinline__ void grid_wait(uint32_t *bar, uint32_t target, uint32_t *err) {
    if (threadIdx.x == 0) {
        const uint32_t lim = g_bar_poll_limit ? g_bar_poll_limit : BAR_SPIN_LIMIT;
        if (g_bar_unreachable) target = 0xFFFFFFFFu;
        uint32_t it = 0;
        while (ld_acquire_gpu(bar) < target) {
            if (++it > lim) {
                if (err) atomicOr(err, ERR_TIMEOUT);
                break;
            }
            if (it > 64) __nanosleep(64);
        }
    }
    __syncthreads();
}

__device__ __forceinline__ void grid_barrier(uint32_t *bar, uint32_t target, uint32_t *err) {
    grid_arrive(bar);
    grid_wait(bar, target, err);
}

template <typename V, int NB>
struct CoopSmem {
    uint64_t k[COOP_TILE];
    V v[COOP_TILE];
    uint32_t whist[8][NB];
    uint32_t gbase[NB];
    uint32_t ldig[NB];
    uint32_t wsum[8];
    uint64_t wsum64[8];
};

template <typename V>
__device__ __forceinline__ V ld_cg(const V *p) {
    return __ldcg(p);
}
template <>
__device__ __forceinline__ uint16_t ld_cg<uint16_t>(const uint16_t *p) {
    return (uint16_t)__ldcg(reinterpret_cast<const unsigned short *>(p));
}

// Tile t is keys [t * tile_len, min(n, (t+1) * tile_len)), tile_len <=
// COOP_TILE; warp w of a tile takes a contiguous run of ceil(tile_len / 8)
// of them.  Digits of RB bits (NB = 2^RB of them, 8 or 9 bits: the digit
// passes of sort_digit_next); thread tid owns the NB / 256 adjacent digits
// from tid * NB / 256.  counts is [NB][G] (digit-major, for the column
// scans), offs [G][NB] (tile-major, one row per CTA), totals [NB].
template <typename V, int RB>
__global__ void __launch_bounds__(SORT_TPB, 2) k_coop_sort(uint64_t *k0, V *v0, uint64_t *k1, V *v1, uint32_t n,
                                                           uint32_t tile_len, SortMask mask, uint32_t *counts,
                                                           uint32_t *offs, uint32_t *totals, uint32_t *bar,
                                                           uint32_t *err) {
    constexpr int NB = 1 << RB, PER = NB / SORT_TPB;
    static_assert(PER >= 1 && NB % SORT_TPB == 0, "whole digits per thread");
    griddep_wait();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CoopSmem<V, NB> &S = *reinterpret_cast<CoopSmem<V, NB> *>(smem_raw);
    const uint32_t G = gridDim.x, tile = blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    uint64_t rem = sort_digit_bits(mask);  // bits the remaining passes cover
    const uint64_t base = (uint64_t)tile * tile_len;
    const uint32_t nvalid = (uint32_t)umin64(tile_len, n - base);
    const uint32_t pw = (tile_len + 7) / 8;  // keys per warp
    const uint32_t wbeg = (uint32_t)umin64((uint64_t)w * pw, nvalid), wend = (uint32_t)umin64(wbeg + pw, nvalid);
    const int rounds = (int)((wend - wbeg + 31) / 32);
    uint32_t target = 0;
    for (uint32_t pass = 0; rem; pass++) {
        const int sh = sort_digit_next(rem, RB);
        const bool odd = pass & 1;
        const uint64_t *ki = odd ? k1 : k0;
        const V *vi = odd ? v1 : v0;
        uint64_t *ko = odd ? k0 : k1;
        V *vo = odd ? v0 : v1;
        for (int i = tid; i < 8 * NB; i += SORT_TPB) (&S.whist[0][0])[i] = 0;
        __syncthreads();
        // keys written by other CTAs in the previous pass: load through L2
        uint64_t k[COOP_IPT];
        V v[COOP_IPT];
        uint32_t vmask = 0;
#pragma unroll
        for (int i = 0; i < COOP_IPT; i++) {
            const uint32_t q = wbeg + i * 32 + lane;
            if (q < wend) {
                k[i] = __ldcg(ki + base + q);
                v[i] = ld_cg<V>(vi + base + q);
                vmask |= 1u << i;
            } else {
                k[i] = ~0ull;
                v[i] = V(0);
            }
        }
        uint32_t rank[COOP_IPT];
        warp_rank<COOP_IPT, RB>(k, vmask, sh, S.whist[w], rank, rounds);
        __syncthreads();
        // per digit: warp-exclusive offsets and the tile's count
        uint32_t tc[PER], tsum = 0;
#pragma unroll
        for (int r = 0; r < PER; r++) {
            const int d = tid * PER + r;
            uint32_t c0 = 0;
#pragma unroll
            for (int ww = 0; ww < 8; ww++) {
                const uint32_t c = S.whist[ww][d];
                S.whist[ww][d] = c0;
                c0 += c;
            }
            counts[(size_t)d * G + tile] = c0;
            tc[r] = c0;
            tsum += c0;
        }
        {
            uint32_t run = block_excl_scan_256(tsum, S.wsum, nullptr);
#pragma unroll
            for (int r = 0; r < PER; r++) {
                S.ldig[tid * PER + r] = run;
                run += tc[r];
            }
        }
        target += G;
        grid_arrive(bar);
        // while the other tiles publish their counts: reorder this tile by
        // the pass digit in shared memory (local offsets only)
#pragma unroll
        for (int i = 0; i < COOP_IPT; i++) {
            if ((vmask >> i) & 1u) {
                const uint32_t d = (uint32_t)((k[i] >> sh) & (NB - 1));
                const uint32_t pos = S.ldig[d] + S.whist[w][d] + rank[i];
                S.k[pos] = k[i];
                S.v[pos] = v[i];
            }
        }
        grid_wait(bar, target, err);
        // column scans: offs[d][t] = sum of counts[d][t' < t], totals[d].
        // Groups of S threads (S = G rounded up to a power of two) scan one
        // column each, so the NB columns take NB / 256 or 2 NB / 256 rounds
        // of the grid whatever G is (G <= 512; above 256 a thread takes two
        // entries).
        if (G > 256 && NB == 512) {
            // thread tid takes the adjacent entries 2 tid and 2 tid + 1 of
            // the columns d and d + 256, scanned together in u64 halves
            const uint32_t i0 = 2 * (uint32_t)tid, i1 = i0 + 1;
            for (uint32_t d = tile; d < 256; d += G) {
                const uint32_t *ca = counts + (size_t)d * G, *cb = counts + (size_t)(d + 256) * G;
                const uint32_t a0 = i0 < G ? __ldcg(ca + i0) : 0u, a1 = i1 < G ? __ldcg(ca + i1) : 0u;
                const uint32_t b0 = i0 < G ? __ldcg(cb + i0) : 0u, b1 = i1 < G ? __ldcg(cb + i1) : 0u;
                uint64_t tot = 0;
                const uint64_t e = block_excl_scan_256_u64((uint64_t)(a0 + a1) | ((uint64_t)(b0 + b1) << 32),
                                                           S.wsum64, &tot);
                const uint32_t ea = (uint32_t)e, eb = (uint32_t)(e >> 32);
                if (i0 < G) offs[(size_t)i0 * NB + d] = ea, offs[(size_t)i0 * NB + d + 256] = eb;
                if (i1 < G) offs[(size_t)i1 * NB + d] = ea + a0, offs[(size_t)i1 * NB + d + 256] = eb + b0;
                if (tid == 0) totals[d] = (uint32_t)tot, totals[d + 256] = (uint32_t)(tot >> 32);
            }
        } else if (G > 256) {
            // thread tid takes the adjacent entries 2 tid and 2 tid + 1
            const uint32_t i0 = 2 * (uint32_t)tid, i1 = i0 + 1;
            for (uint32_t d = tile; d < (uint32_t)NB; d += G) {
                const uint32_t *c = counts + (size_t)d * G;
                const uint32_t x0 = i0 < G ? __ldcg(c + i0) : 0u;
                const uint32_t x1 = i1 < G ? __ldcg(c + i1) : 0u;
                uint32_t tot = 0;
                const uint32_t e = block_excl_scan_256(x0 + x1, S.wsum, &tot);
                if (i0 < G) offs[(size_t)i0 * NB + d] = e;
                if (i1 < G) offs[(size_t)i1 * NB + d] = e + x0;
                if (tid == 0) totals[d] = tot;
            }
        } else {
            const uint32_t Sg = G <= 1 ? 1u : 1u << (32 - __clz(G - 1));  // power of two >= G
            const uint32_t per = 256 / Sg, grp = tid / Sg, t = tid % Sg;
            for (uint32_t d0 = tile * per; d0 < (uint32_t)NB; d0 += G * per) {
                const uint32_t d = d0 + grp;
                const bool live = d < (uint32_t)NB && t < G;
                const uint32_t x = live ? __ldcg(counts + (size_t)d * G + t) : 0u;
                uint32_t v = x, tot;
                if (Sg <= 32) {
                    for (uint32_t o = 1; o < Sg; o <<= 1) {
                        const uint32_t y = __shfl_up_sync(0xffffffffu, v, o, Sg);
                        if (t >= o) v += y;
                    }
                    tot = __shfl_sync(0xffffffffu, v, Sg - 1, Sg);
                } else {
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const uint32_t y = __shfl_up_sync(0xffffffffu, v, o);
                        if (lane >= o) v += y;
                    }
                    if (lane == 31) S.wsum[w] = v;
                    __syncthreads();
                    const int wpg = (int)(Sg / 32), w0 = w - w % wpg;
                    uint32_t pre = 0;
                    tot = 0;
                    for (int ww = w0; ww < w0 + wpg; ww++) {
                        if (ww < w) pre += S.wsum[ww];
                        tot += S.wsum[ww];
                    }
                    v += pre;
                    __syncthreads();
                }
                if (live) offs[(size_t)t * NB + d] = v - x;
                if (d < (uint32_t)NB && t == 0) totals[d] = tot;
            }
        }
        target += G;
        grid_barrier(bar, target, err);
        {
            uint32_t T[PER], tsum2 = 0;
#pragma unroll
            for (int r = 0; r < PER; r++) {
                T[r] = __ldcg(totals + tid * PER + r);
                tsum2 += T[r];
            }
            uint32_t run = block_excl_scan_256(tsum2, S.wsum, nullptr);
#pragma unroll
            for (int r = 0; r < PER; r++) {
                const int d = tid * PER + r;
                S.gbase[d] = run + __ldcg(offs + (size_t)tile * NB + d);
                run += T[r];
            }
        }
        __syncthreads();
        for (uint32_t p = tid; p < nvalid; p += SORT_TPB) {
            const uint64_t kk = S.k[p];
            const uint32_t d = (uint32_t)((kk >> sh) & (NB - 1));
            const uint32_t g = S.gbase[d] + (p - S.ldig[d]);
            if (g < n) {  // always, unless a barrier wait gave up
                ko[g] = kk;
                vo[g] = S.v[p];
            }
        }
        if (rem) {
            target += G;
            grid_barrier(bar, target, err);
        }
    }
}

// ---------------------------------------------------------------- one-CTA sort
template <typename V>
struct SmallSmem {
    uint64_t k[2][SORT_TILE];
    V v[2][SORT_TILE];
    uint32_t whist[8][256];
    uint32_t ldig[256];
    uint32_t wsum[8];
};

template <typename V>
__global__ void __launch_bounds__(SORT_TPB) k_small_sort(uint64_t *keys, V *vals, uint32_t n, SortMask mask) {
    const uint32_t byte_mask = active_bytes(mask);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SmallSmem<V> &S = *reinterpret_cast<SmallSmem<V> *>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    for (uint32_t p = tid; p < n; p += SORT_TPB) {
        S.k[0][p] = keys[p];
        S.v[0][p] = vals[p];
    }
    int cur = 0;
    for (int byte = 0; byte < 8; byte++) {
        if (!((byte_mask >> byte) & 1u)) continue;
        const int sh = byte * 8;
        for (int i = tid; i < 8 * 256; i += SORT_TPB) (&S.whist[0][0])[i] = 0;
        __syncthreads();
        uint64_t k[SORT_IPT];
        V v[SORT_IPT];
        uint32_t vmask = 0;
#pragma unroll
        for (int i = 0; i < SORT_IPT; i++) {
            uint32_t p = w * 32 * SORT_IPT + i * 32 + lane;
            if (p < n) {
                k[i] = S.k[cur][p];
                v[i] = S.v[cur][p];
                vmask |= 1u << i;
            } else {
                k[i] = ~0ull;
                v[i] = V(0);
            }
        }
        uint32_t rank[SORT_IPT];
        warp_rank<SORT_IPT>(k, vmask, sh, S.whist[w], rank);
        __syncthreads();
        uint32_t tcount = 0;
#pragma unroll
        for (int ww = 0; ww < 8; ww++) {
            uint32_t c = S.whist[ww][tid];
            S.whist[ww][tid] = tcount;
            tcount += c;
        }
        uint32_t ldig = block_excl_scan_256(tcount, S.wsum, nullptr);
        S.ldig[tid] = ldig;
        __syncthreads();
#pragma unroll
        for (int i = 0; i < SORT_IPT; i++) {
            if ((vmask >> i) & 1u) {
                uint32_t d = (uint32_t)((k[i] >> sh) & 0xFF);
                uint32_t pos = S.ldig[d] + S.whist[w][d] + rank[i];
                S.k[cur ^ 1][pos] = k[i];
                S.v[cur ^ 1][pos] = v[i];
            }
        }
        cur ^= 1;
        __syncthreads();
    }
    for (uint32_t p = tid; p < n; p += SORT_TPB) {
        keys[p] = S.k[cur][p];
        vals[p] = S.v[cur][p];
    }
}

// ---------------------------------------------------------------- one-CTA sort, 8K keys
// Keys stay in registers between passes; each pass ranks them (ballots),
// places them in shared memory at their stable position and reloads them
// in that order.  One launch and one SM for batches up to 8192 pairs, so
// that many small batches of different graphs sort side by side.
struct BlockSortSmem {
    uint64_t k[BLOCK_SORT_MAX];
    uint16_t v[BLOCK_SORT_MAX];
    uint32_t whist[BLOCK_SORT_TPB / 32][256];
    uint32_t ldig[256];
    uint32_t wsum[8];
};

// in place, keys in registers; act = the digit bytes to sort.  Every warp
// holds R = ceil(n / 1024) rounds of 32 consecutive keys (warp w the range
// [32 R w, 32 R (w + 1))), so a small batch still spreads over all 32 warps
// and each warp ranks only R rounds per pass.
__device__ __forceinline__ void block_sort_inreg(uint64_t *keys, uint16_t *vals, uint32_t n, uint32_t act) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    BlockSortSmem &S = *reinterpret_cast<BlockSortSmem *>(smem_raw);
    constexpr int IPT = BLOCK_SORT_IPT, NW = BLOCK_SORT_TPB / 32;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int R = (int)((n + BLOCK_SORT_TPB - 1) / BLOCK_SORT_TPB);  // 1..IPT
    uint64_t k[IPT];
    uint16_t v[IPT];
    uint32_t vmask = 0;
#pragma unroll
    for (int i = 0; i < IPT; i++) {
        const uint32_t p = w * 32 * R + i * 32 + lane;
        if (i < R && p < n) {
            k[i] = keys[p];
            v[i] = vals[p];
            vmask |= 1u << i;
        } else {
            k[i] = ~0ull;
            v[i] = 0;
        }
    }
    for (int byte = 0; byte < 8; byte++) {
        if (!((act >> byte) & 1u)) continue;
        const int sh = 8 * byte;
        for (int i = tid; i < NW * 256; i += BLOCK_SORT_TPB) (&S.whist[0][0])[i] = 0;
        __syncthreads();
        uint32_t rank[IPT];
        warp_rank<IPT>(k, vmask, sh, S.whist[w], rank, R);
        __syncthreads();
        // digit d (thread d < 256): warp-exclusive offsets and the tile count
        uint32_t tcount = 0;
        if (tid < 256) {
            for (int ww = 0; ww < NW; ww++) {
                const uint32_t c = S.whist[ww][tid];
                S.whist[ww][tid] = tcount;
                tcount += c;
            }
        }
        // exclusive scan of the 256 digit counts by the first eight warps
        uint32_t incl = tcount;
        if (tid < 256) {
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += y;
            }
            if (lane == 31) S.wsum[w] = incl;
        }
        __syncthreads();
        if (tid < 256) {
            uint32_t base = 0;
            for (int ww = 0; ww < w; ww++) base += S.wsum[ww];
            S.ldig[tid] = base + incl - tcount;
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < IPT; i++) {
            if ((vmask >> i) & 1u) {
                const uint32_t d = (uint32_t)((k[i] >> sh) & 0xFF);
                const uint32_t pos = S.ldig[d] + S.whist[w][d] + rank[i];
                S.k[pos] = k[i];
                S.v[pos] = v[i];
            }
        }
        __syncthreads();
#pragma unroll
        for (int i = 0; i < IPT; i++) {
            const uint32_t p = w * 32 * R + i * 32 + lane;
            if (i < R && p < n) {
                k[i] = S.k[p];
                v[i] = S.v[p];
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < IPT; i++) {
        const uint32_t p = w * 32 * R + i * 32 + lane;
        if (i < R && p < n) {
            keys[p] = k[i];
            vals[p] = v[i];
        }
    }
}

// The block tier: n <= RANK2_MAX pairs sorted by ranks, in two launches.
// Phase 1 sorts tiles of RANK_TILE pairs by all-pairs rank: the stable
// position of key i in its tile is the number of the tile's keys below it
// plus its equal keys earlier in the input.  Each CTA stages its tile in
// shared memory and ranks RANK_KEYS of its keys, RANK_SPLIT threads a key
// over interleaved slices of the tile, so a batch of 1024 keys spreads over
// 32 SMs (about 900 instructions a thread) where one CTA's digit passes
// serialise on one SM.  The ranked tiles land in (k1, v1).  Phase 2 puts
// every pair at its final position in (k0, v0): its place in its tile plus,
// for each other tile, the keys that precede it there (keys <= it in earlier
// tiles, < it in later ones: equal keys keep their input order), by binary
// searches over the whole batch staged in shared memory.  A single tile is
// copied back instead.
constexpr uint32_t RANK_TILE = 2048, RANK2_MAX = 8 * RANK_TILE, RANK_TPB = 256, RANK_SPLIT = 8,
                   RANK_KEYS = RANK_TPB / RANK_SPLIT, RANK_CPT = RANK_TILE / RANK_KEYS;

__global__ void __launch_bounds__(RANK_TPB) k_rank_tiles(const uint64_t *__restrict__ k0, const uint16_t *__restrict__ v0,
                                                         uint64_t *__restrict__ k1, uint16_t *__restrict__ v1,
                                                         uint32_t n) {
    __shared__ uint64_t sk[RANK_TILE];
    griddep_wait();
    const uint32_t tile = blockIdx.x / RANK_CPT, part_blk = blockIdx.x % RANK_CPT;
    const uint32_t off = tile * RANK_TILE;
    if (off >= n) return;
    const uint32_t len = min(RANK_TILE, n - off);
    for (uint32_t i = threadIdx.x; i < len; i += RANK_TPB) sk[i] = k0[off + i];
    __syncthreads();
    const uint32_t i = part_blk * RANK_KEYS + threadIdx.x / RANK_SPLIT, part = threadIdx.x % RANK_SPLIT;
    const uint64_t ki = i < len ? sk[i] : 0ull;
    uint32_t rank = 0;
    if (i < len)
        for (uint32_t j = part; j < len; j += RANK_SPLIT) {
            const uint64_t kj = sk[j];
            rank += (kj < ki || (kj == ki && j < i)) ? 1u : 0u;
        }
#pragma unroll
    for (uint32_t o = RANK_SPLIT / 2; o; o >>= 1) rank += __shfl_down_sync(0xffffffffu, rank, o, RANK_SPLIT);
    if (part == 0 && i < len) {
        k1[off + rank] = ki;
        v1[off + rank] = v0[off + i];
    }
}

// phase 2 of a one-tile batch: the sorted tile goes home
__global__ void __launch_bounds__(1024) k_rank_back(uint64_t *__restrict__ k0, uint16_t *__restrict__ v0,
                                                    const uint64_t *__restrict__ k1, const uint16_t *__restrict__ v1,
                                                    uint32_t n) {
    griddep_wait();
    for (uint32_t i = threadIdx.x; i < n && n <= RANK_TILE; i += 1024) {
        k0[i] = k1[i];
        v0[i] = v1[i];
    }
}

// phase 2 of a batch of several tiles (n * 8 bytes of dynamic shared memory)
__global__ void __launch_bounds__(RANK_TPB) k_rank_merge(uint64_t *__restrict__ k0, uint16_t *__restrict__ v0,
                                                         const uint64_t *__restrict__ k1,
                                                         const uint16_t *__restrict__ v1, uint32_t n) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    uint64_t *sk = reinterpret_cast<uint64_t *>(smem_raw);
    griddep_wait();
    if (n > RANK2_MAX) return;
    for (uint32_t i = threadIdx.x; i < n; i += RANK_TPB) sk[i] = k1[i];
    __syncthreads();
    const uint32_t i = blockIdx.x * RANK_TPB + threadIdx.x;
    if (i >= n) return;
    const uint64_t key = sk[i];
    const uint32_t t = i / RANK_TILE, ntiles = (n + RANK_TILE - 1) / RANK_TILE;
    uint32_t rank = i - t * RANK_TILE;
    for (uint32_t u = 0; u < ntiles; u++) {
        if (u == t) continue;
        const uint32_t a = u * RANK_TILE, len = min(RANK_TILE, n - a);
        uint32_t L = 0, R = len;  // keys of tile u that precede `key`
        while (L < R) {
            const uint32_t mid = (L + R) >> 1;
            const uint64_t x = sk[a + mid];
            if (u < t ? x <= key : x < key)
                L = mid + 1;
            else
                R = mid;
        }
        rank += L;
    }
    k0[rank] = key;
    v0[rank] = v1[i];
}

// ---------------------------------------------------------------- tile-merge sort
// A batch of 2049..TM_MAX pairs, or the batch of one graph in a batched
// update: tiles of J.tile (1024 or 2048) pairs sorted in registers, one CTA
// each, then stable merge-path rounds (runs of J.tile << r pairs merged two
// by two, FOREST_MERGE_SLICE outputs per CTA).  Round r reads (k0, p0) when
// r is even; the tile is chosen so that the round count is even, so the
// result always ends in (k0, p0).

// tile t of job J, in place
__device__ __forceinline__ void tm_tile_body(const ForestSortJob &J, uint32_t t) {
    const uint32_t off = t * J.tile;
    if (off >= J.n) return;
    const uint32_t len = J.n - off < J.tile ? J.n - off : J.tile;
    block_sort_inreg(J.k0 + off, J.p0 + off, len, active_bytes(SortMask{J.andor, 0xFFu, 0u}));
}

// merge path: how many of the first d outputs of the stable merge of A
// (a keys) and B (b keys) come from A (ties go to A)
__device__ __forceinline__ uint32_t merge_split(const uint64_t *A, uint32_t a, const uint64_t *B, uint32_t b,
                                                uint32_t d) {
    uint32_t lo = d > b ? d - b : 0, hi = d < a ? d : a;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (A[mid] <= B[d - mid - 1])
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// The same split found by one warp: each step evaluates the merge-path
// predicate at 32 evenly spaced candidates at once (one memory round trip)
// and keeps the interval between the last true and the first false, so a
// run of 2^k keys takes about k / 5 round trips instead of k.
__device__ __forceinline__ uint32_t merge_split_warp(const uint64_t *A, uint32_t a, const uint64_t *B, uint32_t b,
                                                     uint32_t d) {
    const int lane = threadIdx.x & 31;
    uint32_t lo = d > b ? d - b : 0, hi = d < a ? d : a;  // answer in [lo, hi]
    while (hi - lo > 32) {
        const uint32_t span = hi - lo;
        // candidate i = lo + span * (lane + 1) / 33, strictly inside (lo, hi)
        const uint32_t i = lo + (uint32_t)(((uint64_t)span * (uint32_t)(lane + 1)) / 33u);
        const bool p = A[i] <= B[d - i - 1];  // true: the answer is above i
        const uint32_t t = __ballot_sync(0xffffffffu, p);
        // the predicate is monotone (true then false): count the trues
        const int nt = __popc(t);
        const uint32_t new_lo = nt ? lo + (uint32_t)(((uint64_t)span * (uint32_t)nt) / 33u) + 1 : lo;
        const uint32_t new_hi = nt < 32 ? lo + (uint32_t)(((uint64_t)span * (uint32_t)(nt + 1)) / 33u) : hi;
        lo = new_lo, hi = new_hi;
    }
    // at most 32 candidates left: one more round over lo .. hi - 1
    const uint32_t i = lo + (uint32_t)lane;
    const bool p = i < hi && A[i] <= B[d - i - 1];
    return lo + (uint32_t)__popc(__ballot_sync(0xffffffffu, p));
}

constexpr int MERGE_TPB = 256, MERGE_IPT = FOREST_MERGE_SLICE / MERGE_TPB;

// merge round r of job J, output slice c (FOREST_MERGE_SLICE outputs)
__device__ __forceinline__ void tm_merge_body(const ForestSortJob &J, uint32_t round, uint32_t c) {
    __shared__ uint64_t sk[FOREST_MERGE_SLICE];
    __shared__ uint16_t sv[FOREST_MERGE_SLICE];
    __shared__ uint32_t split[2];
    const uint64_t *__restrict__ ks = (round & 1) ? J.k1 : J.k0;
    const uint16_t *__restrict__ vs = (round & 1) ? J.p1 : J.p0;
    uint64_t *__restrict__ kd = (round & 1) ? J.k0 : J.k1;
    uint16_t *__restrict__ vd = (round & 1) ? J.p0 : J.p1;
    const uint32_t n = J.n, L = J.tile << round;
    const uint32_t o0 = c * FOREST_MERGE_SLICE;
    if (o0 >= n) return;
    const uint32_t base = o0 / (2 * L) * (2 * L);
    const uint32_t a = n - base < L ? n - base : L;
    const uint32_t b = n - base > L ? (n - base - L < L ? n - base - L : L) : 0;
    const uint64_t *A = ks + base, *B = A + a;  // b > 0 only when a == L
    const uint32_t d0 = o0 - base, d1 = d0 + FOREST_MERGE_SLICE < a + b ? d0 + FOREST_MERGE_SLICE : a + b;
    if (threadIdx.x < 64) {  // warp 0: the slice's start, warp 1: its end
        const uint32_t r = merge_split_warp(A, a, B, b, threadIdx.x < 32 ? d0 : d1);
        if ((threadIdx.x & 31) == 0) split[threadIdx.x >> 5] = r;
    }
    __syncthreads();
    const uint32_t i0 = split[0], i1 = split[1], j0 = d0 - i0;
    const uint32_t na = i1 - i0, nt = d1 - d0;  // nt <= FOREST_MERGE_SLICE
    for (uint32_t t = threadIdx.x; t < nt; t += MERGE_TPB) {
        const uint32_t src = t < na ? base + i0 + t : base + a + j0 + (t - na);
        sk[t] = ks[src];
        sv[t] = vs[src];
    }
    __syncthreads();
    const uint32_t nb = nt - na;
    const uint32_t q0 = threadIdx.x * MERGE_IPT < nt ? threadIdx.x * MERGE_IPT : nt;
    uint32_t i = merge_split(sk, na, sk + na, nb, q0), j = q0 - i;
    uint64_t ok[MERGE_IPT];
    uint16_t ov[MERGE_IPT];
#pragma unroll
    for (int q = 0; q < MERGE_IPT; q++) {
        if (q0 + q < nt) {
            const bool take_a = j >= nb || (i < na && sk[i] <= sk[na + j]);
            const uint32_t p = take_a ? i++ : na + j++;
            ok[q] = sk[p];
            ov[q] = sv[p];
        }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < MERGE_IPT; q++)
        if (q0 + q < nt) sk[q0 + q] = ok[q], sv[q0 + q] = ov[q];
    __syncthreads();
    for (uint32_t t = threadIdx.x; t < nt; t += MERGE_TPB) {
        kd[o0 + t] = sk[t];
        vd[o0 + t] = sv[t];
    }
}

// one batch: CTA per tile / per output slice
__global__ void __launch_bounds__(BLOCK_SORT_TPB, 1) k_tm_tiles(ForestSortJob J) {
    griddep_wait();
    tm_tile_body(J, blockIdx.x);
}

__global__ void __launch_bounds__(MERGE_TPB) k_tm_merge(ForestSortJob J, uint32_t round) {
    griddep_wait();
    tm_merge_body(J, round, blockIdx.x);
}

// many graphs' batches: a block finds its job in the launch's offset table
__global__ void __launch_bounds__(BLOCK_SORT_TPB, 1) k_forest_tile_sort(const ForestSortJob *__restrict__ jobs,
                                                                         const uint32_t *__restrict__ boff,
                                                                         uint32_t G) {
    const uint32_t g = forest_job_of(boff, G, blockIdx.x);
    const ForestSortJob J = jobs[g];
    tm_tile_body(J, blockIdx.x - boff[g]);
}

__global__ void __launch_bounds__(MERGE_TPB) k_forest_merge(const ForestSortJob *__restrict__ jobs,
                                                            const uint32_t *__restrict__ boff, uint32_t G,
                                                            uint32_t round) {
    const uint32_t g = forest_job_of(boff, G, blockIdx.x);
    const ForestSortJob J = jobs[g];
    tm_merge_body(J, round, blockIdx.x - boff[g]);
}

// ---------------------------------------------------------------- scans
constexpr int SCAN_TPB = 256, SCAN_IPT = 8, SCAN_TILE = SCAN_TPB * SCAN_IPT;

template <typename T>
__global__ void __launch_bounds__(SCAN_TPB) k_scan_reduce(const T *__restrict__ in, uint32_t n, uint32_t *tmp) {
    __shared__ uint32_t wsum[8];
    uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < SCAN_IPT; i++) {
        uint64_t p = base + (uint64_t)i * SCAN_TPB + threadIdx.x;
        if (p < n) s += (uint32_t)in[p];
    }
    uint32_t tot;
    block_excl_scan_256(s, wsum, &tot);
    if (threadIdx.x == 0) tmp[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(1024) k_scan_top(uint32_t *tmp, uint32_t nb, uint32_t *total) {
    __shared__ uint32_t ws[32];
    __shared__ uint32_t carry;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint32_t b0 = 0; b0 < nb; b0 += 1024) {
        uint32_t i = b0 + threadIdx.x;
        uint32_t x = i < nb ? tmp[i] : 0, v = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += y;
        }
        if (lane == 31) ws[w] = v;
        __syncthreads();
        if (w == 0) {
            uint32_t s = ws[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
                if (lane >= o) s += y;
            }
            ws[lane] = s;
        }
        __syncthreads();
        uint32_t excl = carry + (w ? ws[w - 1] : 0) + v - x;
        if (i < nb) tmp[i] = excl;
        __syncthreads();
        if (threadIdx.x == 0) carry += ws[31];
        __syncthreads();
    }
    if (threadIdx.x == 0 && total) *total = carry;
}

// Warp w of a block scans elements [tile + 256 w, tile + 256 w + 256) as 8
// rows of 32 (lane l holds element 32 i + l of row i): each row is a shuffle
// scan carried into the next, so every load and store instruction of a warp
// covers consecutive elements (one 128-byte line of u32 output).
template <typename T>
__global__ void __launch_bounds__(SCAN_TPB) k_scan_down(const T *__restrict__ in, uint32_t *out, uint32_t n,
                                                       const uint32_t *tmp, uint32_t *total_single) {
    __shared__ uint32_t wsum[SCAN_TPB / 32];
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE + (uint64_t)w * (32 * SCAN_IPT) + lane;
    uint32_t x[SCAN_IPT];
#pragma unroll
    for (int i = 0; i < SCAN_IPT; i++) {
        const uint64_t p = base + 32 * i;
        x[i] = p < n ? (uint32_t)in[p] : 0u;
    }
    uint32_t run = 0;  // the warp's elements before row i
#pragma unroll
    for (int i = 0; i < SCAN_IPT; i++) {
        uint32_t v = x[i];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= (uint32_t)o) v += y;
        }
        const uint32_t row = __shfl_sync(0xffffffffu, v, 31);
        x[i] = run + v - x[i];  // exclusive, within the warp
        run += row;
    }
    if (lane == 0) wsum[w] = run;
    __syncthreads();
    uint32_t woff = 0, tot = 0;
#pragma unroll
    for (uint32_t k = 0; k < SCAN_TPB / 32; k++) {
        const uint32_t y = wsum[k];
        woff += k < w ? y : 0u;
        tot += y;
    }
    const uint32_t off = woff + (tmp ? tmp[blockIdx.x] : 0u);
#pragma unroll
    for (int i = 0; i < SCAN_IPT; i++) {
        const uint64_t p = base + 32 * i;
        if (p < n) out[p] = off + x[i];
    }
    if (total_single && threadIdx.x == 0) *total_single = tot;
}

template <typename T>
cudaError_t scan_impl(const T *in, uint32_t *out, uint32_t n, uint32_t *total, uint32_t *tmp, cudaStream_t st) {
    if (n == 0) {
        if (total) return cudaMemsetAsync(total, 0, 4, st);
        return cudaSuccess;
    }
    uint32_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    ProfScope ps("scan", st);
    if (nb == 1) {
        k_scan_down<T><<<1, SCAN_TPB, 0, st>>>(in, out, n, nullptr, total);
        note_launch();
        return cudaGetLastError();
    }
    k_scan_reduce<T><<<nb, SCAN_TPB, 0, st>>>(in, n, tmp);
    k_scan_top<<<1, 1024, 0, st>>>(tmp, nb, total);
    k_scan_down<T><<<nb, SCAN_TPB, 0, st>>>(in, out, n, tmp, nullptr);
    note_launch(3);
    return cudaGetLastError();
}

}  // namespace

size_t scan_tmp_words(uint32_t n) { return (n + SCAN_TILE - 1) / SCAN_TILE + 1; }

cudaError_t scan_u32(const uint32_t *in, uint32_t *out, uint32_t n, uint32_t *total, uint32_t *tmp,
                     cudaStream_t st) {
    return scan_impl<uint32_t>(in, out, n, total, tmp, st);
}
cudaError_t scan_u8_to_u32(const uint8_t *in, uint32_t *out, uint32_t n, uint32_t *total, uint32_t *tmp,
                           cudaStream_t st) {
    return scan_impl<uint8_t>(in, out, n, total, tmp, st);
}

// Per device: resident CTAs of k_coop_sort<u16/u32/u64, 8-bit digits> and
// of k_coop_sort<u16, 9-bit digits>, measured by sort_prepare with the
// device current (the shared-memory opt-ins it sets are per device too).
struct CoopCtas {
    uint32_t n[4];
};
PerDevice<CoopCtas> g_sort_setup;

// the current device's figure for one slot; 0 before sort_prepare ran on it
static uint32_t coop_max_ctas(int slot) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    const CoopCtas *c = g_sort_setup.peek(dev);
    return c ? c->n[slot] : 0u;
}

template <typename V>
constexpr int coop_slot(bool wide) {
    return wide ? 3 : (sizeof(V) == 2 ? 0 : (sizeof(V) == 4 ? 1 : 2));
}

// cooperative-sort geometry for n keys: tiles of at least COOP_MIN_TILE
// keys, spread over every resident CTA slot so that the SMs carry equal work
// (wide: 9-bit digits, 16-bit payloads only)
template <typename V>
static bool coop_geometry(uint32_t n, const SortScratch &s, uint32_t *tile_len_out, uint32_t *G_out,
                          bool wide = false) {
    if (wide && sizeof(V) != 2) return false;
    const uint32_t mc = coop_max_ctas(coop_slot<V>(wide));
    const uint32_t maxG = mc < 512u ? mc : 512u;
    const uint32_t tile_len = maxG ? std::max<uint32_t>(COOP_MIN_TILE, (n + maxG - 1) / maxG) : 0u;
    const uint32_t G = tile_len ? (n + tile_len - 1) / tile_len : 0u;
    const size_t nb = wide ? 512 : 256;
    *tile_len_out = tile_len;
    *G_out = G;
    return s.bar && n > (uint32_t)SORT_TILE && tile_len && tile_len <= (uint32_t)COOP_TILE && G <= maxG &&
           s.status_words >= 2 * nb * (size_t)G + nb;
}

template <typename V>
static bool tier_ok(SortTier t, uint32_t n, const SortScratch &s) {
    uint32_t tl, G;
    switch (t) {
        case TIER_SMALL: return n <= (uint32_t)SORT_TILE;
        case TIER_BLOCK: return sizeof(V) == 2 && n <= RANK2_MAX;
        case TIER_TILE_MERGE: return sizeof(V) == 2 && n <= (1u << 24);
        case TIER_COOP: return coop_geometry<V>(n, s, &tl, &G);
        case TIER_MULTIPASS:
            return n > (uint32_t)SORT_TILE &&
                   s.status_words >= 2 * (size_t)((n + SORT_TILE - 1) / SORT_TILE) * 256;
        default: return false;
    }
}

// the measured cutovers of this build (used until a tuning run says otherwise)
template <typename V>
static SortTier tier_default(uint32_t n, const SortScratch &s) {
    if (sizeof(V) == 2 && n <= RANK2_MAX) return TIER_BLOCK;
    if (sizeof(V) == 2 && n > TM_TILE_MAX && n <= TM_MAX) return TIER_TILE_MERGE;
    if (tier_ok<V>(TIER_COOP, n, s)) return TIER_COOP;
    if (n <= (uint32_t)SORT_TILE) return TIER_SMALL;
    // without a cooperative launch (concurrent handles) the merge rounds beat
    // three launches per digit pass up to 2^19 keys (measured: 113 against
    // 148 us at 2^19, 226 against 187 at 2^20)
    if (n <= (1u << 19) && tier_ok<V>(TIER_TILE_MERGE, n, s)) return TIER_TILE_MERGE;
    return TIER_MULTIPASS;
}

// tuned tier per (sort mode, ceil(log2 n)) for 16-bit payloads; 0 = none
static std::atomic<uint8_t> g_tier_table[2][33];

static uint32_t log2_bucket(uint32_t n) { return n <= 1 ? 0u : 32u - (uint32_t)__builtin_clz(n - 1); }

template <typename V>
static cudaError_t sort_impl(uint64_t *k0, V *v0, uint64_t *k1, V *v1, uint32_t n, SortMask mask, SortScratch &s,
                             cudaStream_t st, SortTier tier) {
    if (n < 2 || mask.host_mask == 0) return cudaSuccess;
    cudaError_t e;
    if (tier == TIER_AUTO || !tier_ok<V>(tier, n, s)) tier = tier_default<V>(n, s);
    if (tier == TIER_TILE_MERGE) {
        // the round count is even: the result ends in (k0, v0)
        const ForestSortJob J{k0, k1, reinterpret_cast<uint16_t *>(v0), reinterpret_cast<uint16_t *>(v1), mask.andor,
                              n, tm_tile(n)};
        {
            ProfScope ps("sort_tiles", st);
            launch_pdl(k_tm_tiles, dim3((n + J.tile - 1) / J.tile), dim3(BLOCK_SORT_TPB), sizeof(BlockSortSmem), st, J);
            note_launch();
        }
        const uint32_t rounds = tm_rounds(n);
        for (uint32_t r = 0; r < rounds; r++) {
            ProfScope ps("sort_merge", st);
            launch_pdl(k_tm_merge, dim3(forest_merge_ctas(n)), dim3(MERGE_TPB), 0, st, J, r);
            note_launch();
        }
        return cudaGetLastError();
    }
    if (tier == TIER_BLOCK) {
        if (sizeof(V) != 2 || n > RANK2_MAX) return cudaErrorInvalidValue;
        ProfScope ps("sort_block", st);
        uint16_t *p0 = reinterpret_cast<uint16_t *>(v0), *p1 = reinterpret_cast<uint16_t *>(v1);
        const uint32_t ntiles = (n + RANK_TILE - 1) / RANK_TILE;
        if (mask.pingpong == 2u && ntiles > 1) return cudaErrorInvalidValue;
        launch_pdl(k_rank_tiles, dim3((ntiles - 1) * RANK_CPT + (n - (ntiles - 1) * RANK_TILE + RANK_KEYS - 1) / RANK_KEYS),
                   dim3(RANK_TPB), 0, st, k0, p0, k1, p1, n);
        if (ntiles > 1)
            launch_pdl(k_rank_merge, dim3((n + RANK_TPB - 1) / RANK_TPB), dim3(RANK_TPB), (size_t)n * 8, st, k0, p0, k1,
                       p1, n);
        else if (mask.pingpong != 2u)  // the caller reads the tile where it is when pingpong is 2
            launch_pdl(k_rank_back, dim3(1), dim3(1024), 0, st, k0, p0, k1, p1, n);
        note_launch(ntiles > 1 || mask.pingpong != 2u ? 2 : 1);
        return cudaGetLastError();
    }
    // the 9-bit digit plan belongs to the cooperative sort alone: the
    // consumers of the result compute its parity from the same mask
    if (mask.wide && (tier != TIER_COOP || sizeof(V) != 2)) return cudaErrorInvalidValue;
    if (tier == TIER_COOP) {
        const bool wide = mask.wide != 0;
        uint32_t tile_len, G;
        if (!coop_geometry<V>(n, s, &tile_len, &G, wide)) return cudaErrorInvalidValue;
        if (!s.bar_cleared && (e = cudaMemsetAsync(s.bar, 0, sizeof(uint32_t), st))) return e;
        const size_t nb = wide ? 512 : 256;
        uint32_t *counts = s.status, *offs = s.status + nb * G, *totals = s.status + 2 * nb * G;
        uint32_t *bar = s.bar, *err = s.err;
        uint32_t tl = tile_len;
        void *args[] = {&k0, &v0, &k1, &v1, &n, &tl, &mask, &counts, &offs, &totals, &bar, &err};
        ProfScope ps("sort_coop", st);
        // cooperative, and a programmatic dependent of the kernel before it
        // (the sort waits for it with griddepcontrol.wait)
        cudaLaunchAttribute attr[2];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[1].val.programmaticStreamSerializationAllowed = 1;
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = dim3(G);
        cfg.blockDim = dim3(SORT_TPB);
        cfg.stream = st;
        cfg.attrs = attr;
        cfg.numAttrs = 2;
        const void *fn = (const void *)k_coop_sort<V, 8>;
        cfg.dynamicSmemBytes = sizeof(CoopSmem<V, 256>);
        if constexpr (sizeof(V) == 2) {
            if (wide) {
                fn = (const void *)k_coop_sort<V, WIDE_DIGIT_BITS>;
                cfg.dynamicSmemBytes = sizeof(CoopSmem<V, 512>);
            }
        }
        e = cudaLaunchKernelExC(&cfg, fn, args);
        note_launch();
        return e;
    }
    if (tier == TIER_SMALL) {
        const size_t sm = sizeof(SmallSmem<V>);
        ProfScope ps("sort_small", st);
        k_small_sort<V><<<1, SORT_TPB, sm, st>>>(k0, v0, n, mask);
        note_launch();
        return cudaGetLastError();
    }
    const uint32_t tiles = (n + SORT_TILE - 1) / SORT_TILE;
    if (s.status_words < 2 * (size_t)tiles * 256) return cudaErrorInvalidValue;
    uint32_t *counts = s.status, *offs = s.status + (size_t)tiles * 256;
    if ((e = cudaMemsetAsync(s.hist, 0, 8 * 256 * sizeof(uint32_t), st))) return e;
    const uint32_t hb = tiles < 1024 ? tiles : 1024;
    {
        ProfScope ps("sort_hist", st);
        k_hist<<<hb, 256, 0, st>>>(k0, n, s.hist);
    }
    note_launch();
    const size_t sm = sizeof(PassSmem<V>);
    for (int b = 0; b < 8; b++) {
        if (!((mask.host_mask >> b) & 1u)) continue;
        {
            ProfScope ps("sort_upsweep", st);
            k_upsweep<<<tiles, SORT_TPB, 0, st>>>(k0, k1, n, b, mask, counts, tiles);
        }
        {
            ProfScope ps("sort_dscan", st);
            k_dscan<<<32, 256, 0, st>>>(counts, tiles, s.hist + 256 * b, offs, b, mask);
        }
        {
            ProfScope ps("sort_downsweep", st);
            k_downsweep<V><<<tiles, SORT_TPB, sm, st>>>(k0, v0, k1, v1, n, b, mask, offs, tiles);
        }
        note_launch(3);
    }
    return cudaGetLastError();
}

cudaError_t forest_sort(const ForestSortJob *d_jobs, uint32_t G, const uint32_t *d_boff, const uint32_t *nblk,
                        uint32_t rounds, cudaStream_t st) {
    if (!G) return cudaSuccess;
    cudaError_t e = sort_prepare();
    if (e != cudaSuccess) return e;
    {
        ProfScope ps("forest_tile_sort", st);
        if (nblk[0]) k_forest_tile_sort<<<nblk[0], BLOCK_SORT_TPB, sizeof(BlockSortSmem), st>>>(d_jobs, d_boff, G);
        note_launch();
    }
    for (uint32_t r = 0; r < rounds; r++) {
        if (!nblk[1 + r]) continue;
        ProfScope ps("forest_merge", st);
        k_forest_merge<<<nblk[1 + r], MERGE_TPB, 0, st>>>(d_jobs, d_boff + (size_t)(1 + r) * (G + 1), G, r);
        note_launch();
    }
    return cudaGetLastError();
}

uint32_t coop_sort_max_keys() {
    const uint32_t mc = coop_max_ctas(0);
    const uint32_t g = mc < 512u ? mc : 512u;
    return g * (uint32_t)COOP_TILE;
}

// Shared-memory opt-ins of the sort kernels and the cooperative sort's
// occupancy, set once per device (with that device current) outside any
// stream capture.  cudaFuncSetAttribute applies to the current device only,
// so a process that uses several devices runs this on each.
static cudaError_t sort_setup_device(int dev, CoopCtas &out) {
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(k_small_sort<uint16_t>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)sizeof(SmallSmem<uint16_t>))))
        return e;
    if ((e = cudaFuncSetAttribute(k_small_sort<uint64_t>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)sizeof(SmallSmem<uint64_t>))))
        return e;
    if ((e = cudaFuncSetAttribute(k_downsweep<uint16_t>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)sizeof(PassSmem<uint16_t>))))
        return e;
    if ((e = cudaFuncSetAttribute(k_downsweep<uint64_t>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)sizeof(PassSmem<uint64_t>))))
        return e;
    if ((e = cudaFuncSetAttribute(k_rank_merge, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)(RANK2_MAX * sizeof(uint64_t)))) ||
        (e = cudaFuncSetAttribute(k_forest_tile_sort, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)sizeof(BlockSortSmem))) ||
        (e = cudaFuncSetAttribute(k_tm_tiles, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)sizeof(BlockSortSmem))))
        return e;
    {
        int sms = 0, per[4] = {0, 0, 0, 0};
        if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev))) return e;
        if ((e = cudaFuncSetAttribute(k_coop_sort<uint16_t, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)sizeof(CoopSmem<uint16_t, 256>))) ||
            (e = cudaFuncSetAttribute(k_coop_sort<uint32_t, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)sizeof(CoopSmem<uint32_t, 256>))) ||
            (e = cudaFuncSetAttribute(k_coop_sort<uint64_t, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)sizeof(CoopSmem<uint64_t, 256>))) ||
            (e = cudaFuncSetAttribute(k_coop_sort<uint16_t, WIDE_DIGIT_BITS>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(CoopSmem<uint16_t, 512>))))
            return e;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per[0], k_coop_sort<uint16_t, 8>, SORT_TPB,
                                                               sizeof(CoopSmem<uint16_t, 256>))) ||
            (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per[1], k_coop_sort<uint32_t, 8>, SORT_TPB,
                                                               sizeof(CoopSmem<uint32_t, 256>))) ||
            (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per[2], k_coop_sort<uint64_t, 8>, SORT_TPB,
                                                               sizeof(CoopSmem<uint64_t, 256>))) ||
            (e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per[3], k_coop_sort<uint16_t, WIDE_DIGIT_BITS>,
                                                               SORT_TPB, sizeof(CoopSmem<uint16_t, 512>))))
            return e;
        for (int i = 0; i < 4; i++) out.n[i] = (uint32_t)(per[i] * sms);
    }
    return cudaSuccess;
}

cudaError_t set_barrier_debug(uint32_t poll_limit, uint32_t unreachable) {
    cudaError_t e = cudaMemcpyToSymbol(g_bar_poll_limit, &poll_limit, sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_bar_unreachable, &unreachable, sizeof(uint32_t));
    return e;
}

cudaError_t sort_prepare() {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    return (cudaError_t)g_sort_setup.get(
        dev, [](int d, CoopCtas &v) { return (int)sort_setup_device(d, v); }, nullptr, (int)cudaErrorInvalidDevice);
}

template <typename V>
cudaError_t sort_pairs(uint64_t *k0, V *v0, uint64_t *k1, V *v1, uint32_t n, uint64_t diff_bits, SortScratch &s,
                       uint32_t *err, cudaStream_t st, int *which) {
    (void)err;
    uint32_t byte_mask = 0;
    for (int b = 0; b < 8; b++)
        if ((diff_bits >> (8 * b)) & 0xFF) byte_mask |= 1u << b;
    cudaError_t e = sort_prepare();
    if (e != cudaSuccess) return e;
    const SortTier t = tier_default<V>(n, s);
    *which = (n >= 2 && !sort_tier_in_place(t)) ? (__builtin_popcount(byte_mask) & 1) : 0;
    return sort_impl<V>(k0, v0, k1, v1, n, SortMask{nullptr, byte_mask, 0u}, s, st, t);
}

SortTier sort_tier_for_update(uint32_t n, const SortScratch &s) {
    const uint32_t t = g_tier_table[s.bar ? 1 : 0][log2_bucket(n)].load(std::memory_order_relaxed);
    if (t && tier_ok<uint16_t>((SortTier)t, n, s)) return (SortTier)t;
    return tier_default<uint16_t>(n, s);
}

bool sort_tier_usable(SortTier t, uint32_t n, const SortScratch &s) { return tier_ok<uint16_t>(t, n, s); }

SortMask update_sort_mask(const unsigned long long *andor, SortTier t, uint32_t n, const SortScratch &s) {
    uint32_t tl, G;
    const bool wide = t == TIER_COOP && coop_geometry<uint16_t>(n, s, &tl, &G, true);
    const uint32_t pp = t == TIER_BLOCK && n <= RANK_TILE ? 2u : sort_tier_in_place(t) ? 0u : 1u;
    return SortMask{andor, 0xFFu, pp, wide ? 1u : 0u};
}

void sort_tier_set(uint32_t bucket, int concurrent, SortTier t) {
    if (bucket < 33) g_tier_table[concurrent ? 0 : 1][bucket].store((uint8_t)t, std::memory_order_relaxed);
}

SortTier sort_tier_get(uint32_t bucket, int concurrent) {
    return bucket < 33 ? (SortTier)g_tier_table[concurrent ? 0 : 1][bucket].load(std::memory_order_relaxed) : TIER_AUTO;
}

template <typename V>
cudaError_t sort_pairs_dev(uint64_t *k0, V *v0, uint64_t *k1, V *v1, uint32_t n, SortMask mask, SortScratch &s,
                           cudaStream_t st, SortTier tier) {
    return sort_impl<V>(k0, v0, k1, v1, n, mask, s, st, tier);
}

template cudaError_t sort_pairs_dev<uint16_t>(uint64_t *, uint16_t *, uint64_t *, uint16_t *, uint32_t, SortMask,
                                              SortScratch &, cudaStream_t, SortTier);
template cudaError_t sort_pairs<uint16_t>(uint64_t *, uint16_t *, uint64_t *, uint16_t *, uint32_t, uint64_t,
                                          SortScratch &, uint32_t *, cudaStream_t, int *);
template cudaError_t sort_pairs<uint64_t>(uint64_t *, uint64_t *, uint64_t *, uint64_t *, uint32_t, uint64_t,
                                          SortScratch &, uint32_t *, cudaStream_t, int *);
template cudaError_t sort_pairs<uint32_t>(uint64_t *, uint32_t *, uint64_t *, uint32_t *, uint32_t, uint64_t,
                                          SortScratch &, uint32_t *, cudaStream_t, int *);

}  // namespace lpma
