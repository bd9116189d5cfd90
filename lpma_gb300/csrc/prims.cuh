// Device-wide primitives of the engine: LSD radix sort of (u64 key, payload)
// pairs and exclusive scans.  Hand-written for sm_103a; no CUB/Thrust.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace lpma {

constexpr int SORT_TPB = 256;
constexpr int SORT_IPT = 8;
constexpr int SORT_TILE = SORT_TPB * SORT_IPT;  // 2048 keys per tile

struct SortScratch {
    uint32_t *hist = nullptr;      // 8 x 256 global digit counts
    uint32_t *status = nullptr;    // (digit, tile) counts and offsets of one pass
    uint32_t *counters = nullptr;  // unused by the reduce-then-scan passes
    size_t status_words = 0;
    // Set both to sort batches of up to coop_sort_max_keys() keys in one
    // cooperative launch: bar is a barrier counter word (cleared by the
    // sort), err receives ERR_TIMEOUT if a bounded barrier wait gives up.
    uint32_t *bar = nullptr;
    uint32_t *err = nullptr;
    // the caller's previous kernel on the stream cleared *bar (no memset
    // before the cooperative launch)
    bool bar_cleared = false;
};

// Digit bytes to sort: host_mask, intersected (when andor is set) with the
// bytes where the device words andor[0] (AND of all keys) and andor[1] (OR
// of all keys) differ.
// pingpong: the sort that produced the batch is a ping-pong one (one
// buffer swap per digit pass), so its result is in the second buffer pair
// when the number of digit passes is odd; 0: the result is in place; 2: the
// result is in the second buffer pair (the rank sort of a single tile,
// which then skips the copy back).
// wide: the cooperative sort's 9-bit digits (set only with andor and
// host_mask 0xFF): digit windows of up to 9 bits placed greedily over the
// bits where the keys differ, instead of one pass per differing byte.
struct SortMask {
    const unsigned long long *andor;
    uint32_t host_mask;
    uint32_t pingpong;
    uint32_t wide;
};

// The sort algorithms ("tiers") of a batch sort.  All give the same stable
// order; they differ in speed per batch size and in where the result lands.
enum SortTier : uint32_t {
    TIER_AUTO = 0,        // the tuned choice, else the default cutovers
    TIER_SMALL = 1,       // one CTA through shared memory, <= 2048 keys, in place
    TIER_BLOCK = 2,       // ranks: tiles of 2048 by all-pairs rank, then merged by binary searches, <= 16384 keys, in place
    TIER_TILE_MERGE = 3,  // register-sorted tiles + merge-path rounds, <= 2^24 keys, in place
    TIER_COOP = 4,        // one cooperative launch, all digit passes, ping-pong
    TIER_MULTIPASS = 5,   // three launches per digit pass, ping-pong
    TIER_COUNT = 6
};
inline __host__ __device__ bool sort_tier_in_place(SortTier t) {
    return t == TIER_SMALL || t == TIER_BLOCK || t == TIER_TILE_MERGE;
}
// The tier the update front sorts a batch of n 16-bit-payload pairs with:
// the tuned table's entry for ceil(log2 n) and the scratch's mode
// (cooperative or concurrent), when set and usable, else the default.
SortTier sort_tier_for_update(uint32_t n, const SortScratch &s);
bool sort_tier_usable(SortTier t, uint32_t n, const SortScratch &s);
// The mask of an update batch sorted with tier t: digits from the device
// words andor (AND, OR of the keys), ping-pong parity for the ping-pong
// tiers, 9-bit digits for the cooperative tier when its scratch allows.
SortMask update_sort_mask(const unsigned long long *andor, SortTier t, uint32_t n, const SortScratch &s);
void sort_tier_set(uint32_t bucket, int concurrent, SortTier t);
SortTier sort_tier_get(uint32_t bucket, int concurrent);

// Which digit bytes a sort pass must handle: either fixed by the host, or
// read from the device (bytes where the keys' AND and OR differ, restricted
// to the host mask) so that no host round trip is needed before the sort.
__device__ inline uint32_t active_bytes(SortMask m) {
    if (!m.andor) return m.host_mask;
    const uint64_t d = m.andor[0] ^ m.andor[1];
    uint32_t r = 0;
#pragma unroll
    for (int b = 0; b < 8; b++)
        if ((d >> (8 * b)) & 0xFF) r |= 1u << b;
    return r & m.host_mask;
}

// One CTA of BLOCK_SORT_TPB threads sorts up to BLOCK_SORT_MAX (key, u16
// payload) pairs in shared memory, in place: the tiles of the tile-merge
// sort and of a batched update's sort.
constexpr int BLOCK_SORT_TPB = 1024, BLOCK_SORT_IPT = 8;
constexpr int BLOCK_SORT_MAX = BLOCK_SORT_TPB * BLOCK_SORT_IPT;  // 8192


// The digit passes of a sort.  The bits to cover: byte digits cover the
// active bytes, wide digits the bits where the keys differ.  A pass takes
// the window of W bits (8, or 9 when wide) that starts at the lowest bit
// still to cover; sort_digit_next returns that shift and removes the window
// from rem.  With byte digits this is one pass per active byte.
constexpr int WIDE_DIGIT_BITS = 9;
__device__ inline uint64_t sort_digit_bits(SortMask m) {
    if (m.wide && m.andor) return m.andor[0] ^ m.andor[1];
    const uint32_t act = active_bytes(m);
    uint64_t r = 0;
#pragma unroll
    for (int b = 0; b < 8; b++)
        if ((act >> b) & 1u) r |= 0xFFull << (8 * b);
    return r;
}
__device__ __forceinline__ int sort_digit_next(uint64_t &rem, int W) {
    const int sh = __ffsll((long long)rem) - 1;
    rem = sh + W >= 64 ? 0ull : (rem >> (sh + W)) << (sh + W);
    return sh;
}
__device__ inline uint32_t sort_digit_passes(SortMask m) {
    uint64_t rem = sort_digit_bits(m);
    const int W = m.wide ? WIDE_DIGIT_BITS : 8;
    uint32_t np = 0;
    for (; rem; np++) sort_digit_next(rem, W);
    return np;
}

// true when sort_pairs_dev<uint16_t> left its result in the second buffer pair
__device__ inline bool sort_result_odd(SortMask m, uint32_t n) {
    return n >= 2 && (m.pingpong == 2u || (m.pingpong == 1u && (sort_digit_passes(m) & 1)));
}

// Device-decided variant, sorted with `tier` (TIER_AUTO: the tuned or
// default choice): an in-place tier leaves the result in (k0, v0); a
// ping-pong tier leaves it in (k1, v1) when the number of active bytes is
// odd.  The caller sets mask.pingpong to match (sort_tier_in_place), and
// kernels that consume the result compute the same parity
// (sort_result_odd).
template <typename V>
cudaError_t sort_pairs_dev(uint64_t *k0, V *v0, uint64_t *k1, V *v1, uint32_t n, SortMask mask, SortScratch &s,
                           cudaStream_t st, SortTier tier);

// Sorts n pairs by key (stable).  Only the bytes set in diff_bits are sorted
// (bytes equal across all keys need no pass).  The result lands either in
// (k0, v0) or in (k1, v1); *which receives 0 or 1.  err is kept for the
// interface (no kernel of the sort waits on another CTA).
template <typename V>
cudaError_t sort_pairs(uint64_t *k0, V *v0, uint64_t *k1, V *v1, uint32_t n, uint64_t diff_bits,
                       SortScratch &s, uint32_t *err, cudaStream_t st, int *which);

// Status words needed for n keys: per-pass (digit, tile) counts and
// offsets of the reduce-then-scan passes (tiles of SORT_TILE keys), or of
// the cooperative sort (tiles of at least COOP_MIN_TILE keys, plus 256
// digit totals), whichever is larger.
constexpr int COOP_MIN_TILE = 1024;
constexpr size_t sort_status_words(uint32_t n) {
    return (2 * (((size_t)n + SORT_TILE - 1) / SORT_TILE) * 256 + 2) >
                   (512 * (((size_t)n + COOP_MIN_TILE - 1) / COOP_MIN_TILE) + 256)
               ? (2 * (((size_t)n + SORT_TILE - 1) / SORT_TILE) * 256 + 2)
               : (512 * (((size_t)n + COOP_MIN_TILE - 1) / COOP_MIN_TILE) + 256);
}
// The same with room for the cooperative sort's 9-bit digits (512 counts
// and 512 offsets per tile, plus 512 digit totals): the scratch of the
// update front.
constexpr size_t sort_status_words_wide(uint32_t n) {
    return sort_status_words(n) > 1024 * (((size_t)n + COOP_MIN_TILE - 1) / COOP_MIN_TILE) + 512
               ? sort_status_words(n)
               : 1024 * (((size_t)n + COOP_MIN_TILE - 1) / COOP_MIN_TILE) + 512;
}

// One-time kernel attribute setup (outside stream capture).
cudaError_t sort_prepare();

// Test setting of the cooperative sort's grid barrier on the current device
// (poll_limit 0: the default limit; unreachable: every wait gives up).
cudaError_t set_barrier_debug(uint32_t poll_limit, uint32_t unreachable);

// Tile-merge sort of 16-bit-payload pairs: batches of TM_TILE_MAX + 1 ..
// TM_MAX pairs on their own, and the batch of each graph of a batched
// update (lpma_update_batch, any size up to FOREST_SORT_MAX).  The batch is
// cut into tiles of 1024 or 2048 pairs, whichever makes the number of merge
// rounds even; one launch sorts every tile in registers, one CTA per tile,
// over the digit bytes where andor[0] (AND) and andor[1] (OR) of the batch
// differ.  Then rounds of stable merge-path merges join runs pairwise, one
// launch per round, FOREST_MERGE_SLICE outputs per CTA.  Round r reads
// (k0, p0) when r is even and (k1, p1) when odd, so with an even round
// count the result is in (k0, p0), as after an in-place sort.
constexpr uint32_t TM_TILE_MAX = 2048;  // up to here one CTA sorts the whole batch
constexpr uint32_t TM_MAX = 1u << 15;  // measured: the cooperative sort wins from ~48K keys
constexpr uint32_t FOREST_MERGE_SLICE = 2048;
constexpr uint32_t FOREST_SORT_MAX = 1u << 17;
constexpr uint32_t FOREST_MERGE_ROUNDS_MAX = 7;  // 131072 / 1024 = 128 tiles
inline uint32_t tm_rounds_for(uint32_t n, uint32_t tile) {
    const uint32_t t = (n + tile - 1) / tile;
    uint32_t r = 0;
    while ((1u << r) < t) r++;
    return r;
}
inline uint32_t tm_tile(uint32_t n) { return (tm_rounds_for(n, 1024) & 1) ? 2048u : 1024u; }
inline uint32_t tm_rounds(uint32_t n) { return tm_rounds_for(n, tm_tile(n)); }
// A batched update sorts for throughput (many graphs' tiles fill the GPU):
// one tile up to 8192 pairs, else tiles of 8192 or 4096 (even rounds);
// bigger tiles sort more keys per SM-microsecond.
inline uint32_t tm_tile_forest(uint32_t n) {
    if (n <= 8192) return 8192;
    return (tm_rounds_for(n, 8192) & 1) ? 4096u : 8192u;
}
inline uint32_t forest_sort_tiles(uint32_t n) { return (n + tm_tile_forest(n) - 1) / tm_tile_forest(n); }
inline uint32_t forest_sort_rounds(uint32_t n) { return tm_rounds_for(n, tm_tile_forest(n)); }
inline uint32_t forest_merge_ctas(uint32_t n) { return (n + FOREST_MERGE_SLICE - 1) / FOREST_MERGE_SLICE; }
struct ForestSortJob {
    uint64_t *k0, *k1;
    uint16_t *p0, *p1;
    const unsigned long long *andor;
    uint32_t n;
    uint32_t tile;  // tm_tile(n)
};
// d_boff: (1 + rounds) tables of G + 1 cumulative CTA counts per job (the
// tile launch, then merge rounds 0 .. rounds-1); nblk: the CTA total of
// each launch (host).
cudaError_t forest_sort(const ForestSortJob *d_jobs, uint32_t G, const uint32_t *d_boff, const uint32_t *nblk,
                        uint32_t rounds, cudaStream_t st);

// Which job block b of a launch over many jobs belongs to: the last g with
// boff[g] <= b (boff holds G + 1 cumulative block counts).  Called by whole
// warps.
__device__ inline uint32_t forest_job_of(const uint32_t *__restrict__ boff, uint32_t G, uint32_t b) {
    // every lane of the warp asks for the same b: 32 entries are probed per
    // memory round trip (two for a few hundred jobs, instead of eight
    // dependent loads of a plain binary search)
    const uint32_t lane = threadIdx.x & 31;
    uint32_t lo = 0, hi = G;  // boff[lo] <= b, and the answer is below hi
    while (hi - lo > 32) {
        const uint32_t span = hi - lo;
        const uint32_t i = lo + (uint32_t)(((uint64_t)span * (lane + 1)) / 33u);
        const int nt = __popc(__ballot_sync(0xffffffffu, boff[i] <= b));
        const uint32_t new_lo = nt ? lo + (uint32_t)(((uint64_t)span * (uint32_t)nt) / 33u) : lo;
        const uint32_t new_hi = nt < 32 ? lo + (uint32_t)(((uint64_t)span * (uint32_t)(nt + 1)) / 33u) : hi;
        lo = new_lo, hi = new_hi;
    }
    const bool p = lo + lane < hi && boff[lo + lane] <= b;
    return lo + (uint32_t)__popc(__ballot_sync(0xffffffffu, p)) - 1;
}

// Keys per tile of the cooperative sort, and the largest batch it takes on
// this device (tiles that can be resident at once x tile); valid after
// sort_prepare().
constexpr int COOP_IPT = 16;
constexpr int COOP_TILE = SORT_TPB * COOP_IPT;  // 4096 keys per CTA
uint32_t coop_sort_max_keys();

// Exclusive scan of n u32 values; out may alias in.  total (device, may be
// null) receives the sum.  tmp needs scan_tmp_words(n) words.
cudaError_t scan_u32(const uint32_t *in, uint32_t *out, uint32_t n, uint32_t *total, uint32_t *tmp,
                     cudaStream_t st);
// same over u8 inputs (segment counts) into u32 outputs
cudaError_t scan_u8_to_u32(const uint8_t *in, uint32_t *out, uint32_t n, uint32_t *total, uint32_t *tmp,
                           cudaStream_t st);
size_t scan_tmp_words(uint32_t n);

// launch counter shared by every translation unit of the library
void note_launch(int k = 1);

// Optional per-kernel timing: when enabled, every launcher brackets its
// launch with CUDA events on the launching stream.
// Programmatic dependent launch.  A kernel launched with launch_pdl may
// start (be scheduled, run its prologue) while its predecessor on the stream
// drains; it calls griddep_wait() before it touches anything the
// predecessor writes, which waits for the whole predecessor grid and its
// memory.  Without a programmatic predecessor the wait returns at once.
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args... args) {
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// Host wait for everything enqueued on s.  blocking: the calling thread
// spins briefly, then sleeps until the GPU signals (an event created with
// cudaEventBlockingSync); for the many threads of a request pool, whose
// spins would crowd the host cores.
cudaError_t host_wait(cudaStream_t s, bool blocking);
// Wait for an event created with cudaEventBlockingSync: spin for up to 40 us,
// then sleep until it completes.
cudaError_t event_wait(cudaEvent_t ev);

// In-library profiler: the kernels launched inside a scope are timed with
// a CUDA event pair on its stream.  Profiled calls launch kernel by kernel
// (no graph), so before the first event the scope puts a short bounded
// delay kernel on the stream: the host enqueues the timed launch while the
// GPU is still busy, and the pair measures device time, not the host's
// launch latency.
struct ProfScope {
    ProfScope(const char *name, cudaStream_t s);
    ~ProfScope();
    int idx;
    cudaStream_t s;
};
bool prof_enabled();

}  // namespace lpma
