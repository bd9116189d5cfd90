// Shared definitions of the GB300 LPMA engine: key layout, segment-tree index
// algebra, the device status block and small device utilities.
//
// Layout in HBM.  A tree of height H has 2^(H+1) - 1 segments of 32 slots.
// The reference stores tree level i as its own array of 32 << i slots
// (rpma.cuh:1396-1415); here the level arrays are laid end to end in one
// allocation, which is heap (Eytzinger) order: segment j of level i sits at
// heap index 2^i - 1 + pos, slots [32 j, 32 j + 32).  Adding a level appends
// 32 << (H+1) slots and moves nothing.  The logical ("linear") order of the
// segments is the in-order traversal: linear segment s lives at level
// H - ctz(s+1), position (s+1) >> (ctz(s+1)+1) (GET_IDX/GET_LANE,
// rpma.cuh:132-134).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace lpma {

constexpr uint64_t KEY_NONE = ~0ull;                        // rpma.cuh:38
constexpr uint8_t VAL_TOMB = 0xFF;                          // VALUE_NONE, rpma.cuh:41 / gpma.cuh:33
constexpr uint64_t TIME_MASK = 0x00000000000FFFFFull;       // rpma.cuh:47
constexpr uint64_t DST_MASK = 0x000003FFFFF00000ull;        // rpma.cuh:45
constexpr uint64_t DST_AND_TIME_MASK = 0x000003FFFFFFFFFFull;  // rpma.cuh:48
constexpr uint64_t DST_AND_TIME_END = 0x000003FFFFEFFFFFull;   // rpma.cuh:49
constexpr uint32_t SRC_SHIFT = 42, DST_SHIFT = 20;
constexpr uint32_t NBR_END = 0x003FFFFEu;                   // rpma.cuh:50
constexpr uint32_t SEG = 32;                                // rpma.cuh:1769
constexpr uint32_t MAX_HEIGHT = 24;
constexpr uint32_t KIND_NOP = 0, KIND_INS = 1, KIND_DEL = 2;
constexpr uint32_t EXEC_OVF = 0xFF;                         // no window absorbed the segment
constexpr uint32_t SMALL_WIN_SEGS = 32;                     // warp-grain windows: <= 32 segments

// error bits of DevStatus::error
constexpr uint32_t ERR_KEY = 1u, ERR_INTERNAL = 2u, ERR_TIMEOUT = 4u;

__host__ __device__ inline uint64_t umin64(uint64_t a, uint64_t b) { return a < b ? a : b; }

__host__ __device__ inline uint64_t nseg_of(uint32_t H) { return (2ull << H) - 1; }
__host__ __device__ inline uint64_t nslots_of(uint32_t H) { return 32ull * nseg_of(H); }

// heap index of linear segment s in a tree of height H
__host__ __device__ inline uint64_t heap_of_linear(uint64_t s, uint32_t H) {
    uint64_t s1 = s + 1;
#ifdef __CUDA_ARCH__
    uint32_t t = (uint32_t)__ffsll((long long)s1) - 1;
#else
    uint32_t t = (uint32_t)__builtin_ctzll(s1);
#endif
    uint32_t level = H - t;
    return ((1ull << level) - 1) + (s1 >> (t + 1));
}

// heap_of_linear in 32-bit arithmetic, for segment indexes below 2^31 (every
// tree here: at most 2^(LPMA_MAX_HEIGHT + 1) segments)
__device__ __forceinline__ uint32_t heap_of_linear32(uint32_t s, uint32_t H) {
    const uint32_t s1 = s + 1, t = (uint32_t)__ffs((int)s1) - 1;
    return ((1u << (H - t)) - 1) + (s1 >> (t + 1));
}

// linear segment of heap index j at level `level` of a tree of height H
__host__ __device__ inline uint64_t linear_of_heap(uint64_t j, uint32_t level, uint32_t H) {
    uint64_t pos = j - ((1ull << level) - 1);
    return ((2 * pos + 1) << (H - level)) - 1;
}

__host__ __device__ inline bool is_sentinel(uint64_t key) {
    return (key & DST_AND_TIME_MASK) == DST_AND_TIME_END;
}

__host__ __device__ inline bool kept_slot(uint64_t key, uint8_t val, uint32_t thres) {
    return key != KEY_NONE && val != VAL_TOMB && (key & TIME_MASK) >= (uint64_t)thres;
}

// first destination rank of segment k when m items spread over f segments:
// item i goes to segment floor(f*i/m) (rpma.cuh:677-679, 965-967), so
// segment k starts at ceil(k*m/f) and its items are packed from lane 0.
__host__ __device__ inline uint64_t first_rank(uint64_t k, uint64_t m, uint64_t f) {
    return (k * m + f - 1) / f;
}

// Device status block, one per handle.  The host reads it at the two sync
// points of an update call.
struct DevStatus {
    uint32_t error;
    uint32_t min_t_ins;       // min timestamp over inserted keys (atomicMin)
    unsigned long long key_and, key_or;
    uint32_t n_u;             // compacted updates
    uint32_t n_ins, n_del, n_upsert, n_noop;
    uint32_t n_cand, n_single, n_small4, n_small, n_big;
    uint32_t big_tiles;       // 32-segment tiles of the big windows
    uint32_t root, ovf;
    uint32_t exec_levels;     // bit l: some window of level l executes
    uint32_t empty_found;     // fill_empty_segs check
    unsigned long long slots_small, slots_big;
    unsigned long long live_total;   // sum of live counts (thres pass)
    unsigned long long cnt_total;    // sum of occupancy counts (recount)
    unsigned long long total_items;  // keys stored before the call (set by the host)
    uint32_t err_info[4];            // first offending input index, internal-check site
    uint32_t plan_done;              // planner CTAs finished (the front's status publish)
    // Not reset per call (the reset copies the fields above only): the
    // executors set ERR_INTERNAL here after the call may have returned.
    uint32_t sticky;
    uint32_t sticky_site;  // which internal check set ERR_INTERNAL (first one)
    // Meaningful in the host mirror only: set to 1 by the planner's last CTA
    // after it wrote the words above into the mirror (k_plan_max, publish).
    uint32_t published;
};

// A rebalance window chosen by the planner (maximal executed window); 8-byte
// aligned so that a record loads as three 64-bit words.
struct __align__(8) Window {
    uint32_t a;      // first linear segment
    uint32_t f;      // segments (clipped)
    uint32_t m;      // items after the update
    uint32_t level;
    uint32_t lo, hi; // range in the compacted update list
};

struct Tables {
    uint32_t lower[32];  // trunc(0.42 * 32 * 2^i), rpma.cuh:164
    uint32_t allowed;    // bit l: windows of level l may execute
    // the flat (GPMA) layout: slots per segment and segment count (0: the
    // leveled tree's 32 and 2^(H+1) - 1)
    uint32_t seg_len;
    unsigned long long nseg;
    // executor grain cut-overs (0: the defaults): windows of up to cut_group
    // segments go to the 8-lane-group executor, up to cut_shared to the
    // shared-memory one, larger ones to the tile grain
    uint32_t cut_group, cut_shared;
};
constexpr uint32_t CUT_GROUP_DEFAULT = 4, CUT_GROUP_MAX = 4;

__device__ inline uint32_t lanemask_lt() {
    uint32_t r;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(r));
    return r;
}

}  // namespace lpma
