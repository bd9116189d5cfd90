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
};

// Sorts n pairs by key (stable).  Only the bytes set in diff_bits are sorted
// (bytes equal across all keys need no pass).  The result lands either in
// (k0, v0) or in (k1, v1); *which receives 0 or 1.  err is kept for the
// interface (no kernel of the sort waits on another CTA).
template <typename V>
cudaError_t sort_pairs(uint64_t *k0, V *v0, uint64_t *k1, V *v1, uint32_t n, uint64_t diff_bits,
                       SortScratch &s, uint32_t *err, cudaStream_t st, int *which);

// Bytes of scratch status words needed for n keys.
inline size_t sort_status_words(uint32_t n) {
    size_t tiles = (n + SORT_TILE - 1) / SORT_TILE;
    return 2 * tiles * 256 + 2;  // per-pass (digit, tile) counts and offsets
}

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
struct ProfScope {
    ProfScope(const char *name, cudaStream_t s);
    ~ProfScope();
    int idx;
    cudaStream_t s;
};
bool prof_enabled();

}  // namespace lpma
