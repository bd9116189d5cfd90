// lpma_shuffle_static: lpma_shuffle without any allocation.
//
// lpma_shuffle takes its scratch (a second key buffer, hashes, payloads and
// the radix sort's counters) from cudaMalloc on every call.  This variant
// takes the same scratch from one fixed device array declared below, so a
// caller that must not allocate or free device memory can still shuffle.
// The kernels and their order are the ones lpma_shuffle runs, so the result
// is the same bit for bit.
#include <cstddef>
#include <cstdint>
#include <mutex>

#include "kernels.cuh"
#include "lpma.h"
#include "per_device.h"
#include "prims.cuh"

using namespace lpma;

namespace {

constexpr size_t MAXN = LPMA_SHUFFLE_STATIC_MAX_KEYS;
constexpr size_t round256(size_t x) { return (x + 255) & ~size_t(255); }

// Radix-sort status words for MAXN keys (counts and offsets per tile and digit).
constexpr size_t STATUS_WORDS = sort_status_words((uint32_t)MAXN);

// Layout of the scratch array; every piece starts on a 256-byte boundary.
constexpr size_t OFF_TMP = 0;                                   // u64 keys, second buffer of sort 1
constexpr size_t OFF_HASH = OFF_TMP + round256(8 * MAXN);       // u64 hash of each key
constexpr size_t OFF_HASH2 = OFF_HASH + round256(8 * MAXN);     // u64 second buffer of sort 2
constexpr size_t OFF_PAY2 = OFF_HASH2 + round256(8 * MAXN);     // u64 payload buffer of sort 2
constexpr size_t OFF_P0 = OFF_PAY2 + round256(8 * MAXN);        // u16 payload of sort 1
constexpr size_t OFF_P1 = OFF_P0 + round256(2 * MAXN);          // u16 second payload buffer
constexpr size_t OFF_STATUS = OFF_P1 + round256(2 * MAXN);      // u32 per-pass tile counts
constexpr size_t OFF_HIST = OFF_STATUS + round256(4 * STATUS_WORDS);  // u32 8 x 256 digit counts
constexpr size_t OFF_COUNTERS = OFF_HIST + round256(4 * 8 * 256);     // u32 x 16
constexpr size_t USED_BYTES = OFF_COUNTERS + round256(4 * 16);
static_assert(USED_BYTES <= (size_t)LPMA_SHUFFLE_STATIC_SCRATCH_BYTES, "scratch layout exceeds the stated size");

// The scratch: one array per device, shared by every call in the process.
static __device__ __align__(256) unsigned char g_shuffle_scratch[LPMA_SHUFFLE_STATIC_SCRATCH_BYTES];

PerDevice<unsigned char *> g_scratch_ptr;  // device address of the array, per device

// One-time set-up for the current device: the array's device address (the
// host must pass this address to kernels, not the symbol) and the sort
// kernels' shared-memory attributes.
lpma_status_t scratch_for_current_device(unsigned char **out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return LPMA_ERR_CUDA;
    unsigned char *const *p = nullptr;
    const int r = g_scratch_ptr.get(
        dev,
        [](int, unsigned char *&ptr) -> int {
            const cudaError_t e = cudaGetSymbolAddress((void **)&ptr, g_shuffle_scratch);
            if (e != cudaSuccess || ptr == nullptr) return (int)LPMA_ERR_CUDA;
            return sort_prepare() != cudaSuccess ? (int)LPMA_ERR_CUDA : 0;
        },
        &p, (int)LPMA_ERR_INVALID_ARGUMENT);
    if (r) return (lpma_status_t)r;
    *out = *p;
    return LPMA_OK;
}

}  // namespace

extern "C" {

lpma_status_t lpma_shuffle_static(uint64_t seed, uint64_t *d_keys, size_t n, lpma_stream_t stream) {
    // a null pointer is reported before the size, whatever the size
    if (!d_keys && n) return LPMA_ERR_INVALID_ARGUMENT;
    if (n > MAXN) return LPMA_ERR_SCRATCH_LIMIT;
    unsigned char *base = nullptr;
    const lpma_status_t r = scratch_for_current_device(&base);
    if (r != LPMA_OK) return r;
    if (n < 2) return LPMA_OK;
    if (sort_status_words((uint32_t)n) > STATUS_WORDS) return LPMA_ERR_INTERNAL;
    cudaStream_t s = (cudaStream_t)stream;
    uint64_t *tmp = (uint64_t *)(base + OFF_TMP);
    uint64_t *hash = (uint64_t *)(base + OFF_HASH);
    uint64_t *hash2 = (uint64_t *)(base + OFF_HASH2);
    uint64_t *pay2 = (uint64_t *)(base + OFF_PAY2);
    uint16_t *p0 = (uint16_t *)(base + OFF_P0);
    uint16_t *p1 = (uint16_t *)(base + OFF_P1);
    SortScratch ss;
    ss.status = (uint32_t *)(base + OFF_STATUS);
    ss.status_words = STATUS_WORDS;
    ss.hist = (uint32_t *)(base + OFF_HIST);
    ss.counters = (uint32_t *)(base + OFF_COUNTERS);
    // the first sort carries a dummy payload: give it defined contents
    cudaError_t e = cudaMemsetAsync(p0, 0, n * sizeof(uint16_t), s);
    int which = 0;
    // (hash, key) order: keys ascending, then a stable sort by hash
    if (!e) e = sort_pairs<uint16_t>(d_keys, p0, tmp, p1, (uint32_t)n, ~0ull, ss, nullptr, s, &which);
    uint64_t *sorted = which ? tmp : d_keys;
    if (!e) {
        launch_hash_keys(seed, sorted, hash, n, s);
        e = cudaGetLastError();
    }
    if (!e) e = sort_pairs<uint64_t>(hash, sorted, hash2, pay2, (uint32_t)n, ~0ull, ss, nullptr, s, &which);
    uint64_t *res = which ? pay2 : sorted;
    if (!e && res != d_keys) e = cudaMemcpyAsync(d_keys, res, n * sizeof(uint64_t), cudaMemcpyDeviceToDevice, s);
    if (e) return e == cudaErrorMemoryAllocation ? LPMA_ERR_OUT_OF_MEMORY : LPMA_ERR_CUDA;
    return LPMA_OK;
}

}  // extern "C"
