// CSR view / export kernels and the synthetic workload generator.
#include "kernels.cuh"
#include "prims.cuh"

namespace lpma {
namespace {

constexpr int TPB = 256;

// to_csr_rpma (rpma.cuh:2249-2295): the present keys in linear order,
// compacted.  One warp per segment; P is the exclusive prefix of the
// per-segment counts, so the writes of a warp are one contiguous run.
__global__ void __launch_bounds__(TPB) k_csr_fill(Geo g, const uint8_t *__restrict__ cnt, const uint32_t *__restrict__ P,
                                                  uint32_t *row_offset, uint32_t *col_index, uint8_t *values,
                                                  uint64_t *ek, uint8_t *ev) {
    const uint64_t nseg = nseg_of(g.H);
    const int lane = threadIdx.x & 31;
    for (uint64_t s = (blockIdx.x * (uint64_t)TPB + threadIdx.x) >> 5; s < nseg;
         s += (gridDim.x * (uint64_t)TPB) >> 5) {
        const uint32_t c = cnt[s];
        if ((uint32_t)lane >= c) continue;
        const uint64_t j = heap_of_linear(s, g.H);
        const uint64_t key = g.keys[32 * j + lane];
        const uint8_t val = g.vals[32 * j + lane];
        const uint32_t pos = P[s] + lane;
        if (col_index) {
            const uint32_t src = (uint32_t)(key >> SRC_SHIFT);
            const uint32_t dst = (uint32_t)((key & DST_MASK) >> DST_SHIFT);
            if (dst == NBR_END) {
                col_index[pos] = src;
                values[pos] = VAL_TOMB;
                row_offset[src + 1] = pos + 1;
            } else {
                col_index[pos] = dst;
                values[pos] = val;
            }
        }
        if (ek) {
            ek[pos] = key;
            ev[pos] = val;
        }
    }
}

__device__ inline uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// R-MAT: per edge and bit level one 64-bit hash, high 32 bits against the
// quadrant thresholds; self loops become ~0 (dropped by the dedup).
__global__ void __launch_bounds__(TPB) k_rmat(uint64_t s0, uint32_t scale, uint64_t n, uint32_t ta, uint32_t tab,
                                              uint32_t tabc, uint64_t *out) {
    for (uint64_t e = blockIdx.x * (uint64_t)TPB + threadIdx.x; e < n; e += gridDim.x * (uint64_t)TPB) {
        uint64_t src = 0, dst = 0;
        for (uint32_t b = 0; b < scale; b++) {
            const uint32_t r = (uint32_t)(mix64(s0 ^ ((e << 6) | b)) >> 32);
            const uint64_t sb = r >= tab, db = (r >= ta && r < tab) || r >= tabc;
            src = (src << 1) | sb;
            dst = (dst << 1) | db;
        }
        out[e] = src == dst ? KEY_NONE : (src << SRC_SHIFT) | (dst << DST_SHIFT);
    }
}

__global__ void __launch_bounds__(TPB) k_hash_keys(uint64_t seed, const uint64_t *keys, uint64_t *hash, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)TPB + threadIdx.x; i < n; i += gridDim.x * (uint64_t)TPB)
        hash[i] = mix64(seed ^ keys[i]);
}

__global__ void __launch_bounds__(TPB) k_unique_flags(const uint64_t *keys, uint64_t n, uint32_t *flags) {
    for (uint64_t i = blockIdx.x * (uint64_t)TPB + threadIdx.x; i < n; i += gridDim.x * (uint64_t)TPB)
        flags[i] = keys[i] != KEY_NONE && (i == 0 || keys[i - 1] != keys[i]);
}

__global__ void __launch_bounds__(TPB) k_scatter_flags(const uint64_t *keys, const uint32_t *pos,
                                                       const uint32_t *flags, uint64_t n, uint64_t *out) {
    for (uint64_t i = blockIdx.x * (uint64_t)TPB + threadIdx.x; i < n; i += gridDim.x * (uint64_t)TPB)
        if (flags[i]) out[pos[i]] = keys[i];
}

__global__ void __launch_bounds__(TPB) k_sentinels(uint32_t V, uint64_t *keys, uint8_t *vals) {
    for (uint64_t v = blockIdx.x * (uint64_t)TPB + threadIdx.x; v < V; v += gridDim.x * (uint64_t)TPB) {
        keys[v] = (v << SRC_SHIFT) + DST_AND_TIME_END;  // col_idx_none, rpma.cuh:1797-1805
        vals[v] = 0;                                     // rpma.cuh:1814
    }
}

inline uint32_t grid_for(uint64_t n, uint32_t per_block, uint32_t cap = 152 * 16) {
    uint64_t g = (n + per_block - 1) / per_block;
    if (g == 0) g = 1;
    return (uint32_t)(g < cap ? g : cap);
}

}  // namespace

void launch_csr_fill(Geo g, const uint8_t *cnt, const uint32_t *P, uint32_t *row_offset, uint32_t *col_index,
                     uint8_t *values, uint64_t *export_keys, uint8_t *export_vals, cudaStream_t s) {
    ProfScope ps_("csr_fill", s);
    k_csr_fill<<<grid_for(nseg_of(g.H), TPB / 32), TPB, 0, s>>>(g, cnt, P, row_offset, col_index, values, export_keys,
                                                                export_vals);
    note_launch();
}

void launch_sentinels(uint32_t V, uint64_t *keys, uint8_t *vals, cudaStream_t s) {
    ProfScope ps_("sentinels", s);
    k_sentinels<<<grid_for(V, TPB), TPB, 0, s>>>(V, keys, vals);
    note_launch();
}

void launch_rmat(uint64_t seed, uint32_t scale, uint64_t n, uint32_t ta, uint32_t tab, uint32_t tabc, uint64_t *out,
                 cudaStream_t s) {
    ProfScope ps_("gen_rmat", s);
    uint64_t s0 = seed;
    // same seeding as the CPU generator: s0 = mix64(seed)
    s0 += 0x9E3779B97F4A7C15ull;
    s0 = (s0 ^ (s0 >> 30)) * 0xBF58476D1CE4E5B9ull;
    s0 = (s0 ^ (s0 >> 27)) * 0x94D049BB133111EBull;
    s0 = s0 ^ (s0 >> 31);
    k_rmat<<<grid_for(n, TPB), TPB, 0, s>>>(s0, scale, n, ta, tab, tabc, out);
    note_launch();
}

void launch_hash_keys(uint64_t seed, const uint64_t *keys, uint64_t *hash, uint64_t n, cudaStream_t s) {
    ProfScope ps_("hash_keys", s);
    k_hash_keys<<<grid_for(n, TPB), TPB, 0, s>>>(seed, keys, hash, n);
    note_launch();
}

void launch_unique_flags(const uint64_t *keys, uint64_t n, uint32_t *flags, cudaStream_t s) {
    ProfScope ps_("unique_flags", s);
    k_unique_flags<<<grid_for(n, TPB), TPB, 0, s>>>(keys, n, flags);
    note_launch();
}

void launch_scatter_flags(const uint64_t *keys, const uint32_t *pos, const uint32_t *flags, uint64_t n, uint64_t *out,
                          cudaStream_t s) {
    ProfScope ps_("scatter_flags", s);
    k_scatter_flags<<<grid_for(n, TPB), TPB, 0, s>>>(keys, pos, flags, n, out);
    note_launch();
}

}  // namespace lpma
