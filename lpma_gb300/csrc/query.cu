// Read paths over the PMA: batched neighbour lists with a time window,
// edge queries, BFS and PageRank.  They read the structure in place (no CSR
// view is built): the keys of vertex v are the occupied slots strictly
// between the sentinel of v-1 and the sentinel of v in linear slot order.
#include <climits>

#include "kernels.cuh"
#include "prims.cuh"

namespace lpma {
namespace {

constexpr int TPB = 256;

// linear slot (32 * linear segment + lane) of a heap slot index
__device__ inline uint64_t linear_slot(uint32_t heap_slot, uint32_t H) {
    const uint64_t j = heap_slot >> 5;
    const uint32_t level = 63 - __clzll((long long)(j + 1));
    return 32 * linear_of_heap(j, level, H) + (heap_slot & 31);
}

// linear slot range [p0, p1) that holds vertex v's keys (empty slots
// included; a slot is occupied when its lane is below the segment's count)
__device__ inline void vertex_range(const uint32_t *sent, uint32_t v, uint32_t H, uint64_t &p0, uint64_t &p1) {
    p0 = v ? linear_slot(sent[v - 1], H) + 1 : 0;
    p1 = linear_slot(sent[v], H);
}

// One 8-lane group reads linear segment s: lane gl holds slots 4gl..4gl+3.
// Returns the mask of slots that are occupied and inside [p0, p1).
__device__ inline uint32_t load_seg_part(Geo g, const uint8_t *cnt, uint64_t s, uint64_t p0, uint64_t p1, int gl,
                                         uint64_t (&k)[4], uint8_t (&v)[4]) {
    const uint64_t j = heap_of_linear(s, g.H);
    const uint32_t c = cnt[s];
    const uint64_t base = 32 * s;
    const uint32_t a = p0 > base ? (uint32_t)(p0 - base) : 0u;
    const uint32_t b0 = p1 < base + 32 ? (uint32_t)(p1 - base) : 32u;
    const uint32_t b = b0 < c ? b0 : c;
    uint32_t m = 0;
    if (4 * (uint32_t)gl < b && 4 * (uint32_t)gl + 4 > a) {
        const ulonglong2 *kp = reinterpret_cast<const ulonglong2 *>(g.keys + 32 * j + 4 * gl);
        const ulonglong2 x = kp[0], y = kp[1];
        const uint32_t v4 = *reinterpret_cast<const uint32_t *>(g.vals + 32 * j + 4 * gl);
        k[0] = x.x, k[1] = x.y, k[2] = y.x, k[3] = y.y;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            v[q] = (uint8_t)(v4 >> (8 * q));
            const uint32_t slot = 4 * gl + q;
            if (slot >= a && slot < b && v[q] != VAL_TOMB) m |= 1u << q;
        }
    }
    return m;
}

__device__ inline bool in_window(uint64_t key, uint32_t lb, uint32_t ub) {
    const uint32_t t = (uint32_t)(key & TIME_MASK);
    return t >= lb && t <= ub;
}

// ---------------------------------------------------------------- neighbour lists
// query_rpma (rpma.cuh:1827-2036): for query i, the neighbours of srcs[i]
// whose timestamp lies in [windows[i] >> 32, windows[i] & 0xFFFFFFFF], in
// key order.  One warp per query, four segments per round (one per 8-lane
// group).  Pass 1 counts, pass 2 writes at offsets[i].
__global__ void __launch_bounds__(TPB) k_nbr_count(const uint32_t *__restrict__ srcs,
                                                   const uint64_t *__restrict__ windows, uint32_t n, Geo g,
                                                   const uint8_t *__restrict__ cnt, const uint32_t *__restrict__ sent,
                                                   uint32_t V, uint32_t *qcnt) {
    const int lane = threadIdx.x & 31, gl = lane & 7, grp = lane >> 3;
    for (uint64_t i = (blockIdx.x * (uint64_t)TPB + threadIdx.x) >> 5; i < n; i += (gridDim.x * (uint64_t)TPB) >> 5) {
        const uint32_t src = srcs[i];
        uint32_t total = 0;
        if (src < V) {
            const uint64_t w = windows[i];
            const uint32_t lb = (uint32_t)(w >> 32), ub = (uint32_t)w;
            uint64_t p0, p1;
            vertex_range(sent, src, g.H, p0, p1);
            if (p1 > p0) {
                const uint64_t S0 = p0 >> 5, S1 = (p1 - 1) >> 5;
                for (uint64_t s = S0 + grp; s <= S1; s += 4) {
                    uint64_t k[4];
                    uint8_t v[4];
                    const uint32_t m = load_seg_part(g, cnt, s, p0, p1, gl, k, v);
#pragma unroll
                    for (int q = 0; q < 4; q++)
                        if (((m >> q) & 1u) && in_window(k[q], lb, ub)) total++;
                }
            }
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) total += __shfl_xor_sync(0xffffffffu, total, o);
        if (lane == 0) qcnt[i] = total;
    }
}

__global__ void __launch_bounds__(TPB) k_nbr_fill(const uint32_t *__restrict__ srcs,
                                                  const uint64_t *__restrict__ windows, uint32_t n, Geo g,
                                                  const uint8_t *__restrict__ cnt, const uint32_t *__restrict__ sent,
                                                  uint32_t V, const uint32_t *__restrict__ offsets, uint32_t *nbrs,
                                                  uint8_t *vals) {
    const int lane = threadIdx.x & 31, gl = lane & 7, grp = lane >> 3;
    for (uint64_t i = (blockIdx.x * (uint64_t)TPB + threadIdx.x) >> 5; i < n; i += (gridDim.x * (uint64_t)TPB) >> 5) {
        const uint32_t src = srcs[i];
        if (src >= V) continue;  // warp-uniform
        const uint64_t w = windows[i];
        const uint32_t lb = (uint32_t)(w >> 32), ub = (uint32_t)w;
        uint64_t p0, p1;
        vertex_range(sent, src, g.H, p0, p1);
        if (p1 <= p0) continue;
        const uint64_t S0 = p0 >> 5, S1 = (p1 - 1) >> 5;
        uint32_t out = offsets[i];
        for (uint64_t s0 = S0; s0 <= S1; s0 += 4) {
            const uint64_t s = s0 + grp;
            uint64_t k[4];
            uint8_t v[4];
            uint32_t m = 0;
            if (s <= S1) m = load_seg_part(g, cnt, s, p0, p1, gl, k, v);
#pragma unroll
            for (int q = 0; q < 4; q++)
                if (((m >> q) & 1u) && !in_window(k[q], lb, ub)) m &= ~(1u << q);
            // warp-wide exclusive prefix in (group, lane, slot) order = key order
            const uint32_t c = __popc(m);
            uint32_t incl = c;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += y;
            }
            uint32_t pos = out + incl - c;
#pragma unroll
            for (int q = 0; q < 4; q++) {
                if ((m >> q) & 1u) {
                    nbrs[pos] = (uint32_t)((k[q] & DST_MASK) >> DST_SHIFT);
                    vals[pos] = v[q];
                    pos++;
                }
            }
            out += __shfl_sync(0xffffffffu, incl, 31);
        }
    }
}

// ---------------------------------------------------------------- edge queries
// For key (src, dst, t): the number of stored keys (src, dst, t') with
// t - window <= t' <= t (the edge-query check of test.cu:46-62; window =
// 0xFFFFF with t = 0xFFFFF gives check_edge_kernel's any-time test,
// rpma.cuh:2040-2066).  Binary search over src's segments for the first
// segment whose last key reaches (src, dst, lb), then a forward count.
__global__ void __launch_bounds__(TPB) k_edge_query(const uint64_t *__restrict__ q, uint32_t n, uint32_t window, Geo g,
                                                    const uint8_t *__restrict__ cnt,
                                                    const ulonglong2 *__restrict__ fl,
                                                    const uint32_t *__restrict__ sent, uint32_t V, uint32_t *res) {
    for (uint64_t i = blockIdx.x * (uint64_t)TPB + threadIdx.x; i < n; i += gridDim.x * (uint64_t)TPB) {
        const uint64_t key = q[i];
        const uint32_t src = (uint32_t)(key >> SRC_SHIFT);
        const uint32_t dst = (uint32_t)((key & DST_MASK) >> DST_SHIFT);
        uint32_t found = 0;
        if (src < V && dst < NBR_END) {
            const uint32_t t = (uint32_t)(key & TIME_MASK);
            const uint32_t lb = t > window ? t - window : 0;
            const uint64_t pre = key & ~TIME_MASK;
            const uint64_t lo = pre | lb, hi = pre | t;
            uint64_t p0, p1;
            vertex_range(sent, src, g.H, p0, p1);
            if (p1 > p0) {
                const uint64_t S0 = p0 >> 5, S1 = (p1 - 1) >> 5;
                // first non-empty segment in [S0, S1] whose last key >= lo
                uint64_t L = S0, R = S1 + 1, ans = S1 + 1;
                while (L < R) {
                    const uint64_t mid = (L + R) >> 1;
                    uint64_t ms = mid;
                    while (ms < R && cnt[ms] == 0) ms++;
                    if (ms == R) {
                        R = mid;
                        continue;
                    }
                    const uint64_t last = fl[heap_of_linear(ms, g.H)].y;
                    if (last >= lo) {
                        ans = ms;
                        R = mid;
                    } else {
                        L = ms + 1;
                    }
                }
                bool done = false;
                for (uint64_t s = ans; s <= S1 && !done; s++) {
                    const uint32_t c = cnt[s];
                    const uint64_t j = heap_of_linear(s, g.H);
                    for (uint32_t l = 0; l < c; l++) {
                        const uint64_t pos = 32 * s + l;
                        if (pos < p0) continue;
                        if (pos >= p1) {
                            done = true;
                            break;
                        }
                        const uint64_t kk = g.keys[32 * j + l];
                        if (kk > hi) {
                            done = true;
                            break;
                        }
                        if (kk >= lo && g.vals[32 * j + l] != VAL_TOMB) found++;
                    }
                }
            }
        }
        res[i] = found;
    }
}

// ---------------------------------------------------------------- BFS
__global__ void __launch_bounds__(TPB) k_bfs_init(int32_t *dist, uint32_t V) {
    for (uint64_t v = blockIdx.x * (uint64_t)TPB + threadIdx.x; v < V; v += gridDim.x * (uint64_t)TPB)
        dist[v] = INT_MAX;
}

__global__ void __launch_bounds__(TPB) k_bfs_seed(const uint32_t *__restrict__ sources, uint32_t n, uint32_t V,
                                                  int32_t *dist, uint32_t *frontier, uint32_t *count) {
    for (uint64_t i = blockIdx.x * (uint64_t)TPB + threadIdx.x; i < n; i += gridDim.x * (uint64_t)TPB) {
        const uint32_t s = sources[i];
        if (s < V && atomicCAS(&dist[s], INT_MAX, 0) == INT_MAX) frontier[atomicAdd(count, 1u)] = s;
    }
}

// one warp per frontier vertex; a neighbour first reached at this level gets
// dist = level + 1 and joins the next frontier
__global__ void __launch_bounds__(TPB) k_bfs_expand(const uint32_t *__restrict__ frontier,
                                                    const uint32_t *__restrict__ nf_p, int32_t level, Geo g,
                                                    const uint8_t *__restrict__ cnt,
                                                    const uint32_t *__restrict__ sent, int32_t *dist, uint32_t *next,
                                                    uint32_t *next_count) {
    const int lane = threadIdx.x & 31, gl = lane & 7, grp = lane >> 3;
    const uint32_t nf = *nf_p;
    for (uint64_t i = (blockIdx.x * (uint64_t)TPB + threadIdx.x) >> 5; i < nf; i += (gridDim.x * (uint64_t)TPB) >> 5) {
        const uint32_t u = frontier[i];
        uint64_t p0, p1;
        vertex_range(sent, u, g.H, p0, p1);
        if (p1 <= p0) continue;
        const uint64_t S0 = p0 >> 5, S1 = (p1 - 1) >> 5;
        for (uint64_t s = S0 + grp; s <= S1; s += 4) {
            uint64_t k[4];
            uint8_t v[4];
            const uint32_t m = load_seg_part(g, cnt, s, p0, p1, gl, k, v);
#pragma unroll
            for (int q = 0; q < 4; q++) {
                if ((m >> q) & 1u) {
                    const uint32_t d = (uint32_t)((k[q] & DST_MASK) >> DST_SHIFT);
                    if (atomicCAS(&dist[d], INT_MAX, level + 1) == INT_MAX) next[atomicAdd(next_count, 1u)] = d;
                }
            }
        }
    }
}

// ---------------------------------------------------------------- PageRank
// out-degree: one 8-lane group per segment, one atomic per run of equal
// sources within a lane's four slots
__global__ void __launch_bounds__(TPB) k_outdeg(Geo g, const uint8_t *__restrict__ cnt, uint32_t *deg) {
    const uint64_t nseg = nseg_of(g.H);
    const int gl = threadIdx.x & 7;
    for (uint64_t s = (blockIdx.x * (uint64_t)TPB + threadIdx.x) >> 3; s < nseg; s += (gridDim.x * (uint64_t)TPB) >> 3) {
        uint64_t k[4];
        uint8_t v[4];
        const uint32_t m = load_seg_part(g, cnt, s, 0, ~0ull, gl, k, v);
        uint32_t run_src = 0xFFFFFFFFu, run = 0;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            if (((m >> q) & 1u) && !is_sentinel(k[q])) {
                const uint32_t src = (uint32_t)(k[q] >> SRC_SHIFT);
                if (src != run_src) {
                    if (run) atomicAdd(&deg[run_src], run);
                    run_src = src;
                    run = 0;
                }
                run++;
            }
        }
        if (run) atomicAdd(&deg[run_src], run);
    }
}

// contrib[v] = rank[v] / deg[v]; the rank of vertices without out-edges is
// summed into *dangling
__global__ void __launch_bounds__(TPB) k_pr_contrib(const double *__restrict__ rank, const uint32_t *__restrict__ deg,
                                                    uint32_t V, double *contrib, double *dangling) {
    __shared__ double ws[TPB / 32];
    double d = 0;
    for (uint64_t v = blockIdx.x * (uint64_t)TPB + threadIdx.x; v < V; v += gridDim.x * (uint64_t)TPB) {
        const uint32_t c = deg[v];
        contrib[v] = c ? rank[v] / (double)c : 0.0;
        if (!c) d += rank[v];
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = d;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int i = 0; i < TPB / 32; i++) t += ws[i];
        if (t != 0.0) atomicAdd(dangling, t);
    }
}

__global__ void __launch_bounds__(TPB) k_pr_push(Geo g, const uint8_t *__restrict__ cnt,
                                                 const double *__restrict__ contrib, double *acc) {
    const uint64_t nseg = nseg_of(g.H);
    const int gl = threadIdx.x & 7;
    for (uint64_t s = (blockIdx.x * (uint64_t)TPB + threadIdx.x) >> 3; s < nseg; s += (gridDim.x * (uint64_t)TPB) >> 3) {
        uint64_t k[4];
        uint8_t v[4];
        const uint32_t m = load_seg_part(g, cnt, s, 0, ~0ull, gl, k, v);
#pragma unroll
        for (int q = 0; q < 4; q++) {
            if (((m >> q) & 1u) && !is_sentinel(k[q])) {
                const uint32_t src = (uint32_t)(k[q] >> SRC_SHIFT);
                const uint32_t dst = (uint32_t)((k[q] & DST_MASK) >> DST_SHIFT);
                atomicAdd(&acc[dst], contrib[src]);
            }
        }
    }
}

// rank = (1 - alpha) / V + alpha * (acc + dangling / V); clears acc and
// leaves the dangling sum for the next iteration at zero
__global__ void __launch_bounds__(TPB) k_pr_finish(double *rank, double *acc, uint32_t V, double alpha,
                                                   const double *__restrict__ dangling) {
    const double base = (1.0 - alpha) / (double)V, dv = *dangling / (double)V;
    for (uint64_t v = blockIdx.x * (uint64_t)TPB + threadIdx.x; v < V; v += gridDim.x * (uint64_t)TPB) {
        rank[v] = base + alpha * (acc[v] + dv);
        acc[v] = 0.0;
    }
}

__global__ void k_zero_f64(double *p) { *p = 0.0; }

__global__ void __launch_bounds__(TPB) k_fill_f64(double *p, uint64_t n, double x) {
    for (uint64_t i = blockIdx.x * (uint64_t)TPB + threadIdx.x; i < n; i += gridDim.x * (uint64_t)TPB) p[i] = x;
}

inline uint32_t grid_for(uint64_t n, uint32_t per_block, uint32_t cap = 152 * 16) {
    const uint64_t b = (n + per_block - 1) / per_block;
    return (uint32_t)(b == 0 ? 1 : (b < cap ? b : cap));
}

}  // namespace

void launch_nbr_count(const uint32_t *srcs, const uint64_t *windows, uint32_t n, Geo g, const uint8_t *cnt,
                      const uint32_t *sent, uint32_t V, uint32_t *qcnt, cudaStream_t s) {
    ProfScope ps_("nbr_count", s);
    k_nbr_count<<<grid_for(n, TPB / 32, 152 * 16), TPB, 0, s>>>(srcs, windows, n, g, cnt, sent, V, qcnt);
    note_launch();
}

void launch_nbr_fill(const uint32_t *srcs, const uint64_t *windows, uint32_t n, Geo g, const uint8_t *cnt,
                     const uint32_t *sent, uint32_t V, const uint32_t *offsets, uint32_t *nbrs, uint8_t *vals,
                     cudaStream_t s) {
    ProfScope ps_("nbr_fill", s);
    k_nbr_fill<<<grid_for(n, TPB / 32, 152 * 16), TPB, 0, s>>>(srcs, windows, n, g, cnt, sent, V, offsets, nbrs,
                                                                vals);
    note_launch();
}

void launch_edge_query(const uint64_t *q, uint32_t n, uint32_t window, Geo g, const uint8_t *cnt,
                       const ulonglong2 *fl, const uint32_t *sent, uint32_t V, uint32_t *res, cudaStream_t s) {
    ProfScope ps_("edge_query", s);
    k_edge_query<<<grid_for(n, TPB, 152 * 16), TPB, 0, s>>>(q, n, window, g, cnt, fl, sent, V, res);
    note_launch();
}

void launch_bfs_init(const uint32_t *sources, uint32_t n, uint32_t V, int32_t *dist, uint32_t *frontier,
                     uint32_t *count, cudaStream_t s) {
    ProfScope ps_("bfs_init", s);
    k_bfs_init<<<grid_for(V, TPB, 152 * 16), TPB, 0, s>>>(dist, V);
    k_bfs_seed<<<grid_for(n, TPB, 152 * 16), TPB, 0, s>>>(sources, n, V, dist, frontier, count);
    note_launch(2);
}

void launch_bfs_expand(const uint32_t *frontier, const uint32_t *nf, uint32_t nf_host, int32_t level, Geo g,
                       const uint8_t *cnt, const uint32_t *sent, int32_t *dist, uint32_t *next, uint32_t *next_count,
                       cudaStream_t s) {
    ProfScope ps_("bfs_expand", s);
    k_bfs_expand<<<grid_for(nf_host, TPB / 32, 152 * 16), TPB, 0, s>>>(frontier, nf, level, g, cnt, sent, dist, next,
                                                                       next_count);
    note_launch();
}

void launch_outdeg(Geo g, const uint8_t *cnt, uint32_t *deg, cudaStream_t s) {
    ProfScope ps_("outdeg", s);
    k_outdeg<<<grid_for(nseg_of(g.H), TPB / 8, 152 * 16), TPB, 0, s>>>(g, cnt, deg);
    note_launch();
}

void launch_fill_f64(double *p, uint64_t n, double x, cudaStream_t s) {
    k_fill_f64<<<grid_for(n, TPB, 152 * 8), TPB, 0, s>>>(p, n, x);
    note_launch();
}

void launch_pr_iteration(Geo g, const uint8_t *cnt, const uint32_t *deg, uint32_t V, double alpha, double *rank,
                         double *contrib, double *acc, double *dangling, cudaStream_t s) {
    ProfScope ps_("pagerank", s);
    k_zero_f64<<<1, 1, 0, s>>>(dangling);
    k_pr_contrib<<<grid_for(V, TPB, 152 * 8), TPB, 0, s>>>(rank, deg, V, contrib, dangling);
    k_pr_push<<<grid_for(nseg_of(g.H), TPB / 8, 152 * 16), TPB, 0, s>>>(g, cnt, contrib, acc);
    k_pr_finish<<<grid_for(V, TPB, 152 * 8), TPB, 0, s>>>(rank, acc, V, alpha, dangling);
    note_launch(4);
}

}  // namespace lpma
