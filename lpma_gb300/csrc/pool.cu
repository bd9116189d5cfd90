// Request pool over many resident graphs: the batched (many graphs per
// round) and served (requests arriving over time) forms of the update path.
//
// Worker threads, each with its own CUDA stream, take requests from one
// queue.  Requests on different graphs run at the same time on different
// streams; requests on one graph run one at a time in submission order (a
// graph's structure changes with every update).  A request is admitted
// only while the resident graphs plus the scratch of the requests in flight
// fit the HBM budget.  A request is complete when its GPU work is: the
// worker synchronises its stream before it releases the graph.
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include <cuda_runtime.h>

#include "gpma.cuh"
#include "lpma.h"
#include "prims.cuh"

namespace {

uint64_t now_ns() {
    return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

// device scratch a request needs beyond the graph itself (bytes)
uint64_t scratch_estimate(const LpmaRequest *r, uint32_t V) {
    switch (r->kind) {
        case LPMA_REQ_UPDATE: return 64ull * (r->n0 + r->n1) + (1u << 20);
        case LPMA_REQ_NEIGHBORS: return 16ull * r->nv + (1u << 16);
        case LPMA_REQ_BFS: return 12ull * V + (1u << 16);
        case LPMA_REQ_EDGE_QUERY: return 16ull * r->n0;
    }
    return 0;
}

}  // namespace

struct LpmaPool {
    std::mutex mu;
    std::condition_variable work_cv, done_cv;
    std::deque<LpmaRequest *> queue;
    std::unordered_map<LpmaHandle *, uint32_t> busy;        // graphs with a request in flight
    std::unordered_set<LpmaHandle *> seen;                  // scratch of take()
    std::unordered_map<LpmaHandle *, uint64_t> resident;    // device bytes of each graph seen
    uint64_t resident_total = 0, inflight = 0, budget = 0;
    uint32_t running = 0, pending = 0;
    bool stop = false;
    std::vector<std::thread> workers;
    int device = 0;

    LpmaRequest *take(uint64_t &est) {
        std::unique_lock<std::mutex> lk(mu);
        for (;;) {
            if (stop) return nullptr;
            // the oldest request of each graph goes first: a later request
            // of a graph must not overtake an earlier one, admitted or not
            seen.clear();
            for (auto it = queue.begin(); it != queue.end(); ++it) {
                LpmaRequest *r = *it;
                if (!seen.insert(r->graph).second || busy.count(r->graph)) continue;
                uint32_t V = 0;
                lpma_info(r->graph, nullptr, nullptr, &V);
                const uint64_t e = scratch_estimate(r, V);
                if (running > 0 && budget && resident_total + inflight + e > budget) continue;
                queue.erase(it);
                busy[r->graph] = 1;
                inflight += e;
                running++;
                est = e;
                return r;
            }
            work_cv.wait(lk);
        }
    }

    void finish(LpmaRequest *r, uint64_t est) {
        uint64_t bytes = 0;
        lpma_memory_bytes(r->graph, &bytes);
        std::lock_guard<std::mutex> lk(mu);
        busy.erase(r->graph);
        inflight -= est;
        running--;
        uint64_t &old = resident[r->graph];
        resident_total = resident_total - old + bytes;
        old = bytes;
        pending--;
        r->done = 1;
        work_cv.notify_all();
        done_cv.notify_all();
    }

    void worker() {
        cudaSetDevice(device);
        cudaStream_t s = nullptr;
        cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        cudaEvent_t ev0 = nullptr, ev1 = nullptr;
        cudaEventCreate(&ev0);
        cudaEventCreate(&ev1);
        for (;;) {
            uint64_t est = 0;
            LpmaRequest *r = take(est);
            if (!r) break;
            r->t_start_ns = now_ns();
            const uint64_t pool0 = lpma::pool_reserved_bytes();
            cudaEventRecord(ev0, s);
            lpma_status_t st = LPMA_ERR_INVALID_ARGUMENT;
            const lpma_stream_t ls = (lpma_stream_t)s;
            switch (r->kind) {
                case LPMA_REQ_UPDATE:
                    st = r->host_inputs ? lpma_update_host(r->graph, r->keys0, r->vals0, r->n0, r->keys1, r->n1,
                                                           r->thres, ls, &r->stats)
                                        : lpma_update(r->graph, r->keys0, r->vals0, r->n0, r->keys1, r->n1, r->thres,
                                                      ls, &r->stats);
                    break;
                case LPMA_REQ_NEIGHBORS: {
                    size_t total = 0;
                    st = lpma_query_neighbors(r->graph, r->vertices, r->windows, r->nv, r->out_u32, r->out_nbrs,
                                              r->out_vals, r->cap, &total, ls);
                    r->reached = total;
                    break;
                }
                case LPMA_REQ_BFS:
                    st = lpma_bfs(r->graph, r->vertices, r->nv, r->max_depth, r->out_dist, &r->levels, &r->reached,
                                  ls);
                    break;
                case LPMA_REQ_EDGE_QUERY:
                    st = lpma_edge_query(r->graph, r->keys0, r->n0, r->thres, r->out_u32, ls);
                    break;
            }
            r->t_call_ns = now_ns();
            cudaEventRecord(ev1, s);
            const cudaError_t ce = lpma::host_wait(s, true);
            if (st == LPMA_OK && ce != cudaSuccess) st = LPMA_ERR_CUDA;
            r->status = st;
            r->t_end_ns = now_ns();
            float ms = 0.f;
            r->device_ms = cudaEventElapsedTime(&ms, ev0, ev1) == cudaSuccess ? ms : -1.f;
            const uint64_t pool1 = lpma::pool_reserved_bytes();
            r->pool_growth_bytes = pool1 > pool0 ? pool1 - pool0 : 0;
            finish(r, est);
        }
        cudaEventDestroy(ev0);
        cudaEventDestroy(ev1);
        cudaStreamDestroy(s);
    }
};

extern "C" {

lpma_status_t lpma_pool_create(uint32_t n_workers, uint64_t hbm_budget_bytes, LpmaPool **out) {
    if (!out || n_workers == 0 || n_workers > 256) return LPMA_ERR_INVALID_ARGUMENT;
    LpmaPool *p = new LpmaPool();
    p->budget = hbm_budget_bytes;
    if (cudaGetDevice(&p->device) != cudaSuccess) {
        delete p;
        return LPMA_ERR_CUDA;
    }
    for (uint32_t i = 0; i < n_workers; i++) p->workers.emplace_back([p] { p->worker(); });
    *out = p;
    return LPMA_OK;
}

lpma_status_t lpma_pool_submit(LpmaPool *p, LpmaRequest *r) {
    if (!p || !r || !r->graph || r->kind > LPMA_REQ_EDGE_QUERY) return LPMA_ERR_INVALID_ARGUMENT;
    r->done = 0;
    r->status = LPMA_OK;
    r->t_submit_ns = now_ns();
    r->t_start_ns = r->t_end_ns = 0;
    std::lock_guard<std::mutex> lk(p->mu);
    p->queue.push_back(r);
    p->pending++;
    p->work_cv.notify_one();
    return LPMA_OK;
}

lpma_status_t lpma_pool_submit_many(LpmaPool *p, LpmaRequest *reqs, size_t n) {
    if (!p || (n && !reqs)) return LPMA_ERR_INVALID_ARGUMENT;
    for (size_t i = 0; i < n; i++)
        if (!reqs[i].graph || reqs[i].kind > LPMA_REQ_EDGE_QUERY) return LPMA_ERR_INVALID_ARGUMENT;
    const uint64_t t = now_ns();
    std::lock_guard<std::mutex> lk(p->mu);
    for (size_t i = 0; i < n; i++) {
        LpmaRequest *r = &reqs[i];
        r->done = 0;
        r->status = LPMA_OK;
        r->t_submit_ns = t;
        r->t_start_ns = r->t_end_ns = 0;
        p->queue.push_back(r);
    }
    p->pending += (uint32_t)n;
    p->work_cv.notify_all();
    return LPMA_OK;
}

lpma_status_t lpma_pool_wait(LpmaPool *p, LpmaRequest *r) {
    if (!p || !r) return LPMA_ERR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lk(p->mu);
    p->done_cv.wait(lk, [r] { return r->done != 0; });
    return r->status;
}

lpma_status_t lpma_pool_drain(LpmaPool *p) {
    if (!p) return LPMA_ERR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lk(p->mu);
    p->done_cv.wait(lk, [p] { return p->pending == 0; });
    return LPMA_OK;
}

lpma_status_t lpma_pool_destroy(LpmaPool *p) {
    if (!p) return LPMA_ERR_INVALID_ARGUMENT;
    lpma_pool_drain(p);
    {
        std::lock_guard<std::mutex> lk(p->mu);
        p->stop = true;
        p->work_cv.notify_all();
    }
    for (std::thread &t : p->workers) t.join();
    delete p;
    return LPMA_OK;
}

}  // extern "C"
