"""The request pool (many graphs, concurrent workers) against the same
requests run one at a time through the plain entry points.

Each result must be the same alone and in the mix: the final layout of
every graph (slot for slot) and every neighbour-list / BFS answer, bit for
bit.  Requests on one graph keep their submission order in the pool.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(a, dtype=np.uint64):
    import torch
    a = np.ascontiguousarray(a, dtype=dtype)
    view = {np.uint64: np.int64, np.uint32: np.int32}.get(dtype, dtype)
    return torch.from_numpy(a.view(view)).cuda()


def _workload(oracle, n_graphs, seed):
    """Per graph: vertex count, bulk keys and a list of requests."""
    rng = np.random.default_rng(seed)
    graphs = []
    for gi in range(n_graphs):
        scale = int(rng.integers(8, 13))
        e = oracle.shuffle(oracle.rmat_edges(seed * 1000 + gi, scale, int(rng.integers(8, 20))), gi + 5)
        half = e.size // 2
        reqs, pos, stored = [], half, list(e[:half])
        for r in range(int(rng.integers(3, 7))):
            kind = rng.choice(["ins", "del", "mix", "nbr", "bfs"])
            b = int(np.exp(rng.uniform(np.log(10), np.log(3000))))
            if kind in ("ins", "mix"):
                ins = e[pos:pos + b]
                pos += ins.size
            else:
                ins = e[:0]
            if kind in ("del", "mix") and stored:
                dels = rng.choice(np.array(stored, np.uint64), size=min(b // 2 + 1, len(stored)), replace=False)
            else:
                dels = e[:0]
            if kind in ("ins", "del", "mix"):
                reqs.append(("upd", ins, dels))
                stored = sorted(set(stored) - set(dels.tolist()) | set(ins.tolist()))
            elif kind == "nbr":
                srcs = rng.integers(0, 1 << scale, 64).astype(np.uint32)
                reqs.append(("nbr", srcs, np.full(64, 0xFFFFFFFF, np.uint64)))
            else:
                reqs.append(("bfs", rng.integers(0, 1 << scale, 4).astype(np.uint32), int(rng.integers(0, 3))))
        graphs.append((1 << scale, e[:half], reqs))
    return graphs


def _run_alone(engine, graphs):
    out = []
    for V, bulk, reqs in graphs:
        g = engine.Lpma(V)
        g.update(ins=_dev(bulk))
        res = []
        for r in reqs:
            if r[0] == "upd":
                g.update(ins=_dev(r[1]), dels=_dev(r[2]))
            elif r[0] == "nbr":
                o, n, v = g.query_neighbors(_dev(r[1], np.uint32), _dev(r[2]))
                res.append((o.cpu().numpy(), n.cpu().numpy(), v.cpu().numpy()))
            else:
                d, _, _ = g.bfs(_dev(r[1], np.uint32), r[2])
                res.append((d.cpu().numpy(),))
        k, v, s, h = g.layout()
        out.append((res, k, v, s, h))
        g.close()
    return out


def _run_pool(engine, graphs, workers, budget=0):
    import torch
    from lpma_gb300 import rpma
    pool = rpma.Pool(workers, budget)
    handles, pending = [], []
    for V, bulk, reqs in graphs:
        g = engine.Lpma(V, config=rpma.default_config(flags=1))
        g.update(ins=_dev(bulk))
        handles.append(g)
    # submit everything at once, interleaving graphs round by round
    depth = max(len(r) for _, _, r in graphs)
    for i in range(depth):
        for gi, (V, _, reqs) in enumerate(graphs):
            if i >= len(reqs):
                continue
            r, g = reqs[i], handles[gi]
            if r[0] == "upd":
                pending.append((gi, None, pool.update(g, ins=_dev(r[1]), dels=_dev(r[2]))))
            elif r[0] == "nbr":
                srcs, wins = _dev(r[1], np.uint32), _dev(r[2])
                offs = torch.empty(srcs.numel() + 1, dtype=torch.int32, device="cuda")
                nbrs = torch.empty(1 << 18, dtype=torch.int32, device="cuda")
                vals = torch.empty(1 << 18, dtype=torch.uint8, device="cuda")
                pending.append((gi, ("nbr", offs, nbrs, vals), pool.neighbors(g, srcs, wins, offs, nbrs, vals)))
            else:
                dist = torch.empty(V, dtype=torch.int32, device="cuda")
                pending.append((gi, ("bfs", dist), pool.bfs(g, _dev(r[1], np.uint32), dist, r[2])))
    pool.drain()
    res = [[] for _ in graphs]
    for gi, outs, req in pending:
        assert req.done == 1 and req.status == 0, req.status
        assert req.t_submit_ns <= req.t_start_ns <= req.t_end_ns
        if outs is None:
            continue
        if outs[0] == "nbr":
            tot = int(req.reached)
            res[gi].append((outs[1].cpu().numpy(), outs[2][:tot].cpu().numpy(), outs[3][:tot].cpu().numpy()))
        else:
            res[gi].append((outs[1].cpu().numpy(),))
    out = []
    for gi, g in enumerate(handles):
        k, v, s, h = g.layout()
        out.append((res[gi], k, v, s, h))
        g.close()
    pool.close()
    return out


def _same(a, b):
    for (ra, ka, va, sa, ha), (rb, kb, vb, sb, hb) in zip(a, b):
        assert ha == hb and np.array_equal(ka, kb) and np.array_equal(va, vb) and np.array_equal(sa, sb)
        assert len(ra) == len(rb)
        for x, y in zip(ra, rb):
            for p, q in zip(x, y):
                assert np.array_equal(p, q)


def test_pool_results_equal_alone(engine, oracle):
    graphs = _workload(oracle, 24, 3)
    alone = _run_alone(engine, graphs)
    _same(alone, _run_pool(engine, graphs, workers=8))


def test_pool_one_graph_keeps_order(engine, oracle):
    """Many requests on one graph: the pool applies them in submission order."""
    graphs = _workload(oracle, 1, 11)
    V, bulk, reqs = graphs[0]
    # delete, re-insert and delete again overlapping key ranges: only the
    # submission order gives the sequential result
    extra = [("upd", bulk[:0], bulk[:300]), ("upd", bulk[100:200], bulk[:0]), ("upd", bulk[:0], bulk[150:400]),
             ("upd", bulk[:250], bulk[:0]), ("upd", bulk[:0], bulk[240:260])]
    graphs = [(V, bulk, reqs + extra)]
    _same(_run_alone(engine, graphs), _run_pool(engine, graphs, workers=4))


def test_pool_small_budget_still_completes(engine, oracle):
    graphs = _workload(oracle, 6, 21)
    _same(_run_alone(engine, graphs), _run_pool(engine, graphs, workers=4, budget=1))
