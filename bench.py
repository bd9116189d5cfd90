#!/usr/bin/env python3
"""Benchmark of the LPMA batched edge-update path on one GB300.

Workload (the reference metric's configuration): directed R-MAT, scale 21
(2,097,152 vertices), edge factor 16, (a,b,c,d) = (.57,.19,.19,.05), seeded;
self loops and duplicates removed; shuffled; 50% bulk-loaded.  A step is one
update call of B edges (B = 1,048,576 by default), alternately an insert
batch drawn from the unloaded edges and a delete batch drawn from the stored
ones (uniform: the bulk is a shuffled sample); deleted edges return to the
insert pool.  The same stream at batch sizes 1K/10K/100K is reported under
"per_batch_size".  Inputs are generated on the device and stay resident in
HBM; the PMA working set (0.3-0.6 GB) is larger than the 129 MB L2, so no L2
flush is done between steps.

--impl reference runs the CPU baseline (sorted-merge CSR rebuild per batch on
the host cores, the reference's CPU path) on the same workload and metric.
"""
import argparse
import ctypes
import gc
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "updated edges/s vs batch size on 1 GB300 (bit-exact); served p50/p99 batch latency"
WORKLOAD = "rmat-s%d-ef%d stream, 50%% bulk, alternating insert/delete batches"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=4)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--batch", type=int, default=1 << 20)
    ap.add_argument("--scale", type=int, default=21)
    ap.add_argument("--ef", type=int, default=16)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--sweep", default="1024,10240,102400")
    ap.add_argument("--sweep-steps", type=int, default=20)
    ap.add_argument("--cpu-steps", type=int, default=10)
    ap.add_argument("--no-autotune", action="store_true",
                    help="skip the batch-sort autotuner (lpma_autotune) before the stream")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="stream", choices=["stream", "multigraph", "served", "skew", "gpma"],
                    help="stream: the single-graph update stream (the headline line); multigraph: 256 graphs, one "
                         "batch each per round, pooled vs one plain call per graph; served: Poisson arrivals over "
                         "64 resident graphs, pooled vs one request at a time; skew: hub-heavy mixed batches on "
                         "2^20 vertices with 64M edges (resize stress); gpma: the stream on a GPMA-mode handle")
    ap.add_argument("--graphs", type=int, default=256)
    ap.add_argument("--rounds", type=int, default=6)
    ap.add_argument("--workers", type=int, default=16)
    ap.add_argument("--rates", default="500,2000,8000", help="served: Poisson arrival rates (requests/s)")
    ap.add_argument("--duration", type=float, default=3.0, help="served: seconds of arrivals per rate")
    return ap.parse_args()


def max_over_ranks(t, device=None):
    """Slowest rank's time (torch.distributed; NCCL on GPUs, gloo on CPU)."""
    import torch
    import torch.distributed as dist
    if not dist.is_initialized() or dist.get_world_size() == 1:
        return float(t)
    tt = torch.tensor([float(t)], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def replica_seed(seed, rank):
    """Replicas only: each rank updates its own graph from its own stream."""
    return seed + 7919 * rank


def l2_copy_gbs(device):
    """Copy bandwidth with both buffers resident in the 129 MB L2 (two 32 MB
    tensors copied back and forth, read + write bytes over CUDA-event time,
    best of 5): the bound of kernels whose passes run out of L2."""
    import torch
    a = torch.empty(4 << 20, dtype=torch.int64, device=device)
    b = torch.empty_like(a)
    a.fill_(1)
    for _ in range(20):
        b.copy_(a)
        a.copy_(b)
    best = 0.0
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(50):
            b.copy_(a)
            a.copy_(b)
        e1.record()
        torch.cuda.synchronize()
        best = max(best, 100 * 2 * a.numel() * 8 / (e0.elapsed_time(e1) / 1e3) / 1e9)
    return best


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class _Nvml:
    """Read-only NVML queries through the driver's libnvidia-ml (ctypes):
    the SM clock, its maximum and the active clock-event (throttle)
    reasons.  Nothing is set."""

    SM = 1
    REASONS = {"sw_power_cap": 0x4, "hw_slowdown": 0x8, "sw_thermal_slowdown": 0x20, "hw_thermal_slowdown": 0x40,
               "hw_power_brake_slowdown": 0x80}

    def __init__(self, pci_bus_id=None, index=0):
        self.lib = ctypes.CDLL("libnvidia-ml.so.1")
        if self.lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        self.h = ctypes.c_void_p()
        rc = 1
        if pci_bus_id:
            rc = self.lib.nvmlDeviceGetHandleByPciBusId_v2(pci_bus_id.encode(), ctypes.byref(self.h))
        if rc != 0:
            rc = self.lib.nvmlDeviceGetHandleByIndex_v2(index, ctypes.byref(self.h))
        if rc != 0:
            raise OSError("no NVML handle")
        mx = ctypes.c_uint()
        self.lib.nvmlDeviceGetMaxClockInfo(self.h, self.SM, ctypes.byref(mx))
        self.max_mhz = mx.value

    def sample(self):
        c, r = ctypes.c_uint(), ctypes.c_ulonglong()
        self.lib.nvmlDeviceGetClockInfo(self.h, self.SM, ctypes.byref(c))
        fn = getattr(self.lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            self.lib.nvmlDeviceGetCurrentClocksThrottleReasons
        fn(self.h, ctypes.byref(r))
        return c.value, r.value


class Clocks:
    """SM clock and throttle reasons sampled during the timed region: NVML
    every 2 ms (the region of a 200-step run lasts about 65 ms), else
    nvidia-smi every 100 ms."""

    def __init__(self, index=0, pci_bus_id=None):
        self.samples = []
        self.index = index
        self.pci = pci_bus_id
        self.proc = None
        self.nvml = None
        self.stop = False

    def __enter__(self):
        try:
            self.nvml = _Nvml(self.pci, self.index)
            self.t = threading.Thread(target=self._poll, daemon=True)
            self.t.start()
            return self
        except Exception:
            self.nvml = None
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _poll(self):
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        while not self.stop:
            mhz, rs = self.nvml.sample()
            self.samples.append([str(mhz), str(self.nvml.max_mhz), ""] +
                                ["Active" if rs & _Nvml.REASONS[n] else "Not Active" for n in names])
            time.sleep(0.002)

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 7:
                self.samples.append(parts)

    def __exit__(self, *a):
        self.stop = True
        if self.nvml:
            self.t.join(timeout=1)
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = [n for i, n in enumerate(names) if any(s[3 + i].lower() == "active" for s in self.samples)]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples), "source": "nvml" if self.nvml else "nvidia-smi"}


class Stream:
    """Insert/delete batches over the cyclic sequences (U ++ S) and (S ++ U)."""

    def __init__(self, ins_seq, del_seq):
        self.ins_seq, self.del_seq = ins_seq, del_seq
        self.ci = self.cd = 0
        self.n = ins_seq.shape[0]

    def next(self, kind, B):
        if kind == "ins":
            a = self.ci
            self.ci += B
            seq = self.ins_seq
        else:
            a = self.cd
            self.cd += B
            seq = self.del_seq
        # cyclic: past the end the sequence starts over (inserts of U ++ S and
        # deletes of S ++ U advance together, so a full cycle returns the
        # stored set to S)
        a %= self.n
        if a + B <= self.n:
            return seq[a:a + B]
        import torch
        return torch.cat([seq[a:], seq[:a + B - self.n]])


def build_workload(args, device, seed):
    import torch
    import lpma_gb300 as L
    n_raw = (1 << args.scale) * args.ef
    raw = torch.empty(n_raw, dtype=torch.int64, device=device)
    n = L.gen_rmat_device(seed, args.scale, args.ef, raw)
    e = raw[:n]
    L.shuffle_device(seed + 1000, e)
    half = n // 2
    S, U = e[:half], e[half:]
    ins_seq = torch.cat([U, S])
    del_seq = torch.cat([S, U])
    return e, S, ins_seq, del_seq


MIX = 0x9E3779B97F4A7C15
M64 = (1 << 64) - 1


def key_checksum_dev(t):
    """(sum k, sum (k * MIX) ^ (k >> 31)) mod 2^64 of an int64 device tensor
    of keys below 2^63 (two's-complement sums wrap)."""
    import torch
    a = int(t.sum()) & M64
    b = int(torch.bitwise_xor(t * (MIX - (1 << 64)), t >> 31).sum()) & M64
    return a, b


def key_checksum_host(k):
    k = np.asarray(k, dtype=np.uint64)
    with np.errstate(over="ignore"):
        a = int(k.sum(dtype=np.uint64))
        b = int(((k * np.uint64(MIX)) ^ (k >> np.uint64(31))).sum(dtype=np.uint64))
    return a, b


class SetCheck:
    """Size-independent checks of the stored set, outside the timed region:
    every batch of the stream inserts only new keys and deletes only stored
    ones, so each call must report exactly B applied updates; the stored set
    (export_sorted, sentinels included) must be strictly sorted, of the
    expected size, and its two checksums must equal the bulk's plus the
    inserted batches' minus the deleted batches' (computed on the device
    from the batches); the CSR view must hold one sentinel-closed row per
    vertex."""

    def __init__(self, S, V):
        import torch
        sent = (torch.arange(V, dtype=torch.int64, device=S.device) << 42) + 0x000003FFFFEFFFFF
        a1, b1 = key_checksum_dev(S)
        a2, b2 = key_checksum_dev(sent)
        self.sum = [(a1 + a2) & M64, (b1 + b2) & M64]
        self.count = int(S.numel()) + V
        self.V = V
        self.batches = 0
        self.stat_errors = 0
        self.points = []

    def batch(self, kind, x, st, B):
        a, b = key_checksum_dev(x)
        sign = 1 if kind == "ins" else -1
        self.sum = [(self.sum[0] + sign * a) & M64, (self.sum[1] + sign * b) & M64]
        self.count += sign * int(x.numel())
        want = (B, 0) if kind == "ins" else (0, B)
        if (st["n_ins_applied"], st["n_del_applied"]) != want:
            self.stat_errors += 1
        self.batches += 1

    def point(self, g, where):
        k, _ = g.export_sorted()
        ok_count = k.size == self.count
        ok_sorted = bool(k.size < 2 or (k[1:] > k[:-1]).all())
        ok_sum = list(key_checksum_host(k)) == self.sum
        ro, ci, _ = g.to_csr()
        ends = ro[1:].astype(np.int64) - 1
        ok_csr = bool(ro[0] == 0 and (np.diff(ro.astype(np.int64)) >= 1).all() and ro[-1] == k.size and
                      (ci[ends] == np.arange(self.V, dtype=np.uint32)).all())
        self.points.append({"after": where, "keys": int(k.size), "count": ok_count, "sorted": ok_sorted,
                            "checksums": ok_sum, "csr": ok_csr})

    def summary(self):
        ok = self.stat_errors == 0 and all(p["count"] and p["sorted"] and p["checksums"] and p["csr"]
                                           for p in self.points)
        return {"ok": ok, "batches": self.batches, "batches_with_wrong_counts": self.stat_errors,
                "points": self.points}


def gpu_arm(args, rank, world):
    import torch
    import lpma_gb300 as L
    device = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(device)
    V = 1 << args.scale
    tiers = None
    if not args.no_autotune:
        # sort tier per batch-size bucket, timed on this GPU (outside every timed region)
        from lpma_gb300 import rpma
        tiers = {str(r["keys"]): r["tier"] for r in rpma.autotune(max(args.batch, 1 << 11)) if not r["concurrent"]}
    e, S, ins_seq, del_seq = build_workload(args, device, replica_seed(args.seed, rank))
    grain = big_alt = None
    if not args.no_autotune:
        # executor cut-overs for this batch size, timed on a scratch copy of
        # the graph that first runs 20 batches of the stream (the windows of
        # a fill cycle), with the stream's next insert batch (absent keys);
        # the timed handle is not touched
        from lpma_gb300 import rpma
        scratch = L.Lpma(V)
        scratch.build(S)
        sst = Stream(ins_seq, del_seq)
        for i in range(20):
            kind = ("ins", "del")[i % 2]
            x = sst.next(kind, args.batch)
            scratch.update(ins=x) if kind == "ins" else scratch.update(dels=x)
        try:
            timed = rpma.autotune_grain(scratch, sst.next("ins", args.batch), reps=3)
        except L.LpmaError as ex:  # a small graph: the stream's next batch holds stored keys
            timed = str(ex)
        grain = {"timed": timed, "chosen": rpma.grain_get(int(args.batch - 1).bit_length())}
        # the big windows' class: the scratch copy goes on through the stream,
        # profiled, until one of its batches executes a root window (60 at
        # most).  Root windows and rebuilds come early in this stream (the
        # rebuilds settle the tree at a height where the root rarely fills
        # again), so the profiled steps after the timed ones may hold none.
        L.profile_enable(True)
        bst = []
        for i in range(60):
            kind = ("ins", "del")[i % 2]
            x = sst.next(kind, args.batch)
            s_ = scratch.update(ins=x) if kind == "ins" else scratch.update(dels=x)
            bst.append(s_)
            if s_["slots_rewritten"] > s_["slots_small"]:
                break
        torch.cuda.synchronize()
        big_alt = {"prof": L.profile_report(), "pstats": bst,
                   "source": "a scratch copy of the graph after 20 batches of the stream and the cut-over "
                             "tuning: %d more batches, up to its first root window" % len(bst)}
        L.profile_enable(False)
        scratch.close()
    g = L.Lpma(V)
    g.build(S)
    check = SetCheck(S, V)
    st = Stream(ins_seq, del_seq)
    kinds = ["ins", "del"]
    stream = torch.cuda.current_stream()

    def step(kind, B):
        batch = st.next(kind, B)
        s_ = g.update(ins=batch) if kind == "ins" else g.update(dels=batch)
        return batch, s_

    # per-batch-size sweep (1K, 10K, 100K): same stream, 20 steps each
    sweep = {}
    peak, _ = peaks()
    for B in [int(x) for x in args.sweep.split(",") if x]:
        for i in range(2):
            x, s_ = step(kinds[i % 2], B)
            check.batch(kinds[i % 2], x, s_, B)
        # the batches (views of the resident stream) are cut before the
        # timed region: it holds the update calls and their events only
        sw_batches = [(kinds[i % 2], st.next(kinds[i % 2], B)) for i in range(args.sweep_steps)]
        torch.cuda.synchronize()
        evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.sweep_steps + 1)]
        sw_stats = []
        evs[0].record(stream)
        for i, (k_, x) in enumerate(sw_batches):
            sw_stats.append(g.update(ins=x) if k_ == "ins" else g.update(dels=x))
            evs[i + 1].record(stream)
        torch.cuda.synchronize()
        for (k_, x), s_ in zip(sw_batches, sw_stats):
            check.batch(k_, x, s_, B)
        lat = [evs[i].elapsed_time(evs[i + 1]) for i in range(args.sweep_steps)]
        tot = sum(lat) / 1e3
        alg = sum(16 * B + 18 * s_["slots_rewritten"] for s_ in sw_stats)
        sweep[str(B)] = {"edges_per_s": B * args.sweep_steps / tot, "p50_ms": float(np.percentile(lat, 50)),
                         "p99_ms": float(np.percentile(lat, 99)), "hbm_GBps": alg / tot / 1e9,
                         "hbm_frac": alg / tot / 1e9 / peak}

    # main: W warmup + K timed steps at B
    B = args.batch
    for i in range(args.warmup):
        x, s_ = step(kinds[i % 2], B)
        check.batch(kinds[i % 2], x, s_, B)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    props = torch.cuda.get_device_properties(device)
    pci = None
    if all(hasattr(props, a) for a in ("pci_domain_id", "pci_bus_id", "pci_device_id")):
        pci = "%08X:%02X:%02X.0" % (props.pci_domain_id, props.pci_bus_id, props.pci_device_id)
    clk = Clocks(device.index, pci).__enter__()
    if not clk.nvml:
        time.sleep(0.3)  # nvidia-smi needs a moment before its first sample
    batches = [(kinds[(args.warmup + i) % 2], st.next(kinds[(args.warmup + i) % 2], B)) for i in range(args.steps)]
    torch.cuda.synchronize()
    launches0 = L.kernel_launches()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    stats = []
    t0 = time.perf_counter()
    evs[0].record(stream)
    for i, (k_, x) in enumerate(batches):
        stats.append(g.update(ins=x) if k_ == "ins" else g.update(dels=x))
        evs[i + 1].record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clk.__exit__()
    if world > 1:
        torch.distributed.barrier()
    launches = L.kernel_launches() - launches0
    lat = [evs[i].elapsed_time(evs[i + 1]) for i in range(args.steps)]
    t = max_over_ranks(evs[0].elapsed_time(evs[-1]) / 1e3, device)
    # the check of the timed steps, after the timed region
    for (k_, x), s_ in zip(batches, stats):
        check.batch(k_, x, s_, B)
    del batches
    check.point(g, "timed steps")

    # roofline: per-kernel CUDA events over K more steps of the same stream
    L.profile_enable(True)
    pstats = []
    # at least 30 steps, then on until a root window (one every 25 to 70
    # batches on this stream, not periodic) is among them, 150 at most: the
    # big windows' class is measured too
    prof_steps = 0
    while prof_steps < min(args.steps, 150):
        k_ = kinds[(args.warmup + args.steps + prof_steps) % 2]
        x, s_ = step(k_, B)
        pstats.append(s_)
        check.batch(k_, x, s_, B)
        prof_steps += 1
        if prof_steps >= min(args.steps, 30) and any(p["slots_rewritten"] > p["slots_small"] for p in pstats):
            break
    torch.cuda.synchronize()
    prof = L.profile_report()
    L.profile_enable(False)

    # end to end through the host entry point: pinned host batch -> lpma_update_host
    e2e_steps = min(args.steps, 50)
    e2e_warm = 2  # untimed: the host entry allocates its staging buffers on first use
    host_batches = []
    for i in range(e2e_warm + e2e_steps):
        k = (args.warmup + args.steps + prof_steps + i) % 2
        b = st.next(kinds[k], B)
        hb = torch.empty(B, dtype=torch.int64, pin_memory=True)
        hb.copy_(b)
        host_batches.append((k, hb.numpy().view(np.uint64), b))
    warm_stats = [g.update(ins=hb) if k == 0 else g.update(dels=hb) for k, hb, _ in host_batches[:e2e_warm]]
    torch.cuda.synchronize()
    e2e_stats = []
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    t_e0 = time.perf_counter()
    for k, hb, _ in host_batches[e2e_warm:]:
        e2e_stats.append(g.update(ins=hb) if k == 0 else g.update(dels=hb))
    ev1.record(stream)
    torch.cuda.synchronize()
    t_e2e = max(ev0.elapsed_time(ev1) / 1e3, time.perf_counter() - t_e0)
    h2d = sum(s_["h2d_bytes"] for s_ in e2e_stats) / len(e2e_stats)
    d2h = sum(s_["d2h_bytes"] for s_ in e2e_stats) / len(e2e_stats)
    for (k, _, b), s_ in zip(host_batches, warm_stats + e2e_stats):
        check.batch(kinds[k], b, s_, B)
    check.point(g, "end-to-end steps")
    info = g.info()
    res = {"t": t, "lat": lat, "wall": wall, "launches": launches, "clocks": clk.summary(), "stats": stats,
           "pstats": pstats, "prof": prof, "sweep": sweep, "t_e2e": t_e2e, "e2e_steps": e2e_steps, "h2d": h2d, "d2h": d2h,
           "n_edges": int(e.shape[0]), "height": info["height"], "items": info["num_items"], "sort_tiers": tiers,
           "check": check.summary(), "l2_gbs": l2_copy_gbs(device), "grain": grain, "big_alt": big_alt}
    host_edges = None
    if rank == 0 and not args.no_cpu_baseline:
        host_edges = (e.cpu().numpy().view(np.uint64), int(S.shape[0]))
    g.close()
    return res, host_edges


def roofline(res, B, peak, peak_kind, name=None):
    """The dominant kernel's (or `name`'s) algorithmic bytes per launch over
    its average launch time, against the measured HBM and L2 bandwidths."""
    prof = res["prof"]
    if not prof:
        return None
    if name is None:
        name = max(prof, key=lambda k: prof[k][1])
    if name not in prof:
        return None
    cnt, ms = prof[name]
    pst = res["pstats"]
    # algorithmic bytes per launch of the dominant kernel
    if name == "exec_single":
        units = sum(32 * s["windows_single"] for s in pst) / cnt
        per_unit, unit_name = 18, "window slot (8 B key + 1 B value, read and written)"
    elif name == "exec_small":
        units = sum(s["slots_small"] - 32 * s["windows_single"] for s in pst) / cnt
        per_unit, unit_name = 18, "window slot (8 B key + 1 B value, read and written)"
    elif name == "exec_tiles":
        units = sum(s["slots_rewritten"] - s["slots_small"] for s in pst) / cnt
        per_unit, unit_name = 18, "window slot (8 B key + 1 B value, read and written)"
    elif name == "sort_coop":
        units = sum(B * s["sort_passes"] for s in pst) / cnt
        per_unit, unit_name = 20, "key per digit pass (8 B key + 2 B payload, read and written)"
    elif name in ("sort_pass", "sort_downsweep"):
        units = B
        per_unit, unit_name = 20, "key (8 B key + 2 B payload, read and written)"
    elif name == "sort_upsweep":
        units = B
        per_unit, unit_name = 8, "key (8 B read)"
    elif name == "resolve_locate":
        units = B
        per_unit, unit_name = 15, "key (8 B key + 2 B payload read, 1 B kind + 4 B segment written)"
    else:
        units, per_unit, unit_name = B, 8, "key"
    alg = units * per_unit
    avg_s = ms / cnt / 1e3
    achieved = alg / avg_s / 1e9
    traffic = None
    tf = os.path.join(ROOT, "profiles", "traffic_per_launch.txt")
    if os.path.exists(tf):
        for line in open(tf):
            p = line.split()
            if len(p) >= 3 and p[0] == name:
                traffic = float(p[1]) * (units / float(p[2]) if float(p[2]) else 1.0)
    l2 = res.get("l2_gbs")
    return {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
            "l2_peak": l2, "l2_frac": (achieved / l2) if l2 else None,
            "l2_peak_kind": "measured in this run (L2-resident copy, 2 x 32 MB)",
            "bytes_per_launch": alg, "per_unit_bytes": per_unit, "unit_desc": unit_name,
            "launches": cnt, "avg_launch_us": avg_s * 1e6,
            "kernel_share": {k: round(v[1] / sum(x[1] for x in prof.values()), 4) for k, v in prof.items()},
            "kernel_ms_per_step": {k: round(v[1] / len(pst), 4) for k, v in prof.items()}}


REBALANCE_CLASSES = (
    ("single", ("exec_single",)),
    ("small", ("exec_small", "exec_small4", "exec_small32")),
    ("big", ("exec_gather", "exec_spread", "seg_counts", "seg_q", "scan")),
)


def rebalance_roofline(res, peak, peak_kind):
    """Window rewrites of the profiled steps, by executor class and in total:
    18 B per rewritten slot (8 B key + 1 B value, read and written) over the
    summed device time of the class's kernels.  single: one-segment windows;
    small: 2..32 segments; big: larger windows, the root and rebuilds
    (gather / spread with their tile preparation)."""
    prof, pst = res["prof"], res["pstats"]
    if not prof or not pst:
        return None
    n = len(pst)
    single = sum(32 * s["windows_single"] for s in pst) / n
    small = sum(s["slots_small"] for s in pst) / n - single
    big = sum(s["slots_rewritten"] - s["slots_small"] for s in pst) / n
    out = {"peak": peak, "unit": "GB/s", "peak_kind": peak_kind, "steps": n,
           "big_window_steps": sum(1 for s in pst if s["slots_rewritten"] > s["slots_small"])}
    tot_b = tot_ms = 0.0
    for (name, ks), slots in zip(REBALANCE_CLASSES, (single, small, big)):
        ms = sum(prof[k][1] for k in ks if k in prof) / n
        b = 18 * slots
        tot_b += b
        tot_ms += ms
        out[name] = {"bytes_per_step": b, "ms_per_step": ms,
                     "achieved": b / (ms / 1e3) / 1e9 if ms else 0.0,
                     "frac": (b / (ms / 1e3) / 1e9 / peak) if ms else 0.0}
    out["all"] = {"bytes_per_step": tot_b, "ms_per_step": tot_ms, "achieved": tot_b / (tot_ms / 1e3) / 1e9,
                  "frac": tot_b / (tot_ms / 1e3) / 1e9 / peak}
    alt = res.get("big_alt")
    if not big and alt and alt["pstats"] and alt["prof"]:
        # no root window among these steps: the big class from the profiled
        # batches of a scratch copy of the graph up to its first root window
        ap, ps = alt["prof"], alt["pstats"]
        bb = sum(18 * (s["slots_rewritten"] - s["slots_small"]) for s in ps)
        bms = sum(ap[k][1] for k in REBALANCE_CLASSES[2][1] if k in ap)
        if bb and bms:
            out["big"] = {"bytes_per_step": bb / len(ps), "ms_per_step": bms / len(ps),
                          "achieved": bb / (bms / 1e3) / 1e9, "frac": bb / (bms / 1e3) / 1e9 / peak,
                          "source": alt["source"]}
    return out


def cpu_baseline(host_edges, B, steps, threads):
    from oracle import pyoracle as O
    edges, half = host_edges
    S, U = edges[:half], edges[half:]
    ins_seq = np.concatenate([U, S])
    del_seq = np.concatenate([S, U])
    V = int((edges.max() >> np.uint64(42)) + 1) if edges.size else 1
    c = O.CsrBaseline(max(V, 1 << 21), threads=threads)
    t0 = time.perf_counter()
    c.load(S)
    t_load = time.perf_counter() - t0
    lat = []
    n = ins_seq.size
    for i in range(steps):
        seq = ins_seq if i % 2 == 0 else del_seq
        a = ((i // 2) * B) % n  # cyclic, as the device stream
        b = seq[a:a + B] if a + B <= n else np.concatenate([seq[a:], seq[:a + B - n]])
        t0 = time.perf_counter()
        (c.insert if i % 2 == 0 else c.delete)(b)
        lat.append(time.perf_counter() - t0)
    c.close()
    return {"value": B * steps / sum(lat), "lat": lat, "load_s": t_load}


# ------------------------------------------------------------ many graphs
class GraphSet:
    """Independent directed R-MAT graphs, a = .57 b = .19 c = .19: vertex
    counts log-uniform over 2^10..2^18 (powers of two), edge factor uniform
    in 8..32, 50% preloaded, each with its own insert / delete pools."""

    def __init__(self, n, seed, flags=0, device="cuda"):
        import torch
        import lpma_gb300 as L
        from lpma_gb300 import rpma
        rng = np.random.default_rng(seed)
        self.graphs = []
        for i in range(n):
            scale = int(rng.integers(10, 19))
            ef = int(rng.integers(8, 33))
            raw = torch.empty((1 << scale) * ef, dtype=torch.int64, device=device)
            m = L.gen_rmat_device(seed * 100003 + i, scale, ef, raw)
            e = raw[:m].clone()
            del raw
            L.shuffle_device(seed + i, e)
            half = m // 2
            g = L.Lpma(1 << scale, config=rpma.default_config(flags=flags))
            g.build(e[:half])
            self.graphs.append({"g": g, "V": 1 << scale, "st": Stream(torch.cat([e[half:], e[:half]]),
                                                                      torch.cat([e[:half], e[half:]])),
                                "edges": m, "stored": half, "pool_left": m - half})
        torch.cuda.synchronize()

    def batch(self, gi, rng, lo=100, hi=100000, kind=None):
        """(kind, device batch) for graph gi: insert or delete (even odds), size
        log-uniform in [lo, hi], clamped to what the graph can take."""
        G = self.graphs[gi]
        kind = kind or ("ins" if rng.random() < 0.5 else "del")
        b = int(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        avail = G["pool_left"] if kind == "ins" else G["stored"]
        b = max(1, min(b, avail - 1)) if avail > 1 else 0
        if b == 0:
            kind = "del" if kind == "ins" else "ins"
            b = 1
        if G["st"].ci + b > G["st"].n or G["st"].cd + b > G["st"].n:
            G["st"].ci = G["st"].cd = 0  # wrap the cyclic pools (a fresh pass over the same edges)
        x = G["st"].next(kind, b)
        if kind == "ins":
            G["stored"] += b
            G["pool_left"] -= b
        else:
            G["stored"] -= b
            G["pool_left"] += b
        return kind, x

    def close(self):
        for G in self.graphs:
            G["g"].close()


def multigraph_arm(args):
    """256 graphs, one batch per graph per round, three ways: one plain
    update call per graph on one stream; every batch of a round submitted at
    once to the pool (concurrent workers, each graph's calls in order); and
    one lpma_update_batch call over all graphs (shared front launches)."""
    import torch
    from lpma_gb300 import rpma
    gs = GraphSet(args.graphs, args.seed, flags=0)
    rng = np.random.default_rng(args.seed + 1)
    pool = rpma.Pool(args.workers, 0)
    batcher = rpma.Batcher()
    modes = ("plain", "pooled", "batched")
    mode_flags = {"plain": 0, "pooled": 1, "batched": 0}
    res = {m: [] for m in modes}
    warm = 2 * len(modes)  # two rounds of each form: sizes seen twice get their captured front
    for r in range(args.rounds + warm):
        mode = modes[r % len(modes)]
        for G in gs.graphs:  # plain: the one-launch sort; pooled: sorts that may run side by side
            G["g"].set_flags(mode_flags[mode])
        work = [gs.batch(i, rng) for i in range(len(gs.graphs))]
        edges = sum(int(x.numel()) for _, x in work)
        torch.cuda.synchronize()
        lat = []
        t0 = time.perf_counter()
        if mode == "plain":
            # back to back on one stream; per-batch latency from CUDA events
            stream = torch.cuda.current_stream()
            evs = [torch.cuda.Event(enable_timing=True) for _ in range(len(work) + 1)]
            evs[0].record(stream)
            for i, (G, (k, x)) in enumerate(zip(gs.graphs, work)):
                G["g"].update(ins=x) if k == "ins" else G["g"].update(dels=x)
                evs[i + 1].record(stream)
            torch.cuda.synchronize()
            lat = [evs[i].elapsed_time(evs[i + 1]) / 1e3 for i in range(len(work))]
            done = [evs[0].elapsed_time(evs[i + 1]) / 1e3 for i in range(len(work))]
        elif mode == "pooled":
            reqs = pool.update_many([G["g"] for G in gs.graphs], [x for _, x in work], [k for k, _ in work])
            pool.drain()
            t_sub = min(q.t_submit_ns for q in reqs)
            done = []
            for q in reqs:
                assert q.status == 0, q.status
                lat.append((q.t_end_ns - q.t_start_ns) / 1e9)
                done.append((q.t_end_ns - t_sub) / 1e9)
        else:
            # every batch completes with the call: its latency is the call's
            _, status = batcher.update([G["g"] for G in gs.graphs],
                                       [{"ins": x} if k == "ins" else {"dels": x} for k, x in work])
            assert all(q == 0 for q in status), status
            lat = [time.perf_counter() - t0] * len(work)
            done = lat
        t = time.perf_counter() - t0
        if r >= warm:
            res[mode].append({"edges": edges, "t": t, "lat": lat, "done": done})
    pool.close()
    batcher.close()
    out = {}
    for mode, rounds in res.items():
        E = sum(x["edges"] for x in rounds)
        T = sum(x["t"] for x in rounds)
        lat = [l for x in rounds for l in x["lat"]]
        done = [l for x in rounds for l in x["done"]]
        out[mode] = {"edges_per_s": E / T, "round_ms": 1e3 * T / len(rounds),
                     "batch_p50_ms": 1e3 * float(np.percentile(lat, 50)),
                     "batch_p99_ms": 1e3 * float(np.percentile(lat, 99)),
                     "done_p50_ms": 1e3 * float(np.percentile(done, 50)),
                     "done_p99_ms": 1e3 * float(np.percentile(done, 99))}
    gs.close()
    line = {"metric": "aggregate updated edges/s over a round of one batch per graph", "workload":
            "%d R-MAT graphs, V log-uniform 2^10..2^18, edge factor 8..32, 50%% preloaded; one insert or delete batch "
            "per graph per round, size log-uniform 100..100K" % args.graphs,
            "unit": "edges/s", "rounds_per_mode": args.rounds // len(modes), "workers": args.workers,
            "plain": out["plain"], "pooled": out["pooled"], "batched": out["batched"],
            "speedup": out["pooled"]["edges_per_s"] / out["plain"]["edges_per_s"],
            "speedup_batched": out["batched"]["edges_per_s"] / out["plain"]["edges_per_s"],
            "note": "plain: one lpma_update per graph back to back on one stream, wall clock per round (host + "
                    "device), batch latency from CUDA events between calls; pooled: all batches of the round "
                    "submitted to lpma_pool at once, wall clock until drained, batch latency = service time; "
                    "batched: one lpma_update_batch call per round, wall clock, batch latency = the call's; "
                    "done_p50/p99: time from the round's start (all batches available) to each batch's "
                    "completion, the latency a caller with the whole round in hand sees"}
    print(json.dumps(line))


def served_arm(args):
    """Poisson arrivals over 64 resident graphs under a 150 GB admission
    budget: 70% updates (size log-uniform 1..1M, insert:delete 3:1), 30%
    reads (half neighbour list of a random vertex, half 2-hop BFS from 1,024
    random seeds).  The pool (continuous admission, concurrent graphs) vs the
    same arrivals served one request at a time."""
    import torch
    from lpma_gb300 import rpma
    gs = GraphSet(min(64, args.graphs), args.seed, flags=1)
    budget = 150 << 30
    # the update memory pool holds room for the graphs to grow before traffic
    # starts (no new device memory mapped under load)
    reserve = 32 << 30
    rpma.memory_reserve(reserve)
    # read outputs: one buffer set per graph (a graph's requests run one at a time)
    for G in gs.graphs:
        G["nbr_out"] = (torch.empty(2, dtype=torch.int32, device="cuda"),
                        torch.empty(1 << 20, dtype=torch.int32, device="cuda"),
                        torch.empty(1 << 20, dtype=torch.uint8, device="cuda"))
        G["dist"] = torch.empty(G["V"], dtype=torch.int32, device="cuda")
    out = {"rates": []}
    for rate in [float(x) for x in args.rates.split(",") if x]:
        row = {"rate_per_s": rate}
        for mode, workers in (("one_at_a_time", 1), ("pooled", args.workers)):
            rng = np.random.default_rng(int(rate) + 17)
            n_req = max(1, int(rate * args.duration))
            arrivals = np.cumsum(rng.exponential(1.0 / rate, n_req))
            plan = []
            for i in range(n_req):
                gi = int(rng.integers(0, len(gs.graphs)))
                G = gs.graphs[gi]
                u = rng.random()
                if u < 0.7:
                    kind = "ins" if rng.random() < 0.75 else "del"
                    k, x = gs.batch(gi, rng, 1, 1000000, kind)
                    plan.append(("upd", gi, k, x))
                elif u < 0.85:
                    src = torch.tensor([int(rng.integers(0, G["V"]))], dtype=torch.int32, device="cuda")
                    win = torch.full((1,), 0xFFFFFFFF, dtype=torch.int64, device="cuda")
                    plan.append(("nbr", gi, src, win) + G["nbr_out"])
                else:
                    seeds = torch.from_numpy(rng.integers(0, G["V"], 1024).astype(np.int32)).cuda()
                    plan.append(("bfs", gi, seeds, G["dist"]))
            torch.cuda.synchronize()
            pool = rpma.Pool(workers, budget)
            reqs = []
            # The load generator runs without Python's cyclic garbage
            # collector: its full collections over the request objects
            # stalled submissions by up to 54 ms at 8,000 requests/s, which
            # showed up as queueing of every request behind them.
            gc.collect()
            gc.disable()
            try:
                t0 = time.perf_counter()
                t0_ns = time.perf_counter_ns()  # the pool's clock (steady_clock) runs on the same monotonic source
                for at, p in zip(arrivals, plan):
                    d = t0 + at - time.perf_counter()
                    if d > 0:
                        time.sleep(d)
                    if p[0] == "upd":
                        G = gs.graphs[p[1]]["g"]
                        q = pool.update(G, ins=p[3]) if p[2] == "ins" else pool.update(G, dels=p[3])
                    elif p[0] == "nbr":
                        q = pool.neighbors(gs.graphs[p[1]]["g"], *p[2:])
                    else:
                        q = pool.bfs(gs.graphs[p[1]]["g"], p[2], p[3], 2)
                    q.arrival_ns = t0_ns + int(at * 1e9)
                    reqs.append((p[0], q, int(p[3].numel()) if p[0] == "upd" else 0))
                pool.drain()
                t = time.perf_counter() - t0
            finally:
                gc.enable()
            pool.close()
            stat = {"wall_s": t, "updated_edges_per_s": sum(e for _, _, e in reqs) / t}
            for kind in ("upd", "nbr", "bfs"):
                sel = [(q, e) for k, q, e in reqs if k == kind]
                lat = [(q.t_end_ns - min(q.t_submit_ns, q.arrival_ns)) / 1e6 for q, _ in sel]
                bad = sum(1 for q, _ in sel if q.status != 0)
                if lat:
                    # latency = queueing (arrival to a worker taking it) + service
                    wait = [(q.t_start_ns - min(q.t_submit_ns, q.arrival_ns)) / 1e6 for q, _ in sel]
                    serv = [(q.t_end_ns - q.t_start_ns) / 1e6 for q, _ in sel]
                    call = [(q.t_call_ns - q.t_start_ns) / 1e6 for q, _ in sel]
                    dev = [q.device_ms for q, _ in sel]
                    stat[kind] = {"n": len(lat), "p50_ms": float(np.percentile(lat, 50)),
                                  "p99_ms": float(np.percentile(lat, 99)), "errors": bad,
                                  "queue_p99_ms": float(np.percentile(wait, 99)),
                                  "service_p99_ms": float(np.percentile(serv, 99)),
                                  "call_p99_ms": float(np.percentile(call, 99)),
                                  "device_p99_ms": float(np.percentile(dev, 99)),
                                  "pool_growths": sum(1 for q, _ in sel if q.pool_growth_bytes)}
            # the slowest requests of the run: when each arrived, how long it
            # queued, how long it ran, its graph and size
            order = sorted(range(len(reqs)), key=lambda i: reqs[i][1].arrival_ns - reqs[i][1].t_end_ns)[:5]
            stat["slowest"] = [{"kind": reqs[i][0], "at_ms": round((reqs[i][1].arrival_ns - t0_ns) / 1e6, 2),
                                "queue_ms": round((reqs[i][1].t_start_ns - reqs[i][1].arrival_ns) / 1e6, 3),
                                "submit_lag_ms": round((reqs[i][1].t_submit_ns - reqs[i][1].arrival_ns) / 1e6, 3),
                                "service_ms": round((reqs[i][1].t_end_ns - reqs[i][1].t_start_ns) / 1e6, 3),
                                "graph": plan[i][1], "edges": reqs[i][2]} for i in order]
            order = sorted(range(len(reqs)), key=lambda i: reqs[i][1].t_start_ns - reqs[i][1].t_end_ns)[:5]
            stat["longest_service"] = [
                {"kind": reqs[i][0], "at_ms": round((reqs[i][1].arrival_ns - t0_ns) / 1e6, 2),
                 "service_ms": round((reqs[i][1].t_end_ns - reqs[i][1].t_start_ns) / 1e6, 3),
                 "call_ms": round((reqs[i][1].t_call_ns - reqs[i][1].t_start_ns) / 1e6, 3),
                 "device_ms": round(reqs[i][1].device_ms, 3),
                 "pool_growth_mb": round(reqs[i][1].pool_growth_bytes / 2 ** 20, 1), "graph": plan[i][1],
                 "edges": reqs[i][2], "height": [reqs[i][1].stats.height_before, reqs[i][1].stats.height_after],
                 "rebuilt": reqs[i][1].stats.rebuilt} for i in order]
            stat["resident_gb"] = sum(rpma.memory_bytes(G["g"]) for G in gs.graphs) / 1e9
            # how late the load generator submitted (a late submission is
            # counted as queueing, so it is reported)
            lag = [(q.t_submit_ns - q.arrival_ns) / 1e6 for _, q, _ in reqs]
            stat["submit_lag_ms"] = {"p99": float(np.percentile(lag, 99)), "max": float(max(lag))}
            row[mode] = stat
        out["rates"].append(row)
    gs.close()
    line = {"metric": "served p50/p99 request latency and updated edges/s at Poisson arrival rates",
            "workload": "%d resident R-MAT graphs (V 2^10..2^18, edge factor 8..32), 150 GB admission budget; 70%% "
                        "updates (log-uniform 1..1M, insert:delete 3:1), 15%% neighbour lists, 15%% 2-hop BFS from "
                        "1,024 seeds" % len(gs.graphs), "unit": "ms / edges/s", "workers": args.workers,
            "duration_s_per_rate": args.duration, "memory_reserve_gb": reserve / 2 ** 30, **out,
            "note": "latency = completion - planned arrival (queueing and submission lag included); one_at_a_time = "
                    "a pool of one worker; the load generator runs with Python's cyclic GC off"}
    print(json.dumps(line))


def skew_arm(args):
    """Skew and resize stress: 2^20 vertices, 32M uniform + 32M R-MAT
    (a = .7, b = c = .1) edges, 25% preloaded; every batch is 1M edges, half
    inserts (90% with a source among the top 1% out-degrees) and half deletes
    of preloaded edges."""
    import torch
    import lpma_gb300 as L
    scale, ef, B = 20, 32, args.batch
    V = 1 << scale
    raw = torch.empty(2 * V * ef, dtype=torch.int64, device="cuda")
    n1 = L.gen_rmat_device(args.seed, scale, ef, raw[:V * ef], a=0.25, b=0.25, c=0.25)
    n2 = L.gen_rmat_device(args.seed + 1, scale, ef, raw[V * ef:], a=0.7, b=0.1, c=0.1)
    e = torch.unique(torch.cat([raw[:n1], raw[V * ef:V * ef + n2]]))
    del raw
    L.shuffle_device(args.seed + 2, e)
    deg = torch.bincount(e >> 42, minlength=V)
    hub = torch.zeros(V, dtype=torch.bool, device="cuda")
    hub[torch.topk(deg, V // 100).indices] = True
    nb = e.numel() // 4
    bulk, rest = e[:nb], e[nb:]
    rest_hub = hub[rest >> 42]
    hub_pool, cold_pool = rest[rest_hub], rest[~rest_hub]
    g = L.Lpma(V)
    g.build(bulk)
    torch.cuda.synchronize()
    nh, nc, nd = int(B // 2 * 0.9), B // 2 - int(B // 2 * 0.9), B // 2
    steps = min(args.steps, hub_pool.numel() // nh - args.warmup, cold_pool.numel() // nc - args.warmup,
                nb // nd - args.warmup)

    def batch(i):
        ins = torch.cat([hub_pool[i * nh:(i + 1) * nh], cold_pool[i * nc:(i + 1) * nc]])
        return ins, bulk[i * nd:(i + 1) * nd]

    for i in range(args.warmup):
        ins, dels = batch(i)
        g.update(ins=ins, dels=dels)
    stream = torch.cuda.current_stream()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    stats = []
    torch.cuda.synchronize()
    evs[0].record(stream)
    for i in range(steps):
        ins, dels = batch(args.warmup + i)
        stats.append(g.update(ins=ins, dels=dels).as_dict())
        evs[i + 1].record(stream)
    torch.cuda.synchronize()
    lat = [evs[i].elapsed_time(evs[i + 1]) for i in range(steps)]
    t = sum(lat) / 1e3
    info = g.info()
    g.close()
    ev = {k: sum(x[k] for x in stats) for k in ("root_executed", "eager_levelup", "rebuilt", "levelup_path",
                                                 "fill_empty", "windows_big")}
    line = {"metric": "updated edges/s on hub-heavy mixed batches (skew and resize stress)", "value": B * steps / t,
            "unit": "edges/s", "steps": steps, "warmup": args.warmup,
            "workload": "2^20 vertices, %d edges (32M uniform + 32M R-MAT .7/.1/.1, deduplicated), 25%% preloaded; "
                        "batches of %d: %d inserts (90%% from the top-1%% out-degree sources) + %d deletes of stored "
                        "edges" % (e.numel(), B, B // 2, nd),
            "batch_p50_ms": float(np.percentile(lat, 50)), "batch_p99_ms": float(np.percentile(lat, 99)),
            "events": ev, "height_after": info["height"], "items_after": info["num_items"],
            "data": "synthetic (seeded device generators)"}
    print(json.dumps(line))


def gpma_arm(args):
    """GPMA mode (LPMA_FLAG_GPMA: the flat packed memory array of gpma.cuh)
    on the bench's stream: the same R-MAT graph, bulk half and alternating
    insert / delete batches of B edges, keys src << 32 | dst; CUDA events
    per batch on the update stream, inputs resident in HBM."""
    import torch
    import lpma_gb300 as L
    device = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    V = 1 << args.scale
    e, S, ins_seq, del_seq = build_workload(args, device, args.seed)

    def gk(x):
        return ((x >> 42) << 32) | ((x >> 20) & 0x3FFFFF)

    S, ins_seq, del_seq = gk(S), gk(ins_seq), gk(del_seq)
    g = L.Lpma(V, config=L.gpma_config())
    g.build(S)
    st = Stream(ins_seq, del_seq)
    kinds = ("ins", "del")
    B = args.batch
    for i in range(args.warmup):
        x = st.next(kinds[i % 2], B)
        g.update(ins=x) if i % 2 == 0 else g.update(dels=x)
    steps = min(args.steps, 100)
    stream = torch.cuda.current_stream()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    stats = []
    torch.cuda.synchronize()
    evs[0].record(stream)
    for i in range(steps):
        k = (args.warmup + i) % 2
        x = st.next(kinds[k], B)
        stats.append(g.update(ins=x) if k == 0 else g.update(dels=x))
        evs[i + 1].record(stream)
    torch.cuda.synchronize()
    lat = [evs[i].elapsed_time(evs[i + 1]) for i in range(steps)]
    t = sum(lat) / 1e3
    applied = sum(s_["n_ins_applied"] + s_["n_del_applied"] for s_ in stats)
    # per-kernel device time over 10 more batches (kernels timed one at a time)
    L.profile_enable(True)
    for i in range(10):
        k = (args.warmup + steps + i) % 2
        x = st.next(kinds[k], B)
        g.update(ins=x) if k == 0 else g.update(dels=x)
    torch.cuda.synchronize()
    prof = L.profile_report()
    L.profile_enable(False)
    (_, _, _), (size, seg, height) = g.gpma_view()
    info = g.info()
    g.close()
    line = {"metric": "updated edges/s, GPMA mode (the flat array of gpma.cuh), 1M-edge batches",
            "value": B * steps / t, "unit": "edges/s", "steps": steps, "warmup": args.warmup,
            "config": dict(config_of(args, int(e.shape[0]), 1), workload="rmat-s%d-ef%d stream in GPMA mode, 50%% bulk, "
                           "alternating insert/delete batches" % (args.scale, args.ef)),
            "batch_p50_ms": float(np.percentile(lat, 50)), "batch_p99_ms": float(np.percentile(lat, 99)),
            "applied_per_step": applied / steps, "resizes": sum(s_["rebuilt"] for s_ in stats),
            "size_after": size, "segment_length": seg, "height": height, "items_after": info["num_items"],
            "kernel_ms_per_step": {k: round(v[1] / 10, 4) for k, v in prof.items()},
            "data": "synthetic (seeded device R-MAT)"}
    print(json.dumps(line))


def main():
    args = parse()
    if args.workload != "stream":
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        return {"multigraph": multigraph_arm, "served": served_arm, "skew": skew_arm, "gpma": gpma_arm}[args.workload](args)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        return reference_arm(args, rank, world)
    import torch
    if world > 1:
        torch.distributed.init_process_group("nccl")
    peak, peak_kind = peaks()
    res, host_edges = gpu_arm(args, rank, world)
    B = args.batch
    value = B * args.steps * world / res["t"]
    out = {
        "metric": METRIC, "value": value, "unit": "edges/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": res["t"] * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic (seeded device R-MAT)",
        "config": config_of(args, res["n_edges"], world),
        "tree_height": res["height"],
        "l2": "PMA working set (0.3-0.6 GB) > 129 MB L2: no flush between steps",
        "timing": "CUDA events on the update stream",
        "batch_latency_ms": {"p50": float(np.percentile(res["lat"], 50)), "p99": float(np.percentile(res["lat"], 99))},
        "per_batch_size": dict(res["sweep"], **{str(B): {
            "edges_per_s": B * args.steps / res["t"], "p50_ms": float(np.percentile(res["lat"], 50)),
            "p99_ms": float(np.percentile(res["lat"], 99)),
            "hbm_GBps": sum(16 * B + 18 * x["slots_rewritten"] for x in res["stats"]) / res["t"] / 1e9,
            "hbm_frac": sum(16 * B + 18 * x["slots_rewritten"] for x in res["stats"]) / res["t"] / 1e9 / peak}}),
        "roofline": roofline(res, B, peak, peak_kind),
        # the batch sort runs out of L2: its figure against both bounds
        "sort_roofline": roofline(res, B, peak, peak_kind, "sort_coop"),
        "rebalance_roofline": rebalance_roofline(res, peak, peak_kind),
        "e2e": {"value": B * res["e2e_steps"] * world / res["t_e2e"], "unit": "edges/s", "h2d_bytes_per_step": res["h2d"],
                "d2h_bytes_per_step": res["d2h"], "entry": "lpma_update_host (pinned host batch)"},
        "gpu_launches": res["launches"],
        "sort_tiers": res["sort_tiers"],
        "grain": res["grain"],
        "clocks": res["clocks"],
        "check": res["check"],
    }
    s = res["stats"]
    out["events"] = {k: sum(x[k] for x in s) for k in ("root_executed", "eager_levelup", "rebuilt", "levelup_path",
                                                       "fill_empty")}
    out["slots_rewritten_per_step"] = sum(x["slots_rewritten"] for x in s) / len(s)
    out["single_windows_per_step"] = sum(x["windows_single"] for x in s) / len(s)
    out["multi_windows_per_step"] = sum(x["windows_small"] - x["windows_single"] for x in s) / len(s)
    alg = 16 * B + 18 * out["slots_rewritten_per_step"]
    out["batch_hbm"] = {"alg_bytes_per_step": alg, "achieved_GBps": alg / (res["t"] / args.steps) / 1e9,
                        "frac": alg / (res["t"] / args.steps) / 1e9 / peak}
    if rank == 0 and host_edges is not None:
        threads = os.cpu_count() or 1
        cb = cpu_baseline(host_edges, B, args.cpu_steps, threads)
        cb1 = cpu_baseline(host_edges, B, 2, 1)
        out["cpu_baseline"] = {"value": cb["value"], "unit": "edges/s", "cores": threads, "kind": "port",
                               "load_s": cb["load_s"], "value_1_thread": cb1["value"], "load_s_1_thread": cb1["load_s"],
                               "sample": "%d alternating insert/delete batches of %d edges on the scale-%d stream "
                                         "(sorted-merge CSR rebuild per batch, oracle/lpma_oracle.c), after the "
                                         "bulk load of the stored half (load_s); one-thread figure over 2 batches"
                                         % (args.cpu_steps, B, args.scale)}
    if not res["check"]["ok"]:
        print("bench: the stored set failed its check: %s" % json.dumps(res["check"]), file=sys.stderr)
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


def config_of(args, n_edges, world):
    """The workload's configuration, identical in both arms."""
    return {"workload": WORKLOAD % (args.scale, args.ef), "scale": args.scale, "edge_factor": args.ef, "batch": args.batch, "edges": n_edges,
            "bulk": n_edges // 2, "parallelism": "replicas" if world > 1 else "single"}


def reference_arm(args, rank, world):
    """The reference's CPU path for this workload on the host cores (rank 0
    only), over the same edge stream as the GPU arm, generated here by the
    CPU restatement of the device generator (the two are tested equal bit
    for bit)."""
    if rank != 0:
        return
    from oracle import pyoracle as O
    edges = O.shuffle(O.rmat_edges(replica_seed(args.seed, 0), args.scale, args.ef), replica_seed(args.seed, 0) + 1000)
    n = int(edges.size)
    threads = os.cpu_count() or 1
    B = args.batch
    steps = args.steps
    cb = cpu_baseline((edges, n // 2), B, steps, threads)
    out = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": "edges/s", "n_gpus": world,
           "steps": steps, "warmup": args.warmup, "ms_per_step": sum(cb["lat"]) * 1e3 / steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
           "data": "synthetic (seeded R-MAT)", "config": config_of(args, n, world),
           "cpu_baseline": {"value": cb["value"], "unit": "edges/s", "cores": threads, "kind": "port",
                            "load_s": cb["load_s"],
                            "sample": "%d alternating insert/delete batches of %d edges (sorted-merge CSR rebuild "
                                      "per batch, after the bulk load of the stored half; the reference GPU build "
                                      "does not compile under CUDA 13)" % (steps, B)},
           "e2e": {"value": cb["value"], "unit": "edges/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
