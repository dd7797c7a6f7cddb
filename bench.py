"""Benchmark of the CDE query path: collision queries/s on one GB300.

Workload (one "step" = one batch): the star-container layout — a 64-vertex star container of
radius 2000 with 4 rectangular holes and 2 inferior-quality zones, 300 placed items of 40 star
types with 8-200 vertices — and 1,048,576 uniform queries (item, rotation, translation) checked
with the HazardFilter that ignores the quality-1 zone.  A query's verdict is
detect_surrogate_collision || detect_poly_collision (lbf/benches/ci_bench.rs:107-121).

  value   — device throughput: queries resident in HBM, one kernel launch per step, CUDA events on
            the launching stream, L2 flushed (256 MB write) between steps;
  e2e     — the same metric through the C ABI's host entry point (jcde_detect_batch_host) from
            pinned host memory: host->device copy, kernel, device->host copy every step;
  roofline— algorithmic bytes per launch (oracle-counted per-query work of the same workload)
            over the kernel's event time, against the measured HBM peak;
  cpu_baseline — the oracle (C++ restatement of the reference CDE) on all host cores, bounded sample.

`--impl reference` times the CPU restatement of the reference on the host cores instead (the
reference itself is Rust and cannot be built here).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "jagua-rs_gb300"))

N_QUERIES = 1 << 20
SEED = 0xC1
WORKLOAD = ("star container r=2000 (64 v) + 4 rect holes + 2 quality zones; 300 placed items of 40 star "
            "types (8-200 v); 1,048,576 uniform queries; HazKeyFilter ignoring the quality-1 zone")


def profiler_range(on: bool) -> None:
    """cudaProfilerStart/Stop around the timed region, so that `ncu --profile-from-start off`
    captures exactly the timed launches (no-ops when no profiler is attached)."""
    import torch

    try:
        rt = torch.cuda.cudart()
        rt.cudaProfilerStart() if on else rt.cudaProfilerStop()
    except Exception:
        pass


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    from jcde.shards import dist_env as env

    return env()


def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


# ----------------------------------------------------------------------------------------------
# clocks: nvidia-smi sampled during the timed region
# ----------------------------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap,power.draw")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "20"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 8:
                continue
            try:
                sm.append(float(p[0]))
                mx.append(float(p[1]))
            except ValueError:
                continue
            for n, v in zip(names, p[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------------------------------------
# workload
# ----------------------------------------------------------------------------------------------
def make_layout(backend):
    from jcde import workload as W

    t = time.time()
    lay, eng = W.star_container_layout(backend)
    log(f"[bench] layout: {len(lay.hazards)} hazards, {len(lay.items)} item types, "
        f"{lay.n_failed_placements} failed placements ({time.time() - t:.1f}s, {backend.name})")
    return lay, eng


def gpu_engine_for(lay):
    import jcde

    eng = jcde.CDEngine(lay.cde_bbox, (), jcde.CDEConfig(quadtree_depth=lay.depth, cd_threshold=lay.cd_threshold))
    for it in lay.items:
        eng.register_item(it.xy, it.poi, it.poles)
    for hz in lay.hazards:
        eng.register_hazard(jcde.Hazard(hz.kind, hz.xy, hz.poi, hz.dynamic, hz.tag))
    return eng


def oracle_engine_for(lay):
    from jcde import workload as W
    from oracle import oracle as O

    O.build()
    return W.replay(O.OracleBackend, lay)


def item_stats(lay, q):
    nv = np.array([len(it.xy) for it in lay.items], np.float64)[q["item"]].mean() if len(q) else 0.0
    nff = np.array([it.n_ff_poles for it in lay.items], np.float64)[q["item"]].mean() if len(q) else 0.0
    return nv, nff


def tree_bytes(counts: np.ndarray, n: int) -> float:
    """16 B per quadtree node visited, 8 B per node-hazard entry scanned, 16 B per hazard edge
    tested, 16 B per point-in-polygon edge (per query, counted by the oracle)."""
    c = counts.astype(np.float64) / max(1, n)
    return 16.0 * c[0] + 8.0 * c[1] + 16.0 * c[2] + 16.0 * c[3]


def cpu_baseline(lay, queries, n_sample: int, repeats: int = 3):
    """The oracle on all host cores over the first n_sample queries (best of `repeats`), plus the
    algorithmic work of each pass on that sample (the roofline numerators)."""
    oeng = oracle_engine_for(lay)
    q = queries[:n_sample]
    cores = host_cores()
    oeng.detect_batch(q, ignored=lay.filter_keys, n_threads=cores)   # warm-up
    best = float("inf")
    verdicts = None
    for _ in range(repeats):
        t = time.perf_counter()
        verdicts = oeng.detect_batch(q, ignored=lay.filter_keys, n_threads=cores)
        best = min(best, time.perf_counter() - t)
    # per-pass work: surrogate on every query, polygon on those the surrogate leaves undecided
    c_s = np.zeros(4, np.uint64)
    surr = oeng.detect_batch(q, ignored=lay.filter_keys, n_threads=cores, counts=c_s, mode=1)
    pend = q[surr == 0]
    c_p = np.zeros(4, np.uint64)
    oeng.detect_batch(pend, ignored=lay.filter_keys, n_threads=cores, counts=c_p, mode=2)
    nv_all, nff = item_stats(lay, q)
    nv_pend, _ = item_stats(lay, pend)
    work = {
        # bytes per query of the batch: query in + verdict out + poles + tree walk
        "k_surrogate": 21.0 + 12.0 * nff + tree_bytes(c_s, len(q)),
        # bytes per undecided query: query in + verdict out + item vertices + tree walk + PIP
        "k_poly_per_pending": 21.0 + 8.0 * nv_pend + tree_bytes(c_p, len(pend)),
        "pending_fraction": len(pend) / len(q),
    }
    return {"value": n_sample / best, "unit": "queries/s", "cores": cores, "kind": "port",
            "sample": f"first {n_sample} queries of the batch, best of {repeats}"}, work, verdicts


def read_traffic(kernel: str):
    """DRAM bytes per launch of `kernel` on this workload, from the committed ncu summary."""
    path = os.path.join(REPO, "profiles", f"{kernel}_star_1m.txt")
    try:
        for line in open(path):
            if line.startswith("dram_bytes_per_launch"):
                return float(line.split("=")[1])
    except OSError:
        pass
    return None


# ----------------------------------------------------------------------------------------------
# arms
# ----------------------------------------------------------------------------------------------
def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from jcde import workload as W
    from oracle import oracle as O

    O.build()
    lay, oeng = make_layout(O.OracleBackend)
    q = W.queries_for(lay, N_QUERIES, SEED)
    cores = host_cores()
    sample = 1 << 17
    for i in range(args.warmup):
        oeng.detect_batch(q[:sample], ignored=lay.filter_keys, n_threads=cores)
    times = []
    for i in range(args.steps):
        s = q[(i * sample) % N_QUERIES:][:sample]
        t = time.perf_counter()
        oeng.detect_batch(s, ignored=lay.filter_keys, n_threads=cores)
        times.append(time.perf_counter() - t)
    value = sample * args.steps / sum(times)
    desc = f"{sample} queries per step of the {N_QUERIES}-query batch"
    line = {
        "metric": "collision queries/s", "value": value, "unit": "queries/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "impl": "reference",
        "config": {"workload": WORKLOAD, "queries_per_step": sample, "quadtree_depth": lay.depth,
                   "cd_threshold": lay.cd_threshold},
        "cpu_baseline": {"value": value, "unit": "queries/s", "cores": cores, "kind": "port", "sample": desc},
        "e2e": {"value": value, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "CPU restatement of the reference CDE (Rust reference not buildable here), all host cores",
    }
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args):
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    import jcde
    from jcde import workload as W

    jcde.lib()
    lay, _ = make_layout(jcde.GpuBackend)
    eng = gpu_engine_for(lay)
    # weak scaling: every rank answers its own batch of N_QUERIES (distinct query stream per rank)
    from jcde.shards import max_over_ranks, rank_queries

    q = rank_queries(lay, N_QUERIES, SEED, rank)
    dq = torch.from_numpy(q.view(np.uint8).copy()).cuda()
    out = torch.empty(N_QUERIES, dtype=torch.uint8, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    filt = lay.filter_keys
    # launch choices timed on this batch before the run (jcde_autotune; verdicts checked identical)
    tuning, tune_ms = eng.autotune(dq, filter=filt, stream=stream) if args.autotune else (eng.get_tuning(), None)

    for _ in range(args.warmup):
        eng.detect_batch(dq, filter=filt, out=out, stream=stream)
    torch.cuda.synchronize()

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    launches0 = eng.kernel_launches()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clk = ClockSampler(local)
    clk.__enter__()   # sampled through the device loop, its profiled twin and the e2e loop
    profiler_range(True)
    t0 = time.perf_counter()
    for i in range(args.steps):
        flush.zero_()
        ev[i][0].record(stream)
        eng.detect_batch(dq, filter=filt, out=out, stream=stream)
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    profiler_range(False)
    launches = eng.kernel_launches() - launches0
    step_ms = [a.elapsed_time(b) for a, b in ev]
    # per-kernel event times of the same steps (a second, profiled run of the timed loop)
    eng.profile(True)
    eng.profile_read(reset=True)
    for i in range(args.steps):
        flush.zero_()
        eng.detect_batch(dq, filter=filt, out=out, stream=stream)
    torch.cuda.synchronize()
    kprof = eng.profile_read(reset=True)
    eng.profile(False)
    dev_s = max_over_ranks(sum(step_ms) / 1e3)
    value = world * N_QUERIES * args.steps / dev_s
    verdicts = out.cpu().numpy()

    # e2e: host buffers through the C ABI, copies inside the timed region
    hq = torch.from_numpy(q.view(np.uint8).copy()).pin_memory()
    hout = torch.empty(N_QUERIES, dtype=torch.uint8).pin_memory()
    from jcde._ffi import lib

    fobj = jcde.engine._Filter(filt)
    for _ in range(args.warmup):
        lib().jcde_detect_batch_host(eng.h, hq.data_ptr(), N_QUERIES, fobj.ref, hout.data_ptr())
    e2e_times = []
    for i in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t = time.perf_counter()
        st = lib().jcde_detect_batch_host(eng.h, hq.data_ptr(), N_QUERIES, fobj.ref, hout.data_ptr())
        e2e_times.append(time.perf_counter() - t)
        assert st == 0
    # collect mode on the same batch (cd_engine.rs:261-310): all colliding hazard keys per query
    cap = 4 * N_QUERIES
    c_off = torch.empty(N_QUERIES, dtype=torch.int32, device="cuda")
    c_cnt = torch.empty(N_QUERIES, dtype=torch.int32, device="cuda")
    c_ids = torch.empty(cap, dtype=torch.int32, device="cuda")
    c_tot = torch.zeros(1, dtype=torch.int32, device="cuda")

    def collect_once():
        st = lib().jcde_collect_batch(eng.h, dq.data_ptr(), N_QUERIES, fobj.ref, c_off.data_ptr(), c_cnt.data_ptr(),
                                      c_ids.data_ptr(), cap, c_tot.data_ptr(), stream.cuda_stream)
        assert st == 0

    for _ in range(args.warmup):
        collect_once()
    c_ms = []
    for i in range(args.steps):
        flush.zero_()
        a_ev, b_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a_ev.record(stream)
        collect_once()
        b_ev.record(stream)
        c_ms.append((a_ev, b_ev))
    torch.cuda.synchronize()
    collect_s = sum(a.elapsed_time(b) for a, b in c_ms) / 1e3
    collect_total = int(c_tot.item())
    clk.__exit__(None, None, None)
    e2e_s = max_over_ranks(sum(e2e_times))
    e2e_value = world * N_QUERIES * args.steps / e2e_s
    e2e_same = bool(np.array_equal(hout.numpy(), verdicts))

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return 0

    # CPU baseline + algorithmic bytes per query (oracle on a bounded sample of the same queries)
    cpu, work, cpu_verdicts = cpu_baseline(lay, q, n_sample=args.cpu_sample)
    sample_ok = bool(np.array_equal(cpu_verdicts, verdicts[: args.cpu_sample]))
    # collect parity on a small sample: sorted key sets per query against the oracle
    n_cs = min(8192, args.cpu_sample)
    ocnt, oids = oracle_engine_for(lay).collect_batch(q[:n_cs], ignored=lay.filter_keys, n_threads=host_cores())
    g_off, g_cnt, g_ids = c_off.cpu().numpy(), c_cnt.cpu().numpy(), c_ids.cpu().numpy()
    o_off = np.concatenate([[0], np.cumsum(ocnt.astype(np.int64))])
    collect_ok = all(np.array_equal(g_ids[g_off[i]:g_off[i] + g_cnt[i]], oids[o_off[i]:o_off[i + 1]]) for i in range(n_cs))
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    kernels = {}
    for name, kind, bytes_per_launch in (
        ("k_surrogate", "surrogate", work["k_surrogate"] * N_QUERIES),
        ("k_poly", "poly", work["k_poly_per_pending"] * work["pending_fraction"] * N_QUERIES),
    ):
        ms, cnt = kprof[kind]
        avg_s = ms / 1e3 / max(1, cnt)
        kernels[name] = {"avg_ms": 1e3 * avg_s, "launches": cnt, "bytes_per_launch": bytes_per_launch,
                         "achieved_gbs": bytes_per_launch / avg_s / 1e9 if avg_s > 0 else None}
    dom = max(kernels, key=lambda k: kernels[k]["avg_ms"])
    achieved = kernels[dom]["achieved_gbs"]
    traffic = read_traffic(dom)
    order_ms, order_n = kprof["order"]
    clocks = clk.summary()
    line = {
        "metric": "collision queries/s", "value": value, "unit": "queries/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dev_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "queries_per_step": N_QUERIES, "quadtree_depth": lay.depth,
                   "cd_threshold": lay.cd_threshold, "l2": "flushed between steps (256 MB write)",
                   "parallelism": f"{world} rank(s), queries per rank, layout replicated"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "kernel": dom,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (burst copy)" if peaks else "fallback 6.8 TB/s",
                     "kernels": kernels, "ordering_ms_per_step": order_ms / max(1, order_n)},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "queries/s", "h2d_bytes_per_step": N_QUERIES * 20,
                "d2h_bytes_per_step": N_QUERIES, "same_verdicts": e2e_same},
        "collect": {"value": N_QUERIES * args.steps / collect_s, "unit": "queries/s", "kernel": "k_collect",
                    "ms_per_step": 1e3 * collect_s / args.steps, "keys_per_query": collect_total / N_QUERIES,
                    "parity_sample": {"queries": n_cs, "bit_exact": bool(collect_ok)}},
        "gpu_launches": launches,
        "tuning": {"chosen": tuning, "autotuned": bool(args.autotune), "median_ms_at_tuning": tune_ms},
        "clocks": clocks,
        "wall_s_timed": wall,
        "parity_sample": {"queries": args.cpu_sample, "bit_exact": sample_ok},
        "collision_rate": float(verdicts.mean()),
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_multi(args):
    """The multi-layout workload: 64 independent bin layouts, log-uniform 4,096-262,144 queries each, answered by
    one launch sequence (CUDA graph) versus 64 per-layout jcde_detect_batch calls."""
    import torch

    import jcde
    from jcde import workload as W

    jcde.lib()
    t = time.time()
    lays = W.multi_layouts(jcde.GpuBackend)
    log(f"[bench] {len(lays)} layouts, {sum(len(l.hazards) for l, _ in lays)} hazards ({time.time() - t:.1f}s)")
    engines = [e.eng for _, e in lays]
    q, offs = W.multi_queries(lays)
    n = int(offs[-1])
    dq = torch.from_numpy(q.view(np.uint8).copy()).cuda()
    out_plain = torch.empty(n, dtype=torch.uint8, device="cuda")
    out_multi = torch.empty(n, dtype=torch.uint8, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.Stream()
    m = jcde.MultiEngine(engines)
    qb = W.QUERY_DTYPE.itemsize
    # launch choices of the batched sequence timed on this batch (jcde_multi_autotune; verdicts checked)
    multi_tuning, _ = m.autotune(dq, offs, stream=stream) if args.autotune else ({"poly_chunk": 2, "ordered": True}, 0)

    def plain():
        for l, eng in enumerate(engines):
            a, b = int(offs[l]), int(offs[l + 1])
            eng.detect_batch(dq[a * qb:b * qb], out=out_plain[a:b], stream=stream)

    def batched():
        m.detect(dq, offs, out=out_multi, stream=stream, graph=True)

    res = {}
    with torch.cuda.stream(stream):
        for name, fn in (("plain", plain), ("batched", batched)):
            for _ in range(args.warmup):
                fn()
            stream.synchronize()
            ms = []
            for _ in range(args.steps):
                flush.zero_()
                a_ev, b_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a_ev.record(stream)
                fn()
                b_ev.record(stream)
                ms.append((a_ev, b_ev))
            stream.synchronize()
            res[name] = sum(a.elapsed_time(b) for a, b in ms) / args.steps
    same = bool(torch.equal(out_plain, out_multi))
    line = {
        "metric": "multi-layout collision queries/s", "value": n / (res["batched"] / 1e3), "unit": "queries/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": res["batched"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{len(lays)} star-container bins (32-128 v), 20-400 items each from 40 star types "
                               f"(8-200 v), log-uniform 4,096-262,144 queries per bin ({n} total)",
                   "batched": "one ordering + surrogate + polygon launch sequence, CUDA-graph replay",
                   "plain": f"{len(lays)} jcde_detect_batch calls, one per layout",
                   "l2": "flushed between steps (256 MB write)"},
        "plain": {"value": n / (res["plain"] / 1e3), "ms_per_step": res["plain"]},
        "speedup_vs_plain": res["plain"] / res["batched"],
        "batched_tuning": multi_tuning,
        "same_verdicts": same,
        "impl": "jcde",
    }
    print(json.dumps(line), flush=True)
    return 0


def run_proxy(args):
    """The gradient-separation workload: the star layout with surrogate poles on every interior hazard; 1,048,576 colliding
    candidates; 20 gradient steps on the pole-overlap proxy then the exact verdict, versus 20 random
    perturbations per candidate judged by the exact verdict.  Metric: verified collision-free
    placements per second."""
    import torch

    import jcde
    from jcde import workload as W

    jcde.lib()
    lay, _ = make_layout(jcde.GpuBackend)
    eng = gpu_engine_for(lay)
    hp = W.hazard_poles(jcde.GpuBackend, lay)
    keys = hp[:, 3].view(np.uint32)
    for k in np.unique(keys):
        eng.set_hazard_poles(int(k), hp[keys == k, :3])
    filt = lay.filter_keys
    n_target = N_QUERIES
    # candidate pool: uniform placements that collide (exact verdict) and overlap some pole
    st = W.Stream(0xC4, 1)
    got_p, got_i = [], []
    have = 0
    while have < n_target:
        params, items = W.random_params(st, 1 << 21, len(lay.items), lay.cde_bbox)
        dp = torch.from_numpy(params).cuda()
        di = torch.from_numpy(items.astype(np.int32)).cuda()
        q0, p0 = eng.separate_batch(dp.clone(), di, steps=0, filter=filt)
        v0 = eng.detect_batch(q0, filter=filt)
        keep = (v0 == 1) & (p0 > 0)
        got_p.append(dp[keep])
        got_i.append(di[keep])
        have += int(keep.sum().item())
    P0 = torch.cat(got_p)[:n_target].contiguous()
    I0 = torch.cat(got_i)[:n_target].contiguous()
    n = P0.shape[0]
    mean_r = float(np.mean([it.poles[0, 2] for it in lay.items]))
    K = 20
    CLEARANCE = 20.0   # poles under-cover the star items' spikes: separate the poles by a margin
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    out_k = torch.empty(n * K, dtype=torch.uint8, device="cuda")

    def gd():
        p = P0.clone()
        q, _ = eng.separate_batch(p, I0, steps=20, step_t=0.25, step_th=0.25, clearance=CLEARANCE, filter=filt)
        v = eng.detect_batch(q, filter=filt)
        return (v == 0).sum()

    def rnd():
        q = eng.resample_batch(P0, I0, k=K, sigma_t=mean_r, sigma_th=0.25, seed=7)
        eng.detect_batch(q, filter=filt, out=out_k)
        return (out_k.view(n, K) == 0).any(dim=1).sum()

    res = {}
    for name, fn in (("gradient", gd), ("random", rnd)):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        ms, succ = 0.0, 0
        for _ in range(args.steps):
            flush.zero_()
            a_ev, b_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a_ev.record()
            s_ = fn()
            b_ev.record()
            torch.cuda.synchronize()
            ms += a_ev.elapsed_time(b_ev)
            succ += int(s_.item())
        res[name] = {"placements_per_s": succ / (ms / 1e3), "verified_free": succ // args.steps,
                     "ms_per_step": ms / args.steps, "candidates": n}
    # the other settings of both methods (one timed run each): descent lengths and copies per candidate
    def once(fn):
        fn()
        torch.cuda.synchronize()
        a_ev, b_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        flush.zero_()
        a_ev.record()
        s_ = fn()
        b_ev.record()
        torch.cuda.synchronize()
        return int(s_.item()) / (a_ev.elapsed_time(b_ev) / 1e3)

    sweep = {}
    for steps in (5, 10, 20):
        def gd_s(steps=steps):
            q, _ = eng.separate_batch(P0.clone(), I0, steps=steps, step_t=0.25, step_th=0.25, clearance=CLEARANCE,
                                      filter=filt)
            return (eng.detect_batch(q, filter=filt) == 0).sum()
        sweep[f"gradient_{steps}_steps"] = once(gd_s)
    for kk in (1, 2, 5, 10, 20):
        out_kk = torch.empty(n * kk, dtype=torch.uint8, device="cuda")
        def rnd_k(kk=kk, out_kk=out_kk):
            q = eng.resample_batch(P0, I0, k=kk, sigma_t=mean_r, sigma_th=0.25, seed=7)
            eng.detect_batch(q, filter=filt, out=out_kk)
            return (out_kk.view(n, kk) == 0).any(dim=1).sum()
        sweep[f"random_{kk}_copies"] = once(rnd_k)
    best_g = max(v for k, v in sweep.items() if k.startswith("gradient"))
    best_r = max(v for k, v in sweep.items() if k.startswith("random"))
    # gradient accuracy on a sample against the FP64 oracle (test infrastructure, CPU leg)
    from oracle import oracle as O

    O.build()
    ns = 4096
    val, grad = eng.proxy_batch(P0[:ns].contiguous(), I0[:ns].contiguous(), filter=filt)
    v64, g64 = O.proxy_f64(P0[:ns].cpu().numpy(), I0[:ns].cpu().numpy().astype(np.uint32),
                           [it.poles for it in lay.items], hp, ignored=filt)
    g32 = grad.cpu().numpy().astype(np.float64)
    on = v64 > 1e-2
    rel = np.linalg.norm(g32[on] - g64[on], axis=1) / np.linalg.norm(g64[on], axis=1)
    line = {
        "metric": "CDE-verified collision-free placements/s (gradient separation)",
        "value": res["gradient"]["placements_per_s"], "unit": "placements/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": res["gradient"]["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"star layout with surrogate poles on {len(np.unique(keys))} hazards; {n} colliding "
                               "candidates; 20 descent steps on the pole-overlap proxy (hazard poles grown by a "
                               "20-unit clearance) then jcde_detect_batch",
                   "random_arm": f"{K} Gaussian perturbations per candidate (sigma_t={mean_r:.1f}, sigma_th=0.25) "
                                 "then jcde_detect_batch",
                   "l2": "flushed between steps (256 MB write)"},
        "gradient": res["gradient"], "random": res["random"],
        "speedup_vs_random": res["gradient"]["placements_per_s"] / res["random"]["placements_per_s"],
        "settings_sweep_placements_per_s": sweep,
        "best_setting_speedup": best_g / best_r,
        "grad_rel_err_vs_fp64": {"median": float(np.median(rel)), "p99": float(np.percentile(rel, 99)),
                                 "max": float(rel.max()), "samples": int(on.sum())},
        "impl": "jcde",
    }
    print(json.dumps(line), flush=True)
    return 0


def run_prep(args):
    """Item preparation: the poi and surrogate poles (lbf's default limits) of 1024 star item shapes
    of 8-200 vertices, radius 20-60.  One step = the two pole-search launches over the whole batch
    (shapes, areas and poi resident on the device).  e2e = jcde.prep.import_items from host arrays
    (host orientation / area / centring, copies, both launches, poles read back).  CPU baseline: the
    oracle's Importer::import_item restatement on a sample of the shapes, one shape per host thread.
    A second leg imports with lbf's default simplification (tolerance 0.001, shape_modification.rs)."""
    import torch

    import jcde
    from jcde import prep
    from jcde import workload as W

    jcde.lib()
    n_shapes = args.prep_shapes
    st = W.Stream(0xC2, 7)
    raws = []
    for _ in range(n_shapes):
        nv = int(st.randint(8, 200, 1)[0])
        raws.append(W.star_polygon(st, nv, 20.0, 60.0))
    items = prep.import_items(raws)   # also the untimed first run
    shp = [prep.spolygon_shape(r)[0] for r in raws]
    b_raw = prep.ShapeBatch(shp)
    b_int = prep.ShapeBatch([it.xy for it in items])
    area = torch.tensor([it.area for it in items], dtype=torch.float32, device="cuda")
    poi = torch.from_numpy(np.stack([it.poi for it in items])).cuda()
    cap = 128
    out = torch.empty((n_shapes, cap, 3), dtype=torch.float32, device="cuda")
    cnt = torch.empty(n_shapes, dtype=torch.int32, device="cuda")
    sts = torch.empty(n_shapes, dtype=torch.int32, device="cuda")
    poi_o = torch.empty((n_shapes, 3), dtype=torch.float32, device="cuda")
    poi_s = torch.empty(n_shapes, dtype=torch.int32, device="cuda")
    stream = torch.cuda.Stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def step(ev=None):
        with torch.cuda.stream(stream):
            flush.zero_()
            if ev:
                ev[0].record(stream)
            b_raw.poi(poi_o, poi_s, stream=stream)
            if ev:
                ev[1].record(stream)
            b_int.poles(area, poi, cap=cap, out=out, counts=cnt, status=sts, stream=stream)
            if ev:
                ev[2].record(stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clk = ClockSampler(0)
    clk.__enter__()
    t_poi, t_poles = [], []
    for _ in range(args.steps):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        step(ev)
        torch.cuda.synchronize()
        t_poi.append(ev[0].elapsed_time(ev[1]))
        t_poles.append(ev[1].elapsed_time(ev[2]))
    # end to end through the public API from host arrays
    e2e_ms = []
    for _ in range(max(1, min(args.steps, 5))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        got = prep.import_items(raws)
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    # lbf's default import simplifies each item (tolerance 0.001) before its poi and poles: the
    # simplification pass alone on the device, and the whole import with it end to end
    area_o = torch.tensor([it.area for it in items], dtype=torch.float32, device="cuda")
    t_simp = []
    for k in range(args.warmup + args.steps):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        with torch.cuda.stream(stream):
            flush.zero_()
            ev[0].record(stream)
            prep.simplify_device(b_int, area_o, False, 0.001, stream=stream)
            ev[1].record(stream)
        torch.cuda.synchronize()
        if k >= args.warmup:
            t_simp.append(ev[0].elapsed_time(ev[1]))
    e2e_simp = []
    for _ in range(max(1, min(args.steps, 5))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        got_s = prep.import_items(raws, simplify_tolerance=0.001)
        e2e_simp.append((time.perf_counter() - t0) * 1e3)
    clk.__exit__()
    same = all(np.array_equal(g.poles, it.poles) for g, it in zip(got, items))
    ok = bool((sts.cpu().numpy() == 0).all() and (poi_s.cpu().numpy() == 0).all())
    ms = float(np.sum(t_poi) + np.sum(t_poles))
    value = n_shapes * args.steps / (ms / 1e3)
    n_poles = [len(it.poles) for it in items]
    h2d = sum(r.nbytes for r in raws) + 4 * (n_shapes + 1) * 2 + 16 * n_shapes
    d2h = 12 * n_shapes + n_shapes * cap * 12 + 8 * n_shapes
    line = {
        "metric": "item shapes prepared per second (poi + surrogate poles)",
        "value": value, "unit": "shapes/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{n_shapes} star item shapes (8-200 vertices, radius 20-60), poi then surrogate "
                               "poles with lbf's default limits (100, 0), (20, 0.75), (10, 0.9); one step = "
                               "jcde_poi_batch + jcde_surrogate_poles_batch over the batch",
                   "l2": "flushed before each step (256 MB write)"},
        "ms_poi": float(np.median(t_poi)), "ms_poles": float(np.median(t_poles)),
        "poles_per_shape": {"mean": float(np.mean(n_poles)), "min": int(min(n_poles)), "max": int(max(n_poles))},
        "all_status_ok": ok, "gpu_launches": 2 * args.steps,
        "e2e": {"value": n_shapes / (np.median(e2e_ms) / 1e3), "unit": "shapes/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_batch": float(np.median(e2e_ms)),
                "same_poles_as_device_step": bool(same)},
        "with_simplification": {"tolerance": 0.001, "ms_simplify_pass": float(np.median(t_simp)),
                                "vertices_before": int(sum(len(it.xy) for it in items)),
                                "vertices_after": int(sum(len(it.xy) for it in got_s)),
                                "e2e": {"value": n_shapes / (np.median(e2e_simp) / 1e3), "unit": "shapes/s",
                                        "ms_per_batch": float(np.median(e2e_simp))}},
        "clocks": clk.summary(),
        "impl": "jcde",
    }
    if not args.no_cpu:
        from concurrent.futures import ThreadPoolExecutor

        from oracle import oracle as O

        O.build()
        n_s = min(n_shapes, 4 * host_cores())
        t0 = time.perf_counter()
        with ThreadPoolExecutor(host_cores()) as ex:   # ctypes calls release the GIL
            ref = list(ex.map(lambda r: W.import_item(O.OracleBackend, r), raws[:n_s]))
        cpu_s = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": n_s / cpu_s, "unit": "shapes/s", "cores": host_cores(), "kind": "port",
                                "sample": f"first {n_s} of {n_shapes} shapes, oracle import_item, one shape per thread",
                                "same_poles": bool(all(np.array_equal(a.poles, b.poles)
                                                       for a, b in zip(ref, items[:n_s])))}
        t0 = time.perf_counter()
        with ThreadPoolExecutor(host_cores()) as ex:
            ref_s = list(ex.map(lambda r: W.import_item(O.OracleBackend, r, simplify_tolerance=0.001), raws[:n_s]))
        cpu_s2 = time.perf_counter() - t0
        line["with_simplification"]["cpu_baseline"] = {
            "value": n_s / cpu_s2, "unit": "shapes/s", "cores": host_cores(), "kind": "port",
            "same_items": bool(all(np.array_equal(a.poles, b.poles) and np.array_equal(a.xy, b.xy)
                                   for a, b in zip(ref_s, got_s[:n_s])))}
    print(json.dumps(line), flush=True)
    return 0


def run_bpp(args):
    """Bin packing with lbf_bpp.rs's optimizer: a seeded instance of 60 star item types (8-60
    vertices, 2-8 copies each, some needing quality 1 or turning by 90 degrees only) and 6 bins
    with holes and quality zones; 4096 candidates per layout searched.  One step = one whole solve
    on the GPU engines through the package's API (host-driven: every search's layouts judged in one
    multi-layout launch sequence, the choice and the registration on the host).  CPU baseline: the
    same solve on the oracle engines (detect on all host cores), the same placements."""
    import torch

    import jcde
    from jcde import bpp

    jcde.lib()
    inst = bpp.load_bpp(bpp.synthetic_instance(n_types=60, demand_range=(2, 8), n_bins=6))
    spec = bpp.BppSpec(n_cand=4096)
    su = bpp.setup_bpp(jcde.GpuBackend, inst)
    for _ in range(max(1, min(args.warmup, 2))):
        bpp.run_bpp(jcde.GpuBackend, su, spec)
    clk = ClockSampler(0)
    clk.__enter__()
    ts, log = [], None
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        log = bpp.run_bpp(jcde.GpuBackend, su, spec)
        ts.append(time.perf_counter() - t0)
    clk.__exit__()
    t_med = float(np.median(ts))
    sol = bpp.export_solution(su, log)
    n_copies = sum(it.demand for it in inst.items)
    line = {
        "metric": "bin-packing items placed per second (LBF solve, host-driven)",
        "value": len(log.placements) / t_med, "unit": "items/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_med * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"bin packing: {len(inst.items)} star item types, {n_copies} copies, {len(inst.bins)} bins "
                               f"with holes and quality zones, {spec.n_cand} candidates per layout searched; one "
                               "step = one whole solve (wall clock, host-driven through the package API)"},
        "items_placed": int(len(log.placements)), "unplaced": {str(k): v for k, v in log.unplaced.items()},
        "layouts": len(log.layouts), "cost": sol["cost"], "density": sol["density"],
        "candidates_judged_per_s": log.judged / t_med,
        "clocks": clk.summary(),
        "impl": "jcde",
    }
    if not args.no_cpu:
        from oracle import oracle as O

        O.build()
        su_o = bpp.setup_bpp(O.OracleBackend, inst)
        t0 = time.perf_counter()
        log_o = bpp.run_bpp(O.OracleBackend, su_o, spec)
        cpu_s = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": len(log_o.placements) / cpu_s, "unit": "items/s", "cores": host_cores(),
                                "kind": "port", "ms_per_solve": cpu_s * 1e3,
                                "sample": "the whole solve on the oracle engines (layouts searched one by one)",
                                "same_solution": bool(log_o.same_as(log))}
        line["solve_speedup_vs_cpu"] = cpu_s / t_med
    print(json.dumps(line), flush=True)
    return 0


def run_lbf(args):
    """The LBF-style strip build on the device-resident engine.  2000 steps, each: 16384
    candidates generated and searched as lbf's search does (surrogate pass for all; the polygon pass
    for those that could still beat the best free one, search.rs:52-56), the least-cost free one
    registered on the device, and a random placed item deregistered every 50 steps.  A timed step is
    one whole build from the strip's initial state.  Metric: candidate placements searched per
    second over the build."""
    import torch

    import jcde
    from jcde import lbf

    jcde.lib()
    spec = lbf.LbfSpec()
    lay, geng = lbf.setup(jcde.GpuBackend, spec)
    r = jcde.ResidentEngine(geng.eng)
    SPG = 25   # LBF steps per CUDA graph launch
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.Stream()   # a captured graph needs a stream other than the legacy default one
    sh = stream.cuda_stream

    def build(timed):
        r.reset()
        r.lbf_begin(spec.seed, spec.n_cand, spec.n_types, spec.remove_every, spec.steps, spec.box)
        with torch.cuda.stream(stream):
            flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        r.lbf_steps(spec.steps, SPG, stream=sh)
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b)

    for _ in range(args.warmup):
        build(False)
    launches0 = r.kernel_launches()
    clk = ClockSampler(0)
    clk.__enter__()
    profiler_range(True)
    times = [build(True) for _ in range(args.steps)]
    profiler_range(False)
    launches = r.kernel_launches() - launches0
    clk.__exit__()
    ms = float(np.sum(times))
    n_cand_total = spec.steps * spec.n_cand
    value = n_cand_total * args.steps / (ms / 1e3)
    d = r.lbf_read()
    st = r.status()
    # per-kernel shares from one eager, profiled build (events around every launch)
    geng.eng.profile(True)
    r.reset()
    r.lbf_begin(spec.seed, spec.n_cand, spec.n_types, spec.remove_every, spec.steps, spec.box)
    geng.eng.profile_read(reset=True)
    r.lbf_steps(spec.steps, 0, stream=sh)
    kp = geng.eng.profile_read(reset=True)
    geng.eng.profile(False)
    kinds = {k: {"ms_per_build": v[0], "launches": v[1]} for k, v in kp.items() if v[1]}
    dominant = max(kinds, key=lambda k: kinds[k]["ms_per_build"])
    # end to end through the public API: resident copy from the host engine, the build, the log read back
    e2e_ms = []
    h2d = d2h = 0
    for _ in range(max(1, min(args.steps, 5))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        h2d = r.reset()
        log_e2e, _ = lbf.run_device(geng, spec, steps_per_graph=SPG, resident=r)
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
        d2h = (log_e2e.placements.nbytes + log_e2e.removals.nbytes + log_e2e.free_counts.nbytes + 16)
    e2e_value = n_cand_total / (np.median(e2e_ms) / 1e3)
    # the same build with three local-search rounds of 2048 candidates per step (search.rs:80-101 restated)
    spec_ls = lbf.LbfSpec(ls_rounds=3, ls_cand=2048, ls_sigma_t=200.0, ls_sigma_turns=0.05)
    ls_ms = []
    for k in range(2):
        r.reset()
        r.lbf_begin(spec_ls.seed, spec_ls.n_cand, spec_ls.n_types, spec_ls.remove_every, spec_ls.steps, spec_ls.box, 0,
                    spec_ls.ls_rounds, spec_ls.ls_cand, spec_ls.ls_sigma_t, spec_ls.ls_sigma_turns, spec_ls.ls_decay)
        with torch.cuda.stream(stream):
            flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        r.lbf_steps(spec_ls.steps, SPG, stream=sh)
        b.record(stream)
        torch.cuda.synchronize()
        if k:
            ls_ms.append(a.elapsed_time(b))
    d_ls = r.lbf_read()
    ls_cands = spec_ls.steps * (spec_ls.n_cand + spec_ls.ls_rounds * spec_ls.ls_cand)
    local_search = {"ms_per_build": ls_ms[0], "candidates_per_s": ls_cands / (ls_ms[0] / 1e3),
                    "rounds": spec_ls.ls_rounds, "candidates_per_round": spec_ls.ls_cand,
                    "placements_improved_by_local_search": int(((d_ls["placements"][:, 2] >> 24) > 0).sum())}
    # the same build driven step by step from the host through the regular engine (host registration,
    # a re-flattened tree upload per step): a bounded sample of its first steps
    host_steps = 200
    lay_h, geng_h = lbf.setup(jcde.GpuBackend, spec)
    t0 = time.perf_counter()
    hlog = lbf.run_host(lay_h, geng_h, spec, steps=host_steps)
    host_s = time.perf_counter() - t0
    host_ok = bool(np.array_equal(hlog.placements, d["placements"][: len(hlog.placements)]))
    line = {
        "metric": "LBF candidate placements searched per second (device-resident build)",
        "value": value, "unit": "candidates/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"LBF strip build: {spec.n_types} star types ({spec.v_range[0]}-{spec.v_range[1]} "
                               f"vertices), {spec.width:.0f} x {spec.height:.0f} strip, {spec.steps} steps x "
                               f"{spec.n_cand} candidates, removal every {spec.remove_every} steps; one timed step = "
                               "one whole build; register/deregister on the device; "
                               f"{SPG} LBF steps per CUDA graph launch",
                   "l2": "flushed between builds (256 MB write)"},
        "lbf_steps_per_s": spec.steps * args.steps / (ms / 1e3),
        "placed": int(len(d["placements"])), "removed": int(len(d["removals"])), "live": d["n_live"],
        "pool_use": st,
        "kernels_eager_build": kinds, "dominant": dominant,
        "gpu_launches": int(launches),
        "e2e": {"value": e2e_value, "unit": "candidates/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_build": float(np.median(e2e_ms))},
        "with_local_search": local_search,
        "host_driven_gpu": {"value": host_steps * spec.n_cand / host_s, "unit": "candidates/s",
                            "sample": f"first {host_steps} steps", "same_placements": host_ok},
        "clocks": clk.summary(),
        "impl": "jcde",
    }
    if not args.no_cpu:
        from oracle import oracle as O

        O.build()
        cpu_steps = args.lbf_cpu_steps
        lay_o, oeng = lbf.setup(O.OracleBackend, spec)
        t0 = time.perf_counter()
        olog = lbf.run_host(lay_o, oeng, spec, steps=cpu_steps)
        cpu_s = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": cpu_steps * spec.n_cand / cpu_s, "unit": "candidates/s",
                                "cores": host_cores(), "kind": "port",
                                "sample": f"first {cpu_steps} of {spec.steps} steps, oracle detect on all cores, "
                                          "numpy choice, oracle register",
                                "same_placements": bool(np.array_equal(olog.placements,
                                                                       d["placements"][: len(olog.placements)]))}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="jcde", choices=["jcde", "reference"])
    ap.add_argument("--cpu-sample", type=int, default=1 << 17)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--autotune", type=int, default=1, help="1: jcde_autotune on the batch before timing")
    ap.add_argument("--lbf-cpu-steps", type=int, default=2000)
    ap.add_argument("--prep-shapes", type=int, default=1024, help="prep workload: shapes per batch")
    ap.add_argument("--workload", default="star", choices=["star", "multi", "proxy", "lbf", "prep", "bpp"],
                    help="star: the headline single-layout batch; multi: 64 layouts in one launch sequence; "
                         "proxy: gradient separation of colliding candidates vs random resampling; "
                         "lbf: LBF-style build on the device-resident engine; "
                         "prep: poi + surrogate poles of 1024 item shapes on the device; "
                         "bpp: bin packing with lbf's bin-packing optimizer")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "multi":
        return run_multi(args)
    if args.workload == "proxy":
        return run_proxy(args)
    if args.workload == "lbf":
        return run_lbf(args)
    if args.workload == "prep":
        return run_prep(args)
    if args.workload == "bpp":
        return run_bpp(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
