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
  cpu_baseline — the oracle (C++ restatement of the reference CDE) on all host cores, bounded sample;
  roofline.l2 / roofline.issue — the dominant kernel against the project-measured L2 read peak
            (jcde_l2_read_peak) and against its instruction-issue slots (ncu instruction count);
  batched / proxy / lbf — the metric's other workloads in the same run (N=1): 64 layouts in one
            launch sequence vs per-layout launches, grads/s and CDE-verified placements/s of the
            pole-overlap proxy, and the device-resident LBF build, each with its oracle check.

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
            "types (8-200 v); {n:,} uniform queries; HazKeyFilter ignoring the quality-1 zone")


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


# committed ncu summaries per kernel and figure, in order of preference: the instruction count from
# the reduced-batch capture of the current build (it scales with the batch: the same query
# generator, the same undecided fraction), memory figures from the full-size capture (cache hit
# rates depend on the batch size, so those are taken at the size they describe)
PROFILE_FILES = {"k_poly": {"inst": ("k_poly_star_262k.txt", "k_poly_star_1m.txt"),
                            "l2_sectors": ("k_poly_star_1m.txt", "k_poly_star_262k.txt"),
                            "dram": ("k_poly_star_1m.txt",)}}


def read_profile(kernel: str) -> dict:
    """Figures of `kernel` on this workload from its committed ncu summaries (profiles/), per launch of
    a batch of N_QUERIES: DRAM bytes, executed warp instructions, L2 sectors, and the file each came from."""
    keys = {"dram_bytes_per_launch": "dram", "smsp__inst_executed.sum": "inst", "lts__t_sectors.sum": "l2_sectors"}
    default = (f"{kernel}_star_1m.txt",)
    files = PROFILE_FILES.get(kernel, {})
    out = {}
    for name in keys.values():
        for fn in files.get(name, default):
            val, queries = None, float(1 << 20)
            try:
                for line in open(os.path.join(REPO, "profiles", fn)):
                    if line.startswith("queries_per_launch"):
                        queries = float(line.split("=")[1])
                    for k, nm in keys.items():
                        if nm == name and line.startswith(k):
                            val = float(line.split("=")[1])
            except (OSError, ValueError):
                continue
            if val is None:
                continue
            out[name] = val * N_QUERIES / queries
            out[name + "_source"] = f"profiles/{fn}" + ("" if queries == N_QUERIES
                                                         else f" scaled by {N_QUERIES}/{int(queries)} queries")
            break
    return out


def read_traffic(kernel: str):
    """DRAM bytes per launch of `kernel` on this workload, from the committed ncu summary."""
    return read_profile(kernel).get("dram")


def l2_read_peak(sizes=(16 << 20, 32 << 20, 48 << 20), reps: int = 20, tries: int = 3):
    """GB/s of the project's L2 streaming kernel (jcde_l2_read_peak) on an L2-resident buffer: the
    best of `tries` runs for each buffer size (a peak is the best the device shows)."""
    import ctypes as C

    from jcde._ffi import lib

    best = None
    for b in sizes:
        for _ in range(tries):
            g = C.c_double()
            if lib().jcde_l2_read_peak(b, reps, C.byref(g)) == 0:
                best = g.value if best is None else max(best, g.value)
    return best


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
    # every step answers the whole batch, as the GPU arm does (~0.11 s per step on 16 Grace cores)
    sample = N_QUERIES
    for i in range(args.warmup):
        oeng.detect_batch(q, ignored=lay.filter_keys, n_threads=cores)
    times = []
    for i in range(args.steps):
        t = time.perf_counter()
        oeng.detect_batch(q, ignored=lay.filter_keys, n_threads=cores)
        times.append(time.perf_counter() - t)
    value = sample * args.steps / sum(times)
    desc = f"the whole {N_QUERIES}-query batch per step"
    line = {
        "metric": "collision queries/s", "value": value, "unit": "queries/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "impl": "reference",
        "config": {"workload": WORKLOAD.format(n=N_QUERIES), "queries_per_step": sample, "quadtree_depth": lay.depth,
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
    profiler_range(args.profile_range == "detect")
    t0 = time.perf_counter()
    for i in range(args.steps):
        flush.zero_()
        ev[i][0].record(stream)
        eng.detect_batch(dq, filter=filt, out=out, stream=stream)
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    if args.profile_range == "detect":
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
    if args.profile_range == "collect":
        profiler_range(True)
    for i in range(args.steps):
        flush.zero_()
        a_ev, b_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a_ev.record(stream)
        collect_once()
        b_ev.record(stream)
        c_ms.append((a_ev, b_ev))
    torch.cuda.synchronize()
    if args.profile_range == "collect":
        profiler_range(False)
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
    # the bounds this L2-resident, issue-limited kernel actually meets: L2 read bandwidth (the layout
    # lives in L2) and instruction issue (4 schedulers per SM, one warp instruction each per cycle)
    prof = read_profile(dom)
    l2_peak = l2_read_peak()
    n_sms = torch.cuda.get_device_properties(local).multi_processor_count
    avg_s = kernels[dom]["avg_ms"] / 1e3
    sm_hz = (clocks.get("sm_mhz") or 2070.0) * 1e6
    issue = None
    if prof.get("inst"):
        issue = {"inst_per_launch": prof["inst"], "issue_slots_per_launch": n_sms * 4 * sm_hz * avg_s,
                 "frac": prof["inst"] / (n_sms * 4 * sm_hz * avg_s), "sms": n_sms, "sm_mhz": sm_hz / 1e6,
                 "inst_source": prof["inst_source"] + " (ncu smsp__inst_executed.sum, one launch)"}
    l2 = None
    if l2_peak and prof.get("l2_sectors"):
        l2_gbs = prof["l2_sectors"] * 32 / avg_s / 1e9
        l2 = {"achieved": l2_gbs, "peak": l2_peak, "unit": "GB/s", "frac": l2_gbs / l2_peak,
              "bytes_per_launch": prof["l2_sectors"] * 32, "sectors_source": prof["l2_sectors_source"],
              "peak_source": "jcde_l2_read_peak: best of 3 runs x 16/32/48 MB L2-resident buffers, 20 passes of "
                             "16-byte ld.global.cg"}
    sub = {}
    if world == 1 and args.subrecords:
        # the other headline workloads of the metric, measured on this GPU in the same run
        t_sub = time.time()
        sub["batched"] = measure_multi(min(args.steps, 20), args.warmup, bool(args.autotune))
        sub["proxy"] = measure_proxy(min(args.steps, 5), 2, lay=lay)
        sub["lbf"] = measure_lbf(min(args.steps, 5), 2, oracle_check=not args.no_cpu)
        log(f"[bench] sub-records {time.time() - t_sub:.1f}s")
    line = {
        "metric": "collision queries/s", "value": value, "unit": "queries/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dev_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD.format(n=N_QUERIES), "queries_per_step": N_QUERIES, "quadtree_depth": lay.depth,
                   "cd_threshold": lay.cd_threshold, "l2": "flushed between steps (256 MB write)",
                   "parallelism": f"{world} rank(s), queries per rank, layout replicated"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "kernel": dom,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (burst copy)" if peaks else "fallback 6.8 TB/s",
                     "note": "achieved = oracle-counted algorithmic bytes / kernel time, a work rate: the layout is "
                             "L2-resident, so the kernel's real limits are the l2 and issue entries",
                     "l2": l2, "issue": issue,
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
    line.update(sub)
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def measure_multi(steps: int, warmup: int, autotune: bool = True, parity_queries: int = 1024):
    """The batched workload: 64 independent bin layouts, log-uniform 4,096-262,144 queries each, answered by one
    launch sequence (CUDA graph) versus 64 per-layout jcde_detect_batch calls.  Returns the record;
    the first `parity_queries` queries of every layout are checked against the oracle."""
    import torch

    import jcde
    from jcde import workload as W

    jcde.lib()
    t = time.time()
    lays = W.multi_layouts(jcde.GpuBackend)
    gen_s = time.time() - t
    log(f"[bench] {len(lays)} layouts, {sum(len(l.hazards) for l, _ in lays)} hazards ({gen_s:.1f}s)")
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
    multi_tuning, _ = m.autotune(dq, offs, stream=stream) if autotune else ({"poly_chunk": 2, "ordered": True}, 0)

    def plain():
        for l, eng in enumerate(engines):
            a, b = int(offs[l]), int(offs[l + 1])
            eng.detect_batch(dq[a * qb:b * qb], out=out_plain[a:b], stream=stream)

    def batched():
        m.detect(dq, offs, out=out_multi, stream=stream, graph=True)

    res = {}
    with torch.cuda.stream(stream):
        for name, fn in (("plain", plain), ("batched", batched)):
            for _ in range(warmup):
                fn()
            stream.synchronize()
            ms = []
            for _ in range(steps):
                flush.zero_()
                a_ev, b_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a_ev.record(stream)
                fn()
                b_ev.record(stream)
                ms.append((a_ev, b_ev))
            stream.synchronize()
            res[name] = sum(a.elapsed_time(b) for a, b in ms) / steps
    same = bool(torch.equal(out_plain, out_multi))
    # oracle parity on a sample of every layout (CPU leg, after the timed region)
    from oracle import oracle as O

    O.build()
    got = out_multi.cpu().numpy()
    mism = 0
    for l, (lay, _) in enumerate(lays):
        a = int(offs[l])
        ref = W.replay(O.OracleBackend, lay).detect_batch(q[a:a + parity_queries], n_threads=host_cores())
        mism += int((ref != got[a:a + parity_queries]).sum())
    return {
        "value": n / (res["batched"] / 1e3), "unit": "queries/s", "ms_per_step": res["batched"],
        "queries_per_step": n, "layouts": len(lays),
        "plain": {"value": n / (res["plain"] / 1e3), "ms_per_step": res["plain"]},
        "speedup_vs_plain": res["plain"] / res["batched"],
        "batched_tuning": multi_tuning,
        "same_verdicts_as_plain": same,
        "oracle_parity": {"queries": parity_queries * len(lays), "mismatches": mism, "bit_exact": mism == 0},
        "layout_generation_s": gen_s,
    }


def run_multi(args):
    """The multi-layout workload as its own bench line."""
    r = measure_multi(args.steps, args.warmup, bool(args.autotune))
    line = {
        "metric": "multi-layout collision queries/s", "value": r["value"], "unit": "queries/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": MULTI_WORKLOAD.format(n=r["queries_per_step"]),
                   "batched": "one ordering + surrogate + polygon launch sequence, CUDA-graph replay",
                   "plain": f"{r['layouts']} jcde_detect_batch calls, one per layout",
                   "l2": "flushed between steps (256 MB write)"},
        "impl": "jcde",
    }
    line.update({k: v for k, v in r.items() if k not in ("value", "unit", "ms_per_step")})
    print(json.dumps(line), flush=True)
    return 0


MULTI_WORKLOAD = ("64 star-container bins (32-128 v), 20-400 items each from 40 star types (8-200 v), "
                  "log-uniform 4,096-262,144 queries per bin ({n} total)")


def measure_proxy(steps: int, warmup: int, lay=None, grad_check: int = 1 << 16):
    """The gradient-separation workload: the star layout with surrogate poles on every
    interior hazard; 1,048,576 colliding candidates.  Measures (a) grads/s: the pole-overlap proxy and
    its adjoint d/d(theta, tx, ty) for every candidate (jcde_proxy_batch), (b) verified collision-free
    placements/s: 20 descent steps on the proxy then the exact verdict, versus 20 random
    perturbations per candidate judged by the exact verdict, (c) the gradient against an FP64
    evaluation of the same float32 inputs on `grad_check` candidates."""
    import torch

    import jcde
    from jcde import workload as W

    jcde.lib()
    if lay is None:
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
    g_val = torch.empty(n, dtype=torch.float32, device="cuda")
    g_grad = torch.empty(n, 3, dtype=torch.float32, device="cuda")

    def grads():
        eng.proxy_batch(P0, I0, filter=filt, out=(g_val, g_grad))
        return torch.zeros((), dtype=torch.int64, device="cuda") + n

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
    for name, fn in (("grads", grads), ("gradient", gd), ("random", rnd)):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        ms, succ = 0.0, 0
        for _ in range(steps):
            flush.zero_()
            a_ev, b_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a_ev.record()
            s_ = fn()
            b_ev.record()
            torch.cuda.synchronize()
            ms += a_ev.elapsed_time(b_ev)
            succ += int(s_.item())
        res[name] = {"per_s": succ / (ms / 1e3), "count": succ // steps, "ms_per_step": ms / steps, "candidates": n}
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
    for steps_ in (1, 2, 3, 5, 10, 20):
        def gd_s(steps_=steps_):
            q, _ = eng.separate_batch(P0.clone(), I0, steps=steps_, step_t=0.25, step_th=0.25, clearance=CLEARANCE,
                                      filter=filt)
            return (eng.detect_batch(q, filter=filt) == 0).sum()
        sweep[f"gradient_{steps_}_steps"] = once(gd_s)
    for kk in (1, 2, 5, 10, 20):
        out_kk = torch.empty(n * kk, dtype=torch.uint8, device="cuda")
        def rnd_k(kk=kk, out_kk=out_kk):
            q = eng.resample_batch(P0, I0, k=kk, sigma_t=mean_r, sigma_th=0.25, seed=7)
            eng.detect_batch(q, filter=filt, out=out_kk)
            return (out_kk.view(n, kk) == 0).any(dim=1).sum()
        sweep[f"random_{kk}_copies"] = once(rnd_k)
    best_g = max(v for k, v in sweep.items() if k.startswith("gradient"))
    best_r = max(v for k, v in sweep.items() if k.startswith("random"))
    # gradient accuracy against the FP64 evaluation (test infrastructure, CPU leg)
    from oracle import oracle as O

    O.build()
    ns = min(grad_check, n)
    v32 = g_val[:ns].cpu().numpy().astype(np.float64)
    g32 = g_grad[:ns].cpu().numpy().astype(np.float64)
    v64, g64 = O.proxy_f64(P0[:ns].cpu().numpy(), I0[:ns].cpu().numpy().astype(np.uint32),
                           [it.poles for it in lay.items], hp, ignored=filt, n_threads=host_cores())
    n64 = np.linalg.norm(g64, axis=1)
    on = n64 > 0
    rel = np.linalg.norm(g32[on] - g64[on], axis=1) / n64[on]
    rel_v = np.abs(v32[v64 > 0] - v64[v64 > 0]) / v64[v64 > 0]
    return {
        "grads_per_s": res["grads"]["per_s"], "grads_ms_per_step": res["grads"]["ms_per_step"],
        "value": res["gradient"]["per_s"], "unit": "placements/s", "ms_per_step": res["gradient"]["ms_per_step"],
        "candidates": n, "hazards_with_poles": int(len(np.unique(keys))),
        "gradient": {"placements_per_s": res["gradient"]["per_s"], "verified_free": res["gradient"]["count"],
                     "ms_per_step": res["gradient"]["ms_per_step"]},
        "random": {"placements_per_s": res["random"]["per_s"], "verified_free": res["random"]["count"],
                   "ms_per_step": res["random"]["ms_per_step"]},
        "speedup_vs_random": res["gradient"]["per_s"] / res["random"]["per_s"],
        "settings_sweep_placements_per_s": sweep,
        "best_setting_speedup": best_g / best_r,
        "grad_rel_err_vs_fp64": {"median": float(np.median(rel)), "p99": float(np.percentile(rel, 99)),
                                 "max": float(rel.max()), "candidates": int(ns), "with_gradient": int(on.sum()),
                                 "value_max_rel_err": float(rel_v.max()) if len(rel_v) else 0.0},
        "random_arm": f"{K} Gaussian perturbations per candidate (sigma_t={mean_r:.1f}, sigma_th=0.25) then "
                      "jcde_detect_batch",
    }


def run_proxy(args):
    """The gradient-separation workload as its own bench line."""
    r = measure_proxy(args.steps, args.warmup)
    line = {
        "metric": "CDE-verified collision-free placements/s (gradient separation)",
        "value": r["value"], "unit": "placements/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"star layout with surrogate poles on {r['hazards_with_poles']} hazards; "
                               f"{r['candidates']} colliding candidates; 20 descent steps on the pole-overlap proxy "
                               "(hazard poles grown by a 20-unit clearance) then jcde_detect_batch",
                   "random_arm": r["random_arm"], "l2": "flushed between steps (256 MB write)"},
        "impl": "jcde",
    }
    line.update({k: v for k, v in r.items() if k not in ("value", "unit", "ms_per_step", "random_arm")})
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


def measure_lbf(steps: int, warmup: int, oracle_check: bool = True, extras: bool = False, cpu_steps: int = 0):
    """The LBF-style strip build on the device-resident engine.  2000 steps, each: 16384
    candidates generated and searched as lbf's search does (surrogate pass for all; the polygon pass
    for those that could still beat the best free one, search.rs:52-56), the least-cost free one
    registered on the device, and a random placed item deregistered every 50 steps.  A timed step is
    one whole build from the strip's initial state.  Metric: candidate placements searched per
    second over the build.  With `oracle_check` the same build is driven through the oracle and its
    placements, removals and final quadtree are compared with the device build's."""
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

    def build():
        r.reset()
        r.lbf_begin(spec.seed, spec.n_cand, spec.n_types, spec.remove_every, spec.steps, spec.box, 0, 0, 0, (),
                    spec.uniform_rounds)
        with torch.cuda.stream(stream):
            flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        r.lbf_steps(spec.steps, SPG, stream=sh)
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b)

    for _ in range(warmup):
        build()
    launches0 = r.kernel_launches()
    clk = ClockSampler(0)
    clk.__enter__()
    profiler_range(True)
    times = [build() for _ in range(steps)]
    profiler_range(False)
    launches = r.kernel_launches() - launches0
    clk.__exit__()
    ms = float(np.sum(times))
    n_cand_total = spec.steps * spec.n_cand
    d = r.lbf_read()
    st = r.status()
    dev_tree = r.tree_dump()
    rec = {
        "value": n_cand_total * steps / (ms / 1e3), "unit": "candidates/s", "ms_per_build": ms / steps,
        "lbf_steps_per_s": spec.steps * steps / (ms / 1e3),
        "placed": int(len(d["placements"])), "removed": int(len(d["removals"])), "live": d["n_live"],
        "pool_use": st, "gpu_launches": int(launches), "clocks": clk.summary(),
        "workload": (f"LBF strip build: {spec.n_types} star types ({spec.v_range[0]}-{spec.v_range[1]} vertices), "
                     f"{spec.width:.0f} x {spec.height:.0f} strip, {spec.steps} steps x {spec.n_cand} candidates, "
                     f"removal every {spec.remove_every} steps; one timed step = one whole build; register/deregister "
                     f"on the device; {SPG} LBF steps per CUDA graph launch"),
    }
    # end to end through the public API: resident copy from the host engine, the build, the log read back
    e2e_ms = []
    h2d = d2h = 0
    for _ in range(max(1, min(steps, 3))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        h2d = r.reset()
        log_e2e, _ = lbf.run_device(geng, spec, steps_per_graph=SPG, resident=r)
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
        d2h = (log_e2e.placements.nbytes + log_e2e.removals.nbytes + log_e2e.free_counts.nbytes + 16)
    rec["e2e"] = {"value": n_cand_total / (np.median(e2e_ms) / 1e3), "unit": "candidates/s",
                  "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h), "ms_per_build": float(np.median(e2e_ms))}
    from jcde import workload as W

    def strip_length(placements, removals):
        """Largest x of the placed items still live (the strip length the build needs)."""
        gone = set(int(k) for k in removals[:, 1]) if len(removals) else set()
        xs = [W.transform_points(lay.items[int(p[3])].xy, *[np.uint32(v).view(np.float32) for v in p[4:8]])[:, 0].max()
              for p in placements if int(p[1]) not in gone]
        return float(max(xs)) if xs else 0.0

    rec["strip_length"] = strip_length(d["placements"], d["removals"])
    # lbf's search restated in rounds (search.rs:41-101): 4 uniform rounds of 4096, each over the box
    # tightened to the best cost so far / 10, then 3 local-search rounds of 2048 with Normal offsets
    spec_f = lbf.LbfSpec(uniform_rounds=4, ls_rounds=3, ls_cand=2048)
    f_ms = []
    for k in range(3):
        r.reset()
        r.lbf_begin(spec_f.seed, spec_f.n_cand, spec_f.n_types, spec_f.remove_every, spec_f.steps, spec_f.box, 0,
                    spec_f.ls_rounds, spec_f.ls_cand, spec_f.ls_sigmas(), spec_f.uniform_rounds)
        with torch.cuda.stream(stream):
            flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        r.lbf_steps(spec_f.steps, SPG, stream=sh)
        b.record(stream)
        torch.cuda.synchronize()
        if k:
            f_ms.append(a.elapsed_time(b))
    d_f = r.lbf_read()
    f_cands = spec_f.steps * (spec_f.n_cand + spec_f.ls_rounds * spec_f.ls_cand)
    rounds = d_f["placements"][:, 2] >> 24
    rec["lbf_search"] = {
        "ms_per_build": float(np.median(f_ms)), "candidates_per_s": f_cands / (np.median(f_ms) / 1e3),
        "uniform_rounds": spec_f.uniform_rounds, "local_rounds": spec_f.ls_rounds,
        "candidates_per_step": spec_f.n_cand + spec_f.ls_rounds * spec_f.ls_cand,
        "strip_length": strip_length(d_f["placements"], d_f["removals"]),
        "placements_from_tightened_rounds": int(((rounds >= 1) & (rounds < spec_f.uniform_rounds)).sum()),
        "placements_improved_by_local_search": int((rounds >= spec_f.uniform_rounds).sum()),
        "parity": "device build = oracle-driven build: tests/test_gpu_resident.py"}
    if oracle_check:
        from oracle import oracle as O

        O.build()
        lay_o, oeng = lbf.setup(O.OracleBackend, spec)
        t0 = time.perf_counter()
        olog = lbf.run_host(lay_o, oeng, spec)
        cpu_s = time.perf_counter() - t0
        rec["oracle_check"] = {
            "same_placements": bool(np.array_equal(olog.placements, d["placements"])),
            "same_removals": bool(np.array_equal(olog.removals, d["removals"])),
            "same_final_tree": bool(np.array_equal(oeng.tree_dump(), dev_tree)),
            "oracle_build_s": cpu_s, "oracle_cores": host_cores()}
        rec["cpu_baseline"] = {"value": n_cand_total / cpu_s, "unit": "candidates/s", "cores": host_cores(),
                               "kind": "port", "sample": "the whole build: oracle detect on all cores, numpy choice, "
                                                         "oracle register"}
    if extras:
        # per-kernel shares from one eager, profiled build (events around every launch)
        geng.eng.profile(True)
        r.reset()
        r.lbf_begin(spec.seed, spec.n_cand, spec.n_types, spec.remove_every, spec.steps, spec.box, 0, 0, 0, (),
                    spec.uniform_rounds)
        geng.eng.profile_read(reset=True)
        r.lbf_steps(spec.steps, 0, stream=sh)
        kp = geng.eng.profile_read(reset=True)
        geng.eng.profile(False)
        kinds = {k: {"ms_per_build": v[0], "launches": v[1]} for k, v in kp.items() if v[1]}
        rec["kernels_eager_build"] = kinds
        rec["dominant"] = max(kinds, key=lambda k: kinds[k]["ms_per_build"])
        # the same build driven step by step from the host through the regular engine (host
        # registration, a re-flattened tree upload per step): a bounded sample of its first steps
        host_steps = 200
        lay_h, geng_h = lbf.setup(jcde.GpuBackend, spec)
        t0 = time.perf_counter()
        hlog = lbf.run_host(lay_h, geng_h, spec, steps=host_steps)
        host_s = time.perf_counter() - t0
        rec["host_driven_gpu"] = {
            "value": host_steps * spec.n_cand / host_s, "unit": "candidates/s", "sample": f"first {host_steps} steps",
            "same_placements": bool(np.array_equal(hlog.placements, d["placements"][: len(hlog.placements)]))}
    return rec


def run_lbf(args):
    """The LBF build as its own bench line."""
    r = measure_lbf(args.steps, args.warmup, oracle_check=not args.no_cpu, extras=True)
    line = {
        "metric": "LBF candidate placements searched per second (device-resident build)",
        "value": r["value"], "unit": "candidates/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": r["ms_per_build"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": r["workload"], "l2": "flushed between builds (256 MB write)"},
        "impl": "jcde",
    }
    line.update({k: v for k, v in r.items() if k not in ("value", "unit", "workload")})
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
    ap.add_argument("--subrecords", type=int, default=1,
                    help="1: the default (star) line also measures the batched multi-layout, proxy and LBF workloads")
    ap.add_argument("--prep-shapes", type=int, default=1024, help="prep workload: shapes per batch")
    ap.add_argument("--profile-range", default="detect", choices=["detect", "collect"],
                    help="star workload: the timed loop bracketed by cudaProfilerStart/Stop (for ncu captures)")
    ap.add_argument("--queries", type=int, default=1 << 20,
                    help="star workload: queries per step (smaller batches serve profiling captures)")
    ap.add_argument("--workload", default="star", choices=["star", "multi", "proxy", "lbf", "prep", "bpp"],
                    help="star: the headline single-layout batch; multi: 64 layouts in one launch sequence; "
                         "proxy: gradient separation of colliding candidates vs random resampling; "
                         "lbf: LBF-style build on the device-resident engine; "
                         "prep: poi + surrogate poles of 1024 item shapes on the device; "
                         "bpp: bin packing with lbf's bin-packing optimizer")
    args = ap.parse_args()
    global N_QUERIES
    N_QUERIES = args.queries
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
