#!/usr/bin/env python
"""GROUP BY benchmark on GB300.

Workload (one step = one full GROUP BY pass): the high-cardinality radix
GROUP BY — 100,000,000 rows, seed 1; k INT64 Zipf(s=1.1) over 20,000,000
values (ranks mapped into [0, 2^40) by a seeded permutation); x DOUBLE ~
Normal(100, 25);  SELECT k, COUNT(*), SUM(x), AVG(x) FROM t GROUP BY k,
materialising the full result in HBM and the ORDER BY COUNT(*) DESC
LIMIT 10 TopN on it.

  value  — rows/s with the columns resident in HBM (device-timed).
  e2e    — rows/s through the C ABI with pinned HOST buffers: host→HBM copy
           of the columns, the GROUP BY, and the device→host copy of the
           full result, every step.

  parity — the full GROUP BY result and the TopN checked against the
           oracle over the same 100M rows (outside the timed region): keys
           and COUNT equal, SUM/AVG max relative error vs the compensated
           FP64 sum (bar 1e-12), reported per query.

Inputs (1.6 GB) are larger than L2 (129 MB), so no L2 flush is needed.
``--impl reference`` times the CPU restatement of the reference's GROUP BY
(per-thread maps + shard merge, all host cores) over the same 100M rows.
Multi-GPU: the path runs as independent replicas (one full workload per
rank, no collective); value = rows of all ranks / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "GROUP BY rows/s & HBM GB/s at 100M rows; batched queries/s and p99 vs plain"
N_VALUES = 20_000_000
EST_GROUPS = 8_000_000  # planner estimate handed to the operator
# DRAM bytes per input row of the dominant kernel (one ncu capture of the
# 30M-row case of the same workload): (490.7 MB read + 127.5 MB written) /
# 30M rows
TRAFFIC_PER_ROW = {"k_partition": (490.74 + 127.53) * 1e6 / 30e6}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--rows", type=int, default=100_000_000)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--cpu-sample", type=int, default=20_000_000)
    ap.add_argument("--workload", default="zipf100m", choices=["zipf100m", "plain1m", "batch256", "serve",
                                                                      "parquet200m", "parquet200m_snappy",
                                                                      "parquet200m_zstd", "dictsum200m",
                                                                      "distinct100m"])
    ap.add_argument("--pq-rows", type=int, default=200_000_000, help="parquet200m: rows in the file")
    ap.add_argument("--tables", type=int, default=256)
    ap.add_argument("--duration", type=float, default=120.0, help="serve: seconds of Poisson arrivals")
    ap.add_argument("--rate", type=float, default=200.0, help="serve: arrivals per second")
    ap.add_argument("--scale", type=float, default=1.0, help="serve: resident table scale (1.0 = ~66 GB)")
    ap.add_argument("--budget-gb", type=float, default=40.0, help="serve: admission budget")
    ap.add_argument("--lanes", type=int, default=2, help="serve: execution lanes of the batched server")
    ap.add_argument("--capacity-queries", type=int, default=3000,
                    help="serve: queries of the stream submitted at once to measure each mode's capacity")
    return ap.parse_args()


def max_over_ranks(ms, device="cuda"):
    """The slowest rank's time (replicas: every rank runs a full workload)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return ms
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, world_size, ms):
    """Units of all ranks / the max-over-ranks time (weak scaling)."""
    return units_per_rank * world_size / (ms / 1e3)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """SM clocks and throttle reasons sampled during a timed region: NVML
    (libnvidia-ml through ctypes, read-only queries) every 10 ms from a
    thread, so even a region of a few tens of milliseconds gets samples;
    nvidia-smi at 200 ms where NVML cannot be loaded."""

    # nvmlClocksEventReasons bits (nvml.h)
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
               0x80: "hw_power_brake_slowdown"}
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0, period_s=0.01):
        self.idx = gpu_index
        self.period = period_s
        self.sm, self.smax, self.reasons = [], [], set()
        self.nvml = self.dev = None
        self.th = self.p = self.f = None
        try:
            import ctypes
            lib = ctypes.CDLL("libnvidia-ml.so.1")
            if lib.nvmlInit_v2() == 0:
                dev = ctypes.c_void_p()
                if lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(gpu_index), ctypes.byref(dev)) == 0:
                    self.nvml, self.dev = lib, dev
                    self.fn_reasons = (getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None)
                                       or getattr(lib, "nvmlDeviceGetCurrentClocksThrottleReasons", None))
        except Exception:
            self.nvml = None

    def _sample_nvml(self):
        import ctypes
        clk, mx, rs = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_ulonglong()
        while not self.stop_flag:
            try:
                if self.nvml.nvmlDeviceGetClockInfo(self.dev, 1, ctypes.byref(clk)) == 0:  # NVML_CLOCK_SM
                    self.sm.append(float(clk.value))
                if self.nvml.nvmlDeviceGetMaxClockInfo(self.dev, 1, ctypes.byref(mx)) == 0:
                    self.smax.append(float(mx.value))
                if self.fn_reasons is not None and self.fn_reasons(self.dev, ctypes.byref(rs)) == 0:
                    for bit, nm in self.REASONS.items():
                        if rs.value & bit:
                            self.reasons.add(nm)
            except Exception:
                self.reasons.add("sampling error")
                return
            time.sleep(self.period)

    def start(self):
        self.stop_flag = False
        if self.nvml is not None:
            import threading
            self.th = threading.Thread(target=self._sample_nvml, daemon=True)
            self.th.start()
            return
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        self.stop_flag = True
        if self.th is not None:
            self.th.join()
            src = "nvml"
        elif self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["clock sampling unavailable"]}
        else:
            src = "nvidia-smi"
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()
            self.f.flush()
            self.f.seek(0)
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            for ln in self.f.read().splitlines():
                parts = [x.strip() for x in ln.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    self.sm.append(float(parts[1]))
                    self.smax.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, val in zip(names, parts[5:9]):
                    if val.lower().startswith("active"):
                        self.reasons.add(nm)
            os.unlink(self.f.name)
        return {"sm_mhz": statistics.median(self.sm) if self.sm else None,
                "sm_max_mhz": max(self.smax) if self.smax else None,
                "reasons": sorted(self.reasons), "samples": len(self.sm), "source": src}


def gen_data(rows):
    from slothdb_gb300 import datagen
    t = time.time()
    k, x = datagen.zipf(rows, seed=1, n_values=N_VALUES)
    return k, x, time.time() - t


def oracle_zipf(k, x, threads):
    """The oracle's CPU restatement of the reference GROUP BY (per-thread
    maps + sharded merge) over every row given; returns (result, seconds)."""
    import oracle
    aggs = [("count_star", -1), ("sum", 1), ("avg", 1)]
    t = time.perf_counter()
    orc = oracle.run_query([3, 4], [0], aggs, [k, x], nthreads=threads, est_groups=N_VALUES // 4,
                           max_groups=N_VALUES)
    return orc, time.perf_counter() - t


REL_TOL_F64 = 1e-12  # DOUBLE SUM/AVG: relative error against the FP64 compensated sum, per query


def ref_threads(path):
    """Host threads the reference itself uses on a path, which its CPU
    baseline (the oracle port) is timed with: the in-memory chunk loop of
    PhysicalHashAggregate runs on one thread (physical_planner.cpp:7933-8021);
    the fused Parquet path (TLSingle, physical_planner.cpp:7613-7931) runs
    its row groups on up to 8 worker threads."""
    return min(8, os.cpu_count() or 1) if path == "parquet" else 1


def hbm_peak_gbs():
    """(HBM copy bandwidth GB/s, "measured"|"fallback") for the roofline."""
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(peaks["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def oracle_mismatch(res, orc, nk):
    """None when a GPU result (list of (values, valid) per output column,
    keys first) holds the oracle's groups with equal integer aggregates and
    DOUBLE aggregates within REL_TOL_F64 of the compensated sums; else a
    one-line description of the first difference."""
    n = len(res[0][0])
    if n != orc["n_groups"]:
        return "%d groups vs %d" % (n, orc["n_groups"])

    def order(keys, valid):
        cols = []
        for kv, vv in zip(keys, valid):
            kv = np.asarray(kv)
            if kv.dtype == object:
                kv = kv.astype("S")
            cols += [np.where(vv, kv, kv[:0].dtype.type()) if kv.size else kv, ~np.asarray(vv, bool)]
        return np.lexsort(cols[::-1]) if cols else np.arange(n)

    og = order([res[j][0] for j in range(nk)], [res[j][1] for j in range(nk)])
    oo = order(orc["keys"], [~np.asarray(m, bool) for m in orc["key_null"]])
    for j in range(nk):
        gv, gm = np.asarray(res[j][0])[og], np.asarray(res[j][1], bool)[og]
        ov, om = np.asarray(orc["keys"][j])[oo], ~np.asarray(orc["key_null"][j], bool)[oo]
        if gv.dtype == object or ov.dtype == object:
            gv, ov = gv.astype("S"), ov.astype("S")
        if not (np.array_equal(gm, om) and np.array_equal(gv[gm], ov[om])):
            return "key column %d differs" % j
    for i, (ov, onull, comp) in enumerate(orc["aggs"]):
        gv, gm = np.asarray(res[nk + i][0])[og], np.asarray(res[nk + i][1], bool)[og]
        om = ~np.asarray(onull, bool)[oo]
        if not np.array_equal(gm, om):
            return "aggregate %d: NULLs differ" % i
        if gv.dtype == np.float64:
            r = comp[oo][om]
            e = np.abs(gv[gm] - r) / np.maximum(np.abs(r), np.finfo(np.float64).tiny)
            if e.size and float(e.max()) > REL_TOL_F64:
                return "aggregate %d: rel err %.2e" % (i, float(e.max()))
        elif not np.array_equal(gv[gm].astype(np.int64), np.asarray(ov)[oo][om].astype(np.int64)):
            return "aggregate %d differs" % i
    return None


def parity_zipf(k, x, full, top, threads=None):
    """Full-size parity of the 100M-row GROUP BY: the oracle runs the same
    query over the same rows (every host thread, outside the timed region)
    and the GPU's full result and TopN are compared with it.  Group keys,
    COUNT and the TopN keys/counts must be equal; SUM(x) and AVG(x) are
    reported as the max relative error against the oracle's compensated FP64
    sums (bar: 1e-12).  Returns the JSON fields and the oracle's timing."""
    threads = threads or os.cpu_count() or 1
    orc, orc_s = oracle_zipf(k, x, threads)
    ok = orc["keys"][0].astype(np.int64)
    oc = orc["aggs"][0][0].astype(np.int64)
    os_ = orc["aggs"][1][2]
    oa = orc["aggs"][2][2]
    gk = full[0][0].astype(np.int64)
    go_, oo = np.argsort(gk, kind="stable"), np.argsort(ok, kind="stable")
    out = {"n_groups_gpu": int(len(gk)), "n_groups_oracle": int(len(ok)), "groups_equal": False,
           "int_mismatches": None, "max_rel_err_f64": None, "tol_f64": REL_TOL_F64}
    if len(gk) == len(ok) and np.array_equal(gk[go_], ok[oo]):
        out["groups_equal"] = True
        gc = full[1][0].astype(np.int64)[go_]
        out["int_mismatches"] = int(np.count_nonzero(gc != oc[oo]))
        errs = {}
        for name, col, ref in (("sum", 2, os_), ("avg", 3, oa)):
            r = ref[oo]
            e = np.abs(full[col][0][go_] - r) / np.maximum(np.abs(r), np.finfo(np.float64).tiny)
            errs[name] = float(e.max()) if e.size else 0.0
        out["max_rel_err_f64"] = errs
        out["within_tol"] = max(errs.values()) <= REL_TOL_F64
    # TopN 10 by COUNT(*) DESC, ties by key ASC
    order = np.lexsort((ok, -oc))[:10]
    tk, tc = top[0][0].astype(np.int64), top[1][0].astype(np.int64)
    out["topn_equal"] = bool(np.array_equal(tk, ok[order]) and np.array_equal(tc, oc[order]))
    out["top_group_rows"] = int(oc[order[0]]) if len(order) else 0
    out["topn_boundary_tie"] = bool(len(oc) > 10 and np.sort(oc)[::-1][9] == np.sort(oc)[::-1][10])
    if len(order):
        ti = order[0]
        out["top_group_sum_rel_err"] = float(abs(full[2][0][go_][np.searchsorted(gk[go_], ok[ti])] - os_[ti])
                                             / abs(os_[ti])) if out["groups_equal"] else None
    out["oracle"] = {"threads": threads, "seconds": round(orc_s, 2), "rows": int(len(k))}
    return out, orc_s


def zipf_cpu_sample(args, k, x):
    """The CPU baseline's sample of the 100M-row workload: its first
    --cpu-sample rows through the oracle port on the reference's thread
    count; returns (rows/s, cpu_baseline dict)."""
    n = min(args.cpu_sample, len(k))
    thr = ref_threads("memory")
    _, dt = oracle_zipf(k[:n], x[:n], thr)
    return n / dt, {"value": n / dt, "unit": "rows/s", "cores": thr, "kind": "port",
                    "sample": "first %d rows of the workload, oracle port on %d thread (the reference's in-memory "
                              "chunk loop is single-threaded)" % (n, thr)}


def run_reference(args):
    """The CPU arm: the oracle's restatement of the reference GROUP BY on the
    reference's own thread count, a bounded sample of the 100M-row workload
    per step (rank 0 only)."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    k, x, _ = gen_data(args.rows)
    oracle_zipf(k[:100_000], x[:100_000], 1)
    times, cpu = [], None
    for i in range(args.warmup + args.steps):
        if i < args.warmup:  # untimed: a short prefix warms the code and allocator
            oracle_zipf(k[:1_000_000], x[:1_000_000], 1)
            continue
        val, cpu = zipf_cpu_sample(args, k, x)
        times.append(min(args.cpu_sample, len(k)) / val)
    per = statistics.mean(times)
    n = min(args.cpu_sample, len(k))
    val = n / per
    threads = cpu["cores"]
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": "rows/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": per * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int64+f64", "data": "synthetic",
            "config": {"workload": "zipf-groupby-100M", "rows": args.rows, "distinct_values": N_VALUES,
                       "aggs": "COUNT(*),SUM(x),AVG(x)", "sample_rows": n},
            "cpu_baseline": {"value": val, "unit": "rows/s", "cores": threads, "kind": "port",
                             "sample": "first %d rows of the workload per step, %d thread (the reference's "
                                       "in-memory chunk loop is single-threaded)" % (n, threads)},
            "e2e": {"value": val, "unit": "rows/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


PLAIN_AGGS = [("count_star", -1), ("sum", 1), ("min", 1), ("max", 1)]


def run_plain(args):
    """The CPU-runnable plain GROUP BY: 1,000,000 rows, seed 0; k INT32
    uniform over 1,024 values, v INT64 uniform in [0, 10^6); SELECT k,
    COUNT(*), SUM(v), MIN(v), MAX(v) FROM t GROUP BY k.  The 12 MB of
    columns fit in L2, so a 256 MB buffer is written between timed steps
    (outside the CUDA events) and every step reads its inputs from HBM.
    value = rows/s with the columns resident in HBM; e2e = rows/s through
    the C ABI from pinned host buffers with the result read back; parity =
    the oracle's result over the same rows, bit-exact.  Multi-GPU: replicas."""
    ws, rank, local = dist_env()
    from slothdb_gb300 import datagen
    k, v = datagen.plain(1_000_000, seed=0, n_keys=1024)
    rows = len(k)
    if args.impl == "reference":
        return run_plain_reference(args, k, v) if rank == 0 else None
    import torch
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from slothdb_gb300 import capi
    capi.load(build_if_missing=True)
    hbm_peak, peak_src = hbm_peak_gbs()
    types = [capi.INTEGER, capi.BIGINT]
    dk, dv = torch.from_numpy(k).cuda(), torch.from_numpy(v).cuda()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    g = capi.GroupBy(types, [0], PLAIN_AGGS, est_groups=1024)

    def step():
        g.reset()
        g.ingest([dk, dv], nrows=rows, device=True, stream=sp)
        g.finalize(stream=sp)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    g.set_profiling(True)
    flush.fill_(1)
    step()
    prof = {kk: vv[1] / max(1, vv[0]) for kk, vv in g.profile().items()}
    g.set_profiling(False)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = Clocks(local)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    launches = 0
    for i, (e0, e1) in enumerate(evs):
        flush.fill_(i & 255)  # evict the columns from L2 (outside the events)
        e0.record(stream)
        step()
        e1.record(stream)
        launches += g.launches()
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    ms = max_over_ranks(sum(a.elapsed_time(b) for a, b in evs) / args.steps)
    res = g.result()
    in_bytes = rows * 12
    dom = max(prof, key=prof.get) if prof else "k_ingest"
    kms = prof.get(dom, float("nan"))
    roofline = {"bound": "hbm", "achieved": in_bytes / (kms / 1e3) / 1e9, "peak": hbm_peak, "unit": "GB/s",
                "frac": in_bytes / (kms / 1e3) / 1e9 / hbm_peak, "traffic": None, "kernel": dom, "kernel_ms": kms,
                "peak_source": peak_src, "step_GBps": in_bytes / (ms / 1e3) / 1e9, "kernels_ms": prof}
    # e2e from pinned host buffers through the C ABI
    pk, pv = capi.PinnedBuffer(rows * 4), capi.PinnedBuffer(rows * 8)
    pk.view(np.int32)[:] = k
    pv.view(np.int64)[:] = v
    ge = capi.GroupBy(types, [0], PLAIN_AGGS, est_groups=1024)

    def step_e2e():
        ge.reset()
        ge.ingest([pk.ptr, pv.ptr], nrows=rows, stream=sp)
        ge.finalize(stream=sp)
        return ge.result_host_bytes()[1]

    for _ in range(3):
        d2h = step_e2e()
    torch.cuda.synchronize()
    ne = max(10, args.steps)
    tt = time.perf_counter()
    for _ in range(ne):
        d2h = step_e2e()
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - tt) / ne
    ge.close()
    pk.close()
    pv.close()
    parity = cpu = None
    if rank == 0:
        import oracle
        thr = os.cpu_count() or 1
        orc = oracle.run_query(types, [0], PLAIN_AGGS, [k, v], nthreads=thr)
        diff = oracle_mismatch(res, orc, 1)
        parity = {"bit_exact": diff is None, "groups": int(orc["n_groups"]), "first_difference": diff}
        rt = ref_threads("memory")
        reps, tc = 0, time.perf_counter()
        while time.perf_counter() - tc < 5.0:
            oracle.run_query(types, [0], PLAIN_AGGS, [k, v], nthreads=rt)
            reps += 1
        per = (time.perf_counter() - tc) / reps
        cpu = {"value": rows / per, "unit": "rows/s", "cores": rt, "kind": "port",
               "sample": "the full 1M-row query, %d repetitions, %d thread (the reference's in-memory chunk loop)"
                         % (reps, rt)}
        line = {"metric": "plain GROUP BY rows/s (1M rows, 1,024 groups)", "value": whole_job_rate(rows, ws, ms),
                "unit": "rows/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int64",
                "data": "synthetic",
                "config": {"workload": "plain-groupby-1M", "rows": rows, "groups": 1024,
                           "key": "INT32 uniform over 1,024", "aggs": "COUNT(*),SUM(v),MIN(v),MAX(v)",
                           "l2": "inputs 12 MB < L2: 256 MB buffer written between timed steps",
                           "parallelism": "replicas" if ws > 1 else "single"},
                "roofline": roofline, "cpu_baseline": cpu, "parity": parity,
                "e2e": {"value": rows * ws / e2e_s, "unit": "rows/s", "h2d_bytes_per_step": in_bytes,
                        "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s * 1e3},
                "clocks": clk, "gpu_launches": launches}
        print(json.dumps(line), flush=True)
    g.close()
    if ws > 1:
        torch.distributed.destroy_process_group()


def run_plain_reference(args, k, v):
    """The oracle over the same 1M rows on the reference's thread count, one
    query per step."""
    import oracle
    thr = ref_threads("memory")
    times = []
    for i in range(args.warmup + args.steps):
        t = time.perf_counter()
        oracle.run_query([2, 3], [0], PLAIN_AGGS, [k, v], nthreads=thr)
        if i >= args.warmup:
            times.append(time.perf_counter() - t)
    per = statistics.mean(times)
    val = len(k) / per
    line = {"impl": "reference", "metric": "plain GROUP BY rows/s (1M rows, 1,024 groups)", "value": val,
            "unit": "rows/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": per * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int64", "data": "synthetic",
            "config": {"workload": "plain-groupby-1M", "rows": len(k), "groups": 1024},
            "cpu_baseline": {"value": val, "unit": "rows/s", "cores": thr, "kind": "port",
                             "sample": "the full 1M-row query per step, %d thread" % thr},
            "e2e": {"value": val, "unit": "rows/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_batch(args):
    """256 independent GROUP BY tables (rows log-uniform in [10^4, 10^7],
    groups log-uniform in [10^2, 10^6]; 75% (INT32, INT16) keys, 25% VARCHAR
    keys of 8..32 chars; COUNT(*), SUM(INT64), MAX(INT32)), resident in HBM.
    One step runs every query.  value = queries/s through gb_batch (work
    queue + CUDA graph); plain = the same queries one after another, each
    through its own operator handle (ingest + finalize per query)."""
    ws, rank, local = dist_env()
    if args.impl == "reference":  # host cores only; rank 0 alone under torchrun
        return run_batch_reference(args) if rank == 0 else None
    import torch
    torch.cuda.set_device(local)
    from slothdb_gb300 import capi, datagen
    capi.load(build_if_missing=True)
    t0 = time.time()
    shapes = datagen.batch_shapes(n_tables=args.tables, seed=3)
    tables = [datagen.batch_table_device(sh) for sh in shapes]
    torch.cuda.synchronize()
    gen_s = time.time() - t0
    total_rows = sum(sh["rows"] for sh in shapes)
    in_bytes = 0
    for sh, cols in zip(shapes, tables):
        for c in cols:
            if isinstance(c, tuple):
                in_bytes += c[0].numel() * 8 + c[1].numel()
            else:
                in_bytes += c.numel() * c.element_size()

    def spec(sh):
        return datagen.BATCH_COMPOSITE if sh["kind"] == "composite" else datagen.BATCH_VARCHAR

    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    b = capi.Batch()
    for sh, cols in zip(shapes, tables):
        q = spec(sh)
        b.add(q["col_types"], q["group_cols"], q["aggs"], cols, sh["rows"], est_groups=sh["groups"])
    plain = []
    for sh in shapes:
        q = spec(sh)
        plain.append(capi.GroupBy(q["col_types"], q["group_cols"], q["aggs"], est_groups=sh["groups"]))

    def step_plain():
        for g, sh, cols in zip(plain, shapes, tables):
            g.reset()
            g.ingest(cols, nrows=sh["rows"], device=True, stream=sp)
            g.finalize(stream=sp)

    def timed(fn, steps):
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    for _ in range(args.warmup):
        b.run(stream=sp)
        step_plain()
    torch.cuda.synchronize()
    # parity: every batched result equals the same query run alone
    mismatches = 0
    for i, g in enumerate(plain):
        rb, rp = b.result(i), g.result()
        order_b = np.lexsort([rb[k][0] for k in range(len(spec(shapes[i])["group_cols"]))][::-1]) \
            if shapes[i]["kind"] == "composite" else np.argsort(rb[0][0].astype("S"), kind="stable")
        order_p = np.lexsort([rp[k][0] for k in range(len(spec(shapes[i])["group_cols"]))][::-1]) \
            if shapes[i]["kind"] == "composite" else np.argsort(rp[0][0].astype("S"), kind="stable")
        for (vb, nb), (vp, np_) in zip(rb, rp):
            if len(vb) != len(vp) or not (np.array_equal(vb[order_b], vp[order_p])
                                          and np.array_equal(nb[order_b], np_[order_p])):
                mismatches += 1
                break
    slow = b.slow_queries()
    b.set_option("profiling", 1)
    b.run(stream=sp)
    prof = {k: v[1] / max(1, v[0]) for k, v in b.profile().items()}
    b.set_option("profiling", 0)
    b.run(stream=sp)
    clocks = Clocks(local)
    clocks.start()
    launches0 = b.launches()
    ms_batch = timed(lambda: b.run(stream=sp), args.steps)
    launches = b.launches() - launches0
    clk = clocks.stop()
    plain_steps = max(1, min(args.steps, 5))
    ms_plain = timed(step_plain, plain_steps)
    nq = len(shapes)
    value = nq / (ms_batch / 1e3)

    # roofline of the ingest phase (the batch's dominant kernels, one launch
    # per size class): algorithmic bytes = the columns it reads once, 18 B/row
    # for (INT32, INT16) tables (keys 6 + SUM 8 + MAX 4), 20 B/row for VARCHAR
    # tables (8-byte string id + 8 + 4); the string pass (k_batch_strdict)
    # reads offsets 8 B/row + the string bytes and writes the 8-byte ids
    hbm_peak, peak_src = hbm_peak_gbs()
    ing_bytes = sum(sh["rows"] * (18 if sh["kind"] == "composite" else 20) for sh in shapes)
    str_bytes = sum(cols[0][0].numel() * 8 + cols[0][1].numel() + sh["rows"] * 8
                    for sh, cols in zip(shapes, tables) if sh["kind"] == "varchar")
    ing_ms = prof.get("k_batch_ingest", float("nan"))
    str_ms = prof.get("k_batch_strdict", float("nan"))
    roofline = {"bound": "hbm", "achieved": ing_bytes / (ing_ms / 1e3) / 1e9, "peak": hbm_peak, "unit": "GB/s",
                "frac": ing_bytes / (ing_ms / 1e3) / 1e9 / hbm_peak, "traffic": None,
                "kernel": "k_batch_fast/k_batch_generic (ingest phase)", "kernel_ms": ing_ms,
                "algorithmic_bytes": ing_bytes, "peak_source": peak_src,
                "strdict": {"ms": str_ms, "algorithmic_bytes": str_bytes,
                            "GBps": str_bytes / (str_ms / 1e3) / 1e9 if str_bytes else None},
                "step_GBps": in_bytes / (ms_batch / 1e3) / 1e9}

    # e2e through the public API from pinned host memory: every step copies
    # each table's columns host→HBM into the tensors the batch is bound to,
    # runs the batch and reads every query's full result into host memory
    e2e = None
    if not args.no_e2e:
        def pinned(t):
            h = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
            h.copy_(t)
            return h
        host = [[(pinned(c[0]), pinned(c[1])) if isinstance(c, tuple) else pinned(c) for c in cols]
                for cols in tables]
        pairs = []
        for dcols, hcols in zip(tables, host):
            for dc, hc in zip(dcols, hcols):
                pairs += list(zip(dc, hc)) if isinstance(dc, tuple) else [(dc, hc)]
        d2h = 0

        def step_e2e():
            for dc, hc in pairs:
                dc.copy_(hc, non_blocking=True)
            b.run(stream=sp)
            return sum(b.result_host_bytes(i)[1] for i in range(nq))

        step_e2e()
        torch.cuda.synchronize()
        ne = max(1, args.steps // 2)
        tt = time.perf_counter()
        for _ in range(ne):
            d2h = step_e2e()
        torch.cuda.synchronize()
        e2e_s = (time.perf_counter() - tt) / ne
        e2e = {"value": nq / e2e_s, "unit": "queries/s", "h2d_bytes_per_step": in_bytes,
               "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s * 1e3}
        del host, pairs

    # oracle parity: every query's full result against the oracle over the
    # same table (the device columns copied to the host), integers bit-exact;
    # the same pass (one query per host thread) is the timed CPU baseline
    import oracle
    from concurrent.futures import ThreadPoolExecutor
    host_tabs = [[(c[0].cpu().numpy(), c[1].cpu().numpy()) if isinstance(c, tuple) else c.cpu().numpy()
                  for c in cols] for cols in tables]
    thr = os.cpu_count() or 1

    def one(i):
        q = spec(shapes[i])
        return oracle.run_query(q["col_types"], q["group_cols"], q["aggs"], host_tabs[i], nthreads=1,
                                max_groups=shapes[i]["groups"] + 64)

    by_size = sorted(range(nq), key=lambda i: -shapes[i]["rows"])
    tc = time.perf_counter()
    with ThreadPoolExecutor(thr) as ex:
        orcs = dict(zip(by_size, ex.map(one, by_size)))
    orc_s = time.perf_counter() - tc
    diffs = []
    for i in range(nq):
        d = oracle_mismatch(b.result(i), orcs[i], len(spec(shapes[i])["group_cols"]))
        if d:
            diffs.append("q%d (%s, %d rows): %s" % (i, shapes[i]["kind"], shapes[i]["rows"], d))
    del host_tabs, orcs
    smp = BatchCpuSample(args)
    cpu = smp.baseline(smp.seconds(), nq)
    cpu["all_queries_parallel"] = {"value": nq / orc_s, "threads": thr,
                                   "sample": "all %d queries (%d rows), one query per thread (the parity pass)"
                                             % (nq, total_rows)}
    line = {"metric": "batched GROUP BY queries/s (256 uneven tables) vs sequential plain launches",
            "value": value, "unit": "queries/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_batch, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int64", "data": "synthetic",
            "config": {"workload": "batch-%d-tables" % nq, "tables": nq, "total_rows": total_rows,
                       "varchar_tables": sum(sh["kind"] == "varchar" for sh in shapes),
                       "input_bytes": in_bytes, "aggs": "COUNT(*),SUM(INT64),MAX(INT32)",
                       "l2": "inputs %.1f GB > L2 129 MB (no flush needed)" % (in_bytes / 1e9),
                       "datagen_s": round(gen_s, 1)},
            "rows_per_s": total_rows / (ms_batch / 1e3), "input_GBps": in_bytes / (ms_batch / 1e3) / 1e9,
            "plain": {"value": nq / (ms_plain / 1e3), "unit": "queries/s", "ms_per_step": ms_plain,
                      "steps": plain_steps},
            "speedup_vs_plain": ms_plain / ms_batch, "parity_mismatches": mismatches, "slow_queries": slow,
            "parity": {"oracle_mismatches": len(diffs), "queries": nq, "first": diffs[:4],
                       "batch_vs_plain_mismatches": mismatches},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
            "kernels_ms": prof,
            "clocks": clk, "gpu_launches": launches}
    print(json.dumps(line), flush=True)
    b.close()
    for g in plain:
        g.close()


class BatchCpuSample:
    """The batch workload's CPU baseline: the reference's generic chunk loop
    restated in the oracle, queries one after another on one thread each,
    over a bounded sample (the first tables, in generation order, up to
    about 20M rows, host-generated with the same shapes)."""

    def __init__(self, args):
        from slothdb_gb300 import datagen
        shapes = datagen.batch_shapes(n_tables=args.tables, seed=3)
        self.picked, self.rows = [], 0
        for sh in shapes:
            if self.rows + sh["rows"] > 20_000_000 and self.picked:
                continue
            self.picked.append(sh)
            self.rows += sh["rows"]
        self.tabs = [datagen.batch_table_host(sh) for sh in self.picked]

    def seconds(self):
        import oracle
        from slothdb_gb300 import datagen
        t = time.perf_counter()
        for sh, cols in zip(self.picked, self.tabs):
            q = datagen.BATCH_COMPOSITE if sh["kind"] == "composite" else datagen.BATCH_VARCHAR
            oracle.run_query(q["col_types"], q["group_cols"], q["aggs"], cols, nthreads=ref_threads("memory"))
        return time.perf_counter() - t

    def baseline(self, per, n_tables):
        return {"value": len(self.picked) / per, "unit": "queries/s", "cores": ref_threads("memory"),
                "kind": "port", "sample": "%d of the %d tables (%d rows), sequential, 1 thread" % (
                    len(self.picked), n_tables, self.rows)}


def run_batch_reference(args):
    """The batch CPU baseline (BatchCpuSample) timed per step."""
    smp = BatchCpuSample(args)
    picked, rows = smp.picked, smp.rows
    times = []
    for i in range(args.warmup + args.steps):
        dt = smp.seconds()
        if i >= args.warmup:
            times.append(dt)
    per = statistics.mean(times)
    val = len(picked) / per
    line = {"impl": "reference", "metric": "batched GROUP BY queries/s (256 uneven tables) vs sequential plain launches",
            "value": val, "unit": "queries/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": per * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int64", "data": "synthetic",
            "config": {"workload": "batch-%d-tables (bounded sample: %d tables, %d rows)" % (
                args.tables, len(picked), rows)},
            "cpu_baseline": smp.baseline(per, args.tables),
            "e2e": {"value": val, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _serve_stream(srv, queries, t0_wall, on_done):
    """Submit `queries` at their arrival times (seconds after t0_wall) from a
    thread while this thread waits for each ticket in submission order and
    hands it to on_done(i, ticket), which releases it (results are not held
    for the whole stream)."""
    import threading
    tickets = [None] * len(queries)
    ready = threading.Semaphore(0)
    errors = []

    def submitter():
        try:
            for i, q in enumerate(queries):
                delay = t0_wall + q["at"] - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                tickets[i] = srv.submit(q["table"], q["r0"], q["r1"], q["group_cols"], q["aggs"],
                                        filters=q["filters"], est_groups=q["est_groups"])
                ready.release()
        except Exception as e:  # surfaced below
            errors.append(e)
            ready.release()

    th = threading.Thread(target=submitter)
    th.start()
    for i in range(len(queries)):
        ready.acquire()
        if errors:
            break
        srv.wait(tickets[i])
        on_done(i, tickets[i])
    th.join()
    if errors:
        raise errors[0]


def results_mismatch(rb, ra, nk):
    """None when two results of one query (lists of (values, valid), keys
    first) hold the same groups with equal integers and DOUBLE values within
    REL_TOL_F64 of each other; else the first difference."""
    ref = {"n_groups": len(ra[0][0]), "keys": [ra[j][0] for j in range(nk)],
           "key_null": [~np.asarray(ra[j][1], bool) for j in range(nk)],
           "aggs": [(v, ~np.asarray(m, bool), v) for v, m in ra[nk:]]}
    return oracle_mismatch(rb, ref, nk)


def run_serve(args):
    """The served query stream: 10 resident tables (~66 GB at --scale 1),
    Poisson arrivals at --rate q/s for --duration s, each query one of the
    four GROUP BY shapes over a random row range with WHERE selectivity
    U[1%, 100%]; admission budget --budget-gb of estimated device bytes.
    Runs the same stream with continuous batching and one query at a time."""
    ws, rank, local = dist_env()
    if args.impl == "reference":  # host cores only; rank 0 alone under torchrun
        return run_serve_reference(args) if rank == 0 else None
    import torch
    torch.cuda.set_device(local)
    from slothdb_gb300 import capi, datagen
    capi.load(build_if_missing=True)
    t0 = time.time()
    tabs, rows_of, res_bytes = [], {}, 0
    for i, t in enumerate(datagen.SERVE_TABLES):
        cols, n = datagen.serve_table_device(t, scale=args.scale)
        tabs.append((datagen.SERVE_TYPES[t["family"]], cols, n))
        rows_of[i] = n
        for c in cols:
            res_bytes += (c[0].numel() * 8 + c[1].numel()) if isinstance(c, tuple) else c.numel() * c.element_size()
    torch.cuda.synchronize()
    gen_s = time.time() - t0
    queries = datagen.serve_queries(args.duration, args.rate, rows_of, seed=4)
    scanned = 0
    for q in queries:
        types, cols, _ = tabs[q["table"]]
        for c, ty in zip(cols, types):
            if ty == capi.VARCHAR:  # offsets + string bytes of the range
                scanned += (q["r1"] - q["r0"]) * 8 + int((c[0][q["r1"]] - c[0][q["r0"]]).item())
            else:
                scanned += (q["r1"] - q["r0"]) * c.element_size()
    out = {}
    results = {}
    sample = list(range(0, len(queries), max(1, len(queries) // 24)))
    for mode, name in [(0, "batched"), (1, "one_at_a_time")]:
        srv = capi.Server(budget_bytes=int(args.budget_gb * (1 << 30)), max_batch=256, mode=mode,
                          lanes=args.lanes if mode == 0 else 1)
        for types, cols, n in tabs:
            srv.add_table(types, cols, n)
        # warm-up: a few queries of every shape
        warm = [q for q in queries[:64]]
        for q in warm[:16]:
            t = srv.submit(q["table"], q["r0"], q["r1"], q["group_cols"], q["aggs"], filters=q["filters"],
                           est_groups=q["est_groups"])
            srv.wait(t)
            srv.release(t)
        st0 = srv.stats()
        lat = []
        exec_by_shape = {}

        def on_done(i, t):
            qm, em, bs = srv.times(t)
            lat.append(qm + em)
            if mode == 1:
                exec_by_shape.setdefault(queries[i]["shape"], []).append((em, queries[i]["r1"] - queries[i]["r0"]))
            if i in sample:
                results.setdefault(i, []).append(srv.result(t))
            srv.release(t)

        clocks = Clocks(local)
        clocks.start()
        w0 = time.perf_counter()
        _serve_stream(srv, queries, w0, on_done)
        w1 = time.perf_counter()
        clk = clocks.stop()
        st = srv.stats()
        lat = np.array(lat)
        out[name] = {"queries_per_s": len(queries) / (w1 - w0), "wall_s": w1 - w0,
                     "p50_ms": float(np.percentile(lat, 50)), "p95_ms": float(np.percentile(lat, 95)),
                     "p99_ms": float(np.percentile(lat, 99)), "mean_ms": float(lat.mean()),
                     "batches": st["batches"] - st0["batches"], "busy_ms": st["busy_ms"] - st0["busy_ms"],
                     "rejected": st["rejected"], "failed": st["failed"],
                     "peak_admitted_GB": st["peak_admitted_bytes"] / 2**30,
                     "kernel_launches": st["kernel_launches"] - st0["kernel_launches"],
                     "result_bytes": st["result_bytes"] - st0["result_bytes"], "clocks": clk}
        # capacity: the first --capacity-queries queries of the stream, all
        # submitted at once (the server saturated; latency is queueing here)
        capq = [dict(q, at=0.0) for q in queries[:args.capacity_queries]]
        if capq:
            c_st0 = srv.stats()
            c0 = time.perf_counter()
            _serve_stream(srv, capq, c0, lambda i, t: srv.release(t))
            c1 = time.perf_counter()
            c_st = srv.stats()
            out[name]["capacity"] = {"queries": len(capq), "wall_s": c1 - c0, "queries_per_s": len(capq) / (c1 - c0),
                                     "busy_ms": c_st["busy_ms"] - c_st0["busy_ms"],
                                     "batches": c_st["batches"] - c_st0["batches"]}
        if mode == 1:
            out[name]["per_shape"] = {
                str(k): {"queries": len(v), "mean_exec_ms": float(np.mean([e for e, _ in v])),
                         "rows_per_s": float(sum(r for _, r in v) / max(1e-9, sum(e for e, _ in v) / 1e3))}
                for k, v in sorted(exec_by_shape.items())}
        srv.close()
    # per-result identity, mixed (batched) vs alone: integer columns
    # bit-exact, DOUBLE columns within 1e-12 relative (their sums are
    # accumulated in a different order on each run)
    same, why = 0, []
    for i, (rb, ra) in results.items():
        d = results_mismatch(rb, ra, len(queries[i]["group_cols"]))
        if d:
            why.append("q%d shape %d: %s" % (i, queries[i]["shape"], d))
        same += d is None
    # oracle parity of the sampled queries (their row ranges copied to the
    # host); the same oracle pass, all host threads per query, is the timed
    # CPU baseline on that sample of the mix
    import oracle
    thr = os.cpu_count() or 1
    orc_diffs, orc_s, orc_rows = [], 0.0, 0
    for i in sorted(results):
        q = queries[i]
        types, cols, _ = tabs[q["table"]]
        hc = []
        for c in cols:
            if isinstance(c, tuple):
                o = c[0][q["r0"]:q["r1"] + 1].cpu().numpy()
                hc.append((o - o[0], c[1][int(o[0]):int(o[-1])].cpu().numpy()))
            else:
                hc.append(c[q["r0"]:q["r1"]].cpu().numpy())
        tc = time.perf_counter()
        orc = oracle.run_query(types, q["group_cols"], q["aggs"], hc, filters=q["filters"], nthreads=thr)
        orc_s += time.perf_counter() - tc
        orc_rows += q["r1"] - q["r0"]
        d = oracle_mismatch(results[i][0], orc, len(q["group_cols"]))
        if d:
            orc_diffs.append("q%d shape %d: %s" % (i, q["shape"], d))
    smp = ServeCpuSample(args)
    cpu = smp.baseline(smp.seconds())
    cpu["sampled_all_threads"] = {"value": len(results) / orc_s, "threads": thr,
                                  "sample": "the %d parity-sampled queries (%d rows), %d threads each"
                                            % (len(results), orc_rows, thr)}
    hbm_peak, peak_src = hbm_peak_gbs()
    b = out["batched"]
    busy_s = max(1e-9, b["busy_ms"] / 1e3)
    roofline = {"bound": "hbm", "achieved": scanned / busy_s / 1e9, "peak": hbm_peak, "unit": "GB/s",
                "frac": scanned / busy_s / 1e9 / hbm_peak, "traffic": None,
                "kernel": "every kernel of the served batches (dispatcher busy time)", "kernel_ms": b["busy_ms"],
                "algorithmic_bytes": scanned, "peak_source": peak_src}
    line = {"metric": "served GROUP BY queries/s and latency percentiles (Poisson stream, admission budget)",
            "value": b["queries_per_s"], "unit": "queries/s", "n_gpus": 1, "steps": 1, "warmup": 16,
            "ms_per_step": b["wall_s"] * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int64+f64", "data": "synthetic",
            "config": {"workload": "serve-10-tables", "resident_GB": res_bytes / 1e9, "scale": args.scale,
                       "queries": len(queries), "rate_qps": args.rate, "duration_s": args.duration,
                       "budget_GB": args.budget_gb, "scanned_GB": scanned / 1e9, "lanes": args.lanes,
                       "shapes": "1M plain / 100M zipf / 200M filtered / 1e4-1e7 composite|varchar",
                       "datagen_s": round(gen_s, 1)},
            "p50_ms": b["p50_ms"], "p95_ms": b["p95_ms"], "p99_ms": b["p99_ms"],
            "batched": b, "one_at_a_time": out["one_at_a_time"],
            "speedup_vs_one_at_a_time": out["one_at_a_time"]["wall_s"] / b["wall_s"],
            "capacity_speedup_vs_one_at_a_time": (b["capacity"]["queries_per_s"] /
                                                  out["one_at_a_time"]["capacity"]["queries_per_s"])
            if "capacity" in b else None,
            "identity_alone_vs_mixed": "%d/%d sampled results identical (integers bit-exact, DOUBLE within "
                                        "1e-12 relative)" % (same, len(results)),
            "identity_mismatches": why[:6],
            "parity": {"oracle_mismatches": len(orc_diffs), "sampled": len(results), "first": orc_diffs[:4]},
            "roofline": roofline, "cpu_baseline": cpu,
            "e2e": {"value": b["queries_per_s"], "unit": "queries/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": b["result_bytes"],
                    "note": "the served loop is the public API end to end: every result is copied to pinned "
                            "host memory before its query completes; the tables are resident in HBM by the "
                            "workload's definition (no per-query input copy)"},
            "gpu_launches": b["kernel_launches"], "clocks": b["clocks"]}
    print(json.dumps(line), flush=True)


class ServeCpuSample:
    """The served stream's CPU baseline: the oracle (restatement of the
    reference's GROUP BY) on a sample of the query mix, the first queries of
    the stream whose row ranges sum to about 30M rows, over host-generated
    columns of the same families, one query after another on one thread
    (the full stream is infeasible on the CPU)."""

    def __init__(self, args):
        from slothdb_gb300 import datagen
        rows_of = {i: int(t["rows"] * args.scale) for i, t in enumerate(datagen.SERVE_TABLES)}
        queries = datagen.serve_queries(args.duration, args.rate, rows_of, seed=4)
        self.picked, self.rows = [], 0
        for q in queries:
            n = q["r1"] - q["r0"]
            if self.rows + n > 30_000_000:
                continue
            self.picked.append(q)
            self.rows += n
        rng = np.random.default_rng(5)

        def host_cols(q):
            n = q["r1"] - q["r0"]
            fam = datagen.SERVE_TABLES[q["table"]]["family"]
            g = datagen.SERVE_TABLES[q["table"]]["groups"]
            if fam == "plain":
                return [rng.integers(0, g, n, dtype=np.int32), rng.integers(0, 10**6, n, dtype=np.int64)]
            if fam == "zipf":
                return [rng.integers(0, 2**40, n, dtype=np.int64), rng.normal(100, 25, n)]
            if fam == "filter":
                return [rng.integers(0, g, n, dtype=np.int32), rng.integers(0, 1000, n, dtype=np.int16),
                        rng.integers(-10**9, 10**9, n, dtype=np.int64)]
            return datagen.batch_table_host(dict(kind=fam, rows=n, groups=g, seed=int(rng.integers(1 << 30))))

        self.data = [host_cols(q) for q in self.picked]

    def seconds(self):
        import oracle
        from slothdb_gb300 import datagen
        t = time.perf_counter()
        for q, cols in zip(self.picked, self.data):
            types = datagen.SERVE_TYPES[datagen.SERVE_TABLES[q["table"]]["family"]]
            oracle.run_query(types, q["group_cols"], q["aggs"], cols, filters=q["filters"],
                             nthreads=ref_threads("memory"))
        return time.perf_counter() - t

    def baseline(self, per):
        return {"value": len(self.picked) / per, "unit": "queries/s", "cores": ref_threads("memory"),
                "kind": "port", "sample": "first %d queries of the stream (%d rows), sequential, 1 thread" % (
                    len(self.picked), self.rows)}


def run_serve_reference(args):
    """The served stream's CPU baseline (ServeCpuSample) timed per step."""
    smp = ServeCpuSample(args)
    picked, tot = smp.picked, smp.rows
    times = []
    for i in range(args.warmup + max(1, args.steps)):
        dt = smp.seconds()
        if i >= args.warmup:
            times.append(dt)
    per = statistics.mean(times)
    val = len(picked) / per
    line = {"impl": "reference", "metric": "served GROUP BY queries/s and latency percentiles (Poisson stream, "
            "admission budget)", "value": val, "unit": "queries/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": per * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int64+f64", "data": "synthetic",
            "config": {"workload": "serve-10-tables (bounded sample: %d queries, %d rows)" % (len(picked), tot)},
            "cpu_baseline": smp.baseline(per),
            "e2e": {"value": val, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_parquet(args):
    """Fused Parquet decode + filter + GROUP BY: an uncompressed file of
    --pq-rows rows in 1M-row row groups (key INT32 dictionary of 65,536
    values, RLE/bit-packed indices at bit width 16 with runs of mean 4;
    f INT16 PLAIN; v INT64 PLAIN), SELECT key, SUM(v), COUNT(*) WHERE
    f < 100 GROUP BY key.  value = rows/s with the file resident in HBM;
    e2e = rows/s from the file in pinned host memory (row groups copied to
    HBM inside the call)."""
    ws, rank, local = dist_env()
    from slothdb_gb300 import parquet as pq
    if args.impl == "reference" and rank != 0:
        return  # rank 0 alone runs the reference arm
    rows = args.pq_rows
    codec = {"parquet200m_snappy": "snappy", "parquet200m_zstd": "zstd"}.get(args.workload)
    snappy = codec is not None  # compressed pages: decompressed on the GPU per batch
    inflate = "k_pq_unzstd" if codec == "zstd" else "k_pq_inflate"
    cname = {None: "UNCOMPRESSED", "snappy": "SNAPPY", "zstd": "ZSTD"}[codec]
    t0 = time.time()
    data, key, f, v = pq.filter_groupby_file(n_rows=rows, row_group_rows=1_000_000,
                                             codec=codec)
    raw_bytes = len(pq.filter_groupby_file(n_rows=rows, row_group_rows=1_000_000)[0]) if snappy else len(data)
    gen_s = time.time() - t0
    if args.impl == "reference":
        return run_parquet_reference(args, key, f, v, rows)
    import torch
    torch.cuda.set_device(local)
    from slothdb_gb300 import capi
    capi.load(build_if_missing=True)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    file_bytes = len(data)
    types = [capi.INTEGER, capi.SMALLINT, capi.BIGINT]
    aggs = [("sum", 2), ("count_star", -1)]
    filters = [(1, "<", 100)]
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    pf = capi.ParquetFile(data)
    pf.upload(stream=sp)
    g = capi.GroupBy(types, [0], aggs, filters=filters, est_groups=65_536)

    def step(device=True, gg=g, ff=pf):
        gg.reset()
        capi.ingest_parquet(gg, ff, [0, 1, 2], device=device, stream=sp)
        gg.finalize(stream=sp)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    # parity at full size against the oracle on the decoded columns
    import oracle
    orc = oracle.run_query(types, [0], aggs, [key, f.astype(np.int16), v], filters=filters,
                           nthreads=os.cpu_count() or 1)
    res = g.result()
    got = dict(zip(res[0][0].tolist(), zip(res[1][0].tolist(), res[2][0].tolist())))
    ok = len(got) == len(orc["keys"][0]) and all(
        got.get(int(k_)) == (int(s_), int(c_)) for k_, s_, c_ in zip(orc["keys"][0], orc["aggs"][0][0],
                                                                     orc["aggs"][1][0]))
    g.set_profiling(True)
    step()
    prof = {k: vv[1] / max(1, vv[0]) for k, vv in g.profile().items()}
    g.set_profiling(False)
    clocks = Clocks(local)
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    launches = 0
    for _ in range(args.steps):
        step()
        launches += g.launches()
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    scan_ms = prof.get("k_pq_scan", float("nan"))
    # the scan reads the (decompressed) page bytes; the inflate reads the
    # compressed pages and writes the decompressed image
    achieved = raw_bytes / (scan_ms / 1e3) / 1e9
    if snappy:
        inf_ms = prof.get(inflate, float("nan"))
        if inf_ms > scan_ms:
            scan_ms = inf_ms
            achieved = (file_bytes + raw_bytes) / (inf_ms / 1e3) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                "traffic": None, "kernel": (inflate if snappy and scan_ms == prof.get(inflate)
                                            else "k_pq_scan"), "kernel_ms": scan_ms,
                "peak_source": "measured" if "hbm_gbs" in peaks else "fallback",
                "step_GBps": file_bytes / (ms / 1e3) / 1e9, "step_frac": file_bytes / (ms / 1e3) / 1e9 / hbm_peak,
                "kernels_ms": prof}
    # e2e: the file in pinned host memory
    pin = capi.PinnedBuffer(file_bytes)
    pin.view(np.uint8)[:] = np.frombuffer(data, dtype=np.uint8)
    pfh = capi.ParquetFile(pin.view(np.uint8))
    ge = capi.GroupBy(types, [0], aggs, filters=filters, est_groups=65_536)
    for _ in range(2):
        step(device=False, gg=ge, ff=pfh)
    torch.cuda.synchronize()
    tt = time.perf_counter()
    ne = max(1, args.steps // 2)
    d2h = 0
    for _ in range(ne):
        step(device=False, gg=ge, ff=pfh)
        d2h = ge.result_host_bytes()[1]
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - tt) / ne
    ge.close()
    pfh.close()
    pin.close()
    cpu = None
    if rank == 0:
        n = min(args.cpu_sample, rows)
        thr = ref_threads("parquet")
        tc = time.perf_counter()
        oracle.run_query(types, [0], aggs, [key[:n], f[:n].astype(np.int16), v[:n]], filters=filters, nthreads=thr)
        dt = time.perf_counter() - tc
        cpu = {"value": n / dt, "unit": "rows/s", "cores": thr, "kind": "port",
               "sample": "first %d decoded rows, filter + GROUP BY (no page decode), %d threads" % (n, thr)}
    line = {"metric": "fused Parquet decode+filter+GROUP BY rows/s (200M rows, 1M-row RGs%s)" % (
                ", " + cname if snappy else ""),
            "value": rows / (ms / 1e3), "unit": "rows/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int32+int64", "data": "synthetic",
            "config": {"workload": "parquet-filter-groupby-%dM%s" % (rows // 1_000_000, "-" + codec if snappy else ""),
                       "rows": rows, "file_bytes": file_bytes, "page_bytes_uncompressed": raw_bytes,
                       "codec": cname, "row_group_rows": 1_000_000, "dict": 65_536,
                       "predicate": "f < 100", "l2": "file %.1f GB > L2 129 MB (no flush needed)" % (file_bytes / 1e9),
                       "datagen_s": round(gen_s, 1)},
            "parity": "bit-exact vs oracle" if ok else "MISMATCH vs oracle",
            "roofline": roofline, "cpu_baseline": cpu,
            "e2e": {"value": rows / e2e_s, "unit": "rows/s", "h2d_bytes_per_step": file_bytes,
                    "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s * 1e3},
            "clocks": clk, "gpu_launches": launches}
    print(json.dumps(line), flush=True)
    g.close()
    pf.close()


def run_parquet_reference(args, key, f, v, rows):
    """The oracle's filter + GROUP BY over the decoded columns of a bounded
    sample (page decode not included), on the reference's Parquet thread
    count."""
    import oracle
    n = min(args.cpu_sample, rows)
    thr = ref_threads("parquet")
    types = [2, 1, 3]
    times = []
    for i in range(args.warmup + args.steps):
        t = time.perf_counter()
        oracle.run_query(types, [0], [("sum", 2), ("count_star", -1)], [key[:n], f[:n].astype(np.int16), v[:n]],
                         filters=[(1, "<", 100)], nthreads=thr)
        if i >= args.warmup:
            times.append(time.perf_counter() - t)
    per = statistics.mean(times)
    val = n / per
    line = {"impl": "reference", "metric": "fused Parquet decode+filter+GROUP BY rows/s (200M rows, 1M-row RGs%s)" % (
                {"parquet200m_snappy": ", SNAPPY", "parquet200m_zstd": ", ZSTD"}.get(args.workload, "")),
            "value": val, "unit": "rows/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": per * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int32+int64", "data": "synthetic",
            "config": {"workload": "parquet-filter-groupby (bounded sample of %d decoded rows)" % n},
            "cpu_baseline": {"value": val, "unit": "rows/s", "cores": thr, "kind": "port",
                             "sample": "first %d decoded rows per step" % n},
            "e2e": {"value": val, "unit": "rows/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def dictsum_cpu(dictionary, idx, rg_rows, rows):
    """The dictionary histogram on the host (the reference's
    DecodeBigintColumnHistogram per row group, on already-decoded indices:
    no RLE decode), over the first `rows` rows; returns (count, sum, s)."""
    t = time.perf_counter()
    cnt, tot = 0, 0.0
    for r0 in range(0, rows, rg_rows):
        h = np.bincount(idx[r0:min(rows, r0 + rg_rows)], minlength=len(dictionary))
        cnt += int(h.sum())
        tot += float(np.dot(h.astype(np.float64), dictionary.astype(np.float64)))
    return cnt, tot, time.perf_counter() - t


def run_dictsum(args):
    """Ungrouped SUM/COUNT of an INT64 dictionary column through the
    dictionary histogram (gb_pq_dict_sum): --pq-rows rows in 1M-row row
    groups, 65,536 dictionary values, RLE/bit-packed indices (bit width 16,
    runs of mean 4).  value = rows/s with the file resident in HBM (the
    public call: index run tables, histogram, reduce, result to the host);
    e2e = rows/s from the file in host memory (the column's bytes copied
    inside the call)."""
    ws, rank, local = dist_env()
    from slothdb_gb300 import parquet as pq
    if rank != 0:
        return
    rows = args.pq_rows
    t0 = time.time()
    data, dictionary, idx = pq.dict_int64_file(n_rows=rows, row_group_rows=1_000_000)
    gen_s = time.time() - t0
    thr = ref_threads("parquet")
    n_cpu = min(args.cpu_sample, rows)
    metric = "ungrouped SUM/COUNT rows/s of an INT64 dictionary column (dictionary histogram, 200M rows)"
    if args.impl == "reference":
        times = []
        for i in range(args.warmup + args.steps):
            _, _, dt = dictsum_cpu(dictionary, idx, 1_000_000, n_cpu)
            if i >= args.warmup:
                times.append(dt)
        per = statistics.mean(times)
        val = n_cpu / per
        print(json.dumps({"impl": "reference", "metric": metric, "value": val, "unit": "rows/s", "n_gpus": 1,
                          "steps": args.steps, "warmup": args.warmup, "ms_per_step": per * 1e3,
                          "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int64",
                          "data": "synthetic", "config": {"workload": "dictsum-%dM (bounded sample of %d rows)" % (
                              rows // 1_000_000, n_cpu)},
                          "cpu_baseline": {"value": val, "unit": "rows/s", "cores": 1, "kind": "port",
                                           "sample": "first %d rows: per-row-group histogram of the decoded "
                                                     "indices + dot product, 1 thread" % n_cpu},
                          "e2e": {"value": val, "unit": "rows/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}),
              flush=True)
        return
    import torch
    torch.cuda.set_device(local)
    from slothdb_gb300 import capi
    capi.load(build_if_missing=True)
    hbm_peak, peak_src = hbm_peak_gbs()
    pf = capi.ParquetFile(data)
    pf.upload()
    exact = int((np.bincount(idx, minlength=len(dictionary)).astype(object) * dictionary.astype(object)).sum())
    for _ in range(args.warmup):
        got = pf.dict_sum(0, device=True)
    parity = {"count_equal": got[0] == rows, "sum_rel_err": abs(got[1] - exact) / max(1.0, abs(exact)),
              "tol_f64": REL_TOL_F64}
    clocks = Clocks(local)
    clocks.start()
    t = time.perf_counter()
    for _ in range(args.steps):
        pf.dict_sum(0, device=True)
    ms = (time.perf_counter() - t) / args.steps * 1e3
    clk = clocks.stop()
    # the dominant kernel on its own (CUDA events around one call's work:
    # the histogram and its reduce dominate; the run walk is the rest)
    st = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(st)
    pf.dict_sum(0, device=True, stream=st.cuda_stream)
    e1.record(st)
    torch.cuda.synchronize()
    call_ms = e0.elapsed_time(e1)
    te = time.perf_counter()
    ne = max(1, args.steps // 2)
    for _ in range(ne):
        pf.dict_sum(0, device=False)
    e2e_s = (time.perf_counter() - te) / ne
    pf.close()
    _, _, cpu_s = dictsum_cpu(dictionary, idx, 1_000_000, n_cpu)
    file_bytes = len(data)
    achieved = file_bytes / (call_ms / 1e3) / 1e9
    print(json.dumps({"metric": metric, "value": rows / (ms / 1e3), "unit": "rows/s", "n_gpus": 1,
                      "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
                      "scaling": "weak", "vs_baseline": None, "dtype": "int64", "data": "synthetic",
                      "config": {"workload": "dictsum-%dM" % (rows // 1_000_000), "rows": rows,
                                 "file_bytes": file_bytes, "row_group_rows": 1_000_000, "dict": len(dictionary),
                                 "l2": "file %.1f GB > L2 129 MB (no flush needed)" % (file_bytes / 1e9),
                                 "datagen_s": round(gen_s, 1)},
                      "parity": parity,
                      "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                                   "frac": achieved / hbm_peak, "traffic": None,
                                   "kernel": "one gb_pq_dict_sum call (k_pq_runs + k_pq_dict_hist + k_pq_dict_reduce)",
                                   "kernel_ms": call_ms, "peak_source": peak_src,
                                   "note": "algorithmic bytes = the column chunks' bytes (index pages + dictionaries)"},
                      "cpu_baseline": {"value": n_cpu / cpu_s, "unit": "rows/s", "cores": 1, "kind": "port",
                                       "sample": "first %d rows: per-row-group histogram of the decoded indices + "
                                                 "dot product, 1 thread" % n_cpu},
                      "e2e": {"value": rows / e2e_s, "unit": "rows/s", "h2d_bytes_per_step": file_bytes,
                              "d2h_bytes_per_step": 16, "ms_per_step": e2e_s * 1e3},
                      "clocks": clk, "gpu_launches": 3 * args.steps}), flush=True)


DISTINCT_GROUPS, DISTINCT_VALUES = 100_000, 2000


def distinct_data(rows):
    """k INT32 uniform over 100,000 groups, v INT32 uniform over 2,000
    values (seed 5): ~787 distinct values per group, ~79M distinct pairs."""
    rng = np.random.default_rng(5)
    k = rng.integers(0, DISTINCT_GROUPS, rows, dtype=np.int32)
    v = rng.integers(0, DISTINCT_VALUES, rows, dtype=np.int32)
    return k, v


def run_distinct(args):
    """SELECT k, COUNT(DISTINCT v), COUNT(*) FROM t GROUP BY k over --rows
    rows (hash GROUP BY + (group, value) pair sets in HBM).  value = rows/s
    with the columns resident in HBM; parity at full size against exact
    per-group value sets built with numpy."""
    ws, rank, local = dist_env()
    rows = args.rows
    t0 = time.time()
    k, v = distinct_data(rows)
    gen_s = time.time() - t0
    types = [2, 2]
    aggs = [("count_distinct", 1), ("count_star", -1)]
    if args.impl == "reference":  # host cores only; rank 0 alone under torchrun
        return run_distinct_reference(args, k, v, types, aggs) if rank == 0 else None
    import torch
    torch.cuda.set_device(local)
    from slothdb_gb300 import capi
    capi.load(build_if_missing=True)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    dk = torch.from_numpy(k).cuda()
    dv = torch.from_numpy(v).cuda()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    g = capi.GroupBy(types, [0], aggs, est_groups=DISTINCT_GROUPS)

    def step():
        g.reset()
        g.ingest([dk, dv], nrows=rows, device=True, stream=sp)
        g.finalize(stream=sp)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    # parity at full size: exact per-group distinct counts from a bitmap of
    # the (group, value) pairs
    res = g.result()
    seen = np.bincount(k.astype(np.int64) * DISTINCT_VALUES + v, minlength=DISTINCT_GROUPS * DISTINCT_VALUES)
    exp_d = (seen.reshape(DISTINCT_GROUPS, DISTINCT_VALUES) > 0).sum(axis=1)
    exp_c = np.bincount(k, minlength=DISTINCT_GROUPS)
    del seen
    o = np.argsort(res[0][0])
    gk = res[0][0][o].astype(np.int64)
    ok = (np.array_equal(gk, np.nonzero(exp_c)[0]) and np.array_equal(res[1][0][o], exp_d[gk])
          and np.array_equal(res[2][0][o], exp_c[gk]))
    g.set_profiling(True)
    step()
    prof = {kk: vv[1] / max(1, vv[0]) for kk, vv in g.profile().items()}
    g.set_profiling(False)
    clocks = Clocks(local)
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    launches = 0
    for _ in range(args.steps):
        step()
        launches += g.launches()
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    in_bytes = rows * 8
    ing_ms = prof.get("k_ingest", float("nan"))
    achieved = in_bytes / (ing_ms / 1e3) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                "traffic": None, "kernel": "k_ingest", "kernel_ms": ing_ms,
                "peak_source": "measured" if "hbm_gbs" in peaks else "fallback", "kernels_ms": prof}
    e2e = None
    if not args.no_e2e:
        pk = capi.PinnedBuffer(rows * 4)
        pv = capi.PinnedBuffer(rows * 4)
        pk.view(np.int32)[:] = k
        pv.view(np.int32)[:] = v
        ge = capi.GroupBy(types, [0], aggs, est_groups=DISTINCT_GROUPS)
        d2h = 0

        def step_e2e():
            ge.reset()
            ge.ingest([pk.ptr, pv.ptr], nrows=rows, stream=sp)
            ge.finalize(stream=sp)
            return ge.result_host_bytes()[1]

        for _ in range(2):
            d2h = step_e2e()
        torch.cuda.synchronize()
        tt = time.perf_counter()
        ne = max(1, args.steps // 2)
        for _ in range(ne):
            d2h = step_e2e()
        torch.cuda.synchronize()
        e2e_s = (time.perf_counter() - tt) / ne
        e2e = {"value": rows / e2e_s, "unit": "rows/s", "h2d_bytes_per_step": in_bytes, "d2h_bytes_per_step": d2h,
               "ms_per_step": e2e_s * 1e3}
        ge.close()
        pk.close()
        pv.close()
    cpu = None
    if rank == 0:
        import oracle
        n = min(args.cpu_sample, rows)
        thr = ref_threads("memory")
        tc = time.perf_counter()
        oracle.run_query(types, [0], aggs, [k[:n], v[:n]], nthreads=thr)
        dt = time.perf_counter() - tc
        cpu = {"value": n / dt, "unit": "rows/s", "cores": thr, "kind": "port",
               "sample": "first %d rows, %d thread (%.2f s)" % (n, thr, dt)}
    line = {"metric": "COUNT(DISTINCT) GROUP BY rows/s (100M rows, 100K groups)", "value": rows / (ms / 1e3),
            "unit": "rows/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
            "config": {"workload": "count-distinct-groupby-%dM" % (rows // 1_000_000), "rows": rows,
                       "groups": DISTINCT_GROUPS, "values": DISTINCT_VALUES, "distinct_pairs": int(exp_d.sum()),
                       "aggs": "COUNT(DISTINCT v),COUNT(*)",
                       "l2": "inputs %.1f GB + pair sets > L2 129 MB (no flush needed)" % (in_bytes / 1e9),
                       "datagen_s": round(gen_s, 1)},
            "parity": "bit-exact vs exact value sets" if ok else "MISMATCH vs exact value sets",
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk, "gpu_launches": launches}
    print(json.dumps(line), flush=True)
    g.close()


def run_distinct_reference(args, k, v, types, aggs):
    """The oracle's per-group value sets over a bounded sample, on the
    reference's in-memory thread count."""
    import oracle
    n = min(args.cpu_sample, len(k))
    thr = ref_threads("memory")
    times = []
    for i in range(args.warmup + args.steps):
        t = time.perf_counter()
        oracle.run_query(types, [0], aggs, [k[:n], v[:n]], nthreads=thr)
        if i >= args.warmup:
            times.append(time.perf_counter() - t)
    per = statistics.mean(times)
    val = n / per
    line = {"impl": "reference", "metric": "COUNT(DISTINCT) GROUP BY rows/s (100M rows, 100K groups)",
            "value": val, "unit": "rows/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": per * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int32", "data": "synthetic",
            "config": {"workload": "count-distinct-groupby (bounded sample of %d rows)" % n},
            "cpu_baseline": {"value": val, "unit": "rows/s", "cores": thr, "kind": "port",
                             "sample": "first %d rows per step" % n},
            "e2e": {"value": val, "unit": "rows/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.workload == "distinct100m":
        run_distinct(args)
        return
    if args.workload == "plain1m":
        run_plain(args)
        return
    if args.workload == "batch256":
        run_batch(args)
        return
    if args.workload == "serve":
        run_serve(args)
        return
    if args.workload in ("parquet200m", "parquet200m_snappy", "parquet200m_zstd"):
        run_parquet(args)
        return
    if args.workload == "dictsum200m":
        run_dictsum(args)
        return
    if args.impl == "reference":
        run_reference(args)
        return
    ws, rank, local = dist_env()
    import torch
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from slothdb_gb300 import capi
    capi.load(build_if_missing=True)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"

    rows = args.rows
    k, x, gen_s = gen_data(rows)
    dk = torch.from_numpy(k).cuda()
    dx = torch.from_numpy(x).cuda()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    aggs = [("count_star", -1), ("sum", 1), ("avg", 1)]
    g = capi.GroupBy([capi.BIGINT, capi.DOUBLE], [0], aggs, est_groups=EST_GROUPS)
    g.set_topn(1, False, 10)

    def step_device():
        g.reset()
        g.ingest([dk, dx], nrows=rows, device=True, stream=sp)
        g.finalize(stream=sp)

    for _ in range(args.warmup):
        step_device()
    torch.cuda.synchronize()
    # one profiled pass for per-kernel device times (CUDA events on `sp`)
    g.set_profiling(True)
    step_device()
    prof = g.profile()
    g.set_profiling(False)
    launches_before = g.launches()

    clocks = Clocks(local)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    launches = 0
    for _ in range(args.steps):
        step_device()
        launches += g.launches()
    ev1.record(stream)
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    ms = max_over_ranks(ev0.elapsed_time(ev1) / args.steps)
    # full result size: run once without TopN to count groups
    g2 = capi.GroupBy([capi.BIGINT, capi.DOUBLE], [0], aggs, est_groups=EST_GROUPS)
    g2.ingest([dk, dx], nrows=rows, device=True, stream=sp)
    g2.finalize(stream=sp)
    full = g2.result()  # the full GROUP BY result in host memory (parity leg below)
    n_groups = len(full[0][0])
    g2.close()
    top = g.result()  # the TopN of the last timed step

    in_bytes = rows * 16
    out_bytes = n_groups * 32
    alg_bytes = in_bytes + out_bytes
    value = whole_job_rate(rows, ws, ms)

    # roofline: dominant kernel = the row pass (k_partition in radix mode,
    # k_ingest in hash mode); algorithmic bytes = the key + value columns
    # (16 B/row) it reads once
    dom = "k_partition" if "k_partition" in prof else "k_ingest"
    ing = prof.get(dom, (1, float("nan")))
    ing_ms = ing[1] / max(1, ing[0])
    achieved = in_bytes / (ing_ms / 1e3) / 1e9
    # DRAM traffic per row of k_partition from the committed ncu capture
    # (30M-row case, read + write = 617.1 MB), scaled to this launch's rows
    traffic = TRAFFIC_PER_ROW.get(dom)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak, "traffic": traffic * rows if traffic else None,
                "kernel": dom, "kernel_ms": ing_ms,
                "peak_source": peak_src,
                "step_GBps": alg_bytes / (ms / 1e3) / 1e9,
                "step_frac": alg_bytes / (ms / 1e3) / 1e9 / hbm_peak,
                "kernels_ms": {kname: v[1] / max(1, v[0]) for kname, v in prof.items()}}

    # e2e through the C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        pk = capi.PinnedBuffer(rows * 8)
        px = capi.PinnedBuffer(rows * 8)
        pk.view(np.int64)[:] = k
        px.view(np.float64)[:] = x
        ge = capi.GroupBy([capi.BIGINT, capi.DOUBLE], [0], aggs, est_groups=EST_GROUPS)
        d2h = 0

        def step_e2e():
            ge.reset()
            ge.ingest([pk.ptr, px.ptr], nrows=rows, stream=sp)  # host (pinned) pointers
            ge.finalize(stream=sp)
            return ge.result_host_bytes()[1]  # gb_agg_result: full result into host memory

        for _ in range(2):
            d2h = step_e2e()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(max(1, args.steps // 2)):
            d2h = step_e2e()
        torch.cuda.synchronize()
        e2e_s = (time.perf_counter() - t0) / max(1, args.steps // 2)
        e2e = {"value": rows * ws / e2e_s, "unit": "rows/s", "h2d_bytes_per_step": in_bytes,
               "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s * 1e3}
        ge.close()
        pk.close()
        px.close()

    cpu = None
    parity = None
    if rank == 0:
        # full-size parity (oracle over the same 100M rows, outside the timed
        # region); the same oracle pass is the timed CPU baseline
        parity, orc_s = parity_zipf(k, x, full, top)
        _, cpu = zipf_cpu_sample(args, k, x)
        cpu["all_threads"] = {"value": rows / orc_s, "threads": parity["oracle"]["threads"],
                              "sample": "all %d rows (the parity pass)" % rows}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "rows/s", "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "int64+f64", "data": "synthetic",
                "config": {"workload": "zipf-groupby-100M", "rows": rows, "distinct_values": N_VALUES,
                           "observed_groups": n_groups, "key": "INT64 Zipf(1.1)", "aggs": "COUNT(*),SUM(x),AVG(x)",
                           "topn": "ORDER BY COUNT(*) DESC LIMIT 10 (+ full result in HBM)",
                           "l2": "inputs 1.6 GB > L2 129 MB (no flush needed)",
                           "parallelism": "replicas" if ws > 1 else "single",
                           "est_groups_hint": EST_GROUPS, "datagen_s": round(gen_s, 1)},
                "algorithmic_bytes_per_step": alg_bytes,
                "roofline": roofline, "cpu_baseline": cpu, "parity": parity, "e2e": e2e, "clocks": clk,
                "gpu_launches": launches}
        print(json.dumps(line), flush=True)
    g.close()
    if ws > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
