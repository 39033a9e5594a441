"""Autotuner for the GROUP BY operator's execution options.

The reference fixes its execution knobs in code (thread counts such as
RADIX_COUNT_THREADS / MAX_THREADS, src/execution/physical_planner.cpp:
7320, 7520, 7641).  Here the knobs of a handle (hash vs radix mode, radix
partition bits, shared-table capacity, tile size, CTAs per SM) and of a batch
(tile size, shared-table capacity, CTAs per SM, tile order) are chosen by
timing candidates on the actual device-resident input, and the winner is
kept in a JSON cache keyed by the workload shape:

    (kind, rows bucket, estimated-groups bucket, key types, aggregates)

Buckets are powers of four, so nearby shapes share an entry.  The cache file
is ``$SLOTHDB_GB300_TUNE_CACHE`` or ``~/.cache/slothdb_gb300/tune.json``;
it is written atomically (temporary file + rename).

Tuning never changes results: every candidate is a valid execution of the
same plan, and ``tune_groupby`` checks that all candidates return the same
number of groups.
"""
from __future__ import annotations

import json
import math
import os
import tempfile

DEFAULT_CACHE = os.path.join(os.path.expanduser("~"), ".cache", "slothdb_gb300", "tune.json")


def cache_path() -> str:
    return os.environ.get("SLOTHDB_GB300_TUNE_CACHE", DEFAULT_CACHE)


def bucket(x: int) -> int:
    """Power-of-four bucket of a count (0 for 0)."""
    x = int(x)
    return 0 if x <= 0 else int(math.log(x, 4)) + 1


def shape_key(kind: str, rows: int, est_groups: int, key_types, aggs) -> str:
    aggs_s = ",".join("%s:%d" % (k if isinstance(k, str) else str(k), int(c)) for k, c in aggs)
    keys_s = ",".join(str(int(t)) for t in key_types)
    return "%s|r%d|g%d|k%s|a%s" % (kind, bucket(rows), bucket(est_groups), keys_s, aggs_s)


class TuneCache:
    """JSON map shape key -> {"options": {...}, "ms": best time}."""

    def __init__(self, path: str | None = None):
        self.path = path or cache_path()
        self.entries = {}
        try:
            with open(self.path) as f:
                data = json.load(f)
            if isinstance(data, dict):
                self.entries = {k: v for k, v in data.items()
                                if isinstance(v, dict) and isinstance(v.get("options"), dict)}
        except (OSError, ValueError):
            self.entries = {}

    def get(self, key: str):
        e = self.entries.get(key)
        return dict(e["options"]) if e else None

    def put(self, key: str, options: dict, ms: float):
        self.entries[key] = {"options": dict(options), "ms": float(ms)}

    def save(self):
        d = os.path.dirname(self.path) or "."
        os.makedirs(d, exist_ok=True)
        fd, tmp = tempfile.mkstemp(prefix=".tune", dir=d)
        with os.fdopen(fd, "w") as f:
            json.dump(self.entries, f, indent=1, sort_keys=True)
        os.replace(tmp, self.path)


def pick_best(candidates, run_ms, reps: int = 3):
    """Time every candidate with run_ms(candidate) (milliseconds; the first
    call is a warm-up) and return (best candidate, best median ms, table)."""
    table = []
    for c in candidates:
        try:
            run_ms(c)
            ts = sorted(run_ms(c) for _ in range(reps))
        except Exception as e:  # an option set the plan rejects is skipped
            table.append((c, None, str(e)))
            continue
        table.append((c, ts[len(ts) // 2], None))
    ok = [t for t in table if t[1] is not None]
    if not ok:
        raise RuntimeError("no candidate option set ran: %s" % [t[2] for t in table])
    best = min(ok, key=lambda t: t[1])
    return best[0], best[1], table


def groupby_candidates(est_groups: int, radix_ok: bool = True):
    """Option sets for one GROUP BY handle."""
    c = []
    for smem in (0, 1024, 4096):
        for tile in (8192, 32768):
            for ctas in (1, 2):
                c.append({"mode": 1, "smem_slots": smem, "tile_rows": tile, "ctas_per_sm": ctas})
    if radix_ok and est_groups >= (1 << 16):
        for bits in (8, 10, 12):
            for pre in (0, 1):
                c.append({"mode": 2, "radix_bits": bits, "radix_precombine": pre})
    return c


def batch_candidates():
    c = []
    for tile in (8192, 16384, 65536):
        for smem in (2048, 4096):
            for order in (0, 1):
                c.append({"tile_rows": tile, "smem_slots": smem, "order": order})
    return c


def _cuda_ms(fn):
    import torch
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def tune_groupby(col_types, group_cols, aggs, cols, nrows, est_groups=0, cache: TuneCache | None = None,
                 candidates=None, reps: int = 3, save: bool = True):
    """Time candidate options of one GROUP BY on device-resident columns;
    returns (options, ms) and records them in the cache."""
    from . import capi
    cache = cache or TuneCache()
    key = shape_key("groupby", nrows, est_groups, [col_types[g] for g in group_cols], aggs)
    groups_seen = set()

    def run(opts):
        mode_opt = {"mode": opts["mode"]} if "mode" in opts else {}
        g = capi.GroupBy(col_types, group_cols, aggs, est_groups=est_groups, options=mode_opt)
        try:
            for k, v in opts.items():
                if k != "mode":
                    g.set_option(k, v)

            def once():
                g.ingest(cols, nrows=nrows, device=True)
                g.finalize()

            ms = _cuda_ms(once)
            import ctypes as C
            r = capi.Result()
            capi.check(g.lib.gb_agg_result_device(g.h, C.byref(r)))
            groups_seen.add(int(r.n_rows))
            return ms
        finally:
            g.close()

    cands = candidates if candidates is not None else groupby_candidates(est_groups)
    best, ms, _ = pick_best(cands, run, reps)
    if len(groups_seen) != 1:
        raise RuntimeError("candidate option sets disagree on the group count: %s" % sorted(groups_seen))
    cache.put(key, best, ms)
    if save:
        cache.save()
    return best, ms


def tuned_groupby_options(col_types, group_cols, aggs, nrows, est_groups=0, cache: TuneCache | None = None):
    """Cached options for this shape, or None."""
    cache = cache or TuneCache()
    return cache.get(shape_key("groupby", nrows, est_groups, [col_types[g] for g in group_cols], aggs))


def tune_batch(make_batch, shape_desc: str, total_rows: int, n_queries: int, cache: TuneCache | None = None,
               candidates=None, reps: int = 3, save: bool = True):
    """make_batch(options) -> capi.Batch with every query added.  Times one
    run of each candidate (after a warm-up run that captures its graph)."""
    cache = cache or TuneCache()
    key = shape_key("batch:" + shape_desc, total_rows, n_queries, [], [])
    batches = {}

    def run(opts):
        k = json.dumps(opts, sort_keys=True)
        if k not in batches:
            batches[k] = make_batch(opts)
        return _cuda_ms(batches[k].run)

    try:
        cands = candidates if candidates is not None else batch_candidates()
        best, ms, _ = pick_best(cands, run, reps)
    finally:
        for b in batches.values():
            b.close()
    cache.put(key, best, ms)
    if save:
        cache.save()
    return best, ms

