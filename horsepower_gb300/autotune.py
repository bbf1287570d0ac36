"""Autotuner for the library's knobs (hgpuSetTuning).

Knobs and their search ranges:

  tile_rows   probe rows per thread of the tiled join probes (tile = 256 x it)
  hash_load   open-addressing hash-table load factor
  radix_bits  LSD radix digit width of @group / @order
  l2_fetch    largest L2 fetch from DRAM in bytes (sparse sorted gathers prefer
              32, random probes and scattered writes 64)
  join_filter where the join's presence bitmap is read: 0 through L2, 1 from
              the shared memory of a 16-CTA cluster (dense i32 keys)
  radix_pass  how a radix pass of @group / @order finds each tile's offsets:
              0 a decoupled look-back, 1 a counting pass and one scan, 2 the
              counting pass for 32-bit keys only (default)

No knob changes a result (stable sorts, order-preserving compaction,
fixed-order sums), so tuning is a pure search over time: coordinate descent
over the knobs, each candidate timed with CUDA events on the library stream
(median of `reps` runs of the caller's workload), keeping the incumbent on
ties within `tol`.  The caller's workload is a zero-argument function that
runs the plans to be tuned for; `check` (optional) maps its return value to
something comparable, and every candidate's result must equal the default's.
"""
import ctypes as C
import json
import os
import statistics

TILE_ROWS, HASH_LOAD, RADIX_BITS, L2_FETCH, JOIN_FILTER, RADIX_PASS = 2, 0, 1, 3, 4, 5
KNOBS = {"tile_rows": (TILE_ROWS, [8, 16, 32]),
         "hash_load": (HASH_LOAD, [0.5, 0.6, 0.7, 0.8]),
         "radix_bits": (RADIX_BITS, [4, 5, 6, 7, 8]),
         "l2_fetch": (L2_FETCH, [32, 64, 128]),
         "join_filter": (JOIN_FILTER, [0, 1]),
         "radix_pass": (RADIX_PASS, [0, 1, 2])}


def _bind(L):
    L.lib.hgpuSetTuning.argtypes = [C.c_int32, C.c_double]
    L.lib.hgpuSetTuning.restype = C.c_int32
    L.lib.hgpuGetTuning.argtypes = [C.c_int32]
    L.lib.hgpuGetTuning.restype = C.c_double
    L.lib.hgpuTimerStop.restype = C.c_double


def current(L):
    _bind(L)
    return {k: L.lib.hgpuGetTuning(knob) for k, (knob, _) in KNOBS.items()}


def apply(L, setting):
    _bind(L)
    for k, v in setting.items():
        rc = L.lib.hgpuSetTuning(KNOBS[k][0], float(v))
        if rc:
            raise ValueError(f"hgpuSetTuning({k}={v}) returned {rc}")


def _time(L, fn, reps):
    out = None
    ts = []
    for _ in range(reps):
        L.lib.hgpuSync()
        L.lib.hgpuTimerStart()
        out = fn()
        ts.append(L.lib.hgpuTimerStop())
    return statistics.median(ts), out


def tune(L, workload, knobs=("tile_rows", "hash_load", "radix_bits", "l2_fetch"), reps=3, tol=0.02, check=None, log=None):
    """Coordinate descent over `knobs` for `workload`; applies and returns
    (best setting, {knob: {value: ms}})."""
    _bind(L)
    best = current(L)
    apply(L, best)
    base_ms, base_out = _time(L, workload, reps)
    want = check(base_out) if check else None
    table = {}
    for k in knobs:
        table[k] = {}
        for v in KNOBS[k][1]:
            trial = dict(best, **{k: v})
            apply(L, trial)
            ms, out = _time(L, workload, reps)
            if check is not None and check(out) != want:
                raise AssertionError(f"knob {k}={v} changed the result")
            table[k][v] = ms
            if log:
                log(f"autotune {k}={v}: {ms:.3f} ms")
        fastest = min(table[k], key=table[k].get)
        if table[k][fastest] < table[k].get(best[k], base_ms) * (1 - tol):
            best[k] = fastest
        apply(L, best)
    return best, table


def save(path, setting):
    with open(path, "w") as f:
        json.dump(setting, f, indent=1)


def load_saved(L, path):
    if os.path.exists(path):
        with open(path) as f:
            s = json.load(f)
        apply(L, s)
        return s
    return None
