#!/usr/bin/env python3
"""Benchmark of the GB300 HorseIR builtin library.

Workload (one "step"): the join + low-cardinality group-by query on seeded
synthetic tables -- a 59,986,052-row fact table joined to a 15,000,000-row
dimension filtered on a 365-day date window, the matches grouped on two
1-byte columns (6 groups) with sum/avg/count aggregates -- run as the
interpreter's sequence of builtin calls through libhgpu's C ABI.

  value   fact rows / s with the tables resident in HBM
  e2e     the same through the public API from pinned host buffers: the
          step's input columns are copied host->device and the six result
          vectors read back inside the timed region
  roofline  the kernel with the largest device time: algorithmic bytes
          (inputs read once + outputs written once) / its CUDA-event time,
          against the measured HBM copy bandwidth.  Per-kernel times come
          from a second pass of the same K steps with an event pair around
          every launch; the step time is taken without them.
  cpu_baseline  the CPU oracle port (a restatement of the reference's
          builtins, OpenMP like the reference) on the same full-size tables;
          the GPU's six result vectors must equal the oracle's (keys and
          counts bit-exact, f64 aggregates within 1e-12) or the run fails
  parity_vs_oracle  that comparison

`--impl reference` runs the same query on the same full-size tables through
the CPU oracle port on all host cores instead, W warm-up and K timed steps
(the reference library itself cannot be built where its sources are absent).
Multi-GPU: every rank runs its own replica (weak scaling, no collective on
the data path).

Other workloads (`--workload`): builtins (each builtin alone), batched,
served, ingest, and case (one builtin for a kernel profile).
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

from horsepower_gb300 import data as D  # noqa: E402
from horsepower_gb300 import plans as P  # noqa: E402
from horsepower_gb300.abi import Builtins, V0  # noqa: E402

ESIZE = {3: 4, 6: 8, 8: 1, 1: 1, 4: 8, 0: 1}
METRIC = "GB/s & rows/s per builtin; batched q/s and p99 vs plain per-op launches"
WORKLOAD = ("join + group-by: fact 59,986,052 x dim 15,000,000 (365-day filter), "
            "join_index, 5 gathers (2 common-index calls), group on (flag,status) -> 6 groups, sum/avg/count")


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class NvmlClocks:
    """SM clock and clock-event reasons read through NVML (read-only queries)
    every few milliseconds from a thread, so a timed region of a few tens of
    milliseconds still gets samples.  Reason bits (nvml.h): 0x4 sw_power_cap,
    0x8 hw_slowdown, 0x20 sw_thermal_slowdown, 0x40 hw_thermal_slowdown."""
    BITS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown"}

    def __init__(self, period_s=0.003):
        import threading
        self.nv = C.CDLL("libnvidia-ml.so.1")
        if self.nv.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        self.h = C.c_void_p()
        if self.nv.nvmlDeviceGetHandleByIndex_v2(int(os.environ.get("LOCAL_RANK", "0")), C.byref(self.h)) != 0:
            raise OSError("no NVML handle")
        self.reasons_fn = getattr(self.nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            self.nv.nvmlDeviceGetCurrentClocksThrottleReasons
        self.period, self.samples, self.stop_ev, self.th = period_s, [], threading.Event(), None
        self._threading = threading

    def _sample(self):
        mhz, rs = C.c_uint(), C.c_ulonglong()
        if self.nv.nvmlDeviceGetClockInfo(self.h, 1, C.byref(mhz)) == 0 and self.reasons_fn(self.h, C.byref(rs)) == 0:
            self.samples.append((mhz.value, rs.value))

    def start(self):
        def run():
            while not self.stop_ev.is_set():
                self._sample()
                time.sleep(self.period)
        self._sample()
        self.th = self._threading.Thread(target=run, daemon=True)
        self.th.start()

    def stop(self):
        self.stop_ev.set()
        self.th.join()
        self._sample()
        mx = C.c_uint()
        self.nv.nvmlDeviceGetMaxClockInfo(self.h, 1, C.byref(mx))
        reasons = sorted({nm for _, r in self.samples for b, nm in self.BITS.items() if r & b})
        sm = [m for m, _ in self.samples]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": float(mx.value), "reasons": reasons,
                "samples": len(sm), "source": "nvml"}


def Clocks():
    try:
        return NvmlClocks()
    except Exception:
        return SmiClocks()


class SmiClocks:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    def __init__(self):
        self.proc = None
        import tempfile
        self.path = os.path.join(tempfile.gettempdir(), f"hgpu_clocks_{os.getpid()}.csv")

    def start(self):
        os.makedirs(os.path.dirname(self.path), exist_ok=True)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", os.environ.get("LOCAL_RANK", "0")],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        self.f.close()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm), "source": "nvidia-smi"}


def pin_local_gpu():
    """One rank per GPU: before the library makes its CUDA context (it uses
    device 0), narrow CUDA_VISIBLE_DEVICES to this rank's LOCAL_RANK-th GPU.
    NVML (the clock samples) still addresses the GPU by LOCAL_RANK."""
    if int(os.environ.get("WORLD_SIZE", "1")) <= 1 or "LOCAL_RANK" not in os.environ:
        return
    lr = int(os.environ["LOCAL_RANK"])
    vis = [v for v in os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",") if v.strip()]
    os.environ["CUDA_VISIBLE_DEVICES"] = vis[lr] if lr < len(vis) else str(lr)


def dist_init(n_gpus):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    pin_local_gpu()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        return rank, ws, dist
    return 0, 1, None


def barrier_max(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def algorithmic_bytes(F, Dn, Dp, M, G):
    """Per-kernel compulsory bytes of one step (inputs read once + outputs
    written once), by kernel name; hash tables and sort passes not counted."""
    return {
        "compare": 2 * (4 + 1) * Dn,                          # two date compares over the dimension
        "logic": 3 * Dn,                                      # and of the two masks
        "compact": (1 + 4) * Dn + 4 * Dp,                     # compress pk by the mask
        "hash_build": 4 * Dp,                                 # build keys
        "join_probe": 4 * F + 8 * M,                          # probe keys in, staged u32 pairs out
        "join_emit": 8 * M + 16 * M,                          # staged pairs in, i64 index pairs out
        "gather_many": 2 * 8 * M + 2 * 2 * M + 3 * 16 * M,   # row ids (two calls) + values in, values out
        "gather": 2 * 8 * G * 2,                              # the group keys' flag and status
        "onesweep": 2 * 2 * M,                                # group key bytes (2 x 1 byte) in
        "widen": 8 * M,
        "seg_chunk": 3 * (8 + 8) * M,                         # rows + values of three aggregates
        "seg_warps": 3 * (8 + 8) * M,
    }


def run_gb300(args, rank, ws, dist, dim, fact):
    import horsepower_gb300
    gpu = horsepower_gb300.load()
    Lb = gpu.lib
    Lb.hgpuTimerStop.restype = C.c_double
    Lb.hgpuLaunchCount.restype = C.c_longlong
    Lb.hgpuSyncCount.restype = C.c_longlong
    Lb.hgpuProfileRead.restype = C.c_int32
    Lb.hgpuProfileRead.argtypes = [C.c_int32, C.POINTER(C.c_char_p), C.POINTER(C.c_double), C.POINTER(C.c_longlong)]
    Lb.initV.restype = C.c_void_p
    Lb.initV.argtypes = [C.c_void_p, C.c_int32, C.c_longlong]
    Lb.getHeapOffset.restype = C.c_longlong
    Lb.setHeapOffset.argtypes = [C.c_longlong]

    F, Dn = args.fact, args.dim
    if args.l2_fetch:
        Lb.hgpuSetTuning.argtypes = [C.c_int32, C.c_double]
        assert Lb.hgpuSetTuning(3, float(args.l2_fetch)) == 0  # HGPU_TUNE_L2_FETCH
    # device-resident copies of the tables
    host = {}
    dev = {}
    for tab, cols, types in (("dim", dim, P.DIM_TYPES), ("fact", fact, P.FACT_TYPES)):
        for k, v in cols.items():
            hv = gpu.vec(v, types[k])
            dv = V0()
            rc = Lb.hgpuToDevice(C.byref(dv), C.byref(hv))
            assert rc == 0, rc
            host[(tab, k)] = hv
            dev[(tab, k)] = dv
    Lb.hgpuSync()
    ddim = {k: dev[("dim", k)] for k in dim}
    dfact = {k: dev[("fact", k)] for k in fact}

    # the query as compiled C (queries/join_group.c), the form HorseIR runs a
    # query in; the Python statement sequence (plans.join_group) must give the
    # same bits
    query = P.join_group_compiled if P.compiled_queries(gpu) else P.join_group
    if query is not P.join_group:
        mark = Lb.getHeapOffset()
        a = [gpu.to_py(r) for r in P.join_group(gpu, ddim, dfact)]
        b = [gpu.to_py(r) for r in query(gpu, ddim, dfact)]
        Lb.setHeapOffset(mark)
        assert all(x.tobytes() == y.tobytes() for x, y in zip(a, b)), "compiled query differs from the statement sequence"

    def step(d_, f_):
        mark = Lb.getHeapOffset()
        out = query(gpu, d_, f_)
        Lb.hgpuSync()
        Lb.setHeapOffset(mark)
        return out

    for _ in range(args.warmup):
        step(ddim, dfact)
    # shapes of one step, for the algorithmic bytes
    mark = Lb.getHeapOffset()
    res = query(gpu, ddim, dfact)
    res_np = [gpu.to_py(r) for r in res]
    Lb.setHeapOffset(mark)
    M = int(res_np[5].sum())
    sel = ((dim["date"] >= D.WIN_LO) & (dim["date"] < D.WIN_HI))
    Dp = int(sel.sum())
    G = len(res_np[0])
    # the gathers' sector-level floor: the matched fact rows (ascending, as
    # the join emits them) touch these 32-byte sectors of each column; DRAM
    # cannot deliver less than whole sectors
    present = np.zeros(Dn, bool)
    present[dim["pk"][sel]] = True
    fi = np.flatnonzero(present[fact["fk"]])
    assert fi.size == M

    def sectors(es):
        return int(np.unique(fi * es // 32).size) * 32
    gather_floor = 2 * 8 * M + 2 * sectors(1) + 3 * sectors(8) + (2 * 1 + 3 * 8) * M

    # ---- timed region (device resident), no per-launch instrumentation
    clocks = Clocks()
    if dist:
        dist.barrier()
    Lb.hgpuSync()
    launches0 = Lb.hgpuLaunchCount()
    syncs0 = Lb.hgpuSyncCount()
    clocks.start()
    Lb.hgpuTimerStart()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step(ddim, dfact)
    ms = Lb.hgpuTimerStop()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    launches = Lb.hgpuLaunchCount() - launches0
    syncs = Lb.hgpuSyncCount() - syncs0

    # ---- the same K steps again with a CUDA event pair around every launch,
    # for the per-kernel durations (roofline, breakdown); the event records
    # add host work between launches, so this pass is not the step time
    Lb.hgpuSync()
    Lb.hgpuProfileReset()
    Lb.hgpuProfile(1)
    Lb.hgpuTimerStart()
    for _ in range(args.steps):
        step(ddim, dfact)
    ms_profiled = Lb.hgpuTimerStop()
    Lb.hgpuProfile(0)
    cap = 128
    names = (C.c_char_p * cap)()
    tot = (C.c_double * cap)()
    cnt = (C.c_longlong * cap)()
    nk = Lb.hgpuProfileRead(cap, names, tot, cnt)
    kernels = sorted(((names[i].decode(), tot[i], cnt[i]) for i in range(min(nk, cap))), key=lambda r: -r[1])
    ms = barrier_max(dist, ms)
    step_ms = ms / args.steps

    # ---- e2e: host (pinned) buffers -> device inside the timed region, results back
    pinned = {}
    for key, hv in host.items():
        pv = V0()
        Lb.initV(C.byref(pv), hv.typ, hv.len)  # caller allocation: pinned host arena
        C.memmove(pv.g, hv.g, hv.len * ESIZE[hv.typ])
        pinned[key] = pv
    h2d = sum(v.len * ESIZE[v.typ] for v in pinned.values())

    # uploads in the order the query first reads the columns; each runs on the
    # copy stream and a builtin waits only for the columns it reads
    first_use = [("dim", "date"), ("dim", "pk"), ("fact", "fk"), ("fact", "flag"), ("fact", "status"),
                 ("fact", "qty"), ("fact", "price"), ("fact", "disc")]
    upload_order = [k for k in first_use if k in pinned] + [k for k in pinned if k not in first_use]

    def e2e_step():
        mark = Lb.getHeapOffset()
        dv = {}
        for key in upload_order:
            z = V0()
            Lb.hgpuToDeviceAsync(C.byref(z), C.byref(pinned[key]))
            dv[key] = z
        out = query(gpu, {k: dv[("dim", k)] for k in dim}, {k: dv[("fact", k)] for k in fact})
        vals = [gpu.to_py(o) for o in out]
        Lb.setHeapOffset(mark)
        return vals

    for _ in range(max(1, args.warmup // 2)):
        e2e_step()
    if dist:
        dist.barrier()
    Lb.hgpuSync()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        vals = e2e_step()
    e2e_s = barrier_max(dist, time.perf_counter() - t0)
    d2h = sum(v.nbytes for v in vals)

    out = dict(rows_per_step=F, step_ms=step_ms, wall_s=wall, launches=launches, syncs=syncs, kernels=kernels,
               driver="compiled C query (queries/join_group.c)" if query is not P.join_group else "python statements",
               profiled_step_ms=ms_profiled / args.steps,
               clocks=clk, e2e_rows_s=ws * F * args.steps / e2e_s, e2e_ms=1000 * e2e_s / args.steps,
               h2d=h2d, d2h=d2h, shapes=dict(F=F, D=Dn, Dp=Dp, M=M, G=G), result=[v.tolist() for v in res_np],
               gather_floor=gather_floor)
    return out


def run_batched(args):
    """256 independent join + group-by plans over device-resident synthetic
    tables (fact rows log-uniform in [1e4, 2e7], dim = fact / 4, seed
    3000 + p): hgpuBatchJoinGroup against the same plans one at a time
    through the builtins.  Returns the JSON line."""
    import horsepower_gb300
    from horsepower_gb300 import batch as B
    gpu = horsepower_gb300.load()
    Lb = gpu.lib
    Lb.hgpuTimerStop.restype = C.c_double
    Lb.hgpuLaunchCount.restype = C.c_longlong
    Lb.getHeapOffset.restype = C.c_longlong
    Lb.setHeapOffset.argtypes = [C.c_longlong]
    sizes = B.log_uniform_sizes(args.plans, 10_000, args.max_fact, seed=3000)
    tabs = [B.synth_tables(gpu, 3000 + p, int(n), max(1, int(n) // 4)) for p, n in enumerate(sizes)]
    plans = [B.make_plan(d, f) for d, f in tabs]
    total_rows = int(sizes.sum())

    def batched():
        mark = Lb.getHeapOffset()
        r = B.run_batch(gpu, plans)
        Lb.setHeapOffset(mark)
        return r

    plain_query = P.join_group_compiled if P.compiled_queries(gpu) else P.join_group

    def one_at_a_time():
        out = []
        for d, f in tabs:
            mark = Lb.getHeapOffset()
            r = plain_query(gpu, d, f)
            out.append([gpu.to_py(v) for v in r])
            Lb.setHeapOffset(mark)
        return out

    for _ in range(args.warmup):
        got = batched()
    from horsepower_gb300 import autotune
    tuned, table = autotune.tune(gpu, batched, reps=2)
    got = batched()
    ref = one_at_a_time()
    exact = all(np.array_equal(g[k], np.asarray(w[k]).astype(g[k].dtype)) for g, w in zip(got, ref) for k in range(6))
    clocks = Clocks()
    Lb.hgpuSync()
    l0 = Lb.hgpuLaunchCount()
    clocks.start()
    Lb.hgpuTimerStart()
    for _ in range(args.steps):
        batched()
    ms_b = Lb.hgpuTimerStop() / args.steps
    clk = clocks.stop()
    launches = (Lb.hgpuLaunchCount() - l0) // args.steps
    Lb.hgpuSync()
    t_plain = []
    for _ in range(max(1, min(args.steps, 3))):
        Lb.hgpuTimerStart()
        one_at_a_time()
        t_plain.append(Lb.hgpuTimerStop())
    ms_p = statistics.median(t_plain)
    n = len(plans)
    # per-kernel device time of one batched call (CUDA events per launch; outside the timed region)
    Lb.hgpuProfileRead.restype = C.c_int32
    Lb.hgpuProfileRead.argtypes = [C.c_int32, C.POINTER(C.c_char_p), C.POINTER(C.c_double), C.POINTER(C.c_longlong)]
    Lb.hgpuProfileReset()
    Lb.hgpuProfile(1)
    batched()
    Lb.hgpuProfile(0)
    names, tot, cnt = (C.c_char_p * 128)(), (C.c_double * 128)(), (C.c_longlong * 128)()
    nk = Lb.hgpuProfileRead(128, names, tot, cnt)
    kern = sorted(((names[i].decode(), tot[i]) for i in range(min(nk, 128))), key=lambda r: -r[1])
    return {
        "metric": "batched join + group-by plans: queries/s", "value": n / (ms_b / 1000), "unit": "queries/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_b, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32+f64", "data": "synthetic (seeded, on device)",
        "config": {"workload": f"{n} join + group-by plans, fact rows log-uniform [1e4, {args.max_fact:.0e}], "
                               f"dim = fact/4, {total_rows:,} fact rows in all", "l2": "inputs larger than L2"},
        "plain_one_at_a_time": {"value": n / (ms_p / 1000), "unit": "queries/s", "ms": ms_p},
        "speedup_vs_plain": ms_p / ms_b, "bit_exact_vs_plain": bool(exact),
        "fact_rows_per_s": total_rows / (ms_b / 1000),
        "gpu_launches": int(launches), "clocks": clk,
        "kernels_ms": {k: round(t, 4) for k, t in kern},
        "autotune": {"chosen": tuned, "ms": {k: {str(v): round(t, 3) for v, t in d.items()} for k, d in table.items()}},
    }


def run_served(args):
    """The served form: lineitem (6,001,215 rows), the join tables (59,986,052 x
    15,000,000) and the order table (150,000,000 rows, Zipf(1.1) keys over
    10,000,000 values) resident in HBM; Poisson request streams of the
    60/30/10 filter-aggregate / join + group-by / top-1000 mix at several
    rates, through the continuous-batching loop and through the plain
    one-request-at-a-time builtin path.  Returns the JSON line."""
    import horsepower_gb300
    from horsepower_gb300 import batch as B
    from horsepower_gb300 import serve as S
    gpu = horsepower_gb300.load()
    Lb = gpu.lib
    line = S.line_table(gpu, 6_001_215, seed=0)
    dim, fact = B.synth_tables(gpu, 1, args.fact, args.dim)
    order = S.order_table(gpu, args.order_rows, seed=2)
    srv = S.Server(gpu, line, dim, fact, order, budget=args.budget_gb << 30)
    warm = S.request_stream(64, 0.0, seed=99)
    for _ in range(args.warmup):
        srv.run(warm)
        srv.run(warm[:16], S.PLAIN)
    rates = [int(r) for r in args.rates.split(",")]
    table = []
    clocks = Clocks()
    clocks.start()
    l0 = Lb.hgpuLaunchCount()
    for rate in rates:
        secs = args.serve_seconds if rate <= 5000 else min(args.serve_seconds, 5000 * args.serve_seconds / rate * 2)
        n = max(50, int(rate * secs))
        reqs = S.request_stream(n, rate, seed=7 + rate)
        row = {"rate": rate, "requests": n}
        for name, mode in (("served", S.BATCHED), ("plain", S.PLAIN)):
            _, st, meta = srv.run(reqs, mode)
            row[name] = {"qps": round(st.qps, 1), "p50_ms": round(st.p50_ms, 3), "p99_ms": round(st.p99_ms, 3),
                         "mean_ms": round(st.mean_ms, 3), "steps": st.steps, "max_step_requests": st.max_step_requests,
                         "max_step_gb": round(st.max_step_bytes / 2 ** 30, 3), "rejected": st.rejected}
            # the longest steps: their duration and request mix
            steps = {}
            for r, m in zip(reqs, meta):
                e = steps.setdefault(m["step"], [m["admit_s"], m["done_s"], [0, 0, 0]])
                e[2][r.kind] += 1
            longest = sorted(steps.values(), key=lambda e: e[0] - e[1])[:3]
            row[name]["longest_steps"] = [{"ms": round(1e3 * (e[1] - e[0]), 2), "filter_agg/join/topk": e[2]}
                                          for e in longest]
        table.append(row)
    launches = Lb.hgpuLaunchCount() - l0
    clk = clocks.stop()
    # per-kernel device time of one burst of 256 requests admitted together
    # (CUDA events per launch; outside the timed streams)
    Lb.hgpuProfileRead.restype = C.c_int32
    Lb.hgpuProfileRead.argtypes = [C.c_int32, C.POINTER(C.c_char_p), C.POINTER(C.c_double), C.POINTER(C.c_longlong)]
    burst = S.request_stream(256, 0.0, seed=5)
    Lb.hgpuProfileReset()
    Lb.hgpuProfile(1)
    _, bst, _ = srv.run(burst)
    Lb.hgpuProfile(0)
    names, tot, cnt = (C.c_char_p * 128)(), (C.c_double * 128)(), (C.c_longlong * 128)()
    nk = Lb.hgpuProfileRead(128, names, tot, cnt)
    kern = sorted(((names[i].decode(), tot[i], cnt[i]) for i in range(min(nk, 128))), key=lambda r: -r[1])
    srv.close()
    top = table[-1]
    return {
        "metric": "served requests: queries/s and p99 latency (continuous batching vs one request per launch sequence)",
        "value": top["served"]["qps"], "unit": "queries/s", "n_gpus": 1, "steps": len(rates), "warmup": args.warmup,
        "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "int32+int64+f64", "data": "synthetic (seeded; join and order tables generated on the device)",
        "config": {"workload": "Poisson request stream: 60% q6 filter-aggregate (random 365-day window), "
                               "30% join + group-by (random 365-day dim window), 10% top-1000 order on a random "
                               "key range; tables resident", "lineitem_rows": 6_001_215, "fact_rows": args.fact,
                   "dim_rows": args.dim, "order_rows": args.order_rows, "budget_gb": args.budget_gb,
                   "seconds_per_rate": args.serve_seconds},
        "p99_ms": top["served"]["p99_ms"], "p50_ms": top["served"]["p50_ms"],
        "plain": top["plain"], "speedup_qps_vs_plain": round(top["served"]["qps"] / max(top["plain"]["qps"], 1e-9), 2),
        "rates": table, "gpu_launches": int(launches), "clocks": clk,
        "burst_256": {"wall_ms": round(1e3 * bst.wall_s, 2), "steps": bst.steps,
                      "kernels_ms": {k: [round(t, 3), int(c)] for k, t, c in kern[:24]}},
    }


def run_builtins(args):
    """Each accelerated builtin alone on device-resident inputs of the
    configurations' shapes: call time (CUDA events on the library stream,
    host work and result-size reads included), the device time of its
    kernels, rows/s, and algorithmic GB/s (inputs read once, outputs written
    once) against the measured HBM copy bandwidth.  Returns the JSON line."""
    import horsepower_gb300
    from horsepower_gb300 import batch as B
    from horsepower_gb300 import serve as S
    from horsepower_gb300.abi import H_B, H_C, H_E, H_I, H_L
    gpu = horsepower_gb300.load()
    Lb = gpu.lib
    Lb.hgpuTimerStop.restype = C.c_double
    Lb.getHeapOffset.restype = C.c_longlong
    Lb.setHeapOffset.argtypes = [C.c_longlong]
    Lb.hgpuProfileRead.restype = C.c_int32
    Lb.hgpuProfileRead.argtypes = [C.c_int32, C.POINTER(C.c_char_p), C.POINTER(C.c_double), C.POINTER(C.c_longlong)]
    hbm, src = peaks()
    rng = np.random.default_rng(17)
    dev = lambda a, t: B.to_device(gpu, a, t)
    rows = {}

    def measure(name, fn, nrows, nbytes, reps=args.steps):
        for _ in range(max(1, args.warmup)):
            m = Lb.getHeapOffset(); fn(); Lb.setHeapOffset(m)
        ts = []
        for _ in range(reps):
            m = Lb.getHeapOffset()
            Lb.hgpuSync()
            Lb.hgpuTimerStart()
            fn()
            ts.append(Lb.hgpuTimerStop())
            Lb.setHeapOffset(m)
        Lb.hgpuProfileReset()
        Lb.hgpuProfile(1)
        m = Lb.getHeapOffset(); fn(); Lb.setHeapOffset(m)
        Lb.hgpuProfile(0)
        names, tot, cnt = (C.c_char_p * 64)(), (C.c_double * 64)(), (C.c_longlong * 64)()
        nk = Lb.hgpuProfileRead(64, names, tot, cnt)
        # the call's compute kernels; the one-warp copies of its counts to the
        # host (read_back) are listed under "kernels" but not summed
        kern_ms = sum(tot[i] for i in range(min(nk, 64)) if names[i].decode() != "read_back")
        call_ms = statistics.median(ts)
        rows[name] = {"rows": nrows, "call_ms": round(call_ms, 4), "kernel_ms": round(kern_ms, 4),
                      "rows_per_s": nrows / (call_ms / 1e3), "gbs_call": round(nbytes / (call_ms / 1e3) / 1e9, 1),
                      "gbs_kernels": round(nbytes / (kern_ms / 1e3) / 1e9, 1) if kern_ms > 0 else None,
                      "frac_kernels": round(nbytes / (kern_ms / 1e3) / 1e9 / hbm, 3) if kern_ms > 0 else None,
                      "algorithmic_bytes": int(nbytes),
                      "kernels": {names[i].decode(): [round(tot[i], 4), int(cnt[i])] for i in range(min(nk, 64))}}

    # ---- filter-aggregate table (6,001,215 rows) and a 60M-row stream
    t0 = D.filter_table(6_001_215, seed=0)
    ship, qty = dev(t0["shipdate"], H_I), dev(t0["qty"], H_I)
    disc, price = dev(t0["disc"], H_E), dev(t0["price"], H_E)
    m6 = gpu.call("pfnAnd", gpu.call("pfnGeq", ship, gpu.scalar(D.WIN_LO, H_I)), gpu.call("pfnLt", ship, gpu.scalar(D.WIN_HI, H_I)))
    n6 = 6_001_215
    sel6 = int(((t0["shipdate"] >= D.WIN_LO) & (t0["shipdate"] < D.WIN_HI)).sum())
    # compress: the mask and the values read once, the kept values written once (9 B/row + 8 B/kept)
    measure("compress_f64_6M", lambda: gpu.call("pfnCompress", m6, price), n6, 9 * n6 + 8 * sel6)
    ch = P.Chain(gpu, P.Q6_CHAIN.format(lo=D.WIN_LO, hi=D.WIN_HI))
    measure("q6_fused_chain_6M", lambda: ch.run([ship, qty, disc, price]), n6, 24 * n6)
    measure("q6_builtins_6M", lambda: P.filter_aggregate(gpu, dict(shipdate=ship, qty=qty, disc=disc, price=price)),
            n6, 24 * n6)
    N = 60_000_000
    a = dev(rng.standard_normal(N), H_E)
    b = dev(rng.standard_normal(N), H_E)
    mk = dev(rng.random(N) < 0.5, H_B)
    mk2 = dev(rng.random(N) < 0.5, H_B)
    measure("compare_f64_60M", lambda: gpu.call("pfnGt", a, gpu.scalar(0.25, H_E)), N, 9 * N)
    measure("arith_mul_f64_60M", lambda: gpu.call("pfnMul", a, b), N, 24 * N)
    measure("logic_and_60M", lambda: gpu.call("pfnAnd", mk, mk2), N, 3 * N)
    measure("compress_f64_60M_half", lambda: gpu.call("pfnCompress", mk, a), N, 9 * N + 8 * (N // 2))
    measure("where_60M_half", lambda: gpu.call("pfnWhere", mk), N, N + 8 * (N // 2))
    measure("sum_f64_60M", lambda: gpu.call("pfnSum", a), N, 8 * N)
    measure("max_f64_60M", lambda: gpu.call("pfnMax", a), N, 8 * N)
    idx = dev(np.flatnonzero(rng.random(N) < 0.145).astype(np.int64), H_L)
    M = int(idx.len)
    measure("index_f64_asc_8.7M_of_60M", lambda: gpu.call("pfnIndex", a, idx), M, 24 * M)
    ridx = dev(rng.integers(0, N, M).astype(np.int64), H_L)
    measure("index_f64_random_8.7M_of_60M", lambda: gpu.call("pfnIndex", a, ridx), M, 24 * M)
    # ---- join (the join + group-by configuration)
    dim, fact = B.synth_tables(gpu, 1, args.fact, args.dim)
    keep = gpu.call("pfnCompress", gpu.call("pfnAnd", gpu.call("pfnGeq", dim["date"], gpu.scalar(D.WIN_LO, H_I)),
                                            gpu.call("pfnLt", dim["date"], gpu.scalar(D.WIN_HI, H_I))), dim["pk"])
    eqs = gpu.sym("eq")
    j = gpu.call("pfnJoinIndex", keep, fact["fk"], eqs)
    Mj = int(V0.from_address(j.g).len)
    measure("join_index_60M_x_2.2M", lambda: gpu.call("pfnJoinIndex", keep, fact["fk"], eqs), args.fact,
            4 * args.fact + 4 * int(keep.len) + 16 * Mj)
    measure("member_60M_in_2.2M", lambda: gpu.call("pfnMember", fact["fk"], keep), args.fact,
            4 * args.fact + 4 * int(keep.len) + args.fact)
    measure("index_of_60M_in_2.2M", lambda: gpu.call("pfnIndexOf", keep, fact["fk"]), args.fact,
            4 * args.fact + 4 * int(keep.len) + 8 * args.fact)
    # ---- enum / foreign-key path: the fact's foreign key over the 15M-row key column
    #      (a permutation: hashed), the same keys sorted and sparse (binary search),
    #      and the semi-join mask carried through the enum's index
    nd = int(dim["pk"].len)
    measure("enum_fk_60M_over_15M_hash", lambda: gpu.call("pfnEnum", dim["pk"], fact["fk"]), args.fact,
            4 * args.fact + 4 * nd + 8 * args.fact)
    en = gpu.call("pfnEnum", dim["pk"], fact["fk"])
    ev = gpu.call("pfnValues", en)
    dmask = gpu.call("pfnLt", dim["date"], gpu.scalar(D.WIN_HI, H_I))
    measure("enum_semijoin_mask_60M", lambda: gpu.call("pfnIndex", dmask, ev), args.fact, 8 * args.fact + args.fact)
    spk = dev(np.arange(nd, dtype=np.int64) * 4 + 1, H_L)
    sfk = gpu.call("pfnIndex", spk, fact["fk"])
    measure("enum_fk_60M_over_15M_sorted_i64", lambda: gpu.call("pfnEnum", spk, sfk), args.fact,
            8 * args.fact + 8 * nd + 8 * args.fact)
    g2 = gpu.call("pfnGroup", gpu.list([fact["flag"], fact["status"]]))
    measure("group_trie_2x1B_60M", lambda: gpu.call("pfnGroup", gpu.list([fact["flag"], fact["status"]])), args.fact,
            2 * args.fact + 8 * args.fact)
    # ---- high-cardinality group-by and stable order (150M rows)
    o = S.order_table(gpu, args.order_rows, seed=2)
    pay = dev(rng.uniform(0.0, 1e5, args.order_rows), H_E)
    n2 = args.order_rows
    g = gpu.call("pfnGroup", o["key"])
    vals = gpu.call("pfnValues", g)
    ng = int(gpu.call("pfnKeys", g).len)
    # group: keys in (8N), row lists (8N) + group keys and starts (16G) out
    measure("group_i64_zipf_150M", lambda: gpu.call("pfnGroup", o["key"]), n2, 16 * n2 + 16 * ng,
            reps=max(2, args.steps // 2))
    measure("group_sum_f64_150M", lambda: gpu.call("hgpuGroupSum", pay, vals), n2, 16 * n2 + 8 * ng)
    measure("group_len_150M", lambda: gpu.call("hgpuGroupLen", pay, vals), n2, 16 * ng)  # group starts in, lengths out
    dirs = gpu.vec(np.array([1, 1], bool), H_B)
    measure("order_i64_i32_150M", lambda: gpu.call("pfnOrderBy", gpu.list([o["key"], o["sec"]]), dirs), n2, 20 * n2,
            reps=max(2, args.steps // 2))
    top = max(rows.items(), key=lambda kv: kv[1]["kernel_ms"])
    return {
        "metric": "GB/s & rows/s per builtin", "value": top[1]["gbs_kernels"], "unit": "GB/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "per builtin", "data": "synthetic (seeded)",
        "config": {"workload": "each builtin alone on the configurations' shapes; inputs resident in HBM, "
                               "larger than L2 (except the 6M-row table)", "peak_gbs": hbm, "peak_source": src},
        "builtins": rows,
    }


def run_extras(args):
    """The rest of the metric, measured in the same process after the
    headline: each builtin alone (the configurations' shapes, C0's plain and
    fused q6 chain, C2's group / group-sum / order at 150M rows), the batched
    256-plan form against the same plans one at a time (C3), and the served
    loop against one request per launch sequence at 1,000 and 5,000 req/s and
    at an offered rate above its capacity (C4).  Each part has its own timed
    regions and clock samples; a part that fails is reported, not fatal."""
    import horsepower_gb300
    Lb = horsepower_gb300.load().lib
    Lb.getHeapOffset.restype = C.c_longlong
    Lb.setHeapOffset.argtypes = [C.c_longlong]
    out = {}
    sub = argparse.Namespace(**vars(args))
    sub.steps = min(args.steps, 10)
    sub.warmup = min(args.warmup, 3)
    sub.rates = "1000,5000,20000"
    sub.serve_seconds = 1.0
    for name, fn in (("builtins", run_builtins), ("batched", run_batched), ("served", run_served)):
        mark = Lb.getHeapOffset()
        t0 = time.perf_counter()
        try:
            r = fn(sub)
            if name == "builtins":
                r = {"peak_gbs": r["config"]["peak_gbs"], "peak_source": r["config"]["peak_source"],
                     "note": "algorithmic bytes (inputs read once + outputs written once) / summed CUDA-event time "
                             "of the call's compute kernels (its read-back copy of result sizes to the host not "
                             "counted); call_ms includes host work and those reads",
                     "table": {k: {"rows": v["rows"], "call_ms": v["call_ms"], "kernel_ms": v["kernel_ms"],
                                   "rows_per_s": round(v["rows_per_s"]), "gbs": v["gbs_kernels"],
                                   "frac_of_peak": v["frac_kernels"]} for k, v in r["builtins"].items()}}
            elif name == "batched":
                r = {k: r[k] for k in ("metric", "value", "unit", "ms_per_step", "plain_one_at_a_time",
                                        "speedup_vs_plain", "bit_exact_vs_plain", "fact_rows_per_s", "gpu_launches",
                                        "clocks", "config")} | {"autotune_chosen": r["autotune"]["chosen"]}
            else:
                r = {"metric": r["metric"], "clocks": r["clocks"], "gpu_launches": r["gpu_launches"],
                     "rates": [{"offered_req_s": row["rate"], "requests": row["requests"],
                                "served": {k: row["served"][k] for k in ("qps", "p50_ms", "p99_ms", "max_step_requests")},
                                "plain": {k: row["plain"][k] for k in ("qps", "p50_ms", "p99_ms")},
                                "qps_vs_plain": round(row["served"]["qps"] / max(row["plain"]["qps"], 1e-9), 2)}
                               for row in r["rates"]]}
        except Exception as e:  # reported in the line; the headline stands
            r = {"error": f"{type(e).__name__}: {e}"}
        r["wall_s"] = round(time.perf_counter() - t0, 1)
        out[name] = r
        Lb.hgpuSync()
        Lb.setHeapOffset(mark)
    return out


def run_ingest(args):
    """readCSV of a 6,001,215-row lineitem-shaped .tbl (the reference's
    load_db.cc lineitem schema) from the page cache into HBM, and the same
    table through readSerializeV.  Text GB/s and rows/s end to end (file
    read, host-to-device copy, parse, symbols, strings), the kernels' split,
    and the oracle's readCSV (the reference's serial fgets/strtod loop) on a
    bounded sample of the same file."""
    import tempfile
    import horsepower_gb300
    from horsepower_gb300.abi import table_columns  # noqa: F401
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    from ingest_run import Ingest
    gpu = horsepower_gb300.load()
    Lb = gpu.lib
    Lb.hgpuTimerStop.restype = C.c_double
    Lb.getHeapOffset.restype = C.c_longlong
    Lb.setHeapOffset.argtypes = [C.c_longlong]
    Lb.hgpuProfileRead.restype = C.c_int32
    Lb.hgpuProfileRead.argtypes = [C.c_int32, C.POINTER(C.c_char_p), C.POINTER(C.c_double), C.POINTER(C.c_longlong)]
    hbm, src = peaks()
    rows = args.ingest_rows
    text, _ = D.lineitem_csv(rows, seed=9)
    tmp = tempfile.mkdtemp(prefix="hgpu_ingest_")
    path = os.path.join(tmp, "lineitem.tbl")
    with open(path, "wb") as f:
        f.write(text)
    nbytes = len(text)
    del text
    ing = Ingest(gpu)
    clocks = Clocks()

    def one():
        m = Lb.getHeapOffset()
        Lb.hgpuSync()
        t0 = time.perf_counter()
        rc, t = ing.csv(path, D.LINEITEM_TYPES, D.LINEITEM_NAMES)
        Lb.hgpuSync()
        dt = time.perf_counter() - t0
        if rc:
            raise RuntimeError(Lb.hgpuLastError())
        return dt, m, t

    for _ in range(max(1, args.warmup)):
        _, m, _ = one()
        Lb.setHeapOffset(m)
    clocks.start()
    ts = []
    for _ in range(args.steps):
        dt, m, _ = one()
        ts.append(dt)
        Lb.setHeapOffset(m)
    clk = clocks.stop()
    Lb.hgpuProfileReset()
    Lb.hgpuProfile(1)
    _, m, t = one()
    Lb.hgpuProfile(0)
    names, tot, cnt = (C.c_char_p * 64)(), (C.c_double * 64)(), (C.c_longlong * 64)()
    nk = Lb.hgpuProfileRead(64, names, tot, cnt)
    kern = sorted(((names[i].decode(), tot[i], int(cnt[i])) for i in range(min(nk, 64))), key=lambda k: -k[1])
    # string and symbol builtins on the loaded table (comments matched in HBM)
    vals = V0.from_address(t.g + 32)
    col = lambda j: V0.from_address(vals.g + 32 * j)  # noqa: E731
    pat = gpu.strs([b"%special%requests%"])
    smode = gpu.sym("MAIL")

    def timed_call(fn, reps=args.steps):
        for _ in range(max(1, args.warmup)):
            mm = Lb.getHeapOffset(); fn(); Lb.setHeapOffset(mm)
        out = []
        for _ in range(reps):
            mm = Lb.getHeapOffset()
            Lb.hgpuSync()
            Lb.hgpuTimerStart()
            fn()
            out.append(Lb.hgpuTimerStop())
            Lb.setHeapOffset(mm)
        return statistics.median(out)
    strings = {
        "like_comment_ms": timed_call(lambda: gpu.call("pfnLike", col(15), pat)),
        "like_shipmode_ms": timed_call(lambda: gpu.call("pfnLike", col(14), gpu.sym("%AIR%"))),
        "lt_shipmode_ms": timed_call(lambda: gpu.call("pfnLt", col(14), smode)),
    }
    strings["like_comment_gbs"] = (nbytes * 43 / 161) / (strings["like_comment_ms"] / 1e3) / 1e9
    # the binary format of the same table
    binp = os.path.join(tmp, "lineitem.bin")
    assert ing.save(binp, t) == 0
    bsize = os.path.getsize(binp)
    Lb.setHeapOffset(m)
    bts = []
    for k in range(max(1, args.warmup) + args.steps):
        m2 = Lb.getHeapOffset()
        t0 = time.perf_counter()
        rc, _ = ing.load(binp)
        Lb.hgpuSync()
        if k >= max(1, args.warmup):
            bts.append(time.perf_counter() - t0)
        Lb.setHeapOffset(m2)
        assert rc == 0
    sec = statistics.median(ts)
    parse_ms = dict((k, v) for k, v, _ in kern).get("csv_parse")
    col_bytes = rows * (4 * 4 + 8 * 4 + 2 + 4 * 3 + 8 * 2 + 8)  # values written (strings as pointers)
    # CPU: the oracle's readCSV on the first rows of the same file
    sample_rows = max(1, rows // args.cpu_scale)
    spath = os.path.join(tmp, "sample.tbl")
    with open(path, "rb") as f, open(spath, "wb") as g:
        for _ in range(sample_rows):
            g.write(f.readline())
    ora = Builtins(os.path.join(ROOT, "oracle", "_build", "liboracle.so"), "oracle")
    oing = Ingest(ora)
    ctimes = []
    for _ in range(args.cpu_reps):
        mo = ora.lib.getHeapOffset()
        t0 = time.perf_counter()
        rc, _ = oing.csv(spath, D.LINEITEM_TYPES, D.LINEITEM_NAMES)
        ctimes.append(time.perf_counter() - t0)
        ora.lib.setHeapOffset(mo)
        assert rc == 0
    cpu_rows_s = sample_rows / statistics.median(ctimes)
    rc, ot = oing.csv(spath, D.LINEITEM_TYPES, D.LINEITEM_NAMES)
    ovals = V0.from_address(ot.g + 32)
    ocol = lambda j: V0.from_address(ovals.g + 32 * j)  # noqa: E731
    t0 = time.perf_counter()
    ora.call("pfnLike", ocol(15), ora.strs([b"%special%requests%"]))
    cpu_like_rows_s = sample_rows / (time.perf_counter() - t0)
    for q in (path, binp, spath):
        os.remove(q)
    os.rmdir(tmp)
    achieved = (nbytes + col_bytes) / (parse_ms / 1e3) / 1e9 if parse_ms else None
    return {
        "metric": "readCSV text GB/s and rows/s (lineitem .tbl -> table in HBM)", "value": nbytes / sec / 1e9,
        "unit": "GB/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": sec * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8 text -> i32/f64/char/date/sym/str",
        "data": "synthetic (seeded lineitem-shaped text, space-padded fields)",
        "config": {"workload": f"readCSV lineitem {rows:,} rows, 16 columns (load_db.cc:111-129 types), "
                               "file in the page cache", "bytes": nbytes},
        "rows_per_s": rows / sec,
        "e2e": {"value": nbytes / sec / 1e9, "unit": "GB/s", "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": rows * 40, "rows_per_s": rows / sec},
        "kernels_ms": {k: [round(v, 3), c] for k, v, c in kern[:16]},
        "roofline": {"bound": "hbm", "kernel": "csv_parse", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm if achieved else None, "peak_source": src,
                     "algorithmic_bytes": nbytes + col_bytes, "traffic": None},
        "strings": dict(strings, rows=rows, cpu_like_rows_s=cpu_like_rows_s,
                        cpu_like_note=f"oracle pfnLike (OpenMP, {os.cpu_count()} threads) on the {sample_rows:,}-row sample"),
        "binary_load": {"bytes": bsize, "ms": statistics.median(bts) * 1e3,
                        "gbs": bsize / statistics.median(bts) / 1e9},
        "cpu_baseline": {"value": cpu_rows_s, "unit": "rows/s", "cores": 1, "kind": "port",
                         "sample": f"first {sample_rows:,} rows of the same file, oracle readCSV (serial, as "
                                   f"the reference's fgets loop), median of {len(ctimes)}",
                         "gbs": cpu_rows_s * nbytes / rows / 1e9},
        "gpu_launches": int(sum(c for _, _, c in kern)), "clocks": clk,
    }


CASES = ["join", "compress", "group", "groupkey", "order", "gather", "sum", "q6", "shared", "csv",
         "elementwise", "member", "index_of", "groupsum", "like", "quicksort"]


def run_case(args):
    """Single-builtin workloads for kernel profiling (ncu) and micro-benchmarks:
    `python bench.py --workload case --case NAME [--rows N] [--reps R]
    [--tune knob=value]`.  Inputs are seeded and uploaded once; the case runs
    --reps times on device-resident data and prints the CUDA-event time per
    call (not a bench line).

      join         @join_index, 2.17M build keys x 60M probe keys
      compress     @compress f64, 6M rows, 1.8% selected
      group        @group on two 1-byte columns, 8.67M rows
      groupkey     @group on i64 Zipf keys, 150M rows
      order        @order (i64 key, i32 sec), 20M rows
      gather       @index f64 by 14.5% ascending row ids of 60M
      sum          @sum then @max of f64, 60M rows
      q6           the fused q6 chain, 6M rows
      shared       16 batched join plans over one pair of tables
      csv          readCSV of a lineitem-shaped .tbl, 1M rows
      elementwise  @gt f64 vs scalar, @mul f64, @and, 60M rows
      member       @member of 60M probe keys in 2.17M keys
      index_of     @index_of of 60M probe keys in 2.17M keys
      groupsum     hgpuGroupSum of 3 f64 columns over the 6 (flag, status)
                   groups of 8.67M rows (the join + group-by aggregates)
      like         @like '%special%requests%' over loaded lineitem comments
      quicksort    @order of one f64 column with ties (the reference's
                   quicksort path), 2M rows
    """
    import horsepower_gb300
    from horsepower_gb300.abi import H_B, H_C, H_E, H_I, H_L
    L = horsepower_gb300.load()
    Lb = L.lib
    Lb.hgpuTimerStop.restype = C.c_double
    Lb.getHeapOffset.restype = C.c_longlong
    Lb.setHeapOffset.argtypes = [C.c_longlong]
    if args.tune:
        from horsepower_gb300 import autotune
        autotune.apply(L, {kv.split("=")[0]: float(kv.split("=")[1]) for kv in args.tune})
    rng = np.random.default_rng(5)
    keep_alive = []

    def dev(arr, typ):
        h = L.vec(arr, typ)
        d = V0()
        assert Lb.hgpuToDevice(C.byref(d), C.byref(h)) == 0
        keep_alive.append(d)
        return d

    last_fn = [None]

    def timed(fn):
        last_fn[0] = fn
        out = []
        for _ in range(args.reps):
            mark = Lb.getHeapOffset()
            Lb.hgpuSync()
            Lb.hgpuTimerStart()
            fn()
            out.append(Lb.hgpuTimerStop())
            Lb.setHeapOffset(mark)
        return out

    c = args.case
    if c in ("join", "member", "index_of"):
        F = args.rows or 59_986_052
        D_ = 15_000_000
        pk = rng.permutation(D_).astype(np.int32)
        keep = (rng.integers(0, D.NDAYS, D_) < 365)
        x = dev(pk[keep], H_I)
        y = dev(rng.integers(0, D_, F).astype(np.int32), H_I)
        f = L.sym("eq")
        fn = {"join": lambda: L.call("pfnJoinIndex", x, y, f), "member": lambda: L.call("pfnMember", y, x),
              "index_of": lambda: L.call("pfnIndexOf", x, y)}[c]
        t = timed(fn)
    elif c == "compress":
        n = args.rows or 6_001_215
        m = dev(rng.random(n) < 0.018, H_B)
        v = dev(rng.standard_normal(n), H_E)
        t = timed(lambda: L.call("pfnCompress", m, v))
    elif c == "group":
        n = args.rows or 8_662_796
        f = dev(rng.integers(0, 3, n).astype(np.int8), H_C)
        s_ = dev(rng.integers(0, 2, n).astype(np.int8), H_C)
        lst = L.list([f, s_])
        t = timed(lambda: L.call("pfnGroup", lst))
    elif c == "groupkey":
        from horsepower_gb300 import serve as S
        o = S.order_table(L, args.rows or 150_000_000, seed=2)
        t = timed(lambda: L.call("pfnGroup", o["key"]))
    elif c == "order":
        n = args.rows or 20_000_000
        key = dev(np.minimum(rng.zipf(1.1, n), 10_000_000).astype(np.int64), H_L)
        sec = dev(rng.integers(0, 2 ** 20 + 1, n).astype(np.int32), H_I)
        lst = L.list([key, sec])
        d = L.vec(np.array([1, 1], bool), H_B)
        t = timed(lambda: L.call("pfnOrderBy", lst, d))
    elif c == "gather":
        n = args.rows or 59_986_052
        x = dev(rng.standard_normal(n), H_E)
        idx = dev(np.flatnonzero(rng.random(n) < 0.1445).astype(np.int64), H_L)
        t = timed(lambda: L.call("pfnIndex", x, idx))
    elif c == "sum":
        n = args.rows or 60_000_000
        x = dev(rng.uniform(0, 1e5, n), H_E)
        t = timed(lambda: (L.call("pfnSum", x), L.call("pfnMax", x)))
    elif c == "elementwise":
        n = args.rows or 60_000_000
        a = dev(rng.standard_normal(n), H_E)
        b = dev(rng.standard_normal(n), H_E)
        m1, m2 = dev(rng.random(n) < 0.5, H_B), dev(rng.random(n) < 0.5, H_B)
        sc = L.scalar(0.25, H_E)
        t = timed(lambda: (L.call("pfnGt", a, sc), L.call("pfnMul", a, b), L.call("pfnAnd", m1, m2)))
    elif c == "groupsum":
        n = args.rows or 8_662_796
        f = dev(rng.integers(0, 3, n).astype(np.int8), H_C)
        s_ = dev(rng.integers(0, 2, n).astype(np.int8), H_C)
        g = L.call("pfnGroup", L.list([f, s_]))
        vals = L.call("pfnValues", g)
        cols = [dev(rng.uniform(0, 1e5, n), H_E) for _ in range(3)]
        t = timed(lambda: [L.call("hgpuGroupSum", col, vals) for col in cols])
    elif c == "shared":
        from horsepower_gb300 import batch as B
        n = args.rows or 59_986_052
        dim, fact = B.synth_tables(L, 1, n, n // 4)
        plans = [B.make_plan(dim, fact, D.DAYS0 + 100 * k, D.DAYS0 + 100 * k + 365) for k in range(16)]
        t = timed(lambda: B.run_batch(L, plans))
    elif c in ("csv", "like"):
        import tempfile
        text, _ = D.lineitem_csv(args.rows or 1_000_000, seed=9)
        fd, path = tempfile.mkstemp(suffix=".tbl")
        os.write(fd, text)
        os.close(fd)
        ty = (C.c_longlong * 16)(*D.LINEITEM_TYPES)
        sy = (C.c_longlong * 16)(*[Lb.getSymbol(nm.encode()) for nm in D.LINEITEM_NAMES])
        Lb.hgpuReadCSV.argtypes = [C.c_void_p, C.c_char_p, C.c_longlong, C.c_void_p, C.c_void_p]

        def load_table():
            z = V0()
            assert Lb.hgpuReadCSV(C.addressof(z), path.encode(), 16, ty, sy) == 0
            return z
        if c == "csv":
            t = timed(load_table)
        else:
            tab = load_table()
            keep_alive.append(tab)
            vals = V0.from_address(tab.g + 32)
            comment = V0.from_address(vals.g + 32 * 15)
            pat = L.strs([b"%special%requests%"])
            t = timed(lambda: L.call("pfnLike", comment, pat))
        os.remove(path)
    elif c == "quicksort":
        n = args.rows or 2_000_000
        x = dev(np.round(rng.standard_normal(n), 2), H_E)
        d = L.vec(np.array([1], bool), H_B)
        t = timed(lambda: L.call("pfnOrderBy", x, d))
    else:
        tb = D.filter_table(args.rows or 6_001_215)
        nodes = {k: dev(v, P.FILTER_TYPES[k]) for k, v in tb.items()}
        ch = P.Chain(L, P.Q6_CHAIN.format(lo=D.WIN_LO, hi=D.WIN_HI))
        t = timed(lambda: ch.run([nodes["shipdate"], nodes["qty"], nodes["disc"], nodes["price"]]))
    print(f"{c}: ms per call {[round(v, 4) for v in t]}")
    if args.kernels:  # one more call with an event pair around every launch
        Lb.hgpuProfileRead.restype = C.c_int32
        Lb.hgpuProfileRead.argtypes = [C.c_int32, C.POINTER(C.c_char_p), C.POINTER(C.c_double),
                                       C.POINTER(C.c_longlong)]
        Lb.hgpuProfileReset()
        Lb.hgpuProfile(1)
        reps, args.reps = args.reps, 1
        timed(last_fn[0])
        args.reps = reps
        Lb.hgpuProfile(0)
        cap = 128
        names, tot, cnt = (C.c_char_p * cap)(), (C.c_double * cap)(), (C.c_longlong * cap)()
        nk = Lb.hgpuProfileRead(cap, names, tot, cnt)
        for i in sorted(range(min(nk, cap)), key=lambda i: -tot[i]):
            print(f"  {names[i].decode():24s} {tot[i]:9.4f} ms  x{cnt[i]}")


def cpu_full(args, dim, fact, reps, warmup=0):
    """The oracle port (the reference's builtins restated in C, OpenMP like
    the reference) running the same query on the same full-size tables, on
    all host cores.  Returns (the cpu_baseline record, the result vectors)."""
    ora = Builtins(os.path.join(ROOT, "oracle", "_build", "liboracle.so"), "oracle")
    hd, hf = P.host_nodes(ora, dim, P.DIM_TYPES), P.host_nodes(ora, fact, P.FACT_TYPES)
    times, res = [], None
    for k in range(warmup + reps):
        mark = ora.lib.getHeapOffset()
        t0 = time.perf_counter()
        out = P.join_group(ora, hd, hf)
        dt = time.perf_counter() - t0
        if k >= warmup:
            times.append(dt)
        if res is None:
            res = [ora.to_py(v) for v in out]
        ora.lib.setHeapOffset(mark)
    t = statistics.median(times)
    F, Dn = len(fact["fk"]), len(dim["pk"])
    rec = dict(value=F / t, unit="rows/s", cores=int(os.environ.get("OMP_NUM_THREADS", os.cpu_count())),
               kind="port", ms_per_step=1000 * t,
               sample=f"the full workload: fact {F:,} x dim {Dn:,} rows (the same seeded tables), "
                      f"median of {len(times)} steps after {warmup} warm-up")
    return rec, res


def check_result(gpu_res, cpu_res, rtol=1e-12):
    """The query's six result vectors: group keys (flag, status) and counts
    bit-exact, the f64 aggregates within rtol of the oracle (whose OpenMP sum
    order depends on the thread count, like the reference's)."""
    g = [np.asarray(v) for v in gpu_res]
    c = [np.asarray(v) for v in cpu_res]
    exact = all(np.array_equal(g[k], c[k].astype(g[k].dtype)) for k in (0, 1, 5))
    close = all(g[k].shape == c[k].shape and np.allclose(g[k], c[k], rtol=rtol, atol=0) for k in (2, 3, 4))
    err = max(float(np.max(np.abs(g[k] - c[k]) / np.maximum(np.abs(c[k]), 1e-300))) if g[k].size else 0.0
              for k in (2, 3, 4))
    return {"keys_counts_bit_exact": bool(exact), "aggregates_within_1e-12": bool(close),
            "max_rel_err": err, "ok": bool(exact and close)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--fact", type=int, default=59_986_052)
    ap.add_argument("--dim", type=int, default=15_000_000)
    ap.add_argument("--cpu-scale", type=int, default=10, help="ingest workload: CPU sample = rows / this")
    ap.add_argument("--cpu-reps", type=int, default=3)
    ap.add_argument("--workload", default="join_group",
                    choices=["join_group", "batched", "served", "builtins", "ingest", "case"])
    ap.add_argument("--case", choices=CASES, default="join", help="with --workload case: the builtin to run")
    ap.add_argument("--rows", type=int, default=0, help="with --workload case: rows (0 = the case's default)")
    ap.add_argument("--reps", type=int, default=3, help="with --workload case: calls to time")
    ap.add_argument("--tune", action="append", default=[], help="with --workload case: knob=value")
    ap.add_argument("--kernels", action="store_true", help="with --workload case: per-kernel times of one more call")
    ap.add_argument("--ingest-rows", type=int, default=6_001_215)
    ap.add_argument("--l2-fetch", type=int, default=0,
                    help="default workload: the library's L2 fetch granularity knob (32, 64, 128; 0 = library default)")
    ap.add_argument("--headline-only", action="store_true",
                    help="default workload: skip the per-builtin, batched and served parts after the headline")
    ap.add_argument("--rates", default="200,1000,5000")
    ap.add_argument("--serve-seconds", type=float, default=1.5)
    ap.add_argument("--order-rows", type=int, default=150_000_000)
    ap.add_argument("--budget-gb", type=int, default=32)
    ap.add_argument("--plans", type=int, default=256)
    ap.add_argument("--max-fact", type=int, default=20_000_000)
    args = ap.parse_args()
    if args.workload == "case":
        run_case(args)
        return
    rank, ws, dist = dist_init(args.gpus)
    if args.workload in ("batched", "served", "builtins", "ingest") and args.impl == "gb300":
        line = {"batched": run_batched, "served": run_served, "builtins": run_builtins,
                "ingest": run_ingest}[args.workload](args)
        if rank == 0:
            print(json.dumps(line))
        return

    if args.impl == "reference":
        os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count()))
        if rank != 0:
            return
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
        dim, fact = D.join_tables(args.fact, args.dim, seed=1)
        cb, _ = cpu_full(args, dim, fact, reps=args.steps, warmup=args.warmup)
        print(json.dumps({"metric": METRIC, "value": cb["value"], "unit": "rows/s", "n_gpus": args.gpus,
                          "steps": args.steps, "warmup": args.warmup, "ms_per_step": cb["ms_per_step"],
                          "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32+f64",
                          "data": "synthetic (seeded, reference-shaped)", "impl": "reference",
                          "config": {"workload": WORKLOAD, "fact_rows": args.fact, "dim_rows": args.dim,
                                     "sample": cb["sample"]},
                          "cpu_baseline": cb,
                          "e2e": {"value": cb["value"], "unit": "rows/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return

    dim, fact = D.join_tables(args.fact, args.dim, seed=1 + rank)
    r = run_gb300(args, rank, ws, dist, dim, fact)
    if rank != 0:
        return
    hbm, src = peaks()
    sh = r["shapes"]
    alg = algorithmic_bytes(sh["F"], sh["D"], sh["Dp"], sh["M"], sh["G"])
    # the dominant kernel among those with algorithmic bytes (the read-back
    # copies of counts to the host are not HBM kernels)
    top = next((k for k in r["kernels"] if k[0] in alg), r["kernels"][0])
    per_step_ms = {k: t / args.steps for k, t, _ in r["kernels"]}
    tb = alg.get(top[0])
    achieved = (tb / (top[1] / args.steps / 1000) / 1e9) if tb else None
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        traffic = json.load(open(tpath)).get(top[0])
    builtins = {}
    for k, t, n in r["kernels"]:
        b = alg.get(k)
        builtins[k] = {"ms_per_step": round(t / args.steps, 4), "launches_per_step": n / args.steps,
                       "gbs": round(b / (t / args.steps / 1000) / 1e9, 1) if b else None}
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count()))
    cpu, cpu_res = cpu_full(args, dim, fact, reps=args.cpu_reps)
    parity = check_result(r["result"], cpu_res)
    if not parity["ok"]:
        raise SystemExit(f"the GPU result differs from the oracle's: {parity}")
    value = ws * sh["F"] / (r["step_ms"] / 1000)
    line = {
        "metric": METRIC, "value": value, "unit": "rows/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["step_ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32+f64", "data": "synthetic (seeded, reference-shaped)",
        "config": {"workload": WORKLOAD, "fact_rows": sh["F"], "dim_rows": sh["D"], "dim_selected": sh["Dp"],
                   "matches": sh["M"], "groups": sh["G"], "l2": "inputs larger than L2 (1.9 GB per step)",
                   "driver": r["driver"],
                   "parallelism": f"replicas x{ws}"},
        "e2e": {"value": r["e2e_rows_s"], "unit": "rows/s", "h2d_bytes_per_step": r["h2d"],
                "d2h_bytes_per_step": r["d2h"], "ms_per_step": r["e2e_ms"]},
        "roofline": {"bound": "hbm", "kernel": top[0], "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": (achieved / hbm) if achieved else None, "peak_source": src,
                     "traffic": traffic, "algorithmic_bytes_per_step": tb,
                     "traffic_gbs": (traffic / (top[1] / args.steps / 1000) / 1e9) if traffic else None,
                     "traffic_frac": (traffic / (top[1] / args.steps / 1000) / 1e9 / hbm) if traffic else None,
                     "sector_floor_bytes_per_step": r["gather_floor"] if top[0] == "gather_many" else None,
                     "frac_vs_sector_floor": (r["gather_floor"] / (top[1] / args.steps / 1000) / 1e9 / hbm)
                     if top[0] == "gather_many" else None},
        "cpu_baseline": cpu,
        "parity_vs_oracle": parity,
        "gpu_launches": r["launches"],
        "host_syncs_per_step": r["syncs"] / args.steps,
        "clocks": r["clocks"],
        "kernels_ms_per_step": {k: round(v, 4) for k, v in per_step_ms.items()},
        "kernel_times": ("a second pass of the same K steps with a CUDA event pair around every launch "
                         f"({r['profiled_step_ms']:.3f} ms per step with those events; ms_per_step is the pass "
                         "without them)"),
        "builtins": builtins,
    }
    if not args.headline_only:
        line["configs"] = run_extras(args)
    print(json.dumps(line))


if __name__ == "__main__":
    main()
