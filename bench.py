#!/usr/bin/env python
"""bench.py — HBM throughput of the assign + reduce hot path on GB300.

Headline workload (one step, `value`): the strided/axis-work configuration —
x float32 AND float64 of shape (256, 512, 1024), N(0,1), seed 1 — evaluated
through the C ABI:  t = transpose(x, {2,0,1}) into a contiguous array;
y = (x - mean(x,{2},keep_dims)) / sqrt(variance(x,{2},keep_dims) + 1e-5);
amax(x, {0,2}); int32 argmax(x, 1).  Inputs (0.5 / 1 GiB) are larger than
L2 (129 MB), so no flush is needed between steps.

value      = algorithmic bytes of one step (each input read once, each output
             written once) / device time per step, GB/s, inputs resident in HBM;
e2e        = the same metric with host buffers: pinned host->device copies of
             the inputs and device->host copies of every result inside the
             timed region (copies in, kernels and copies out on three
             streams with two device buffer sets, so consecutive steps
             overlap on the link);
roofline   = the dominant kernel's algorithmic GB/s (CUDA events on its
             launching stream) over the measured HBM copy bandwidth;
cpu_baseline = the compiled CPU port of the reference's code path
             (oracle/xt_baseline.c, pinned to the oracle) on the host cores;
parity     = the step's GPU results against the port's results on the same
             inputs (transpose / amax / argmax bit-exact, the normalisation
             within its stated tolerance and the reference's envelope).

Sub-results in the same line (`--sub`, default all), each with its own
timing, roofline fraction, CPU baseline, accuracy or parity, and e2e leg
where the workload has host-side inputs:
  c0  plain small: E = A*b + exp(-A*A) (2048, 2048) and sum(E, {1});
  c2  precision: sum / mean / variance / norm_l2 of 2^28 float32 and bf16
      values, and the int32 -> int64 sum;
  c3  batching: 4096 uneven float32 instances of sum(A*v + C, {1}), one
      persistent launch replayed from a CUDA graph, vs a C loop of one
      xtg_reduce call per instance;
  c4  serving: Poisson request mix, served vs plain, p50 / p99 latency and
      throughput per offered rate over several repeats.

--impl reference times the CPU port alone on the headline workload (the
reference itself cannot be built: it needs xtl, absent on this image).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

SHAPE = (256, 512, 1024)
N = SHAPE[0] * SHAPE[1] * SHAPE[2]
NOMINAL_HBM_GBS = 8000.0  # GB300 HBM3e, nominal

METRIC = "HBM GB/s (frac of roofline) assign+reduce; served p50/p99 ms vs plain"
WORKLOAD = ("strided/axis work: x float32+float64 (256,512,1024) N(0,1) seed 1; transpose {2,0,1} to contiguous; "
            "y=(x-mean(x,{2},kd))/sqrt(var(x,{2},kd)+1e-5); amax {0,2}; int32 argmax axis 1")


def op_bytes(s: int) -> dict:
    """Algorithmic bytes per op for element size s."""
    return {
        "transpose": 2 * N * s,
        "normalize": 2 * N * s,
        "amax": N * s + SHAPE[1] * s,
        "argmax": N * s + SHAPE[0] * SHAPE[2] * 4,
    }


# The step's order: the four writers, then the readers, float64 amax first.
# A kernel that follows a writer pays the write-back of the writer's last
# dirty L2 lines (~100 MB, ~17 us on this part: a 512 MiB read takes 96 us
# after a 512 MiB copy and 79 us after a read); the order puts that cost on
# the largest read (amax float64, 1 GiB) instead of a 512 MiB one.  The
# operations are independent, so the order changes no result.
STEP_ORDER = (("transpose", 0), ("normalize", 0), ("transpose", 1), ("normalize", 1),
              ("amax", 1), ("argmax", 1), ("amax", 0), ("argmax", 0))


def step_bytes() -> int:
    return sum(op_bytes(4).values()) + sum(op_bytes(8).values())


def c1_config() -> dict:
    """The workload description both arms print (identical keys and values)."""
    return {"workload": WORKLOAD, "elements": N, "algorithmic_bytes_per_step": step_bytes(),
            "l2": "inputs (512 MiB f32, 1 GiB f64) larger than L2 (129 MB): no flush"}


def peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Barrier + max-over-ranks over gloo (timings only: the workload is
    replicated per GPU, there is no data-path collective)."""

    def __init__(self):
        self.ws, self.rank, self.local = dist_info()
        self.pg = None
        if self.ws > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.ws > 1:
            self.dist.barrier()

    def max(self, v: float) -> float:
        if self.ws == 1:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())


# ------------------------------------------------------------------------------ clocks
class Clocks:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.12)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------------------ workload
def make_inputs():
    g = np.random.default_rng(1)
    x32 = g.standard_normal(SHAPE, dtype=np.float32)
    x64 = g.standard_normal(SHAPE, dtype=np.float64)
    return x32, x64


class GpuStep:
    """The step as prebuilt C-ABI calls (lowered once, launched every step)."""

    def __init__(self, x32, x64, stream):
        import xtensor_gb300 as xg
        from xtensor_gb300 import ops
        from xtensor_gb300.device import DeviceArray
        from xtensor_gb300.expr import lower

        self.xg, self.lib = xg, xg.lib()
        self.stream = stream
        by_op = {}
        self.keep = []
        self.dev_in, self.dev_out = [], []
        for a, x in enumerate((x32, x64)):
            s = x.dtype.itemsize
            dx = DeviceArray.from_numpy(x)
            t = DeviceArray.empty((SHAPE[2], SHAPE[0], SHAPE[1]), x.dtype)
            y = DeviceArray.empty(SHAPE, x.dtype)
            am = DeviceArray.empty((SHAPE[1],), x.dtype)
            ai = DeviceArray.empty((SHAPE[0], SHAPE[2]), "int32")
            self.dev_in.append(dx)
            self.dev_out.append((t, y, am, ai))
            e_t, k1 = lower(dx.transpose((2, 0, 1)))
            o_t = t.xtg_array()
            e_y, k2 = lower((dx - xg.rmean(dx)) / xg.sqrt(xg.rvar(dx) + 1e-5))
            o_y = y.xtg_array()
            e_x, k3 = lower(dx)
            rd = ops.make_desc("amax", axes=[0, 2])
            o_am = am.xtg_array()
            o_ai = ai.xtg_array()
            self.keep += [e_t, k1, o_t, e_y, k2, o_y, e_x, k3, rd, o_am, o_ai]
            L, st = self.lib, stream
            by_op[("transpose", a)] = (s, lambda e=e_t, o=o_t: L.xtg_assign(C.byref(e), C.byref(o), st), 0)
            by_op[("normalize", a)] = (s, lambda e=e_y, o=o_y: L.xtg_assign(C.byref(e), C.byref(o), st), 1)
            by_op[("amax", a)] = (s, lambda e=e_x, r=rd, o=o_am: L.xtg_reduce(C.byref(e), C.byref(r), C.byref(o), st), 2)
            by_op[("argmax", a)] = (s, lambda e=e_x, o=o_ai: L.xtg_argreduce(C.byref(e), 0, 1, 1, C.byref(o), st), 3)
        # (op name, element size, fn, input index, output index) in step order
        self.calls = [(nm, *by_op[(nm, a)][:2], a, by_op[(nm, a)][2]) for nm, a in STEP_ORDER]

    def run(self, events=None):
        from xtensor_gb300._ffi import check
        for i, (_, _, fn, _, _) in enumerate(self.calls):
            if events is not None:
                check(self.lib.xtg_event_record(events[i], self.stream))
            check(fn())
        if events is not None:
            check(self.lib.xtg_event_record(events[len(self.calls)], self.stream))


def writeback_probe(step, lib, stream, reps) -> dict:
    """amax float32 timed (CUDA events) right after the float32 normalisation
    and right after the float32 argmax: the difference is the write-back of
    the writer's dirty L2 lines, which lands on whichever kernel follows it."""
    from xtensor_gb300._ffi import check
    fn = {(nm, a): f for nm, _, f, a, _ in step.calls}
    res = {}
    for label, prev in (("after_normalize_f32", fn[("normalize", 0)]), ("after_argmax_f32", fn[("argmax", 0)])):
        evs = [ev_create(lib, 2) for _ in range(reps)]
        for k in range(reps):
            check(prev())
            check(lib.xtg_event_record(evs[k][0], stream))
            check(fn[("amax", 0)]())
            check(lib.xtg_event_record(evs[k][1], stream))
        check(lib.xtg_stream_sync(stream))
        res[f"amax_f32_ms_{label}"] = round(sum(ev_ms(lib, a, b) for a, b in evs) / reps, 4)
    res["note"] = ("a kernel that follows a writer pays the write-back of the writer's last dirty L2 lines; "
                   "the step orders writers first and the float64 amax right after them")
    return res


def ev_create(lib, n):
    from xtensor_gb300._ffi import check
    evs = []
    for _ in range(n):
        e = C.c_void_p()
        check(lib.xtg_event_create(C.byref(e)))
        evs.append(e.value)
    return evs


def ev_ms(lib, a, b) -> float:
    from xtensor_gb300._ffi import check
    f = C.c_float()
    check(lib.xtg_event_elapsed_ms(a, b, C.byref(f)))
    return float(f.value)


# ------------------------------------------------------------------------------ CPU port
def cpu_port_time(x32, x64, reps_budget_s=20.0):
    """Time the compiled CPU port of the reference's path on the host cores."""
    from oracle.oracle import SO, lib as olib  # noqa: F401
    olib()
    L = C.CDLL(str(SO))
    P = C.c_void_p
    i64 = C.c_int64
    for nm in ("transpose_201", "amax_02"):
        for t in ("f32", "f64"):
            getattr(L, f"bl_{nm}_{t}").argtypes = [P, P, i64, i64, i64]
    for t in ("f32", "f64"):
        getattr(L, f"bl_normalize_{t}").argtypes = [P, P, i64, i64, C.c_double]
        getattr(L, f"bl_argmax_1_{t}").argtypes = [P, P, i64, i64, i64, P]
    outs = {}
    for x in (x32, x64):
        outs[x.dtype.itemsize] = dict(
            t=np.empty((SHAPE[2], SHAPE[0], SHAPE[1]), x.dtype), y=np.empty(SHAPE, x.dtype),
            am=np.empty((SHAPE[1],), x.dtype), ai=np.empty((SHAPE[0], SHAPE[2]), np.int32),
            tmp=np.empty((SHAPE[0], SHAPE[2], SHAPE[1]), x.dtype))

    def one():
        t0 = time.perf_counter()
        for x in (x32, x64):
            tn = "f32" if x.dtype == np.float32 else "f64"
            o = outs[x.dtype.itemsize]
            d0, d1, d2 = SHAPE
            getattr(L, f"bl_transpose_201_{tn}")(x.ctypes.data, o["t"].ctypes.data, d0, d1, d2)
            getattr(L, f"bl_normalize_{tn}")(x.ctypes.data, o["y"].ctypes.data, d0 * d1, d2, 1e-5)
            getattr(L, f"bl_amax_02_{tn}")(x.ctypes.data, o["am"].ctypes.data, d0, d1, d2)
            getattr(L, f"bl_argmax_1_{tn}")(x.ctypes.data, o["ai"].ctypes.data, d0, d1, d2, o["tmp"].ctypes.data)
        return time.perf_counter() - t0

    times = [one()]
    while sum(times) < reps_budget_s and len(times) < 3:
        times.append(one())
    return min(times), len(times), outs


def cores() -> int:
    return int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))


# ------------------------------------------------------------------------------ arms
def run_reference(args):
    ws, rank, local = dist_info()
    if rank != 0:
        return 0
    x32, x64 = make_inputs()
    total = step_bytes()
    times = []
    for i in range(args.warmup + args.steps):
        t, _, _ = cpu_port_time(x32, x64, reps_budget_s=0.0)
        if i >= args.warmup:
            times.append(t)
    sec = statistics.median(times)
    val = total / sec / 1e9
    line = {
        "metric": METRIC, "value": round(val, 3), "unit": "GB/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(sec * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32,f64", "data": "synthetic", "impl": "reference",
        "config": c1_config(),
        "cpu_baseline": {"value": round(val, 3), "unit": "GB/s", "cores": cores(), "kind": "port",
                         "sample": "full workload per step (compiled C port of the reference's loops, OpenMP)"},
        "e2e": {"value": round(val, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference itself cannot be built (xtl 0.8.0 is absent); oracle/xt_baseline.c restates its code path",
    }
    print(json.dumps(line))
    return 0


def run_gpu(args):
    import xtensor_gb300 as xg
    from xtensor_gb300._ffi import check

    D = Dist()
    xg.init(D.local)
    lib = xg.lib()
    st = C.c_void_p()
    check(lib.xtg_stream_create(C.byref(st)))
    stream = st.value
    x32, x64 = make_inputs()
    step = GpuStep(x32, x64, stream)
    nops = len(step.calls)
    for _ in range(args.warmup):
        step.run()
    check(lib.xtg_stream_sync(stream))

    # ---- device-resident timing
    evs = [ev_create(lib, nops + 1) for _ in range(args.steps)]
    per_op = [0.0] * nops
    t0, t1 = ev_create(lib, 2)
    clocks = Clocks(D.local)
    clocks.start()
    time.sleep(0.15)
    D.barrier()
    check(lib.xtg_device_sync())
    l0 = xg.jit_stats()["launches"]
    check(lib.xtg_event_record(t0, stream))
    for k in range(args.steps):
        step.run(evs[k])
    check(lib.xtg_event_record(t1, stream))
    check(lib.xtg_event_sync(t1))
    check(lib.xtg_device_sync())
    l1 = xg.jit_stats()["launches"]
    D.barrier()
    clk = clocks.stop()
    for k in range(args.steps):
        for i in range(nops):
            per_op[i] += ev_ms(lib, evs[k][i], evs[k][i + 1])
    kern_ms = sum(per_op) / args.steps  # device time inside the kernels
    wall_ms = ev_ms(lib, t0, t1) / args.steps
    ms = D.max(wall_ms)
    total = step_bytes() * D.ws
    value = total / (ms / 1e3) / 1e9

    # dominant kernel
    names = [f"{nm}_{'f32' if s == 4 else 'f64'}" for nm, s, *_ in step.calls]
    avg = [t / args.steps for t in per_op]
    dom = int(np.argmax(avg))
    nm, s, *_ = step.calls[dom]
    dom_bytes = op_bytes(s)[nm]
    achieved = dom_bytes / (avg[dom] / 1e3) / 1e9
    peak, peak_kind = peaks()
    traffic = None
    tf = ROOT / "profiles" / "traffic.json"
    if tf.exists():
        try:
            traffic = json.loads(tf.read_text()).get(names[dom])
        except Exception:
            traffic = None
    per_kernel = {names[i]: {"ms": round(avg[i], 4), "GB/s": round(op_bytes(step.calls[i][1])[step.calls[i][0]] / (avg[i] / 1e3) / 1e9, 1),
                             "frac": round(op_bytes(step.calls[i][1])[step.calls[i][0]] / (avg[i] / 1e3) / 1e9 / peak, 3),
                             "frac_nominal": round(op_bytes(step.calls[i][1])[step.calls[i][0]] / (avg[i] / 1e3) / 1e9
                                                   / NOMINAL_HBM_GBS, 3)}
                  for i in range(nops)}

    # ---- write-back attribution: amax float32 right after the float32
    # normalisation (a writer) and right after the float32 argmax (a reader)
    wb = writeback_probe(step, lib, stream, max(5, min(args.steps, 20)))

    # ---- end to end through the C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(lib, step, x32, x64, stream, max(2, min(args.steps, 10)), D)

    # ---- CPU baseline (rank 0, N=1) and parity of the step's GPU results
    cpu = parity = None
    if D.rank == 0 and D.ws == 1 and not args.no_cpu:
        sec, reps, cpu_outs = cpu_port_time(x32, x64)
        cpu = {"value": round(step_bytes() / sec / 1e9, 3), "unit": "GB/s", "cores": cores(), "kind": "port",
               "sample": f"full workload, best of {reps} (compiled C port of the reference's loops, OpenMP {cores()} threads)"}
        parity = c1_parity(step, cpu_outs, x32, x64)
        del cpu_outs
    del step

    # ---- the other configurations, each with its own timing, roofline,
    # CPU baseline, parity / accuracy and end-to-end leg (rank 0, N=1)
    subs = {}
    wanted = [w for w in args.sub.split(",") if w and w != "none"]
    if D.rank == 0 and D.ws == 1:
        for nm in wanted:
            fn = {"c0": lambda: c0_section(args, stream), "c2": lambda: c2_section(args, stream),
                  "c3": lambda: c3_section(args), "c4": lambda: c4_section(args),
                  "chunked": lambda: chunked_section(args)}[nm]
            t0 = time.perf_counter()
            try:
                subs[nm] = fn()
            except Exception as ex:  # reported in the line; the headline stands
                subs[nm] = {"error": f"{type(ex).__name__}: {ex}"}
            subs[nm]["section_wall_s"] = round(time.perf_counter() - t0, 1)

    if D.rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "GB/s", "n_gpus": D.ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32,f64", "data": "synthetic",
            "config": c1_config(), "parallelism": f"replicas x{D.ws}", "kernel_ms_per_step": round(kern_ms, 4),
            "roofline": {"bound": "hbm", "kernel": names[dom], "achieved": round(achieved, 1), "peak": peak,
                         "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": traffic,
                         "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback 6800 GB/s"},
            "per_kernel": per_kernel,
            # the same throughputs against the nominal 8000 GB/s HBM3e figure
            "vs_nominal_hbm": {"peak": NOMINAL_HBM_GBS, "step_frac": round(value / D.ws / NOMINAL_HBM_GBS, 4),
                               "kernel_frac": round(achieved / NOMINAL_HBM_GBS, 4)},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "parity": parity,
            "l2_writeback": wb,
            "gpu_launches": int(l1 - l0),
            "clocks": clk,
            **subs,
        }
        print(json.dumps(line))
    return 0


def run_e2e(lib, step, x32, x64, stream, steps, D):
    """The step end to end through the C ABI from pinned host memory: every
    step copies both inputs in and every output back.  Copies in, kernels and
    copies out run on three streams ordered by events, with two device buffer
    sets, so step k's outputs stream back while step k+1's inputs stream in
    (the link carries both directions at once)."""
    from xtensor_gb300._ffi import check
    H2D, D2H = 1, 2
    sets = [step, GpuStep(x32, x64, stream)]

    def mkstream():
        sp = C.c_void_p()
        check(lib.xtg_stream_create(C.byref(sp)))
        return sp.value
    s_in, s_out = mkstream(), mkstream()
    hin = []
    for x in (x32, x64):
        p = C.c_void_p()
        check(lib.xtg_host_alloc(C.byref(p), x.nbytes))
        C.memmove(p.value, x.ctypes.data, x.nbytes)
        hin.append((p.value, x.nbytes))
    hout = []
    for o in [o for outs in step.dev_out for o in outs]:
        p = C.c_void_p()
        check(lib.xtg_host_alloc(C.byref(p), o.nbytes))
        hout.append((p.value, o.nbytes))
    h2d = sum(n for _, n in hin)
    d2h = sum(n for _, n in hout)
    nops = len(step.calls)
    ev = [{"in": ev_create(lib, 2), "out": ev_create(lib, nops), "comp": ev_create(lib, 1)[0],
           "d2h": ev_create(lib, 1)[0]} for _ in sets]
    # here the calls run grouped by input (float32 first), so the kernels of
    # the first input overlap the copy of the second
    order = sorted(range(nops), key=lambda i: (step.calls[i][3], i))
    per = len(step.dev_out[0])

    def one(k):
        b = k % 2
        S, E = sets[b], ev[b]
        if k >= 2:
            check(lib.xtg_stream_wait_event(s_in, E["comp"]))    # inputs no longer read
            check(lib.xtg_stream_wait_event(stream, E["d2h"]))   # outputs copied out
        for a, (h, n) in enumerate(hin):
            check(lib.xtg_memcpy(S.dev_in[a].ptr, h, n, H2D, s_in))
            check(lib.xtg_event_record(E["in"][a], s_in))
        waited = set()
        for i in order:
            _, _, fn, a, oi = S.calls[i]
            if a not in waited:
                check(lib.xtg_stream_wait_event(stream, E["in"][a]))
                waited.add(a)
            check(fn())
            check(lib.xtg_event_record(E["out"][i], stream))
        check(lib.xtg_event_record(E["comp"], stream))
        for i in order:
            _, _, _, a, oi = S.calls[i]
            check(lib.xtg_stream_wait_event(s_out, E["out"][i]))
            o = S.dev_out[a][oi]
            check(lib.xtg_memcpy(hout[a * per + oi][0], o.ptr, o.nbytes, D2H, s_out))
        check(lib.xtg_event_record(E["d2h"], s_out))

    for k in range(2):
        one(k)
    check(lib.xtg_device_sync())
    t0, t1 = ev_create(lib, 2)
    D.barrier()
    check(lib.xtg_event_record(t0, s_in))
    for k in range(steps):
        one(k)
    check(lib.xtg_event_record(t1, s_out))
    check(lib.xtg_event_sync(t1))
    check(lib.xtg_device_sync())
    ms = D.max(ev_ms(lib, t0, t1) / steps)
    for h, _ in hin + hout:
        lib.xtg_host_free(h)
    return {"value": round(step_bytes() * D.ws / (ms / 1e3) / 1e9, 3), "unit": "GB/s", "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": d2h, "ms_per_step": round(ms, 3), "steps": steps,
            "mode": "3 streams (copy in / kernels / copy out), 2 device buffer sets"}


# ------------------------------------------------------------------------------ shared helpers
def f32_to_bf16_bits(x: np.ndarray) -> np.ndarray:
    """Round-to-nearest-even float32 -> bfloat16 bit patterns (uint16)."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    nan = (u & 0x7FFFFFFF) > 0x7F800000
    r[nan] = ((u[nan] >> 16) | 0x40).astype(np.uint16)
    return r


def port_lib():
    """The compiled CPU port of the reference's loops (oracle/xt_baseline.c),
    with the argument types of every routine the benchmarks time."""
    from oracle.oracle import SO, lib as olib
    olib()
    L = C.CDLL(str(SO))
    P, i64 = C.c_void_p, C.c_int64
    for t in ("f32", "f64"):
        getattr(L, f"bl_transpose_201_{t}").argtypes = [P, P, i64, i64, i64]
        getattr(L, f"bl_amax_02_{t}").argtypes = [P, P, i64, i64, i64]
        getattr(L, f"bl_normalize_{t}").argtypes = [P, P, i64, i64, C.c_double]
        getattr(L, f"bl_argmax_1_{t}").argtypes = [P, P, i64, i64, i64, P]
    L.bl_c0_assign.argtypes = [P, P, P, i64, i64]
    L.bl_c0_sum.argtypes = [P, P, i64, i64]
    L.bl_c3_rowsum_f32.argtypes = [P, P, P, P, i64, i64]
    L.bl_sum_i32_i64.argtypes = [P, i64]
    L.bl_sum_i32_i64.restype = i64
    for t in ("f32", "bf16"):
        for op in C2_OPS:
            f = getattr(L, f"bl_stat_{op}_{t}")
            f.argtypes = [P, i64]
            f.restype = C.c_float if op == "sum" else C.c_double
    return L


class PinnedHost:
    """Page-locked copies of host arrays (the e2e legs copy from these)."""

    def __init__(self, lib, arrays):
        from xtensor_gb300._ffi import check
        self.lib, self.bufs = lib, []
        for a in arrays:
            p = C.c_void_p()
            check(lib.xtg_host_alloc(C.byref(p), max(1, a.nbytes)))
            C.memmove(p.value, a.ctypes.data, a.nbytes)
            self.bufs.append((p.value, a.nbytes))

    @classmethod
    def empty(cls, lib, nbytes_list):
        self = cls(lib, [])
        from xtensor_gb300._ffi import check
        for n in nbytes_list:
            p = C.c_void_p()
            check(lib.xtg_host_alloc(C.byref(p), max(1, n)))
            self.bufs.append((p.value, n))
        return self

    def free(self):
        for p, _ in self.bufs:
            self.lib.xtg_host_free(p)
        self.bufs = []


def pipelined_e2e(lib, sets, hin, hout, stream, steps, algo_bytes, D=None):
    """End to end through the C ABI from pinned host memory: every step copies
    its inputs in (pinned -> device), runs the step's calls and copies every
    output back (device -> pinned).  Copies in, calls and copies out run on
    three streams ordered by events, alternating between two device buffer
    sets, so one step's outputs stream back while the next step's inputs
    stream in.  `sets` are two objects with .dev_in, .dev_out (DeviceArray
    lists, matching hin / hout) and .launch(stream)."""
    from xtensor_gb300._ffi import check
    H2D, D2H = 1, 2

    def mkstream():
        sp = C.c_void_p()
        check(lib.xtg_stream_create(C.byref(sp)))
        return sp.value
    s_in, s_out = mkstream(), mkstream()
    ev = [{"in": ev_create(lib, 1)[0], "comp": ev_create(lib, 1)[0], "d2h": ev_create(lib, 1)[0]} for _ in sets]

    def one(k):
        b = k % 2
        S, E = sets[b], ev[b]
        if k >= 2:
            check(lib.xtg_stream_wait_event(s_in, E["comp"]))    # inputs no longer read
            check(lib.xtg_stream_wait_event(stream, E["d2h"]))   # outputs copied out
        for (h, n), d in zip(hin.bufs, S.dev_in):
            check(lib.xtg_memcpy(d.ptr, h, n, H2D, s_in))
        check(lib.xtg_event_record(E["in"], s_in))
        check(lib.xtg_stream_wait_event(stream, E["in"]))
        S.launch(stream)
        check(lib.xtg_event_record(E["comp"], stream))
        check(lib.xtg_stream_wait_event(s_out, E["comp"]))
        for (h, n), d in zip(hout.bufs, S.dev_out):
            check(lib.xtg_memcpy(h, d.ptr, n, D2H, s_out))
        check(lib.xtg_event_record(E["d2h"], s_out))

    for k in range(2):
        one(k)
    check(lib.xtg_device_sync())
    t0, t1 = ev_create(lib, 2)
    if D is not None:
        D.barrier()
    check(lib.xtg_event_record(t0, s_in))
    for k in range(steps):
        one(k)
    check(lib.xtg_event_record(t1, s_out))
    check(lib.xtg_event_sync(t1))
    check(lib.xtg_device_sync())
    ms = ev_ms(lib, t0, t1) / steps
    if D is not None:
        ms = D.max(ms)
    check(lib.xtg_stream_destroy(s_in))
    check(lib.xtg_stream_destroy(s_out))
    return {"value": round(algo_bytes / (ms / 1e3) / 1e9, 3), "unit": "GB/s",
            "h2d_bytes_per_step": int(sum(n for _, n in hin.bufs)),
            "d2h_bytes_per_step": int(sum(n for _, n in hout.bufs)), "ms_per_step": round(ms, 4), "steps": steps,
            "mode": "3 streams (copy in / kernels / copy out), 2 device buffer sets"}


def scaled_err(got, ref, scale):
    """max |got - ref| / scale over the elements (scale > 0)."""
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    return float(np.max(np.abs(got - ref) / scale)) if got.size else 0.0


# ------------------------------------------------------------------------------ C0: plain small
C0_SHAPE = (2048, 2048)
C0_WORKLOAD = ("plain small: A float32 (2048,2048) U[-1,1], b float32 (2048,) N(0,1) seed 0; "
               "E = A*b + exp(-A*A) into a new array; r = sum(E, {1})")
F32_EPS = 2.0 ** -24


def make_c0_inputs():
    g = np.random.default_rng(0)
    A = g.uniform(-1, 1, C0_SHAPE).astype(np.float32)
    b = g.standard_normal(C0_SHAPE[1]).astype(np.float32)
    return A, b


def c0_bytes() -> dict:
    n, m = C0_SHAPE
    return {"assign": 4 * (2 * n * m + m), "reduce": 4 * (n * m + n), "fused_floor": 4 * (2 * n * m + m + n)}


class C0Step:
    """C0 as prebuilt C-ABI calls: xtg_assign of A*b + exp(-A*A) into E, then
    xtg_reduce(sum, {1}) of E into r (the reference's two statements); with
    fused=True instead one xtg_assign_reduce call, which writes E and r in one
    pass of the row kernel."""

    def __init__(self, A, b, fused=False):
        import xtensor_gb300 as xg
        from xtensor_gb300 import ops
        from xtensor_gb300.device import DeviceArray
        from xtensor_gb300.expr import lower
        self.lib = xg.lib()
        dA, db = DeviceArray.from_numpy(A), DeviceArray.from_numpy(b)
        E = DeviceArray.empty(A.shape, "float32")
        r = DeviceArray.empty((A.shape[0],), "float32")
        self.dev_in, self.dev_out = [dA, db], [E, r]
        e_E, k1 = lower(dA * db + xg.exp(-dA * dA))
        e_r, k2 = lower(E)
        rd = ops.make_desc("sum", axes=[1])
        o_E, o_r = E.xtg_array(), r.xtg_array()
        self.keep = [e_E, k1, e_r, k2, rd, o_E, o_r]
        L = self.lib
        if fused:
            self.calls = [("fused", lambda st: L.xtg_assign_reduce(C.byref(e_E), C.byref(o_E), C.byref(rd),
                                                                   C.byref(o_r), st))]
        else:
            self.calls = [
                ("assign", lambda st: L.xtg_assign(C.byref(e_E), C.byref(o_E), st)),
                ("reduce", lambda st: L.xtg_reduce(C.byref(e_r), C.byref(rd), C.byref(o_r), st)),
            ]

    def launch(self, stream, events=None):
        from xtensor_gb300._ffi import check
        for i, (_, fn) in enumerate(self.calls):
            if events is not None:
                check(self.lib.xtg_event_record(events[i], stream))
            check(fn(stream))
        if events is not None:
            check(self.lib.xtg_event_record(events[len(self.calls)], stream))


def c0_section(args, stream):
    """C0 (2048, 2048): the inputs (16 MiB) fit in L2, so a 256 MiB memset
    flushes L2 before every timed step; CUDA events bracket the C0 kernels
    only.  Parity: E and r against the CPU port of the reference's loops,
    run on the same inputs."""
    import xtensor_gb300 as xg
    from xtensor_gb300._ffi import check
    from xtensor_gb300.device import DeviceArray
    lib = xg.lib()
    A, b = make_c0_inputs()
    step = C0Step(A, b)
    fstep = C0Step(A, b, fused=True)
    flush = DeviceArray.empty((64 << 20,), "float32")  # 256 MiB > L2
    for _ in range(max(3, args.warmup)):
        step.launch(stream)
        fstep.launch(stream)
    check(lib.xtg_stream_sync(stream))
    K = max(args.steps, 20)
    peak, peak_kind = peaks()
    nb = c0_bytes()
    nb["fused"] = nb["fused_floor"]

    def timed(st_):
        evs = [ev_create(lib, len(st_.calls) + 1) for _ in range(K)]
        l0 = xg.jit_stats()["launches"]
        for k in range(K):
            check(lib.xtg_memset(flush.ptr, k & 0xFF, flush.nbytes, stream))
            st_.launch(stream, evs[k])
        check(lib.xtg_stream_sync(stream))
        l1 = xg.jit_stats()["launches"]
        per = [sum(ev_ms(lib, evs[k][i], evs[k][i + 1]) for k in range(K)) / K for i in range(len(st_.calls))]
        return per, int(l1 - l0)
    per, launches = timed(step)
    fper, flaunches = timed(fstep)
    per_kernel = {nm: {"ms": round(t, 5), "GB/s": round(nb[nm] / (t / 1e3) / 1e9, 1),
                       "frac": round(nb[nm] / (t / 1e3) / 1e9 / peak, 3)}
                  for (nm, _), t in list(zip(step.calls, per)) + list(zip(fstep.calls, fper))}
    two_ms, fused_ms = sum(per), sum(fper)
    total = nb["assign"] + nb["reduce"]
    E_gpu, r_gpu = step.dev_out[0].to_numpy(), step.dev_out[1].to_numpy()
    E_f, r_f = fstep.dev_out[0].to_numpy(), fstep.dev_out[1].to_numpy()
    out = {
        "workload": C0_WORKLOAD, "value": round(nb["fused"] / (fused_ms / 1e3) / 1e9, 1), "unit": "GB/s",
        "ms_per_step": round(fused_ms, 5), "steps": K, "algorithmic_bytes_per_step": nb["fused"],
        "form": "one xtg_assign_reduce launch (E and r in one pass); the two-call form (xtg_assign, then "
                "xtg_reduce of E) is timed beside it",
        "two_calls": {"ms_per_step": round(two_ms, 5), "algorithmic_bytes_per_step": total,
                      "GB/s": round(total / (two_ms / 1e3) / 1e9, 1), "gpu_launches": launches},
        "fused_equals_two_calls_bitwise": bool(E_f.tobytes() == E_gpu.tobytes() and r_f.tobytes() == r_gpu.tobytes()),
        "l2": "inputs (16 MiB) fit in L2: a 256 MiB memset before every step flushes it (not timed)",
        "per_kernel": per_kernel, "gpu_launches": flaunches,
        "roofline": {"bound": "hbm", "kernel": "fused", "peak": peak, "unit": "GB/s",
                     "achieved": per_kernel["fused"]["GB/s"], "frac": per_kernel["fused"]["frac"],
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                     "note": "below 2^26 elements: launch-bound (a few microseconds per kernel at peak)"},
    }
    if not args.no_cpu:
        L = port_lib()
        n, m = C0_SHAPE
        E_p = np.empty(C0_SHAPE, np.float32)
        r_p = np.empty((n,), np.float32)
        ts = []
        while len(ts) < 5 and sum(ts) < 10.0:
            t0 = time.perf_counter()
            L.bl_c0_assign(A.ctypes.data, b.ctypes.data, E_p.ctypes.data, n, m)
            L.bl_c0_sum(E_p.ctypes.data, r_p.ctypes.data, n, m)
            ts.append(time.perf_counter() - t0)
        best = min(ts[1:]) if len(ts) > 1 else ts[0]
        out["cpu_baseline"] = {"value": round(nb["fused"] / best / 1e9, 3), "unit": "GB/s", "cores": cores(),
                               "kind": "port", "sample": f"full workload, best of {len(ts) - 1 if len(ts) > 1 else 1} "
                               f"after a warm-up (compiled port of the reference's loops, OpenMP {cores()} threads)"}
        # parity against the port (the reference's computation, pinned to the oracle)
        Ad = A.astype(np.float64)
        scale = np.abs(Ad * b) + np.exp(-Ad * Ad)
        Ex = E_p.astype(np.float64)
        exact_r = Ex.sum(1)
        absr = np.abs(Ex).sum(1)
        e_E = scaled_err(E_f, E_p, scale)
        e_r = float(np.max(np.abs(r_f - exact_r) / absr))
        env = np.abs(r_p.astype(np.float64) - exact_r) + 1e-6 * absr
        r_gpu = r_f
        out["parity"] = {
            "against": "CPU port of the reference's loops (oracle/xt_baseline.c, pinned to the oracle), same inputs",
            "E_max_err_over_scale": e_E, "E_bound": 4 * F32_EPS,
            "r_max_err_vs_fp64_over_sum_abs": e_r, "r_bound": 1e-6,
            "r_within_reference_envelope": bool((np.abs(r_gpu - r_p) <= env).all()),
            "ok": bool(e_E <= 4 * F32_EPS and e_r <= 1e-6 and (np.abs(r_gpu - r_p) <= env).all()),
        }
    if not args.no_e2e:
        sets = [fstep, C0Step(A, b, fused=True)]
        hin = PinnedHost(lib, [A, b])
        hout = PinnedHost.empty(lib, [o.nbytes for o in fstep.dev_out])
        out["e2e"] = pipelined_e2e(lib, sets, hin, hout, stream, max(20, args.steps), nb["fused"])
        hin.free()
        hout.free()
    return out


# ------------------------------------------------------------------------------ C2: precision
C2_N = 1 << 28
C2_OPS = ("sum", "mean", "variance", "norm_l2")
C2_WORKLOAD = ("precision: 2^28-element float32 and bf16 arrays of sign-random lognormal(0,2) values, seed 2; "
               "sum/mean/variance/norm_l2 with compensated FP32 accumulation; int32 U[-2^20,2^20] summed to int64")


def make_c2_inputs():
    g = np.random.default_rng(2)
    mag = g.lognormal(0.0, 2.0, C2_N).astype(np.float32)
    sign = g.integers(0, 2, C2_N, dtype=np.int8) * 2 - 1
    x = mag * sign.astype(np.float32)
    del mag, sign
    bf = f32_to_bf16_bits(x)
    i = np.random.default_rng(2).integers(-(1 << 20), (1 << 20) + 1, C2_N, dtype=np.int32)
    return x, bf, i


class C2Step:
    """C2 as prebuilt C-ABI calls: for float32 and bfloat16, one xtg_reduce
    each of sum, mean, variance and norm_l2 over all axes; the int32 ->
    int64 sum."""

    def __init__(self, x, bf, ints):
        import xtensor_gb300 as xg
        from xtensor_gb300 import ops
        from xtensor_gb300.device import DeviceArray
        from xtensor_gb300.expr import lower
        self.lib = L = xg.lib()
        dx = DeviceArray.from_numpy(x)
        db = DeviceArray.from_numpy(bf, "bfloat16")
        di = DeviceArray.from_numpy(ints)
        self.dev_in = [dx, db, di]
        self.dev_out, self.calls, self.keep = [], [], []
        for tag, d, ops_ in (("f32", dx, C2_OPS), ("bf16", db, C2_OPS), ("i32", di, ("sum",))):
            e, k = lower(d)
            for op in ops_:
                kw = {"acc_dtype": "int64"} if tag == "i32" else {}
                shape, dt = ops.reduce_shape(op, d, **kw)
                o = DeviceArray.empty(shape, dt)
                rd = ops.make_desc(op, **kw)
                oa = o.xtg_array()
                self.keep += [e, k, rd, oa]
                self.dev_out.append(o)
                self.calls.append((f"{op}_{tag}", d.nbytes + o.nbytes,
                                   lambda st, e=e, rd=rd, oa=oa: L.xtg_reduce(C.byref(e), C.byref(rd), C.byref(oa), st)))

    def launch(self, stream, events=None):
        from xtensor_gb300._ffi import check
        for i, (_, _, fn) in enumerate(self.calls):
            if events is not None:
                check(self.lib.xtg_event_record(events[i], stream))
            check(fn(stream))
        if events is not None:
            check(self.lib.xtg_event_record(events[len(self.calls)], stream))

    def results(self) -> dict:
        return {nm: o.to_numpy() for (nm, _, _), o in zip(self.calls, self.dev_out)}


class C2Moments(C2Step):
    """C2's float32 and bfloat16 statistics as one xtg_reduce_moments call
    each (sum, mean, variance, norm_l2 from one read of the input)."""

    def __init__(self, step: C2Step):
        from xtensor_gb300 import ops
        from xtensor_gb300._ffi import Array
        from xtensor_gb300.device import DeviceArray
        from xtensor_gb300.expr import lower
        self.lib = L = step.lib
        self.dev_out, self.calls, self.keep, self.names = [], [], [], []
        for tag, d in (("f32", step.dev_in[0]), ("bf16", step.dev_in[1])):
            e, k = lower(d)
            outs = []
            for op in C2_OPS:
                shape, dt = ops.reduce_shape(op, d)
                outs.append(DeviceArray.empty(shape, dt))
            rd = ops.make_desc("variance")
            arrs = [o.xtg_array() for o in outs]
            self.keep += [e, k, rd, arrs]
            self.dev_out += outs
            self.names += [f"{op}_{tag}" for op in C2_OPS]
            self.calls.append((f"moments_{tag}", d.nbytes + sum(o.nbytes for o in outs),
                               lambda st, e=e, rd=rd, a=arrs: L.xtg_reduce_moments(
                                   C.byref(e), C.byref(rd), *[C.byref(x) for x in a], st)))

    def results(self) -> dict:
        return {nm: o.to_numpy() for nm, o in zip(self.names, self.dev_out)}


def c2_exact(x, bf):
    """FP64 values of the C2 reductions over the (rounded) data."""
    res = {}
    for tag, v in (("f32", x), ("bf16", (bf.astype(np.uint32) << 16).view(np.float32))):
        s = 0.0
        sa = 0.0
        q = 0.0
        for k in range(0, C2_N, 1 << 25):
            c = v[k:k + (1 << 25)].astype(np.float64)
            s += float(c.sum())
            sa += float(np.abs(c).sum())
            q += float((c * c).sum())
        m = s / C2_N
        var = 0.0
        for k in range(0, C2_N, 1 << 25):
            c = v[k:k + (1 << 25)].astype(np.float64) - m
            var += float((c * c).sum())
        res[tag] = {"sum": s, "sum_abs": sa, "mean": m, "variance": var / C2_N, "norm_l2": float(np.sqrt(q))}
    return res


def c2_section(args, stream):
    """C2 at 2^28 elements: each input (1 GiB float32, 512 MiB bfloat16,
    1 GiB int32) is larger than L2, so no flush is needed; CUDA events
    bracket every reduction.  Accuracy of every result against FP64."""
    import xtensor_gb300 as xg
    from xtensor_gb300._ffi import check
    lib = xg.lib()
    x, bf, ints = make_c2_inputs()
    step = C2Step(x, bf, ints)
    for _ in range(max(3, args.warmup)):
        step.launch(stream)
    check(lib.xtg_stream_sync(stream))
    K = args.steps
    evs = [ev_create(lib, len(step.calls) + 1) for _ in range(K)]
    l0 = xg.jit_stats()["launches"]
    for k in range(K):
        step.launch(stream, evs[k])
    check(lib.xtg_stream_sync(stream))
    l1 = xg.jit_stats()["launches"]
    per = [sum(ev_ms(lib, evs[k][i], evs[k][i + 1]) for k in range(K)) / K for i in range(len(step.calls))]
    peak, peak_kind = peaks()
    per_kernel = {nm: {"ms": round(t, 4), "GB/s": round(nb / (t / 1e3) / 1e9, 1),
                       "frac": round(nb / (t / 1e3) / 1e9 / peak, 3)} for (nm, nb, _), t in zip(step.calls, per)}
    total = sum(nb for _, nb, _ in step.calls)
    ms = sum(per)
    dom = max(per_kernel, key=lambda k: per_kernel[k]["ms"])
    got = step.results()
    # the same statistics from one pass per input (xtg_reduce_moments)
    mstep = C2Moments(step)
    for _ in range(max(3, args.warmup)):
        mstep.launch(stream)
    check(lib.xtg_stream_sync(stream))
    mevs = [ev_create(lib, len(mstep.calls) + 1) for _ in range(K)]
    for k in range(K):
        mstep.launch(stream, mevs[k])
    check(lib.xtg_stream_sync(stream))
    mper = [sum(ev_ms(lib, mevs[k][i], mevs[k][i + 1]) for k in range(K)) / K for i in range(len(mstep.calls))]
    mgot = mstep.results()
    one_pass = {
        "form": "one xtg_reduce_moments call per input: sum, mean, variance and norm_l2 from one read",
        "algorithmic_bytes_per_step": sum(nb for _, nb, _ in mstep.calls),
        "ms_per_step": round(sum(mper), 4),
        "per_kernel": {nm: {"ms": round(t, 4), "GB/s": round(nb / (t / 1e3) / 1e9, 1),
                            "frac": round(nb / (t / 1e3) / 1e9 / peak, 3)} for (nm, nb, _), t in zip(mstep.calls, mper)},
        "separate_calls_ms": round(sum(per[:2 * len(C2_OPS)]), 4),
        "results_equal_separate_calls_bitwise": all(mgot[k].tobytes() == got[k].tobytes() for k in mgot),
    }
    ex = c2_exact(x, bf)
    acc = {}
    for tag in ("f32", "bf16"):
        for op in C2_OPS:
            g_ = float(got[f"{op}_{tag}"])
            e_ = ex[tag][op]
            acc[f"{op}_{tag}"] = abs(g_ - e_) / abs(e_)
        acc[f"sum_{tag}_vs_sum_abs"] = abs(float(got[f"sum_{tag}"]) - ex[tag]["sum"]) / ex[tag]["sum_abs"]
    exact_i = int(np.sum(ints, dtype=np.int64))
    out = {
        "workload": C2_WORKLOAD, "value": round(total / (ms / 1e3) / 1e9, 1), "unit": "GB/s",
        "ms_per_step": round(ms, 4), "steps": K, "algorithmic_bytes_per_step": total,
        "l2": "inputs (1 GiB / 512 MiB / 1 GiB) larger than L2: no flush",
        "per_kernel": per_kernel, "gpu_launches": int(l1 - l0),
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": per_kernel[dom]["GB/s"], "peak": peak,
                     "unit": "GB/s", "frac": per_kernel[dom]["frac"],
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"},
        "one_pass": one_pass,
        "accuracy": {"rel_err_vs_fp64": {k: float(f"{v:.3e}") for k, v in acc.items()}, "bound": 1e-6,
                     "int32_to_int64_sum_bit_exact": int(got["sum_i32"]) == exact_i,
                     "ok": bool(max(acc.values()) <= 1e-6 and int(got["sum_i32"]) == exact_i)},
    }
    if not args.no_cpu:
        L = port_lib()
        t0 = time.perf_counter()
        port = {}
        for tag, arr in (("f32", x), ("bf16", bf)):
            for op in C2_OPS:
                port[f"{op}_{tag}"] = float(getattr(L, f"bl_stat_{op}_{tag}")(arr.ctypes.data, C2_N))
        port["sum_i32"] = int(L.bl_sum_i32_i64(ints.ctypes.data, C2_N))
        sec = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": round(total / sec / 1e9, 3), "unit": "GB/s", "cores": 1, "kind": "port",
                               "sample": "full workload once (compiled port of the reference's lazy reducers: one "
                                         "sequential single-threaded pass per reduction, as the reference runs them)"}
        out["accuracy"]["reference_rel_err_vs_fp64"] = {
            k: float(f"{abs(port[k] - ex[k.split('_')[-1]][k.rsplit('_', 1)[0]]) / abs(ex[k.split('_')[-1]][k.rsplit('_', 1)[0]]):.3e}")
            for k in port if not k.endswith("i32")}
        out["accuracy"]["reference_int64_sum_equal"] = port["sum_i32"] == int(got["sum_i32"])
    if not args.no_e2e:
        del got
        sets = [step, C2Step(x, bf, ints)]
        hin = PinnedHost(lib, [x, bf, ints])
        hout = PinnedHost.empty(lib, [o.nbytes for o in step.dev_out])
        out["e2e"] = pipelined_e2e(lib, sets, hin, hout, stream, max(3, min(args.steps, 10)), total)
        hin.free()
        hout.free()
    return out


# ------------------------------------------------------------------------------ C1 parity
def c1_parity(step, cpu_outs, x32, x64) -> dict:
    """The GPU results of the C1 step against the CPU port's results on the
    same inputs (the port is pinned to the oracle bit for bit): transpose,
    amax and argmax must be bit-identical; the normalisation must lie within
    rel * scale of the FP64 value (rel 4e-6 for float32, 1e-12 for float64,
    scale = (|x| + |mean|) / sqrt(var + eps)) and within the reference's own
    error envelope around it."""
    res = {"against": "CPU port of the reference's loops (oracle/xt_baseline.c, pinned to the oracle), same inputs"}
    ok = True
    for x in (x32, x64):
        s = x.dtype.itemsize
        tag = "f32" if s == 4 else "f64"
        t, y, am, ai = (o.to_numpy() for o in step.dev_out[0 if s == 4 else 1])
        po = cpu_outs[s]
        r = {"transpose_bit_exact": bool(np.array_equal(t.view(np.uint8), po["t"].view(np.uint8))),
             "amax_bit_exact": bool(np.array_equal(am.view(np.uint8), po["am"].view(np.uint8))),
             "argmax_bit_exact": bool(np.array_equal(ai, po["ai"]))}
        rel = 4e-6 if s == 4 else 1e-12
        worst, worst_ref, inside = 0.0, 0.0, True
        for i in range(0, SHAPE[0], 16):
            xd = x[i:i + 16].astype(np.float64)
            m = xd.mean(-1, keepdims=True)
            sd = np.sqrt(xd.var(-1, keepdims=True) + 1e-5)
            exact = (xd - m) / sd
            scale = (np.abs(xd) + np.abs(m)) / sd
            g_ = y[i:i + 16].astype(np.float64)
            p_ = po["y"][i:i + 16].astype(np.float64)
            worst = max(worst, float(np.max(np.abs(g_ - exact) / scale)))
            worst_ref = max(worst_ref, float(np.max(np.abs(p_ - exact) / scale)))
            inside = inside and bool((np.abs(g_ - p_) <= np.abs(p_ - exact) + rel * scale).all())
        r.update(normalize_max_err_over_scale=worst, normalize_bound=rel, reference_max_err_over_scale=worst_ref,
                 normalize_within_reference_envelope=inside)
        r["ok"] = bool(r["transpose_bit_exact"] and r["amax_bit_exact"] and r["argmax_bit_exact"]
                       and worst <= rel and inside)
        ok = ok and r["ok"]
        res[tag] = r
    res["ok"] = ok
    return res


PLAIN_LOOP_C = r"""
#include "xtg.h"
/* The plain form of a C/C++ call site that evaluates sum(A * v + C, {1})
   instance after instance: one xtg_reduce call (one launch per expression)
   per instance, in order, expressions lowered beforehand. */
xtg_status plain_reduce_loop(int n, const xtg_expr* const* e, const xtg_reduce_desc* rd,
                             const xtg_array* const* o, xtg_stream s, int reps) {
    for (int r = 0; r < reps; ++r)
        for (int i = 0; i < n; ++i) {
            xtg_status st = xtg_reduce(e[i], rd, o[i], s);
            if (st != XTG_OK) return st;
        }
    return XTG_OK;
}
"""


def plain_loop_lib():
    """Compile (once) and load the C loop above against libxtg.so."""
    import hashlib
    bdir = ROOT / "xtensor_gb300" / "_build"
    bdir.mkdir(parents=True, exist_ok=True)
    tag = hashlib.sha1(PLAIN_LOOP_C.encode()).hexdigest()[:10]
    so = bdir / f"libbench_plain_{tag}.so"
    libdir = ROOT / "xtensor_gb300" / "lib"
    if not so.exists():
        src = bdir / f"bench_plain_{tag}.c"
        src.write_text(PLAIN_LOOP_C)
        subprocess.check_call(["gcc", "-O2", "-shared", "-fPIC", "-I", str(ROOT / "include"), str(src), "-o", str(so),
                               "-L", str(libdir), "-lxtg", f"-Wl,-rpath,{libdir}"])
    L = C.CDLL(str(so))
    L.plain_reduce_loop.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
    L.plain_reduce_loop.restype = C.c_int
    return L


C3_WORKLOAD = ("batching: 4096 float32 instances rows U{1..4096} cols U{16..2048} seed 3; "
               "per instance sum(A*v + C, {1}), E never materialised")


def c3_section(args):
    """Batching configuration: 4096 float32 instances, rows U{1..4096},
    cols U{16..2048}, seed 3; per instance sum(A * v + C, {1}) (E is never
    materialised).  Plain = one xtg_reduce call per instance from a C loop
    (expressions lowered beforehand, so only the C-ABI calls are timed);
    batched = one persistent launch; graph = the same launch replayed from a
    CUDA graph.  The instances total 68.9 GB, far larger than L2."""
    import xtensor_gb300 as xg
    from xtensor_gb300._ffi import check
    from xtensor_gb300 import ops
    from xtensor_gb300.batch import Batch, fill_random
    from xtensor_gb300.device import DeviceArray, Stream
    from xtensor_gb300.expr import lower

    lib = xg.lib()
    n_inst = args.instances
    g = np.random.default_rng(3)
    rows = g.integers(1, 4097, n_inst)
    cols = g.integers(16, 2049, n_inst)
    inst = []
    for i in range(n_inst):
        r, c = int(rows[i]), int(cols[i])
        A = fill_random(DeviceArray.empty((r, c), "float32"), "uniform", -1, 1, 3_000_000 + 3 * i)
        v = fill_random(DeviceArray.empty((c,), "float32"), "normal", 0, 1, 3_000_000 + 3 * i + 1)
        Cm = fill_random(DeviceArray.empty((r, c), "float32"), "uniform", -1, 1, 3_000_000 + 3 * i + 2)
        out = DeviceArray.empty((r,), "float32")
        inst.append((A, v, Cm, out))
    check(lib.xtg_device_sync())
    total = int(sum(4 * (2 * int(r) * int(c) + int(c) + int(r)) for r, c in zip(rows, cols)))
    s = Stream()
    rd = ops.make_desc("sum", axes=[1])
    keep, eptr, optr = [], [], []
    for A, v, Cm, out in inst:
        ex, k = lower(A * v + Cm)
        o = out.xtg_array()
        keep += [ex, k, o]
        eptr.append(C.addressof(ex))
        optr.append(C.addressof(o))
    E_arr = (C.c_void_p * n_inst)(*eptr)
    O_arr = (C.c_void_p * n_inst)(*optr)
    PL = plain_loop_lib()

    def plain(reps=1):
        check(PL.plain_reduce_loop(n_inst, E_arr, C.addressof(rd), O_arr, s.handle, reps))

    def timed(fn, reps):
        fn()
        s.sync()
        t0, t1 = ev_create(lib, 2)
        check(lib.xtg_event_record(t0, s.handle))
        w0 = time.perf_counter()
        for _ in range(reps):
            fn()
        check(lib.xtg_event_record(t1, s.handle))
        check(lib.xtg_event_sync(t1))
        wall = (time.perf_counter() - w0) / reps
        return max(ev_ms(lib, t0, t1) / reps, wall * 1e3)

    plain_ms = timed(plain, max(3, min(args.steps, 5)))
    plain_out = [o.to_numpy() for *_, o in inst[:16]]
    A0, v0, C0_, o0 = inst[0]
    b = Batch(A0 * v0 + C0_, reduce="sum")
    for A, v, Cm, out in inst:
        b.add(A * v + Cm, out)
    t_build = time.perf_counter()
    b.build(autotune=not args.no_tune, stream=s)
    t_build = time.perf_counter() - t_build
    l0 = xg.jit_stats()["launches"]
    batch_ms = timed(lambda: b.run(s), args.steps)
    b.capture(s)
    graph_ms = timed(lambda: b.replay(s), args.steps)
    l1 = xg.jit_stats()["launches"]
    # accuracy on a sample: FP64 of the same device data, and batched vs plain
    worst, worst_plain = 0.0, 0.0
    for k in range(16):
        A, v, Cm, out = inst[k]
        E = A.to_numpy().astype(np.float64) * v.to_numpy().astype(np.float64) + Cm.to_numpy().astype(np.float64)
        got = out.to_numpy().astype(np.float64)
        sa = np.abs(E).sum(1)
        worst = max(worst, float(np.max(np.abs(got - E.sum(1)) / sa)))
        worst_plain = max(worst_plain, float(np.max(np.abs(plain_out[k] - E.sum(1)) / sa)))
    peak, peak_kind = peaks()
    info = b.info()
    b.close()
    gbs = total / (graph_ms / 1e3) / 1e9
    cpu = None
    if not args.no_cpu:
        # the port of the reference's lazy row sum over a bounded sample: the
        # first 192 instances (about 3 GB), copied to the host, best of 2
        Lp = port_lib()
        k_s = min(192, n_inst)
        host = [(A.to_numpy(), v.to_numpy(), Cm.to_numpy(), np.empty(out.shape, np.float32))
                for A, v, Cm, out in inst[:k_s]]
        sb = int(sum(4 * (2 * a.size + vv.size + o.size) for a, vv, _, o in host))

        def port_run():
            for a, vv, cm, o in host:
                Lp.bl_c3_rowsum_f32(a.ctypes.data, vv.ctypes.data, cm.ctypes.data, o.ctypes.data, a.shape[0],
                                    a.shape[1])
        port_run()
        ts = []
        for _ in range(2):
            t0 = time.perf_counter()
            port_run()
            ts.append(time.perf_counter() - t0)
        dev_err = max(float(np.max(np.abs(out.to_numpy().astype(np.float64) - o.astype(np.float64)) /
                                   (np.abs(a.astype(np.float64) * vv.astype(np.float64)) +
                                    np.abs(cm.astype(np.float64))).sum(1)))
                      for (a, vv, cm, o), (_, _, _, out) in zip(host, inst))
        cpu = {"value": round(sb / min(ts) / 1e9, 3), "unit": "GB/s", "cores": cores(), "kind": "port",
               "sample": f"the first {k_s} of the {n_inst} instances ({sb / 1e9:.2f} GB), best of 2 after a warm-up "
                         f"(compiled port of the reference's lazy row sum, OpenMP {cores()} threads over rows)",
               "gpu_vs_port_max_err_over_sum_abs": dev_err}
    return {
        "workload": C3_WORKLOAD, "instances": n_inst, "algorithmic_bytes": total, "elements": int(info["elements"]),
        "value": round(gbs, 1), "unit": "GB/s", "l2": "68.9 GB of operands, far larger than L2: no flush",
        "plain_ms": round(plain_ms, 3), "batched_ms": round(batch_ms, 3), "graph_ms": round(graph_ms, 3),
        "plain_GBps": round(total / (plain_ms / 1e3) / 1e9, 1),
        "batched_GBps": round(total / (batch_ms / 1e3) / 1e9, 1),
        "speedup_graph_vs_plain": round(plain_ms / graph_ms, 2),
        "plain_form": "a C loop of xtg_reduce calls, one launch per instance (expressions lowered beforehand)",
        "roofline": {"bound": "hbm", "kernel": "k_batch_rowreduce", "achieved": round(gbs, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(gbs / peak, 4),
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"},
        "tuning": {k: info[k] for k in ("group_lanes", "tile_elems", "ctas_per_sm", "tuned", "tiles")},
        "build_s": round(t_build, 2), "gpu_launches": int(l1 - l0),
        "accuracy": {"max_rel_err_vs_fp64_sum_abs": worst, "plain_max_rel_err_vs_fp64_sum_abs": worst_plain,
                     "bound": 1e-6, "sample": "first 16 instances"},
        "cpu_baseline": cpu,
        "e2e": None,
        "e2e_note": "operands are generated and kept on the device by definition of the batching workload",
    }


def run_c3(args):
    import xtensor_gb300 as xg
    xg.init(0)
    r = c3_section(args)
    line = {"metric": "batched throughput GB/s (uneven-shape mix) vs plain one-launch-per-expression",
            "unit": "GB/s", "value": r["value"], "higher_is_better": True, "n_gpus": 1, "steps": args.steps,
            "dtype": "f32", "data": "synthetic (device generator, seed 3)",
            "config": {"workload": r["workload"], "algorithmic_bytes": r["algorithmic_bytes"]}, **{
                k: v for k, v in r.items() if k not in ("value", "unit", "workload")}}
    print(json.dumps(line))
    return 0


def run_scan(args):
    """Accumulator workload (the scan row next to the hot path): x float32 and
    float64 (256, 512, 1024) N(0,1) seed 1 and int32 U[-1000, 1000]:
    cumsum along axis 2 (row scan: 131072 rows of 1024), along axis 1 (column
    scan) and over the flattening (tile scan: one row of 2^27), through the C
    ABI with inputs resident in HBM.  Algorithmic bytes: one read of the input
    and one write of the result per call.  CPU baseline: the compiled port of
    the reference's accumulate loop (oracle/xt_baseline.c bl_cumsum_*, OpenMP
    over independent outer rows) on the same arrays."""
    import xtensor_gb300 as xg
    from xtensor_gb300._ffi import check
    from xtensor_gb300.device import DeviceArray
    from xtensor_gb300.expr import lower
    lib = xg.lib()
    st = C.c_void_p()
    check(lib.xtg_stream_create(C.byref(st)))
    stream = st.value
    g = np.random.default_rng(1)
    xs = {"f32": g.standard_normal(SHAPE, dtype=np.float32), "f64": g.standard_normal(SHAPE, dtype=np.float64),
          "i32": g.integers(-1000, 1001, SHAPE, dtype=np.int32)}
    calls, keep = [], []
    for nm, x in xs.items():
        dx = DeviceArray.from_numpy(x)
        e, k = lower(dx)
        keep += [dx, e, k]
        for ax, tag in ((2, "rows"), (1, "cols"), (None, "flat")):
            if nm == "i32" and tag != "cols":
                continue
            oshape = SHAPE if ax is not None else (N,)
            out = DeviceArray.empty(oshape, x.dtype)
            o = out.xtg_array()
            keep += [out, o]
            calls.append((f"cumsum_{tag}_{nm}", 2 * x.nbytes,
                          lambda e=e, o=o, ax=ax: lib.xtg_accumulate(C.byref(e), 0, 0 if ax is None else 1,
                                                                      0 if ax is None else ax, -1, C.byref(o), stream)))
    for _ in range(args.warmup):
        for _, _, fn in calls:
            check(fn())
    check(lib.xtg_stream_sync(stream))
    evs = [ev_create(lib, len(calls) + 1) for _ in range(args.steps)]
    clocks = Clocks(0)
    clocks.start()
    time.sleep(0.15)
    l0 = xg.jit_stats()["launches"]
    for k in range(args.steps):
        for i, (_, _, fn) in enumerate(calls):
            check(lib.xtg_event_record(evs[k][i], stream))
            check(fn())
        check(lib.xtg_event_record(evs[k][len(calls)], stream))
    check(lib.xtg_stream_sync(stream))
    l1 = xg.jit_stats()["launches"]
    clk = clocks.stop()
    per = [sum(ev_ms(lib, evs[k][i], evs[k][i + 1]) for k in range(args.steps)) / args.steps for i in range(len(calls))]
    step_ms = sum(per)
    total = sum(b for _, b, _ in calls)
    peak, peak_kind = peaks()
    per_kernel = {nm: {"ms": round(t, 4), "GB/s": round(b / (t / 1e3) / 1e9, 1), "frac": round(b / (t / 1e3) / 1e9 / peak, 3)}
                  for (nm, b, _), t in zip(calls, per)}
    dom = int(np.argmax(per))
    cpu = None
    if not args.no_cpu:
        from oracle.oracle import SO, lib as olib  # noqa: F401
        olib()
        L = C.CDLL(str(SO))
        fns = {"f32": L.bl_cumsum_f32, "f64": L.bl_cumsum_f64, "i32": L.bl_cumsum_i32}
        t_cpu, b_cpu = 0.0, 0
        for nm, b, _ in calls:
            tag, dt = nm.split("_")[1], nm.split("_")[2]
            x = xs[dt]
            r = np.empty_like(x)
            ax = {"rows": 2, "cols": 1, "flat": -1}[tag]
            args_c = (x.ctypes.data_as(C.c_void_p), r.ctypes.data_as(C.c_void_p), C.c_int64(SHAPE[0]),
                      C.c_int64(SHAPE[1]), C.c_int64(SHAPE[2]), C.c_int(ax))
            fns[dt](*args_c)
            t0 = time.perf_counter()
            fns[dt](*args_c)
            t_cpu += time.perf_counter() - t0
            b_cpu += b
        cpu = {"value": round(b_cpu / t_cpu / 1e9, 3), "unit": "GB/s", "cores": cores(), "kind": "port",
               "sample": "full workload, one timed run after one warm-up (compiled port of the reference's "
                         f"accumulate loop, OpenMP {cores()} threads over outer rows; the flattened scan is sequential)"}
    line = {
        "metric": "HBM GB/s (frac of roofline) of xt::cumsum through the C ABI", "unit": "GB/s",
        "value": round(total / (step_ms / 1e3) / 1e9, 3), "higher_is_better": True, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(step_ms, 4), "scaling": "weak",
        "vs_baseline": None, "dtype": "f32,f64,i32", "data": "synthetic",
        "config": {"workload": "accumulators: cumsum of x (256,512,1024) f32/f64 along axis 2, axis 1 and flattened; "
                               "int32 along axis 1", "algorithmic_bytes_per_step": total,
                   "l2": "inputs larger than L2: no flush"},
        "roofline": {"bound": "hbm", "kernel": calls[dom][0], "achieved": per_kernel[calls[dom][0]]["GB/s"],
                     "peak": peak, "unit": "GB/s", "frac": per_kernel[calls[dom][0]]["frac"], "traffic": None,
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"},
        "per_kernel": per_kernel, "cpu_baseline": cpu, "e2e": None, "gpu_launches": int(l1 - l0), "clocks": clk,
    }
    print(json.dumps(line))
    return 0


def run_views(args):
    """Writes and reads through views on x float32 (256, 512, 1024) N(0,1)
    seed 1, through the C ABI with operands resident in HBM:
    masked_view(x, m) += 1.5 (m bool, ~50% true); filter(y, y > 1) (read,
    1-D result); filtration(z, y > 1) *= 0.5; index_view(x, idx) read and
    += 1 for 2^24 random distinct coordinates.  Algorithmic bytes: what the
    call must read and write (the mask, the selected elements, the
    coordinates and the gathered values; the filter reads x once for the
    condition and once for the values)."""
    import xtensor_gb300 as xg
    from xtensor_gb300 import ops
    from xtensor_gb300._ffi import check
    from xtensor_gb300.device import DeviceArray
    lib = xg.lib()
    g = np.random.default_rng(1)
    x = g.standard_normal(SHAPE, dtype=np.float32)
    m = g.random(SHAPE) < 0.5
    nidx = 1 << 24
    flat = g.choice(N, nidx, replace=False)
    idx = np.stack(np.unravel_index(flat, SHAPE), 1).astype(np.int64)
    dx, dm, di = DeviceArray.from_numpy(x), DeviceArray.from_numpy(m), DeviceArray.from_numpy(idx)
    # the filters select on y (never written), so the selected count is fixed
    dy, dz = DeviceArray.from_numpy(x), DeviceArray.from_numpy(x)
    sel = int((x > 1).sum())
    gout = DeviceArray.empty((nidx,), "float32")
    fout = DeviceArray.empty((sel,), "float32")
    calls = [
        ("masked_add", N * 4 * 2 + N, lambda: ops.masked_assign(dx, dm, 1.5, "+=")),
        ("filter_read", 2 * N * 4 + sel * 4, lambda: ops.filter(dy, dy > 1, out=fout)),
        ("filtration_mul", N * 4 + 2 * sel * 4, lambda: ops.filter_assign(dz, dy > 1, 0.5, "*=")),
        ("index_read", nidx * 24 + 2 * nidx * 4, lambda: ops.index_view(dx, di, out=gout)),
        ("index_add", nidx * 24 + 2 * nidx * 4, lambda: ops.index_assign(dx, di, 1.0, "+=")),
    ]
    for _ in range(args.warmup):
        for _, _, fn in calls:
            fn()
    check(lib.xtg_device_sync())
    evs = [ev_create(lib, len(calls) + 1) for _ in range(args.steps)]
    for k in range(args.steps):
        for i, (_, _, fn) in enumerate(calls):
            check(lib.xtg_event_record(evs[k][i], None))
            fn()
        check(lib.xtg_event_record(evs[k][len(calls)], None))
    check(lib.xtg_device_sync())
    per = [sum(ev_ms(lib, evs[k][i], evs[k][i + 1]) for k in range(args.steps)) / args.steps for i in range(len(calls))]
    peak, peak_kind = peaks()
    total = sum(b for _, b, _ in calls)
    step_ms = sum(per)
    per_kernel = {nm: {"ms": round(t, 4), "GB/s": round(b / (t / 1e3) / 1e9, 1), "frac": round(b / (t / 1e3) / 1e9 / peak, 3)}
                  for (nm, b, _), t in zip(calls, per)}
    dom = int(np.argmax(per))
    print(json.dumps({
        "metric": "HBM GB/s (frac of roofline) of reads and writes through index / filter / masked views",
        "unit": "GB/s", "value": round(total / (step_ms / 1e3) / 1e9, 3), "higher_is_better": True, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(step_ms, 4), "dtype": "f32",
        "data": "synthetic", "config": {"workload": "views on x f32 (256,512,1024): masked +=, filter, filtration *=, "
                                                    "index_view read / += over 2^24 coordinates",
                                        "algorithmic_bytes_per_step": total, "selected": sel},
        "roofline": {"bound": "hbm", "kernel": calls[dom][0], "achieved": per_kernel[calls[dom][0]]["GB/s"],
                     "peak": peak, "unit": "GB/s", "frac": per_kernel[calls[dom][0]]["frac"],
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"},
        "per_kernel": per_kernel,
    }))
    return 0


def c4_pool(n_templates, seed=4):
    """Request templates of the serving mix: kinds of the four configurations,
    element counts log-uniform in [1e3, 1e8], dtypes float32/float64/int32 at
    50/25/25 %, operands generated on the device (seeded)."""
    import xtensor_gb300 as xg
    from xtensor_gb300 import ops
    from xtensor_gb300.batch import fill_random
    from xtensor_gb300.device import DeviceArray
    from xtensor_gb300.server import ARGREDUCE, ASSIGN, REDUCE

    g = np.random.default_rng(seed)
    pool = []
    sd = [0]

    def arr(shape, dt):
        sd[0] += 1
        a = DeviceArray.empty(shape, dt)
        if dt == "int32":
            return fill_random(a, "integers", -1000, 1000, 4_000_000 + sd[0])
        return fill_random(a, "normal", 0, 1, 4_000_000 + sd[0])

    for i in range(n_templates):
        n = int(round(10 ** g.uniform(3, 8)))
        dt = ["float32", "float32", "float64", "int32"][g.integers(0, 4)]
        kinds = ["c0", "c1", "c2", "c3"] if dt != "int32" else ["c1", "c2", "c3"]
        k = kinds[g.integers(0, len(kinds))]
        cols = int(min(4096, max(16, 2 ** round(np.log2(max(n, 16) ** 0.5)))))
        rows = max(1, n // cols)
        if k == "c0":
            A, b = arr((rows, cols), dt), arr((cols,), dt)
            e = A * b + xg.exp(-A * A)
            if g.integers(0, 2):
                pool.append((ASSIGN, None, e, None, (rows, cols), [A, b], 2 * rows * cols + cols))
            else:
                pool.append((REDUCE, "sum", e, [1], (rows,), [A, b], rows * cols + cols + rows))
        elif k == "c3":
            A, v, Cm = arr((rows, cols), dt), arr((cols,), dt), arr((rows, cols), dt)
            pool.append((REDUCE, "sum", A * v + Cm, [1], (rows,), [A, v, Cm], 2 * rows * cols + cols + rows))
        elif k == "c2":
            x = arr((n,), dt)
            op = "sum" if dt == "int32" else ["sum", "mean", "variance", "norm_l2"][g.integers(0, 4)]
            pool.append((REDUCE, op, x, None, (), [x], n + 1))
        else:
            d2 = min(1024, cols)
            d1 = max(1, min(512, rows))
            d0 = max(1, n // (d1 * d2))
            x = arr((d0, d1, d2), dt)
            sub = ["transpose", "normalize", "amax", "argmax"][g.integers(0, 4)] if dt != "int32" else \
                ["transpose", "amax", "argmax"][g.integers(0, 3)]
            m = d0 * d1 * d2
            if sub == "transpose":
                pool.append((ASSIGN, None, x.transpose((2, 0, 1)), None, (d2, d0, d1), [x], 2 * m))
            elif sub == "normalize":
                pool.append((ASSIGN, None, (x - xg.rmean(x)) / xg.sqrt(xg.rvar(x) + 1e-5), None, (d0, d1, d2), [x], 2 * m))
            elif sub == "amax":
                pool.append((REDUCE, "amax", x, [0, 2], (d1,), [x], m + d1))
            else:
                pool.append((ARGREDUCE, "argmax", x, 1, (d0, d2), [x], m + d0 * d2))
    return pool


C4_WORKLOAD = ("serving: Poisson arrivals, kinds of configs 0-3, elements log-uniform 1e3..1e8, "
               "float32/float64/int32 50/25/25, operands device-resident")


def c4_section(args):
    """Serving: Poisson arrivals (rate sweep, `repeats` runs per rate with
    fresh arrival draws) of requests drawn from the pool; served (xtg_server:
    admission by HBM budget, continuous batching, multi-stream overlap) vs
    plain (each request evaluated synchronously in arrival order, one launch
    per expression).  Latency = completion - arrival."""
    import xtensor_gb300 as xg
    from xtensor_gb300._ffi import check
    from xtensor_gb300 import ops
    from xtensor_gb300.device import DeviceArray, Stream
    from xtensor_gb300.server import ARGREDUCE, ASSIGN, REDUCE, Server

    lib = xg.lib()
    t_setup = time.perf_counter()
    pool = c4_pool(args.templates)
    outs = []
    for kind, op, e, axes, shape, keep, elems in pool:
        if kind == ASSIGN:
            outs.append(DeviceArray.empty(shape, xg.expr_dtype(e)))
        elif kind == ARGREDUCE:
            outs.append(DeviceArray.empty(shape, "int64"))
        else:
            sh, code = ops.reduce_shape(op, e, axes=axes)
            outs.append(DeviceArray.empty(sh, code))
    check(lib.xtg_device_sync())

    def req_bytes(i):
        kind, op, e, axes, shape, keep, elems = pool[i]
        return sum(a.nbytes for a in keep) + outs[i].nbytes

    dispatch_threads = args.dispatch_threads
    xg.set_option("server.dispatch_threads", dispatch_threads)
    srv = Server(streams=8, max_inflight=128, batch_min_group=2)
    reqs = [srv.request(kind, e, outs[i], op=op, axes=axes, arg_axis=axes)[0] for i, (kind, op, e, axes, *_r) in
            enumerate(pool)]
    s = Stream()

    def plain_one(i):
        kind = pool[i][0]
        r = reqs[i]
        if kind == ASSIGN:
            check(lib.xtg_assign(C.byref(r.expr), C.byref(r.out), s.handle))
        elif kind == REDUCE:
            check(lib.xtg_reduce(C.byref(r.expr), C.byref(r.rd), C.byref(r.out), s.handle))
        else:
            check(lib.xtg_argreduce(C.byref(r.expr), r.arg_op, r.has_axis, r.axis, C.byref(r.out), s.handle))
        s.sync()

    # warm-up: every template once through both paths (kernel compilation)
    for i in range(len(pool)):
        plain_one(i)
    ids = []
    for i in range(len(pool)):
        rid = C.c_uint64()
        check(srv.L.xtg_server_submit(srv.h, C.byref(reqs[i]), C.byref(rid)))
        ids.append(rid.value)
    for rid in ids:
        srv.wait(rid, 600000)
    srv.reset_stats()
    t_setup = time.perf_counter() - t_setup

    g = np.random.default_rng(44)
    rates = [float(r) for r in args.rates.split(",")]
    results = []
    l0 = xg.jit_stats()["launches"]
    for rate in rates:
        runs = []
        for rep in range(args.repeats):
            n = args.requests
            arrivals = np.cumsum(g.exponential(1.0 / rate, n))
            picks = g.integers(0, len(pool), n)
            total_bytes = sum(req_bytes(int(p)) for p in picks)
            lat = []
            t0 = time.perf_counter()
            for a, p in zip(arrivals, picks):
                while time.perf_counter() - t0 < a:
                    pass
                plain_one(int(p))
                lat.append((time.perf_counter() - t0 - a) * 1e3)
            plain_wall = time.perf_counter() - t0
            srv.reset_stats()
            ids = []
            t0 = time.perf_counter()
            for a, p in zip(arrivals, picks):
                while time.perf_counter() - t0 < a:
                    pass
                rid = C.c_uint64()
                check(srv.L.xtg_server_submit(srv.h, C.byref(reqs[int(p)]), C.byref(rid)))
                ids.append(rid.value)
            submit_s = time.perf_counter() - t0
            srv.drain(600000)
            served_wall = time.perf_counter() - t0
            for rid in ids:
                srv.wait(rid, 600000)
            st = srv.stats()
            lat.sort()
            runs.append({
                "plain": {"p50_ms": round(lat[n // 2], 3), "p99_ms": round(lat[int(0.99 * (n - 1))], 3),
                          "req_s": round(n / plain_wall, 1), "GB/s": round(total_bytes / plain_wall / 1e9, 1)},
                "served": {"p50_ms": round(st["p50_ms"], 3), "p99_ms": round(st["p99_ms"], 3),
                           "req_s": round(n / served_wall, 1), "GB/s": round(total_bytes / served_wall / 1e9, 1),
                           "batched_requests": st["batched_requests"], "batch_launches": st["batch_launches"],
                           "waves": st["waves"],
                           # the rate the client managed to submit at (the offered rate when the
                           # arrival loop kept up with its schedule)
                           "submitted_req_s": round(n / submit_s, 1),
                           # host time the dispatch threads spent launching, per second of the run and thread
                           "dispatch_busy": round(st["dispatch_ms"] / (served_wall * 1e3 * dispatch_threads), 3)},
            })
        med = lambda arm, k: float(np.median([r[arm][k] for r in runs]))  # noqa: E731
        results.append({
            "rate_req_s": rate, "requests": args.requests, "repeats": len(runs), "runs": runs,
            "median": {arm: {k: med(arm, k) for k in ("p50_ms", "p99_ms", "req_s")} for arm in ("plain", "served")},
            "served_over_plain_req_s_min": round(min(r["served"]["req_s"] / r["plain"]["req_s"] for r in runs), 3),
            "batched_share": round(sum(r["served"]["batched_requests"] for r in runs) / (len(runs) * args.requests), 4),
        })
    l1 = xg.jit_stats()["launches"]
    srv.close()
    best = max(results, key=lambda r: r["median"]["served"]["req_s"])
    return {
        "workload": C4_WORKLOAD, "templates": len(pool), "pool_bytes": int(sum(req_bytes(i) for i in range(len(pool)))),
        "value": best["median"]["served"]["req_s"], "unit": "req/s", "setup_s": round(t_setup, 1),
        "served_ge_plain_every_run": all(r["served_over_plain_req_s_min"] >= 1.0 for r in results),
        "dispatch_threads": dispatch_threads,
        "sweep": results, "gpu_launches": int(l1 - l0),
        "e2e": None, "e2e_note": "operands are device-resident by definition of the serving workload",
    }


def run_c4(args):
    import xtensor_gb300 as xg
    xg.init(0)
    r = c4_section(args)
    line = {"metric": "served p50/p99 ms vs plain (Poisson mix of the four expression kinds)", "unit": "req/s",
            "value": r["value"], "higher_is_better": True, "n_gpus": 1, "dtype": "f32,f64,int32",
            "data": "synthetic (device generator, seed 4)",
            "config": {"workload": r["workload"], "templates": r["templates"], "pool_bytes": r["pool_bytes"]},
            **{k: v for k, v in r.items() if k not in ("value", "unit", "workload", "templates", "pool_bytes")}}
    print(json.dumps(line))
    return 0


CHUNK_WORKLOAD = ("chunked arrays: x float32 (256,512,1024) N(0,1) seed 1 as xt::chunked_array in chunks "
                  "(64,256,1024) and, with edge chunks, (100,200,1000); a = x*2+1 into the chunks, "
                  "b = a read back dense, sum(a, {2}), sum(a)")


def run_chunked(args):
    """The chunked-array workload as its own line."""
    import xtensor_gb300 as xg
    xg.init(0)
    r = chunked_section(args)
    line = {"metric": "HBM GB/s (frac of roofline) of chunked-array assignment, read-back and reductions",
            "unit": "GB/s", "value": r["value"], "higher_is_better": True, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": CHUNK_WORKLOAD, "algorithmic_bytes_per_step": r["algorithmic_bytes_per_step"],
                       "l2": r["l2"]},
            **{k: v for k, v in r.items() if k not in ("value", "unit", "ms_per_step", "workload",
                                                       "algorithmic_bytes_per_step", "l2")}}
    print(json.dumps(line))
    return 0


def chunked_section(args):
    """Chunked arrays (xt::xchunked_array) over device chunks: assignment of
    an expression into every chunk (one K12 launch), reading the chunked
    array into a dense one (K12), sum over the last axis and the full sum.  Chunk shapes: whole chunks
    (64, 256, 1024) = 8 chunks of 64 MiB, and (100, 200, 1000) = 3 x 3 x 2
    chunks of 80 MB with edge chunks on every axis.  Algorithmic bytes: the
    array's 512 MiB read and 512 MiB written for the assignment and the
    read-back; 512 MiB read (+ the result) for the sums.  CPU baseline: the
    compiled port of the reference's chunk-by-chunk assignment, element-wise
    read-back and lazy sum over the last axis (oracle/xt_baseline.c
    bl_chunked_*, pinned to the oracle).  The chunked arrays sit in one slab,
    so each sum is one strided reduction per class of equal chunks; the same
    sums over the dense array are timed beside them (`dense`)."""
    import xtensor_gb300 as xg
    from xtensor_gb300._ffi import check
    from xtensor_gb300.chunked import ChunkedArray, chunked_reduce
    from xtensor_gb300.device import DeviceArray
    lib = xg.lib()
    g = np.random.default_rng(1)
    x = g.standard_normal(SHAPE, dtype=np.float32)
    dx = DeviceArray.from_numpy(x)
    nb = x.nbytes
    peak, peak_kind = peaks()
    res = {}
    calls = []
    for tag, cs in (("whole", (64, 256, 1024)), ("edges", (100, 200, 1000))):
        a = ChunkedArray(SHAPE, cs, "float32")
        dense = DeviceArray.empty(SHAPE, "float32")
        s2 = DeviceArray.empty(SHAPE[:2], "float32")
        s0 = DeviceArray.empty((), "float32")
        calls += [
            (f"assign_{tag}", 2 * nb, lambda a=a: a.assign(dx * 2.0 + 1.0)),
            (f"read_{tag}", 2 * nb, lambda a=a, d=dense: a.to_device(d)),
            (f"sum2_{tag}", nb + s2.nbytes, lambda a=a, o=s2: chunked_reduce("sum", a, axes=[2], out=o)),
            (f"sum_{tag}", nb + 4, lambda a=a, o=s0: chunked_reduce("sum", a, out=o)),
        ]
        res[tag] = (a, dense, s2, s0, cs)
    for _ in range(max(3, args.warmup)):
        for _, _, fn in calls:
            fn()
    check(lib.xtg_device_sync())
    K = args.steps
    evs = [ev_create(lib, len(calls) + 1) for _ in range(K)]
    l0 = xg.jit_stats()["launches"]
    for k in range(K):
        for i, (_, _, fn) in enumerate(calls):
            check(lib.xtg_event_record(evs[k][i], None))
            fn()
        check(lib.xtg_event_record(evs[k][len(calls)], None))
    check(lib.xtg_device_sync())
    l1 = xg.jit_stats()["launches"]
    per = [sum(ev_ms(lib, evs[k][i], evs[k][i + 1]) for k in range(K)) / K for i in range(len(calls))]
    per_kernel = {nm: {"ms": round(t, 4), "GB/s": round(b / (t / 1e3) / 1e9, 1), "frac": round(b / (t / 1e3) / 1e9 / peak, 3)}
                  for (nm, b, _), t in zip(calls, per)}
    total = sum(b for _, b, _ in calls)
    ms = sum(per)
    dom = max(per_kernel, key=lambda k: per_kernel[k]["ms"])
    # the same sums over the dense array, for comparison (not in the totals)
    from xtensor_gb300 import ops
    s2d, s0d = DeviceArray.empty(SHAPE[:2], "float32"), DeviceArray.empty((), "float32")
    dcalls = [("sum2", nb + s2d.nbytes, lambda: ops.reduce("sum", dx, [2], out=s2d)),
              ("sum", nb + 4, lambda: ops.reduce("sum", dx, None, out=s0d))]
    for _ in range(3):
        for _, _, fn in dcalls:
            fn()
    check(lib.xtg_device_sync())
    devs = [ev_create(lib, len(dcalls) + 1) for _ in range(K)]
    for k in range(K):
        for i, (_, _, fn) in enumerate(dcalls):
            check(lib.xtg_event_record(devs[k][i], None))
            fn()
        check(lib.xtg_event_record(devs[k][len(dcalls)], None))
    check(lib.xtg_device_sync())
    dms = [sum(ev_ms(lib, devs[k][i], devs[k][i + 1]) for k in range(K)) / K for i in range(len(dcalls))]
    dense_ref = {nm: {"ms": round(t, 4), "GB/s": round(b / (t / 1e3) / 1e9, 1), "frac": round(b / (t / 1e3) / 1e9 / peak, 3)}
                 for (nm, b, _), t in zip(dcalls, dms)}
    # parity against an FP64 evaluation of the same values (the port is
    # checked against the oracle by the tests)
    parity = {}
    want = x * np.float32(2.0) + np.float32(1.0)
    wd = want.astype(np.float64)
    sa2 = np.abs(wd).sum(2)
    for tag, (a, dense, s2, s0, cs) in res.items():
        parity[tag] = {"read_back_bit_exact": bool(np.array_equal(dense.to_numpy(), want)),
                       "sum2_max_err_over_sum_abs": float(np.max(np.abs(s2.to_numpy() - wd.sum(2)) / sa2)),
                       "sum_err_over_sum_abs": float(abs(float(s0.to_numpy()) - float(wd.sum())) / float(np.abs(wd).sum()))}
    parity["ok"] = all(v["read_back_bit_exact"] and v["sum2_max_err_over_sum_abs"] <= 1e-6 and
                       v["sum_err_over_sum_abs"] <= 1e-6 for v in parity.values())
    cpu = None
    if not args.no_cpu:
        from oracle.oracle import SO, lib as olib
        olib()
        L = C.CDLL(str(SO))
        PP = C.POINTER(C.c_void_p)
        L.bl_chunked_axpb_f32.argtypes = [C.c_void_p, PP, C.c_void_p, C.c_void_p, C.c_float, C.c_float]
        L.bl_chunked_read_f32.argtypes = [PP, C.c_void_p, C.c_void_p, C.c_void_p]
        L.bl_chunked_sum2_f32.argtypes = [PP, C.c_void_p, C.c_void_p, C.c_void_p]
        cs = (64, 256, 1024)
        n = int(np.prod([(d + c - 1) // c for d, c in zip(SHAPE, cs)]))
        chunks = [np.empty(cs, np.float32) for _ in range(n)]
        tab = (C.c_void_p * n)(*[c.ctypes.data for c in chunks])
        d = np.array(SHAPE, np.int64)
        c = np.array(cs, np.int64)
        dense_h = np.empty(SHAPE, np.float32)
        s2_h = np.empty(SHAPE[:2], np.float32)
        t0 = time.perf_counter()
        L.bl_chunked_axpb_f32(x.ctypes.data, tab, d.ctypes.data, c.ctypes.data, 2.0, 1.0)
        L.bl_chunked_read_f32(tab, dense_h.ctypes.data, d.ctypes.data, c.ctypes.data)
        L.bl_chunked_sum2_f32(tab, s2_h.ctypes.data, d.ctypes.data, c.ctypes.data)
        t1 = time.perf_counter()
        cb = 2 * nb + 2 * nb + nb
        cpu = {"value": round(cb / (t1 - t0) / 1e9, 3), "unit": "GB/s", "cores": cores(), "kind": "port",
               "sample": f"assignment, read-back and sum over axis 2 in chunks {cs}, once (compiled port of the "
                         f"reference's chunk-by-chunk assignment and element-wise access, OpenMP {cores()} threads)"}
    return {
        "workload": CHUNK_WORKLOAD, "value": round(total / (ms / 1e3) / 1e9, 3), "unit": "GB/s",
        "ms_per_step": round(ms, 4), "steps": K, "algorithmic_bytes_per_step": total,
        "l2": "512 MiB arrays, larger than L2: no flush",
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": per_kernel[dom]["GB/s"], "peak": peak, "unit": "GB/s",
                     "frac": per_kernel[dom]["frac"], "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"},
        "per_kernel": per_kernel, "dense": dense_ref, "parity": parity, "cpu_baseline": cpu, "e2e": None,
        "e2e_note": "the chunked arrays are device containers by definition of the workload",
        "gpu_launches": int(l1 - l0),
    }


def run_section(args, name):
    """One sub-result of the default line as its own line (profiling runs)."""
    import xtensor_gb300 as xg
    from xtensor_gb300._ffi import check
    global C2_N
    C2_N = 1 << args.c2_log2n
    xg.init(0)
    st = C.c_void_p()
    check(xg.lib().xtg_stream_create(C.byref(st)))
    r = (c0_section if name == "c0" else c2_section)(args, st.value)
    print(json.dumps({"metric": METRIC, "workload": name, **r, **({"elements": C2_N} if name == "c2" else {})}))
    return 0


def _npy_dir(need: int) -> str:
    import shutil
    import tempfile
    for d in ("/dev/shm", tempfile.gettempdir()):
        try:
            if os.path.isdir(d) and shutil.disk_usage(d).free > 3 * need:
                return tempfile.mkdtemp(prefix="xtg_npy_", dir=d)
        except OSError:
            continue
    return tempfile.mkdtemp(prefix="xtg_npy_")


def run_npy(args):
    """.npy I/O workload (xt::dump_npy / xt::load_npy): x float32
    (256, 512, 1024) N(0,1) seed 1, 512 MiB.  Per step: dump_npy(path, x)
    from device memory; load_npy(path) into a row-major device array; the same
    values in a Fortran-order file loaded into a row-major array (reordered on
    the device); load_npy of the in-memory file image (pageable bytes).  The
    files sit in the page cache (tmpfs when it has room).  Bytes per call: the
    array's 512 MiB.  Timer: host wall clock (each call returns once the
    bytes have landed).  The link bound beside it: one cudaMemcpyAsync of the
    same bytes from / to pinned host memory, timed here.  CPU baseline: the
    reference's own load / dump path (one read into a heap buffer / one
    write), compiled port in oracle/xt_baseline.c, single thread as the
    reference's stream I/O."""
    import shutil
    import xtensor_gb300 as xg
    from xtensor_gb300 import ops
    from xtensor_gb300._ffi import check
    from xtensor_gb300.device import DeviceArray
    lib = xg.lib()
    g = np.random.default_rng(1)
    x = g.standard_normal(SHAPE, dtype=np.float32)
    nb = x.nbytes
    d = _npy_dir(2 * nb)
    fc, ff = os.path.join(d, "x_c.npy"), os.path.join(d, "x_f.npy")
    try:
        dx = DeviceArray.from_numpy(x)
        np.save(ff, np.asfortranarray(x))
        out = DeviceArray.empty(SHAPE, "float32")
        ops.dump_npy(fc, dx)
        img = open(fc, "rb").read()
        calls = [
            ("dump_npy_file", lambda: ops.dump_npy(fc, dx)),
            ("load_npy_file", lambda: ops.load_npy(fc, "float32", out=out)),
            ("load_npy_fortran_file", lambda: ops.load_npy(ff, "float32", out=out)),
            ("load_npy_image", lambda: ops.load_npy(img, "float32", out=out)),
        ]
        for _ in range(args.warmup):
            for _, fn in calls:
                fn()
        check(lib.xtg_device_sync())
        # link bound: pinned host memory <-> device, same bytes
        hp = C.c_void_p()
        check(lib.xtg_host_alloc(C.byref(hp), nb))
        link = {}
        for nm, kind, dst, src in (("h2d", 1, out.ptr, hp.value), ("d2h", 2, hp.value, dx.ptr)):
            ts = []
            for _ in range(3):
                t0 = time.perf_counter()
                check(lib.xtg_memcpy(dst, src, nb, kind, None))
                check(lib.xtg_stream_sync(None))
                ts.append(time.perf_counter() - t0)
            link[nm] = nb / min(ts) / 1e9
        check(lib.xtg_host_free(hp))
        # host ceiling of the load side: 16 threads (as the library's ring)
        # reading the file from the page cache into host memory, no device
        # copy (os.preadv drops the GIL)
        from concurrent.futures import ThreadPoolExecutor
        hb = np.ones(nb, dtype=np.uint8)
        fd = os.open(fc, os.O_RDONLY)
        try:
            ch = 8 << 20
            offs = list(range(0, nb, ch))

            def rd(o):
                os.preadv(fd, [memoryview(hb)[o:o + min(ch, nb - o)]], 128 + o)
            with ThreadPoolExecutor(16) as ex:
                ts = []
                for _ in range(3):
                    t0 = time.perf_counter()
                    list(ex.map(rd, offs))
                    ts.append(time.perf_counter() - t0)
            host_read = nb / min(ts) / 1e9
        finally:
            os.close(fd)
        del hb
        clocks = Clocks(0)
        clocks.start()
        time.sleep(0.15)
        l0 = xg.jit_stats()["launches"]
        per = {nm: [] for nm, _ in calls}
        for _ in range(args.steps):
            for nm, fn in calls:
                t0 = time.perf_counter()
                fn()
                per[nm].append(time.perf_counter() - t0)
        check(lib.xtg_device_sync())
        l1 = xg.jit_stats()["launches"]
        clk = clocks.stop()
        np.testing.assert_array_equal(out.to_numpy()[::7, ::5, ::3], x[::7, ::5, ::3])
        med = {nm: statistics.median(v) for nm, v in per.items()}
        step_s = sum(med.values())
        per_call = {}
        for nm, t in med.items():
            bound = link["d2h"] if nm.startswith("dump") else link["h2d"]
            per_call[nm] = {"ms": round(t * 1e3, 2), "GB/s": round(nb / t / 1e9, 2),
                            "frac_of_link": round(nb / t / 1e9 / bound, 3)}
            if nm.startswith("load"):
                per_call[nm]["frac_of_host_read"] = round(nb / t / 1e9 / host_read, 3)
        dom = max(med, key=med.get)
        cpu = None
        if not args.no_cpu:
            from oracle.oracle import SO, lib as olib
            olib()
            L = C.CDLL(str(SO))
            L.bl_npy_load.restype = C.c_int64
            L.bl_npy_load.argtypes = [C.c_char_p, C.POINTER(C.c_void_p)]
            L.bl_npy_save.argtypes = [C.c_char_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64]
            L.bl_free.argtypes = [C.c_void_p]
            hdr = ops.npy_format_header("float32", SHAPE)
            t_load, t_save = [], []
            for _ in range(3):
                p = C.c_void_p()
                t0 = time.perf_counter()
                n = L.bl_npy_load(fc.encode(), C.byref(p))
                t_load.append(time.perf_counter() - t0)
                assert n == nb
                t0 = time.perf_counter()
                assert L.bl_npy_save(fc.encode(), hdr, len(hdr), p, nb) == 0
                t_save.append(time.perf_counter() - t0)
                L.bl_free(p)
            tl, tsv = statistics.median(t_load), statistics.median(t_save)
            cpu = {"value": round(2 * nb / (tl + tsv) / 1e9, 3), "unit": "GB/s", "cores": 1, "kind": "port",
                   "sample": "full 512 MiB file, median of 3 (port of the reference's load_npy read into a heap "
                             f"buffer: {nb / tl / 1e9:.2f} GB/s; dump_npy write: {nb / tsv / 1e9:.2f} GB/s)"}
        gbs = len(calls) * nb / step_s / 1e9
        line = {
            "metric": "GB/s of array bytes through xt::dump_npy / xt::load_npy (file or host image <-> device)",
            "unit": "GB/s", "value": round(gbs, 3), "higher_is_better": True, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(step_s * 1e3, 3), "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "npy: dump_npy and load_npy of x f32 (256,512,1024) (C-order file, Fortran-order "
                                   "file into a row-major array, in-memory image)", "bytes_per_call": nb,
                       "files": "page cache (" + d.rsplit("/", 1)[0] + ")", "timer": "host wall clock, median"},
            "roofline": {"bound": "link", "kernel": dom, "achieved": per_call[dom]["GB/s"],
                         "peak": round(link["d2h"] if dom.startswith("dump") else link["h2d"], 1), "unit": "GB/s",
                         "frac": per_call[dom]["frac_of_link"], "traffic": None,
                         "peak_source": "measured here: one cudaMemcpyAsync of the same bytes to / from pinned host "
                                        f"memory (h2d {link['h2d']:.1f} GB/s, d2h {link['d2h']:.1f} GB/s)",
                         "host_read_gbs": round(host_read, 1),
                         "host_read_source": "16 threads pread of the same file from the page cache into host memory, "
                                             "no device copy (the load side's ceiling below the link)"},
            "per_call": per_call, "cpu_baseline": cpu,
            "e2e": {"value": round(gbs, 3), "unit": "GB/s", "h2d_bytes_per_step": 3 * nb, "d2h_bytes_per_step": nb,
                    "note": "the path is itself host <-> device: value and e2e are the same calls"},
            "gpu_launches": int(l1 - l0), "clocks": clk,
        }
        print(json.dumps(line))
    finally:
        shutil.rmtree(d, ignore_errors=True)
    return 0


def run_blockwise(args):
    """Blockwise reductions of a host array (xt::blockwise::sum / mean):
    x float32 (1024, 1024, 1024) N(0,1) seed 1, 4 GiB in host memory — the
    out-of-core case, where the array lives in host memory and streams
    through HBM in slabs of whole blocks (512 MiB).  Per step:
    blockwise::sum(x, {16, 256, 256}, {0}) (slab dimension reduced: partials
    merged) and blockwise::mean(x, blocks, {1, 2}) (slab dimension kept),
    from pageable memory (page-locked in place for the call), from pageable
    memory through the staging ring, and from pinned memory.  Bytes per
    call: the array's 4 GiB.  Timer: host wall clock (each call returns once
    the input is no longer read; the result is then synchronised).  The link
    bound beside it: one cudaMemcpyAsync of a pinned 512 MiB slab, timed
    here.  CPU baseline: compiled port of the reference's blockwise loop
    (oracle/xt_baseline.c, OpenMP over outputs) on the same array."""
    import xtensor_gb300 as xg
    from xtensor_gb300 import ops
    from xtensor_gb300._ffi import check
    from xtensor_gb300.device import DeviceArray
    lib = xg.lib()
    shape = (1024, 1024, 1024) if not args.shape else SHAPE
    block = (16, 256, 256)
    nb = int(np.prod(shape)) * 4
    x = np.empty(shape, dtype=np.float32)
    g = np.random.default_rng(1)
    for i in range(0, shape[0], 64):
        x[i:i + 64] = g.standard_normal((min(64, shape[0] - i),) + shape[1:], dtype=np.float32)
    hp = C.c_void_p()
    check(lib.xtg_host_alloc(C.byref(hp), nb))
    xp = np.frombuffer((C.c_char * nb).from_address(hp.value), dtype=np.float32).reshape(shape)
    xp[...] = x
    s0 = DeviceArray.empty(shape[1:], "float32")
    m12 = DeviceArray.empty(shape[:1], "float64")

    def call(kind, which):
        src = xp if kind == "pinned" else x
        xg.set_option("blockwise.register_host", 0 if kind == "ring" else 1)
        if which == "sum0":
            ops.blockwise("sum", src, block, [0], out=s0)
        else:
            ops.blockwise("mean", src, block, [1, 2], out=m12)
        check(lib.xtg_device_sync())
    calls = [(f"{w}_{k}", (lambda k=k, w=w: call(k, w))) for k in ("pageable", "ring", "pinned")
             for w in ("sum0", "mean12")]
    for _ in range(args.warmup):
        for _, fn in calls:
            fn()
    # link bound: pinned slab -> device
    slab = 512 << 20
    dbuf = DeviceArray.empty((slab // 4,), "float32")
    ts = []
    for _ in range(3):
        t0 = time.perf_counter()
        check(lib.xtg_memcpy(dbuf.ptr, hp.value, slab, 1, None))
        check(lib.xtg_stream_sync(None))
        ts.append(time.perf_counter() - t0)
    link = slab / min(ts) / 1e9
    clocks = Clocks(0)
    clocks.start()
    time.sleep(0.15)
    l0 = xg.jit_stats()["launches"]
    per = {nm: [] for nm, _ in calls}
    for _ in range(args.steps):
        for nm, fn in calls:
            t0 = time.perf_counter()
            fn()
            per[nm].append(time.perf_counter() - t0)
    l1 = xg.jit_stats()["launches"]
    clk = clocks.stop()
    xg.set_option("blockwise.register_host", 1)
    # correctness against float64 numpy on the same array
    np.testing.assert_allclose(s0.to_numpy()[::97, ::89], x[:, ::97, ::89].sum(0, dtype=np.float64), rtol=1e-4,
                               atol=1e-3)
    np.testing.assert_allclose(m12.to_numpy()[::31], x[::31].mean((1, 2), dtype=np.float64), rtol=1e-6, atol=1e-9)
    check(lib.xtg_host_free(hp))
    del xp
    med = {nm: statistics.median(v) for nm, v in per.items()}
    per_call = {nm: {"ms": round(t * 1e3, 2), "GB/s": round(nb / t / 1e9, 2), "frac_of_link": round(nb / t / 1e9 / link, 3),
                     "all_ms": [round(v * 1e3, 1) for v in per[nm]]}
                for nm, t in med.items()}
    headline = [nm for nm in med if nm.endswith("_pageable")]
    step_s = sum(med[nm] for nm in headline)
    dom = max(headline, key=med.get)
    cpu = None
    if not args.no_cpu:
        from oracle.oracle import SO, lib as olib
        olib()
        L = C.CDLL(str(SO))
        L.bl_blockwise_sum_axis0_f32.argtypes = [C.c_void_p, C.c_void_p] + [C.c_int64] * 4
        L.bl_blockwise_mean_12_f32.argtypes = [C.c_void_p, C.c_void_p] + [C.c_int64] * 5
        o0 = np.empty(shape[1:], np.float32)
        o1 = np.empty(shape[:1], np.float64)
        t_cpu = []
        for _ in range(2):
            t0 = time.perf_counter()
            L.bl_blockwise_sum_axis0_f32(x.ctypes.data, o0.ctypes.data, *shape, block[0])
            L.bl_blockwise_mean_12_f32(x.ctypes.data, o1.ctypes.data, *shape, block[1], block[2])
            t_cpu.append(time.perf_counter() - t0)
        np.testing.assert_allclose(o1[::31], m12.to_numpy()[::31], rtol=1e-6)
        cpu = {"value": round(2 * nb / min(t_cpu) / 1e9, 3), "unit": "GB/s", "cores": cores(), "kind": "port",
               "sample": "full 4 GiB array, both calls, best of 2 (port of the reference's blockwise loop: per-block "
                         f"sums in the plain reducer's order folded in grid order; OpenMP {cores()} threads over outputs)"}
    gbs = len(headline) * nb / step_s / 1e9
    line = {
        "metric": "GB/s of host-resident input reduced by xt::blockwise::sum / mean (streamed through HBM)",
        "unit": "GB/s", "value": round(gbs, 3), "higher_is_better": True, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(step_s * 1e3, 3), "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": "blockwise: sum over axis 0 and mean over axes (1, 2) of x f32 (1024,1024,1024) in "
                               "pageable host memory, blocks (16, 256, 256), 512 MiB slabs", "bytes_per_call": nb,
                   "timer": "host wall clock, median", "l2": "inputs larger than L2: no flush"},
        "roofline": {"bound": "link", "kernel": dom, "achieved": per_call[dom]["GB/s"], "peak": round(link, 1),
                     "unit": "GB/s", "frac": per_call[dom]["frac_of_link"], "traffic": None,
                     "peak_source": "measured here: one cudaMemcpyAsync of a pinned 512 MiB slab to the device"},
        "per_call": per_call, "cpu_baseline": cpu,
        "e2e": {"value": round(gbs, 3), "unit": "GB/s", "h2d_bytes_per_step": len(headline) * nb,
                "d2h_bytes_per_step": 0,
                "note": "the input is host-resident by definition of the workload: value and e2e are the same calls"},
        "gpu_launches": int(l1 - l0), "clocks": clk,
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="xtg", choices=["xtg", "reference"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--shape", default=None, help="profiling only: d0,d1,d2 instead of 256,512,1024")
    ap.add_argument("--c2-log2n", type=int, default=28, help="profiling only: C2 inputs of 2^n elements")
    ap.add_argument("--workload", default="c1",
                    choices=["c1", "c0", "c2", "c3", "c4", "scan", "views", "npy", "blockwise", "chunked"],
                    help="c1: strided/axis work (default, the headline); c3: batching of uneven instances; "
                         "c4: served Poisson request mix; scan: cumsum along rows, columns and flattened")
    ap.add_argument("--instances", type=int, default=4096)
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--templates", type=int, default=256)
    ap.add_argument("--requests", type=int, default=2000)
    ap.add_argument("--rates", default="2000,16000,48000,96000")
    ap.add_argument("--repeats", type=int, default=3, help="c4: runs per offered rate")
    ap.add_argument("--dispatch-threads", type=int, default=1, help="c4: the server's dispatch threads")
    ap.add_argument("--sub", default="c0,c2,c3,c4,chunked",
                    help="sub-results added to the default line (comma list of c0,c2,c3,c4,chunked; 'none' for none)")
    args = ap.parse_args()
    if args.workload in ("c3", "c4"):
        from xtensor_gb300.build import build
        build()
        return run_c3(args) if args.workload == "c3" else run_c4(args)
    if args.shape:
        global SHAPE, N
        SHAPE = tuple(int(v) for v in args.shape.split(","))
        N = SHAPE[0] * SHAPE[1] * SHAPE[2]
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    from xtensor_gb300.build import build
    build()
    if args.workload == "scan":
        return run_scan(args)
    if args.workload == "views":
        return run_views(args)
    if args.workload == "npy":
        return run_npy(args)
    if args.workload == "blockwise":
        return run_blockwise(args)
    if args.workload == "chunked":
        return run_chunked(args)
    if args.workload in ("c0", "c2"):
        return run_section(args, args.workload)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
