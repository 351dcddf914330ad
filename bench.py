"""Benchmark of the fused SoA expression path (large streaming FP64 workload).

One step = the two kernels of the large streaming FP64 workload:
  (a) d = sqrt(a*a+b*b) * log1p(|c|) + rsqrt(1 + d0*d0) over four
      Array<double,3> inputs of 2^26 samples (uniform[-4,4) from Philox seed 7,
      substreams 0..3), one Array<double,3> output: 120 B/sample;
  (b) an in-place Philox normal fill (Box-Muller) of 2^28 doubles (substream 4
      of seed 7): 8 B/sample, write only.
value = algorithmic bytes of both kernels / device time (inputs resident in
HBM, CUDA events on the launching stream). Inputs are larger than L2, so no
flush runs between steps. e2e = the same step through the C-ABI with pinned
host buffers: host->device copies of the four inputs and device->host copies
of both outputs inside the timed region, pipelined over sample blocks
(partition_view) on three streams so uploads, kernels and downloads overlap.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "fused SoA expr HBM GB/s (% of peak); served samples/s, p50/p99 vs plain launch"
UNIT = "GB/s"
N_EXPR = 1 << 26          # samples of the expression kernel
N_FILL = 1 << 28          # doubles of the normal fill
BYTES_EXPR = N_EXPR * 120
BYTES_FILL = N_FILL * 8
WORKLOAD = ("large streaming FP64: 4 x Array<double,3> of 2^26 samples -> "
            "sqrt(a*a+b*b)*log1p(|c|)+rsqrt(1+d0*d0); + Philox normal fill of 2^28 doubles")


def peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_figures():
    """Per-kernel figures from the committed ncu summaries (profiles/ncu_traffic.txt):
    {kernel name: {"kernel": name, "bytes_per_sample": B, "inst_per_sample": I}},
    and under each kind the first line of that kind. Each line reads
    `<kind> <kernel name> <dram bytes/sample> <thread instructions/sample>`."""
    path = os.path.join(REPO, "profiles", "ncu_traffic.txt")
    out = {}
    try:
        for line in open(path):
            f = line.split()
            if len(f) == 4 and not line.startswith("#"):
                rec = {"kernel": f[1], "bytes_per_sample": float(f[2]), "inst_per_sample": float(f[3])}
                out.setdefault(f[0], rec)
                out[f[1]] = rec
    except OSError:
        pass
    return out


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def cpu_leg(steps, warmup, nthreads=0, expr_samples=1 << 23, fill_samples=1 << 25):
    """The reference's CPU algorithm (OpenMP user loop, oracle/ restatement)
    on a bounded sample of the same workload. Returns (GB/s, seconds/step)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import numpy as np
    import pyoracle as po
    nt = nthreads or po.max_threads()
    n = expr_samples
    k7 = po.generator_key(7)
    ins = [po.fill_uniform_f64(po.substream_key(k7, s), -4.0, 4.0, 3, n, nthreads=nt) for s in range(4)]
    key_fill = po.substream_key(k7, 4)
    # outputs allocated and touched once, reused by every step, as the
    # reference's own loop reuses its arrays (first-touch page faults would
    # otherwise be timed with the arithmetic)
    d_out = np.ones_like(ins[0])
    z_out = np.ones((1, fill_samples), dtype=np.float64)
    times = []
    for i in range(max(1, warmup) + steps):
        t0 = time.perf_counter()
        po.cfg2a(*ins, nthreads=nt, out=d_out)
        po.fill_normal_f64(key_fill, 0.0, 1.0, 1, fill_samples, nthreads=nt, out=z_out)
        dt = time.perf_counter() - t0
        if i >= max(1, warmup):
            times.append(dt)
    t = statistics.median(times)
    gbs = (n * 120 + fill_samples * 8) / t / 1e9
    sample = ("expression on %d samples (2^%d) + normal fill of %d doubles (2^%d) per step, median of %d"
              % (n, n.bit_length() - 1, fill_samples, fill_samples.bit_length() - 1, len(times)))
    return gbs, t, nt, sample, (ins, d_out, z_out)


LOWERINGS = {0: "native FP64", 1: "emulated FP64 (double-float)", 3: "FP64-grade (triple-float)"}


def fill_math(math):
    """The fill's lowering for an expression lowering: the normals of the
    double-float draw are within the reference's own normal tolerance (1e-12
    abs+rel, random/detail/Backend.h:44-51), so the FP64-grade step draws them
    that way; native FP64 keeps native draws."""
    return 0 if math == 0 else 1


def check_against_oracle(arrs, d, z, ins, d_ref, z_ref, math, math_z=None):
    """The GPU step's results on the CPU leg's sample against the oracle's
    (same seeded inputs): inputs bit for bit, the expression in units of
    2^-53 of its term scale, the normals in the reference's abs+rel form,
    each against the stated bound of the lowering (aether_gb300.accuracy)."""
    import numpy as np
    from aether_gb300 import accuracy as acc
    n, nz = d_ref.shape[1], z_ref.shape[1]
    same_inputs = all(np.array_equal(x.data[:, :n].cpu().numpy(), r[:, :n]) for x, r in zip(arrs, ins))
    got = d.data[:, :n].cpu().numpy()
    a, b, c, d0 = (r[:, :n] for r in ins)
    scale = np.maximum(np.abs(np.sqrt(a * a + b * b) * np.log1p(np.abs(c))), np.abs(1.0 / np.sqrt(1.0 + d0 * d0)))
    e_expr = acc.term_scale_error_2m53(got, d_ref[:, :n], scale)
    e_norm = acc.abs_rel_error_2m53(z.data[:, :nz].cpu().numpy(), z_ref[:, :nz])
    math_z = fill_math(math) if math_z is None else math_z
    out = {"lowering": LOWERINGS[math], "fill_lowering": LOWERINGS[math_z], "inputs_bit_exact": bool(same_inputs),
           "expr_samples": int(n), "expr_max_err_2m53_of_terms": round(e_expr, 2),
           "normal_samples": int(nz), "normal_max_err_2m53_abs_rel": round(e_norm, 2), "reference_normal_tol": 1e-12}
    nb = acc.NATIVE_NORMAL_BOUND_2M53 if math_z == 0 else acc.EMU_NORMAL_BOUND_2M53
    if math in (0, 3):
        # native and FP64-grade: ulp of the largest term, the unit the native bound is stated in
        e_ulp = acc.term_scale_error_ulp(got, d_ref[:, :n], scale)
        out.update({"expr_max_err_ulp_of_terms": round(e_ulp, 2), "expr_bound_ulp_of_terms": acc.NATIVE_EXPR_ULPS,
                    "normal_bound_2m53": nb,
                    "within_bounds": bool(same_inputs and e_ulp <= acc.NATIVE_EXPR_ULPS and e_norm <= nb)})
    else:
        out.update({"expr_bound_2m53": acc.EMU_EXPR_BOUND_2M53, "normal_bound_2m53": nb,
                    "within_bounds": bool(same_inputs and e_expr <= acc.EMU_EXPR_BOUND_2M53 and e_norm <= nb)})
    return out


def run_reference(args):
    ws, rank, local = dist_env()
    if rank != 0:
        return 0
    gbs, t, nt, sample, _ = cpu_leg(args.steps, args.warmup)
    line = {
        "impl": "reference", "metric": METRIC, "value": round(gbs, 3), "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (Philox seed 7)",
        "config": {"workload": WORKLOAD, "sample": sample, "l2": "inputs larger than L2"},
        "cpu_baseline": {"value": round(gbs, 3), "unit": UNIT, "cores": nt, "kind": "port", "sample": sample},
        "e2e": {"value": round(gbs, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def link_rates(L, dev, h_in, a_in, h_out, a_out, nbytes, s_up, s_down):
    """Host->device, device->host and two-way copy rates (GB/s) of pinned
    buffers through aether_copy, timed with events on the copy streams."""
    import ctypes
    import torch
    up, down = ctypes.c_void_p(s_up.cuda_stream), ctypes.c_void_p(s_down.cuda_stream)
    src_in, dst_in = ctypes.c_void_p(h_in.data_ptr()), ctypes.c_void_p(a_in.data.data_ptr())
    src_out, dst_out = ctypes.c_void_p(a_out.data.data_ptr()), ctypes.c_void_p(h_out.data_ptr())

    def one(do_up, do_down):
        best = None
        for _ in range(3):
            torch.cuda.synchronize()
            e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            e0.record(s_up)
            s_down.wait_event(e0)
            if do_up:
                ag_check(L.aether_copy(1, dev, dst_in, 2, 0, src_in, nbytes, up))
            if do_down:
                ag_check(L.aether_copy(2, 0, dst_out, 1, dev, src_out, nbytes, down))
            e1.record(s_down)
            s_up.wait_event(e1)
            e2.record(s_up)
            e2.synchronize()
            ms = e0.elapsed_time(e2)
            best = ms if best is None else min(best, ms)
        return (int(do_up) + int(do_down)) * nbytes / (best * 1e-3) / 1e9

    return {"h2d_gbs": round(one(True, False), 1), "d2h_gbs": round(one(False, True), 1),
            "both_gbs": round(one(True, True), 1), "bytes_each_way": nbytes}


def h2d_probe(L, dev, h_in, a_in, nbytes, s_up):
    """One host->device copy of nbytes, timed with events on the upload stream (GB/s)."""
    import ctypes
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(s_up)
    ag_check(L.aether_copy(1, dev, ctypes.c_void_p(a_in.data.data_ptr()), 2, 0, ctypes.c_void_p(h_in.data_ptr()),
                           nbytes, ctypes.c_void_p(s_up.cuda_stream)))
    e1.record(s_up)
    e1.synchronize()
    return nbytes / (e0.elapsed_time(e1) * 1e-3) / 1e9


def ag_check(rc):
    from aether_gb300 import _abi
    _abi.check(rc)


def _time_ms(fn, reps=5, warmup=2):
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def secondary_config1(ag):
    """Config 1: d = a + b*c + sin(a)*exp(-c*c), Array<double,3>, 2^20 samples."""
    n = 1 << 20
    g = ag.Generator(42)
    arrs = [ag.Array("f64", (3,), n) for _ in range(3)]
    for k, x in enumerate(arrs):
        ag.assign(x, g.substream(k).uniform(3, -1.0, 1.0))
    a, b, c = (x.view() for x in arrs)
    d = ag.Array("f64", (3,), n)
    e = a + b * c + ag.cwiseSin(a) * ag.cwiseExp((c * c) * (-1.0))
    out = {"samples": n, "bytes_per_sample": 96}
    for name, m in (("native", 0), ("emulated", 1), ("fp64_grade", 3)):
        L = ag.prepare(d, e, math=m, tune=True)
        ms = _time_ms(L, reps=20)
        out[name] = {"ms": round(ms, 4), "gbs": round(n * 96 / (ms * 1e-3) / 1e9, 1)}
    return out


PRECISION_LOG2 = 27


def secondary_config3(ag, n=None):
    """Config 3 (precision form): per-sample dot of two Array<float,8> plus one
    global sum, FP32 storage with float-float working values, against the same
    workload in FP64 storage (best of the native and emulated FP64 lowerings)."""
    import torch
    n = n or (1 << PRECISION_LOG2)
    g = ag.Generator(3)

    def loguniform(arr, k):
        sign = g.substream(2 * k).bernoulli(8, 0.5) * 2.0 - 1.0
        mag = ag.cwiseExp(g.substream(2 * k + 1).uniform(8, -6.0, 6.0) * 2.302585092994046)
        ag.assign(arr, sign * mag)

    x32, y32 = ag.Array("f32", (8,), n), ag.Array("f32", (8,), n)
    loguniform(x32, 0)
    loguniform(y32, 1)
    d32 = ag.Array("f32", (1,), n)
    red32 = torch.zeros(2, dtype=torch.float64, device="cuda")
    L32 = ag.prepare(d32, x32.view().dot(y32.view()), op="setsum", reduce_out=red32, math=2, tune=True)
    ms32 = _time_ms(L32)
    # the same FP32 values widened to FP64 storage
    x64, y64 = ag.Array("f64", (8,), n), ag.Array("f64", (8,), n)
    x64.data.copy_(x32.data)
    y64.data.copy_(y32.data)
    del x32, y32
    d64 = ag.Array("f64", (1,), n)
    red64 = torch.zeros(2, dtype=torch.float64, device="cuda")
    res = {"samples": n, "bytes_per_sample_f32": 68, "bytes_per_sample_f64": 136,
           "ff_ms": round(ms32, 4), "ff_samples_per_s": round(n / (ms32 * 1e-3), 1)}
    best = None
    for name, m in (("f64_native", 0), ("f64_emulated", 1)):
        L64 = ag.prepare(d64, x64.view().dot(y64.view()), op="setsum", reduce_out=red64, math=m, tune=True)
        ms = _time_ms(L64)
        res[name + "_ms"] = round(ms, 4)
        best = ms if best is None else min(best, ms)
    torch.cuda.synchronize()
    # agreement of the two forms on this workload (per-sample and global sum)
    a32 = d32.data[0, :n].double()
    a64 = d64.data[0, :n]
    scale = torch.sum(torch.abs(x64.data[:, :n] * y64.data[:, :n]), dim=0)
    res["max_rel_diff_f32_out_vs_f64"] = float(torch.max(torch.abs(a32 - a64) / scale).item())
    s32, s64 = red32.cpu().tolist(), red64.cpu().tolist()
    res["global_sum_rel_diff"] = abs((s32[0] + s32[1]) - (s64[0] + s64[1])) / abs(s64[0] + s64[1])
    res["speedup_vs_fp64"] = round(best / ms32, 3)
    res["speedup_vs_native_fp64"] = round(res["f64_native_ms"] / ms32, 3)
    res["gbs_ff"] = round(n * 68 / (ms32 * 1e-3) / 1e9, 1)
    del x64, y64, d64, d32
    torch.cuda.empty_cache()
    res["p1_p2"] = config3_expressions(ag, n)
    return res


def config3_expressions(ag, n):
    """Config 3 P1 and P2: the plain fused expression (a up to +-1e5, so the
    sine reduces in FP64) and the large streaming expression (log-uniform
    magnitudes 1e-6..1e6, random sign) on Array<float,3> inputs with
    float-float outputs, against the same FP32 values in FP64 storage; error
    per output relative to native FP64 evaluation (CUDA's FP64 functions)."""
    import torch
    g = ag.Generator(31)

    def loguniform(arr, k):
        sign = g.substream(2 * k).bernoulli(3, 0.5) * 2.0 - 1.0
        ag.assign(arr, sign * ag.cwiseExp(g.substream(2 * k + 1).uniform(3, -6.0, 6.0) * 2.302585092994046))

    def p1(v):
        a, b, c = v
        return a + b * c + ag.cwiseSin(a) * ag.cwiseExp((c * c) * (-1.0))

    def p2(v):
        a, b, c, d0 = v
        return ag.cwiseSqrt(a * a + b * b) * ag.cwiseLog1p(ag.cwiseAbs(c)) + \
            ag.cwiseRsqrt(ag.constant(1.0, (3,)) + d0 * d0)

    out = {}
    for name, fn, k_in, fill, bff, b64 in (("p1", p1, 3, "p1", 60, 96), ("p2", p2, 4, "log", 72, 120)):
        ins = [ag.Array("f32", (3,), n) for _ in range(k_in)]
        for k, x in enumerate(ins):
            if fill == "p1":
                lo, hi = (-1e5, 1e5) if k == 0 else (-1.0, 1.0)
                ag.assign(x, g.substream(40 + k).uniform(3, lo, hi))
            else:
                loguniform(x, 10 + k)
        dff = ag.Array("ff", (3,), n)
        Lff = ag.prepare(dff, fn([x.view() for x in ins]), math=2)
        ms_ff = _time_ms(Lff)
        ins64 = []
        for x in ins:
            y = ag.Array("f64", (3,), n)
            y.data.copy_(x.data)
            ins64.append(y)
        del ins
        d64 = ag.Array("f64", (3,), n)
        best = None
        per = {}
        for m in (0, 1):
            L64 = ag.prepare(d64, fn([x.view() for x in ins64]), math=m)
            ms = _time_ms(L64)
            per[m] = ms
            best = ms if best is None else min(best, ms)
        ag.prepare(d64, fn([x.view() for x in ins64]), math=0)()   # FP64 reference values
        torch.cuda.synchronize()
        v = dff.data[:3, :n].double() + dff.data[3:, :n].double()
        ref = d64.data[:, :n]
        rel = torch.abs(v - ref) / torch.clamp(torch.abs(ref), min=1e-300)
        finite = torch.isfinite(ref)
        out[name] = {"ff_ms": round(ms_ff, 4), "f64_ms": round(best, 4), "speedup_vs_fp64": round(best / ms_ff, 3),
                     "f64_native_ms": round(per[0], 4), "f64_emulated_ms": round(per[1], 4),
                     "speedup_vs_native_fp64": round(per[0] / ms_ff, 3), "kernel": Lff.plan.name,
                     "ff_samples_per_s": round(n / (ms_ff * 1e-3), 1), "bytes_per_sample_ff": bff,
                     "bytes_per_sample_f64": b64, "max_rel_err_vs_fp64": float(torch.max(rel[finite]).item()),
                     "median_rel_err_vs_fp64": float(torch.median(rel[finite]).item())}
        del ins64, d64, dff
        torch.cuda.empty_cache()
    return out


def config4_workload(ag, n_items=4096, median=4096, sigma=1.5, lo=64, hi=1 << 21, seed=4, math=1):
    """Config 4: uneven arrays cycling cross product (Vec3d), quaternion rotate
    and the guarded 3x3 inverse; lognormal sizes."""
    import numpy as np
    rng = np.random.default_rng(seed)
    sizes = np.clip(np.round(rng.lognormal(np.log(median), sigma, n_items)), lo, hi).astype(int)
    g = ag.Generator(seed)
    launches, keep, nbytes = [], [], 0
    for i, n in enumerate(sizes):
        gi = g.substream(i)
        if i % 3 == 0:
            a, b, out = ag.Array("f64", (3,), n), ag.Array("f64", (3,), n), ag.Array("f64", (3,), n)
            ag.assign(a, gi.substream(0).uniform(3, -1.0, 1.0))
            ag.assign(b, gi.substream(1).uniform(3, -1.0, 1.0))
            e, bps, ins = a.view().cross(b.view()), 72, (a, b)
        elif i % 3 == 1:
            q, v, out = ag.Array("f64", (4,), n), ag.Array("f64", (3,), n), ag.Array("f64", (3,), n)
            ag.assign(q, gi.substream(0).uniform(4, -1.0, 1.0))
            ag.assign(v, gi.substream(1).uniform(3, -1.0, 1.0))
            e, bps, ins = q.view().quatRotate(v.view()), 80, (q, v)
        else:
            m, out = ag.Array("f64", (3, 3), n), ag.Array("f64", (3, 3), n)
            ag.assign(m, gi.substream(0).uniform(9, -1.0, 1.0).reshape((3, 3)))
            M = m.view()
            e, bps, ins = ag.select(ag.cwiseAbs(M.det()) > 1e-300, M.inverse(), ag.constant(0.0, (3, 3))), 144, (m,)
        launches.append(ag.prepare(out, e, math=math))
        keep.append((out, ins))
        nbytes += int(n) * bps
    return launches, keep, nbytes, sizes


def secondary_config4(ag):
    import torch
    launches, keep, nbytes, sizes = config4_workload(ag)
    batch = ag.Batch(launches, block=256)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        each_ms = _time_ms(batch.launch_each, reps=3, warmup=1)
        batch_ms = _time_ms(batch.launch, reps=5)
        batch.capture(s.cuda_stream)
        graph_ms = _time_ms(lambda: batch.replay(s.cuda_stream), reps=5)
    return {"items": len(launches), "samples": int(sizes.sum()), "bytes": nbytes,
            "per_call_ms": round(each_ms, 3), "batch_ms": round(batch_ms, 3), "graph_ms": round(graph_ms, 3),
            "speedup_batch": round(each_ms / batch_ms, 2), "speedup_graph": round(each_ms / graph_ms, 2),
            "gbs_graph": round(nbytes / (graph_ms * 1e-3) / 1e9, 1), "math": "emulated FP64"}


SERVE_RATES = (1000, 2000, 5000, 10000, 20000, 50000)


def secondary_config5(ag, rates=SERVE_RATES, seconds=1.0, budget=120 << 30, saturation_requests=20000):
    """Mixed serving: Poisson arrivals of the eight standard shapes, lognormal
    sizes (median 65,536, sigma 1, clipped to [1,024, 4,194,304]), operands
    reused with p = 0.7 and copied in from pinned host memory otherwise, a
    120 GB arena. Each rate runs the same trace through continuous batching
    and through one plain launch per request; latency is arrival (scheduled)
    to completion seen by the host, over all but the first 10% of requests.
    Saturation: every request arrives at time 0."""
    from aether_gb300 import serve
    shapes = serve.standard_shapes()
    pools = serve.HostPools()

    def run(mode, trace, grouping="per_plan", **kw):
        with serve.Server(shapes, budget, mode=mode, grouping=grouping, **kw) as srv:
            reqs = []
            for s, n, ids, t in trace:
                sh = shapes[s]
                hosts = [pools.window(dt, i, sh.operand_bytes(k, n)) for k, ((dt, _), i) in enumerate(zip(sh.operands, ids))]
                reqs.append(srv.request(s, n, ids, hosts, arrival_ns=t))
            sts = srv.wait_all(srv.feed(reqs))
            st = srv.stats()
        span = (st["last_done_ns"] - st["first_arrival_ns"]) * 1e-9
        samples = sum(n for _, n, _, _ in trace)
        out = {"requests": len(trace), "req_per_s": round(len(trace) / span, 1),
               "samples_per_s": round(samples / span, 1), "gbs": round(st["bytes"] / span / 1e9, 1),
               "launches": st["launches"], "items_per_launch": round(st["launched_items"] / max(1, st["launches"]), 2),
               "resident_hit_rate": round(st["resident_hits"] / max(1, st["resident_hits"] + st["resident_misses"]), 3),
               "uploaded_gb": round(st["uploaded_bytes"] / 1e9, 2), "evictions": st["evictions"],
               "enqueue_us_per_launch": round(st["enqueue_ns"] / 1e3 / max(1, st["launches"]), 2),
               "admit_us_per_launch": round(st["admit_ns"] / 1e3 / max(1, st["launches"]), 2),
               "arena_peak_gb": round(st["arena_peak_bytes"] / 1e9, 1), "failed": st["failed"]}
        out.update(serve.latency_summary(sts[len(sts) // 10:]))
        return out

    # warm-up, not reported: every kernel the loop can launch (each plan alone,
    # the batched kernel, the operand gather) is loaded before the first timed
    # request, so no request pays a first-use cost
    warm = serve.make_trace(shapes, 2000, None, seed=99)
    run("batched", warm)
    run("plain", warm)
    res = {"shapes": [s.name for s in shapes], "budget_bytes": budget, "reuse": 0.7,
           "sizes": "lognormal median 65536 sigma 1.0 clipped [1024, 4194304]",
           "latency": "scheduled arrival to completion seen by the host", "outputs": "left in HBM", "rates": {},
           "warmup": "2000 requests at time 0 through both modes before the first rate"}
    for i, rate in enumerate(rates):
        n = int(min(60000, max(1000, rate * seconds)))
        trace = serve.make_trace(shapes, n, float(rate), seed=100 + i)
        res["rates"][str(rate)] = {"batched": run("batched", trace), "plain": run("plain", trace)}
    for name, reuse in (("saturation", 0.7), ("saturation_resident", 1.0)):
        trace = serve.make_trace(shapes, saturation_requests, None, seed=7, reuse=reuse)
        b, p = run("batched", trace), run("plain", trace)
        res[name] = {"batched": b, "plain": p, "speedup_req_per_s": round(b["req_per_s"] / p["req_per_s"], 2)}
        if reuse == 1.0:
            # the same trace through one work-list kernel holding every plan,
            # and with other launch sizes and slot counts
            m = run("batched", trace, grouping="mixed")
            res[name]["batched_one_kernel"] = m
            res[name]["speedup_one_kernel_req_per_s"] = round(m["req_per_s"] / p["req_per_s"], 2)
            sweep = {}
            for items, inflight in ((1024, 4), (1024, 8), (4096, 4)):
                r = run("batched", trace, max_items=items, max_inflight=inflight)
                sweep["items%d_slots%d" % (items, inflight)] = {k: r[k] for k in (
                    "req_per_s", "gbs", "launches", "items_per_launch", "enqueue_us_per_launch",
                    "admit_us_per_launch", "p50_us", "p99_us")}
            res[name]["batched_sweep"] = sweep
    res["grouping"] = ("a launch's requests grouped by plan, one work-list kernel per plan "
                       "(a lone request runs its plan's own kernel)")
    return res


def time_steps(k_expr, k_fill, steps, stream):
    """`steps` back-to-back steps with events around each kernel on the
    launching stream: (total ms, [expression ms], [fill ms])."""
    import torch
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for i in range(steps):
        ev[i][0].record(stream)
        k_expr()
        ev[i][1].record(stream)
        k_fill()
        ev[i][2].record(stream)
    end.record(stream)
    torch.cuda.synchronize()
    return (start.elapsed_time(end), [e[0].elapsed_time(e[1]) for e in ev], [e[1].elapsed_time(e[2]) for e in ev])


def l2_twin_gbs(launch, samples, bytes_per_sample, reps=40, min_ms=0.1):
    """The same kernel on an L2-resident slice (its working set well inside
    the 129 MB L2), back to back: the rate the kernel reaches when HBM is not
    what limits it, i.e. its compute ceiling, in the same algorithmic bytes.
    None when one launch on the slice runs under min_ms: its ramp-up and tail
    would then weigh more than its compute, and the rate would understate the
    ceiling (the fast lowerings of the expression at 2^19 samples)."""
    ms = _time_ms(launch, reps=reps, warmup=3)
    if ms < min_ms:
        return None
    return samples * bytes_per_sample / (ms * 1e-3) / 1e9


def kernel_roofline(name, kernel, nbytes, ms, peak, twin_gbs, prof, samples, clock_mhz, sms):
    """One kernel's roofline entry: HBM fraction of the measured copy peak;
    the issue ceiling (the profiled thread instructions per sample at SMs x 4
    schedulers x 32 lanes x the sampled clock) and the DRAM traffic of the
    committed capture when it is of this very kernel; the rate of the same
    kernel on an L2-resident slice when one was timed; and the bound: the
    lower of the HBM and issue ceilings."""
    achieved = nbytes / (ms * 1e-3) / 1e9
    e = {"kernel": kernel, "bytes_per_launch": nbytes, "ms": round(ms, 4), "achieved": round(achieved, 2),
         "frac": round(achieved / peak, 4)}
    if twin_gbs:
        e["l2_resident_gbs"] = round(twin_gbs, 1)
    p = prof.get(kernel) or prof.get(name)
    e["bound"] = "hbm"
    if p and p["kernel"] == kernel:
        e["traffic"] = round(p["bytes_per_sample"] * samples)
        if clock_mhz:
            issue_ms = p["inst_per_sample"] * samples / (sms * 4 * 32 * clock_mhz * 1e6) * 1e3
            issue_gbs = nbytes / (issue_ms * 1e-3) / 1e9
            e["inst_per_sample"] = p["inst_per_sample"]
            e["issue_roof_gbs"] = round(issue_gbs, 1)
            e["frac_of_issue_roof"] = round(achieved / issue_gbs, 4)
            e["bound"] = "issue" if issue_gbs < peak else "hbm"
    else:
        e["traffic"] = None
        e["traffic_note"] = ("no committed ncu capture of this kernel" if not p else
                             "committed capture is of %s, not of the kernel that ran" % p["kernel"])
    return e


def lowered_step(ag, arrs, d, z, expr, g, steps, stream, ref, math, clock_mhz=None, sms=152):
    """The same step in another lowering, timed like the headline and checked
    against the oracle on the CPU leg's slice: native FP64 (math 0, CUDA's FP64
    functions on the FP64 pipe) or FP64-grade triple-float (math 3, within the
    native bound of the oracle; its fill draws double-float normals, inside the
    reference's normal tolerance)."""
    k_expr = ag.prepare(d, expr, math=math, tune=True)
    k_fill = ag.prepare(z, g.substream(4).normal(1, 0.0, 1.0), math=fill_math(math), tune=True)
    for _ in range(2):
        k_expr()
        k_fill()
    total, te, tf = time_steps(k_expr, k_fill, max(3, min(steps, 5)), stream)
    n_tw = min(N_EXPR, 1 << 19)
    twin = l2_twin_gbs(ag.prepare(d, expr, n=n_tw, math=math, tune=True), n_tw, 120)
    te, tf = statistics.mean(te), statistics.mean(tf)
    peak, _ = peaks()
    n_steps = max(3, min(steps, 5))
    out = {"lowering": LOWERINGS[math], "fill_lowering": LOWERINGS[fill_math(math)],
           "ms_per_step": round(total / n_steps, 4),
           "value": round((BYTES_EXPR + BYTES_FILL) / (total / n_steps * 1e-3) / 1e9, 2),
           "expr": {"kernel": k_expr.plan.name, "ms": round(te, 4), "gbs": round(BYTES_EXPR / (te * 1e-3) / 1e9, 1),
                    "frac": round(BYTES_EXPR / (te * 1e-3) / 1e9 / peak, 4),
                    "roofline": kernel_roofline("expr", k_expr.plan.name + "_v", BYTES_EXPR, te, peak, twin,
                                                profile_figures(), N_EXPR, clock_mhz, sms)},
           "fill": {"kernel": k_fill.plan.name, "ms": round(tf, 4), "gbs": round(BYTES_FILL / (tf * 1e-3) / 1e9, 1),
                    "frac": round(BYTES_FILL / (tf * 1e-3) / 1e9 / peak, 4)}}
    if ref is not None:
        out["gpu_vs_oracle"] = check_against_oracle(arrs, d, z, *ref, math=math)
    return out


def run_ours(args):
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import aether_gb300 as ag
    from aether_gb300 import shard

    math_mode = args.math
    math_z = fill_math(math_mode)
    stream = torch.cuda.current_stream()
    g = ag.Generator(7)
    arrs = [ag.Array("f64", (3,), N_EXPR) for _ in range(4)]
    for k, a in enumerate(arrs):
        ag.assign(a, g.substream(k).uniform(3, -4.0, 4.0))
    d = ag.Array("f64", (3,), N_EXPR)
    z = ag.Array("f64", (1,), N_FILL)
    a, b, c, d0 = (x.view() for x in arrs)
    expr = ag.cwiseSqrt(a * a + b * b) * ag.cwiseLog1p(ag.cwiseAbs(c)) + ag.cwiseRsqrt(ag.constant(1.0, (3,)) + d0 * d0)
    k_expr = ag.prepare(d, expr, math=math_mode, tune=not args.no_tune)
    k_fill = ag.prepare(z, g.substream(4).normal(1, 0.0, 1.0), math=math_z, tune=not args.no_tune)
    torch.cuda.synchronize()

    def step():
        k_expr()
        k_fill()

    for _ in range(max(args.warmup, 0)):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    with ClockSampler(local) as clk:
        time.sleep(0.3)
        total_ms, t_expr, t_fill = time_steps(k_expr, k_fill, args.steps, stream)
    total_ms = shard.max_over_ranks(total_ms, group=dist.group.WORLD if dist else None)
    ms_step = total_ms / args.steps
    value = ws * (BYTES_EXPR + BYTES_FILL) / (ms_step * 1e-3) / 1e9

    # e2e through the C-ABI: pinned host buffers, copies inside the timed region.
    e2e = None
    if not args.no_e2e:
        L = ag._abi.lib()
        import ctypes
        nb = N_EXPR * 3 * 8
        # host buffers from the C-ABI's pinned chunks
        host_in = [ag.pinned_empty((3, N_EXPR)) for _ in range(4)]
        for h, x in zip(host_in, arrs):
            h.copy_(x.data[:, :N_EXPR])
        host_out = ag.pinned_empty((3, N_EXPR))
        host_fill = ag.pinned_empty((1, N_FILL))
        # The step cut into K sample blocks (partition_view) through a
        # three-stage pipeline: uploads on one stream, kernels on a second,
        # downloads on a third, joined by events, so block r+1 copies in
        # while block r computes and block r-1 copies out, and neither copy
        # direction waits behind the other. Consecutive steps run back to
        # back: block r of a step uploads once the previous step's kernels
        # have read block r, and computes once its previous results have been
        # copied out; the timed region ends with one synchronisation after
        # the last step's downloads.
        K = max(1, args.e2e_chunks)
        streams = [torch.cuda.Stream() for _ in range(3)]
        s_up, s_run, s_down = streams
        ev_up = [torch.cuda.Event() for _ in range(K)]
        ev_run = [torch.cuda.Event() for _ in range(K)]
        ev_down = [torch.cuda.Event() for _ in range(K)]
        pitch_e = ag.padded_block_samples(N_EXPR, K)
        pitch_f = ag.padded_block_samples(N_FILL, K)
        chunks = []
        for r in range(K):
            bi = [ag.partition_view(x, K, r) for x in arrs]
            bo = ag.partition_view(d, K, r)
            bz = ag.partition_view(z, K, r)
            if bo.n == 0 and bz.n == 0:
                continue
            a_, b_, c_, d0_ = (x.view() for x in bi)
            e_r = ag.cwiseSqrt(a_ * a_ + b_ * b_) * ag.cwiseLog1p(ag.cwiseAbs(c_)) + \
                ag.cwiseRsqrt(ag.constant(1.0, (3,)) + d0_ * d0_)
            ke = ag.prepare(bo, e_r, math=math_mode, tune=not args.no_tune) if bo.n else None
            kf = ag.prepare(bz, g.substream(4).normal(1, 0.0, 1.0), sample_offset=r * pitch_f, math=math_z,
                            tune=not args.no_tune) if bz.n else None
            chunks.append((r * pitch_e, bo.n, r * pitch_f, bz.n, ke, kf))
        cap = arrs[0].capacity

        up_p, down_p = ctypes.c_void_p(s_up.cuda_stream), ctypes.c_void_p(s_down.cuda_stream)

        def e2e_step():
            for k, (e0, en, f0, fn, ke, kf) in enumerate(chunks):
                s_up.wait_event(ev_run[k])     # the previous step's kernels are done with block k
                for h, x in zip(host_in, arrs):
                    for c in range(3):
                        ag._abi.check(L.aether_copy(1, local, ctypes.c_void_p(x.data.data_ptr() + (c * cap + e0) * 8), 2, 0,
                                                    ctypes.c_void_p(h.data_ptr() + (c * N_EXPR + e0) * 8), en * 8, up_p))
                ev_up[k].record(s_up)
                s_run.wait_event(ev_up[k])
                s_run.wait_event(ev_down[k])   # the previous step's results of block k are out
                if ke is not None:
                    ke(s_run.cuda_stream)
                if kf is not None:
                    kf(s_run.cuda_stream)
                ev_run[k].record(s_run)
                s_down.wait_event(ev_run[k])
                for c in range(3):
                    ag._abi.check(L.aether_copy(2, 0, ctypes.c_void_p(host_out.data_ptr() + (c * N_EXPR + e0) * 8), 1,
                                                local, ctypes.c_void_p(d.data.data_ptr() + (c * cap + e0) * 8), en * 8, down_p))
                ag._abi.check(L.aether_copy(2, 0, ctypes.c_void_p(host_fill.data_ptr() + f0 * 8), 1, local,
                                            ctypes.c_void_p(z.data.data_ptr() + f0 * 8), fn * 8, down_p))
                ev_down[k].record(s_down)

        # warm-up: the first passes over freshly pinned buffers run well below
        # the link rate on some boxes
        for _ in range(3):
            e2e_step()
        ag._abi.check(L.aether_stream_sync(local, down_p))
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        # Timed runs of e_steps back-to-back steps each; the median run is
        # reported, every run beside it.
        # Five timed runs, each preceded by a one-copy probe of the
        # host->device rate, so a slow run can be told from a busy link.
        e_steps = max(3, min(args.steps, 6))
        runs, probes = [], []
        for _ in range(5):
            probes.append(h2d_probe(L, local, host_in[0], arrs[0], nb // 4, s_up))
            t0 = time.perf_counter()
            for _ in range(e_steps):
                e2e_step()
            ag._abi.check(L.aether_stream_sync(local, down_p))
            runs.append((time.perf_counter() - t0) * 1e3 / e_steps)
        e_ms = statistics.median(runs)
        e_ms = shard.max_over_ranks(e_ms, group=dist.group.WORLD if dist else None)
        e2e = {"value": round(ws * (BYTES_EXPR + BYTES_FILL) / (e_ms * 1e-3) / 1e9, 3), "unit": UNIT,
               "h2d_bytes_per_step": 4 * nb, "d2h_bytes_per_step": nb + N_FILL * 8, "ms_per_step": round(e_ms, 3),
               "pipeline": "%d sample blocks: upload, compute and download streams; %d steps back to back, "
                           "one synchronisation after the last; median of 5 runs" % (len(chunks), e_steps),
               "ms_per_step_runs": [round(r, 3) for r in runs],
               "h2d_gbs_before_runs": [round(p, 1) for p in probes]}
        # The host link measured in the same process: one large copy each
        # way, then both at once; the copy time of one step at those rates
        # is the bound the end-to-end number is read against.
        link = link_rates(L, local, host_in[0], arrs[0], host_out, d, nb, s_up, s_down)
        h2d_b, d2h_b = 4 * nb, nb + N_FILL * 8
        bound_ms = 1e3 * max(h2d_b / (link["h2d_gbs"] * 1e9), d2h_b / (link["d2h_gbs"] * 1e9),
                             (h2d_b + d2h_b) / (link["both_gbs"] * 1e9))
        link["step_copy_bound_ms"] = round(bound_ms, 3)
        link["frac"] = round(bound_ms / e_ms, 3)
        e2e["link"] = link

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0

    peak, peak_kind = peaks()
    te = statistics.mean(t_expr)
    tf = statistics.mean(t_fill)
    clocks = clk.summary()
    props = torch.cuda.get_device_properties(local)
    prof = profile_figures()
    # memory-free twins: the write-only fill on a 2^23-double (64 MB) slice and
    # the expression on 2^19 samples (63 MB of operands and output), both well
    # inside the 129 MB L2 and enough chunks to fill every SM
    n_tw_f = min(N_FILL, 1 << 23)
    n_tw_e = min(N_EXPR, 1 << 19)
    twin_e = l2_twin_gbs(ag.prepare(d, expr, n=n_tw_e, math=math_mode, tune=not args.no_tune), n_tw_e, 120)
    twin_f = l2_twin_gbs(ag.prepare(z, g.substream(4).normal(1, 0.0, 1.0), n=n_tw_f, math=math_z,
                                    tune=not args.no_tune), n_tw_f, 8)
    kernels = {
        "expr": kernel_roofline("expr", k_expr.plan.name + "_v", BYTES_EXPR, te, peak, twin_e, prof, N_EXPR,
                                clocks.get("sm_mhz"), props.multi_processor_count),
        "fill": kernel_roofline("fill", k_fill.plan.name + "_v", BYTES_FILL, tf, peak, twin_f, prof, N_FILL,
                                clocks.get("sm_mhz"), props.multi_processor_count),
    }
    dom = "fill" if tf >= te else "expr"
    k = kernels[dom]
    roofline = {"bound": "hbm", "achieved": k["achieved"], "peak": peak, "unit": "GB/s", "frac": k["frac"],
                "peak_kind": peak_kind, "traffic": k["traffic"],
                "kernel": dom + ": " + k["kernel"] + " (the larger share of the step)",
                "share_of_step": round(max(te, tf) / (te + tf), 3), "binding_roof": k["bound"],
                "issue_roof_gbs": k.get("issue_roof_gbs"), "frac_of_issue_roof": k.get("frac_of_issue_roof"),
                "kernels": kernels,
                "issue_roof": "profiled thread instructions per sample (profiles/ncu_traffic.txt) at SMs x 4 "
                              "schedulers x 32 lanes x the sampled SM clock; l2_resident_gbs: the memory-free "
                              "twin, the same kernel timed on a slice that stays in L2 (2^23 fill doubles, 2^19 "
                              "expression samples): its compute ceiling in the same algorithmic bytes, reported "
                              "when one launch on the slice runs 0.1 ms or more"}
    cpu = None
    ref = None
    if not args.no_cpu:
        gbs, t, nt, sample, ref = cpu_leg(1, 1)
        cpu = {"value": round(gbs, 3), "unit": UNIT, "cores": nt, "kind": "port", "sample": sample}
        # the oracle doubles as the checker of this run's GPU results
        cpu["gpu_vs_oracle"] = check_against_oracle(arrs, d, z, *ref, math=math_mode, math_z=math_z)
    secondary = None
    if not args.no_secondary:
        # the other configurations, measured after the timed region
        secondary = {}
        wanted = set(args.secondary.split(",")) if args.secondary else None
        for name, m in (("native_fp64_step", 0), ("fp64_grade_step", 3)):
            if math_mode == m or (wanted is not None and name not in wanted):
                continue
            try:
                secondary[name] = lowered_step(ag, arrs, d, z, expr, g, args.steps, stream, ref, m,
                                               clocks.get("sm_mhz"), props.multi_processor_count)
            except Exception as ex:   # reported, never hidden
                secondary[name] = {"error": str(ex).splitlines()[0][:300] if str(ex) else repr(ex)}
        for name, fn in (("config1_plain", secondary_config1), ("config3_precision_form", secondary_config3),
                         ("config4_batch", secondary_config4), ("config5_serving", secondary_config5)):
            if wanted is not None and name not in wanted:
                continue
            try:
                secondary[name] = fn(ag)
            except Exception as ex:   # reported, never hidden
                secondary[name] = {"error": str(ex).splitlines()[0][:300] if str(ex) else repr(ex)}
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_step, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (Philox4x32-10 seed 7, generated on device)",
        "config": {"workload": WORKLOAD, "samples_expr": N_EXPR, "samples_fill": N_FILL,
                   "l2": "inputs larger than L2 (no flush)", "math": LOWERINGS[math_mode], "fill_math": LOWERINGS[math_z],
                   "lowering_expr": {"block": k_expr.plan.info().block, "ipt": k_expr.plan.info().ipt,
                                     "vec": k_expr.plan.info().vec, "registers": k_expr.plan.info().registers},
                   "lowering_fill": {"block": k_fill.plan.info().block, "ipt": k_fill.plan.info().ipt,
                                     "vec": k_fill.plan.info().vec, "registers": k_fill.plan.info().registers},
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
        "gpu_launches": 2 * args.steps, "clocks": clocks, "secondary": secondary,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--math", type=int, default=1, choices=[0, 1, 3],
                    help="lowering of the expression: 0 native FP64, 1 emulated FP64 (double-float), "
                         "3 FP64-grade (triple-float); the fill follows (native for 0, double-float otherwise)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-tune", action="store_true", help="default lowering instead of the autotuned one")
    ap.add_argument("--no-secondary", action="store_true", help="skip configs 1, 3, 4 and 5 after the timed region")
    ap.add_argument("--e2e-chunks", type=int, default=4, help="sample blocks of the pipelined end-to-end step")
    ap.add_argument("--secondary", default="", help="comma-separated subset of the secondary measurements "
                                                     "(native_fp64_step, fp64_grade_step, config1_plain, "
                                                     "config3_precision_form, "
                                                     "config4_batch, config5_serving); default all")
    ap.add_argument("--expr-log2", type=int, default=26, help="log2 samples of the expression kernel")
    ap.add_argument("--fill-log2", type=int, default=28, help="log2 doubles of the normal fill")
    ap.add_argument("--precision-log2", type=int, default=27, help="log2 samples of the precision-form parts")
    args = ap.parse_args()
    global N_EXPR, N_FILL, BYTES_EXPR, BYTES_FILL, PRECISION_LOG2
    N_EXPR, N_FILL = 1 << args.expr_log2, 1 << args.fill_log2
    PRECISION_LOG2 = args.precision_log2
    BYTES_EXPR, BYTES_FILL = N_EXPR * 120, N_FILL * 8
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
