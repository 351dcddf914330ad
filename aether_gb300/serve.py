"""Serving: a request loop with continuous batching (aether_serve_*).

A Server owns a device arena of a fixed byte budget. Each request evaluates
one of the server's plans over n samples; its operands are named by residency
ids, copied in from host memory the first time and reused while they stay
resident. Requests that arrive while others run are admitted as launch slots
and arena bytes free up, and the admitted ones go to the device together in
one persistent batched launch (mode "batched") or one plain launch each
(mode "plain", the per-call baseline). Each request runs its plan's own
arithmetic, so its result does not depend on the mode or on the other
requests in its launch.

ShapeTemplate turns an expression over placeholder operands into a plan and
records the order in which the plan reads them; standard_shapes() are the
eight expression shapes of the mixed serving workload (make_trace).
"""

import ctypes
import math as _math

import numpy as np

from . import _abi
from .expr import IrContext, Operand, plan_text

MODES = {"batched": 0, "plain": 1}
KEEP_OUTPUT = 1
STATES = {0: "queued", 1: "running", 2: "done", 3: "failed"}
_ES = {"f64": 8, "f32": 4}


def capacity(n):
    """Samples per plane of an array of n samples (the SoA capacity rule)."""
    return (int(n) + 31) // 32 * 32


class ShapeTemplate:
    """One served expression shape: `build(*leaves)` over placeholder operands.

    operands: list of (dtype, shape) of the leaves, in the order build() takes
    them. The plan reads them in its own order; `order[k]` is the template
    index of the plan's operand k."""

    def __init__(self, name, out_dtype, out_shape, operands, build, math=0, contract=-1):
        from . import get_plan
        self.name = name
        self.out_dtype = out_dtype
        self.out_shape = tuple(out_shape)
        self.operands = [(dt, tuple(sh)) for dt, sh in operands]
        leaves = [Operand(i + 1, 0, dt, sh) for i, (dt, sh) in enumerate(self.operands)]
        expr = build(*leaves)
        ctx = IrContext()
        self.ir = plan_text(out_dtype, self.out_shape, "set", expr, ctx)
        self.order = [int(ptr) - 1 for (ptr, _p, _d, _c, _o) in ctx.operands]
        self.scalars = list(ctx.scalars)
        self.keys = list(ctx.keys)
        self.build = build
        self.math, self.contract = math, contract
        self.plan = get_plan(self.ir, math=math, contract=contract, **self._tuned())
        self.out_comps = int(np.prod(self.out_shape)) if self.out_shape else 1

    def _tuned(self):
        """The autotuned lowering of this shape's plan on this device, if any
        (aether_gb300.tune; tune_standard_shapes measures them)."""
        try:
            from . import tune
            low = tune.tuned(self.ir, self.math, self.contract, regime="serve")
        except Exception:   # no device to key the cache on
            low = None
        return dict(low) if low else {}

    def operand_bytes(self, k, n):
        dt, sh = self.operands[k]
        return int(np.prod(sh) if sh else 1) * capacity(n) * _ES[dt]

    def bytes_per_sample(self):
        b = sum((int(np.prod(sh)) if sh else 1) * _ES[dt] for dt, sh in self.operands)
        return b + self.out_comps * _ES[self.out_dtype]


def standard_shapes():
    """The eight shapes of the mixed serving workload: the plain fused
    expression and the large streaming expression in FP64 and in the FP32
    precision form, an 8-component per-sample dot product in FP32, and the
    cross product, quaternion rotation and guarded 3x3 inverse in FP64.
    Component counts 1, 3, 4, 8 and 9 all occur."""
    from . import cwiseAbs, cwiseExp, cwiseLog1p, cwiseRsqrt, cwiseSin, cwiseSqrt, select
    from .expr import constant

    def cfg1(a, b, c):
        return a + b * c + cwiseSin(a) * cwiseExp((c * c) * (-1.0))

    def cfg2(a, b, c, d):
        return cwiseSqrt(a * a + b * b) * cwiseLog1p(cwiseAbs(c)) + cwiseRsqrt(constant(1.0, (3,)) + d * d)

    def inv(m):
        return select(cwiseAbs(m.det()) > 1e-300, m.inverse(), constant(0.0, (3, 3)))

    v3, v4, v8, m9 = (3,), (4,), (8,), (3, 3)
    return [
        ShapeTemplate("expr1_f64", "f64", v3, [("f64", v3)] * 3, cfg1, math=1),
        ShapeTemplate("expr1_f32", "f32", v3, [("f32", v3)] * 3, cfg1, math=2),
        ShapeTemplate("expr2_f64", "f64", v3, [("f64", v3)] * 4, cfg2, math=1),
        ShapeTemplate("expr2_f32", "f32", v3, [("f32", v3)] * 4, cfg2, math=2),
        ShapeTemplate("dot8_f32", "f32", (), [("f32", v8)] * 2, lambda x, y: x.dot(y), math=2),
        ShapeTemplate("cross_f64", "f64", v3, [("f64", v3)] * 2, lambda a, b: a.cross(b), math=1),
        ShapeTemplate("quatrot_f64", "f64", v3, [("f64", v4), ("f64", v3)], lambda q, v: q.quatRotate(v), math=1),
        ShapeTemplate("inv3_f64", "f64", m9, [("f64", m9)], inv, math=1),
    ]


def tune_standard_shapes(n=1 << 21, shapes=None, verbose=False):
    """Autotune the plan of every served shape on device arrays of n samples
    (uniform values in [-1, 1)) and cache the winners under the "serve" regime
    (aether_gb300.tune).
    Shapes built afterwards take the tuned lowering, and so do the serving
    loop's per-plan work-list kernels."""
    import aether_gb300 as ag
    from . import tune
    shapes = shapes or standard_shapes()
    results = {}
    for k, sh in enumerate(shapes):
        arrays = []
        for j, (dt, shape) in enumerate(sh.operands):
            a = ag.Array(dt, shape, n)
            comps = int(np.prod(shape)) if shape else 1
            ag.assign(a, ag.Generator(1000 + k).substream(j).uniform(comps, -1.0, 1.0).reshape(shape)
                      if len(shape) > 1 else ag.Generator(1000 + k).substream(j).uniform(comps, -1.0, 1.0))
            arrays.append(a)
        dst = ag.Array(sh.out_dtype, sh.out_shape, n)
        expr = sh.build(*[a.view() for a in arrays])

        def make(**low):
            return ag.prepare(dst, expr, math=sh.math, contract=sh.contract, **low)

        best, res = tune.tune(make, sh.ir, sh.math, sh.contract, verbose=verbose, regime="serve")
        results[sh.name] = (best, res[0][0] if res else None)
    return results


class HostPools:
    """Pinned host bytes that stand for operand contents: each residency id
    reads a fixed window of a pool of uniform values in [-1, 1), so equal
    ids always carry equal bytes."""

    def __init__(self, f64_bytes=512 << 20, f32_bytes=256 << 20, seed=5):
        import torch
        g = torch.Generator().manual_seed(seed)
        self.pools = {}
        for dt, nbytes, tdt in (("f64", f64_bytes, torch.float64), ("f32", f32_bytes, torch.float32)):
            from . import pinned_empty
            t = pinned_empty((nbytes // _ES[dt],), dt)
            t.uniform_(-1.0, 1.0, generator=g)
            self.pools[dt] = t

    def window(self, dt, ident, nbytes):
        t = self.pools[dt]
        total = t.numel() * _ES[dt]
        if nbytes > total:
            raise ValueError("operand of %d bytes exceeds the %s pool" % (nbytes, dt))
        slots = (total - nbytes) // 256 + 1
        off = (int(ident) * 0x9E3779B97F4A7C15 % (1 << 64)) % slots * 256
        return t.data_ptr() + off

    def array(self, dt, ident, comps, n):
        """The host contents behind an id, as a (comps, n) numpy array."""
        pitch = capacity(n)
        ptr = self.window(dt, ident, comps * pitch * _ES[dt])
        t = self.pools[dt]
        start = (ptr - t.data_ptr()) // _ES[dt]
        return t[start:start + comps * pitch].numpy().reshape(comps, pitch)[:, :n]


class _Req:
    """ctypes image of one request plus the buffers it points into."""

    __slots__ = ("c", "ops", "sc", "keys", "out")

    def __init__(self, shape, plan_index, n, ids, hosts, host_out=None, keep=False, arrival_ns=0):
        self.ops = (_abi.AetherServeOperand * max(1, len(shape.order)))()
        for k, t in enumerate(shape.order):
            self.ops[k].id = int(ids[t])
            self.ops[k].host = hosts[t] or 0
            self.ops[k].pitch = capacity(n)
        self.sc = (ctypes.c_double * max(1, len(shape.scalars)))(*shape.scalars)
        self.keys = (ctypes.c_uint64 * max(1, len(shape.keys)))(*shape.keys)
        self.out = host_out
        c = _abi.AetherServeRequest()
        c.plan = plan_index
        c.flags = KEEP_OUTPUT if keep else 0
        c.n = int(n)
        c.operands = self.ops
        c.n_operands = len(shape.order)
        c.scalars = self.sc
        c.n_scalars = len(shape.scalars)
        c.keys = self.keys
        c.n_keys = len(shape.keys)
        c.host_out = host_out.data_ptr() if host_out is not None else 0
        c.arrival_ns = int(arrival_ns)
        self.c = c


def _status_dict(s):
    return {"state": STATES.get(s.state, s.state), "launch_items": s.launch_items,
            "t_arrival_ns": s.t_arrival_ns, "t_dispatch_ns": s.t_dispatch_ns, "t_done_ns": s.t_done_ns,
            "latency_ns": (s.t_done_ns - s.t_arrival_ns) if s.state == 2 else None,
            "output": s.output, "out_pitch": s.out_pitch, "bytes": s.bytes, "uploaded_bytes": s.uploaded_bytes}


class Server:
    """aether_serve_open over `shapes` (ShapeTemplate list)."""

    def __init__(self, shapes, budget_bytes, mode="batched", max_inflight=0, max_items=0, block=0, ipt=0,
                 idle_spin_us=0, upload_engine="gather", grouping="per_plan"):
        self.shapes = list(shapes)
        arr = (ctypes.c_void_p * len(self.shapes))(*[s.plan.handle for s in self.shapes])
        cfg = _abi.AetherServeConfig(int(budget_bytes), MODES[mode], max_inflight, max_items, block, ipt,
                                     idle_spin_us, {"gather": 0, "copy": 1}[upload_engine],
                                     {"per_plan": 0, "mixed": 1}[grouping])
        h = ctypes.c_void_p()
        _abi.check(_abi.lib().aether_serve_open(arr, len(self.shapes), ctypes.byref(cfg), ctypes.byref(h)))
        self.handle = h
        self._live = {}

    def request(self, plan_index, n, ids, hosts, host_out=None, keep=False, arrival_ns=0):
        return _Req(self.shapes[plan_index], plan_index, n, ids, hosts, host_out, keep, arrival_ns)

    def submit(self, req):
        t = ctypes.c_uint64()
        _abi.check(_abi.lib().aether_serve_submit(self.handle, ctypes.byref(req.c), ctypes.byref(t)))
        self._live[t.value] = req
        return t.value

    def feed(self, reqs):
        """Submit each request at its arrival_ns after the call starts."""
        n = len(reqs)
        arr = (_abi.AetherServeRequest * max(1, n))()
        for i, r in enumerate(reqs):
            arr[i] = r.c
        tickets = (ctypes.c_uint64 * max(1, n))()
        _abi.check(_abi.lib().aether_serve_feed(self.handle, arr, n, tickets))
        out = list(tickets[:n])
        for t, r in zip(out, reqs):
            self._live[t] = r
        return out

    def status(self, ticket):
        s = _abi.AetherServeStatus()
        _abi.check(_abi.lib().aether_serve_status(self.handle, ticket, ctypes.byref(s)))
        return _status_dict(s)

    def wait(self, ticket, timeout=120.0):
        s = _abi.AetherServeStatus()
        _abi.check(_abi.lib().aether_serve_wait(self.handle, ticket, float(timeout), ctypes.byref(s)))
        return _status_dict(s)

    def wait_all(self, tickets, timeout=300.0):
        return [self.wait(t, timeout) for t in tickets]

    def release(self, ticket):
        _abi.check(_abi.lib().aether_serve_release(self.handle, ticket))

    def stats(self):
        s = _abi.AetherServeStats()
        _abi.check(_abi.lib().aether_serve_stats(self.handle, ctypes.byref(s)))
        return {name: getattr(s, name) for name, _ in _abi.AetherServeStats._fields_}

    def close(self):
        if self.handle:
            _abi.lib().aether_serve_close(self.handle)
            self.handle = None
            self._live.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def make_trace(shapes, n_requests, rate, seed=11, reuse=0.7, median=65536, sigma=1.0, lo=1024, hi=4194304,
               recent=32):
    """Poisson arrivals at `rate` requests/s (rate None: all at time 0); each
    request picks a shape uniformly, then with probability `reuse` one of the
    last `recent` datasets of that shape (same n, same operand ids), else a
    new dataset with n ~ lognormal(median, sigma) clipped to [lo, hi] and new
    ids. Returns a list of (shape index, n, ids, arrival_ns)."""
    rng = np.random.default_rng(seed)
    per_shape = [[] for _ in shapes]
    next_id = [1]
    t = 0.0
    out = []
    for _ in range(n_requests):
        if rate:
            t += rng.exponential(1.0 / rate)
        s = int(rng.integers(len(shapes)))
        if per_shape[s] and rng.random() < reuse:
            hist = per_shape[s][-recent:]
            n, ids = hist[int(rng.integers(len(hist)))]
        else:
            n = int(np.clip(round(rng.lognormal(_math.log(median), sigma)), lo, hi))
            ids = list(range(next_id[0], next_id[0] + len(shapes[s].operands)))
            next_id[0] += len(ids)
            per_shape[s].append((n, ids))
        out.append((s, n, ids, int(t * 1e9)))
    return out


def latency_summary(statuses):
    lat = np.array([s["latency_ns"] for s in statuses if s["latency_ns"] is not None], dtype=np.float64) / 1e3
    if lat.size == 0:
        return {}
    return {"p50_us": round(float(np.percentile(lat, 50)), 1), "p99_us": round(float(np.percentile(lat, 99)), 1),
            "mean_us": round(float(lat.mean()), 1), "max_us": round(float(lat.max()), 1)}
