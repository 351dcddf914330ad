"""Autotuner: choose block shape, lane groups per thread, vector width and
occupancy bound per plan, by timing candidate lowerings on the device.

Results are cached in a JSON file keyed by the plan text, the math mode, the
device name, the digest of the device headers every kernel includes and the
digest of the kernel text the generator writes for the plan
($AETHER_GB300_TUNE_CACHE, else ~/.cache/aether_gb300/tune.json), so a plan
is tuned once per device and code version and later processes reuse the
winner. Candidates are valid by construction (block a multiple of 32 up to
1024, vec in {1, 2, 4}, ipt in {1, 2, 4}); a candidate that fails to compile
or launch is skipped, never retried.
"""

import hashlib
import json
import os
import threading

_lock = threading.Lock()

DEFAULT_CANDIDATES = [
    dict(block=b, ipt=i, vec=v, min_blocks=m)
    for b in (128, 256, 512)
    for i in (1, 2)
    for v in (0, 1)
    for m in (0, 2, 3, 4)
    if not (b == 512 and m == 4) and not (b < 512 and m == 2)   # 512 x 2 CTAs caps a thread at 64 registers
]


def cache_path():
    p = os.environ.get("AETHER_GB300_TUNE_CACHE")
    if p:
        return p
    base = os.environ.get("XDG_CACHE_HOME") or os.path.join(os.path.expanduser("~"), ".cache")
    return os.path.join(base, "aether_gb300", "tune.json")


def _device_name():
    import torch
    return torch.cuda.get_device_name(torch.cuda.current_device())


# Device headers only FP64-grade (math 3) kernels include.
_TF_HEADERS = ("ag_tf64.cuh", "ag_tf64_tables.cuh", "ag_tf64_trig.cuh", "ag_tf64_trig_tables.cuh")


def _code_digest(math=0):
    """Digest of the device runtime a generated kernel of this lowering can
    include (the payload headers under their bare names; the consumer headers
    under aether/ never reach a generated kernel, and the triple-float headers
    only reach math-3 kernels): a tuning result stays valid only for the code
    it was measured on."""
    from . import rtc
    h = hashlib.sha1()
    for name, src in sorted(rtc.payload().headers.items()):
        if name.startswith("aether/") or (name in _TF_HEADERS and math != 3):
            continue
        h.update(name.encode())
        h.update(src)
    return h.hexdigest()[:16]


def _generated_digest(ir, math, contract):
    """Digest of the kernel text the generator writes for this plan (at the
    default lowering): a tuning result also goes stale when the generator
    changes what it emits."""
    from . import _abi
    try:
        src = _abi.generate(ir, _abi.lowering(math=math, contract=contract))
    except Exception:
        return "-"
    return hashlib.sha1(src.encode()).hexdigest()[:16]


def _key(ir, math, contract, regime=""):
    """The cache key of a plan's tuning. `regime` names the launch sizes it was
    measured at: "" for whole-array launches (the benchmarks' 2^26..2^28
    samples), "serve" for served requests (2^21 samples), whose winners differ
    (tail effects favour smaller blocks)."""
    h = hashlib.sha1(("%s|%d|%d|%s|%s|%s" % (ir, math, contract, _device_name(), _code_digest(math),
                                             _generated_digest(ir, math, contract))).encode()).hexdigest()
    return regime_key(h, regime)


def regime_key(key, regime):
    """The key of `regime`'s entry from the whole-array key of the same plan."""
    return key if not regime else hashlib.sha1(("%s|%s" % (key, regime)).encode()).hexdigest()


SHIPPED = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuned.json")


def load(include_shipped=True):
    """The user's tuning cache over the winners shipped with the package
    (tuned.json, measured on GB300 for the plans the benchmarks use)."""
    data = {}
    if include_shipped and os.environ.get("AETHER_GB300_TUNE_SHIPPED", "1") != "0":
        try:
            with open(SHIPPED) as f:
                data.update(json.load(f))
        except Exception:
            pass
    try:
        with open(cache_path()) as f:
            data.update(json.load(f))
    except Exception:
        pass
    return data


def store(key, rec):
    with _lock:
        data = load(include_shipped=False)
        data[key] = rec
        path = cache_path()
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + ".tmp%d" % os.getpid()
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1)
        os.replace(tmp, path)


def tuned(ir, math=0, contract=-1, regime=""):
    """The cached winning lowering for a plan, or None."""
    rec = load().get(_key(ir, math, contract, regime))
    return rec["lowering"] if rec else None


def tune(make_launch, ir, math=0, contract=-1, candidates=None, reps=5, warmup=2, verbose=False, regime=""):
    """Time `make_launch(**lowering)` for each candidate lowering and cache the
    fastest. `make_launch` returns a callable that enqueues one evaluation on
    the current stream (aether_gb300.prepare(...)). Returns (best, results)."""
    import torch
    results = []
    for cand in candidates or DEFAULT_CANDIDATES:
        try:
            L = make_launch(**cand)
            for _ in range(warmup):
                L()
            torch.cuda.synchronize()
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            ev[0].record()
            for _ in range(reps):
                L()
            ev[1].record()
            torch.cuda.synchronize()
            ms = ev[0].elapsed_time(ev[1]) / reps
            info = L.plan.info()
            results.append((ms, cand, info.registers, info.blocks_per_sm))
            if verbose:
                print("tune %-45s %8.4f ms  regs %3d  blocks/SM %d" % (cand, ms, info.registers, info.blocks_per_sm))
        except Exception as e:   # candidate does not compile or launch: skip it
            if verbose:
                print("tune %s skipped: %s" % (cand, str(e).splitlines()[0] if str(e) else e))
    if not results:
        raise RuntimeError("autotune: no candidate lowering ran")
    results.sort(key=lambda r: r[0])
    best = results[0]
    store(_key(ir, math, contract, regime), {"lowering": best[1], "ms": best[0], "registers": best[2],
                                      "blocks_per_sm": best[3], "candidates": len(results)})
    return best[1], results
