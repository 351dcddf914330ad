"""Runtime-typed strided evaluation (aether_runtime_eval) against the oracle:
the reference's own cases (tests/test_RuntimeEval.cpp: copies, both casts,
the five arithmetic ops, a strided view that must leave the gaps untouched,
refusals), then seeded random views of rank 0..6 with permuted, padded and
broadcast (stride 0) strides. Bit-exact: every element is one IEEE operation
(or two, rounded separately) on the same inputs."""

import sys
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import aether_gb300 as ag
from aether_gb300 import RuntimeOp, runtime_eval

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import pyoracle as po  # noqa: E402

gpu = pytest.mark.gpu


def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _fill(c, n):
    # tests/test_RuntimeEval.cpp:36-46
    idx = np.arange(n, dtype=np.float64)[None, :]
    comp = np.arange(c, dtype=np.float64)[:, None]
    return idx * 0.75 + comp * 0.1 - 3.0, idx * -0.5 + comp + 1.25


def _dev(x, dtype=torch.float64):
    return torch.as_tensor(np.ascontiguousarray(x)).to(dtype).cuda()


# -- refusals are decided before any device call: they run without a GPU ----

def _host_view(shape, dtype=torch.float64):
    return torch.zeros(shape, dtype=dtype)


def test_shape_mismatch_refused():
    with pytest.raises(ag.AetherError, match="shape mismatch: a vs out"):
        runtime_eval(RuntimeOp.Assign, _host_view((3, 5)), None, _host_view((3, 4)))
    with pytest.raises(ag.AetherError, match="shape mismatch: b vs out"):
        runtime_eval(RuntimeOp.Add, _host_view((3, 5)), _host_view((5, 3)), _host_view((3, 5)))


def test_dtype_rules_refused():
    with pytest.raises(ag.AetherError, match="dtype mismatch: b vs out"):
        runtime_eval(RuntimeOp.Add, _host_view((3, 5)), _host_view((3, 5), torch.float32), _host_view((3, 5)))
    with pytest.raises(ag.AetherError, match=r"dtype mismatch: a vs out \(only Assign"):
        runtime_eval(RuntimeOp.Scale, _host_view((3, 5), torch.float32), None, _host_view((3, 5)), 2.0)
    with pytest.raises(ag.AetherError, match="unsupported input dtype"):
        runtime_eval(RuntimeOp.Assign, _host_view((3, 5), torch.int32), None, _host_view((3, 5), torch.int32))
    with pytest.raises(ag.AetherError, match="runtimeEval failed on cuda"):
        runtime_eval(RuntimeOp.Add, _host_view((3, 5)), None, _host_view((3, 5)))


def test_host_memory_refused_no_host_path():
    a = _host_view((3, 5))
    with pytest.raises(ag.AetherError, match="device memory"):
        runtime_eval(RuntimeOp.Assign, a, None, _host_view((3, 5)))


# -- the reference's cases on the device -------------------------------------

@gpu
@pytest.mark.parametrize("op", [RuntimeOp.Assign, RuntimeOp.Add, RuntimeOp.Sub, RuntimeOp.Scale, RuntimeOp.AddScaled,
                                RuntimeOp.SubScaled])
def test_reference_cases(op):
    _gpu()
    a, b = _fill(3, 5)
    s = 1.75
    out = torch.full((3, 5), -1.0, dtype=torch.float64, device="cuda")
    runtime_eval(op, _dev(a), _dev(b), out, s)
    ref = po.runtime_eval(op, a, b, np.float64, s)
    assert np.array_equal(out.cpu().numpy(), ref)


@gpu
def test_casts_both_ways():
    _gpu()
    a, _ = _fill(3, 5)
    out32 = torch.full((3, 5), -1.0, dtype=torch.float32, device="cuda")
    runtime_eval(RuntimeOp.Assign, _dev(a), None, out32)
    assert np.array_equal(out32.cpu().numpy(), a.astype(np.float32))
    a32 = (np.arange(15, dtype=np.float32) * 0.5 - 1.25).reshape(3, 5)
    out64 = torch.full((3, 5), -1.0, dtype=torch.float64, device="cuda")
    runtime_eval(RuntimeOp.Assign, _dev(a32, torch.float32), None, out64)
    assert np.array_equal(out64.cpu().numpy(), a32.astype(np.float64))


@gpu
def test_strided_view_leaves_gaps():
    _gpu()
    buf_a = torch.as_tensor(np.arange(10, dtype=np.float64) * 1.5 - 3.0).cuda()
    buf_o = torch.full((10,), -1.0, dtype=torch.float64, device="cuda")
    runtime_eval(RuntimeOp.Assign, buf_a.as_strided((5,), (2,)), None, buf_o.as_strided((5,), (2,)))
    got = buf_o.cpu().numpy()
    assert np.array_equal(got[0::2], buf_a.cpu().numpy()[0::2])
    assert np.all(got[1::2] == -1.0)


def _random_view(rng, shape, dtype, pad_max=3):
    """A view of `shape` over a larger buffer: a random permutation of the
    modes in memory, random padding per mode, sometimes stride 0 (broadcast
    inputs only). Returns (tensor view, base buffer)."""
    rank = len(shape)
    order = rng.permutation(rank)
    strides = [0] * rank
    acc = 1
    for k in order[::-1]:
        strides[k] = acc
        acc *= shape[k] + int(rng.integers(0, pad_max + 1))
    size = max(1, acc)
    base = torch.empty(size + 8, dtype=dtype, device="cuda")
    off = int(rng.integers(0, 8))
    return base, off, strides


@gpu
@pytest.mark.parametrize("seed", range(12))
def test_random_strided_views(seed):
    _gpu()
    rng = np.random.default_rng(seed)
    rank = int(rng.integers(0, 7))
    shape = tuple(int(rng.integers(1, 7)) for _ in range(rank))
    op = int(rng.integers(0, 6))
    t_in = torch.float64 if rng.random() < 0.6 else torch.float32
    t_out = t_in if op != RuntimeOp.Assign else (torch.float32 if rng.random() < 0.5 else torch.float64)
    views = []
    for role in ("a", "b", "out"):
        base, off, strides = _random_view(rng, shape, t_out if role == "out" else t_in)
        if role != "out" and rank and rng.random() < 0.25:
            strides[int(rng.integers(0, rank))] = 0          # broadcast mode in an input
        if role == "out":
            base.fill_(-7.0)
        else:
            base.copy_(torch.as_tensor(rng.uniform(-5, 5, base.numel())).to(base.dtype))
        views.append((base, off, strides))
    (ba, oa, sa), (bb, ob, sb), (bo, oo, so) = views
    A = ba.as_strided(shape, sa, oa)
    B = bb.as_strided(shape, sb, ob)
    O = bo.as_strided(shape, so, oo)
    scalar = float(rng.uniform(-3, 3))
    runtime_eval(op, A, B if op in (1, 2, 4, 5) else None, O, scalar)
    npd = {torch.float64: np.float64, torch.float32: np.float32}
    ref = po.runtime_eval(op, A.cpu().numpy(), B.cpu().numpy(), npd[t_out], scalar)
    assert np.array_equal(O.cpu().numpy(), ref)
    # bytes outside the view are untouched
    touched = torch.zeros(bo.numel(), dtype=torch.bool, device="cuda")
    touched.as_strided(shape, so, oo).fill_(True)
    assert torch.all(bo[~touched] == -7.0)


@gpu
@pytest.mark.parametrize("dtypes", [(torch.float64, torch.float64), (torch.float64, torch.float32),
                                    (torch.float32, torch.float64), (torch.float32, torch.float32)])
def test_large_contiguous_and_padded(dtypes):
    _gpu()
    ti, to = dtypes
    n = (1 << 20) + 3
    g = torch.Generator(device="cuda").manual_seed(5)
    a = torch.rand((3, n), generator=g, device="cuda", dtype=torch.float64).to(ti)
    b = torch.rand((3, n), generator=g, device="cuda", dtype=torch.float64).to(ti)
    out = torch.empty((3, n), dtype=to, device="cuda")
    runtime_eval(RuntimeOp.Assign, a, None, out)
    assert torch.equal(out, a.to(to))
    if ti == to:
        runtime_eval(RuntimeOp.SubScaled, a, b, out, 0.3)
        ref = po.runtime_eval(RuntimeOp.SubScaled, a.cpu().numpy(), b.cpu().numpy(), out.cpu().numpy().dtype, 0.3)
        assert np.array_equal(out.cpu().numpy(), ref)
    # SoA planes with capacity padding: the strided kernel (pitch != n)
    cap = (n + 31) // 32 * 32
    pa = torch.zeros(3 * cap, dtype=ti, device="cuda")
    po_ = torch.full((3 * cap,), -2.0, dtype=to, device="cuda")
    va, vo = pa.as_strided((3, n), (cap, 1)), po_.as_strided((3, n), (cap, 1))
    va.copy_(a)
    runtime_eval(RuntimeOp.Assign, va, None, vo)
    assert torch.equal(vo, a.to(to))
    assert torch.all(po_.view(3, cap)[:, n:] == -2.0)


@gpu
def test_rank0_and_empty():
    _gpu()
    a = torch.tensor(2.5, dtype=torch.float64, device="cuda")
    o = torch.tensor(0.0, dtype=torch.float64, device="cuda")
    runtime_eval(RuntimeOp.Scale, a, None, o, 3.0)
    assert o.item() == 7.5
    e = torch.empty((3, 0), dtype=torch.float64, device="cuda")
    runtime_eval(RuntimeOp.Assign, e, None, e.clone())


def test_fastdiv_matches_hardware_divide(tmp_path):
    """The invariant-divisor division of the strided kernels, built for the
    host from the same header, against / and % on edge and random values."""
    import shutil
    import subprocess
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    exe = str(tmp_path / "fastdiv_check")
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", os.path.join(repo, "include"),
                    os.path.join(repo, "tests", "cpp", "fastdiv_check.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0 and "fastdiv ok" in r.stdout, r.stdout
