"""aether_plan_launch_noalloc: a sum plan launched with the library's static
scratch instead of an allocation, for callers that cannot call cudaMalloc
where they launch (fixed device-memory budgets, latency loops). Checked
through the C-ABI against aether_plan_launch on the same plan, on two calls in
a row, at the largest size the scratch holds and one chunk beyond it. This
file is collected last on purpose."""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _setup(n):
    import aether_gb300 as ag
    x = ag.Array("f64", (8,), n)
    y = ag.Array("f64", (8,), n)
    ag.assign(x, ag.Generator(41).uniform(8, -1.0, 1.0))
    ag.assign(y, ag.Generator(42).uniform(8, -1.0, 1.0))
    return ag, x, y


def _launch_args(ag, x, y, n, out):
    ops = (ag._abi.AetherOperand * 2)()
    ops[0].ptr, ops[0].pitch = x.data.data_ptr(), x.capacity
    ops[1].ptr, ops[1].pitch = y.data.data_ptr(), y.capacity
    a = ag._abi.AetherLaunch()
    a.n = n
    a.operands = ops
    a.n_operands = 2
    a.reduce_out = out.data_ptr()
    return a, ops


IR = "(plan f64 [] sum (dot (in 0 f64 [8]) (in 1 f64 [8])))"


def _check_two_calls(n):
    ag, x, y = _setup(n)
    L = ag._abi.lib()
    plan = ag.get_plan(IR)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ref = torch.zeros(2, dtype=torch.float64, device="cuda")
    a, keep = _launch_args(ag, x, y, n, ref)
    ag._abi.check(L.aether_plan_launch(plan.handle, ctypes.byref(a), stream))
    torch.cuda.synchronize()
    r = ref.cpu().numpy()
    absmag = float(torch.sum(torch.abs(x.data[:, :n] * y.data[:, :n])).item())
    for _ in range(2):
        out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
        b, keep2 = _launch_args(ag, x, y, n, out)
        ag._abi.check(L.aether_plan_launch_noalloc(plan.handle, ctypes.byref(b), stream))
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        # same kernel, same chunk tree: the compensated sums agree to the
        # tolerance of the other sum tests (and in practice bit for bit)
        assert abs((got[0] + got[1]) - (r[0] + r[1])) <= 4e-16 * absmag


def test_noalloc_sum_matches_plan_launch_on_two_calls():
    _check_two_calls(300001)


def _largest_accepted(ag, plan):
    # the scratch need grows by 16 bytes per chunk of samples: find the
    # largest n whose need fits the 1 MiB array
    L = ag._abi.lib()

    def need(n):
        b = ctypes.c_uint64()
        ag._abi.check(L.aether_plan_workspace_size(plan.handle, n, ctypes.byref(b)))
        return b.value

    lo, hi = 1, 1 << 31
    assert need(lo) <= 1 << 20 < need(hi)
    while hi - lo > 1:
        mid = (lo + hi) // 2
        lo, hi = (mid, hi) if need(mid) <= 1 << 20 else (lo, mid)
    return lo


def test_noalloc_edge_of_the_scratch():
    import aether_gb300 as ag
    L = ag._abi.lib()
    plan = ag.get_plan(IR)
    n_max = _largest_accepted(ag, plan)
    _check_two_calls(n_max)
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    a = ag._abi.AetherLaunch()
    a.n = n_max + 1   # one chunk more than the scratch holds
    a.reduce_out = out.data_ptr()
    rc = L.aether_plan_launch_noalloc(plan.handle, ctypes.byref(a), None)
    assert rc == 1
    assert b"static scratch holds" in L.aether_last_error()


def test_noalloc_refuses_sizes_beyond_its_scratch():
    import aether_gb300 as ag
    L = ag._abi.lib()
    plan = ag.get_plan(IR)
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    a = ag._abi.AetherLaunch()
    a.n = 1 << 30   # needs more than the 1 MiB of scratch
    a.reduce_out = out.data_ptr()
    rc = L.aether_plan_launch_noalloc(plan.handle, ctypes.byref(a), None)
    assert rc == 1
    assert b"static scratch holds" in L.aether_last_error()


def test_noalloc_refuses_plans_without_scratch():
    import aether_gb300 as ag
    L = ag._abi.lib()
    plan = ag.get_plan("(plan f64 [8] set (in 0 f64 [8]))")
    a = ag._abi.AetherLaunch()
    a.n = 10
    rc = L.aether_plan_launch_noalloc(plan.handle, ctypes.byref(a), None)
    assert rc == 1 and b"only sum plans" in L.aether_last_error()
