"""One sum plan launched on two streams at once with its own (default)
workspaces: each launch draws a separate workspace from the plan's pool, so
both results equal the serial launches' bit for bit. A launch recorded into a
CUDA graph without a caller workspace is refused rather than sharing one."""

import ctypes

import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

IR = "(plan f64 [] sum (dot (in 0 f64 [8]) (in 1 f64 [8])))"


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _args(ag, x, y, n, out):
    ops = (ag._abi.AetherOperand * 2)()
    ops[0].ptr, ops[0].pitch = x.data.data_ptr(), x.capacity
    ops[1].ptr, ops[1].pitch = y.data.data_ptr(), y.capacity
    a = ag._abi.AetherLaunch()
    a.n = n
    a.operands = ops
    a.n_operands = 2
    a.reduce_out = out.data_ptr()
    return a, ops


def test_sum_plan_on_two_streams_matches_serial():
    import aether_gb300 as ag
    L = ag._abi.lib()
    n = 1 << 22
    xs = [ag.Array("f64", (8,), n) for _ in range(4)]
    for k, x in enumerate(xs):
        ag.assign(x, ag.Generator(100 + k).uniform(8, -1.0, 1.0))
    plan = ag.get_plan(IR)
    torch.cuda.synchronize()

    # serial reference: one launch at a time on the current stream
    serial = []
    for (x, y) in ((xs[0], xs[1]), (xs[2], xs[3])):
        out = torch.zeros(2, dtype=torch.float64, device="cuda")
        a, keep = _args(ag, x, y, n, out)
        ag._abi.check(L.aether_plan_launch(plan.handle, ctypes.byref(a), None))
        torch.cuda.synchronize()
        serial.append(out.cpu())

    # concurrent: the two sums back to back on two streams, several rounds
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    for _ in range(5):
        outs = [torch.full((2,), float("nan"), dtype=torch.float64, device="cuda") for _ in range(2)]
        torch.cuda.synchronize()
        keep = []
        for out, (x, y), s in zip(outs, ((xs[0], xs[1]), (xs[2], xs[3])), (s1, s2)):
            a, ops = _args(ag, x, y, n, out)
            keep.append((a, ops))
            ag._abi.check(L.aether_plan_launch(plan.handle, ctypes.byref(a), ctypes.c_void_p(s.cuda_stream)))
        torch.cuda.synchronize()
        for got, want in zip(outs, serial):
            assert torch.equal(got.cpu(), want)


def test_sum_plan_capture_needs_a_workspace():
    import aether_gb300 as ag
    L = ag._abi.lib()
    n = 4096
    x = ag.Array("f64", (8,), n)
    y = ag.Array("f64", (8,), n)
    ag.assign(x, ag.Generator(1).uniform(8, -1.0, 1.0))
    ag.assign(y, ag.Generator(2).uniform(8, -1.0, 1.0))
    plan = ag.get_plan(IR)
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    ws_bytes = ctypes.c_uint64()
    ag._abi.check(L.aether_plan_workspace_size(plan.handle, n, ctypes.byref(ws_bytes)))
    ws = torch.empty(ws_bytes.value, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        a, keep = _args(ag, x, y, n, out)
        rc = L.aether_plan_launch(plan.handle, ctypes.byref(a), ctypes.c_void_p(s.cuda_stream))
        refused = (rc, L.aether_last_error())
        b, keep2 = _args(ag, x, y, n, out)
        b.workspace = ws.data_ptr()
        b.workspace_bytes = ws_bytes.value
        ag._abi.check(L.aether_plan_launch(plan.handle, ctypes.byref(b), ctypes.c_void_p(s.cuda_stream)))
    assert refused[0] == 1 and b"needs its own workspace" in refused[1]
    g.replay()
    torch.cuda.synchronize()
    got = out.cpu()
    ref = torch.zeros(2, dtype=torch.float64, device="cuda")
    c, keep3 = _args(ag, x, y, n, ref)
    ag._abi.check(L.aether_plan_launch(plan.handle, ctypes.byref(c), None))
    torch.cuda.synchronize()
    assert torch.equal(got, ref.cpu())
