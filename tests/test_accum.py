"""Per-sample compensated accumulation (accum/AccumPlane.h): many terms
added into a plane in separate launches deliver the exactly rounded sum
(compared with math.fsum per sample), where a plain += drifts; atomic
accumulation from two streams at once delivers the same; the plan text is
refused for non-f64 planes and in the precision form."""

import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import aether_gb300 as ag
from aether_gb300 import _abi


def test_accumulation_plans_generate_and_refuse_bad_forms():
    ok = "(plan f64 [3] acc (mul (in 0 f64 [3]) (in 1 f64 [3])))"
    assert "two_sum_err" in _abi.generate(ok, _abi.lowering(math=0))
    assert "atomicAdd" in _abi.generate(ok.replace(" acc ", " accat "), _abi.lowering(math=1))
    with pytest.raises(ag.AetherError, match="accumulation planes are f64"):
        _abi.generate("(plan f32 [3] acc (in 0 f32 [3]))", _abi.lowering(math=2))


def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _terms(n, k, seed):
    """Per sample: a large B, k-2 terms of magnitude 1e-3..1e3 with mixed
    signs, then -B. The exact sum is that of the small terms, which a plain
    running sum mostly loses under B."""
    rng = np.random.default_rng(seed)
    small = 10.0 ** rng.uniform(-3, 3, size=(k - 2, 3, n)) * rng.choice([-1.0, 1.0], size=(k - 2, 3, n))
    big = 10.0 ** rng.uniform(6, 9, size=(1, 3, n)) * rng.choice([-1.0, 1.0], size=(1, 3, n))
    return np.concatenate([big, small, -big])


@pytest.mark.gpu
@pytest.mark.parametrize("math_mode", [0, 1])
def test_compensated_plane_delivers_the_exact_sum(math_mode):
    _gpu()
    n, k = 777, 40
    terms = _terms(n, k, 5)
    plane = ag.AccumPlane((3,), n)
    plain = ag.Array("f64", (3,), n)
    t = ag.Array("f64", (3,), n)
    v = ag.Array("f64", (3,), n)
    added = []
    for j in range(k):
        t.upload(terms[j])
        plane.add(t.view() * 1.0, math=math_mode)
        ag.assign_add(plain, t.view() * 1.0, math=math_mode)
        # the term exactly as the plan computes it (emulated FP64 rounds its
        # inputs to 2^-48, so it need not equal the uploaded value)
        ag.assign(v, t.view() * 1.0, math=math_mode)
        added.append(v.host().copy())
    torch.cuda.synchronize()
    got = plane.delivered().host()
    added = np.array(added)
    exact = np.array([[math.fsum(added[:, c, i]) for i in range(n)] for c in range(3)])
    ulp = np.spacing(np.abs(exact))
    err_plane = np.abs(got - exact) / ulp
    err_plain = np.abs(plain.host() - exact) / ulp
    assert err_plane.max() <= 2.0, err_plane.max()
    assert err_plain.max() > 1e3   # the workload does defeat a plain running sum


@pytest.mark.gpu
def test_atomic_accumulation_from_two_streams():
    _gpu()
    n, k = 4097, 24
    terms = _terms(n, k, 9)
    plane = ag.AccumPlane((3,), n)
    arrs = []
    for j in range(k):
        a = ag.Array("f64", (3,), n)
        a.upload(terms[j])
        arrs.append(a)
    torch.cuda.synchronize()
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    for j, a in enumerate(arrs):
        s = s1 if j % 2 else s2
        plane.add(a.view() * 1.0, atomic=True, stream=s.cuda_stream)
    s1.synchronize()
    s2.synchronize()
    got = plane.delivered().host()
    exact = np.array([[math.fsum(terms[:, c, i]) for i in range(n)] for c in range(3)])
    err = np.abs(got - exact) / np.spacing(np.abs(exact))
    assert err.max() <= 2.0, err.max()


def _profiles(bodies, n, seed):
    """Two families of per-body terms (bodies x 3 x n): a magnitude spread
    over eleven decades with mixed signs, and a cancellation family of
    +-A (1 - d) pairs whose differences d run from 0 to 1e-3."""
    rng = np.random.default_rng(seed)
    jit = 1.0 + 0.4375 * rng.random((bodies, 3, n))
    rel = np.array([1.0, 1.1e-3, 3.1e-6, 6.0e-7, 5.0e-8, 1.0e-10, 4.0e-12, 8.0e-13])
    sign = rng.choice([-1.0, 1.0], size=(bodies, 3, n))
    sign[0] = 1.0
    spread = 8.0e-3 * rel[np.arange(bodies) % 8][:, None, None] * jit * sign
    dl = np.array([0.0, 2.22e-16, 9.1e-13, 9.3e-10, 9.5e-7, 9.8e-4])[np.arange(n) % 6]
    A = 1.0e-2 * jit
    cancel = np.where((np.arange(bodies) % 2 == 0)[:, None, None], A, -A * (1.0 - dl))
    return {"spread": spread, "cancel": cancel}


@pytest.mark.gpu
@pytest.mark.parametrize("profile", ["spread", "cancel"])
def test_atomic_accumulation_bitwise_under_permuted_launch_orders(profile):
    """One launch per body in four orders (identity, reverse, two shuffles),
    alternating two streams: every order delivers the same bits
    (tests/test_AccumOrderPermutation.cu), within an ulp of the exact sum."""
    _gpu()
    bodies, n = 8, 128
    terms = _profiles(bodies, n, 11)[profile]
    arrs = []
    for k in range(bodies):
        a = ag.Array("f64", (3,), n)
        a.upload(terms[k])
        arrs.append(a)
    torch.cuda.synchronize()
    rng = np.random.default_rng(3)
    orders = [list(range(bodies)), list(reversed(range(bodies))), list(rng.permutation(bodies)),
              list(rng.permutation(bodies))]
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    delivered = []
    for order in orders:
        plane = ag.AccumPlane((3,), n)
        torch.cuda.synchronize()
        for j, k in enumerate(order):
            plane.add(arrs[k].view() * 1.0, atomic=True, stream=(s1 if j % 2 else s2).cuda_stream)
        s1.synchronize()
        s2.synchronize()
        delivered.append(plane.delivered().host().copy())
    for d in delivered[1:]:
        assert np.array_equal(d.view(np.int64), delivered[0].view(np.int64))
    exact = np.array([[math.fsum(terms[:, c, i]) for i in range(n)] for c in range(3)])
    nz = exact != 0.0
    err = np.abs(delivered[0][nz] - exact[nz]) / np.spacing(np.abs(exact[nz]))
    assert err.max() <= 1.0, err.max()
    assert np.all(delivered[0][~nz] == 0.0)
