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
