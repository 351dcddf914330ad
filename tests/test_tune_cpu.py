"""Autotuner cache logic on the host (tune.py): keys follow the plan, the
lowering mode and the code version; stored winners come back; the shipped
table is layered under the user cache and can be switched off."""

import json

import pytest

import aether_gb300 as ag
from aether_gb300 import tune
from aether_gb300.expr import IrContext, Operand, plan_text


def _ir(expr_fn):
    a = Operand(0x10000, 1024, "f64", (3,))
    return plan_text("f64", (3,), "set", expr_fn(a), IrContext())


@pytest.fixture
def cache(tmp_path, monkeypatch):
    path = tmp_path / "tune.json"
    monkeypatch.setenv("AETHER_GB300_TUNE_CACHE", str(path))
    monkeypatch.setenv("AETHER_GB300_TUNE_SHIPPED", "0")
    monkeypatch.setattr(tune, "_device_name", lambda: "test-device")
    return path


def test_keys_follow_plan_and_mode(cache):
    ir1 = _ir(lambda a: ag.cwiseSqrt(a * a))
    ir2 = _ir(lambda a: ag.cwiseLog1p(ag.cwiseAbs(a)))
    assert tune._key(ir1, 1, -1) == tune._key(ir1, 1, -1)
    assert tune._key(ir1, 1, -1) != tune._key(ir2, 1, -1)
    assert tune._key(ir1, 0, -1) != tune._key(ir1, 1, -1)
    # the generated kernel text is part of the key
    assert tune._generated_digest(ir1, 1, -1) != tune._generated_digest(ir1, 0, -1)


def test_store_and_reload(cache):
    ir = _ir(lambda a: a * 2.0)
    assert tune.tuned(ir, 1) is None
    low = dict(block=256, ipt=2, vec=1, min_blocks=3)
    tune.store(tune._key(ir, 1, -1), {"lowering": low, "ms": 1.0, "registers": 40, "blocks_per_sm": 3,
                                      "candidates": 1})
    assert tune.tuned(ir, 1) == low
    assert json.loads(cache.read_text())


def test_shipped_table_under_the_user_cache(cache, monkeypatch, tmp_path):
    ir = _ir(lambda a: a + a)
    key = tune._key(ir, 1, -1)
    shipped = tmp_path / "shipped.json"
    shipped.write_text(json.dumps({key: {"lowering": {"block": 128, "ipt": 1, "vec": 0, "min_blocks": 0}}}))
    monkeypatch.setattr(tune, "SHIPPED", str(shipped))
    assert tune.tuned(ir, 1) is None                       # switched off
    monkeypatch.setenv("AETHER_GB300_TUNE_SHIPPED", "1")
    assert tune.tuned(ir, 1)["block"] == 128               # shipped entry
    tune.store(key, {"lowering": {"block": 512, "ipt": 2, "vec": 0, "min_blocks": 0}})
    assert tune.tuned(ir, 1)["block"] == 512               # the user cache wins


def test_regimes_keep_separate_winners(cache):
    """A plan's serving winner (2^21-sample requests) and its whole-array
    winner are separate entries; the whole-array key is the regime-free one."""
    ir = _ir(lambda a: a * 3.0)
    assert tune._key(ir, 1, -1, "") == tune._key(ir, 1, -1)
    assert tune._key(ir, 1, -1, "serve") == tune.regime_key(tune._key(ir, 1, -1), "serve")
    assert tune._key(ir, 1, -1, "serve") != tune._key(ir, 1, -1)
    tune.store(tune._key(ir, 1, -1), {"lowering": {"block": 512, "ipt": 1, "vec": 0, "min_blocks": 0}})
    assert tune.tuned(ir, 1, regime="serve") is None
    tune.store(tune._key(ir, 1, -1, "serve"), {"lowering": {"block": 128, "ipt": 2, "vec": 1, "min_blocks": 0}})
    assert tune.tuned(ir, 1)["block"] == 512
    assert tune.tuned(ir, 1, regime="serve")["block"] == 128
