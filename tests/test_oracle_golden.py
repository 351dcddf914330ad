"""The oracle pinned against the reference: golden rows of
tests/random/golden_random.h and outputs of the reference headers themselves
(tests/golden/make_golden.py). CPU only."""

import numpy as np
import pytest

from conftest import ulp_diff


def test_philox_core_rows_exact(oracle, philox_golden):
    L = oracle.lib()
    rows = philox_golden["core"]
    assert len(rows) == 315
    for r in rows:
        s, g, c = r["seed"], r["global"], r["counter"]
        assert L.orc_random_bits64(s, g, c) == r["bits64"]
        assert np.float64(L.orc_uniform01_f64(s, g, c)).view(np.uint64) == r["uniform_double_bits"]
        assert np.float32(L.orc_uniform01_f32(s, g, c)).view(np.uint32) == r["uniform_float_bits"]


def test_philox_normal_rows_tolerance(oracle, philox_golden):
    # TIER-TOL of the reference: abs+rel 1e-12 (double) and 1e-5 (float).
    L = oracle.lib()
    td, tf = philox_golden["normal_double_tol"], philox_golden["normal_float_tol"]
    for r in philox_golden["core"]:
        s, g, c = r["seed"], r["global"], r["counter"]
        nd = L.orc_normal_f64(s, g, c)
        assert abs(nd - r["normal_double"]) <= td * (1 + abs(r["normal_double"]))
        nf = L.orc_normal_f32(s, g, c)
        assert abs(nf - r["normal_float"]) <= tf * (1 + abs(r["normal_float"]))


def test_keying_rows_exact(oracle, philox_golden):
    for k in philox_golden["keys"]:
        key = oracle.generator_key(k["seed"], k["stream_id"])
        assert key == k["key"]
        assert oracle.substream_key(key, k["substream_k"]) == k["substream_key"]


def test_python_keying_matches_oracle(oracle, philox_golden):
    from aether_gb300.expr import Generator
    for k in philox_golden["keys"]:
        g = Generator(k["seed"], k["stream_id"])
        assert g.key == k["key"]
        assert g.substream(k["substream_k"]).key == k["substream_key"]


def _fill(oracle, seed, sub, lo, hi, comps, n):
    return oracle.fill_uniform_f64(oracle.substream_key(oracle.generator_key(seed), sub), lo, hi, comps, n)


def test_uniform_fills_match_reference(oracle, ref_cases):
    for sub, name in enumerate(["cfg1_a", "cfg1_b", "cfg1_c"]):
        assert np.array_equal(_fill(oracle, 42, sub, -1.0, 1.0, 3, 1000), ref_cases[name])
    for sub, name in enumerate(["cfg2a_a", "cfg2a_b", "cfg2a_c", "cfg2a_d0"]):
        assert np.array_equal(_fill(oracle, 7, sub, -4.0, 4.0, 3, 1000), ref_cases[name])
    k3 = oracle.substream_key(oracle.generator_key(3), 0)
    assert np.array_equal(oracle.fill_uniform_f32(k3, -1.0, 1.0, 3, 1000), ref_cases["f32_uniform"])


def test_normal_fill_matches_reference(oracle, ref_cases):
    k = oracle.substream_key(oracle.generator_key(7), 4)
    x = oracle.fill_normal_f64(k, 0.0, 1.0, 1, 4096)
    # Same glibc as the one that ran the reference here: bit-exact; on another
    # libm the double normals may move by an ulp of log/sqrt/sin.
    assert ulp_diff(x, ref_cases["cfg2b_x"]).max() <= 2


CFG1 = ("(plan f64 [3] set (add (add (in 0 f64 [3]) (mul (in 1 f64 [3]) (in 2 f64 [3]))) "
        "(mul (sin (in 0 f64 [3])) (exp (scale (mul (in 2 f64 [3]) (in 2 f64 [3])) (sc 0))))))")
CFG2A = ("(plan f64 [3] set (add (mul (sqrt (add (mul (in 0 f64 [3]) (in 0 f64 [3])) (mul (in 1 f64 [3]) "
         "(in 1 f64 [3])))) (log1p (abs (in 2 f64 [3])))) (rsqrt (add (bcast (sc 0) [3]) (mul (in 3 f64 [3]) "
         "(in 3 f64 [3]))))))")


def test_interpreter_config1_config2a_exact(oracle, ref_cases):
    z = ref_cases
    d, _ = oracle.eval_ir(CFG1, 1000, [z["cfg1_a"], z["cfg1_b"], z["cfg1_c"]], scalars=[-1.0], dst_comps=3)
    assert ulp_diff(d, z["cfg1_d"]).max() <= 1
    d, _ = oracle.eval_ir(CFG2A, 1000, [z["cfg2a_a"], z["cfg2a_b"], z["cfg2a_c"], z["cfg2a_d0"]], scalars=[1.0],
                          dst_comps=3)
    assert ulp_diff(d, z["cfg2a_d"]).max() <= 1


def test_config_loops_match_interpreter(oracle, ref_cases):
    z = ref_cases
    a, b, c = (np.ascontiguousarray(z[k]) for k in ("cfg1_a", "cfg1_b", "cfg1_c"))
    d, _ = oracle.eval_ir(CFG1, 1000, [a, b, c], scalars=[-1.0], dst_comps=3)
    assert np.array_equal(oracle.cfg1(a, b, c), d)
    a, b, c, d0 = (np.ascontiguousarray(z[k]) for k in ("cfg2a_a", "cfg2a_b", "cfg2a_c", "cfg2a_d0"))
    d, _ = oracle.eval_ir(CFG2A, 1000, [a, b, c, d0], scalars=[1.0], dst_comps=3)
    assert np.array_equal(oracle.cfg2a(a, b, c, d0), d)


LEAVES = {
    "leaf_lognormal": "(plan f64 [2] set (lognormal 0 (sc 0) (sc 1) 2))",
    "leaf_exponential": "(plan f64 [2] set (exponential 0 (sc 0) 2))",
    "leaf_bernoulli": "(plan f64 [2] set (bernoulli 0 (sc 0) 2))",
}
LEAF_SCALARS = {"leaf_lognormal": [0.1, 0.5], "leaf_exponential": [1.5], "leaf_bernoulli": [0.3]}


@pytest.mark.parametrize("name", sorted(LEAVES))
def test_distribution_leaves_match_reference(oracle, ref_cases, name):
    key = oracle.generator_key(11)
    d, _ = oracle.eval_ir(LEAVES[name], 1000, [], scalars=LEAF_SCALARS[name], keys=[key], dst_comps=2)
    assert ulp_diff(d, ref_cases[name]).max() <= 1


def test_uniform_item_parameters(oracle, ref_cases):
    key = oracle.generator_key(11)
    ir = "(plan f64 [2] set (uniform 0 (stack (sc 0) (sc 1)) (stack (sc 2) (sc 3)) 2))"
    d, _ = oracle.eval_ir(ir, 1000, [], scalars=[-2.0, 10.0, 2.0, 11.0], keys=[key], dst_comps=2)
    assert np.array_equal(d, ref_cases["leaf_uniform_item"])


ITEM_LEAVES = {
    # (substream, IR, scalars): per-component parameters as stacked scalars,
    # the Items of the reference driver's Generator(21) cases
    "leafi_normal": (0, "(plan f64 [3] set (normal 0 (stack (sc 0) (sc 1) (sc 2)) (stack (sc 3) (sc 4) (sc 5)) 3))",
                     [-1.0, 0.0, 2.5, 0.5, 1.0, 3.0]),
    "leafi_lognormal": (1, "(plan f64 [3] set (lognormal 0 (stack (sc 0) (sc 1) (sc 2)) "
                           "(stack (sc 3) (sc 4) (sc 5)) 3))", [-1.0, 0.0, 2.5, 0.5, 1.0, 3.0]),
    "leafi_exponential": (2, "(plan f64 [3] set (exponential 0 (stack (sc 0) (sc 1) (sc 2)) 3))", [0.5, 2.0, 8.0]),
    "leafi_bernoulli": (3, "(plan f64 [3] set (bernoulli 0 (stack (sc 0) (sc 1) (sc 2)) 3))", [0.1, 0.5, 0.9]),
}


@pytest.mark.parametrize("name", sorted(ITEM_LEAVES))
def test_item_parameter_leaves_match_reference(oracle, ref_cases, name):
    sub, ir, scalars = ITEM_LEAVES[name]
    key = oracle.substream_key(oracle.generator_key(21), sub)
    d, _ = oracle.eval_ir(ir, 1000, [], scalars=scalars, keys=[key], dst_comps=3)
    assert ulp_diff(d, ref_cases[name]).max() <= 1


GEO = {
    "geo_cross": ("(plan f64 [3] set (cross (in 0 f64 [3]) (in 1 f64 [3])))", ["geo_a", "geo_b"], 3),
    "geo_qrot": ("(plan f64 [3] set (qrot (in 0 f64 [4]) (in 1 f64 [3])))", ["geo_q", "geo_a"], 3),
    "geo_qmul": ("(plan f64 [4] set (qmul (in 0 f64 [4]) (in 1 f64 [4])))", ["geo_q", "geo_p"], 4),
    "geo_unit_item": ("(plan f64 [3] set (unit (in 0 f64 [3])))", ["geo_a"], 3),
    "geo_unit": ("(plan f64 [3] set (scale (in 0 f64 [3]) (at0 (rnorm (in 0 f64 [3])))))", ["geo_a"], 3),
    "geo_inv": ("(plan f64 [3,3] set (inv (in 0 f64 [3,3])))", ["geo_m"], 9),
    "geo_det": ("(plan f64 [] set (det (in 0 f64 [3,3])))", ["geo_m"], 1),
    "geo_trace": ("(plan f64 [] set (trace (in 0 f64 [3,3])))", ["geo_m"], 1),
}


@pytest.mark.parametrize("name", sorted(GEO))
def test_geometry_nodes_exact(oracle, ref_cases, name):
    ir, ins, comps = GEO[name]
    n = ref_cases[ins[0]].shape[1]
    d, _ = oracle.eval_ir(ir, n, [ref_cases[k] for k in ins], dst_comps=comps)
    assert np.array_equal(d, ref_cases[name]), name


def test_dot8_fold_order_exact(oracle, ref_cases):
    z = ref_cases
    d, _ = oracle.eval_ir("(plan f64 [] set (dot (in 0 f64 [8]) (in 1 f64 [8])))", 600, [z["dot_x"], z["dot_y"]])
    assert np.array_equal(d, z["dot_d"])
    f, _ = oracle.eval_ir("(plan f32 [] set (dot (in 0 f32 [8]) (in 1 f32 [8])))", 600, [z["dot_xf"], z["dot_yf"]],
                          dst_dtype=np.float32)
    assert np.array_equal(f, z["dot_f"])


CW = {
    "cw_sqrt": "(sqrt X)", "cw_rsqrt": "(rsqrt X)", "cw_exp": "(exp X)", "cw_log": "(log X)", "cw_sin": "(sin X)",
    "cw_cos": "(cos X)", "cw_tan": "(tan X)", "cw_asin": "(asin X)", "cw_acos": "(acos X)", "cw_atan": "(atan X)",
    "cw_tanh": "(tanh X)", "cw_abs": "(abs X)", "cw_sign": "(sign X)", "cw_mins": "(mins X (sc 0))",
    "cw_maxs": "(maxs X (sc 1))", "cw_min": "(min X Y)", "cw_max": "(max X Y)", "cw_clamp": "(clamp X (sc 2) (sc 3))",
    "cw_div": "(div X Y)", "cw_pow": "(pow (abs X) Y)", "cw_pows": "(pows (abs X) (sc 4))",
    "cw_scale": "(scale X (sc 5))", "cw_divs": "(scale X (sc 6))", "cw_sub": "(sub X Y)",
}
CW_SCALARS = [0.25, -0.25, -0.5, 0.5, 1.75, 2.5, 1.0 / 3.0]


@pytest.mark.parametrize("name", sorted(CW))
def test_elementwise_nodes_exact(oracle, ref_cases, name):
    x, y = ref_cases["cw_x"], ref_cases["cw_y"]
    body = CW[name].replace("X", "(in 0 f64 [1])").replace("Y", "(in 1 f64 [1])")
    d, _ = oracle.eval_ir("(plan f64 [1] set %s)" % body, x.shape[1], [x, y], scalars=CW_SCALARS)
    assert ulp_diff(d, ref_cases[name]).max() <= 0 or np.array_equal(d, ref_cases[name], equal_nan=True), name


def test_reduce32_twin(oracle):
    import ctypes
    rng = np.random.default_rng(5)
    h = rng.standard_normal(32) * 10.0 ** rng.integers(-8, 8, 32)
    c = np.zeros(32)
    oh, oc = ctypes.c_double(), ctypes.c_double()
    oracle.lib().orc_reduce32_f64(h.ctypes.data, c.ctypes.data, ctypes.byref(oh), ctypes.byref(oc))
    exact = sum(map(float, h))   # float sum is not exact; compare with fsum
    import math
    assert abs((oh.value + oc.value) - math.fsum(h)) <= 1e-16 * np.abs(h).sum()
