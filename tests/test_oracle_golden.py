"""The CPU oracle and the product's host-side tables against golden data
parsed from the reference (tests/golden/make_golden.py) and against the
invariants the velocity sets must satisfy."""
import ctypes as C
import ctypes.util
import json
import math
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "velocity_sets.json")))["sets"]
DEFAULTS = json.load(open(os.path.join(HERE, "golden", "lbm_defaults.json")))["defaults"]
FLOW = {"D2Q9": 2, "D3Q15": 3, "D3Q19": 4, "D3Q27": 5}
THERMAL_OF = {"D2Q9": "D2Q5", "D3Q15": "D3Q7", "D3Q19": "D3Q7", "D3Q27": "D3Q7"}


@pytest.mark.parametrize("name", sorted(FLOW))
def test_product_tables_match_reference_text(product_lib, name):
    import boltzmannfluids_gb300 as bf
    t = bf.get_velosity_vectors(FLOW[name])
    g = GOLD[name]
    assert t.shape == (len(g), 4)
    for row, gr in zip(t, g):
        assert list(row[:3]) == gr["c"]
        # the reference uploads float(double fraction): bit-exact FP32 weights
        assert row[3] == np.float32(gr["w_num"] / gr["w_den"])
    tt = bf.get_velosity_vectors(FLOW[name], thermal=True)
    gt = GOLD[THERMAL_OF[name]]
    for row, gr in zip(tt, gt):
        assert list(row[:3]) == gr["c"]
        assert row[3] == np.float32(gr["w_num"] / gr["w_den"])


@pytest.mark.parametrize("name", sorted(GOLD))
def test_velocity_set_invariants(name):
    rows = GOLD[name]
    c = np.array([r["c"] for r in rows], float)
    from fractions import Fraction
    w = [Fraction(r["w_num"], r["w_den"]) for r in rows]
    assert sum(w) == 1
    for a in range(3):
        assert sum(wi * int(ci[a]) for wi, ci in zip(w, c)) == 0
    # opposite directions in adjacent (odd, odd+1) pairs, as collide.comp:219-222 assumes
    for i in range(1, len(rows), 2):
        assert np.all(c[i] == -c[i + 1])
        assert w[i] == w[i + 1]
    if name in ("D2Q5", "D3Q7"):
        return
    dims = 2 if name == "D2Q9" else 3
    for a in range(dims):
        for b in range(dims):
            s = sum(wi * int(ci[a]) * int(ci[b]) for wi, ci in zip(w, c))
            assert s == (Fraction(1, 3) if a == b else 0)


def test_reference_defaults_are_the_abi_defaults(product_lib):
    import boltzmannfluids_gb300.lbm as L
    import ctypes as C
    d = L._InitDesc()
    product_lib.bf_init_desc_default(C.byref(d))
    assert d.velocity_limit == np.float32(DEFAULTS["velocity_limit"])
    assert d.velocity_limit_extreme == np.float32(DEFAULTS["velocity_limit_extreme"])
    assert d.relaxation_time == np.float32(DEFAULTS["relaxation_time"])
    assert d.thermal_expansion_coefficient == np.float32(DEFAULTS["thermal_expension_coeficient"])
    assert d.intermolecular_interaction_strength == np.float32(DEFAULTS["intermolecular_interaction_strength"])
    assert d.thermal_relaxation_time == np.float32(DEFAULTS["initialize_fields_thermal_relaxation_time"])


def reference_bits(count):
    # LBM.cpp:569, evaluated with Python floats
    if count <= 1:
        return 0
    return int(2 ** math.ceil(math.log2(math.ceil(math.log2(count)))))


def test_bits_per_boundry_table(product_lib, oracle_mod):
    import boltzmannfluids_gb300 as bf
    for n in range(1, 257):
        b = reference_bits(n)
        assert bf.bits_per_boundry(n) == b
        assert oracle_mod.bits_per_boundry(n) == b
        assert b in (0, 1, 2, 4, 8)
        if n > 1:
            assert (1 << b) >= n or b == 8


@pytest.mark.parametrize("bits", [1, 2, 4, 8])
def test_boundary_packing_bit_exact(product_lib, oracle_mod, bits):
    import boltzmannfluids_gb300 as bf
    rng = np.random.default_rng(bits)
    for n in (1, 7, 31, 32, 33, 1000, 4099):
        ids = rng.integers(0, 1 << bits, n).astype(np.uint32)
        a = bf.pack_boundries(ids, bits)
        o = oracle_mod.pack_boundries(ids, bits)
        assert a.dtype == np.uint32 and np.array_equal(a, o)
        # unpack as the shader does (collide.comp:401-418)
        for v in range(n):
            b0 = v * bits
            got = (int(a[b0 // 32]) >> (b0 % 32)) & ((1 << bits) - 1)
            assert got == ids[v]


def test_half_codec_matches_ieee_rne(oracle_mod):
    lib = oracle_mod.load()
    rng = np.random.default_rng(0)
    vals = np.concatenate([rng.standard_normal(20000).astype(np.float32) * 10 ** rng.uniform(-9, 5, 20000).astype(np.float32),
                           np.array([0.0, -0.0, 65504, 65519.99, 65520, 6.1e-5, 5.96e-8, 2.98e-8, 1e-10], np.float32)])
    for v in vals:
        h = lib.orc32_f32_to_f16(float(v))
        assert h == int(np.float32(v).astype(np.float16).view(np.uint16)), v
        back = lib.orc32_f16_to_f32(h)
        assert np.float32(back) == np.float32(np.float16(v)) or (np.isinf(back) and np.isinf(np.float16(v)))


def test_scaled_half_codec(oracle_mod):
    """fp16c holds g = f - w as the IEEE half of g * 2^12: the round trip is
    half rounding of the scaled value, exact powers of two survive, and small
    shifted populations keep the half's relative precision where fp16s (the
    half of g itself) turns subnormal."""
    lib = oracle_mod.load()
    rng = np.random.default_rng(1)
    xs = (rng.standard_normal(20000) * 10.0 ** rng.uniform(-8, 0.5, 20000)).astype(np.float32)
    for x in xs:
        got = lib.orc32_fp16c_round(float(x))
        want = np.float32(np.float16(np.float32(x) * np.float32(4096.0))) / np.float32(4096.0)
        assert np.float32(got) == want, x
    for k in range(-26, 4):
        assert lib.orc32_fp16c_round(2.0 ** k) == 2.0 ** k
    # relative error of the round trip at |g| = 1e-6: 2^-11 for fp16c, far more for fp16s
    g = np.float32(1.2345e-6)
    e_c = abs(lib.orc32_fp16c_round(float(g)) - g) / g
    e_s = abs(lib.orc32_f16_to_f32(lib.orc32_f32_to_f16(float(g))) - g) / g
    assert e_c <= 2.0 ** -11 and e_s > 10 * e_c


def test_exp_f32_error_bound(oracle_mod):
    """psi = 1 - exp(-rho) uses one hand-written exp (Cody-Waite reduction,
    degree-7 Taylor polynomial) in the kernels and the oracle.  Over the
    densities a flow reaches, rho in [0, 10], it stays within 1.5 ulp of the
    exact exponential and within 2 ulp of the C library's expf."""
    lib = oracle_mod.load()
    libm = C.CDLL(ctypes.util.find_library("m") or "libm.so.6")
    libm.expf.argtypes = [C.c_float]
    libm.expf.restype = C.c_float
    rho = np.concatenate([np.linspace(0, 10, 50001), np.random.default_rng(3).uniform(0, 10, 20000)]).astype(np.float32)
    got = np.array([lib.orc32_exp_f32(float(-r)) for r in rho], np.float64)
    exact = np.exp(-rho.astype(np.float64))
    ulp = np.spacing(exact.astype(np.float32)).astype(np.float64)
    assert (np.abs(got - exact) / ulp).max() <= 1.5
    ref = np.array([libm.expf(float(-r)) for r in rho], np.float64)
    assert (np.abs(got - ref) / ulp).max() <= 2.0
