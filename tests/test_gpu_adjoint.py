"""GPU discrete adjoint (bf_adjoint_*) against the FP64 reverse-mode
reference (oracle/adjoint_oracle.c) and against central finite differences
of the GPU forward solve.  Bar: gradients within 1e-4 relative (L2) of the
FP64 reference."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _lib(product_lib, oracle_mod):
    yield


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def run_pair(res, q, steps, K, tau=0.6, resident=0):
    import boltzmannfluids_gb300 as bf
    from boltzmannfluids_gb300.adjoint import AdjointChannel, channel_setup
    from oracle.oracle import AdjointOracle
    s, u_in, tgt = channel_setup(res, box=min(64, res[0] // 2, res[1] // 2))
    vs = bf.VelocitySet.D2Q9 if q == 9 else bf.VelocitySet.D3Q19
    g = AdjointChannel(res, tau, vs, steps, K, resident_states=resident)
    g.set_parameters(s, u_in)
    g.set_target(tgt)
    J = g.forward()
    gs, gu = g.backward()
    o = AdjointOracle(res, tau, steps, q, s.astype(np.float64), u_in.astype(np.float64), tgt.astype(np.float64))
    Jr = o.forward()
    gsr, gur = o.backward()
    return (J, gs, gu), (Jr, gsr, gur), g


def test_adjoint_d2q9_matches_fp64_reverse_mode():
    (J, gs, gu), (Jr, gsr, gur), _ = run_pair((64, 32, 1), 9, 2000, 100)
    assert abs(J - Jr) <= 1e-5 * abs(Jr)
    assert rel(gs, gsr) <= 1e-4, rel(gs, gsr)
    assert rel(gu, gur) <= 1e-4, rel(gu, gur)


@pytest.mark.parametrize("res,steps,K,resident", [
    ((16, 12, 6), 200, 30, 0),
    # 32^3 over 500 steps, the pool schedule recomputing in chunks (R = 120, K = 50)
    ((32, 32, 32), 500, 50, 120),
])
def test_adjoint_d3q19_matches_fp64_reverse_mode(res, steps, K, resident):
    (J, gs, gu), (Jr, gsr, gur), g = run_pair(res, 19, steps, K, resident=resident)
    assert g.resident_states == resident
    assert abs(J - Jr) <= 1e-5 * abs(Jr)
    assert rel(gs, gsr) <= 1e-4, rel(gs, gsr)
    assert rel(gu, gur) <= 1e-4, rel(gu, gur)


def gradients(res, vs, steps, K, resident=0):
    from boltzmannfluids_gb300.adjoint import AdjointChannel, channel_setup
    s, u_in, tgt = channel_setup(res, box=16)
    g = AdjointChannel(res, 0.6, vs, steps, K, resident_states=resident)
    g.set_parameters(s, u_in)
    g.set_target(tgt)
    J = g.forward()
    return (J,) + g.backward(), g.resident_states


def test_checkpoint_interval_does_not_change_gradients():
    import boltzmannfluids_gb300 as bf
    out = [gradients((48, 24, 1), bf.VelocitySet.D2Q9, 500, K)[0] for K in (100, 13, 500)]
    for J, gs, gu in out[1:]:
        assert J == out[0][0]
        assert np.array_equal(gs, out[0][1]) and np.array_equal(gu, out[0][2])


@pytest.mark.parametrize("vs,res,steps,cases", [
    # (K, R): the smallest pool, chunks that do not divide the prefix, every
    # state resident, more slots than states, and the automatic size
    (9, (48, 24, 1), 500, [(13, 12), (13, 50), (13, 499), (100, 1000), (100, -1), (7, 480)]),
    (19, (16, 12, 6), 120, [(10, 9), (10, 25), (10, 119), (1, 3), (10, -1)]),
])
def test_resident_pool_gives_identical_gradients(vs, res, steps, cases):
    """The pool schedule (forward states kept in device memory, the rest
    recomputed from checkpoints in chunks) gives the segment-buffer
    schedule's objective and gradients bit for bit."""
    import boltzmannfluids_gb300 as bf
    v = bf.VelocitySet.D2Q9 if vs == 9 else bf.VelocitySet.D3Q19
    ref, r0 = gradients(res, v, steps, 10)
    assert r0 == 0
    for K, R in cases:
        got, r = gradients(res, v, steps, K, R)
        assert r == (steps - 1 if R < 0 else min(R, steps - 1)), (K, R, r)
        assert got[0] == ref[0], (K, R)
        assert np.array_equal(got[1], ref[1]) and np.array_equal(got[2], ref[2]), (K, R)


def test_resident_pool_rejects_too_few_slots():
    import boltzmannfluids_gb300 as bf
    from boltzmannfluids_gb300.adjoint import AdjointChannel
    with pytest.raises(bf.LBMError):
        AdjointChannel((48, 24, 1), 0.6, bf.VelocitySet.D2Q9, 500, 13, resident_states=11)
    with pytest.raises(bf.LBMError):
        AdjointChannel((48, 24, 1), 0.6, bf.VelocitySet.D2Q9, 500, 13, resident_states=-2)
    # fewer steps than the interval: every state fits
    assert AdjointChannel((48, 24, 1), 0.6, bf.VelocitySet.D2Q9, 5, 13, resident_states=4).resident_states == 4


def test_adjoint_full_size_against_central_differences():
    """512x256 D2Q9, T = 2000, K = 100: 16 random directions in (s, u_in),
    central differences of the FP32 GPU forward with eps = 1e-3."""
    import boltzmannfluids_gb300 as bf
    from boltzmannfluids_gb300.adjoint import AdjointChannel, channel_setup
    res = (512, 256, 1)
    s, u_in, tgt = channel_setup(res)
    g = AdjointChannel(res, 0.6, bf.VelocitySet.D2Q9, 2000, 100)
    g.set_parameters(s, u_in)
    g.set_target(tgt)
    g.forward()
    gs, gu = g.backward()
    rng = np.random.default_rng(7)
    # perturb s only where s +- eps*ds stays inside [0, 1] (|ds| <= 10): a
    # solid fraction above 1 amplifies populations and the flow diverges
    inner = (s > 0.02) & (s < 0.98)
    eps = 1e-3
    worst = 0.0
    for k in range(16):
        ds = (np.clip(rng.standard_normal(s.size), -10, 10) * inner).astype(np.float32)
        du = (0.01 * rng.standard_normal(u_in.size)).astype(np.float32)
        g.set_parameters(s + eps * ds, u_in + eps * du)
        jp = g.forward()
        g.set_parameters(s - eps * ds, u_in - eps * du)
        jm = g.forward()
        fd = (jp - jm) / (2 * eps)
        ad_s, ad_u = float(gs @ ds), float(gu @ du)
        ad = ad_s + ad_u
        # the FP32 forward leaves ~5e-3 absolute noise in these differences,
        # so the error is measured against the size of the two contributions
        # (their sum can cancel)
        err = abs(fd - ad) / (abs(ad_s) + abs(ad_u))
        worst = max(worst, err)
        assert np.isfinite(jp) and np.isfinite(jm)
        assert err <= 2e-2, (k, fd, ad, ad_s, ad_u)
