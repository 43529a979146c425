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


def run_pair(res, q, steps, K, tau=0.6):
    import boltzmannfluids_gb300 as bf
    from boltzmannfluids_gb300.adjoint import AdjointChannel, channel_setup
    from oracle.oracle import AdjointOracle
    s, u_in, tgt = channel_setup(res, box=min(64, res[0] // 2, res[1] // 2))
    vs = bf.VelocitySet.D2Q9 if q == 9 else bf.VelocitySet.D3Q19
    g = AdjointChannel(res, tau, vs, steps, K)
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


def test_adjoint_d3q19_matches_fp64_reverse_mode():
    (J, gs, gu), (Jr, gsr, gur), _ = run_pair((16, 12, 6), 19, 200, 30)
    assert abs(J - Jr) <= 1e-5 * abs(Jr)
    assert rel(gs, gsr) <= 1e-4, rel(gs, gsr)
    assert rel(gu, gur) <= 1e-4, rel(gu, gur)


def test_checkpoint_interval_does_not_change_gradients():
    import boltzmannfluids_gb300 as bf
    from boltzmannfluids_gb300.adjoint import AdjointChannel, channel_setup
    res = (48, 24, 1)
    s, u_in, tgt = channel_setup(res, box=16)
    out = []
    for K in (100, 13, 500):
        g = AdjointChannel(res, 0.6, bf.VelocitySet.D2Q9, 500, K)
        g.set_parameters(s, u_in)
        g.set_target(tgt)
        J = g.forward()
        out.append((J,) + g.backward())
    for J, gs, gu in out[1:]:
        assert J == out[0][0]
        assert np.array_equal(gs, out[0][1]) and np.array_equal(gu, out[0][2])


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
