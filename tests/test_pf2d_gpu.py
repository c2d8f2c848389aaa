"""GPU parity of the legacy bootstrap PF (pf2D's ParticleFilter with its own
my_gmm prior) against the FP64 oracle, teacher-forced frame by frame with the
filter's own Philox draws."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _model(d=10, K=3, seed=5):
    rng = np.random.default_rng(seed)
    lo = np.array([100.0, 100.0] * (d // 2))
    hi = np.array([540.0, 380.0] * (d // 2))
    mean = rng.uniform(lo, hi, (K, d))
    cov = np.zeros((K, d, d))
    for k in range(K):
        A = rng.normal(0, 1, (d, d))
        cov[k] = np.diag(rng.uniform(120.0, 180.0, d) ** 2) + 400.0 * (A @ A.T) / d
    w = rng.dirichlet(np.ones(K) * 2)
    return mean, cov, w


def _frames(pf, om, olib, zs, first_frame=0):
    torch = pf.torch
    for t, z in enumerate(zs):
        f = first_frame + t
        s0 = pf.read()
        x0, w0 = s0["x"].cpu().numpy(), s0["w"].cpu().numpy()
        pf.update(z, frame=f)
        g = {k: (v.cpu().numpy() if hasattr(v, "cpu") else v) for k, v in pf.read().items()}
        eps, u = (a.cpu().numpy() for a in pf.draws(f))
        U = int(olib.draw_block(pf.seed, pf.track_id, f, 0xFFFFFFFF, 0x100)[0])
        x, wts, wout, anc, reinit = om.update(x0, w0, np.asarray(z, np.float64).ravel(), U, u, eps)
        assert g["reinit"] == reinit
        # the GMM prior uses single-precision expf on both sides (different libraries): 1e-6 relative
        np.testing.assert_allclose(g["w"], wts, rtol=2e-6, atol=0)
        if reinit:
            assert (g["anc"] == -1).all()
            np.testing.assert_array_equal(g["x"], x)
        else:
            # ancestors: bit-exact against the oracle's resampler on the GPU's own weights
            anc_gpu_w, fb = olib.resample(g["w"], pf.N, U)
            assert not fb
            np.testing.assert_array_equal(g["anc"], anc_gpu_w)
            assert (g["anc"] == anc).mean() > 0.99
            xp = x0[g["anc"]].copy()
            xp[:, :8] += 5.0 * eps
            np.testing.assert_array_equal(g["x"], xp)
        est = pf.getEstimator().cpu().numpy()
        np.testing.assert_allclose(est, (g["w"][:, None] * g["x"]).sum(0), rtol=1e-12, atol=1e-9)
        torch.cuda.synchronize()


def test_pf2d_init_and_frames(cuda, olib):
    from mkfbodytracker_pdaf_gb300.filters import LegacyParticleFilter
    mean, cov, w = _model()
    N = 1000
    for side in (0, 1):
        pf = LegacyParticleFilter(N, mean, cov, w, side=side, seed=11, track_id=side)
        om = olib.Pf2d(mean, cov, w, side=side)
        _, u0 = (a.cpu().numpy() for a in pf.draws(0xFFFFFFFF))
        x_init, w_init = om.init(u0)
        s = pf.read()
        np.testing.assert_array_equal(s["x"].cpu().numpy(), x_init)
        np.testing.assert_array_equal(s["w"].cpu().numpy(), w_init)
        rng = np.random.default_rng(side)
        head, hand = np.array([320.0, 110.0]), np.array([250.0, 300.0])
        zs = []
        for t in range(8):
            head = head + rng.normal(0, 3, 2)
            hand = hand + rng.normal(0, 6, 2)
            zs.append(np.stack([head, hand]))
        _frames(pf, om, olib, zs)


def test_pf2d_reinitialises_when_all_weights_vanish(cuda, olib):
    from mkfbodytracker_pdaf_gb300.filters import LegacyParticleFilter
    mean, cov, w = _model(seed=9)
    N = 512
    pf = LegacyParticleFilter(N, mean, cov, w, seed=4, track_id=7)
    om = olib.Pf2d(mean, cov, w)
    far = np.array([[-1.0e4, -1.0e4], [-1.0e4, -1.0e4]])
    near = np.array([[320.0, 120.0], [260.0, 300.0]])
    _frames(pf, om, olib, [near, far, near, near], first_frame=3)
