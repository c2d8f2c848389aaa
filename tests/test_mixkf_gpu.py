"""GPU mixture-KF log-likelihood and hand-written adjoint (sqrt(T)
checkpointing) against the FP64 CPU forward/adjoint and FP64 central finite
differences."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(olib, n_tracks=6, T=40, K=6, seed=5):
    from mkfbodytracker_pdaf_gb300 import mixkf, synth
    b = synth.make_mix_batch(seed, n_tracks, T, K=K, d=12)
    tt = b.theta_true()
    om = olib.MixModel(tt["mu"], tt["a"], tt["Lq"], tt["sigma"], tt["pi"], tt["S0"])
    th = om.theta()
    g = mixkf.MixtureKF(b, tt["pi"], tt["S0"])
    return b, om, th, g


def test_forward_matches_oracle(cuda, olib):
    b, om, th, g = _setup(olib)
    g.set_theta(th)
    tot = g.forward().item()
    ll = g.ll.cpu().numpy()
    L, ll_ref = olib.mix_batch(om, b)
    np.testing.assert_allclose(ll, ll_ref, rtol=1e-4)
    assert abs(tot - L) <= 1e-4 * abs(L)
    assert g.status() == 0


def test_gradient_matches_fp64_adjoint_and_fd(cuda, olib):
    b, om, th, g = _setup(olib, n_tracks=4, T=37)        # T not a multiple of the checkpoint stride
    g.set_theta(th)
    g.forward()
    grad = g.backward().cpu().numpy()
    L, _, gref = olib.mix_batch(om, b, grad=True)
    rng = np.random.default_rng(3)
    rel = []
    for _ in range(16):
        v = rng.standard_normal(th.size)
        v /= np.linalg.norm(v)
        rel.append(abs(v @ grad - v @ gref) / max(abs(v @ gref), 1e-6))
    assert max(rel) < 1e-3, max(rel)          # random projections: ill-conditioned where v.grad ~ 0
    # normwise: the whole FP32 gradient against the FP64 adjoint
    nw = np.linalg.norm(grad - gref) / np.linalg.norm(gref)
    print("d12 K6 normwise rel err vs FP64 adjoint: %.3g" % nw)
    assert nw < 5e-5, nw
    # per-block agreement with FP64 central differences (relative step 1e-6)
    K, d = 6, 12
    blocks = {"mu": slice(0, K * d), "a": slice(K * d, 2 * K * d), "Lq": slice(2 * K * d, th.size - 1),
              "sigma": slice(th.size - 1, th.size)}
    for name, sl in blocks.items():
        v = np.zeros(th.size)
        v[sl] = rng.standard_normal(v[sl].size)
        v /= np.linalg.norm(v)
        h = 1e-6 * max(1.0, np.abs(th).max())
        Lp, _ = olib.mix_batch(om.with_theta(th + h * v), b)
        Lm, _ = olib.mix_batch(om.with_theta(th - h * v), b)
        fd = (Lp - Lm) / (2 * h)
        assert abs(v @ gref - fd) <= 1e-6 * max(1.0, abs(fd)), (name, v @ gref, fd)
        print("d12 K6 block %s: rel err vs FD %.3g" % (name, abs(v @ grad - fd) / max(1.0, abs(fd))))
        assert abs(v @ grad - fd) <= 1e-4 * max(1.0, abs(fd)), (name, v @ grad, fd)


def test_three_ctas_per_sm_instantiation_matches_oracle(cuda, olib):
    """More tracks than two CTAs per SM hold: the create call picks the
    80-register instantiation of both kernels (three CTAs per SM) that the
    1024-track workload runs.  Forward and gradient against the FP64 CPU."""
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    b, om, th, g = _setup(olib, n_tracks=2 * sms + 16, T=12, K=15, seed=9)
    g.set_theta(th)
    g.forward()
    ll = g.ll.cpu().numpy()
    grad = g.backward().cpu().numpy()
    L, ll_ref, gref = olib.mix_batch(om, b, grad=True)
    np.testing.assert_allclose(ll, ll_ref, rtol=1e-4)
    nw = np.linalg.norm(grad - gref) / np.linalg.norm(gref)
    print("d12 K15 %d tracks normwise rel err vs FP64 adjoint: %.3g" % (b.n_tracks, nw))
    assert nw < 5e-5, nw
    assert g.status() == 0


def test_gradient_deterministic(cuda, olib):
    b, om, th, g = _setup(olib, n_tracks=5, T=20)
    g.set_theta(th)
    g.forward()
    g1 = g.backward().cpu().numpy().copy()
    g.forward()
    g2 = g.backward().cpu().numpy()
    np.testing.assert_array_equal(g1, g2)


def test_checkpoint_stride_does_not_change_the_gradient(cuda, olib):
    b, om, th, g = _setup(olib, n_tracks=5, T=29)
    g.set_theta(th)
    ref = None
    for C in (0, 1, 3, 29):
        g.set_checkpoint_stride(C)
        if C:
            assert g.checkpoint_stride == C
        L = g.forward().item()
        grad = g.backward().cpu().numpy().copy()
        if ref is None:
            ref = (L, grad)
            continue
        assert L == ref[0]                                  # the forward does not depend on C
        np.testing.assert_allclose(grad, ref[1], rtol=1e-5, atol=1e-6 * np.abs(ref[1]).max())
    # the backward needs the checkpoints of a forward at the current stride
    g.set_checkpoint_stride(4)
    from mkfbodytracker_pdaf_gb300._native import MkfError
    with pytest.raises(MkfError):
        g.backward()


def test_fit_resumes_from_a_saved_state(cuda, olib, tmp_path):
    """Four Adam steps in one go equal two steps, a save/load of the fitting
    state, and two more steps (the kernels are deterministic)."""
    from mkfbodytracker_pdaf_gb300 import mixkf
    b, om, th, g = _setup(olib, n_tracks=4, T=16)
    th0 = th * 1.01
    full, _ = g.fit_adam(th0, 4, lr=1e-2)
    full = full.cpu().numpy()
    g.fit_adam(th0, 2, lr=1e-2)
    p = str(tmp_path / "fit.bin")
    mixkf.save_fit_state(p, g.fit_state)
    st = mixkf.load_fit_state(p)
    assert st.step == 2 and st.theta.size == th.size
    resumed, _ = g.fit_adam(None, 2, lr=1e-2, resume=st)
    np.testing.assert_array_equal(resumed.cpu().numpy(), full)


def _setup_body8(olib, n_tracks=3, T=40, seed=9):
    """The motion-model-fitting shape: K=32 components over d=24 (8 joints x 3D,
    head and both hands measured), lambda=5."""
    from mkfbodytracker_pdaf_gb300 import mixkf, synth
    b = synth.make_mix_batch(seed, n_tracks, T, K=32, d=24, lam=5.0, pd=0.9, layout="body8")
    tt = b.theta_true()
    om = olib.MixModel(tt["mu"], tt["a"], tt["Lq"], tt["sigma"], tt["pi"], tt["S0"], J=b.J)
    th = om.theta()
    g = mixkf.MixtureKF(b, tt["pi"], tt["S0"])
    return b, om, th, g


def test_body8_k32_forward_and_gradient_match_fp64(cuda, olib):
    """d=24, K=32, J=3: per-track logL against the FP64 forward, the gradient
    against the FP64 adjoint along random directions, and per parameter block
    against FP64 central differences (relative step 1e-6)."""
    b, om, th, g = _setup_body8(olib)
    g.set_theta(th)
    g.forward()
    ll = g.ll.cpu().numpy()
    grad = g.backward().cpu().numpy()
    L, ll_ref, gref = olib.mix_batch(om, b, grad=True)
    np.testing.assert_allclose(ll, ll_ref, rtol=1e-5)
    assert g.status() == 0
    rng = np.random.default_rng(11)
    rel = []
    for _ in range(16):
        v = rng.standard_normal(th.size)
        v /= np.linalg.norm(v)
        rel.append(abs(v @ grad - v @ gref) / max(abs(v @ gref), 1e-6))
    print("body8 K32 max rel err vs FP64 adjoint: %.3g" % max(rel))
    assert max(rel) < 1e-3, max(rel)
    nw = np.linalg.norm(grad - gref) / np.linalg.norm(gref)
    print("body8 K32 normwise rel err vs FP64 adjoint: %.3g" % nw)
    assert nw < 5e-5, nw
    K, d = 32, 24
    blocks = {"mu": slice(0, K * d), "a": slice(K * d, 2 * K * d), "Lq": slice(2 * K * d, th.size - 1),
              "sigma": slice(th.size - 1, th.size)}
    for name, sl in blocks.items():
        v = np.zeros(th.size)
        v[sl] = rng.standard_normal(v[sl].size)
        v /= np.linalg.norm(v)
        h = 1e-6 * max(1.0, np.abs(th).max())
        Lp, _ = olib.mix_batch(om.with_theta(th + h * v), b)
        Lm, _ = olib.mix_batch(om.with_theta(th - h * v), b)
        fd = (Lp - Lm) / (2 * h)
        assert abs(v @ gref - fd) <= 1e-6 * max(1.0, abs(fd)), (name, v @ gref, fd)
        print("body8 K32 block %s: rel err vs FD %.3g" % (name, abs(v @ grad - fd) / max(1.0, abs(fd))))
        assert abs(v @ grad - fd) <= 1e-4 * max(1.0, abs(fd)), (name, v @ grad, fd)


def test_fit_recovers_the_model_when_the_likelihood_is_exact(cuda, olib):
    """One component, no clutter, detection probability 0.999: the filter's
    likelihood is the model's own (up to the EKF linearisation), so fitting by
    the device adjoint from the config-4-style start (means + N(0, 0.3),
    covariances x 1.5) must recover the parameters to their statistical
    precision, and the fitted logL must exceed the generating parameters' by
    about half the parameter count (the maximum-likelihood excess), not more."""
    from mkfbodytracker_pdaf_gb300 import mixkf, synth
    b = synth.fit_batch_exact(n_tracks=64, T=150)
    tt = b.theta_true()
    K, d = 1, 12
    th_true = mixkf.theta_from(tt["mu"], tt["a"], tt["Lq"], tt["sigma"])
    rng = np.random.default_rng(4)
    th0 = mixkf.theta_from(tt["mu"] + rng.normal(0, 0.3, tt["mu"].shape), tt["a"], tt["Lq"] * np.sqrt(1.5),
                           tt["sigma"] * np.sqrt(1.5))
    g = mixkf.MixtureKF(b, tt["pi"], tt["S0"])
    g.set_theta(th_true)
    L_true = g.forward().item()
    th, _ = g.fit_adam(th0, 200, lr=0.02)
    thf = th.cpu().numpy()
    g.set_theta(thf)
    L_fit = g.forward().item()
    mu0 = mixkf.theta_split(th0, K, d)[0]
    mu_f, a_f, _, s_f = mixkf.theta_split(thf, K, d)
    mae0, mae = np.abs(mu0 - tt["mu"]).mean(), np.abs(mu_f - tt["mu"]).mean()
    print("exact-case fit: mu MAE %.4f -> %.4f, sigma %.3f, a MAE %.4f, logL fit - true %.1f (half the parameters %.1f)"
          % (mae0, mae, s_f, np.abs(a_f - tt["a"]).mean(), L_fit - L_true, 0.5 * th_true.size))
    assert mae < 0.4 * mae0
    assert abs(s_f - tt["sigma"]) < 0.2
    assert 0.0 < L_fit - L_true < th_true.size
