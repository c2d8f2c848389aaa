"""The oracle pinned to the reference's own code.

tests/golden/refpin.npz holds what the reference's KF_model.cpp, my_gmm.cpp and
pf2DRao.cpp computed, compiled unmodified from the reference checkout against
stand-in OpenCV/ROS headers (oracle/refpin, made by
tests/golden/make_refpin_golden.py).  Each test runs the oracle's restatement
on the same inputs and asserts agreement: FP64 values to rounding, indices
exactly.  The stand-in restates the OpenCV calls the reference makes (shallow
Mat headers with in-place expression assignment, LU inverse, Cholesky with
either diagonal convention, injected RNG draws), so what these tests pin is
the oracle's reading of the reference's own sequencing, formulas, quirks and
control flow, executed from the reference's source.
"""
import os

import numpy as np
import pytest

G = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "refpin.npz"))


def test_kf_predict_update_equals_reference_kf_model(olib):
    """KF_model::predict / ::update (KF_model.cpp:11-25) on 20 random systems."""
    for i in range(G["kf_x"].shape[0]):
        x, P = olib.kf_predict(G["kf_F"][i], G["kf_B"][i], G["kf_Q"][i], G["kf_x"][i], G["kf_P"][i])
        np.testing.assert_allclose(x, G["kf_xp"][i], rtol=1e-13, atol=1e-13)
        np.testing.assert_allclose(P, G["kf_Pp"][i], rtol=1e-13, atol=1e-13)
        x, P, ok = olib.kf_update(G["kf_H"][i], G["kf_BH"][i], G["kf_R"][i], G["kf_z"][i], x, P)
        assert ok
        np.testing.assert_allclose(x, G["kf_xu"][i], rtol=1e-11, atol=1e-12)
        np.testing.assert_allclose(P, G["kf_Pu"][i], rtol=1e-11, atol=1e-12)


@pytest.mark.parametrize("arm", [0, 1])
def test_load_gaussian_equals_reference_my_gmm(olib, arm):
    """my_gmm::loadGaussian (my_gmm.cpp:45-75) on both shipped models: F, B, Q,
    the selector-built H and BH, R = 100 I."""
    p = "loadg%d_" % arm
    for k in range(G[p + "mu"].shape[0]):
        out = olib.load_gaussian_ref(G[p + "mu"][k], G[p + "covs"][k], G[p + "Hpca"], G[p + "mpca"], G[p + "g"][k])
        for key in ("F", "B", "Q", "H", "BH", "R"):
            ref = G[p + "out_" + key][k].reshape(out[key].shape)
            np.testing.assert_allclose(out[key], ref, rtol=1e-14, atol=1e-14, err_msg="%s k=%d" % (key, k))


def test_resample_wheel_equals_reference_resample(olib):
    """ParticleFilter::resample (pf2DRao.cpp:175-210): random, sparse, tied,
    unnormalised (the % L wrap) and all-zero weights (its fallback draws)."""
    c = 0
    while "wheel%d_w" % c in G:
        w, u, fb, idx = (G["wheel%d_%s" % (c, k)] for k in ("w", "u", "fb", "idx"))
        got = olib.resample_wheel(w, len(idx), float(u[0]), fallback=fb)
        np.testing.assert_array_equal(got, idx, err_msg="case %d" % c)
        c += 1
    assert c == 10


@pytest.mark.parametrize("conv,mode", [(24, 1), (3, 2)])
def test_mvn_quirk_modes_equal_reference_chol_mvnpdf(olib, conv, mode):
    """ParticleFilter::chol + ::mvnpdf (pf2DRao.cpp:34-67) under each diagonal
    convention of the Cholesky call against the oracle's matching quirk mode;
    the exact mode agrees with the reference wherever the quirk is exact (a
    diagonal covariance under the OpenCV-2.4 convention)."""
    for i in range(G["mvn_x"].shape[0]):
        x, u, S = G["mvn_x"][i], G["mvn_u"][i], G["mvn_S"][i]
        p_ref = G["mvn%d_p" % conv][i]
        lp = olib.mvn_logpdf(x, u, S, mode)
        if p_ref == 0.0:
            assert lp < -700.0, (i, lp)
        else:
            assert abs(lp - np.log(p_ref)) <= 1e-9 * max(1.0, abs(lp)), (i, lp, np.log(p_ref))
        if conv == 24 and np.count_nonzero(S - np.diag(np.diag(S))) == 0:
            assert abs(olib.mvn_logpdf(x, u, S, 0) - np.log(p_ref)) <= 1e-9 * max(1.0, abs(lp))


@pytest.mark.parametrize("conv,mode", [(24, 1), (3, 2)])
def test_rbpf_literal_update_equals_reference_update(olib, conv, mode):
    """resetTracker then four ParticleFilter::update calls (pf2DRao.cpp:125-158)
    on the shipped left-arm model, N=48, with the reference's shallow
    copy-assign resampling (its tracks share buffers from the second update on):
    the oracle's literal update (wheel, quirk Gaussian, linear-domain weights,
    shared-buffer emulation) reproduces every track's state and covariance and
    getEstimator after every update, and takes the all-zero fallback exactly
    where the reference does.  Without the shared-buffer emulation the states
    differ from the second update on, so the emulation is what is pinned."""
    p = "loadg0_"
    K = G[p + "mu"].shape[0]
    comps = [olib.load_gaussian_ref(G[p + "mu"][k], G[p + "covs"][k], G[p + "Hpca"], G[p + "mpca"], G[p + "g"][k])
             for k in range(K)]
    st = lambda key: np.stack([c[key] for c in comps])
    d, m = 12, 6
    model = olib.RbpfModel(d, m, K, st("F"), st("B"), st("Q"), st("R"), G[p + "w"], H=st("H"), BH=st("BH"))
    for alias in (True, False):
        bins = G["rbpf_bins"]
        x = G[p + "mu"][bins].copy()
        P = G[p + "covs"][bins].copy()
        prev = None
        errs = []
        for t in range(G["rbpf_z"].shape[0]):
            out = model.update_literal(x, P, G["rbpf_z"][t].T, G["rbpf_u_ind"][t], G["rbpf_u_anc"][t], mode,
                                       alias_prev_anc=prev if alias else None, fb_anc=G["rbpf_fb"][t])
            x, P = out["x"], out["P"]
            errs.append(np.abs(x - G["rbpf%d_x" % conv][t]).max())
            if alias:
                assert out["fallback"] == bool(G["rbpf%d_fallback" % conv][t]), t
                np.testing.assert_allclose(x, G["rbpf%d_x" % conv][t], rtol=1e-9, atol=1e-9, err_msg="frame %d" % t)
                np.testing.assert_allclose(P, G["rbpf%d_P" % conv][t], rtol=1e-9, atol=1e-9, err_msg="frame %d" % t)
                np.testing.assert_allclose(x.mean(0), G["rbpf%d_est" % conv][t], rtol=1e-9, atol=1e-9)
            prev = out["anc"]
        if not alias:
            assert max(errs[1:]) > 1e-3          # the shared buffers change the result
