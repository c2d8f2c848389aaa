"""CPU tests of the oracle: published known-answer vectors, the reference's
literal wheel on exactly-representable inputs, and independent closed forms."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


# ----------------------------------------------------------------- Philox KATs
# Random123 known-answer vectors for philox4x32_10 (ctr, key) -> out
PHILOX_KAT = [
    ([0, 0, 0, 0], [0, 0], [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
    ([0xffffffff] * 4, [0xffffffff] * 2, [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
    ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0],
     [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]),
]


@pytest.mark.parametrize("ctr,key,out", PHILOX_KAT)
def test_philox_kat(olib, ctr, key, out):
    assert list(olib.philox4x32_10(ctr, key)) == out


def test_box_muller_moments(olib):
    eps = np.array([olib.particle_draws(7, 3, f, i, 12)[0] for f in range(40) for i in range(100)])
    assert abs(eps.mean()) < 0.03
    assert abs(eps.var() - 1.0) < 0.05
    uc = np.array([olib.particle_draws(7, 3, 0, i, 12)[1] for i in range(4000)])
    assert 0.0 <= uc.min() and uc.max() < 1.0 and abs(uc.mean() - 0.5) < 0.02


# ----------------------------------------------------------------- resampler (A6)
def test_resample_hand_kat(olib):
    # weights 1/4, 0, 1/2, 1/4; N = 4; u = 1/2 -> targets 1/8, 3/8, 5/8, 7/8
    w = np.array([0.25, 0.0, 0.5, 0.25])
    assert list(olib.resample_wheel(w, 4, 0.5)) == [0, 2, 2, 3]
    idx, fb = olib.resample(w, 4, 1 << 31)
    assert list(idx) == [0, 2, 2, 3] and not fb
    # ties go to the lower index (strict '>' in the wheel)
    w = np.array([0.5, 0.5])
    assert list(olib.resample_wheel(w, 2, 0.0)) == [0, 0]
    assert list(olib.resample(w, 2, 0)[0]) == [0, 0]


def test_resample_dyadic_matches_literal_wheel(olib):
    """On weights that are multiples of 2^-k summing to 1, N a power of two and
    u = U/2^32, every FP operation of the reference wheel is exact, so the
    exact resampler must reproduce it bit for bit (zeros and ties included)."""
    rng = np.random.default_rng(1)
    for t in range(3000):
        L = int(rng.integers(1, 40))
        k = int(rng.integers(0, 9))
        N = 2 ** int(rng.integers(0, 9))
        units = 2 ** k
        cuts = np.sort(rng.integers(0, units + 1, size=L - 1))
        w = np.diff(np.concatenate([[0], cuts, [units]])).astype(float) / units
        U = 0 if t % 5 == 0 else int(rng.integers(0, 2 ** 32))
        a = olib.resample_wheel(w, N, U / 2 ** 32)
        b, fb = olib.resample(w, N, U)
        assert not fb
        np.testing.assert_array_equal(a, b)


def test_resample_random_mismatch_vs_wheel(olib):
    rng = np.random.default_rng(2)
    mism = total = 0
    for _ in range(100):
        w = rng.random(1000) ** 3
        w /= w.sum()
        U = int(rng.integers(0, 2 ** 32))
        a = olib.resample_wheel(w, 1000, U / 2 ** 32)
        b, _ = olib.resample(w, 1000, U)
        mism += int((a != b).sum())
        total += 1000
    assert mism <= 2, (mism, total)


def test_resample_offspring_property(olib):
    """Systematic resampling: offspring counts are floor or ceil of N q_j / Q."""
    rng = np.random.default_rng(3)
    for dt in (np.float32, np.float64):
        for _ in range(20):
            L, N = int(rng.integers(1, 3000)), int(rng.integers(1, 3000))
            w = (rng.random(L) ** 4).astype(dt)
            w[rng.random(L) < 0.2] = 0
            if w.max() == 0:
                w[0] = 1
            idx, fb = olib.resample(w, N, int(rng.integers(0, 2 ** 32)))
            q, ok = olib.quantize(w)
            assert ok and not fb
            assert np.all(np.diff(idx) >= 0)
            cnt = np.bincount(idx, minlength=L)
            expct = N * q.astype(np.float64) / q.astype(np.float64).sum()
            assert np.all(cnt >= np.floor(expct) - 1e-9) and np.all(cnt <= np.ceil(expct) + 1e-9)


def test_resample_fallback(olib):
    idx, fb = olib.resample(np.zeros(7), 50, 12345)
    assert fb and idx.min() >= 0 and idx.max() < 7
    idx2, fb2 = olib.resample(np.full(7, np.nan), 50, 12345)
    assert fb2 and np.array_equal(idx, idx2)
    idx3, fb3 = olib.resample(np.array([0.0, np.inf, 1.0]), 5, 1)
    assert fb3


# ----------------------------------------------------------------- KF_model (A4/A5)
def test_kf_predict_update_closed_form(olib):
    rng = np.random.default_rng(4)
    d, m = 12, 6
    F = np.diag(rng.uniform(0.8, 1.0, d))
    B = rng.standard_normal(d)
    A = rng.standard_normal((d, d))
    Q = A @ A.T / d + 0.1 * np.eye(d)
    x = rng.standard_normal(d)
    P = Q.copy()
    x1, P1 = olib.kf_predict(F, B, Q, x, P)
    np.testing.assert_allclose(x1, F @ x + B, rtol=1e-12)
    np.testing.assert_allclose(P1, F @ P @ F.T + Q, rtol=1e-12)
    H = rng.standard_normal((m, d))
    BH = rng.standard_normal(m)
    R = 100 * np.eye(m)
    z = rng.standard_normal(m)
    x2, P2, ok = olib.kf_update(H, BH, R, z, x1, P1)
    y = z - (H @ x1 + BH)
    S = H @ P1 @ H.T + R
    K = P1 @ H.T @ np.linalg.inv(S)
    assert ok
    np.testing.assert_allclose(x2, x1 + K @ y, rtol=1e-10)
    np.testing.assert_allclose(P2, (np.eye(d) - K @ H) @ P1, rtol=1e-9, atol=1e-12)
    # masked rows: only rows 0,1 used
    x3, P3, _ = olib.kf_update(H, BH, R, z, x1, P1, mask=0b11)
    Hm, Rm = H[:2], R[:2, :2]
    Km = P1 @ Hm.T @ np.linalg.inv(Hm @ P1 @ Hm.T + Rm)
    np.testing.assert_allclose(x3, x1 + Km @ (z[:2] - Hm @ x1 - BH[:2]), rtol=1e-10)


def test_mvn_logpdf_and_chol_quirk(olib):
    from scipy.stats import multivariate_normal
    rng = np.random.default_rng(5)
    m = 6
    A = rng.standard_normal((m, m))
    S = A @ A.T + m * np.eye(m)
    x, u = rng.standard_normal(m), rng.standard_normal(m)
    ref = multivariate_normal(u, S).logpdf(x)
    assert abs(olib.mvn_logpdf(x, u, S, 0) - ref) < 1e-10
    # the chol() quirk (pf2DRao.cpp:34-53) is exact for a diagonal covariance
    # under the OpenCV-2.4 diagonal convention, wrong under the later one
    Sd = np.diag(rng.uniform(1, 30, m))
    ref_d = multivariate_normal(u, Sd).logpdf(x)
    assert abs(olib.mvn_logpdf(x, u, Sd, 1) - ref_d) < 1e-10
    assert abs(olib.mvn_logpdf(x, u, Sd, 2) - ref_d) > 1e-3
    # dense innovation covariance: the quirk is only approximate
    assert np.isfinite(olib.mvn_logpdf(x, u, S, 1))


# ----------------------------------------------------------------- model loading (A1) on the shipped models
def test_load_gaussian_reference_models(olib):
    z = np.load(os.path.join(HERE, "golden", "ref_models.npz"))
    # pfPose.cpp:52-53 reads gamma for both arms from the right-arm file
    np.testing.assert_array_equal(z["arm0_gamma"], z["arm1_gamma"])
    assert not np.array_equal(z["arm0_gamma_own_file"], z["arm1_gamma"]) or True
    for a in range(2):
        means, covs = z["arm%d_means" % a], z["arm%d_covs" % a]
        Hp, mp, g = z["arm%d_pca_proj" % a], z["arm%d_pca_mean" % a], z["arm%d_gamma" % a]
        K, d = means.shape
        assert (K, d) == (15, 12) and covs.shape == (K * d, d) and Hp.shape == (d, 22)
        assert abs(z["arm%d_weights" % a].sum() - 1.0) < 1e-9
        for k in (0, 7, 14):
            s = covs[k * d:(k + 1) * d]
            out = olib.load_gaussian_ref(means[k], s, Hp, mp, g[k])
            np.testing.assert_allclose(out["F"], g[k] * np.eye(d))
            np.testing.assert_allclose(out["Q"], (1 - g[k] ** 2) * s)
            np.testing.assert_allclose(out["B"], (1 - g[k]) * means[k])
            sel = [9, 10, 0, 1, 12, 13]   # H1 of my_gmm.cpp:61-67
            np.testing.assert_allclose(out["H"], Hp[:, sel].T)
            np.testing.assert_allclose(out["BH"], mp[sel])
            np.testing.assert_allclose(out["R"], 100 * np.eye(6))
            # every shipped covariance block is symmetric positive definite
            np.linalg.cholesky(s)


def test_cvyaml_reader_roundtrip(tmp_path):
    from mkfbodytracker_pdaf_gb300 import cvyaml
    txt = ("%YAML:1.0\nM: !!opencv-matrix\n   rows: 2\n   cols: 3\n   dt: d\n"
           "   data: [ 1., 2.5e+00,\n       -3., 4., 5.,\n       6. ]\nn: 640\nname: cam/left\n"
           "K:\n  rows: 1\n  cols: 2\n  data: [7, 8]\n")
    out = cvyaml.parse(txt)
    np.testing.assert_array_equal(out["M"], [[1, 2.5, -3], [4, 5, 6]])
    assert out["n"] == 640 and out["name"] == "cam/left"
    np.testing.assert_array_equal(out["K"], [[7, 8]])


# ----------------------------------------------------------------- PDAF weights (A9)
def test_pdaf_weights_formula(olib):
    rng = np.random.default_rng(6)
    cand = rng.uniform(0, 640, (9, 2))
    own, oth, var, Pa, c = np.array([300., 200.]), np.array([350., 260.]), 0.8 * 40, 0.05, 1e-4

    def g(p, u):
        return np.exp(-0.5 * ((p - u) ** 2).sum(-1) / var) / (2 * np.pi * var)
    Z = Pa * g(cand, own) + Pa * g(cand, oth) + c * (1 - 2 * Pa)
    np.testing.assert_allclose(olib.pdaf_weights(cand, own, oth, var), Pa * g(cand, own) / Z, rtol=1e-12)
    L = rng.random(9)
    np.testing.assert_allclose(olib.pdaf_weights(cand, own, oth, var, Lc=L), L / Z, rtol=1e-12)
    Z1 = Pa * g(cand, own) + c * (1 - Pa)
    np.testing.assert_allclose(olib.pdaf_weights(cand, own, None, var), Pa * g(cand, own) / Z1, rtol=1e-12)


# ----------------------------------------------------------------- bootstrap PF pieces (A13)
def test_bpf_pieces_vs_numpy(olib):
    from mkfbodytracker_pdaf_gb300 import synth
    b = synth.sweep_batch(64, n_frames=3)
    m, t = b.model, b.tracks[0]
    prm, keep = olib.bpf_params(m, 0, t)
    d, K = m["d"], m["K"]
    Lq = synth.unpack_lower(m["Lq"][0].astype(np.float64), d)
    S0 = synth.unpack_lower(m["S0c"][0].astype(np.float64), d)
    rng = np.random.default_rng(7)
    for trial in range(20):
        eps = rng.standard_normal(d)
        uc = np.float32(rng.random())
        k = int(np.argmax(uc < m["cumpi"][0])) if (uc < m["cumpi"][0]).any() else K - 1
        assert olib.lib().mko_pick_component(m["cumpi"][0].ctypes.data, K, float(uc)) == k
        x0 = olib.bpf_prior(prm, eps, uc)
        np.testing.assert_allclose(x0, m["mu"][0, k] + S0[k] @ eps, rtol=1e-6, atol=1e-6)
        x1 = olib.bpf_propagate(prm, x0, eps, uc)
        np.testing.assert_allclose(x1, m["a"][0, k] * x0 + m["mb"][0, k] + Lq[k] @ eps, rtol=1e-6, atol=1e-6)
        off = b.det_off[trial % 3 * 2: trial % 3 * 2 + 3].astype(np.int32)
        ll = olib.bpf_loglik(prm, x1, off, b.det)
        tot = 0.0
        for j in range(m["J"]):
            p = m["Bm"][0, j].astype(np.float64) @ x1 + m["mm"][0, j]
            u = 525 * p[0] / p[2] + 319.5
            v = 525 * p[1] / p[2] + 239.5
            dets = b.det[off[j]:off[j + 1]].astype(np.float64)
            s2 = t["sigma"] ** 2
            acc = np.exp(-0.5 * (((dets - [u, v]) ** 2).sum(-1)) / s2).sum()
            tot += np.log((1 - t["pd"]) * t["kappa"] + t["pd"] * acc / (2 * np.pi * s2))
        assert abs(ll - tot) < 1e-6 * max(1, abs(tot))


def test_bpf_forced_frames_replays_the_frame_loop(olib):
    """The C teacher-forced replay (used for the full-horizon GPU check) equals
    the frame loop of pf2D.cpp:148-210 written out per particle here, when it
    is given that loop's own draws and ancestors; it also reports the weight
    error against given weights, split over two calls (chunked replay)."""
    from mkfbodytracker_pdaf_gb300 import synth
    b = synth.make_bpf_batch(5, [40], [7], [4.0], [0.9])
    m, t = b.model, b.tracks[0]
    prm, keep = olib.bpf_params(m, 0, t)
    d, J, N, T = m["d"], m["J"], 40, 7
    seed, trk = int(t["seed"]), int(t["track_id"])

    def draws(f):
        e, u = zip(*[olib.particle_draws(seed, trk, f, i, d) for i in range(N)])
        return np.asarray(e, np.float32), np.asarray(u, np.float32)

    e0, u0 = draws(0xFFFFFFFF)
    x = np.stack([olib.bpf_prior(prm, e0[i].astype(np.float64), u0[i]) for i in range(N)])
    np.testing.assert_array_equal(olib.bpf_prior_set(prm, e0, u0), x)
    anc = np.arange(N)
    eps_all, uc_all, anc_all, w_all, est_ref, ll_ref = [], [], [], [], [], []
    for f in range(T):
        eps, uc = draws(f)
        xn = np.stack([olib.bpf_propagate(prm, x[anc[i]], eps[i].astype(np.float64), uc[i]) for i in range(N)])
        off = b.det_off[f * J:f * J + J + 1].astype(np.int32)
        ll = np.array([olib.bpf_loglik(prm, xn[i], off, b.det) for i in range(N)])
        w = np.exp(ll - ll.max())
        est_ref.append((w[:, None] * xn).sum(0) / w.sum())
        ll_ref.append(ll.max() + np.log(w.sum()) - np.log(N))
        U = int(olib.draw_block(seed, trk, f, 0xFFFFFFFF, 0x100)[0])
        anc, _ = olib.resample(w, N, U)
        eps_all.append(eps); uc_all.append(uc); anc_all.append(anc); w_all.append(w.astype(np.float32))
        x = xn
    x2 = olib.bpf_prior_set(prm, e0, u0)
    outs = []
    for f0, f1 in ((0, 3), (3, T)):       # two chunks: the state carries over
        prev = np.arange(N, dtype=np.int32) if f0 == 0 else anc_all[f0 - 1]
        outs.append(olib.bpf_forced_frames(prm, x2, prev, np.stack(eps_all[f0:f1]), np.stack(uc_all[f0:f1]),
                                           np.stack(anc_all[f0:f1]), np.stack(w_all[f0:f1]),
                                           b.det_off[f0 * J:f1 * J + 1], b.det))
    est = np.concatenate([o[0] for o in outs])
    ll = np.concatenate([o[1] for o in outs])
    werr = np.concatenate([o[3] for o in outs])
    np.testing.assert_allclose(est, np.stack(est_ref), rtol=0, atol=1e-12)
    np.testing.assert_allclose(ll, ll_ref, rtol=1e-13)
    assert werr.max() <= 2 ** -24 and werr.max() > 0            # float32 rounding of the given weights
    np.testing.assert_allclose(x2, x, rtol=0, atol=1e-12)


# ----------------------------------------------------------------- RBPF update (A8)
def _numpy_rbpf(model, x, P, z, ind, U_anc, olib):
    """Independent numpy restatement of pf2DRao.cpp:125-158 given the indicators."""
    N, d = x.shape
    logw = np.zeros(N)
    xs, Ps = x.copy(), P.copy()
    for j in range(N):
        k = ind[j]
        xs[j] = model["F"][k] @ xs[j] + model["B"][k]
        Ps[j] = model["F"][k] @ Ps[j] @ model["F"][k].T + model["Q"][k]
        H, BH = model["H"][k], model["BH"][k]
        S = H @ Ps[j] @ H.T + model["R"][k]
        r = z[j] - (H @ xs[j] + BH)
        logw[j] = -0.5 * r @ np.linalg.solve(S, r) - 0.5 * np.linalg.slogdet(S)[1] - 0.5 * len(r) * np.log(2 * np.pi)
        K = Ps[j] @ H.T @ np.linalg.inv(S)
        xs[j] = xs[j] + K @ r
        Ps[j] = (np.eye(d) - K @ H) @ Ps[j]
    return xs, Ps, logw


def test_rbpf_update_reference_models(olib):
    """A8 on the shipped yml models (LINEAR measurement H x + BH, m = 6)."""
    z = np.load(os.path.join(HERE, "golden", "ref_models.npz"))
    K, d, m = 15, 12, 6
    comps = [olib.load_gaussian_ref(z["arm0_means"][k], z["arm0_covs"][k * d:(k + 1) * d],
                                    z["arm0_pca_proj"], z["arm0_pca_mean"], z["arm0_gamma"][k])
             for k in range(K)]
    model = {key: np.stack([c[key] for c in comps]) for key in ("F", "B", "Q", "H", "BH", "R")}
    rm = olib.RbpfModel(d, m, K, model["F"], model["B"], model["Q"], model["R"], z["arm0_weights"],
                        H=model["H"], BH=model["BH"])
    N = 200
    bins, _ = olib.resample(z["arm0_weights"], N, 99)
    x = z["arm0_means"][bins].copy()
    P = np.stack([z["arm0_covs"][k * d:(k + 1) * d] for k in bins])
    rng = np.random.default_rng(8)
    zz = np.tile(np.array([320., 120., 300., 330., 320., 200.]), (N, 1)) + rng.normal(0, 5, (N, m))
    out = rm.update(x, P, zz, U_ind=1234567, U_anc=7654321)
    ind_ref, _ = olib.resample(z["arm0_weights"], N, 1234567)
    np.testing.assert_array_equal(out["ind"], ind_ref)
    assert np.all(np.diff(out["ind"]) >= 0)       # systematic indicators are sorted
    xs, Ps, lw = _numpy_rbpf(model, x, P, zz, out["ind"], 7654321, olib)
    np.testing.assert_allclose(out["logw"], lw, rtol=1e-9, atol=1e-9)
    wn = np.exp(lw - lw.max())
    wn /= wn.sum()
    np.testing.assert_allclose(out["wn"], wn, rtol=1e-9)
    anc_ref, _ = olib.resample(out["wn"], N, 7654321)
    np.testing.assert_array_equal(out["anc"], anc_ref)
    np.testing.assert_allclose(out["x"], xs[out["anc"]], rtol=1e-9, atol=1e-9)
    np.testing.assert_allclose(out["P"], Ps[out["anc"]], rtol=1e-9, atol=1e-9)


def test_rbpf_alias_quirk_changes_duplicates_only(olib):
    """--ref-alias emulation (pf2DRao.cpp:153-156): the first member of each
    duplicate run matches the independent-copy filter; later members do not."""
    from mkfbodytracker_pdaf_gb300 import synth
    sc = synth.make_rbpf_scene(T=3)
    arm = sc.arms[0]
    rm = olib.RbpfModel(12, 4, 15, arm["F"], arm["B"], arm["Q"], arm["R"], arm["weight"],
                        Bm=arm["Bm"], mm=arm["mm"])
    N = 64
    bins, _ = olib.resample(arm["weight"], N, 5)
    x = arm["mu"][bins].copy()
    P = arm["Sigma"][bins].copy()
    zz = np.tile(np.array([320., 100., 330., 330.]), (N, 1))
    prev = np.sort(np.random.default_rng(9).integers(0, N, N)).astype(np.int32)
    xg, Pg = x[prev], P[prev]
    a = rm.update(xg, Pg, zz, 11, 12)
    b = rm.update(xg, Pg, zz, 11, 12, alias_prev_anc=prev)
    first = np.r_[True, prev[1:] != prev[:-1]]
    np.testing.assert_allclose(a["logw"][first], b["logw"][first], rtol=1e-12)
    if (~first).any():
        assert not np.allclose(a["logw"][~first], b["logw"][~first])


def test_pf2d_oracle_pieces(olib):
    """Legacy pf2D restatement: constructor ranges, GMM prior density against a
    direct evaluation, re-initialisation when every weight vanishes, and the
    estimator as the weighted particle sum."""
    rng = np.random.default_rng(2)
    d, K, N = 8, 2, 64
    mean = rng.uniform(100, 400, (K, d))
    cov = np.stack([np.diag(rng.uniform(100, 160, d) ** 2) for _ in range(K)])
    w = np.array([0.3, 0.7])
    for side in (0, 1):
        om = olib.Pf2d(mean, cov, w, width=640, height=480, side=side)
        u = rng.uniform(0, 1, (N, d))
        x, wt = om.init(u)
        assert (x[:, 6] >= 320 * side + 1).all() and (x[:, 6] < 320 + 320 * side).all()
        assert (x[:, 1] < 480).all() and (x[:, 0] < 640).all() and (x[:, 0] >= 1).all()
        np.testing.assert_array_equal(wt, np.full(N, 1.0 / N))
    om = olib.Pf2d(mean, cov, w)
    x, wt = om.init(rng.uniform(0, 1, (N, d)))
    z = np.array([300.0, 120.0, 260.0, 300.0])
    eps = rng.normal(0, 1, (N, 8))
    xn, wn, wout, anc, reinit = om.update(x, wt, z, 12345, rng.uniform(0, 1, (N, d)), eps)
    assert not reinit
    prior = np.zeros(N)
    for k in range(K):
        dx = x - mean[k]
        q = np.einsum("ni,ij,nj->n", dx, np.linalg.inv(cov[k]), dx)
        prior += w[k] * np.exp(-0.5 * q) / np.sqrt((2 * np.pi) ** d * np.linalg.det(cov[k]))
    c = 1.0 / (2 * np.pi * 15.0)
    lik = c * np.exp(-0.5 * ((x[:, 6] - z[0]) ** 2 + (x[:, 7] - z[1]) ** 2) / 15.0) * \
        c * np.exp(-0.5 * ((x[:, 0] - z[2]) ** 2 + (x[:, 1] - z[3]) ** 2) / 15.0)
    ref = prior * lik / (prior * lik).sum()
    np.testing.assert_allclose(wout, ref, rtol=1e-5, atol=1e-300)
    np.testing.assert_array_equal(wn, wout)        # weights stay as normalised (not reset after resampling)
    a2, _ = olib.resample(wout, N, 12345)
    np.testing.assert_array_equal(anc, a2)
    np.testing.assert_array_equal(xn[:, :8], x[anc][:, :8] + 5.0 * eps)
    np.testing.assert_array_equal(xn[:, 8:], x[anc][:, 8:])
    np.testing.assert_allclose(om.estimate(xn, wn), (wn[:, None] * xn).sum(0), rtol=1e-13)
    ru = rng.uniform(0, 1, (N, d))
    xr, wr, _, ar, reinit = om.update(x, wt, np.array([-1e4, -1e4, -1e4, -1e4]), 1, ru, eps)
    assert reinit and (ar == -1).all()
    np.testing.assert_array_equal(wr, np.full(N, 1.0 / N))
    x2, _ = om.init(ru)
    x2[:, :8] += 5.0 * eps
    np.testing.assert_array_equal(xr, x2)


def test_pose3d_oracle_against_closed_form(olib):
    """get3Dpose restatement: the back-projected points re-project through
    K [R | t] onto (u, v) with depth scale Z, and R is a rotation."""
    rng = np.random.default_rng(4)
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_models.npz"))
    for a in range(2):
        H, m = z["arm%d_pca_proj" % a], z["arm%d_pca_mean" % a]
        x = z["arm%d_means" % a][rng.integers(0, 15)] + rng.normal(0, 0.5, 12)
        e = olib.pose_decode(H, m, x)
        np.testing.assert_allclose(e, H.T @ x + m, rtol=1e-13, atol=1e-12)
        p = olib.pose3d(e)
        r, pi, y = e[16], e[17], e[15]
        R1 = np.array([[1, 0, 0], [0, np.cos(r), -np.sin(r)], [0, np.sin(r), np.cos(r)]])
        R2 = np.array([[np.cos(pi), 0, np.sin(pi)], [0, 1, 0], [-np.sin(pi), 0, np.cos(pi)]])
        R3 = np.array([[np.cos(y), -np.sin(y), 0], [np.sin(y), np.cos(y), 0], [0, 0, 1]])
        R = R3 @ R2 @ R1
        P = olib.KINECT_K @ np.hstack([R, e[18:21, None]])
        proj = P @ np.vstack([p, np.ones((1, 5))])
        for k in range(5):
            Zk = e[3 * k + 2]
            np.testing.assert_allclose(proj[:, k], [e[3 * k] * Zk, e[3 * k + 1] * Zk, Zk], rtol=1e-9, atol=1e-9)
    e1, e2 = rng.normal(0, 100, 22), rng.normal(0, 100, 22)
    rec = olib.pose2d_record(e1, e2)
    np.testing.assert_array_equal(rec[0], e1[0:2])
    np.testing.assert_array_equal(rec[1], e2[0:2])
    np.testing.assert_array_equal(rec[2], 0.5 * (e1[9:11] + e2[9:11]))
    np.testing.assert_array_equal(rec[3], 0.5 * (e1[12:14] + e2[12:14]))
    np.testing.assert_array_equal(rec[4:], np.stack([e1[3:5], e2[3:5], e1[6:8], e2[6:8]]))


def test_blur_oracle_against_float64_convolution(olib):
    """GaussianBlur restatement (15x15, sigma 3, reflect-101, 8-bit): against a
    float64 separable convolution it differs by at most one grey level, and a
    constant image stays constant."""
    rng = np.random.default_rng(6)
    img = rng.integers(0, 256, (48, 64)).astype(np.uint8)
    out = olib.gaussian_blur_u8(img)
    x = np.arange(15) - 7.0
    g = np.exp(-x * x / 18.0)
    g /= g.sum()
    pad = np.pad(img.astype(np.float64), 7, mode="reflect")          # numpy "reflect" = reflect-101
    hz = sum(g[k] * pad[:, k:k + 64] for k in range(15))
    ref = sum(g[k] * hz[k:k + 48, :] for k in range(15))
    assert np.abs(out.astype(np.int64) - np.rint(ref).astype(np.int64)).max() <= 1
    const = np.full((20, 30), 137, np.uint8)
    np.testing.assert_array_equal(olib.gaussian_blur_u8(const), const)
    cand = np.array([[0.0, 5.0], [10.5, 7.9], [63.99, 47.5], [64.0, 1.0], [3.0, -1.0]])
    L = olib.image_lookup(cand, out)
    np.testing.assert_array_equal(L, [0.0, out[7, 10] / 255.0, out[47, 63] / 255.0, 0.0, 0.0])


# ----------------------------------------------------------------- mixture KF (A11)
def test_mixkf_oracle_adjoint_against_central_differences(olib):
    """The FP64 CPU adjoint of the mixture-KF log-likelihood (the GPU adjoint's
    checker) against FP64 central differences of the FP64 forward, per
    parameter block (mu, a, L_Q, sigma) and along random directions."""
    from mkfbodytracker_pdaf_gb300 import synth
    b = synth.make_mix_batch(9, 3, 14, K=3, d=12)
    tt = b.theta_true()
    om = olib.MixModel(tt["mu"], tt["a"], tt["Lq"], tt["sigma"], tt["pi"], tt["S0"])
    th = om.theta()
    L, ll, g = olib.mix_batch(om, b, grad=True)
    assert np.isfinite(L) and np.all(np.isfinite(g))
    np.testing.assert_allclose(ll.sum(), L, rtol=1e-12)
    K, d = 3, 12
    blocks = [slice(0, K * d), slice(K * d, 2 * K * d), slice(2 * K * d, th.size - 1), slice(th.size - 1, th.size)]
    rng = np.random.default_rng(11)
    dirs = []
    for sl in blocks:
        v = np.zeros(th.size)
        v[sl] = rng.standard_normal(v[sl].size)
        dirs.append(v)
    dirs += [rng.standard_normal(th.size) for _ in range(3)]
    for v in dirs:
        v = v / np.linalg.norm(v)
        h = 1e-6 * max(1.0, np.abs(th).max())
        Lp, _ = olib.mix_batch(om.with_theta(th + h * v), b)
        Lm, _ = olib.mix_batch(om.with_theta(th - h * v), b)
        fd = (Lp - Lm) / (2 * h)
        assert abs(v @ g - fd) <= 1e-6 * max(1.0, abs(fd)), (v @ g, fd)
