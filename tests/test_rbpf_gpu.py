"""GPU parity of the Rao-Blackwellised PF (pf2DRao) and the PDAF association
against the FP64 oracle: shipped yml models (LINEAR, m = 6) and the two-arm
synthetic scene (PINHOLE, m = 4)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def _ref_arm(olib, z, a):
    K, d = 15, 12
    comps = [olib.load_gaussian_ref(z["arm%d_means" % a][k], z["arm%d_covs" % a][k * d:(k + 1) * d],
                                    z["arm%d_pca_proj" % a], z["arm%d_pca_mean" % a], z["arm%d_gamma" % a][k])
             for k in range(K)]
    return {key: np.stack([c[key] for c in comps]) for key in ("F", "B", "Q", "H", "BH", "R")}


def _compare_frames(torch, olib, pf, om, x, P, T, meas_fn, mask_fn, rng):
    N = pf.N
    for t in range(T):
        z = meas_fn(t)
        mask = mask_fn(t)
        Ui, Ua = int(rng.integers(0, 2 ** 32)), int(rng.integers(0, 2 ** 32))
        pf.update(torch.from_numpy(z).cuda(), mask=mask, U=(Ui, Ua))
        g = {k: v.cpu().numpy() for k, v in pf.read().items()}
        ref = om.update(x, P, z, Ui, Ua, mask=mask)
        np.testing.assert_array_equal(g["ind"], ref["ind"])
        np.testing.assert_allclose(g["logw"], ref["logw"], rtol=1e-9, atol=1e-9)
        anc_from_gpu_w, _ = olib.resample(g["wn"], N, Ua)
        np.testing.assert_array_equal(g["anc"], anc_from_gpu_w)
        np.testing.assert_array_equal(g["anc"], ref["anc"])
        np.testing.assert_allclose(g["x"], ref["x"], rtol=1e-8, atol=1e-8)
        np.testing.assert_allclose(g["P"], ref["P"], rtol=1e-8, atol=1e-8)
        est = pf.getEstimator().cpu().numpy()
        np.testing.assert_allclose(est, ref["x"].mean(0), rtol=1e-10, atol=1e-10)
        x, P = ref["x"], ref["P"]


def test_rbpf_reference_models_parity(cuda, olib):
    from mkfbodytracker_pdaf_gb300.filters import RaoBlackwellisedPF
    torch = cuda
    z = np.load(os.path.join(HERE, "golden", "ref_models.npz"))
    K, d, m, N = 15, 12, 6, 500
    pf = RaoBlackwellisedPF(d, m, K, N, seed=3, track_id=0)
    for k in range(K):
        pf.loadGaussian(k, z["arm0_means"][k], z["arm0_covs"][k * d:(k + 1) * d], z["arm0_pca_proj"],
                        z["arm0_pca_mean"], z["arm0_weights"][k], z["arm0_gamma"][k])
    mdl = _ref_arm(olib, z, 0)
    om = olib.RbpfModel(d, m, K, mdl["F"], mdl["B"], mdl["Q"], mdl["R"], z["arm0_weights"], H=mdl["H"], BH=mdl["BH"])
    bins, _ = olib.resample(z["arm0_weights"], N, 77)
    pf.resetTracker(bins)
    x = z["arm0_means"][bins].copy()
    P = np.stack([z["arm0_covs"][k * d:(k + 1) * d] for k in bins])
    rng = np.random.default_rng(0)
    base = np.array([320., 120., 300., 330., 320., 200.])
    _compare_frames(torch, olib, pf, om, x, P, 6,
                    lambda t: np.tile(base + 3 * t, (N, 1)) + rng.normal(0, 8, (N, m)),
                    lambda t: 0b111111 if t != 3 else 0b110011, rng)
    assert pf.status() == 0


def test_rbpf_reset_from_mixture_weights(cuda, olib):
    from mkfbodytracker_pdaf_gb300 import synth
    from mkfbodytracker_pdaf_gb300.filters import MEAS_PINHOLE, RaoBlackwellisedPF
    torch = cuda
    sc = synth.make_rbpf_scene(T=2)
    arm = sc.arms[0]
    pf = RaoBlackwellisedPF(12, 4, 15, 777, meas_mode=MEAS_PINHOLE, seed=9, track_id=0)
    for k in range(15):
        pf.set_component(k, arm["mu"][k], np.diag(arm["F"][k]), arm["Q"][k], arm["Sigma"][k], arm["R"][k],
                         arm["weight"][k])
    pf.set_pinhole(arm["Bm"], arm["mm"], synth.CAM)
    pf.resetTracker()                       # bins = resample(pi, N) with the library's draw
    g = pf.read()
    U0 = int(olib.draw_block(9, 0, 0xFFFFFFFF, 0xFFFFFFFF, 0x102)[0])
    bins, _ = olib.resample(arm["weight"], 777, U0)
    np.testing.assert_array_equal(g["x"].cpu().numpy(), arm["mu"][bins])
    np.testing.assert_array_equal(g["P"].cpu().numpy(), arm["Sigma"][bins])


def test_rbpf_pinhole_parity(cuda, olib):
    from mkfbodytracker_pdaf_gb300 import synth
    from mkfbodytracker_pdaf_gb300.filters import MEAS_PINHOLE, RaoBlackwellisedPF
    torch = cuda
    sc = synth.make_rbpf_scene(T=8)
    arm = sc.arms[1]
    N = 1000
    pf = RaoBlackwellisedPF(12, 4, 15, N, meas_mode=MEAS_PINHOLE, seed=1, track_id=1)
    for k in range(15):
        pf.set_component(k, arm["mu"][k], np.diag(arm["F"][k]), arm["Q"][k], arm["Sigma"][k], arm["R"][k],
                         arm["weight"][k])
    pf.set_pinhole(arm["Bm"], arm["mm"], synth.CAM)
    om = olib.rbpf_model_from_arm(arm)
    bins, _ = olib.resample(arm["weight"], N, 5)
    pf.resetTracker(bins)
    x, P = arm["mu"][bins].copy(), arm["Sigma"][bins].copy()
    rng = np.random.default_rng(1)
    truth_px = [np.r_[olib.project_joint(arm, sc.truth[1, t], 0), olib.project_joint(arm, sc.truth[1, t], 1)]
                for t in range(8)]
    _compare_frames(torch, olib, pf, om, x, P, 8,
                    lambda t: np.tile(truth_px[t], (N, 1)) + rng.normal(0, 4, (N, 4)),
                    lambda t: 0b1111 if t % 3 else 0b0011, rng)


def test_pdaf_associate_parity(cuda, olib):
    from mkfbodytracker_pdaf_gb300 import synth
    from mkfbodytracker_pdaf_gb300.filters import MEAS_PINHOLE, RaoBlackwellisedPF, pdaf_associate
    torch = cuda
    sc = synth.make_rbpf_scene(T=30)
    N = 640
    arms = []
    for a in range(2):
        arm = sc.arms[a]
        pf = RaoBlackwellisedPF(12, 4, 15, N, meas_mode=MEAS_PINHOLE, seed=11, track_id=a)
        for k in range(15):
            pf.set_component(k, arm["mu"][k], np.diag(arm["F"][k]), arm["Q"][k], arm["Sigma"][k], arm["R"][k],
                             arm["weight"][k])
        pf.set_pinhole(arm["Bm"], arm["mm"], synth.CAM)
        pf.set_hand_decode(joint=1)
        pf.resetTracker()
        arms.append(pf)
    for t in range(30):
        fr = sc.frames[t]
        if any(len(h) == 0 for h in fr["heads"]) or len(fr["hands"]) == 0:
            continue
        roi = np.stack([olib.scene_roi(fr["heads"][a]) for a in range(2)])
        cand = torch.from_numpy(fr["hands"]).cuda()
        m0, m1, b0, b1 = pdaf_associate(arms[0], arms[1], t, roi, cand)
        xs = [a.read()["x"].cpu().numpy() for a in arms]
        hats = [olib.project_joint(sc.arms[a], xs[a].mean(0), 1) for a in range(2)]
        for a, (mg, bg) in enumerate(((m0, b0), (m1, b1))):
            w = olib.pdaf_weights(fr["hands"], hats[a], hats[1 - a], 0.8 * roi[a, 2])
            U = int(olib.draw_block(11, a, t, 0xFFFFFFFF, 0x103)[0])
            bins, _ = olib.resample(w / w.sum(), N, U)
            np.testing.assert_array_equal(bg.cpu().numpy(), bins)
            mg = mg.cpu().numpy()
            np.testing.assert_allclose(mg[:, 2:4], fr["hands"][bins])
            np.testing.assert_allclose(mg[:, 0], roi[a, 0] + roi[a, 2] / 2)
        # advance both filters one frame so the estimates move
        for a in range(2):
            mg = (m0, m1)[a]
            arms[a].update(mg, frame=t)


def test_pose_tracker_two_arm_scene(cuda, olib):
    """Two-arm pose scene (K=15, d=12, N=1000, FP64): the GPU PoseTracker and
    the CPU restatement of the PFTracker loop agree to 1e-4 relative."""
    from mkfbodytracker_pdaf_gb300 import synth
    from mkfbodytracker_pdaf_gb300.filters import MEAS_PINHOLE, PoseTracker, RaoBlackwellisedPF
    torch = cuda
    T, N, seed = 60, 1000, 20140601
    sc = synth.make_rbpf_scene(T=T)
    arms = []
    for a in range(2):
        arm = sc.arms[a]
        pf = RaoBlackwellisedPF(12, 4, 15, N, meas_mode=MEAS_PINHOLE, seed=seed, track_id=a)
        for k in range(15):
            pf.set_component(k, arm["mu"][k], np.diag(arm["F"][k]), arm["Q"][k], arm["Sigma"][k], arm["R"][k],
                             arm["weight"][k])
        pf.set_pinhole(arm["Bm"], arm["mm"], synth.CAM)
        pf.set_hand_decode(joint=1)
        pf.resetTracker()
        arms.append(pf)
    trk = PoseTracker(arms[0], arms[1])
    est_g = np.full((2, T, 12), np.nan)
    for t in range(T):
        fr = sc.frames[t]
        roi = None if any(len(h) == 0 for h in fr["heads"]) else np.stack(
            [olib.scene_roi(fr["heads"][a]) for a in range(2)])
        cand = torch.from_numpy(fr["hands"]).cuda() if len(fr["hands"]) else None
        e = trk.step(t, roi, cand)
        if e is not None:
            for a in range(2):
                est_g[a, t] = e[a].cpu().numpy()
    est_c, skipped = olib.pose_tracker_run(sc, N, seed, T=T)
    ok = ~skipped
    rel = np.abs(est_g[:, ok] - est_c[:, ok]).max() / np.abs(est_c[:, ok]).max()
    assert rel <= 1e-4, rel
