"""The standalone C++ harness (PFTracker's frame loop over the C ABI) gives the
same per-frame arm estimates as the Python drop-in path making the same calls,
skips no-face frames, and its batched decode / get3Dpose / point record match
the FP64 oracle on its own estimates."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def test_harness_matches_python_path(cuda, olib, tmp_path):
    from mkfbodytracker_pdaf_gb300 import build, cvyaml, harness_io, synth
    from mkfbodytracker_pdaf_gb300.filters import PoseTracker, RaoBlackwellisedPF
    torch = cuda
    build.build_harness()
    z = np.load(os.path.join(HERE, "golden", "ref_models.npz"))
    paths = []
    for a in range(2):
        p = str(tmp_path / ("arm%d.yml" % a))
        cvyaml.save_arm_model(p, z["arm%d_means" % a], z["arm%d_covs" % a], z["arm%d_weights" % a],
                              z["arm%d_pca_proj" % a], z["arm%d_pca_mean" % a], z["arm%d_gamma_own_file" % a]
                              if a == 0 else z["arm1_gamma"])
        paths.append(p)
    arms = cvyaml.load_reference_models(paths[0], paths[1])
    T, N, seed = 40, 500, 9
    _, _, rois, cands = synth.make_reference_scene(arms, T=T, no_face_every=9)
    fpath, opath = str(tmp_path / "frames.bin"), str(tmp_path / "out.bin")
    harness_io.write_frames(fpath, list(range(T)), rois, cands)
    line = json.loads(harness_io.run_track(paths[0], paths[1], fpath, opath, particles=N, seed=seed))
    out = harness_io.read_output(opath)
    assert line["frames"] == T and line["valid_frames"] == sum(r is not None for r in rois)
    assert line["status"] == [0, 0]

    pfs = []
    for a in range(2):
        arm = arms[a]
        pf = RaoBlackwellisedPF(12, 6, 15, N, seed=seed, track_id=a)
        for k in range(15):
            pf.loadGaussian(k, arm["means"][k], arm["covs"][k * 12:(k + 1) * 12], arm["pca_proj"], arm["pca_mean"],
                            arm["weights"][k], arm["gamma"][k])
        pf.set_hand_decode(arm["pca_proj"][:, 0:2].T.copy(), arm["pca_mean"][0:2].copy())
        pf.resetTracker()
        pfs.append(pf)
    trk = PoseTracker(pfs[0], pfs[1])
    for t in range(T):
        c = torch.from_numpy(np.ascontiguousarray(cands[t], np.float64)).cuda() if len(cands[t]) else None
        e = trk.step(t, rois[t], c)
        assert (e is not None) == bool(out["valid"][t])
        if e is None:
            continue
        for a in range(2):
            np.testing.assert_array_equal(out["est"][t, a], e[a].cpu().numpy())
    for t in np.nonzero(out["valid"])[0]:
        for a in range(2):
            eo = olib.pose_decode(arms[a]["pca_proj"], arms[a]["pca_mean"], out["est"][t, a])
            np.testing.assert_allclose(out["e"][t, a], eo, rtol=1e-12, atol=1e-9)
            np.testing.assert_allclose(out["pos3d"][t, a], olib.pose3d(eo), rtol=1e-9, atol=1e-9)
        np.testing.assert_allclose(out["points"][t], olib.pose2d_record(out["e"][t, 0], out["e"][t, 1]),
                                   rtol=1e-12, atol=1e-9)
    # the tracker follows the hands it was shown
    ok = out["valid"] == 1
    hands = np.stack([np.stack([c[0], c[1]]) for c in cands])[ok]
    err = np.abs(out["points"][ok][:, 0:2] - hands).mean()
    assert err < 60.0, err


def test_harness_image_path_matches_python(cuda, olib, tmp_path):
    """Likelihood-image frames (the reference node's own input): the harness and
    the Python PoseTracker.step_image give the same estimates bit for bit, and
    no-face frames restart the proposals in both."""
    from mkfbodytracker_pdaf_gb300 import build, cvyaml, harness_io, synth
    from mkfbodytracker_pdaf_gb300.filters import PoseTracker, RaoBlackwellisedPF
    torch = cuda
    build.build_harness()
    z = np.load(os.path.join(HERE, "golden", "ref_models.npz"))
    paths = []
    for a in range(2):
        p = str(tmp_path / ("arm%d.yml" % a))
        cvyaml.save_arm_model(p, z["arm%d_means" % a], z["arm%d_covs" % a], z["arm%d_weights" % a],
                              z["arm%d_pca_proj" % a], z["arm%d_pca_mean" % a],
                              z["arm0_gamma_own_file"] if a == 0 else z["arm1_gamma"])
        paths.append(p)
    arms = cvyaml.load_reference_models(paths[0], paths[1])
    T, N, seed = 12, 200, 5
    _, e, rois, _ = synth.make_reference_scene(arms, T=T, no_face_every=5)
    rng = np.random.default_rng(9)
    yy, xx = np.mgrid[0:480, 0:640]
    images = []
    for t in range(T):
        img = rng.uniform(0, 30, (480, 640))
        for a in range(2):
            img += 255.0 * np.exp(-0.5 * ((xx - e[a, t, 0]) ** 2 + (yy - e[a, t, 1]) ** 2) / 10.0 ** 2)
        images.append(np.clip(img, 0, 255).astype(np.uint8))
    fpath, opath = str(tmp_path / "frames2.bin"), str(tmp_path / "out2.bin")
    harness_io.write_frames(fpath, list(range(T)), rois, [None] * T, images=images)
    line = json.loads(harness_io.run_track(paths[0], paths[1], fpath, opath, particles=N, seed=seed))
    assert line["input"] == "likelihood images" and line["status"] == [0, 0]
    out = harness_io.read_output(opath)
    pfs = []
    for a in range(2):
        arm = arms[a]
        pf = RaoBlackwellisedPF(12, 6, 15, N, seed=seed, track_id=a)
        for k in range(15):
            pf.loadGaussian(k, arm["means"][k], arm["covs"][k * 12:(k + 1) * 12], arm["pca_proj"], arm["pca_mean"],
                            arm["weights"][k], arm["gamma"][k])
        pf.set_hand_decode(arm["pca_proj"][:, 0:2].T.copy(), arm["pca_mean"][0:2].copy())
        pf.resetTracker()
        pfs.append(pf)
    trk = PoseTracker(pfs[0], pfs[1])
    for t in range(T):
        est = trk.step_image(t, rois[t], torch.from_numpy(images[t]).cuda())
        assert (est is not None) == bool(out["valid"][t])
        if est is not None:
            for a in range(2):
                np.testing.assert_array_equal(out["est"][t, a], est[a].cpu().numpy())
