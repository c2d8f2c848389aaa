"""The seeded synthetic workloads have the shapes, sizes and value
distributions of the workloads they stand in for (motion model, camera, the
batched uneven-track spread, detections and clutter)."""
import numpy as np

from mkfbodytracker_pdaf_gb300 import synth


def test_motion_model_parameters():
    rng = np.random.default_rng(1)
    g = synth.make_gmm(rng, 12, 15, n=200)
    assert g["mu"].shape == (200, 15, 12) and g["a"].shape == (200, 15, 12)
    assert g["a"].min() >= 0.85 and g["a"].max() <= 0.99
    np.testing.assert_allclose(g["Lq"] @ np.swapaxes(g["Lq"], -1, -2), np.broadcast_to(0.05 * np.eye(12), g["Lq"].shape))
    np.testing.assert_allclose(g["pi"].sum(-1), 1.0, rtol=1e-12)
    # Sigma = Wishart(d + 2, 0.1 I) / (d + 2): mean 0.1 I, symmetric positive definite
    S = g["Sigma"]
    np.testing.assert_allclose(S, np.swapaxes(S, -1, -2))
    assert np.linalg.eigvalsh(S).min() > 0
    np.testing.assert_allclose(S.mean((0, 1)), 0.1 * np.eye(12), atol=0.01)
    assert abs(g["mu"].mean()) < 0.02 and abs(g["mu"].std() - 1.0) < 0.02


def test_body_and_camera():
    rng = np.random.default_rng(2)
    Bs, mbar, measured = synth.make_body(rng, 12, n=500)
    assert measured == (0, 3)                                    # head, hand
    # orthonormal basis scaled to 0.1 m per latent unit
    np.testing.assert_allclose(Bs @ np.swapaxes(Bs, -1, -2), np.broadcast_to(0.01 * np.eye(12), Bs.shape), atol=1e-12)
    z = mbar.reshape(500, 4, 3)[..., 2]
    assert z.min() > 1.5 - 0.2 and z.max() < 3.0 + 0.2         # depth U[1.5, 3] m around the layout
    assert synth.CAM == (525.0, 525.0, 319.5, 239.5) and (synth.IMG_W, synth.IMG_H) == (640, 480)
    px = synth.project(np.array([[0.0, 0.0, 2.0], [1.0, -0.5, 2.0]]))
    np.testing.assert_allclose(px, [[319.5, 239.5], [319.5 + 262.5, 239.5 - 131.25]])


def test_batched_uneven_track_spread():
    N, T, lam, pd = synth.uneven_tracks_spec(n_tracks=8192)
    assert T.min() >= 50 and T.max() <= 2000 and abs(T.mean() - 1025) < 25
    assert N.min() >= 128 and N.max() <= 8192
    # log-uniform in [128, 8192]: mean (8192 - 128) / ln 64 = 1939
    assert abs(N.mean() - 1939) < 60
    assert abs(np.median(np.log(N)) - 0.5 * (np.log(128) + np.log(8192))) < 0.1
    assert lam.min() >= 0 and lam.max() <= 12 and pd.min() >= 0.7 and pd.max() <= 1.0
    assert int(T.sum()) > 8.2e6                                   # about 8.4e6 track-frames


def test_detection_lists():
    b = synth.make_bpf_batch(3, [100] * 40, [300] * 40, [4.0] * 40, [0.9] * 40)
    J = b.model["J"]
    cnt = np.diff(b.det_off).reshape(-1, J)
    assert cnt.max() <= 16 and cnt.min() >= 0
    # P_D = 0.9 true detections plus Poisson(4) clutter per list, before the cap at 16
    assert abs(cnt.mean() - (0.9 + 4.0)) < 0.15
    assert np.isfinite(b.det).all()
    t = b.tracks[0]
    assert abs(t["kappa"] - 4.0 / (640 * 480)) < 1e-15 and t["sigma"] == synth.SIGMA_PX == 4.0
