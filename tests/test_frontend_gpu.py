"""GPU parity of the likelihood-image front end: the 15x15 Gaussian blur is
bit-exact against the oracle, and the image proposal (uniform box on the first
frame, Gaussian around the decoded hands afterwards, L / Z weights) resamples
bit-exactly the same bins as the oracle on the GPU's own candidates."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_blur_bit_exact(cuda, olib):
    from mkfbodytracker_pdaf_gb300.filters import likelihood_blur
    torch = cuda
    rng = np.random.default_rng(1)
    for H, W in ((480, 640), (37, 53), (8, 8)):
        img = rng.integers(0, 256, (H, W)).astype(np.uint8)
        img[: H // 3] = 0                               # flat and saturated regions too
        img[H // 3: H // 2, : W // 2] = 255
        g = likelihood_blur(torch.from_numpy(img).cuda()).cpu().numpy()
        np.testing.assert_array_equal(g, olib.gaussian_blur_u8(img))


def _hand_image(rng, hands, H=480, W=640, sigma=12.0):
    yy, xx = np.mgrid[0:H, 0:W]
    img = np.zeros((H, W))
    for h in hands:
        img += 255.0 * np.exp(-0.5 * ((xx - h[0]) ** 2 + (yy - h[1]) ** 2) / sigma ** 2)
    img += rng.uniform(0, 40, (H, W))
    return np.clip(img, 0, 255).astype(np.uint8)


def test_image_proposal_parity(cuda, olib):
    from mkfbodytracker_pdaf_gb300 import synth
    from mkfbodytracker_pdaf_gb300.filters import (MEAS_PINHOLE, RaoBlackwellisedPF, likelihood_blur,
                                                   pdaf_propose_image)
    torch = cuda
    sc = synth.make_rbpf_scene(T=8)
    N, M = 400, 4000
    arms = []
    for a in range(2):
        arm = sc.arms[a]
        pf = RaoBlackwellisedPF(12, 4, 15, N, meas_mode=MEAS_PINHOLE, seed=21, track_id=a)
        for k in range(15):
            pf.set_component(k, arm["mu"][k], np.diag(arm["F"][k]), arm["Q"][k], arm["Sigma"][k], arm["R"][k],
                             arm["weight"][k])
        pf.set_pinhole(arm["Bm"], arm["mm"], synth.CAM)
        pf.set_hand_decode(joint=1)
        pf.resetTracker()
        arms.append(pf)
    rng = np.random.default_rng(2)
    done = 0
    for t in range(8):
        fr = sc.frames[t]
        if any(len(h) == 0 for h in fr["heads"]):
            continue
        roi = np.stack([olib.scene_roi(fr["heads"][0])] * 2)        # the reference uses ROIs[0] for both arms
        hands = [olib.project_joint(sc.arms[a], sc.truth[a, t], 1) for a in range(2)]
        img = torch.from_numpy(_hand_image(rng, hands)).cuda()
        blur = likelihood_blur(img)
        init = done == 0
        m0, m1, b0, b1, c0, c1 = pdaf_propose_image(arms[0], arms[1], t, roi, blur, M, init)
        bl = blur.cpu().numpy()
        xs = [a.read()["x"].cpu().numpy() for a in arms]
        hats = [olib.project_joint(sc.arms[a], xs[a].mean(0), 1) for a in range(2)]
        for a, (mg, bg, cg) in enumerate(((m0, b0, c0), (m1, b1, c1))):
            cand = cg.cpu().numpy()
            if init:   # uniform in the box below the face, exact from the Philox words
                xo, yo, wi, hi = (int(v) for v in roi[a])
                xmin, xmax = max(xo - 4 * wi, 0), min(xo + 5 * wi, 640)
                ymin, ymax = min(yo + hi, 480), min(yo + 7 * hi, 480)
                for j in (0, 1, M - 1):
                    wd = olib.draw_block(21, a, t, j, 0x104)
                    assert cand[j, 0] == xmin + wd[0] / 2.0 ** 32 * (xmax - xmin)
                    assert cand[j, 1] == ymin + wd[1] / 2.0 ** 32 * (ymax - ymin)
            else:      # N(hand, (0.8 w)^2): standardised draws look standard normal
                z = (cand - hats[a]) / (0.8 * roi[a, 2])
                assert abs(z.mean()) < 0.1 and abs(z.std() - 1.0) < 0.1
            L = olib.image_lookup(cand, bl)
            w = olib.pdaf_weights(cand, hats[a], hats[1 - a], 0.8 * roi[a, 2], Lc=L)
            U = int(olib.draw_block(21, a, t, 0xFFFFFFFF, 0x103)[0])
            bins, fb = olib.resample(w / w.sum(), N, U)
            assert not fb
            np.testing.assert_array_equal(bg.cpu().numpy(), bins)
            mg = mg.cpu().numpy()
            np.testing.assert_array_equal(mg[:, 2:4], cand[bins])
        for a in range(2):
            arms[a].update((m0, m1)[a], frame=t)
        done += 1
    assert done >= 3
