"""GPU parity of the batched pose decode, get3Dpose back-projection and the
publish2Dpos record against the FP64 oracle (shipped arm models)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def test_pose_decode_batched_parity(cuda, olib):
    from mkfbodytracker_pdaf_gb300.pose import PoseDecoder, pose2d_record
    torch = cuda
    z = np.load(os.path.join(HERE, "golden", "ref_models.npz"))
    rng = np.random.default_rng(8)
    B = 1000
    es = []
    for a in range(2):
        H, m = z["arm%d_pca_proj" % a], z["arm%d_pca_mean" % a]
        x = z["arm%d_means" % a][rng.integers(0, 15, B)] + rng.normal(0, 0.5, (B, 12))
        dec = PoseDecoder(H, m)
        e, p3 = dec.decode(torch.from_numpy(x).cuda())
        e, p3 = e.cpu().numpy(), p3.cpu().numpy()
        for b in range(0, B, 37):
            eo = olib.pose_decode(H, m, x[b])
            np.testing.assert_allclose(e[b], eo, rtol=1e-12, atol=1e-9)
            np.testing.assert_allclose(p3[b], olib.pose3d(eo), rtol=1e-9, atol=1e-9)
        assert int(dec.status.item()) == 0
        es.append(e)
    pts = pose2d_record(torch.from_numpy(es[0]).cuda(), torch.from_numpy(es[1]).cuda()).cpu().numpy()
    for b in range(0, B, 53):
        np.testing.assert_array_equal(pts[b], olib.pose2d_record(es[0][b], es[1][b]))
    # empty batch is a no-op
    e0, _ = dec.decode(torch.zeros((0, 12), dtype=torch.float64, device="cuda"))
    assert e0.shape == (0, 22)
