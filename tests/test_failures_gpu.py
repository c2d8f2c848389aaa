"""Failure detection without a GPU fault: faults are made on the host (NaN
detections, an over-long detection list, a far-away measurement) and the
kernels must report them in their status words, take the reference's
recovery path (uniform fallback ancestors), and keep tracking afterwards."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ST_FALLBACK, ST_NAN, ST_TRUNC = 1, 2, 8


def _poisoned_batch():
    from mkfbodytracker_pdaf_gb300 import synth
    batch = synth.make_bpf_batch(13, [700, 1500, 300], [8, 8, 8], [3.0, 3.0, 3.0], [0.9, 0.9, 0.9])
    J = batch.model["J"]
    det = batch.det.copy()
    off = batch.det_off.astype(np.int64).copy()
    # track 0, frame 3: every detection NaN (every particle's log-likelihood is NaN)
    g = int(batch.tracks[0]["frame_base"]) + 3
    det[off[g * J]:off[(g + 1) * J]] = np.nan
    # track 1, frame 2, joint 0: 20 detections (more than the 16 a list may hold)
    g1 = int(batch.tracks[1]["frame_base"]) + 2
    lo, hi = off[g1 * J], off[g1 * J + 1]
    extra = np.tile(det[lo:hi][:1] if hi > lo else np.array([[320.0, 240.0]], np.float32), (20 - (hi - lo), 1))
    det = np.concatenate([det[:hi], extra, det[hi:]]).astype(np.float32)
    off[g1 * J + 1:] += len(extra)
    batch.det, batch.det_off = det, off.astype(batch.det_off.dtype)
    return batch, g


@pytest.mark.parametrize("variant", [3, 11], ids=["search", "search_lowsmem"])
def test_batched_reports_and_recovers(cuda, olib, variant):
    """Both search layouts; the over-long list is in frame 2, so it reaches the
    kernel through the next-frame list copy, not the first frame's direct read."""
    from mkfbodytracker_pdaf_gb300.filters import BatchedBootstrapPF
    torch = cuda
    batch, g_nan = _poisoned_batch()
    runner = BatchedBootstrapPF(batch, block_threads=256, ctas_per_sm=3 if variant == 11 else 0, variant=variant)
    N0, T0 = int(batch.tracks[0]["n_particles"]), int(batch.tracks[0]["n_frames"])
    wd = torch.zeros((T0, N0), dtype=torch.float32, device="cuda")
    ad = torch.zeros((T0, N0), dtype=torch.int32, device="cuda")
    runner.set_debug(0, wd, ad)
    est, ll, ess, st = runner.run(*runner.device_inputs())
    torch.cuda.synchronize()
    st = st.cpu().numpy()
    assert st[0] & ST_FALLBACK and st[0] & ST_NAN
    assert st[1] & ST_TRUNC and not st[1] & (ST_FALLBACK | ST_NAN)
    assert st[2] == 0
    # the NaN frame resampled with the reference's uniform fallback: floor(u_i N)
    f = g_nan - int(batch.tracks[0]["frame_base"])
    U = int(olib.draw_block(int(batch.tracks[0]["seed"]), int(batch.tracks[0]["track_id"]), f, 0xFFFFFFFF, 0x100)[0])
    anc_ref, fb = olib.resample(np.zeros(N0, np.float32), N0, U)
    assert fb
    np.testing.assert_array_equal(ad[f].cpu().numpy(), anc_ref)
    # tracking resumes: every later frame's estimate is finite
    e = est.cpu().numpy()
    g0 = int(batch.tracks[0]["frame_base"])
    assert np.isfinite(e[g_nan + 1:g0 + T0]).all()
    assert np.isfinite(e[int(batch.tracks[1]["frame_base"]):]).all()


def test_batched_first_frame_truncation(cuda):
    """An over-long list in a track's first frame (read directly, not copied
    ahead) is truncated and reported the same way."""
    from mkfbodytracker_pdaf_gb300 import synth
    from mkfbodytracker_pdaf_gb300.filters import BatchedBootstrapPF
    batch = synth.make_bpf_batch(17, [400, 900], [3, 3], [2.0, 2.0], [0.9, 0.9])
    J = batch.model["J"]
    det = batch.det.copy()
    off = batch.det_off.astype(np.int64).copy()
    g = int(batch.tracks[1]["frame_base"])          # track 1, frame 0, joint 0
    lo, hi = off[g * J], off[g * J + 1]
    extra = np.tile(np.array([[320.0, 240.0]], np.float32), (20 - (hi - lo), 1))
    det = np.concatenate([det[:hi], extra, det[hi:]]).astype(np.float32)
    off[g * J + 1:] += len(extra)
    batch.det, batch.det_off = det, off.astype(batch.det_off.dtype)
    for variant, cps in ((3, 0), (11, 3)):
        runner = BatchedBootstrapPF(batch, block_threads=256, ctas_per_sm=cps, variant=variant)
        est, ll, ess, st = runner.run(*runner.device_inputs())
        cuda.cuda.synchronize()
        st = st.cpu().numpy()
        assert st[0] == 0 and st[1] == ST_TRUNC, (variant, st)
        assert np.isfinite(est.cpu().numpy()).all()


def test_plain_path_reports_nan_frame(cuda):
    from mkfbodytracker_pdaf_gb300.filters import BootstrapParticleFilter
    torch = cuda
    batch, g_nan = _poisoned_batch()
    t = batch.tracks[0]
    J = batch.model["J"]
    pf = BootstrapParticleFilter(batch.model, t)
    pf.reset()
    g0 = int(t["frame_base"])
    ests = []
    for f in range(int(t["n_frames"])):
        lo = batch.det_off[(g0 + f) * J:(g0 + f) * J + J + 1].astype(np.int64)
        det = torch.from_numpy(np.ascontiguousarray(batch.det[lo[0]:lo[-1]])).cuda()
        off = torch.from_numpy((lo - lo[0]).astype(np.int32)).cuda()
        ests.append(pf.update(f, off, det).cpu().numpy().copy())
    assert pf.status() & ST_FALLBACK and pf.status() & ST_NAN
    assert np.isfinite(np.stack(ests[g_nan - g0 + 1:])).all()


def test_rbpf_nan_measurement_takes_fallback(cuda, olib):
    from mkfbodytracker_pdaf_gb300 import synth
    from mkfbodytracker_pdaf_gb300.filters import MEAS_PINHOLE, RaoBlackwellisedPF
    torch = cuda
    sc = synth.make_rbpf_scene(T=4)
    arm = sc.arms[0]
    N = 256
    pf = RaoBlackwellisedPF(12, 4, 15, N, meas_mode=MEAS_PINHOLE, seed=2, track_id=0)
    for k in range(15):
        pf.set_component(k, arm["mu"][k], np.diag(arm["F"][k]), arm["Q"][k], arm["Sigma"][k], arm["R"][k],
                         arm["weight"][k])
    pf.set_pinhole(arm["Bm"], arm["mm"], synth.CAM)
    pf.resetTracker()
    z = torch.full((N, 4), float("nan"), dtype=torch.float64, device="cuda")
    pf.update(z, frame=0)
    assert pf.status() & ST_FALLBACK
    anc = pf.read()["anc"].cpu().numpy()
    assert ((anc >= 0) & (anc < N)).all()
    good = torch.from_numpy(np.tile([320.0, 200.0, 300.0, 300.0], (N, 1))).cuda()
    pf.update(good, frame=1)
    assert np.isfinite(pf.getEstimator().cpu().numpy()).all()
