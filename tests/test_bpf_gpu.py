"""GPU parity of the bootstrap particle filter (draws, resampler, plain
per-track path, batched persistent path) against the FP64 oracle."""
import ctypes as C

import numpy as np
import pytest

from bpf_check import check_track, gpu_draws

pytestmark = pytest.mark.gpu


def _stream(torch):
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def test_draws_match_oracle(cuda, olib):
    torch = cuda
    for d in (12, 24):
        eps, uc = gpu_draws(torch, 20140601, 5, 17, 2000, d)
        for i in range(0, 2000, 97):
            e_ref, u_ref = olib.particle_draws(20140601, 5, 17, i, d)
            assert uc[i] == np.float32(u_ref)                         # exact
            np.testing.assert_allclose(eps[i], e_ref, rtol=0, atol=2e-5)  # MUFU vs libm
        assert abs(eps.mean()) < 0.02 and abs(eps.var() - 1) < 0.03


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_resample_bit_exact(cuda, olib, dtype):
    from mkfbodytracker_pdaf_gb300 import _native as N
    torch = cuda
    rng = np.random.default_rng(11)
    cases = [(15, 1000), (1000, 1000), (5000, 3000), (4096, 4096), (70000, 20000), (3, 100000)]
    for L, Np in cases:
        for kind in ("pow", "sparse", "dyadic", "zeros"):
            w = rng.random(L) ** 6
            if kind == "sparse":
                w[rng.random(L) < 0.9] = 0
                w[0] = 0
            if kind == "dyadic":
                w = np.floor(w * 16) / 16
            if kind == "zeros" or w.max() == 0:
                w = np.zeros(L)
            w = w.astype(dtype)
            U = int(rng.integers(0, 2 ** 32))
            ref, fb_ref = olib.resample(w, Np, U)
            dw = torch.from_numpy(w).cuda()
            idx = torch.empty(Np, dtype=torch.int32, device="cuda")
            fb = torch.zeros(1, dtype=torch.int32, device="cuda")
            fn = N.lib().mkf_resample_f32 if dtype == np.float32 else N.lib().mkf_resample_f64
            N.check(fn(C.c_void_p(dw.data_ptr()), L, Np, U, C.c_void_p(idx.data_ptr()),
                       C.c_void_p(fb.data_ptr()), _stream(torch)), "resample")
            torch.cuda.synchronize()
            assert bool(fb.item()) == fb_ref, (L, Np, kind)
            np.testing.assert_array_equal(idx.cpu().numpy(), ref, err_msg="%s L=%d N=%d" % (kind, L, Np))


def _run_stream(torch, batch, b, T, debug=True):
    from mkfbodytracker_pdaf_gb300.filters import BootstrapParticleFilter
    t = batch.tracks[b]
    pf = BootstrapParticleFilter(batch.model, t)
    pf.set_debug(debug)
    pf.reset()
    J = batch.model["J"]
    g0 = int(t["frame_base"])
    frames = []
    for f in range(T):
        lo = batch.det_off[(g0 + f) * J:(g0 + f) * J + J + 1].astype(np.int32)
        det = torch.from_numpy(batch.det[lo[0]:lo[-1]].copy()).cuda()
        off = torch.from_numpy(lo - lo[0]).cuda()
        est = pf.update(f, off, det)
        x, lw, w, anc = pf.debug_views()
        torch.cuda.synchronize()
        frames.append(dict(est=est.double().cpu().numpy().copy(), loglik=float(pf.loglik.item()),
                           ess=float(pf.ess.item()), x=x.cpu().numpy(), w=w.cpu().numpy(),
                           anc=anc.cpu().numpy(), logw=lw.cpu().numpy()))
    return frames, pf


def test_plain_path_teacher_forced_parity(cuda, olib):
    from mkfbodytracker_pdaf_gb300 import synth
    torch = cuda
    batch = synth.sweep_batch(3000, n_frames=6)     # a dozen propagate and search tiles on 152 SMs
    frames, pf = _run_stream(torch, batch, 0, 6)
    rep = check_track(torch, olib, batch, 0, frames)
    assert rep.anc_frames == 6
    assert pf.status() == 0


def test_plain_path_single_tile_parity(cuda, olib):
    from mkfbodytracker_pdaf_gb300 import synth
    torch = cuda
    batch = synth.make_bpf_batch(78, [100], [4], [5.0], [0.85])    # one block per kernel
    frames, _ = _run_stream(torch, batch, 0, 4)
    check_track(torch, olib, batch, 0, frames)


def test_plain_path_multi_tile_parity(cuda, olib):
    from mkfbodytracker_pdaf_gb300 import synth
    torch = cuda
    batch = synth.make_bpf_batch(77, [9000], [3], [8.0], [0.8])   # ~36 propagate and search tiles
    frames, _ = _run_stream(torch, batch, 0, 3)
    check_track(torch, olib, batch, 0, frames)


def test_plain_path_offspring_property_large(cuda, olib):
    """Size-independent check at 2^20 particles: ancestors are sorted and every
    particle's offspring count is the floor or ceil of N q_j / Q."""
    from mkfbodytracker_pdaf_gb300 import synth
    torch = cuda
    N = 1 << 20
    batch = synth.sweep_batch(N, n_frames=3)
    frames, _ = _run_stream(torch, batch, 0, 3)
    for f in frames:
        anc = f["anc"]
        assert np.all(np.diff(anc) >= 0)
        q, ok = olib.quantize(f["w"])
        cnt = np.bincount(anc, minlength=N)
        e = N * q.astype(np.float64) / q.astype(np.float64).sum()
        assert np.all(cnt >= np.floor(e) - 1e-6) and np.all(cnt <= np.ceil(e) + 1e-6)
        assert np.isfinite(f["est"]).all() and np.isfinite(f["loglik"])
        assert 1.0 <= f["ess"] <= N


# (block_threads, ctas_per_sm, variant): every load/resampler variant of the
# d = 12 kernel (bits: 1 float4 loads, 2 search, 4 pairs, 8 search with the
# ancestors in global memory) and the four launch-bound shapes, including the
# autotuned one
BATCHED_SHAPES = [(256, 0, 0), (256, 0, 1), (256, 2, 2), (256, 2, 3), (256, 2, 7), (256, 3, 3), (512, 0, 3),
                  (384, 2, 3), (256, 3, 11), (384, 2, 11), (512, 0, 11)]


@pytest.mark.parametrize("shape", BATCHED_SHAPES, ids=lambda s: "tb%d_cps%d_v%d" % s)
def test_batched_teacher_forced_parity(cuda, olib, shape):
    from mkfbodytracker_pdaf_gb300 import synth
    from mkfbodytracker_pdaf_gb300.filters import BatchedBootstrapPF
    torch = cuda
    Ns = [100, 257, 1024, 3000, 5000, 8192, 64, 700]
    Ts = [7, 5, 9, 4, 3, 2, 12, 0]
    batch = synth.make_bpf_batch(31, Ns, Ts, [3.0, 0.0, 12.0, 6.0, 1.0, 4.0, 2.0, 5.0],
                                 [0.9, 0.7, 0.99, 0.8, 0.75, 0.95, 0.9, 0.9])
    tb, cps, var = shape
    runner = BatchedBootstrapPF(batch, block_threads=tb, ctas_per_sm=cps, variant=var)
    det_off, det = runner.device_inputs()
    for dbg_track in (0, 3, 5):
        N = int(batch.tracks[dbg_track]["n_particles"])
        T = int(batch.tracks[dbg_track]["n_frames"])
        wd = torch.zeros((max(T, 1), N), dtype=torch.float32, device="cuda")
        ad = torch.zeros((max(T, 1), N), dtype=torch.int32, device="cuda")
        runner.set_debug(dbg_track, wd, ad)
        est, ll, ess, st = runner.run(det_off, det)
        torch.cuda.synchronize()
        assert (st.cpu().numpy() & ~8 == 0).all()
        g0 = int(batch.tracks[dbg_track]["frame_base"])
        frames = [dict(est=est[g0 + f].double().cpu().numpy(), loglik=float(ll[g0 + f].item()),
                       w=wd[f].cpu().numpy(), anc=ad[f].cpu().numpy()) for f in range(T)]
        check_track(torch, olib, batch, dbg_track, frames)


@pytest.mark.parametrize("shape", BATCHED_SHAPES, ids=lambda s: "tb%d_cps%d_v%d" % s)
def test_batched_matches_plain_path(cuda, olib, shape):
    """Both launch shapes run the same per-particle code on the same draws."""
    from mkfbodytracker_pdaf_gb300 import synth
    from mkfbodytracker_pdaf_gb300.filters import BatchedBootstrapPF
    torch = cuda
    batch = synth.make_bpf_batch(41, [500, 2048, 4000], [10, 6, 4], [3.0, 5.0, 2.0], [0.9, 0.9, 0.8])
    tb, cps, var = shape
    runner = BatchedBootstrapPF(batch, block_threads=tb, ctas_per_sm=cps, variant=var)
    est, ll, ess, st = runner.run(*runner.device_inputs())
    torch.cuda.synchronize()
    for b in range(3):
        frames, _ = _run_stream(torch, batch, b, int(batch.tracks[b]["n_frames"]), debug=False)
        g0 = int(batch.tracks[b]["frame_base"])
        for f, fr in enumerate(frames):
            np.testing.assert_allclose(est[g0 + f].cpu().numpy(), fr["est"], rtol=1e-4, atol=1e-4)
            assert abs(ll[g0 + f].item() - fr["loglik"]) <= 1e-4 * max(1, abs(fr["loglik"]))


def test_batched_host_buffers_match_device_run(cuda):
    from mkfbodytracker_pdaf_gb300 import synth
    from mkfbodytracker_pdaf_gb300.filters import BatchedBootstrapPF
    torch = cuda
    batch = synth.uneven_tracks_batch(n_tracks=64)
    runner = BatchedBootstrapPF(batch)
    est, ll, ess, st = runner.run(*runner.device_inputs())
    G = batch.n_frames_total
    outs = (np.zeros((G, 12), np.float32), np.zeros(G, np.float32), np.zeros(G, np.float32),
            np.zeros(batch.n_tracks, np.int32))
    runner.run_host(batch.det_off.astype(np.int32), batch.det.astype(np.float32), outs)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(outs[0], est.cpu().numpy())   # deterministic
    np.testing.assert_array_equal(outs[1], ll.cpu().numpy())
    assert np.isfinite(outs[0]).all()
    # tracking sanity: the filter follows the ground truth on average
    err = np.abs(outs[0] - batch.truth).mean()
    assert err < 0.6, err


def test_batched_host_run_head_and_tail_in_any_track_order(cuda):
    """The host-buffer run launches the first grid-size tracks of the
    longest-first order as soon as their own lists are copied, and the rest
    after the bulk copy; outputs go straight into pinned caller buffers or
    through device staging for pageable ones.  With more tracks than the head
    and the tracks listed out of frame order, both forms equal the single
    device-resident launch bit for bit, on repeated calls."""
    from mkfbodytracker_pdaf_gb300 import synth
    from mkfbodytracker_pdaf_gb300.filters import BatchedBootstrapPF
    torch = cuda
    base = synth.uneven_tracks_batch(n_tracks=600, t_range=(3, 30), n_range=(64, 1024))
    perm = np.random.default_rng(5).permutation(base.n_tracks)
    batch = synth.BpfBatch(base.model, [base.tracks[b] for b in perm], base.det_off, base.det, base.truth)
    runner = BatchedBootstrapPF(batch)
    est, ll, ess, st = runner.run(*runner.device_inputs())
    ref = [x.cpu().numpy() for x in (est, ll, ess, st)]
    G = batch.n_frames_total
    for pinned in (False, True, True):
        outs = [torch.full((G, 12), float("nan")), torch.zeros(G), torch.zeros(G),
                torch.zeros(batch.n_tracks, dtype=torch.int32)]
        if pinned:
            outs = [o.pin_memory() for o in outs]
        outs = [o.numpy() for o in outs]
        runner.run_host(batch.det_off.astype(np.int32), batch.det.astype(np.float32), outs)
        for o, r in zip(outs, ref):
            np.testing.assert_array_equal(o, r)


def test_batched_variant_flags_checked(cuda):
    """The search with global ancestors needs float4 loads and the search, not pairs."""
    from mkfbodytracker_pdaf_gb300 import _native as N, synth
    from mkfbodytracker_pdaf_gb300.filters import BatchedBootstrapPF
    batch = synth.make_bpf_batch(3, [64], [2], [1.0], [0.9])
    runner = BatchedBootstrapPF(batch, block_threads=256, ctas_per_sm=0, variant=3)
    for bad in (8, 9, 10, 15, 16):
        assert N.lib().mkf_bpf_batch_set_variant(runner.h, bad) == 1, bad          # MKF_ERR_ARG
    assert N.lib().mkf_bpf_batch_set_variant(runner.h, 11) == 0
    runner.run(*runner.device_inputs())
    cuda.cuda.synchronize()
    assert runner.last_grid() == 1          # capped at the number of tracks


@pytest.mark.parametrize("shape", [(256, 3, 11), (256, 0, 3)], ids=["lowsmem", "search"])
def test_batched_tiny_tracks_parity(cuda, olib, shape):
    """Tracks of 1, 2, 3, 31, 33 and 257 particles (a single particle, fewer
    particles than a warp, one past a warp, one past a CTA) against the oracle,
    teacher-forced, in one batch with a 4096-particle track (so that the small
    tracks keep their ancestors in shared memory under the LOW layout)."""
    from mkfbodytracker_pdaf_gb300 import synth
    from mkfbodytracker_pdaf_gb300.filters import BatchedBootstrapPF
    torch = cuda
    Ns = [1, 2, 3, 31, 33, 257, 4096]
    Ts = [6, 5, 4, 6, 3, 4, 2]
    batch = synth.make_bpf_batch(53, Ns, Ts, [2.0, 0.0, 5.0, 8.0, 1.0, 3.0, 4.0],
                                 [0.9, 0.95, 0.8, 0.7, 0.9, 0.85, 0.9])
    tb, cps, var = shape
    runner = BatchedBootstrapPF(batch, block_threads=tb, ctas_per_sm=cps, variant=var)
    det_off, det = runner.device_inputs()
    for dbg_track in range(len(Ns) - 1):
        N = int(batch.tracks[dbg_track]["n_particles"])
        T = int(batch.tracks[dbg_track]["n_frames"])
        wd = torch.zeros((T, N), dtype=torch.float32, device="cuda")
        ad = torch.zeros((T, N), dtype=torch.int32, device="cuda")
        runner.set_debug(dbg_track, wd, ad)
        est, ll, ess, st = runner.run(det_off, det)
        torch.cuda.synchronize()
        assert (st.cpu().numpy() & ~8 == 0).all()
        g0 = int(batch.tracks[dbg_track]["frame_base"])
        frames = [dict(est=est[g0 + f].double().cpu().numpy(), loglik=float(ll[g0 + f].item()),
                       w=wd[f].cpu().numpy(), anc=ad[f].cpu().numpy()) for f in range(T)]
        check_track(torch, olib, batch, dbg_track, frames)
        if N == 1:
            assert (ad.cpu().numpy() == 0).all()
            assert np.allclose(ess[g0:g0 + T].cpu().numpy(), 1.0)


@pytest.mark.parametrize("n", [1, 3, 33, 257])
def test_plain_path_tiny_tracks_parity(cuda, olib, n):
    """The per-track streaming kernels with a single particle, fewer than a
    warp, one past a warp and one past a block, against the oracle."""
    from mkfbodytracker_pdaf_gb300 import synth
    torch = cuda
    batch = synth.make_bpf_batch(60 + n, [n], [4], [3.0], [0.9])
    frames, pf = _run_stream(torch, batch, 0, 4)
    rep = check_track(torch, olib, batch, 0, frames)
    assert rep.anc_frames == 4
    assert pf.status() == 0
