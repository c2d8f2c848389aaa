"""Teacher-forced comparison of a GPU bootstrap-PF run with the FP64 oracle.

Each frame the oracle starts from its own FP64 particle set, resampled with the
GPU's ancestors, propagates it with the GPU's own draws (dumped through
mkf_draw_particles), and scores it in FP64.  Compared per frame: particles
(when given), normalised weights, the weighted-mean estimate, the
log-likelihood increment, and the ancestors (bit-exact, from the GPU's
weights and the frame's resampling uniform).
"""
import ctypes as C

import numpy as np

PRIOR = 0xFFFFFFFF


def gpu_draws(torch, seed, track, frame, n, d):
    from mkfbodytracker_pdaf_gb300 import _native as N
    eps = torch.empty((n, d), dtype=torch.float32, device="cuda")
    uc = torch.empty(n, dtype=torch.float32, device="cuda")
    st = N.lib().mkf_draw_particles(seed, track, frame, n, d, C.c_void_p(eps.data_ptr()),
                                    C.c_void_p(uc.data_ptr()), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    N.check(st, "mkf_draw_particles")
    return eps.double().cpu().numpy(), uc.cpu().numpy()


class Report:
    def __init__(self):
        self.max_rel_est = 0.0
        self.max_abs_ll = 0.0
        self.max_abs_w = 0.0
        self.max_rel_x = 0.0
        self.anc_frames = 0


def check_track(torch, olib, batch, b, frames, tol=1e-4):
    """frames: list over t of dict(est, loglik, w, anc[, x]) produced by the GPU."""
    m, t = batch.model, batch.tracks[b]
    prm, keep = olib.bpf_params(m, t["param_index"], t)
    d, J, N = m["d"], m["J"], int(t["n_particles"])
    seed, trk = int(t["seed"]), int(t["track_id"])
    g0 = int(t["frame_base"])
    eps, uc = gpu_draws(torch, seed, trk, PRIOR, N, d)
    x = np.stack([olib.bpf_prior(prm, eps[i], uc[i]) for i in range(N)])
    anc = np.arange(N)
    rep = Report()
    for f, gf in enumerate(frames):
        eps, uc = gpu_draws(torch, seed, trk, f, N, d)
        xn = np.stack([olib.bpf_propagate(prm, x[anc[i]], eps[i], uc[i]) for i in range(N)])
        off = batch.det_off[(g0 + f) * J:(g0 + f) * J + J + 1].astype(np.int32)
        ll = np.array([olib.bpf_loglik(prm, xn[i], off, batch.det) for i in range(N)])
        if "x" in gf:
            xg = np.asarray(gf["x"], np.float64)          # (d, N)
            rel = np.abs(xg.T - xn).max() / max(1.0, np.abs(xn).max())
            rep.max_rel_x = max(rep.max_rel_x, rel)
        M = ll.max()
        w = np.exp(ll - M)
        wg = np.asarray(gf["w"], np.float64)
        rep.max_abs_w = max(rep.max_abs_w, np.abs(w - wg).max())
        est = (w[:, None] * xn).sum(0) / w.sum()
        rep.max_rel_est = max(rep.max_rel_est, np.abs(est - gf["est"]).max() / max(1.0, np.abs(est).max()))
        lz = M + np.log(w.sum()) - np.log(N)
        rep.max_abs_ll = max(rep.max_abs_ll, abs(lz - gf["loglik"]) / max(1.0, abs(lz)))
        U = int(olib.draw_block(seed, trk, f, 0xFFFFFFFF, 0x100)[0])
        anc_ref, fb = olib.resample(np.asarray(gf["w"], np.float32), N, U)
        assert not fb
        np.testing.assert_array_equal(np.asarray(gf["anc"]), anc_ref,
                                      err_msg="ancestors differ at frame %d" % f)
        rep.anc_frames += 1
        x, anc = xn, np.asarray(gf["anc"])
    assert rep.max_rel_est <= tol, rep.max_rel_est
    assert rep.max_abs_ll <= tol, rep.max_abs_ll
    assert rep.max_abs_w <= tol, rep.max_abs_w
    assert rep.max_rel_x <= tol, rep.max_rel_x
    return rep
