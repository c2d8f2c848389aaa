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


def _draw_into(torch, seed, track, frame, eps, uc):
    from mkfbodytracker_pdaf_gb300 import _native as N
    n, d = eps.shape
    st = N.lib().mkf_draw_particles(seed, track, frame, n, d, C.c_void_p(eps.data_ptr()),
                                    C.c_void_p(uc.data_ptr()), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    N.check(st, "mkf_draw_particles")


def gpu_draws(torch, seed, track, frame, n, d, f64=True):
    eps = torch.empty((n, d), dtype=torch.float32, device="cuda")
    uc = torch.empty(n, dtype=torch.float32, device="cuda")
    _draw_into(torch, seed, track, frame, eps, uc)
    return (eps.double() if f64 else eps).cpu().numpy(), uc.cpu().numpy()


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


class FullReport:
    """Errors of one track's device run against its FP64 teacher-forced replay.

    rel_est[f] = max_c |est_dev - est_64| / max(1, max_c |est_64|) (posterior
    mean, the latent state vector of frame f); rel_ll[f] = |ll_dev - ll_64| /
    max(1, |ll_64|) (log-likelihood increment); w_err[f] = max_i |w_dev - w_64|
    (weights normalised to max 1)."""

    def __init__(self, T):
        self.rel_est = np.zeros(T)
        self.rel_ll = np.zeros(T)
        self.w_err = np.zeros(T)
        self.anc_frames = 0

    def summary(self):
        T = len(self.rel_est)
        q = [0, T // 4, T // 2, 3 * T // 4, T]
        return {"frames": T, "ancestor_frames_bit_exact": self.anc_frames,
                "max_rel_est": float(self.rel_est.max(initial=0.0)),
                "max_rel_loglik": float(self.rel_ll.max(initial=0.0)),
                "max_abs_weight": float(self.w_err.max(initial=0.0)),
                "max_rel_est_by_quarter": [float(self.rel_est[q[k]:q[k + 1]].max(initial=0.0)) for k in range(4)]}


def check_track_full(torch, olib, batch, b, w_dev, anc_dev, est_dev, ll_dev, chunk=100):
    """Teacher-forced FP64 replay of every frame of batched track b.

    w_dev, anc_dev: (T, N) device tensors from the batched kernel's debug dump;
    est_dev (G, d), ll_dev (G): the run's frame-indexed outputs (host arrays).
    The replay takes the device's draws (mkf_draw_particles, one frame at a
    time) and ancestors, and propagates, scores, weights and averages in FP64
    (oracle.bpf_forced_frames); the ancestors are also recomputed from the
    device's weights with the oracle's exact resampler and must match bit for
    bit.  Returns a FullReport."""
    m, t = batch.model, batch.tracks[b]
    prm, keep = olib.bpf_params(m, t["param_index"], t)
    d, J, N, T = m["d"], m["J"], int(t["n_particles"]), int(t["n_frames"])
    seed, trk, g0 = int(t["seed"]), int(t["track_id"]), int(t["frame_base"])
    eps0, uc0 = gpu_draws(torch, seed, trk, PRIOR, N, d, f64=False)
    x = olib.bpf_prior_set(prm, eps0, uc0)
    anc_prev = np.arange(N, dtype=np.int32)
    rep = FullReport(T)
    eps = torch.empty((chunk, N, d), dtype=torch.float32, device="cuda")
    uc = torch.empty((chunk, N), dtype=torch.float32, device="cuda")
    for f0 in range(0, T, chunk):
        nf = min(chunk, T - f0)
        for f in range(nf):
            _draw_into(torch, seed, trk, f0 + f, eps[f], uc[f])
        eps_h = eps[:nf].cpu().numpy()
        uc_h = uc[:nf].cpu().numpy()
        anc_h = anc_dev[f0:f0 + nf].cpu().numpy()
        w_h = w_dev[f0:f0 + nf].cpu().numpy()
        off = batch.det_off[(g0 + f0) * J:(g0 + f0 + nf) * J + 1]
        e, ll, _, werr = olib.bpf_forced_frames(prm, x, anc_prev, eps_h, uc_h, anc_h, w_h, off, batch.det)
        eg = np.asarray(est_dev[g0 + f0:g0 + f0 + nf], np.float64)
        lg = np.asarray(ll_dev[g0 + f0:g0 + f0 + nf], np.float64)
        rep.rel_est[f0:f0 + nf] = np.abs(eg - e).max(1) / np.maximum(1.0, np.abs(e).max(1))
        rep.rel_ll[f0:f0 + nf] = np.abs(lg - ll) / np.maximum(1.0, np.abs(ll))
        rep.w_err[f0:f0 + nf] = werr
        for f in range(nf):
            U = int(olib.draw_block(seed, trk, f0 + f, 0xFFFFFFFF, 0x100)[0])
            anc_ref, fb = olib.resample(w_h[f], N, U)
            assert not fb, "fallback resampling at frame %d" % (f0 + f)
            np.testing.assert_array_equal(anc_h[f], anc_ref, err_msg="ancestors differ at frame %d" % (f0 + f))
            rep.anc_frames += 1
        anc_prev = anc_h[nf - 1].copy()
    return rep
