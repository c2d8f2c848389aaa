"""Host-side mirror of the reference's filter classes over the C ABI.

``BootstrapParticleFilter`` follows pf2D's ``ParticleFilter`` (pf2D.h:25-51:
construct, predict+update per frame, getEstimator) with the mixture motion
model of ``my_gmm`` (my_gmm.cpp:45-75); ``BatchedBootstrapPF`` runs thousands
of such filters over uneven tracks in one persistent launch.  Device buffers
are torch CUDA tensors (plumbing only); all arithmetic runs in
libmkf_gb300.so.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


class Models:
    """Stacked model arrays (mkf_bpf_models) from a synthetic/user model dict with
    keys a, mu, Lq (packed), S0c (packed), pi, Bm, mm, cam, d, K, J."""

    def __init__(self, model, index=None):
        sel = (lambda a: a) if index is None else (lambda a: a[index:index + 1])
        self.arrays = {k: _f32(sel(model[k])) for k in ("a", "mu", "Lq", "S0c", "pi", "Bm", "mm")}
        n = self.arrays["a"].shape[0]
        fx, fy, cx, cy = model["cam"]
        ptr = {k: v.ctypes.data_as(C.c_void_p) for k, v in self.arrays.items()}
        self.s = N.BpfModels(n, model["d"], model["K"], model["J"], ptr["a"], ptr["mu"], ptr["Lq"],
                             ptr["S0c"], ptr["pi"], ptr["Bm"], ptr["mm"], fx, fy, cx, cy)
        self.d = model["d"]
        self.J = model["J"]


def _track_struct(t, model_index=None, frame_base=None):
    return N.BpfTrack(int(t["n_particles"]), int(t["n_frames"]),
                      int(t["frame_base"] if frame_base is None else frame_base),
                      int(t["seed"]), int(t["track_id"]),
                      int(t["param_index"] if model_index is None else model_index),
                      float(t["kappa"]), float(t["pd"]), float(t["sigma"]))


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _stream(torch, stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


class BootstrapParticleFilter:
    """One track: ParticleFilter(N) with reset / update(frame, detections) / getEstimator."""

    def __init__(self, model, track, model_index=None):
        import torch
        self.torch = torch
        mi = track["param_index"] if model_index is None else model_index
        self.models = Models(model, index=mi)
        self.track = track
        self.d = model["d"]
        self.N = int(track["n_particles"])
        h = C.c_void_p()
        N.check(N.lib().mkf_bpf_create(C.byref(self.models.s), C.byref(_track_struct(track, 0)),
                                       C.byref(h)), "mkf_bpf_create")
        self.h = h
        dev = torch.device("cuda")
        self.est = torch.zeros(self.d, dtype=torch.float32, device=dev)
        self.loglik = torch.zeros(1, dtype=torch.float32, device=dev)
        self.ess = torch.zeros(1, dtype=torch.float32, device=dev)

    def set_debug(self, on=True):
        N.check(N.lib().mkf_bpf_set_debug(self.h, int(on)), "mkf_bpf_set_debug")

    def reset(self, stream=None):
        N.check(N.lib().mkf_bpf_reset(self.h, _stream(self.torch, stream)), "mkf_bpf_reset")

    def update(self, frame, det_off, det, est=None, loglik=None, ess=None, stream=None):
        """det_off: int32 CUDA tensor (J+1), det: float32 CUDA tensor (M, 2)."""
        est = self.est if est is None else est
        loglik = self.loglik if loglik is None else loglik
        ess = self.ess if ess is None else ess
        N.check(N.lib().mkf_bpf_update(self.h, int(frame), _ptr(det_off), _ptr(det), _ptr(est),
                                       _ptr(loglik), _ptr(ess), _stream(self.torch, stream)),
                "mkf_bpf_update")
        return est

    def getEstimator(self):
        return self.est

    def debug_views(self, stream=None):
        """(x SoA (d,N), logw (N), w (N), anc (N)) copied from the last update."""
        torch = self.torch
        x = torch.empty((self.d, self.N), dtype=torch.float32, device="cuda")
        lw = torch.empty(self.N, dtype=torch.float32, device="cuda")
        w = torch.empty(self.N, dtype=torch.float32, device="cuda")
        anc = torch.empty(self.N, dtype=torch.int32, device="cuda")
        N.check(N.lib().mkf_bpf_read_debug(self.h, _ptr(x), _ptr(lw), _ptr(w), _ptr(anc),
                                           _stream(torch, stream)), "mkf_bpf_read_debug")
        return x, lw, w, anc

    def status(self):
        s = C.c_int()
        N.check(N.lib().mkf_bpf_status(self.h, C.byref(s)), "mkf_bpf_status")
        return s.value

    def capture(self, n_frames, det_off, det, est=None, loglik=None, ess=None):
        """Record n_frames consecutive updates into a CUDA graph (FrameGraph).
        det_off: int32 CUDA tensor (n_frames*J + 1) of offsets into det; est
        (n_frames, d), loglik, ess (n_frames): CUDA tensors or None."""
        return FrameGraph(self, n_frames, det_off, det, est, loglik, ess)

    def __del__(self):
        try:
            if getattr(self, "h", None):
                N.lib().mkf_bpf_destroy(self.h)
                self.h = None
        except Exception:
            pass


class FrameGraph:
    """A captured frame loop of one BootstrapParticleFilter; launch(frame0) runs
    frames frame0 .. frame0 + n_frames - 1 from the buffers bound at capture."""

    def __init__(self, pf, n_frames, det_off, det, est, loglik, ess):
        self.pf = pf                      # keeps the filter (and its buffers) alive
        self.n_frames = int(n_frames)
        self.buffers = (det_off, det, est, loglik, ess)
        g = C.c_void_p()
        N.check(N.lib().mkf_bpf_graph_create(pf.h, self.n_frames, _ptr(det_off), _ptr(det), _ptr(est),
                                             _ptr(loglik), _ptr(ess), C.byref(g)), "mkf_bpf_graph_create")
        self.g = g

    def launch(self, frame0=0, stream=None):
        N.check(N.lib().mkf_bpf_graph_launch(self.g, int(frame0) & 0xFFFFFFFF, _stream(self.pf.torch, stream)),
                "mkf_bpf_graph_launch")

    def __del__(self):
        try:
            if getattr(self, "g", None):
                N.lib().mkf_bpf_graph_destroy(self.g)
                self.g = None
        except Exception:
            pass


class BatchedBootstrapPF:
    """All tracks of a synth.BpfBatch (or equivalent) in one persistent launch.
    Launch shape and code variant default to the autotuned choice
    (autotune.load_tuning); any of them can be given explicitly."""

    def __init__(self, batch, block_threads=None, ctas_per_sm=None, variant=None):
        import torch
        from .autotune import load_tuning
        tb, cps, var = load_tuning()
        block_threads = tb if block_threads is None else block_threads
        ctas_per_sm = cps if ctas_per_sm is None else ctas_per_sm
        variant = var if variant is None else variant
        self.torch = torch
        self.batch = batch
        m = batch.model
        self.models = Models(m)
        self.d, self.J = m["d"], m["J"]
        tr = (N.BpfTrack * batch.n_tracks)()
        for b, t in enumerate(batch.tracks):
            tr[b] = _track_struct(t)
        self._tracks = tr
        h = C.c_void_p()
        N.check(N.lib().mkf_bpf_batch_create(C.byref(self.models.s), batch.n_tracks,
                                             C.cast(tr, C.c_void_p), batch.n_frames_total,
                                             C.byref(h)), "mkf_bpf_batch_create")
        self.h = h
        self.set_tuning(block_threads, ctas_per_sm, variant)

    def set_tuning(self, block_threads, ctas_per_sm=0, variant=None):
        N.check(N.lib().mkf_bpf_batch_set_tuning(self.h, int(block_threads), int(ctas_per_sm)),
                "mkf_bpf_batch_set_tuning")
        self.block_threads, self.ctas_per_sm = block_threads, ctas_per_sm
        if variant is not None:
            N.check(N.lib().mkf_bpf_batch_set_variant(self.h, int(variant)), "mkf_bpf_batch_set_variant")
            self.variant = variant

    def device_inputs(self):
        torch = self.torch
        return (torch.from_numpy(np.ascontiguousarray(self.batch.det_off, np.int32)).cuda(),
                torch.from_numpy(np.ascontiguousarray(self.batch.det, np.float32)).cuda())

    def alloc_outputs(self):
        torch = self.torch
        G = self.batch.n_frames_total
        return (torch.empty((G, self.d), dtype=torch.float32, device="cuda"),
                torch.empty(G, dtype=torch.float32, device="cuda"),
                torch.empty(G, dtype=torch.float32, device="cuda"),
                torch.empty(self.batch.n_tracks, dtype=torch.int32, device="cuda"))

    def run(self, det_off, det, outs=None, stream=None):
        outs = self.alloc_outputs() if outs is None else outs
        est, ll, ess, st = outs
        N.check(N.lib().mkf_bpf_batch_run(self.h, _ptr(det_off), _ptr(det), _ptr(est), _ptr(ll),
                                          _ptr(ess), _ptr(st), _stream(self.torch, stream)),
                "mkf_bpf_batch_run")
        return outs

    def run_host(self, det_off, det, outs, stream=None):
        """Host buffers in and out (pinned numpy views recommended)."""
        est, ll, ess, st = outs
        pp = lambda a: a.ctypes.data_as(C.c_void_p)
        N.check(N.lib().mkf_bpf_batch_run_host(self.h, pp(det_off), pp(det), int(det.shape[0]),
                                               pp(est), pp(ll), pp(ess), pp(st),
                                               _stream(self.torch, stream)), "mkf_bpf_batch_run_host")
        return outs

    def set_debug(self, track, w=None, anc=None):
        N.check(N.lib().mkf_bpf_batch_set_debug(self.h, int(track), _ptr(w), _ptr(anc)),
                "mkf_bpf_batch_set_debug")

    def last_grid(self):
        """CTAs of the last run's persistent grid (SMs x resident CTAs per SM)."""
        g = C.c_int()
        N.check(N.lib().mkf_bpf_batch_last_grid(self.h, C.byref(g)), "mkf_bpf_batch_last_grid")
        return g.value

    def __del__(self):
        try:
            if getattr(self, "h", None):
                N.lib().mkf_bpf_batch_destroy(self.h)
                self.h = None
        except Exception:
            pass


# ---------------------------------------------------------------------- RBPF (pf2DRao)
MEAS_LINEAR, MEAS_PINHOLE = 0, 1


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _hp(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


class LegacyParticleFilter:
    """pf2D's ParticleFilter(numParticles, numDims, side) with its own my_gmm
    prior (pf2D.h:12-51): update(measurement) = weight by prior x likelihood,
    normalise, resample (uniform re-initialisation when every weight is 0),
    predict; getEstimator = sum of weights x particles.  FP64 on the GPU."""

    def __init__(self, n_particles, mean, cov, w, side=0, width=640, height=480, seed=0, track_id=0):
        import torch
        self.torch = torch
        mean = _d(mean)
        self.K, self.d = mean.shape
        self.N = int(n_particles)
        h = C.c_void_p()
        N.check(N.lib().mkf_pf2d_create(self.N, self.d, int(side), self.K, _hp(mean), _hp(_d(cov)), _hp(_d(w)),
                                        int(width), int(height), int(seed), int(track_id), C.byref(h)),
                "mkf_pf2d_create")
        self.h = h
        self.est = torch.zeros(self.d, dtype=torch.float64, device="cuda")
        self.seed, self.track_id = int(seed), int(track_id)

    def update(self, measurement, frame, stream=None):
        """measurement: 2x2 (head x, y; hand x, y) on the host."""
        z = _d(measurement).ravel()
        N.check(N.lib().mkf_pf2d_update(self.h, int(frame), _hp(z), _stream(self.torch, stream)), "mkf_pf2d_update")

    def getEstimator(self, out=None, stream=None):
        out = self.est if out is None else out
        N.check(N.lib().mkf_pf2d_estimate(self.h, _ptr(out), _stream(self.torch, stream)), "mkf_pf2d_estimate")
        return out

    def read(self, stream=None):
        t = self.torch
        x = t.empty((self.N, self.d), dtype=t.float64, device="cuda")
        w = t.empty(self.N, dtype=t.float64, device="cuda")
        anc = t.empty(self.N, dtype=t.int32, device="cuda")
        r = C.c_int(0)
        N.check(N.lib().mkf_pf2d_read(self.h, _ptr(x), _ptr(w), _ptr(anc), C.byref(r), _stream(self.torch, stream)),
                "mkf_pf2d_read")
        return {"x": x, "w": w, "anc": anc, "reinit": bool(r.value)}

    def draws(self, frame, stream=None):
        """(eps (N, 8), u (N, d)): this filter's normals and uniforms of one frame."""
        t = self.torch
        eps = t.empty((self.N, 8), dtype=t.float64, device="cuda")
        u = t.empty((self.N, self.d), dtype=t.float64, device="cuda")
        N.check(N.lib().mkf_pf2d_draws(self.seed, self.track_id, int(frame) & 0xFFFFFFFF, self.N, self.d,
                                       _ptr(eps), _ptr(u), _stream(self.torch, stream)), "mkf_pf2d_draws")
        return eps, u

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and h.value:
            N.lib().mkf_pf2d_destroy(h)
            self.h = None


class RaoBlackwellisedPF:
    """pf2DRao ParticleFilter(nParticles) with its my_gmm (pf2DRao.h:13-31):
    loadGaussian / resetTracker / update(measurement) / getEstimator, FP64 on
    the GPU.  Measurements are (N, m) CUDA tensors, one row per particle."""

    def __init__(self, d, m, K, n_particles, meas_mode=MEAS_LINEAR, seed=0, track_id=0):
        import torch
        self.torch = torch
        self.d, self.m, self.K, self.N, self.mode = d, m, K, n_particles, meas_mode
        h = C.c_void_p()
        N.check(N.lib().mkf_rbpf_create(d, m, K, n_particles, meas_mode, int(seed), int(track_id),
                                        C.byref(h)), "mkf_rbpf_create")
        self.h = h
        self.est = torch.zeros(d, dtype=torch.float64, device="cuda")

    # my_gmm::loadGaussian (reference form: F = gI, Q = (1-g^2) s, R = 100 I6, H = H1 Hpca^T)
    def loadGaussian(self, k, u, s, Hpca, mpca, w, g):
        Hpca = _d(Hpca)
        N.check(N.lib().mkf_rbpf_load_gaussian(self.h, k, _hp(_d(u).ravel()), _hp(_d(s)), _hp(Hpca),
                                               _hp(_d(mpca).ravel()), Hpca.shape[1], float(w), float(g)),
                "mkf_rbpf_load_gaussian")

    def set_component(self, k, mu, a, Q, Sigma, R, w, H=None, BH=None):
        N.check(N.lib().mkf_rbpf_set_component(
            self.h, k, _hp(_d(mu)), _hp(_d(a)), _hp(_d(Q)), _hp(_d(Sigma)), _hp(_d(R)), float(w),
            _hp(_d(H) if H is not None else None), _hp(_d(BH) if BH is not None else None)),
            "mkf_rbpf_set_component")

    def set_pinhole(self, Bm, mm, cam):
        fx, fy, cx, cy = cam
        N.check(N.lib().mkf_rbpf_set_pinhole(self.h, _hp(_d(Bm)), _hp(_d(mm)), fx, fy, cx, cy),
                "mkf_rbpf_set_pinhole")

    def set_hand_decode(self, Hd=None, hb=None, joint=1):
        N.check(N.lib().mkf_rbpf_set_hand_decode(self.h, _hp(_d(Hd) if Hd is not None else None),
                                                 _hp(_d(hb) if hb is not None else None), joint),
                "mkf_rbpf_set_hand_decode")

    def resetTracker(self, bins=None, stream=None):
        b = np.ascontiguousarray(bins, np.int32) if bins is not None else None
        N.check(N.lib().mkf_rbpf_reset(self.h, _hp(b), _stream(self.torch, stream)), "mkf_rbpf_reset")

    def update(self, meas, mask=None, frame=0, U=None, stream=None):
        mask = (1 << self.m) - 1 if mask is None else mask
        if U is None:
            N.check(N.lib().mkf_rbpf_update(self.h, int(frame), _ptr(meas), mask, _stream(self.torch, stream)),
                    "mkf_rbpf_update")
        else:
            N.check(N.lib().mkf_rbpf_update_u(self.h, _ptr(meas), mask, int(U[0]), int(U[1]),
                                              _stream(self.torch, stream)), "mkf_rbpf_update_u")

    def getEstimator(self, out=None, stream=None):
        out = self.est if out is None else out
        N.check(N.lib().mkf_rbpf_estimate(self.h, _ptr(out), _stream(self.torch, stream)), "mkf_rbpf_estimate")
        return out

    def read(self, stream=None):
        t = self.torch
        d, Np = self.d, self.N
        o = dict(x=t.empty((Np, d), dtype=t.float64, device="cuda"),
                 P=t.empty((Np, d, d), dtype=t.float64, device="cuda"),
                 logw=t.empty(Np, dtype=t.float64, device="cuda"),
                 wn=t.empty(Np, dtype=t.float64, device="cuda"),
                 ind=t.empty(Np, dtype=t.int32, device="cuda"),
                 anc=t.empty(Np, dtype=t.int32, device="cuda"))
        N.check(N.lib().mkf_rbpf_read(self.h, _ptr(o["x"]), _ptr(o["P"]), _ptr(o["logw"]), _ptr(o["wn"]),
                                      _ptr(o["ind"]), _ptr(o["anc"]), _stream(t, stream)), "mkf_rbpf_read")
        return o

    def write(self, x, P, stream=None):
        N.check(N.lib().mkf_rbpf_write(self.h, _ptr(x), _ptr(P), _stream(self.torch, stream)), "mkf_rbpf_write")

    def status(self):
        s = C.c_int()
        N.check(N.lib().mkf_rbpf_status(self.h, C.byref(s)), "mkf_rbpf_status")
        return s.value

    def __del__(self):
        try:
            if getattr(self, "h", None):
                N.lib().mkf_rbpf_destroy(self.h)
                self.h = None
        except Exception:
            pass


def pdaf_associate(arm0, arm1, frame, roi, cand, Pa=0.05, clutter=1e-4, meas=None, bins=None, stream=None):
    """PFTracker::getMeasurementProposal over a detection list (pfPose.cpp:210-329).
    roi: (2, 4) host array of (x_offset, y_offset, width, height) per arm;
    cand: (M, 2) float64 CUDA tensor.  Returns (meas0, meas1, bins0, bins1)."""
    torch = arm0.torch
    roi = _d(roi).reshape(8)
    if meas is None:
        meas = (torch.zeros((arm0.N, arm0.m), dtype=torch.float64, device="cuda"),
                torch.zeros((arm1.N, arm1.m), dtype=torch.float64, device="cuda"))
    if bins is None:
        bins = (torch.zeros(arm0.N, dtype=torch.int32, device="cuda"),
                torch.zeros(arm1.N, dtype=torch.int32, device="cuda"))
    M = 0 if cand is None else int(cand.shape[0])
    N.check(N.lib().mkf_pdaf_associate(arm0.h, arm1.h, int(frame), _hp(roi), _ptr(cand) if M else None, M,
                                       float(Pa), float(clutter), _ptr(meas[0]), _ptr(meas[1]),
                                       _ptr(bins[0]), _ptr(bins[1]), _stream(torch, stream)),
            "mkf_pdaf_associate")
    return meas[0], meas[1], bins[0], bins[1]


def likelihood_blur(img, out=None, stream=None):
    """GaussianBlur 15x15, sigma 3 of an (H, W) uint8 CUDA tensor (pfPose.cpp:213)."""
    import torch
    img = img.contiguous()
    H, W = img.shape
    out = torch.empty_like(img) if out is None else out
    N.check(N.lib().mkf_likelihood_blur(_ptr(img), W, H, W, _ptr(out), out.stride(0), _stream(torch, stream)),
            "mkf_likelihood_blur")
    return out


def pdaf_propose_image(arm0, arm1, frame, roi, like, M, init, Pa=0.05, clutter=1e-4, meas=None, bins=None,
                       cands=None, stream=None):
    """getMeasurementProposal over a blurred likelihood image (pfPose.cpp:210-329):
    M candidates per arm (uniform box when init, else around the decoded hand),
    weights L / Z, N bins, measurement rows.  like: (H, W) uint8 CUDA tensor.
    Returns (meas0, meas1, bins0, bins1, cand0, cand1)."""
    torch = arm0.torch
    roi = _d(roi).reshape(8)
    H, W = like.shape
    if meas is None:
        meas = (torch.zeros((arm0.N, arm0.m), dtype=torch.float64, device="cuda"),
                torch.zeros((arm1.N, arm1.m), dtype=torch.float64, device="cuda"))
    if bins is None:
        bins = (torch.zeros(arm0.N, dtype=torch.int32, device="cuda"),
                torch.zeros(arm1.N, dtype=torch.int32, device="cuda"))
    if cands is None:
        cands = (torch.zeros((M, 2), dtype=torch.float64, device="cuda"),
                 torch.zeros((M, 2), dtype=torch.float64, device="cuda"))
    N.check(N.lib().mkf_pdaf_propose_image(arm0.h, arm1.h, int(frame), _hp(roi), _ptr(like), W, H, like.stride(0),
                                           int(M), int(bool(init)), float(Pa), float(clutter), _ptr(meas[0]),
                                           _ptr(meas[1]), _ptr(bins[0]), _ptr(bins[1]), _ptr(cands[0]),
                                           _ptr(cands[1]), _stream(torch, stream)), "mkf_pdaf_propose_image")
    return meas[0], meas[1], bins[0], bins[1], cands[0], cands[1]


class PoseTracker:
    """ROS-free replacement of PFTracker's per-frame flow (pfPose.cpp:332-385):
    with a head ROI present, associate hand candidates (PDAF) and update both
    arms, then read both estimates; with no ROI the frame is skipped
    (pfPose.cpp:370-378).  Arms are RaoBlackwellisedPF instances."""

    def __init__(self, arm0, arm1, Pa=0.05, clutter=1e-4):
        self.arms = (arm0, arm1)
        self.Pa, self.clutter = Pa, clutter
        torch = arm0.torch
        self.torch = torch
        self.meas = (torch.zeros((arm0.N, arm0.m), dtype=torch.float64, device="cuda"),
                     torch.zeros((arm1.N, arm1.m), dtype=torch.float64, device="cuda"))
        self.bins = (torch.zeros(arm0.N, dtype=torch.int32, device="cuda"),
                     torch.zeros(arm1.N, dtype=torch.int32, device="cuda"))
        self.est = (torch.zeros(arm0.d, dtype=torch.float64, device="cuda"),
                    torch.zeros(arm1.d, dtype=torch.float64, device="cuda"))

    def step_image(self, frame, roi, likelihood, n_cand=None):
        """The reference's own frame (pfPose.cpp:332-385): blur the MONO8
        likelihood, propose 10 N candidates per arm (uniform box on the first
        frame after a start or a no-face frame), weight, resample, update.
        roi: (2, 4) or None (no face: skip and restart the proposals)."""
        if roi is None:
            self.init = False
            return None
        torch = self.torch
        if getattr(self, "_blur", None) is None or self._blur.shape != likelihood.shape:
            self._blur = torch.empty_like(likelihood)
        likelihood_blur(likelihood, out=self._blur)
        M = 10 * self.arms[0].N if n_cand is None else int(n_cand)
        pdaf_propose_image(self.arms[0], self.arms[1], frame, roi, self._blur, M, not getattr(self, "init", False),
                           self.Pa, self.clutter, meas=self.meas, bins=self.bins)
        self.init = True
        for a in range(2):
            arm = self.arms[a]
            arm.update(self.meas[a], mask=(1 << arm.m) - 1, frame=frame)
            arm.getEstimator(self.est[a])
        return self.est

    def step(self, frame, roi, cand):
        """roi: (2,4) per-arm ROI or None (no face -> skip); cand: (M,2) CUDA float64."""
        if roi is None:
            return None
        M = 0 if cand is None else int(cand.shape[0])
        pdaf_associate(self.arms[0], self.arms[1], frame, roi, cand, self.Pa, self.clutter,
                       meas=self.meas, bins=self.bins)
        for a in range(2):
            arm = self.arms[a]
            mask = (1 << arm.m) - 1
            if M == 0:
                mask &= ~0b1100          # no hand candidate: hand rows unused
            arm.update(self.meas[a], mask=mask, frame=frame)
            arm.getEstimator(self.est[a])
        return self.est
