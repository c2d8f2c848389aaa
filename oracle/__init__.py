"""CPU oracle for the mkfbodytracker_pdaf filtering hot path.

TEST INFRASTRUCTURE ONLY: an FP64 C restatement of the reference's CPU
arithmetic (KF_model.cpp, my_gmm.cpp, pf2DRao.cpp, pf2D.cpp, pfPose.cpp
association), used by the tests as the parity reference, by ``__graft_entry__.smoke()``
and by ``bench.py``'s CPU-baseline and reference legs.  The product package
(``mkfbodytracker_pdaf_gb300``) never imports it.

Pinned to the reference's own code: the reference's KF_model.cpp, my_gmm.cpp
and pf2DRao.cpp, compiled unmodified against stand-in OpenCV/ROS headers
(oracle/refpin/Makefile), produced tests/golden/refpin.npz, against which
tests/test_refpin.py checks the KF predict/update, loadGaussian, the literal
resampling wheel, the chol/mvnpdf quirk modes and the literal RBPF update
(including its shared-buffer effect).  Also pinned: Philox4x32-10 against the
published Random123 known-answer vectors, the exact resampler against the
literal wheel on dyadic weights, and the KF/Gaussian pieces against closed
forms.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_SO = os.path.join(_BUILD, "libmkf_oracle.so")
_SRC = [os.path.join(_HERE, "mkf_oracle.c"), os.path.join(_HERE, "mkf_oracle_mix.c")]
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (no build system).  -ffp-contract=off keeps
    the bit-exact steps unfused on both x86-64 and aarch64."""
    os.makedirs(_BUILD, exist_ok=True)
    newest = max(os.path.getmtime(p) for p in _SRC + [os.path.join(_HERE, "mkf_oracle.h")])
    if not force and os.path.exists(_SO) and os.path.getmtime(_SO) >= newest:
        return _SO
    tmp = _SO + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-std=gnu11",
           "-o", tmp] + _SRC + ["-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, _SO)
    return _SO


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        _declare(_lib)
    return _lib


P = C.c_void_p
I = C.c_int
U32 = C.c_uint32
U64 = C.c_uint64
D = C.c_double
F = C.c_float


class Model(C.Structure):
    """mko_model (RBPF / KF_model set of one arm)."""
    _fields_ = [("d", I), ("m", I), ("K", I), ("meas_mode", I),
                ("F", P), ("B", P), ("Q", P), ("H", P), ("BH", P), ("R", P), ("weight", P),
                ("Bm", P), ("mm", P), ("fx", D), ("fy", D), ("cx", D), ("cy", D)]


class BpfParams(C.Structure):
    _fields_ = [("d", I), ("K", I), ("J", I),
                ("a", P), ("mb", P), ("mu", P), ("Lq", P), ("S0c", P), ("cumpi", P),
                ("Bm", P), ("mm", P), ("fx", F), ("fy", F), ("cx", F), ("cy", F),
                ("kappa", F), ("pd", F), ("sigma", F)]


class Track(C.Structure):
    _fields_ = [("n_particles", I), ("n_frames", I), ("frame_base", C.c_longlong),
                ("seed", C.c_ulonglong), ("track_id", I), ("param_index", I),
                ("kappa", F), ("pd", F), ("sigma", F)]


class Pf2dModel(C.Structure):
    _fields_ = [("d", I), ("K", I), ("mean", P), ("sinv", P), ("det_s", P), ("w", P),
                ("width", I), ("height", I), ("side", I)]


class MixParams(C.Structure):
    _fields_ = [("d", I), ("K", I), ("J", I), ("mu", P), ("a", P), ("Lq", P), ("pi", P), ("S0", P),
                ("sigma", D), ("fx", D), ("fy", D), ("cx", D), ("cy", D)]


def _declare(L):
    L.mko_philox4x32_10.argtypes = [P, P, P]
    L.mko_draw_block.argtypes = [U64, U32, U32, U32, U32, P]
    L.mko_u01_f32.argtypes = [U32]
    L.mko_u01_f32.restype = F
    L.mko_particle_draws.argtypes = [U64, U32, U32, U32, I, P, P]
    L.mko_resample_wheel.argtypes = [P, I, I, D, P, P]
    L.mko_quantize_f64.argtypes = [P, I, P]
    L.mko_quantize_f64.restype = I
    L.mko_quantize_f32.argtypes = [P, I, P]
    L.mko_quantize_f32.restype = I
    L.mko_resample_exact.argtypes = [P, I, I, U32, P]
    L.mko_resample_f64.argtypes = [P, I, I, U32, P]
    L.mko_resample_f64.restype = I
    L.mko_resample_f32.argtypes = [P, I, I, U32, P]
    L.mko_resample_f32.restype = I
    L.mko_kf_predict.argtypes = [I, P, P, P, P, P]
    L.mko_kf_update.argtypes = [I, I, P, P, P, P, C.c_uint, P, P]
    L.mko_kf_update.restype = I
    L.mko_mvn_logpdf.argtypes = [I, P, P, P, I]
    L.mko_mvn_logpdf.restype = D
    L.mko_load_gaussian_ref.argtypes = [I, I, P, P, P, P, D, P, P, P, P, P, P]
    L.mko_measure.argtypes = [C.POINTER(Model), I, P, P, P]
    L.mko_rbpf_update.argtypes = [C.POINTER(Model), I, P, P, P, C.c_uint, U32, U32, P, P, P, P, P]
    L.mko_rbpf_update.restype = I
    L.mko_rbpf_update_literal.argtypes = [C.POINTER(Model), I, P, P, P, C.c_uint, D, P, D, P, I, P, P, P, P, P]
    L.mko_rbpf_update_literal.restype = I
    L.mko_rbpf_estimate.argtypes = [I, I, P, P]
    L.mko_pdaf_weights.argtypes = [I, P, P, P, P, I, D, D, D, P]
    L.mko_pick_component.argtypes = [P, I, F]
    L.mko_pick_component.restype = I
    L.mko_bpf_prior.argtypes = [C.POINTER(BpfParams), P, F, P]
    L.mko_bpf_propagate.argtypes = [C.POINTER(BpfParams), P, F, P]
    L.mko_bpf_loglik.argtypes = [C.POINTER(BpfParams), P, P, P]
    L.mko_bpf_loglik.restype = D
    L.mko_bpf_run_tracks.argtypes = [I, P, I, I, I, P, P, P, P, P, P, P, P,
                                     F, F, F, F, P, P, P, P, P, I]
    L.mko_bpf_forced_frames.argtypes = [C.POINTER(BpfParams), I, I, P, P, P, P, P, P, P, P, P, P, P, P, I]
    L.mko_bpf_prior_set.argtypes = [C.POINTER(BpfParams), I, P, P, P, I]
    L.mko_num_threads.restype = I
    L.mko_gaussian_blur_u8.argtypes = [P, I, I, P]
    L.mko_image_lookup.argtypes = [I, P, P, I, I, P]
    L.mko_pose_decode.argtypes = [I, I, P, P, P, P]
    L.mko_pose3d.argtypes = [P, P, P]
    L.mko_pose2d_record.argtypes = [P, P, P]
    L.mko_pf2d_load.argtypes = [I, I, P, P, P, P]
    L.mko_pf2d_init.argtypes = [C.POINTER(Pf2dModel), I, P, P, P]
    L.mko_pf2d_update.argtypes = [C.POINTER(Pf2dModel), I, P, P, P, U32, P, P, P, P]
    L.mko_pf2d_update.restype = I
    L.mko_pf2d_estimate.argtypes = [I, I, P, P, P]
    L.mko_mix_forward.argtypes = [C.POINTER(MixParams), I, C.c_longlong, P, P, D, D, P, P]
    L.mko_mix_forward.restype = D
    L.mko_mix_adjoint.argtypes = [C.POINTER(MixParams), I, C.c_longlong, P, P, D, D, P, P, P, P, P, P]
    L.mko_mix_adjoint.restype = D
    L.mko_mix_batch.argtypes = [C.POINTER(MixParams), I, P, P, P, P, P, P, P, P, I, P, P, P, P, P, I]
    L.mko_mix_batch.restype = D


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


# ---------------------------------------------------------------- draws
def philox4x32_10(ctr, key):
    c = _c(ctr, np.uint32)
    k = _c(key, np.uint32)
    o = np.zeros(4, np.uint32)
    lib().mko_philox4x32_10(_p(c), _p(k), _p(o))
    return o


def draw_block(seed, track, frame, item, stream):
    o = np.zeros(4, np.uint32)
    lib().mko_draw_block(seed, track, frame, item, stream, _p(o))
    return o


def particle_draws(seed, track, frame, item, d):
    eps = np.zeros(d, np.float64)
    uc = np.zeros(1, np.float32)
    lib().mko_particle_draws(seed, track, frame, item, d, _p(eps), _p(uc))
    return eps, float(uc[0])


# ---------------------------------------------------------------- resampling
def resample_wheel(w, N, u, fallback=None):
    w = _c(w, np.float64)
    idx = np.zeros(N, np.int32)
    fb = _c(fallback, np.int32) if fallback is not None else None
    lib().mko_resample_wheel(_p(w), len(w), N, float(u), _p(fb), _p(idx))
    return idx


def quantize(w):
    w = np.ascontiguousarray(w)
    q = np.zeros(len(w), np.uint64)
    fn = lib().mko_quantize_f32 if w.dtype == np.float32 else lib().mko_quantize_f64
    if w.dtype != np.float32:
        w = _c(w, np.float64)
    ok = fn(_p(w), len(w), _p(q))
    return q, bool(ok)


def resample_exact(q, N, U):
    q = _c(q, np.uint64)
    idx = np.zeros(N, np.int32)
    lib().mko_resample_exact(_p(q), len(q), N, U, _p(idx))
    return idx


def resample(w, N, U):
    """Quantised exact systematic resampler (+ fallback); dtype decides f32/f64."""
    w = np.ascontiguousarray(w)
    idx = np.zeros(N, np.int32)
    if w.dtype == np.float32:
        fb = lib().mko_resample_f32(_p(w), len(w), N, U, _p(idx))
    else:
        w = _c(w, np.float64)
        fb = lib().mko_resample_f64(_p(w), len(w), N, U, _p(idx))
    return idx, bool(fb)


# ---------------------------------------------------------------- KF / Gaussian
def kf_predict(F_, B, Q, x, Pm):
    x = _c(x, np.float64).copy()
    Pm = _c(Pm, np.float64).copy()
    d = len(x)
    lib().mko_kf_predict(d, _p(_c(F_, np.float64)), _p(_c(B, np.float64)), _p(_c(Q, np.float64)),
                         _p(x), _p(Pm))
    return x, Pm


def kf_update(H, BH, R, z, x, Pm, mask=None):
    x = _c(x, np.float64).copy()
    Pm = _c(Pm, np.float64).copy()
    H = _c(H, np.float64)
    m, d = H.shape
    if mask is None:
        mask = (1 << m) - 1
    ok = lib().mko_kf_update(d, m, _p(H), _p(_c(BH, np.float64)), _p(_c(R, np.float64)),
                             _p(_c(z, np.float64)), mask, _p(x), _p(Pm))
    return x, Pm, bool(ok)


def mvn_logpdf(x, u, S, mode=0):
    x = _c(x, np.float64)
    return lib().mko_mvn_logpdf(len(x), _p(x), _p(_c(u, np.float64)), _p(_c(S, np.float64)), mode)


def load_gaussian_ref(u, s, Hpca, mpca, g):
    u = _c(u, np.float64).ravel()
    d = len(u)
    Hpca = _c(Hpca, np.float64)
    Fd = Hpca.shape[1]
    out = dict(F=np.zeros((d, d)), B=np.zeros(d), Q=np.zeros((d, d)), H=np.zeros((6, d)),
               BH=np.zeros(6), R=np.zeros((6, 6)))
    lib().mko_load_gaussian_ref(d, Fd, _p(u), _p(_c(s, np.float64)), _p(Hpca),
                                _p(_c(mpca, np.float64).ravel()), float(g),
                                *[_p(out[k]) for k in ("F", "B", "Q", "H", "BH", "R")])
    return out


# ---------------------------------------------------------------- RBPF (A8)
class RbpfModel:
    """Holds numpy arrays alive for an mko_model."""

    def __init__(self, d, m, K, F_, B, Q, R, weight, H=None, BH=None, Bm=None, mm=None,
                 cam=(525.0, 525.0, 319.5, 239.5)):
        self.arrs = {}

        def keep(name, a):
            if a is None:
                return None
            a = _c(a, np.float64)
            self.arrs[name] = a
            return _p(a)

        mode = 0 if H is not None else 1
        self.s = Model(d, m, K, mode, keep("F", F_), keep("B", B), keep("Q", Q), keep("H", H),
                       keep("BH", BH), keep("R", R), keep("w", weight), keep("Bm", Bm),
                       keep("mm", mm), cam[0], cam[1], cam[2], cam[3])
        self.d, self.m, self.K = d, m, K

    def measure(self, k, x):
        zh = np.zeros(self.m)
        Hx = np.zeros((self.m, self.d))
        lib().mko_measure(C.byref(self.s), k, _p(_c(x, np.float64)), _p(zh), _p(Hx))
        return zh, Hx

    def update(self, x, Pm, z, U_ind, U_anc, mask=None, alias_prev_anc=None):
        """x (N,d), P (N,d,d), z (N,m) -> dict; x,P updated in place copies."""
        x = _c(x, np.float64).copy()
        Pm = _c(Pm, np.float64).copy()
        N = x.shape[0]
        if mask is None:
            mask = (1 << self.m) - 1
        out = dict(ind=np.zeros(N, np.int32), logw=np.zeros(N), wn=np.zeros(N),
                   anc=np.zeros(N, np.int32))
        pa = _c(alias_prev_anc, np.int32) if alias_prev_anc is not None else None
        fb = lib().mko_rbpf_update(C.byref(self.s), N, _p(x), _p(Pm), _p(_c(z, np.float64)),
                                   mask, U_ind, U_anc, _p(pa), _p(out["ind"]), _p(out["logw"]),
                                   _p(out["wn"]), _p(out["anc"]))
        out.update(x=x, P=Pm, fallback=bool(fb))
        return out

    def update_literal(self, x, Pm, z, u_ind, u_anc, mvn_mode, mask=None, alias_prev_anc=None,
                       fb_ind=None, fb_anc=None):
        """The update with the reference's literal pieces (the wheel on double
        uniforms, the Gaussian in mvn_mode, linear-domain weights):
        mko_rbpf_update_literal."""
        x = _c(x, np.float64).copy()
        Pm = _c(Pm, np.float64).copy()
        N = x.shape[0]
        if mask is None:
            mask = (1 << self.m) - 1
        out = dict(ind=np.zeros(N, np.int32), logw=np.zeros(N), wn=np.zeros(N),
                   anc=np.zeros(N, np.int32))
        pa = _c(alias_prev_anc, np.int32) if alias_prev_anc is not None else None
        fi = _c(fb_ind, np.int32) if fb_ind is not None else None
        fa = _c(fb_anc, np.int32) if fb_anc is not None else None
        fb = lib().mko_rbpf_update_literal(C.byref(self.s), N, _p(x), _p(Pm), _p(_c(z, np.float64)), mask,
                                           float(u_ind), _p(fi), float(u_anc), _p(fa), int(mvn_mode), _p(pa),
                                           _p(out["ind"]), _p(out["logw"]), _p(out["wn"]), _p(out["anc"]))
        out.update(x=x, P=Pm, fallback=bool(fb))
        return out


def pdaf_weights(cand, hat_own, hat_other, var, Pa=0.05, clutter=1e-4, Lc=None):
    cand = _c(cand, np.float64).reshape(-1, 2)
    M = cand.shape[0]
    w = np.zeros(M)
    has_other = hat_other is not None
    lib().mko_pdaf_weights(M, _p(cand), _p(_c(Lc, np.float64) if Lc is not None else None),
                           _p(_c(hat_own, np.float64)),
                           _p(_c(hat_other if has_other else [0, 0], np.float64)),
                           int(has_other), float(var), float(Pa), float(clutter), _p(w))
    return w


# ---------------------------------------------------------------- A13
def bpf_params(model, p, track):
    """Build BpfParams for parameter block p of a synthetic.BpfBatch-like model."""
    keep = []

    def ptr(a):
        a = _c(a, np.float32)
        keep.append(a)
        return _p(a)

    d, K, J = model["d"], model["K"], model["J"]
    s = BpfParams(d, K, J, ptr(model["a"][p]), ptr(model["mb"][p]), ptr(model["mu"][p]),
                  ptr(model["Lq"][p]), ptr(model["S0c"][p]), ptr(model["cumpi"][p]),
                  ptr(model["Bm"][p]), ptr(model["mm"][p]), *[float(v) for v in model["cam"]],
                  float(track["kappa"]), float(track["pd"]), float(track["sigma"]))
    return s, keep


def bpf_prior(params, eps, ucomp):
    x = np.zeros(params.d)
    lib().mko_bpf_prior(C.byref(params), _p(_c(eps, np.float64)), float(ucomp), _p(x))
    return x


def bpf_propagate(params, x, eps, ucomp):
    x = _c(x, np.float64).copy()
    lib().mko_bpf_propagate(C.byref(params), _p(_c(eps, np.float64)), float(ucomp), _p(x))
    return x


def bpf_loglik(params, x, det_off, det):
    return lib().mko_bpf_loglik(C.byref(params), _p(_c(x, np.float64)), _p(_c(det_off, np.int32)),
                                _p(_c(det, np.float32)))


def bpf_run_tracks(batch, track_ids, nthreads=0):
    """Run the FP64 CPU bootstrap filter over the listed tracks of a batch
    (synthetic.BpfBatch); returns est, loglik, ess arrays (frame-indexed)."""
    L = lib()
    m = batch.model
    d, K, J = m["d"], m["K"], m["J"]
    tr = (Track * len(track_ids))()
    for n, b in enumerate(track_ids):
        t = batch.tracks[b]
        tr[n] = Track(int(t["n_particles"]), int(t["n_frames"]), int(t["frame_base"]),
                      int(t["seed"]), int(t["track_id"]), int(t["param_index"]),
                      float(t["kappa"]), float(t["pd"]), float(t["sigma"]))
    G = batch.n_frames_total
    est = np.zeros((G, d), np.float32)
    ll = np.zeros(G, np.float32)
    ess = np.zeros(G, np.float32)
    arrs = [_c(m[k], np.float32) for k in ("a", "mb", "mu", "Lq", "S0c", "cumpi", "Bm", "mm")]
    L.mko_bpf_run_tracks(len(track_ids), C.cast(tr, C.c_void_p), d, K, J, *[_p(a) for a in arrs],
                         *[float(v) for v in m["cam"]], _p(_c(batch.det_off, np.int32)),
                         _p(_c(batch.det, np.float32)), _p(est), _p(ll), _p(ess), int(nthreads))
    return est, ll, ess


def bpf_prior_set(params, eps, ucomp, nthreads=0):
    """FP64 prior set (N, d) from the device's prior draws eps (N, d), ucomp (N)."""
    eps = _c(eps, np.float32)
    N = eps.shape[0]
    x = np.zeros((N, params.d))
    lib().mko_bpf_prior_set(C.byref(params), N, _p(eps), _p(_c(ucomp, np.float32)), _p(x), int(nthreads))
    return x


def bpf_forced_frames(params, x, anc_prev, eps, ucomp, anc, w_dev, det_off, det, nthreads=0):
    """Teacher-forced FP64 replay of consecutive frames of one track
    (mkf_oracle.h: mko_bpf_forced_frames).  x (N, d) is updated in place to
    the set of the last frame.  eps (nf, N, d), ucomp / anc / w_dev (nf, N),
    det_off (nf*J + 1) into det.  Returns est (nf, d), loglik, ess, w_err (nf)."""
    eps = _c(eps, np.float32)
    nf, N = eps.shape[0], eps.shape[1]
    assert x.dtype == np.float64 and x.flags.c_contiguous and x.shape == (N, params.d)
    est = np.zeros((nf, params.d))
    ll = np.zeros(nf)
    ess = np.zeros(nf)
    werr = np.zeros(nf)
    wd = _c(w_dev, np.float32) if w_dev is not None else None
    lib().mko_bpf_forced_frames(C.byref(params), N, nf, _p(x), _p(_c(anc_prev, np.int32)), _p(eps),
                                _p(_c(ucomp, np.float32)), _p(_c(anc, np.int32)), _p(wd),
                                _p(_c(det_off, np.int32)), _p(_c(det, np.float32)), _p(est), _p(ll),
                                _p(ess), _p(werr), int(nthreads))
    return est, ll, ess, werr


def num_threads():
    return lib().mko_num_threads()


# ---------------------------------------------------------------- two-arm PFTracker flow
def scene_roi(heads_a):
    """ROI (x_offset, y_offset, width, height) from an arm's head list (cx, cy, w)."""
    cx, cy, w = heads_a[0]
    return np.array([cx - w / 2.0, cy - w / 2.0, w, w])


def rbpf_model_from_arm(arm, cam=(525.0, 525.0, 319.5, 239.5)):
    return RbpfModel(arm["d"], arm["m"], arm["K"], arm["F"], arm["B"], arm["Q"], arm["R"], arm["weight"],
                     Bm=arm["Bm"], mm=arm["mm"], cam=cam)


def project_joint(arm, x, joint, cam=(525.0, 525.0, 319.5, 239.5)):
    p = arm["Bm"][joint] @ x + arm["mm"][joint]
    return np.array([cam[0] * p[0] / p[2] + cam[2], cam[1] * p[1] / p[2] + cam[3]])


def pose_tracker_run(scene, N, seed, T=None, Pa=0.05, clutter=1e-4, hand_joint=1, alias=False):
    """CPU restatement of PFTracker's frame loop (pfPose.cpp:210-385) on the
    two-arm pose scene: per frame, PDAF association of the pooled hand detections
    to each arm (pfPose.cpp:247-301), the per-particle measurement columns
    (303-323), both arms' ParticleFilter::update (325-326) and getEstimator
    (347-348).  A frame without a head ROI for either arm is skipped
    (370-378).  Draws follow the library's Philox conventions."""
    T = len(scene.frames) if T is None else T
    arms = scene.arms
    models = [rbpf_model_from_arm(a) for a in arms]
    d = arms[0]["d"]
    xs, Ps, prev = [], [], [None, None]
    for a in range(2):
        U0 = int(draw_block(seed, a, 0xFFFFFFFF, 0xFFFFFFFF, 0x102)[0])
        bins, _ = resample(arms[a]["weight"], N, U0)
        xs.append(arms[a]["mu"][bins].copy())
        Ps.append(arms[a]["Sigma"][bins].copy())
    est = np.full((2, T, d), np.nan)
    skipped = np.zeros(T, bool)
    for t in range(T):
        fr = scene.frames[t]
        if any(len(fr["heads"][a]) == 0 for a in range(2)):
            skipped[t] = True
            continue
        rois = [scene_roi(fr["heads"][a]) for a in range(2)]
        ests = [xs[a].mean(0) for a in range(2)]
        hats = [project_joint(arms[a], ests[a], hand_joint) for a in range(2)]
        hands = fr["hands"]
        M = len(hands)
        for a in range(2):
            o = 1 - a
            r = rois[a]
            head = (r[0] + r[2] / 2.0, r[1] + 0.5 * r[3])
            z = np.zeros((N, arms[a]["m"]))
            z[:, 0], z[:, 1] = head
            mask = (1 << arms[a]["m"]) - 1
            if M:
                w = pdaf_weights(hands, hats[a], hats[o], 0.8 * r[2], Pa, clutter)
                wn = w / w.sum()
                U = int(draw_block(seed, a, t, 0xFFFFFFFF, 0x103)[0])
                bins, _ = resample(wn, N, U)
                z[:, 2:4] = hands[bins]
            else:
                mask &= ~0b1100
            Ui = int(draw_block(seed, a, t, 0xFFFFFFFF, 0x102)[0])
            Ua = int(draw_block(seed, a, t, 0xFFFFFFFF, 0x100)[0])
            out = models[a].update(xs[a], Ps[a], z, Ui, Ua, mask=mask,
                                   alias_prev_anc=prev[a] if alias else None)
            xs[a], Ps[a] = out["x"], out["P"]
            prev[a] = out["anc"]
        for a in range(2):
            est[a, t] = xs[a].mean(0)
    return est, skipped


# ---------------------------------------------------------------- A11 mixture KF + adjoint
class MixModel:
    """FP64 mixture-KF parameters (theta = mu, a, Lq packed, sigma; fixed pi, S0, camera)."""

    def __init__(self, mu, a, Lq, sigma, pi, S0, cam=(525.0, 525.0, 319.5, 239.5), J=2):
        self.mu, self.a, self.Lq = _c(mu, np.float64), _c(a, np.float64), _c(Lq, np.float64)
        self.pi, self.S0 = _c(pi, np.float64), _c(S0, np.float64)
        self.K, self.d = self.mu.shape
        self.sigma = float(sigma)
        self.cam = cam
        self.J = J
        self.s = MixParams(self.d, self.K, J, _p(self.mu), _p(self.a), _p(self.Lq), _p(self.pi), _p(self.S0),
                           self.sigma, *cam)

    def theta(self):
        return np.concatenate([self.mu.ravel(), self.a.ravel(), self.Lq.ravel(), [self.sigma]])

    def with_theta(self, th):
        K, d = self.K, self.d
        DD = d * (d + 1) // 2
        mu = th[:K * d].reshape(K, d)
        a = th[K * d:2 * K * d].reshape(K, d)
        Lq = th[2 * K * d:2 * K * d + K * DD].reshape(K, DD)
        return MixModel(mu, a, Lq, th[-1], self.pi, self.S0, self.cam, self.J)


def mix_batch(model, batch, grad=False, nthreads=0, tracks=None):
    """Sum over tracks of the mixture-KF logL (and its gradient as a flat theta
    vector) for a synth.MixBatch-like object."""
    ids = list(range(batch.n_tracks)) if tracks is None else list(tracks)
    nf = np.array([batch.tracks[b]["n_frames"] for b in ids], np.int32)
    fb = np.array([batch.tracks[b]["frame_base"] for b in ids], np.int64)
    Bm = _c(np.stack([batch.Bm[batch.tracks[b]["body"]] for b in ids]), np.float64)
    mm = _c(np.stack([batch.mm[batch.tracks[b]["body"]] for b in ids]), np.float64)
    pd = np.array([batch.tracks[b]["pd"] for b in ids], np.float64)
    kp = np.array([batch.tracks[b]["kappa"] for b in ids], np.float64)
    K, d = model.K, model.d
    DD = d * (d + 1) // 2
    ll = np.zeros(len(ids))
    g = [np.zeros(K * d), np.zeros(K * d), np.zeros(K * DD), np.zeros(1)]
    tot = lib().mko_mix_batch(C.byref(model.s), len(ids), _p(nf), _p(fb), _p(Bm), _p(mm), _p(pd), _p(kp),
                              _p(_c(batch.det_off, np.int32)), _p(_c(batch.det, np.float32)), int(grad),
                              _p(ll), *[_p(x) for x in g], int(nthreads))
    if grad:
        return tot, ll, np.concatenate(g)
    return tot, ll


# ---------------------------------------------------------------- A12 legacy pf2D
class Pf2d:
    """FP64 literal restatement of pf2D's ParticleFilter (injected draws)."""

    def __init__(self, mean, cov, w, width=640, height=480, side=0):
        self.mean = _c(mean, np.float64)
        self.K, self.d = self.mean.shape
        self.sinv = np.zeros((self.K, self.d, self.d))
        self.det_s = np.zeros(self.K)
        self.w = _c(w, np.float64)
        lib().mko_pf2d_load(self.d, self.K, _p(self.mean), _p(_c(cov, np.float64)), _p(self.sinv), _p(self.det_s))
        self.s = Pf2dModel(self.d, self.K, _p(self.mean), _p(self.sinv), _p(self.det_s), _p(self.w),
                           width, height, side)

    def init(self, u):
        N = u.shape[0]
        x = np.zeros((N, self.d))
        wts = np.zeros(N)
        lib().mko_pf2d_init(C.byref(self.s), N, _p(_c(u, np.float64)), _p(x), _p(wts))
        return x, wts

    def update(self, x, wts, z, U, reinit_u, eps):
        x = _c(x, np.float64).copy()
        wts = _c(wts, np.float64).copy()
        N = x.shape[0]
        wout = np.zeros(N)
        anc = np.zeros(N, np.int32)
        r = lib().mko_pf2d_update(C.byref(self.s), N, _p(x), _p(wts), _p(_c(z, np.float64)), U,
                                  _p(_c(reinit_u, np.float64)), _p(_c(eps, np.float64)), _p(wout), _p(anc))
        return x, wts, wout, anc, bool(r)

    def estimate(self, x, wts):
        est = np.zeros(self.d)
        lib().mko_pf2d_estimate(x.shape[0], self.d, _p(_c(x, np.float64)), _p(_c(wts, np.float64)), _p(est))
        return est


# ---------------------------------------------------------------- f2 pose decode
KINECT_K = np.array([[525.0, 0.0, 319.5], [0.0, 525.0, 239.5], [0.0, 0.0, 1.0]])


def pose_decode(Hpca, mpca, x):
    Hpca = _c(Hpca, np.float64)
    d, F = Hpca.shape
    e = np.zeros(F)
    lib().mko_pose_decode(d, F, _p(Hpca), _p(_c(mpca, np.float64)), _p(_c(x, np.float64)), _p(e))
    return e


def pose3d(e, Kc=KINECT_K):
    out = np.zeros((3, 5))
    lib().mko_pose3d(_p(_c(e, np.float64)), _p(_c(Kc, np.float64)), _p(out))
    return out


def pose2d_record(e1, e2):
    out = np.zeros(16)
    lib().mko_pose2d_record(_p(_c(e1, np.float64)), _p(_c(e2, np.float64)), _p(out))
    return out.reshape(8, 2)


# ---------------------------------------------------------------- f1 image front end
def gaussian_blur_u8(img):
    img = np.ascontiguousarray(img, np.uint8)
    H, W = img.shape
    out = np.zeros_like(img)
    lib().mko_gaussian_blur_u8(_p(img), W, H, _p(out))
    return out


def image_lookup(cand, img):
    img = np.ascontiguousarray(img, np.uint8)
    H, W = img.shape
    cand = _c(cand, np.float64).reshape(-1, 2)
    L = np.zeros(cand.shape[0])
    lib().mko_image_lookup(cand.shape[0], _p(cand), _p(img), W, H, _p(L))
    return L
