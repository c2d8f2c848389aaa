"""Seeded synthetic workloads standing in for the reference's evaluation data.

The reference's own data (a rosbag of Kinect + webcam frames and ChaLearn
sequences) is not available, so every workload is generated here from a
committed master seed.  Generative model (shared by all workloads):

* motion model (my_gmm.cpp:45-75 generalised): K components over a d-dim PCA
  state; mu_k ~ N(0, I); Sigma_k = Wishart(d+2, 0.1 I)/(d+2); mean reversion
  A_k = diag(U[0.85, 0.99]); process noise Q_k = 0.05 I (L_k = sqrt(0.05) I);
  mixture weights pi ~ Dirichlet(2 * 1).  Per frame a component k ~ pi is drawn
  and x' = A_k x + (I - A_k) mu_k + L_k eps  (the reference redraws the
  component every frame, pf2DRao.cpp:128).
* body: full = Bs x + mbar, Bs = 0.1 m/unit * (random orthonormal d x d basis,
  QR of a Gaussian, sign-fixed); mbar is a fixed joint layout (camera frame,
  y down, z forward) shifted to depth U[1.5, 3] m and x offset U[-0.3, 0.3] m.
* camera: pinhole fx = fy = 525, cx = 319.5, cy = 239.5 (pfPose.cpp:101), 640x480.
* detections: each measured joint (head, hand) is detected with probability
  P_D at its projection + N(0, (4 px)^2); clutter is Poisson(lambda) per list,
  uniform over the image; lists are capped at ``max_det`` entries (true
  detection kept, clutter truncated).  Heads come first in their list (the
  face detector's ROI order, pfPose.cpp:308).
* filter-side clutter density kappa = max(lambda, 0.01)/(640*480) and
  p_detect = min(P_D, 0.999), so that the PDA likelihood
  log[(1-P_D) kappa + P_D sum_i N(z_i; pi(x), sigma^2 I)] is always finite.
"""
from __future__ import annotations

import numpy as np

CAM = (525.0, 525.0, 319.5, 239.5)
IMG_W, IMG_H = 640, 480
SIGMA_PX = 4.0
BASIS_SCALE = 0.1

# joint layouts (metres, camera frame, y down); side = +1 right arm, -1 left arm
_ARM4 = np.array([[0.00, -0.35, 0.00],    # head
                  [0.18, -0.12, 0.02],    # shoulder
                  [0.30, 0.12, -0.02],    # elbow
                  [0.28, 0.30, -0.15]])   # hand
_BODY8 = np.array([[0.00, -0.35, 0.00],   # head
                   [0.00, -0.15, 0.02],   # neck
                   [-0.18, -0.12, 0.02],  # left shoulder
                   [-0.30, 0.12, -0.02],  # left elbow
                   [-0.28, 0.30, -0.15],  # left hand
                   [0.18, -0.12, 0.02],   # right shoulder
                   [0.30, 0.12, -0.02],   # right elbow
                   [0.28, 0.30, -0.15]])  # right hand
MEASURED_ARM4 = (0, 3)          # head, hand
MEASURED_BODY8 = (0, 4, 7)      # head, left hand, right hand


def pack_lower(L):
    """(..., d, d) lower-triangular -> (..., d(d+1)/2) row-major packed."""
    d = L.shape[-1]
    r, c = np.tril_indices(d)
    return L[..., r, c]


def unpack_lower(p, d):
    out = np.zeros(p.shape[:-1] + (d, d), p.dtype)
    r, c = np.tril_indices(d)
    out[..., r, c] = p
    return out


def orthonormal_basis(rng, d, n=None):
    shape = (d, d) if n is None else (n, d, d)
    G = rng.standard_normal(shape)
    Qm, R = np.linalg.qr(G)
    s = np.sign(np.diagonal(R, axis1=-2, axis2=-1))
    s[s == 0] = 1.0
    return Qm * s[..., None, :]


def wishart(rng, df, scale, shape):
    """Wishart(df, scale*I) samples of size shape + (d, d) via sums of outer products."""
    d = scale.shape[0]
    Lc = np.linalg.cholesky(scale)
    G = rng.standard_normal(shape + (df, d)) @ Lc.T
    return np.einsum("...ki,...kj->...ij", G, G)


def make_gmm(rng, d, K, n=None, q_scale=0.05):
    """Motion-model parameters; n stacks independent models (one per track)."""
    lead = () if n is None else (n,)
    mu = rng.standard_normal(lead + (K, d))
    Sigma = wishart(rng, d + 2, 0.1 * np.eye(d), lead + (K,)) / (d + 2)
    a = rng.uniform(0.85, 0.99, lead + (K, d))
    Lq = np.broadcast_to(np.sqrt(q_scale) * np.eye(d), lead + (K, d, d)).copy()
    pi = rng.dirichlet(2.0 * np.ones(K), size=n) if n is not None else rng.dirichlet(2.0 * np.ones(K))
    return dict(mu=mu, Sigma=Sigma, a=a, Lq=Lq, pi=pi)


def make_body(rng, d, n=None, side=1.0, layout="arm4"):
    """Basis and mean pose.  Returns (Bs (..., 3J, d), mbar (..., 3J), measured)."""
    base = _ARM4.copy() if layout == "arm4" else _BODY8.copy()
    if layout == "arm4":
        base[:, 0] *= side
        measured = MEASURED_ARM4
    else:
        measured = MEASURED_BODY8
    J3 = base.size
    assert J3 == d, "state dimension must equal 3 x joints"
    lead = () if n is None else (n,)
    Bs = BASIS_SCALE * orthonormal_basis(rng, d, n)
    depth = rng.uniform(1.5, 3.0, lead)
    xoff = rng.uniform(-0.3, 0.3, lead)
    mbar = np.broadcast_to(base.ravel(), lead + (J3,)).copy()
    mbar = mbar.reshape(lead + (J3 // 3, 3))
    mbar[..., 2] += np.asarray(depth)[..., None]
    mbar[..., 0] += np.asarray(xoff)[..., None]
    return Bs, mbar.reshape(lead + (J3,)), measured


def project(P3, cam=CAM):
    fx, fy, cx, cy = cam
    return np.stack([fx * P3[..., 0] / P3[..., 2] + cx, fy * P3[..., 1] / P3[..., 2] + cy], -1)


def simulate_states(rng, gmm, T, n=None):
    """Ground-truth latent trajectories including the prior draw x_{-1}.
    Single model: returns (T, d).  Stacked (n tracks, common T): (n, T, d)."""
    mu, Sigma, a, Lq, pi = gmm["mu"], gmm["Sigma"], gmm["a"], gmm["Lq"], gmm["pi"]
    if n is None:
        mu, Sigma, a, Lq, pi = mu[None], Sigma[None], a[None], Lq[None], pi[None]
    B_, K, d = mu.shape
    Sc = np.linalg.cholesky(Sigma)
    cum = np.cumsum(pi, -1)
    ar = np.arange(B_)

    def pick():
        u = rng.random(B_)
        return np.minimum((u[:, None] >= cum).sum(-1), K - 1)

    k = pick()
    x = mu[ar, k] + np.einsum("bij,bj->bi", Sc[ar, k], rng.standard_normal((B_, d)))
    out = np.zeros((B_, T, d))
    for t in range(T):
        k = pick()
        x = a[ar, k] * x + (1 - a[ar, k]) * mu[ar, k] + np.einsum(
            "bij,bj->bi", Lq[ar, k], rng.standard_normal((B_, d)))
        out[:, t] = x
    return out[0] if n is None else out


def _lists_from(rng, true_px, detected, lam, max_det, shuffle):
    """Build CSR detection lists.  true_px (L, P, 2) holds P potential true
    detections per list, detected (L, P) bool, lam (L,) clutter rates."""
    Lc = true_px.shape[0]
    ndet = detected.sum(1)
    nclut = rng.poisson(lam)
    nclut = np.minimum(nclut, np.maximum(max_det - ndet, 0))
    cnt = np.minimum(ndet, max_det) + nclut
    off = np.zeros(Lc + 1, np.int64)
    np.cumsum(cnt, out=off[1:])
    pts = np.empty((int(off[-1]), 2), np.float32)
    # true detections first
    P = true_px.shape[1]
    slot = off[:-1].copy()
    for p in range(P):
        m = detected[:, p] & (slot < off[1:])
        pts[slot[m]] = true_px[m, p]
        slot[m] += 1
    # clutter after
    total_c = int(nclut.sum())
    if total_c:
        starts = np.repeat(slot, nclut)
        within = np.arange(total_c) - np.repeat(np.cumsum(nclut) - nclut, nclut)
        pts[starts + within, 0] = rng.uniform(0, IMG_W, total_c)
        pts[starts + within, 1] = rng.uniform(0, IMG_H, total_c)
    if shuffle:
        for i in np.nonzero(cnt > 1)[0]:
            seg = pts[off[i]:off[i + 1]]
            rng.shuffle(seg)
    return off, pts


class BpfBatch:
    """A batch of independent single-arm tracks for the bootstrap PF (A13).

    Frame-indexed arrays use a global frame index g = frame_base[b] + t.
    det_off has G*J + 1 entries: list (g, j) = det[det_off[g*J+j] : det_off[g*J+j+1]].
    Parameter blocks are per track (param_index = b).
    """

    def __init__(self, model, tracks, det_off, det, truth):
        self.model = model
        self.tracks = tracks
        self.det_off = det_off
        self.det = det
        self.truth = truth
        self.n_frames_total = int(sum(int(t["n_frames"]) for t in tracks))

    @property
    def n_tracks(self):
        return len(self.tracks)

    def track_frames(self, b):
        t = self.tracks[b]
        return int(t["frame_base"]), int(t["n_frames"])

    def subset(self, ids):
        """New batch holding only tracks ``ids`` (frames re-based, params kept)."""
        J = self.model["J"]
        tracks, off_chunks, dets, truths = [], [], [], []
        base = 0
        acc = 0
        for b in ids:
            t = dict(self.tracks[b])
            g0, T = self.track_frames(b)
            o = self.det_off[g0 * J:(g0 + T) * J + 1].astype(np.int64)
            dets.append(self.det[o[0]:o[-1]])
            off_chunks.append(o[:-1] - o[0] + acc)
            acc += int(o[-1] - o[0])
            truths.append(self.truth[g0:g0 + T])
            t["frame_base"] = base
            base += T
            tracks.append(t)
        det_off = np.concatenate(off_chunks + [np.array([acc])]).astype(np.int32)
        det = np.concatenate(dets) if dets else np.zeros((0, 2), np.float32)
        return BpfBatch(self.model, tracks, det_off, det, np.concatenate(truths))


def make_bpf_batch(seed, n_particles, n_frames, lam, pd, d=12, K=15, max_det=16,
                   shared_model=False, seed_philox=None):
    """Generate a batch.  n_particles, n_frames, lam, pd: per-track sequences."""
    rng = np.random.default_rng(seed)
    B_ = len(n_particles)
    n_frames = np.asarray(n_frames, np.int64)
    nm = 1 if shared_model else B_
    gmm = make_gmm(rng, d, K, n=nm)
    Bs, mbar, measured = make_body(rng, d, n=nm, layout="arm4" if d == 12 else "body8")
    J = len(measured)
    # simulate in chunks of tracks to bound memory
    G = int(n_frames.sum())
    frame_base = np.zeros(B_, np.int64)
    frame_base[1:] = np.cumsum(n_frames)[:-1]
    truth = np.zeros((G, d), np.float32)
    chunk = 1024
    for s0 in range(0, B_, chunk):
        ids = np.arange(s0, min(B_, s0 + chunk))
        Tc = int(n_frames[ids].max())
        sel = np.zeros(len(ids), np.int64) if shared_model else ids
        g = {k: v[sel] for k, v in gmm.items()}
        xs = simulate_states(rng, g, Tc, n=len(ids))
        for n, b in enumerate(ids):
            T = int(n_frames[b])
            truth[frame_base[b]:frame_base[b] + T] = xs[n, :T]
    # detections: per global frame and measured joint
    pidx = np.repeat(np.arange(B_) if not shared_model else np.zeros(B_, np.int64), n_frames)
    full = np.einsum("gij,gj->gi", Bs[pidx], truth.astype(np.float64)) + mbar[pidx]
    P3 = full.reshape(G, -1, 3)[:, list(measured)]           # (G, J, 3)
    px = project(P3) + rng.normal(0, SIGMA_PX, (G, J, 2))
    pd_f = np.repeat(np.asarray(pd, np.float64), n_frames)
    lam_f = np.repeat(np.asarray(lam, np.float64), n_frames)
    det_mask = rng.random((G, J)) < pd_f[:, None]
    det_mask &= P3[..., 2] > 0.05
    off, pts = _lists_from(rng, px.reshape(G * J, 1, 2), det_mask.reshape(G * J, 1),
                           np.repeat(lam_f, J), max_det, shuffle=False)
    # model arrays for the filter (float32, packed)
    Lq_p = pack_lower(gmm["Lq"]).astype(np.float32)
    S0c = pack_lower(np.linalg.cholesky(gmm["Sigma"])).astype(np.float32)
    pi32 = gmm["pi"].astype(np.float32)
    a32 = gmm["a"].astype(np.float32)
    mu32 = gmm["mu"].astype(np.float32)
    # the library cumulates pi sequentially in float32 and forms (1-a) mu in
    # double from the float32 inputs; the same arrays are built here for the oracle
    cumpi = np.cumsum(pi32, -1, dtype=np.float32)
    model = dict(d=d, K=K, J=J, cam=CAM, pi=pi32,
                 a=a32, mu=mu32,
                 mb=((1.0 - a32.astype(np.float64)) * mu32.astype(np.float64)).astype(np.float32),
                 Lq=Lq_p, S0c=S0c, cumpi=cumpi,
                 Bm=Bs.reshape(nm, -1, 3, d)[:, list(measured)].astype(np.float32),
                 mm=mbar.reshape(nm, -1, 3)[:, list(measured)].astype(np.float32),
                 gmm=gmm, Bs=Bs, mbar=mbar, measured=measured)
    ps = seed if seed_philox is None else seed_philox
    tracks = []
    for b in range(B_):
        tracks.append(dict(n_particles=int(n_particles[b]), n_frames=int(n_frames[b]),
                           frame_base=int(frame_base[b]), seed=int(ps), track_id=b,
                           param_index=0 if shared_model else b,
                           kappa=float(max(lam[b], 0.01) / (IMG_W * IMG_H)),
                           pd=float(min(pd[b], 0.999)), sigma=SIGMA_PX, lam=float(lam[b])))
    return BpfBatch(model, tracks, off.astype(np.int32), pts, truth)


# ----------------------------------------------------------------- workloads
MASTER_SEED = 20140601


def sweep_batch(n_particles, n_frames=200, seed=MASTER_SEED + 1, lam=3.0, pd=0.9):
    """Particle-count sweep: one track, one arm."""
    return make_bpf_batch(seed, [n_particles], [n_frames], [lam], [pd])


def uneven_tracks_spec(seed=MASTER_SEED + 2, n_tracks=8192, t_range=(50, 2000), n_range=(128, 8192),
                 lam_range=(0.0, 12.0), pd_range=(0.7, 1.0)):
    rng = np.random.default_rng(seed)
    T = rng.integers(t_range[0], t_range[1] + 1, n_tracks)
    N = np.exp(rng.uniform(np.log(n_range[0]), np.log(n_range[1]), n_tracks)).round().astype(np.int64)
    N = np.clip(N, n_range[0], n_range[1])
    lam = rng.uniform(*lam_range, n_tracks)
    pd = rng.uniform(*pd_range, n_tracks)
    return N, T, lam, pd


def uneven_tracks_batch(n_tracks=8192, seed=MASTER_SEED + 2, **kw):
    """Batched uneven tracks: per-track GMM, T ~ U{50..2000}, N log-uniform
    in [128, 8192], lambda ~ U[0, 12], P_D ~ U[0.7, 1]."""
    N, T, lam, pd = uneven_tracks_spec(seed, n_tracks, **kw)
    return make_bpf_batch(seed + 100, N, T, lam, pd)


# ----------------------------------------------------------------- two-arm pose scene
class RbpfScene:
    """Two-arm pose scene: two arms, each its own K=15, d=12 GMM and body; per frame
    a head ROI list per arm (true head first) and one pooled, shuffled hand list."""

    def __init__(self, arms, frames, truth):
        self.arms = arms          # list of dicts (model arrays, FP64)
        self.frames = frames      # list of dicts: heads [(M_a,3)], hands (M,2)
        self.truth = truth        # (2, T, d)


def make_rbpf_scene(seed=MASTER_SEED, T=500, d=12, K=15, lam=3.0, pd=0.9, max_det=16):
    rng = np.random.default_rng(seed)
    arms, truths, px_heads, px_hands, zheads = [], [], [], [], []
    for side in (-1.0, 1.0):
        gmm = make_gmm(rng, d, K)
        Bs, mbar, measured = make_body(rng, d, side=side)
        x = simulate_states(rng, gmm, T)
        full = x @ Bs.T + mbar
        P3 = full.reshape(T, -1, 3)
        px = project(P3)
        arms.append(dict(d=d, K=K, m=4, gmm=gmm, Bs=Bs, mbar=mbar,
                         F=np.stack([np.diag(a) for a in gmm["a"]]),
                         B=(1 - gmm["a"]) * gmm["mu"],
                         Q=np.einsum("kij,klj->kil", gmm["Lq"], gmm["Lq"]),
                         R=np.broadcast_to(SIGMA_PX ** 2 * np.eye(4), (K, 4, 4)).copy(),
                         weight=gmm["pi"], mu=gmm["mu"], Sigma=gmm["Sigma"],
                         Bm=Bs.reshape(-1, 3, d)[list(measured)],
                         mm=mbar.reshape(-1, 3)[list(measured)]))
        truths.append(x)
        px_heads.append(px[:, measured[0]])
        px_hands.append(px[:, measured[1]])
        zheads.append(P3[:, measured[0], 2])
    frames = []
    for t in range(T):
        heads = []
        for a in range(2):
            lst = []
            if rng.random() < pd:
                c = px_heads[a][t] + rng.normal(0, SIGMA_PX, 2)
                lst.append([c[0], c[1], 0.16 * CAM[0] / zheads[a][t]])
            for _ in range(min(rng.poisson(lam), max_det - len(lst))):
                lst.append([rng.uniform(0, IMG_W), rng.uniform(0, IMG_H), rng.uniform(20, 60)])
            heads.append(np.array(lst, np.float64).reshape(-1, 3))
        hands = []
        for a in range(2):
            if rng.random() < pd:
                hands.append(px_hands[a][t] + rng.normal(0, SIGMA_PX, 2))
        for _ in range(min(rng.poisson(lam), max_det - len(hands))):
            hands.append([rng.uniform(0, IMG_W), rng.uniform(0, IMG_H)])
        hands = np.array(hands, np.float64).reshape(-1, 2)
        rng.shuffle(hands)
        frames.append(dict(heads=heads, hands=hands))
    return RbpfScene(arms, frames, np.stack(truths))


# ----------------------------------------------------------------- mixture-KF logL and fitting
class MixBatch:
    """Tracks sharing one motion model (theta), each with its own body
    (basis + mean pose + depth) and detection lists.  det_off indexes
    (global frame g, joint j) lists like BpfBatch."""

    def __init__(self, gmm, tracks, Bm, mm, det_off, det, truth, cam=CAM):
        self.gmm, self.tracks, self.Bm, self.mm = gmm, tracks, Bm, mm
        self.det_off, self.det, self.truth, self.cam = det_off, det, truth, cam
        self.n_frames_total = int(sum(t["n_frames"] for t in tracks))
        self.J = Bm.shape[1]

    @property
    def n_tracks(self):
        return len(self.tracks)

    def theta_true(self, sigma=SIGMA_PX):
        return dict(mu=self.gmm["mu"], a=self.gmm["a"], Lq=pack_lower(self.gmm["Lq"]), sigma=sigma,
                    pi=self.gmm["pi"], S0=self.gmm["Sigma"])


def make_mix_batch(seed, n_tracks, T, K=15, d=12, lam=3.0, pd=0.9, layout="arm4", max_det=16, chunk=2048):
    rng = np.random.default_rng(seed)
    gmm = make_gmm(rng, d, K)
    Bs, mbar, measured = make_body(rng, d, n=n_tracks, layout=layout)
    J = len(measured)
    G = n_tracks * T
    truth = np.zeros((G, d), np.float32)
    for s0 in range(0, n_tracks, chunk):
        n = min(chunk, n_tracks - s0)
        g = {k: np.broadcast_to(v, (n,) + v.shape) for k, v in gmm.items()}
        xs = simulate_states(rng, g, T, n=n)
        truth[s0 * T:(s0 + n) * T] = xs.reshape(n * T, d)
    bidx = np.repeat(np.arange(n_tracks), T)
    full = np.einsum("gij,gj->gi", Bs[bidx], truth.astype(np.float64)) + mbar[bidx]
    P3 = full.reshape(G, -1, 3)[:, list(measured)]
    px = project(P3) + rng.normal(0, SIGMA_PX, (G, J, 2))
    det_mask = (rng.random((G, J)) < pd) & (P3[..., 2] > 0.05)
    off, pts = _lists_from(rng, px.reshape(G * J, 1, 2), det_mask.reshape(G * J, 1),
                           np.full(G * J, lam), max_det, shuffle=False)
    tracks = [dict(n_frames=T, frame_base=b * T, body=b, pd=float(min(pd, 0.999)),
                   kappa=float(max(lam, 0.01) / (IMG_W * IMG_H))) for b in range(n_tracks)]
    Bm = Bs.reshape(n_tracks, -1, 3, d)[:, list(measured)].copy()
    mm = mbar.reshape(n_tracks, -1, 3)[:, list(measured)].copy()
    return MixBatch(gmm, tracks, Bm, mm, off.astype(np.int32), pts, truth)


def mixkf_batch_k15(n_tracks=1024, T=1000, seed=MASTER_SEED + 3):
    """Differentiation workload: B=1024 x T=1000, K=15, d=12, PDAF over <=16 candidates."""
    return make_mix_batch(seed, n_tracks, T, K=15, d=12, lam=3.0, pd=0.9)


def fit_batch_k32(n_tracks=16384, T=500, seed=MASTER_SEED + 4):
    """Fitting workload: ground-truth GMM K=32, d=24 (8 joints x 3D), lambda=5."""
    return make_mix_batch(seed, n_tracks, T, K=32, d=24, lam=5.0, pd=0.9, layout="body8")


def fit_batch_exact(n_tracks=128, T=200, seed=MASTER_SEED + 5, K=1):
    """Fitting control case: d=12, arm layout, no clutter and detection
    probability 0.999.  With one component (the default) the mixture-KF
    likelihood is the model's own up to the EKF linearisation of the
    projection; with more, the filter's per-frame collapse of the mixture makes
    it an approximation."""
    return make_mix_batch(seed, n_tracks, T, K=K, d=12, lam=0.0, pd=0.999, layout="arm4")


# ------------------------------------------------- reference-model (LINEAR) scene
def make_reference_scene(arms, T=60, seed=MASTER_SEED + 7, clutter_rate=3.0, sigma_px=4.0, roi_w=40.0,
                         no_face_every=0):
    """A synthetic sequence for the shipped (u, v, Z)-state models: each arm's
    latent state follows the AR(1) of one of its components; per frame the head
    ROI is placed so that its centre and the 1.65-height neck point match the
    decoded head and neck (as PFTracker reads them, pfPose.cpp:303-323); hand
    candidates are both decoded hands + N(0, sigma_px^2) plus Poisson clutter
    over the 640 x 480 image.  arms: dicts of means, covs, weights, pca_proj,
    pca_mean, gamma (cvyaml.load_reference_models)."""
    rng = np.random.default_rng(seed)
    d = arms[0]["means"].shape[1]
    xs = np.zeros((2, T, d))
    for a, arm in enumerate(arms):
        k = int(rng.integers(0, arm["means"].shape[0]))
        g = float(arm["gamma"][k])
        mu = arm["means"][k]
        L = np.linalg.cholesky(arm["covs"][k * d:(k + 1) * d] + 1e-9 * np.eye(d))
        x = mu.copy()
        for t in range(T):
            x = g * x + (1 - g) * mu + np.sqrt(max(1 - g * g, 0.0)) * (L @ rng.normal(0, 1, d))
            xs[a, t] = x
    e = np.stack([xs[a] @ arms[a]["pca_proj"] + arms[a]["pca_mean"] for a in range(2)])
    rois, cands = [], []
    for t in range(T):
        head = 0.5 * (e[0, t, 9:11] + e[1, t, 9:11])
        neck = 0.5 * (e[0, t, 12:14] + e[1, t, 12:14])
        h = max(abs(neck[1] - head[1]) / 1.15, 10.0)
        roi = np.array([head[0] - roi_w / 2, head[1] - h / 2, roi_w, h])
        rois.append(None if (no_face_every and t % no_face_every == no_face_every - 1) else np.stack([roi, roi]))
        c = [e[a, t, 0:2] + rng.normal(0, sigma_px, 2) for a in range(2)]
        nc = rng.poisson(clutter_rate)
        c += [rng.uniform([0, 0], [640, 480]) for _ in range(nc)]
        cands.append(np.array(c))
    return xs, e, rois, cands
