"""Make tests/golden/refpin.npz: outputs of the reference's OWN filter code
(KF_model.cpp, my_gmm.cpp, pf2DRao.cpp from the reference checkout, compiled
unmodified against the stand-in OpenCV/ROS headers of oracle/refpin by
oracle/refpin/Makefile into oracle/_ref/refpin) on seeded inputs, to pin the
oracle's restatement (tests/test_refpin.py).  Run where the reference is
mounted:

    python tests/golden/make_refpin_golden.py <reference checkout>

Cases (all FP64):
  kf      KF_model::predict + ::update on random d=12, m=6 systems
  loadg   my_gmm::loadGaussian on both shipped models (15 components each)
  wheel   ParticleFilter::resample on random, sparse, unnormalised (wrapping)
          and all-zero weights with injected draws
  mvn     ParticleFilter::chol + ::mvnpdf on random 6x6 innovation covariances
          and diagonal ones, under both diagonal conventions of the Cholesky call
  rbpf    resetTracker then 4 ParticleFilter::update calls (N=48) on the left-arm
          model, with injected uniforms, under both conventions: tracks and
          getEstimator after every update, and whether the all-zero branch ran
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from mkfbodytracker_pdaf_gb300 import cvyaml  # noqa: E402


def fmt(a):
    return " ".join("%.17g" % v for v in np.ravel(np.asarray(a, np.float64)))


def spd(rng, n, scale=1.0):
    A = rng.standard_normal((n, n))
    return scale * (A @ A.T / n + 0.5 * np.eye(n))


def parse(out):
    """Output lines 'tag r c v...' (and 'idx n v...', 'p v', 'frame t fallback') -> list of (tag, value)."""
    recs = []
    for line in out.strip().splitlines():
        t = line.split()
        if t[0] == "frame":
            recs.append(("frame", (int(t[1]), int(t[2]))))
        elif t[0] == "p":
            recs.append(("p", float(t[1])))
        elif t[0] == "idx":
            recs.append(("idx", np.array([int(v) for v in t[2:]], np.int32)))
        else:
            r, c = int(t[1]), int(t[2])
            recs.append((t[0], np.array([float(v) for v in t[3:]]).reshape(r, c)))
    return recs


def run(exe, text):
    r = subprocess.run([exe], input=text, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError("refpin failed (%d): %s" % (r.returncode, r.stderr[-400:]))
    return parse(r.stdout)


def model_inputs(path):
    m = cvyaml.load(path)
    K, d = m["means"].shape
    return dict(mu=m["means"].astype(np.float64), covs=m["covs"].astype(np.float64).reshape(K, d, d),
                w=m["weights"].astype(np.float64).ravel(), g=m["gamma"].astype(np.float64).ravel(),
                Hpca=m["pca_proj"].astype(np.float64), mpca=m["pca_mean"].astype(np.float64).ravel())


def components_text(M):
    K, d = M["mu"].shape
    parts = []
    for k in range(K):
        parts.append("%s %s %.17g %.17g" % (fmt(M["mu"][k]), fmt(M["covs"][k]), M["w"][k], M["g"][k]))
    parts.append(fmt(M["Hpca"]))
    parts.append(fmt(M["mpca"]))
    return " ".join(parts)


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_refpin_golden.py <reference checkout>")
    ref = sys.argv[1]
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "refpin"), "REF=" + ref], check=True)
    exe = os.path.join(ROOT, "oracle", "_ref", "refpin")
    rng = np.random.default_rng(20140601)
    out = {}

    # ---- KF_model
    d, m, n = 12, 6, 20
    F = np.stack([np.diag(rng.uniform(0.8, 1.0, d)) + 0.01 * rng.standard_normal((d, d)) for _ in range(n)])
    B = rng.standard_normal((n, d))
    Q = np.stack([spd(rng, d, 0.05) for _ in range(n)])
    H = rng.standard_normal((n, m, d))
    BH = rng.standard_normal((n, m))
    R = np.stack([spd(rng, m, 2.0) for _ in range(n)])
    x = rng.standard_normal((n, d))
    P = np.stack([spd(rng, d) for _ in range(n)])
    z = rng.standard_normal((n, m)) * 3
    text = "".join("KF %d %d %s %s %s %s %s %s %s %s %s\n" % (d, m, fmt(F[i]), fmt(B[i]), fmt(Q[i]), fmt(H[i]),
                                                              fmt(BH[i]), fmt(R[i]), fmt(x[i]), fmt(P[i]), fmt(z[i]))
                   for i in range(n))
    vals = [v for _, v in run(exe, text)]
    out.update(kf_F=F, kf_B=B, kf_Q=Q, kf_H=H, kf_BH=BH, kf_R=R, kf_x=x, kf_P=P, kf_z=z,
               kf_xp=np.stack([vals[4 * i].ravel() for i in range(n)]), kf_Pp=np.stack([vals[4 * i + 1] for i in range(n)]),
               kf_xu=np.stack([vals[4 * i + 2].ravel() for i in range(n)]),
               kf_Pu=np.stack([vals[4 * i + 3] for i in range(n)]))

    # ---- loadGaussian on the shipped models
    for a, fn in enumerate(("data13D_PCA_100000_15_12.yml", "data23D_PCA_100000_15_12.yml")):
        M = model_inputs(os.path.join(ref, fn))
        K, d = M["mu"].shape
        vals = [v for _, v in run(exe, "LOADG %d %d %d %s\n" % (K, d, M["Hpca"].shape[1], components_text(M)))]
        for key in ("mu", "covs", "w", "g", "Hpca", "mpca"):
            out["loadg%d_%s" % (a, key)] = M[key]
        for j, key in enumerate(("F", "B", "Q", "H", "BH", "R")):
            out["loadg%d_out_%s" % (a, key)] = np.stack([vals[6 * k + j] for k in range(K)])

    # ---- the resampling wheel
    cases = []
    for L, N, kind in [(15, 10, "rand"), (15, 500, "rand"), (100, 100, "rand"), (1000, 500, "sparse"),
                       (1000, 1000, "rand"), (64, 64, "unnorm"), (7, 200, "unnorm"), (30, 30, "zeros"),
                       (5, 40, "ties"), (500, 2000, "pow")]:
        w = rng.random(L)
        if kind == "sparse":
            w[rng.random(L) < 0.9] = 0.0
        if kind == "pow":
            w = w ** 8
        if kind == "ties":
            w = np.full(L, 1.0 / L)
        if kind == "zeros":
            w = np.zeros(L)
        if kind != "unnorm" and w.sum() > 0:
            w = w / w.sum()
        if kind == "unnorm":
            w = w / w.sum() * 0.9          # short of 1: the wheel wraps (% L)
        u = float(rng.random())
        i0 = int(rng.integers(0, L))
        fb = rng.integers(0, L, N)
        cases.append((w, N, u, i0, fb))
    text = "".join("RESAMPLE %d %d %s %.17g %d %s\n" % (len(w), N, fmt(w), u, i0, " ".join(str(int(v)) for v in fb))
                   for w, N, u, i0, fb in cases)
    for c, ((w, N, u, i0, fb), (_, idx)) in enumerate(zip(cases, run(exe, text))):
        out["wheel%d_w" % c] = w
        out["wheel%d_u" % c] = np.array([u])
        out["wheel%d_fb" % c] = fb.astype(np.int32)
        out["wheel%d_idx" % c] = idx

    # ---- chol + mvnpdf, both conventions
    m, n = 6, 12
    Ss = [spd(rng, m, 50.0) for _ in range(n // 2)] + [np.diag(rng.uniform(10, 200, m)) for _ in range(n // 2)]
    xs = rng.standard_normal((n, m)) * 5
    us = rng.standard_normal((n, m)) * 5
    for conv in (24, 3):
        text = "CONV %d\n" % conv + "".join("MVN %d %s %s %s\n" % (m, fmt(xs[i]), fmt(us[i]), fmt(Ss[i])) for i in range(n))
        recs = run(exe, text)
        out["mvn%d_p" % conv] = np.array([v for t, v in recs if t == "p"])
        out["mvn%d_chol" % conv] = np.stack([v for t, v in recs if t == "chol"])
    out.update(mvn_x=xs, mvn_u=us, mvn_S=np.stack(Ss))

    # ---- resetTracker + update sequence on the left-arm model
    M = model_inputs(os.path.join(ref, "data13D_PCA_100000_15_12.yml"))
    K, d = M["mu"].shape
    N, T = 48, 4
    bins = rng.integers(0, K, N)
    # measurement column j near the model's prediction for particle j's
    # starting component (the head, hand, neck rows of H1 (H_pca^T mu + m)),
    # with noise, so that the OpenCV-2.4 convention's weights do not all underflow
    sel = [9, 10, 0, 1, 12, 13]
    full = M["Hpca"].T @ M["mu"][bins].T + M["mpca"][:, None]          # (Fd, N)
    zs = [full[sel] + rng.normal(0, 6.0, (6, N)) for _ in range(T)]
    uis = rng.random(T)
    uas = rng.random(T)
    fbs = rng.integers(0, N, (T, N))
    for conv in (24, 3):
        text = "CONV %d\nRBPF %d %d %d %d %d %s %s " % (conv, K, d, M["Hpca"].shape[1], N, T, components_text(M),
                                                        " ".join(str(int(b)) for b in bins))
        text += " ".join("%s %.17g %.17g %s" % (fmt(zs[t]), uis[t], uas[t], " ".join(str(int(v)) for v in fbs[t]))
                         for t in range(T)) + "\n"
        xs_, Ps_, est, fell = [], [], [], []
        frame = -1
        for tag, v in run(exe, text):
            if tag == "frame":
                frame = v[0]
                fell.append(v[1])
                xs_.append([])
                Ps_.append([])
            elif tag == "x":
                xs_[frame].append(v.ravel())
            elif tag == "P":
                Ps_[frame].append(v)
            elif tag == "est":
                est.append(v.ravel())
        out["rbpf%d_x" % conv] = np.array(xs_)
        out["rbpf%d_P" % conv] = np.array(Ps_)
        out["rbpf%d_est" % conv] = np.array(est)
        out["rbpf%d_fallback" % conv] = np.array(fell, np.int32)
    out.update(rbpf_bins=bins.astype(np.int32), rbpf_z=np.stack(zs), rbpf_u_ind=uis, rbpf_u_anc=uas,
               rbpf_fb=fbs.astype(np.int32))
    np.savez_compressed(os.path.join(HERE, "refpin.npz"), **out)
    print("wrote", os.path.join(HERE, "refpin.npz"), len(out), "arrays")


if __name__ == "__main__":
    main()
