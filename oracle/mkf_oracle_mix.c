/*
 * mkf_oracle_mix.c -- FP64 CPU forward and reverse-mode adjoint of the
 * deterministic mixture Kalman filter with PDAF (declared in mkf_oracle.h).
 * TEST INFRASTRUCTURE ONLY: the parity reference of the GPU forward/adjoint kernels and
 * the CPU baseline of the gradient benchmark.  The adjoint stores every
 * frame's collapsed state (no checkpointing) and recomputes each frame's
 * intermediates, so it shares no structure with the GPU's sqrt(T) scheme.
 *
 * Reference pieces: KF_model::predict/update (KF_model.cpp:11-25), the motion
 * model of my_gmm::loadGaussian (my_gmm.cpp:45-75, F = diag(a), B = (1-a) mu,
 * Q = Lq Lq^T), the mixture of components redrawn per frame
 * (pf2DRao.cpp:128) and the PDA association weights (pfPose.cpp:247-298).
 */
#include "mkf_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MXD 24
#define MXJ 4
#define MXC 16
#define MXK 32
#define ZMIN 0.05

typedef struct {
  int vis, n;
  double x[MXD], P[MXD * MXD];            /* inputs of this joint update */
  double p[3], iz, zh[2], Jp[6];
  double H[2 * MXD], U[MXD * 2], S[4], Si[4], ld;
  double nu[MXC * 2], e[MXC], ell, beta[MXC], beta0, nb[2];
  double Kg[MXD * 2], M[4], W[MXD * 2];
} jrec;

typedef struct {
  double xm[MXD], Pm[MXD * MXD];          /* predicted */
  jrec jr[MXJ];
  double x[MXD], P[MXD * MXD], logl;      /* outputs */
} crec;

/* ---------------------------------------------------------------- forward pieces */
static double joint_fwd(const mko_mix_params* p, jrec* r, double* x, double* P, const double* Bj,
                        const double* mj, int n, const float* z, double pd, double kappa) {
  const int d = p->d;
  memcpy(r->x, x, sizeof(double) * d);
  memcpy(r->P, P, sizeof(double) * d * d);
  r->n = n;
  for (int t = 0; t < 3; ++t) {
    double s = mj[t];
    for (int c = 0; c < d; ++c) s += Bj[t * d + c] * x[c];
    r->p[t] = s;
  }
  if (!(r->p[2] > ZMIN)) { r->vis = 0; return log(kappa); }
  r->vis = 1;
  const double iz = 1.0 / r->p[2];
  r->iz = iz;
  r->zh[0] = p->fx * r->p[0] * iz + p->cx;
  r->zh[1] = p->fy * r->p[1] * iz + p->cy;
  double* Jp = r->Jp;
  Jp[0] = p->fx * iz; Jp[1] = 0.0; Jp[2] = -p->fx * r->p[0] * iz * iz;
  Jp[3] = 0.0; Jp[4] = p->fy * iz; Jp[5] = -p->fy * r->p[1] * iz * iz;
  for (int a = 0; a < 2; ++a)
    for (int c = 0; c < d; ++c)
      r->H[a * d + c] = Jp[a * 3] * Bj[c] + Jp[a * 3 + 1] * Bj[d + c] + Jp[a * 3 + 2] * Bj[2 * d + c];
  for (int rr = 0; rr < d; ++rr)
    for (int a = 0; a < 2; ++a) {
      double s = 0.0;
      for (int c = 0; c < d; ++c) s += P[rr * d + c] * r->H[a * d + c];
      r->U[rr * 2 + a] = s;
    }
  const double s2 = p->sigma * p->sigma;
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b) {
      double s = 0.0;
      for (int rr = 0; rr < d; ++rr) s += r->H[a * d + rr] * r->U[rr * 2 + b];
      r->S[a * 2 + b] = s + (a == b ? s2 : 0.0);
    }
  const double det = r->S[0] * r->S[3] - r->S[1] * r->S[2];
  r->Si[0] = r->S[3] / det; r->Si[1] = -r->S[1] / det; r->Si[2] = -r->S[2] / det; r->Si[3] = r->S[0] / det;
  r->ld = log(det);
  const double c0 = pd / (2.0 * M_PI), b = (1.0 - pd) * kappa;
  double ell = b;
  for (int i = 0; i < n; ++i) {
    double n0 = (double)z[2 * i] - r->zh[0], n1 = (double)z[2 * i + 1] - r->zh[1];
    r->nu[2 * i] = n0; r->nu[2 * i + 1] = n1;
    double q = n0 * (r->Si[0] * n0 + r->Si[1] * n1) + n1 * (r->Si[2] * n0 + r->Si[3] * n1);
    r->e[i] = c0 * exp(-0.5 * q - 0.5 * r->ld);
    ell += r->e[i];
  }
  r->ell = ell;
  r->beta0 = b / ell;
  r->nb[0] = r->nb[1] = 0.0;
  double C[4] = {0, 0, 0, 0};
  for (int i = 0; i < n; ++i) {
    r->beta[i] = r->e[i] / ell;
    r->nb[0] += r->beta[i] * r->nu[2 * i];
    r->nb[1] += r->beta[i] * r->nu[2 * i + 1];
    for (int a = 0; a < 2; ++a)
      for (int bb = 0; bb < 2; ++bb) C[a * 2 + bb] += r->beta[i] * r->nu[2 * i + a] * r->nu[2 * i + bb];
  }
  for (int a = 0; a < 2; ++a)
    for (int bb = 0; bb < 2; ++bb) C[a * 2 + bb] -= r->nb[a] * r->nb[bb];
  for (int q = 0; q < 4; ++q) r->M[q] = (1.0 - r->beta0) * r->S[q] - C[q];
  for (int rr = 0; rr < d; ++rr)
    for (int a = 0; a < 2; ++a)
      r->Kg[rr * 2 + a] = r->U[rr * 2] * r->Si[a] + r->U[rr * 2 + 1] * r->Si[2 + a];
  for (int rr = 0; rr < d; ++rr)
    for (int a = 0; a < 2; ++a)
      r->W[rr * 2 + a] = r->Kg[rr * 2] * r->M[a] + r->Kg[rr * 2 + 1] * r->M[2 + a];
  for (int rr = 0; rr < d; ++rr) x[rr] += r->Kg[rr * 2] * r->nb[0] + r->Kg[rr * 2 + 1] * r->nb[1];
  for (int rr = 0; rr < d; ++rr)
    for (int c = 0; c < d; ++c)
      P[rr * d + c] -= r->W[rr * 2] * r->Kg[c * 2] + r->W[rr * 2 + 1] * r->Kg[c * 2 + 1];
  return log(ell);
}

static void comp_fwd(const mko_mix_params* p, int k, const double* xh, const double* Ph, crec* cr,
                     const double* Bm, const double* mm, const int* off, const float* det, double pd,
                     double kappa) {
  const int d = p->d, DD = d * (d + 1) / 2;
  const double* a = p->a + k * d;
  const double* mu = p->mu + k * d;
  const double* L = p->Lq + k * DD;
  for (int r = 0; r < d; ++r) cr->xm[r] = a[r] * xh[r] + (1.0 - a[r]) * mu[r];
  for (int r = 0; r < d; ++r)
    for (int c = 0; c < d; ++c) {
      double q = 0.0;
      for (int s = 0; s <= (r < c ? r : c); ++s) q += L[r * (r + 1) / 2 + s] * L[c * (c + 1) / 2 + s];
      cr->Pm[r * d + c] = a[r] * a[c] * Ph[r * d + c] + q;
    }
  memcpy(cr->x, cr->xm, sizeof(double) * d);
  memcpy(cr->P, cr->Pm, sizeof(double) * d * d);
  double ll = 0.0;
  for (int j = 0; j < p->J; ++j) {
    int n = off[j + 1] - off[j];
    if (n > MXC) n = MXC;
    ll += joint_fwd(p, &cr->jr[j], cr->x, cr->P, Bm + j * 3 * d, mm + j * 3, n, det + 2 * (size_t)off[j], pd, kappa);
  }
  cr->logl = ll;
}

/* one frame: components, mixture, collapse.  Returns c_t; fills w (K). */
static double frame_fwd(const mko_mix_params* p, const double* xh, const double* Ph, crec* cr, double* w,
                        double* xo, double* Po, const double* Bm, const double* mm, const int* off,
                        const float* det, double pd, double kappa) {
  const int d = p->d, K = p->K;
  double l[MXK], mx = -INFINITY;
  for (int k = 0; k < K; ++k) {
    comp_fwd(p, k, xh, Ph, &cr[k], Bm, mm, off, det, pd, kappa);
    l[k] = log(p->pi[k]) + cr[k].logl;
    if (l[k] > mx) mx = l[k];
  }
  double s = 0.0;
  for (int k = 0; k < K; ++k) s += exp(l[k] - mx);
  const double c = mx + log(s);
  for (int k = 0; k < K; ++k) w[k] = exp(l[k] - c);
  for (int r = 0; r < d; ++r) {
    double v = 0.0;
    for (int k = 0; k < K; ++k) v += w[k] * cr[k].x[r];
    xo[r] = v;
  }
  double Pc[MXD * MXD];
  for (int r = 0; r < d; ++r)
    for (int cc = 0; cc < d; ++cc) {
      double v = 0.0;
      for (int k = 0; k < K; ++k)
        v += w[k] * (cr[k].P[r * d + cc] + (cr[k].x[r] - xo[r]) * (cr[k].x[cc] - xo[cc]));
      Pc[r * d + cc] = v;
    }
  for (int r = 0; r < d; ++r)
    for (int cc = 0; cc < d; ++cc) Po[r * d + cc] = 0.5 * (Pc[r * d + cc] + Pc[cc * d + r]);
  return c;
}

static void prior_state(const mko_mix_params* p, double* x, double* P) {
  const int d = p->d, K = p->K;
  for (int r = 0; r < d; ++r) {
    double v = 0.0;
    for (int k = 0; k < K; ++k) v += p->pi[k] * p->mu[k * d + r];
    x[r] = v;
  }
  for (int r = 0; r < d; ++r)
    for (int c = 0; c < d; ++c) {
      double v = 0.0;
      for (int k = 0; k < K; ++k)
        v += p->pi[k] * (p->S0[(size_t)k * d * d + r * d + c] + (p->mu[k * d + r] - x[r]) * (p->mu[k * d + c] - x[c]));
      P[r * d + c] = v;
    }
}

double mko_mix_forward(const mko_mix_params* p, int T, long long frame_base, const double* Bm,
                       const double* mm, double pd, double kappa, const int* det_off, const float* det) {
  const int d = p->d;
  crec* cr = (crec*)malloc(sizeof(crec) * p->K);
  double x[MXD], P[MXD * MXD], xo[MXD], Po[MXD * MXD], w[MXK];
  prior_state(p, x, P);
  double L = 0.0;
  for (int t = 0; t < T; ++t) {
    const int* off = det_off + (frame_base + t) * p->J;
    L += frame_fwd(p, x, P, cr, w, xo, Po, Bm, mm, off, det, pd, kappa);
    memcpy(x, xo, sizeof(double) * d);
    memcpy(P, Po, sizeof(double) * d * d);
  }
  free(cr);
  return L;
}

/* ---------------------------------------------------------------- reverse pieces */
static void joint_bwd(const mko_mix_params* p, const jrec* r, const double* Bj, double pd, double kappa,
                      double* xb, double* Pb, double gl, double* sb) {
  (void)pd;
  const int d = p->d;
  if (!r->vis) return;
  const int n = r->n;
  const double b = (1.0 - pd) * kappa;
  double Kgb[MXD * 2], Wb[MXD * 2], Ub[MXD * 2], Hb[2 * MXD];
  double nbb[2], Mb[4], Sb[4], Sib[4], Cnb[4], zhb[2] = {0, 0};
  double betab[MXC], nub[MXC * 2], eb[MXC];
  /* x' = x + Kg nb */
  for (int rr = 0; rr < d; ++rr)
    for (int a = 0; a < 2; ++a) Kgb[rr * 2 + a] = xb[rr] * r->nb[a];
  for (int a = 0; a < 2; ++a) {
    double s = 0.0;
    for (int rr = 0; rr < d; ++rr) s += r->Kg[rr * 2 + a] * xb[rr];
    nbb[a] = s;
  }
  /* P' = P - W Kg^T : Wb = -Pb' Kg ; Kgb += -Pb'^T W ; Pb (input) = Pb' (+ later) */
  for (int rr = 0; rr < d; ++rr)
    for (int a = 0; a < 2; ++a) {
      double s = 0.0, t = 0.0;
      for (int c = 0; c < d; ++c) {
        s += Pb[rr * d + c] * r->Kg[c * 2 + a];
        t += Pb[c * d + rr] * r->W[c * 2 + a];
      }
      Wb[rr * 2 + a] = -s;
      Kgb[rr * 2 + a] -= t;
    }
  /* W = Kg M */
  for (int rr = 0; rr < d; ++rr)
    for (int a = 0; a < 2; ++a) Kgb[rr * 2 + a] += Wb[rr * 2] * r->M[a * 2] + Wb[rr * 2 + 1] * r->M[a * 2 + 1];
  for (int a = 0; a < 2; ++a)
    for (int bb = 0; bb < 2; ++bb) {
      double s = 0.0;
      for (int rr = 0; rr < d; ++rr) s += r->Kg[rr * 2 + a] * Wb[rr * 2 + bb];
      Mb[a * 2 + bb] = s;
    }
  /* M = (1 - beta0) S - Cn */
  double b0b = 0.0;
  for (int q = 0; q < 4; ++q) {
    Sb[q] = (1.0 - r->beta0) * Mb[q];
    b0b -= Mb[q] * r->S[q];
    Cnb[q] = -Mb[q];
  }
  /* Cn = sum beta_i nu_i nu_i^T - nb nb^T */
  const double Cs[4] = {Cnb[0] + Cnb[0], Cnb[1] + Cnb[2], Cnb[2] + Cnb[1], Cnb[3] + Cnb[3]};
  for (int i = 0; i < n; ++i) {
    const double n0 = r->nu[2 * i], n1 = r->nu[2 * i + 1];
    betab[i] = n0 * (Cnb[0] * n0 + Cnb[1] * n1) + n1 * (Cnb[2] * n0 + Cnb[3] * n1);
    nub[2 * i] = r->beta[i] * (Cs[0] * n0 + Cs[1] * n1);
    nub[2 * i + 1] = r->beta[i] * (Cs[2] * n0 + Cs[3] * n1);
  }
  nbb[0] -= Cs[0] * r->nb[0] + Cs[1] * r->nb[1];
  nbb[1] -= Cs[2] * r->nb[0] + Cs[3] * r->nb[1];
  /* Kg = U Si */
  for (int rr = 0; rr < d; ++rr)
    for (int a = 0; a < 2; ++a) Ub[rr * 2 + a] = Kgb[rr * 2] * r->Si[a * 2] + Kgb[rr * 2 + 1] * r->Si[a * 2 + 1];
  for (int a = 0; a < 2; ++a)
    for (int bb = 0; bb < 2; ++bb) {
      double s = 0.0;
      for (int rr = 0; rr < d; ++rr) s += r->U[rr * 2 + a] * Kgb[rr * 2 + bb];
      Sib[a * 2 + bb] = s;
    }
  /* nb = sum beta_i nu_i */
  for (int i = 0; i < n; ++i) {
    betab[i] += r->nu[2 * i] * nbb[0] + r->nu[2 * i + 1] * nbb[1];
    nub[2 * i] += r->beta[i] * nbb[0];
    nub[2 * i + 1] += r->beta[i] * nbb[1];
  }
  /* beta_i = e_i / ell, beta0 = b / ell, log ell */
  double num = b0b * b;
  for (int i = 0; i < n; ++i) num += betab[i] * r->e[i];
  const double ellb = -num / (r->ell * r->ell) + gl / r->ell;
  double ldb = 0.0;
  for (int i = 0; i < n; ++i) {
    eb[i] = betab[i] / r->ell + ellb;
    const double qb = -0.5 * r->e[i] * eb[i];
    ldb += -0.5 * r->e[i] * eb[i];
    const double n0 = r->nu[2 * i], n1 = r->nu[2 * i + 1];
    /* q = nu^T Si nu */
    nub[2 * i] += qb * ((r->Si[0] + r->Si[0]) * n0 + (r->Si[1] + r->Si[2]) * n1);
    nub[2 * i + 1] += qb * ((r->Si[2] + r->Si[1]) * n0 + (r->Si[3] + r->Si[3]) * n1);
    Sib[0] += qb * n0 * n0; Sib[1] += qb * n0 * n1; Sib[2] += qb * n1 * n0; Sib[3] += qb * n1 * n1;
    zhb[0] -= nub[2 * i];
    zhb[1] -= nub[2 * i + 1];
  }
  /* ld = log det S ; Si = S^-1 */
  Sb[0] += ldb * r->Si[0]; Sb[1] += ldb * r->Si[2]; Sb[2] += ldb * r->Si[1]; Sb[3] += ldb * r->Si[3];
  {
    /* Sb += -Si^T Sib Si^T */
    double T1[4];
    for (int a = 0; a < 2; ++a)
      for (int bb = 0; bb < 2; ++bb) T1[a * 2 + bb] = r->Si[0 * 2 + a] * Sib[0 * 2 + bb] + r->Si[1 * 2 + a] * Sib[1 * 2 + bb];
    for (int a = 0; a < 2; ++a)
      for (int bb = 0; bb < 2; ++bb) Sb[a * 2 + bb] -= T1[a * 2 + 0] * r->Si[bb * 2 + 0] + T1[a * 2 + 1] * r->Si[bb * 2 + 1];
  }
  /* S = H U + sigma^2 I */
  *sb += 2.0 * p->sigma * (Sb[0] + Sb[3]);
  for (int a = 0; a < 2; ++a)
    for (int rr = 0; rr < d; ++rr) Hb[a * d + rr] = Sb[a * 2] * r->U[rr * 2] + Sb[a * 2 + 1] * r->U[rr * 2 + 1];
  for (int rr = 0; rr < d; ++rr)
    for (int bb = 0; bb < 2; ++bb) Ub[rr * 2 + bb] += r->H[rr] * Sb[bb] + r->H[d + rr] * Sb[2 + bb];
  /* U = P H^T : Pb += Ub H ; Hb += Ub^T P */
  for (int rr = 0; rr < d; ++rr)
    for (int c = 0; c < d; ++c) Pb[rr * d + c] += Ub[rr * 2] * r->H[c] + Ub[rr * 2 + 1] * r->H[d + c];
  for (int a = 0; a < 2; ++a)
    for (int c = 0; c < d; ++c) {
      double s = 0.0;
      for (int rr = 0; rr < d; ++rr) s += Ub[rr * 2 + a] * r->P[rr * d + c];
      Hb[a * d + c] += s;
    }
  /* H = Jp Bj */
  double Jb[6];
  for (int a = 0; a < 2; ++a)
    for (int t = 0; t < 3; ++t) {
      double s = 0.0;
      for (int c = 0; c < d; ++c) s += Hb[a * d + c] * Bj[t * d + c];
      Jb[a * 3 + t] = s;
    }
  /* zh = pi(p), Jp = dpi/dp */
  const double iz = r->iz, iz2 = iz * iz, iz3 = iz2 * iz;
  const double* Jp = r->Jp;
  double pb[3];
  pb[0] = Jp[0] * zhb[0] + Jp[3] * zhb[1] + Jb[2] * (-p->fx * iz2);
  pb[1] = Jp[1] * zhb[0] + Jp[4] * zhb[1] + Jb[5] * (-p->fy * iz2);
  pb[2] = Jp[2] * zhb[0] + Jp[5] * zhb[1] + Jb[0] * (-p->fx * iz2) + Jb[2] * (2.0 * p->fx * r->p[0] * iz3) +
          Jb[4] * (-p->fy * iz2) + Jb[5] * (2.0 * p->fy * r->p[1] * iz3);
  /* p = Bj x + mj */
  for (int c = 0; c < d; ++c) xb[c] += Bj[c] * pb[0] + Bj[d + c] * pb[1] + Bj[2 * d + c] * pb[2];
}

static void comp_bwd(const mko_mix_params* p, int k, const double* xh, const double* Ph, const crec* cr,
                     const double* Bm, double pd, double kappa, const double* xkb, const double* Pkb, double lb,
                     double* Xb, double* Pbo, double* g_mu, double* g_a, double* g_Lq, double* g_s) {
  const int d = p->d, DD = d * (d + 1) / 2;
  double xb[MXD], Pb[MXD * MXD];
  memcpy(xb, xkb, sizeof(double) * d);
  memcpy(Pb, Pkb, sizeof(double) * d * d);
  for (int j = p->J - 1; j >= 0; --j) joint_bwd(p, &cr->jr[j], Bm + j * 3 * d, pd, kappa, xb, Pb, lb, g_s);
  const double* a = p->a + k * d;
  const double* mu = p->mu + k * d;
  const double* L = p->Lq + k * DD;
  for (int r = 0; r < d; ++r) {
    Xb[r] += a[r] * xb[r];
    g_mu[k * d + r] += (1.0 - a[r]) * xb[r];
    g_a[k * d + r] += (xh[r] - mu[r]) * xb[r];
  }
  for (int r = 0; r < d; ++r)
    for (int c = 0; c < d; ++c) {
      Pbo[r * d + c] += a[r] * a[c] * Pb[r * d + c];
      g_a[k * d + r] += Pb[r * d + c] * a[c] * Ph[r * d + c];
      g_a[k * d + c] += Pb[r * d + c] * a[r] * Ph[r * d + c];
    }
  for (int r = 0; r < d; ++r)
    for (int c = 0; c <= r; ++c) {
      double s = 0.0;
      for (int t = c; t < d; ++t) s += (Pb[r * d + t] + Pb[t * d + r]) * L[t * (t + 1) / 2 + c];
      g_Lq[k * DD + r * (r + 1) / 2 + c] += s;
    }
}

double mko_mix_adjoint(const mko_mix_params* p, int T, long long frame_base, const double* Bm,
                       const double* mm, double pd, double kappa, const int* det_off, const float* det,
                       double* g_mu, double* g_a, double* g_Lq, double* g_sigma) {
  const int d = p->d, K = p->K, dd = d * d;
  double* xs = (double*)malloc(sizeof(double) * (size_t)(T + 1) * d);
  double* Ps = (double*)malloc(sizeof(double) * (size_t)(T + 1) * dd);
  crec* cr = (crec*)malloc(sizeof(crec) * K);
  double w[MXK];
  prior_state(p, xs, Ps);
  double L = 0.0;
  for (int t = 0; t < T; ++t) {
    const int* off = det_off + (frame_base + t) * p->J;
    L += frame_fwd(p, xs + (size_t)t * d, Ps + (size_t)t * dd, cr, w, xs + (size_t)(t + 1) * d,
                   Ps + (size_t)(t + 1) * dd, Bm, mm, off, det, pd, kappa);
  }
  double Xb[MXD], Pb[MXD * MXD], xo[MXD], Po[MXD * MXD];
  memset(Xb, 0, sizeof(Xb));
  memset(Pb, 0, sizeof(Pb));
  for (int t = T - 1; t >= 0; --t) {
    const int* off = det_off + (frame_base + t) * p->J;
    const double* xh = xs + (size_t)t * d;
    const double* Ph = Ps + (size_t)t * dd;
    frame_fwd(p, xh, Ph, cr, w, xo, Po, Bm, mm, off, det, pd, kappa);
    /* collapse reverse (symmetrisation, moment match, softmax with dc = 1) */
    double Pcb[MXD * MXD], xt[MXD], wb[MXK];
    for (int r = 0; r < d; ++r)
      for (int c = 0; c < d; ++c) Pcb[r * d + c] = 0.5 * (Pb[r * d + c] + Pb[c * d + r]);
    double Dk[MXK][MXD];
    double Dkb[MXK][MXD];
    for (int r = 0; r < d; ++r) xt[r] = Xb[r];
    for (int k = 0; k < K; ++k) {
      for (int r = 0; r < d; ++r) Dk[k][r] = cr[k].x[r] - xo[r];
      for (int r = 0; r < d; ++r) {
        double s = 0.0;
        for (int c = 0; c < d; ++c) s += (Pcb[r * d + c] + Pcb[c * d + r]) * Dk[k][c];
        Dkb[k][r] = w[k] * s;
        xt[r] -= Dkb[k][r];
      }
    }
    double sw = 0.0;
    for (int k = 0; k < K; ++k) {
      double v = 0.0;
      for (int r = 0; r < d; ++r) v += cr[k].x[r] * xt[r];
      for (int r = 0; r < d; ++r)
        for (int c = 0; c < d; ++c) v += Pcb[r * d + c] * (cr[k].P[r * d + c] + Dk[k][r] * Dk[k][c]);
      wb[k] = v;
      sw += w[k] * v;
    }
    double Xn[MXD], Pn[MXD * MXD];
    memset(Xn, 0, sizeof(Xn));
    memset(Pn, 0, sizeof(Pn));
    for (int k = 0; k < K; ++k) {
      if (!(w[k] > 0.0)) continue;
      double xkb[MXD], Pkb[MXD * MXD];
      for (int r = 0; r < d; ++r) xkb[r] = Dkb[k][r] + w[k] * xt[r];
      for (int q = 0; q < dd; ++q) Pkb[q] = w[k] * Pcb[q];
      const double lb = w[k] * (wb[k] - sw) + w[k];
      comp_bwd(p, k, xh, Ph, &cr[k], Bm, pd, kappa, xkb, Pkb, lb, Xn, Pn, g_mu, g_a, g_Lq, g_sigma);
    }
    memcpy(Xb, Xn, sizeof(double) * d);
    memcpy(Pb, Pn, sizeof(double) * dd);
  }
  /* prior: x = sum pi mu, P = sum pi (S0 + D D^T) */
  {
    double x0[MXD];
    for (int r = 0; r < d; ++r) x0[r] = xs[r];
    double xt[MXD], Dkb[MXK][MXD];
    for (int r = 0; r < d; ++r) xt[r] = Xb[r];
    for (int k = 0; k < K; ++k)
      for (int r = 0; r < d; ++r) {
        double s = 0.0;
        for (int c = 0; c < d; ++c) s += (Pb[r * d + c] + Pb[c * d + r]) * (p->mu[k * d + c] - x0[c]);
        Dkb[k][r] = p->pi[k] * s;
        xt[r] -= Dkb[k][r];
      }
    for (int k = 0; k < K; ++k)
      for (int r = 0; r < d; ++r) g_mu[k * d + r] += Dkb[k][r] + p->pi[k] * xt[r];
  }
  free(xs); free(Ps); free(cr);
  return L;
}

double mko_mix_batch(const mko_mix_params* p, int n_tracks, const int* n_frames, const long long* frame_base,
                     const double* Bm, const double* mm, const double* pd, const double* kappa,
                     const int* det_off, const float* det, int grad, double* ll, double* g_mu,
                     double* g_a, double* g_Lq, double* g_sigma, int nthreads) {
  const int d = p->d, K = p->K, J = p->J, DD = d * (d + 1) / 2;
  const int ng = K * d * 2 + K * DD + 1;
  double* G = grad ? (double*)calloc((size_t)n_tracks * ng, sizeof(double)) : NULL;
  double* L = (double*)malloc(sizeof(double) * (size_t)n_tracks);
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
  for (int b = 0; b < n_tracks; ++b) {
    const double* B = Bm + (size_t)b * J * 3 * d;
    const double* m = mm + (size_t)b * J * 3;
    if (grad) {
      double* g = G + (size_t)b * ng;
      L[b] = mko_mix_adjoint(p, n_frames[b], frame_base[b], B, m, pd[b], kappa[b], det_off, det, g, g + K * d,
                             g + 2 * K * d, g + 2 * K * d + K * DD);
    } else {
      L[b] = mko_mix_forward(p, n_frames[b], frame_base[b], B, m, pd[b], kappa[b], det_off, det);
    }
  }
  double tot = 0.0;
  for (int b = 0; b < n_tracks; ++b) {   /* fixed-order reduction */
    tot += L[b];
    if (ll) ll[b] = L[b];
  }
  if (grad) {
    for (int q = 0; q < ng; ++q) {
      double s = 0.0;
      for (int b = 0; b < n_tracks; ++b) s += G[(size_t)b * ng + q];
      if (q < K * d) g_mu[q] += s;
      else if (q < 2 * K * d) g_a[q - K * d] += s;
      else if (q < 2 * K * d + K * DD) g_Lq[q - 2 * K * d] += s;
      else *g_sigma += s;
    }
    free(G);
  }
  free(L);
  return tot;
}
