/*
 * mkf_oracle.c -- FP64 CPU restatement of the mkfbodytracker_pdaf filtering
 * hot path.  TEST INFRASTRUCTURE ONLY (the parity reference of the tests and the timed CPU baseline);
 * the CUDA product never links or calls it.  mkf_oracle.h says how it is
 * pinned to the reference's own code.
 *
 * Compiled with -ffp-contract=off so that the integer/FP steps that must be
 * bit-identical with the GPU (quantisation, component pick) are not fused.
 */
#include "mkf_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef unsigned __int128 u128;

/* ------------------------------------------------------------------------ */
/* K1: Philox4x32-10, restated from Salmon, Moraes, Dror, Shaw, "Parallel     */
/* random numbers: as easy as 1, 2, 3" (SC'11).  Replaces cv::RNG(getTick    */
/* Count()) at pf2DRao.cpp:179, randn at pf2DRao.cpp:96, rand() in pf2D.cpp.  */
/* ------------------------------------------------------------------------ */
#define PHILOX_M0 0xD2511F53u
#define PHILOX_M1 0xCD9E8D57u
#define PHILOX_W0 0x9E3779B9u
#define PHILOX_W1 0xBB67AE85u

void mko_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    if (r) { k0 += PHILOX_W0; k1 += PHILOX_W1; }
    uint64_t p0 = (uint64_t)PHILOX_M0 * c0;
    uint64_t p1 = (uint64_t)PHILOX_M1 * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

void mko_draw_block(uint64_t seed, uint32_t track, uint32_t frame, uint32_t item,
                    uint32_t stream, uint32_t out[4]) {
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32) ^ track};
  uint32_t ctr[4] = {frame, item, stream, 0u};
  mko_philox4x32_10(ctr, key, out);
}

float mko_u01_f32(uint32_t w) { return (float)(w >> 8) * (1.0f / 16777216.0f); }

/* Draw layout for one particle-frame: ceil(d/4) Philox blocks at streams
 * 0,1,..; words 2p,2p+1 feed Box-Muller pair p with 23-bit uniforms from the
 * top bits, u1 = 1 - (w >> 9) 2^-23 in (0,1] and u2 = (w >> 9) 2^-23 in [0,1);
 * the component uniform is the 24-bit value of the low bytes of words 0..2,
 * shifted right by one, times 2^-23. */
void mko_particle_draws(uint64_t seed, uint32_t track, uint32_t frame, uint32_t item,
                        int d, double* eps, float* ucomp) {
  uint32_t W[32];
  int nblk = (d + 3) / 4;
  for (int b = 0; b < nblk; ++b) mko_draw_block(seed, track, frame, item, (uint32_t)b, W + 4 * b);
  for (int p = 0; p < d / 2; ++p) {
    double u1 = 1.0 - (double)(W[2 * p] >> 9) * (1.0 / 8388608.0);
    double u2 = (double)(W[2 * p + 1] >> 9) * (1.0 / 8388608.0);
    double r = sqrt(-2.0 * log(u1));
    double th = M_PI * (2.0 * u2 - 1.0);
    eps[2 * p] = r * cos(th);
    eps[2 * p + 1] = r * sin(th);
  }
  if (ucomp) {
    uint32_t c = (W[0] & 0xFFu) | ((W[1] & 0xFFu) << 8) | ((W[2] & 0xFFu) << 16);
    *ucomp = (float)(c >> 1) * (1.0f / 8388608.0f);
  }
}

/* ------------------------------------------------------------------------ */
/* A6: resampling                                                             */
/* ------------------------------------------------------------------------ */
/* Literal restatement of ParticleFilter::resample (pf2DRao.cpp:175-210) and
 * maxWeight (pf2DRao.cpp:161-172): sequential wheel with strict '>' and the
 * '% L' wrap; beta = u * (1/N). */
void mko_resample_wheel(const double* w, int L, int N, double u, const int* fallback, int* idx) {
  double mw = 0.0;
  for (int i = 0; i < L; ++i) if (w[i] > mw) mw = w[i];
  if (mw == 0.0) {
    for (int i = 0; i < N; ++i) idx[i] = fallback ? fallback[i] : 0;
    return;
  }
  int j = 0;
  double step = 1.0 / (double)N;
  double beta = u * step;
  for (int i = 0; i < N; ++i) {
    while (beta > w[j]) {
      beta -= w[j];
      j = (j + 1) % L;
    }
    beta += step;
    idx[i] = j;
  }
}

#define MKO_QBITS 40

int mko_quantize_f64(const double* w, int L, uint64_t* q) {
  double mx = 0.0;
  for (int j = 0; j < L; ++j) {
    double v = w[j];
    if (isinf(v) && v > 0) return 0;
    if (!(v > 0.0)) continue;            /* NaN, zero, negative -> 0 */
    if (v > mx) mx = v;
  }
  if (mx == 0.0) return 0;
  int e;
  frexp(mx, &e);                          /* mx = f 2^e, f in [0.5,1) */
  for (int j = 0; j < L; ++j) {
    double v = w[j];
    q[j] = (v > 0.0) ? (uint64_t)ldexp(v, MKO_QBITS - e) : 0u;
  }
  return 1;
}

int mko_quantize_f32(const float* w, int L, uint64_t* q) {
  float mx = 0.0f;
  for (int j = 0; j < L; ++j) {
    float v = w[j];
    if (isinf(v) && v > 0) return 0;
    if (!(v > 0.0f)) continue;
    if (v > mx) mx = v;
  }
  if (mx == 0.0f) return 0;
  int e;
  frexpf(mx, &e);
  for (int j = 0; j < L; ++j) {
    float v = w[j];
    q[j] = (v > 0.0f) ? (uint64_t)ldexpf(v, MKO_QBITS - e) : 0u;
  }
  return 1;
}

void mko_resample_exact(const uint64_t* q, int L, int N, uint32_t U, int* idx) {
  uint64_t* Q = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)L);
  uint64_t acc = 0;
  for (int j = 0; j < L; ++j) { acc += q[j]; Q[j] = acc; }
  uint64_t Qt = Q[L - 1];
  int j = 0;
  for (int i = 0; i < N; ++i) {
    u128 rhs = (u128)((((uint64_t)(uint32_t)i) << 32) | (uint64_t)U) * (u128)Qt;
    while (j < L - 1 && (((u128)(uint64_t)N * (u128)Q[j]) << 32) < rhs) ++j;
    idx[i] = j;
  }
  free(Q);
}

static void resample_fallback(int L, int N, uint32_t U, int* idx) {
  uint32_t key[2] = {U, 0x5EEDu};
  for (int i = 0; i < N; ++i) {
    uint32_t ctr[4] = {(uint32_t)i, 0u, 0u, 0u}, o[4];
    mko_philox4x32_10(ctr, key, o);
    idx[i] = (int)(((uint64_t)o[0] * (uint64_t)L) >> 32);
  }
}

int mko_resample_f64(const double* w, int L, int N, uint32_t U, int* idx) {
  uint64_t* q = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)L);
  int ok = mko_quantize_f64(w, L, q);
  if (ok) mko_resample_exact(q, L, N, U, idx);
  else resample_fallback(L, N, U, idx);
  free(q);
  return !ok;
}

int mko_resample_f32(const float* w, int L, int N, uint32_t U, int* idx) {
  uint64_t* q = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)L);
  int ok = mko_quantize_f32(w, L, q);
  if (ok) mko_resample_exact(q, L, N, U, idx);
  else resample_fallback(L, N, U, idx);
  free(q);
  return !ok;
}

/* ------------------------------------------------------------------------ */
/* small dense linear algebra                                                 */
/* ------------------------------------------------------------------------ */
/* Gauss-Jordan inverse with partial pivoting (cv::Mat::inv, DECOMP_LU). */
static int inv_lu(int n, const double* A, double* Ai) {
  double M[64 * 128];
  int w2 = 2 * n;
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < w2; ++c) M[r * w2 + c] = c < n ? A[r * n + c] : (c - n == r ? 1.0 : 0.0);
  for (int c = 0; c < n; ++c) {
    int piv = c;
    double best = fabs(M[c * w2 + c]);
    for (int r = c + 1; r < n; ++r)
      if (fabs(M[r * w2 + c]) > best) { best = fabs(M[r * w2 + c]); piv = r; }
    if (best == 0.0 || !isfinite(best)) return 0;
    if (piv != c)
      for (int k = 0; k < w2; ++k) { double t = M[c * w2 + k]; M[c * w2 + k] = M[piv * w2 + k]; M[piv * w2 + k] = t; }
    double inv = 1.0 / M[c * w2 + c];
    for (int k = 0; k < w2; ++k) M[c * w2 + k] *= inv;
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      double f = M[r * w2 + c];
      if (f == 0.0) continue;
      for (int k = 0; k < w2; ++k) M[r * w2 + k] -= f * M[c * w2 + k];
    }
  }
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) Ai[r * n + c] = M[r * w2 + n + c];
  return 1;
}

/* Lower Cholesky S = L L^T; returns 0 if a pivot is <= 0 (exact mode) */
static int chol_lower(int n, const double* S, double* Lo) {
  memset(Lo, 0, sizeof(double) * (size_t)n * n);
  for (int i = 0; i < n; ++i) {
    for (int j = 0; j <= i; ++j) {
      double s = S[i * n + j];
      for (int k = 0; k < j; ++k) s -= Lo[i * n + k] * Lo[j * n + k];
      if (i == j) {
        if (!(s > 0.0)) return 0;
        Lo[i * n + i] = sqrt(s);
      } else {
        Lo[i * n + j] = s / Lo[j * n + j];
      }
    }
  }
  return 1;
}

/* ------------------------------------------------------------------------ */
/* A4/A5: KF_model::predict / update (KF_model.cpp:11-25)                    */
/* ------------------------------------------------------------------------ */
void mko_kf_predict(int d, const double* F, const double* B, const double* Q, double* x, double* P) {
  double xn[64], T[64 * 64];
  for (int r = 0; r < d; ++r) {                 /* state = F*state + B */
    double s = 0.0;
    for (int c = 0; c < d; ++c) s += F[r * d + c] * x[c];
    xn[r] = s + B[r];
  }
  for (int r = 0; r < d; ++r)                   /* cov = F*cov*F.t() + Q */
    for (int c = 0; c < d; ++c) {
      double s = 0.0;
      for (int k = 0; k < d; ++k) s += F[r * d + k] * P[k * d + c];
      T[r * d + c] = s;
    }
  for (int r = 0; r < d; ++r)
    for (int c = 0; c < d; ++c) {
      double s = 0.0;
      for (int k = 0; k < d; ++k) s += T[r * d + k] * F[c * d + k];
      P[r * d + c] = s + Q[r * d + c];
    }
  memcpy(x, xn, sizeof(double) * (size_t)d);
}

/* generic update with predicted measurement zhat and Jacobian Hx (m x d) */
static int kf_update_generic(int d, int m, const double* Hx, const double* zhat, const double* R,
                             const double* z, unsigned mask, double* x, double* P) {
  int rows[16], mm = 0;
  for (int r = 0; r < m; ++r) if (mask & (1u << r)) rows[mm++] = r;
  if (mm == 0) return 1;
  double H[16 * 64], y[16], S[256], Si[256], PHt[64 * 16], K[64 * 16], T[64 * 64];
  for (int a = 0; a < mm; ++a) {
    y[a] = z[rows[a]] - zhat[rows[a]];          /* y = z - (H x + BH) */
    for (int c = 0; c < d; ++c) H[a * d + c] = Hx[rows[a] * d + c];
  }
  for (int r = 0; r < d; ++r)
    for (int a = 0; a < mm; ++a) {
      double s = 0.0;
      for (int k = 0; k < d; ++k) s += P[r * d + k] * H[a * d + k];
      PHt[r * mm + a] = s;
    }
  for (int a = 0; a < mm; ++a)                  /* S = H P H^T + R */
    for (int b = 0; b < mm; ++b) {
      double s = 0.0;
      for (int k = 0; k < d; ++k) s += H[a * d + k] * PHt[k * mm + b];
      S[a * mm + b] = s + R[rows[a] * m + rows[b]];
    }
  if (!inv_lu(mm, S, Si)) return 0;             /* S.inv() */
  for (int r = 0; r < d; ++r)                   /* K = P H^T S^-1 */
    for (int b = 0; b < mm; ++b) {
      double s = 0.0;
      for (int a = 0; a < mm; ++a) s += PHt[r * mm + a] * Si[a * mm + b];
      K[r * mm + b] = s;
    }
  for (int r = 0; r < d; ++r) {                 /* state = state + K y */
    double s = 0.0;
    for (int a = 0; a < mm; ++a) s += K[r * mm + a] * y[a];
    x[r] += s;
  }
  for (int r = 0; r < d; ++r)                   /* cov = (I - K H) cov */
    for (int c = 0; c < d; ++c) {
      double s = (r == c) ? 1.0 : 0.0;
      for (int a = 0; a < mm; ++a) s -= K[r * mm + a] * H[a * d + c];
      T[r * d + c] = s;
    }
  double Pn[64 * 64];
  for (int r = 0; r < d; ++r)
    for (int c = 0; c < d; ++c) {
      double s = 0.0;
      for (int k = 0; k < d; ++k) s += T[r * d + k] * P[k * d + c];
      Pn[r * d + c] = s;
    }
  memcpy(P, Pn, sizeof(double) * (size_t)d * d);
  return 1;
}

int mko_kf_update(int d, int m, const double* H, const double* BH, const double* R,
                  const double* z, unsigned mask, double* x, double* P) {
  double zhat[16];
  for (int a = 0; a < m; ++a) {
    double s = 0.0;
    for (int c = 0; c < d; ++c) s += H[a * d + c] * x[c];
    zhat[a] = s + BH[a];
  }
  return kf_update_generic(d, m, H, zhat, R, z, mask, x, P);
}

/* ------------------------------------------------------------------------ */
/* A7: chol + mvnpdf (pf2DRao.cpp:34-67)                                      */
/* ------------------------------------------------------------------------ */
double mko_mvn_logpdf(int m, const double* x, const double* u, const double* S, int mode) {
  double Lo[256], v[16];
  const double l2pi = log(2.0 * M_PI);
  if (mode == 0) {
    if (!chol_lower(m, S, Lo)) return -INFINITY;
    double half_logdet = 0.0, q = 0.0;
    for (int i = 0; i < m; ++i) {
      double s = x[i] - u[i];
      for (int k = 0; k < i; ++k) s -= Lo[i * m + k] * v[k];
      v[i] = s / Lo[i * m + i];
      q += v[i] * v[i];
      half_logdet += log(Lo[i * m + i]);
    }
    return -0.5 * q - half_logdet - 0.5 * (double)m * l2pi;
  }
  /* quirk modes: build the reference's "R" from OpenCV's in-place factor.
   * cv::Cholesky fails when a pivot is below DBL_EPSILON; chol() then returns
   * the unfactored clone. */
  double Rm[256], Ri[256];
  int ok = chol_lower(m, S, Lo);
  if (ok) {
    for (int i = 0; i < m; ++i)
      if (Lo[i * m + i] * Lo[i * m + i] < DBL_EPSILON) ok = 0;
  }
  if (!ok) {
    memcpy(Rm, S, sizeof(double) * (size_t)m * m);  /* chol() returns the clone */
  } else {
    for (int e = 0; e < m; ++e) {
      double elem = (mode == 1) ? 1.0 / Lo[e * m + e] : Lo[e * m + e];
      for (int c = 0; c < m; ++c) {
        if (c < e) Rm[e * m + c] = 0.0;
        else if (c == e) Rm[e * m + c] = 1.0 / elem;
        else Rm[e * m + c] = S[e * m + c] * elem;
      }
    }
  }
  if (!inv_lu(m, Rm, Ri)) return NAN;
  double q = 0.0, lsd = 0.0;
  for (int c = 0; c < m; ++c) {                 /* x_u = (x-u)^T R^-1 */
    double s = 0.0;
    for (int r = 0; r < m; ++r) s += (x[r] - u[r]) * Ri[r * m + c];
    q += s * s;
    lsd += log(Rm[c * m + c]);
  }
  return -0.5 * q - lsd - 0.5 * (double)m * l2pi;
}

/* ------------------------------------------------------------------------ */
/* A1: my_gmm::loadGaussian (my_gmm.cpp:45-75)                                */
/* ------------------------------------------------------------------------ */
void mko_load_gaussian_ref(int d, int Fdim, const double* u, const double* s,
                           const double* Hpca, const double* mpca, double g,
                           double* F, double* B, double* Q, double* H, double* BH, double* R) {
  static const int sel[6] = {9, 10, 0, 1, 12, 13};   /* H1 selector, my_gmm.cpp:61-67 */
  for (int r = 0; r < d; ++r)
    for (int c = 0; c < d; ++c) {
      Q[r * d + c] = (1.0 - g * g) * s[r * d + c];
      F[r * d + c] = (r == c) ? g : 0.0;
    }
  for (int r = 0; r < d; ++r) B[r] = (1.0 - g) * u[r];
  for (int a = 0; a < 6; ++a) {
    for (int c = 0; c < d; ++c) H[a * d + c] = Hpca[c * Fdim + sel[a]];  /* H1 * H^T */
    BH[a] = mpca[sel[a]];                                                 /* H1 * m^T */
    for (int b = 0; b < 6; ++b) R[a * 6 + b] = (a == b) ? 100.0 : 0.0;
  }
}

/* ------------------------------------------------------------------------ */
/* measurement model                                                          */
/* ------------------------------------------------------------------------ */
void mko_measure(const mko_model* M, int k, const double* x, double* zhat, double* Hx) {
  int d = M->d, m = M->m;
  if (M->meas_mode == 0) {
    const double* H = M->H + (size_t)k * m * d;
    for (int a = 0; a < m; ++a) {
      double s = 0.0;
      for (int c = 0; c < d; ++c) s += H[a * d + c] * x[c];
      zhat[a] = s + M->BH[(size_t)k * m + a];
      for (int c = 0; c < d; ++c) Hx[a * d + c] = H[a * d + c];
    }
    return;
  }
  int J = m / 2;
  for (int j = 0; j < J; ++j) {
    const double* Bj = M->Bm + (size_t)j * 3 * d;
    double p[3];
    for (int r = 0; r < 3; ++r) {
      double s = 0.0;
      for (int c = 0; c < d; ++c) s += Bj[r * d + c] * x[c];
      p[r] = s + M->mm[j * 3 + r];
    }
    double iz = 1.0 / p[2];
    zhat[2 * j] = M->fx * p[0] * iz + M->cx;
    zhat[2 * j + 1] = M->fy * p[1] * iz + M->cy;
    double du[3] = {M->fx * iz, 0.0, -M->fx * p[0] * iz * iz};
    double dv[3] = {0.0, M->fy * iz, -M->fy * p[1] * iz * iz};
    for (int c = 0; c < d; ++c) {
      double su = 0.0, sv = 0.0;
      for (int r = 0; r < 3; ++r) { su += du[r] * Bj[r * d + c]; sv += dv[r] * Bj[r * d + c]; }
      Hx[(2 * j) * d + c] = su;
      Hx[(2 * j + 1) * d + c] = sv;
    }
  }
}

/* ------------------------------------------------------------------------ */
/* A8: ParticleFilter::update (pf2DRao.cpp:125-158)                          */
/* ------------------------------------------------------------------------ */
/* The update of pf2DRao.cpp:125-158.  lit == 0: the exact quantised
 * resampler on 32-bit uniforms U_ind / U_anc, the exact Gaussian, weights
 * normalised after a max shift.  lit == 1: the reference's literal wheel
 * (pf2DRao.cpp:175-210) on the double uniforms u_ind / u_anc (fb_ind / fb_anc:
 * the indices its all-zero branch draws), the Gaussian in mvn_mode, and the
 * weights normalised in the linear domain as pf2DRao.cpp:138-148 does. */
static int rbpf_update_impl(const mko_model* M, int N, double* x, double* P, const double* z, unsigned mask,
                            int lit, uint32_t U_ind, uint32_t U_anc, double u_ind, const int* fb_ind,
                            double u_anc, const int* fb_anc, int mvn_mode, const int* alias_prev_anc,
                            int* ind_out, double* logw_out, double* wn_out, int* anc_out) {
  int d = M->d, m = M->m, K = M->K;
  int* ind = (int*)malloc(sizeof(int) * (size_t)N);
  int* anc = (int*)malloc(sizeof(int) * (size_t)N);
  double* lw = (double*)malloc(sizeof(double) * (size_t)N);
  double* wn = (double*)malloc(sizeof(double) * (size_t)N);
  double* tx = (double*)malloc(sizeof(double) * (size_t)N * d);
  double* tP = (double*)malloc(sizeof(double) * (size_t)N * d * d);
  int* last_owner = NULL;
  if (alias_prev_anc) {
    last_owner = (int*)malloc(sizeof(int) * (size_t)N);
    for (int j = 0; j < N; ++j) last_owner[j] = -1;
  }
  /* Propose indicators: systematic resampling of the mixture weights (128) */
  if (lit) mko_resample_wheel(M->weight, K, N, u_ind, fb_ind, ind);
  else mko_resample_f64(M->weight, K, N, U_ind, ind);
  for (int j = 0; j < N; ++j) {
    int k = ind[j];
    double* xs = x + (size_t)j * d;
    double* Ps = P + (size_t)j * d * d;
    if (alias_prev_anc) {
      /* shallow copy-assign quirk: tracks resampled from the same ancestor
       * share one cv::Mat buffer, and the in-place predict/update of an
       * earlier sharer is what a later sharer starts from */
      int b = alias_prev_anc[j];
      if (last_owner[b] >= 0) {
        memcpy(xs, tx + (size_t)last_owner[b] * d, sizeof(double) * (size_t)d);
        memcpy(Ps, tP + (size_t)last_owner[b] * d * d, sizeof(double) * (size_t)d * d);
      }
      last_owner[b] = j;
    }
    mko_kf_predict(d, M->F + (size_t)k * d * d, M->B + (size_t)k * d, M->Q + (size_t)k * d * d, xs, Ps);
    double zhat[16], Hx[16 * 64], S[256], zz[16], zh[16];
    mko_measure(M, k, xs, zhat, Hx);
    /* weight = mvnpdf(z, H x + BH, H P H^T + R) over the used rows (138) */
    int rows[16], mm = 0;
    for (int r = 0; r < m; ++r) if (mask & (1u << r)) rows[mm++] = r;
    const double* R = M->R + (size_t)k * m * m;
    for (int a = 0; a < mm; ++a) {
      zz[a] = z[(size_t)j * m + rows[a]];
      zh[a] = zhat[rows[a]];
      for (int b = 0; b < mm; ++b) {
        double s = 0.0;
        for (int r = 0; r < d; ++r) {
          double t = 0.0;
          for (int c = 0; c < d; ++c) t += Ps[r * d + c] * Hx[rows[b] * d + c];
          s += Hx[rows[a] * d + r] * t;
        }
        S[a * mm + b] = s + R[rows[a] * m + rows[b]];
      }
    }
    lw[j] = mm ? mko_mvn_logpdf(mm, zz, zh, S, lit ? mvn_mode : 0) : 0.0;
    kf_update_generic(d, m, Hx, zhat, R, z + (size_t)j * m, mask, xs, Ps);   /* (140) */
    memcpy(tx + (size_t)j * d, xs, sizeof(double) * (size_t)d);               /* temp.push_back */
    memcpy(tP + (size_t)j * d * d, Ps, sizeof(double) * (size_t)d * d);
  }
  int fb;
  if (lit) {
    /* linear-domain weights and their sum (138-139), normalised (145-148) */
    double sum = 0.0;
    for (int j = 0; j < N; ++j) { wn[j] = exp(lw[j]); sum += wn[j]; }
    for (int j = 0; j < N; ++j) wn[j] = wn[j] / sum;
    double mw = 0.0;
    for (int j = 0; j < N; ++j) if (wn[j] > mw) mw = wn[j];
    fb = !(mw > 0.0);
    mko_resample_wheel(wn, N, N, u_anc, fb_anc, anc);                          /* (152) */
  } else {
    /* normalise (145-148), max-shifted so that underflow cannot zero every weight */
    double mx = -INFINITY;
    for (int j = 0; j < N; ++j) if (lw[j] > mx) mx = lw[j];
    double sum = 0.0;
    for (int j = 0; j < N; ++j) { wn[j] = isfinite(mx) ? exp(lw[j] - mx) : 0.0; sum += wn[j]; }
    for (int j = 0; j < N; ++j) wn[j] = wn[j] / sum;
    fb = mko_resample_f64(wn, N, N, U_anc, anc);                              /* (152) */
  }
  for (int j = 0; j < N; ++j) {                                              /* (153-156) */
    memcpy(x + (size_t)j * d, tx + (size_t)anc[j] * d, sizeof(double) * (size_t)d);
    memcpy(P + (size_t)j * d * d, tP + (size_t)anc[j] * d * d, sizeof(double) * (size_t)d * d);
  }
  if (ind_out) memcpy(ind_out, ind, sizeof(int) * (size_t)N);
  if (logw_out) memcpy(logw_out, lw, sizeof(double) * (size_t)N);
  if (wn_out) memcpy(wn_out, wn, sizeof(double) * (size_t)N);
  if (anc_out) memcpy(anc_out, anc, sizeof(int) * (size_t)N);
  free(ind); free(anc); free(lw); free(wn); free(tx); free(tP); free(last_owner);
  return fb;
}

int mko_rbpf_update(const mko_model* M, int N, double* x, double* P, const double* z,
                    unsigned mask, uint32_t U_ind, uint32_t U_anc, const int* alias_prev_anc,
                    int* ind_out, double* logw_out, double* wn_out, int* anc_out) {
  return rbpf_update_impl(M, N, x, P, z, mask, 0, U_ind, U_anc, 0.0, NULL, 0.0, NULL, 0, alias_prev_anc,
                          ind_out, logw_out, wn_out, anc_out);
}

int mko_rbpf_update_literal(const mko_model* M, int N, double* x, double* P, const double* z, unsigned mask,
                            double u_ind, const int* fb_ind, double u_anc, const int* fb_anc, int mvn_mode,
                            const int* alias_prev_anc, int* ind_out, double* logw_out, double* wn_out,
                            int* anc_out) {
  return rbpf_update_impl(M, N, x, P, z, mask, 1, 0u, 0u, u_ind, fb_ind, u_anc, fb_anc, mvn_mode,
                          alias_prev_anc, ind_out, logw_out, wn_out, anc_out);
}

void mko_rbpf_estimate(int N, int d, const double* x, double* est) {
  for (int c = 0; c < d; ++c) est[c] = 0.0;
  double f = 1.0 / (double)N;
  for (int j = 0; j < N; ++j)
    for (int c = 0; c < d; ++c) est[c] += f * x[(size_t)j * d + c];
}

/* ------------------------------------------------------------------------ */
/* A9: PDAF association weights (pfPose.cpp:247-298)                          */
/* ------------------------------------------------------------------------ */
static double gauss2(const double* c, const double* u, double var) {
  double dx = c[0] - u[0], dy = c[1] - u[1];
  return exp(-0.5 * (dx * dx + dy * dy) / var) / (2.0 * M_PI * var);
}

void mko_pdaf_weights(int M, const double* cand, const double* Lc, const double* hat_own,
                      const double* hat_other, int has_other, double var, double Pa,
                      double clutter, double* w) {
  for (int j = 0; j < M; ++j) {
    double po = gauss2(cand + 2 * j, hat_own, var);
    double pt = has_other ? gauss2(cand + 2 * j, hat_other, var) : 0.0;
    double Z = has_other ? (po * Pa + pt * Pa + clutter * (1.0 - 2.0 * Pa))
                         : (po * Pa + clutter * (1.0 - Pa));
    w[j] = Lc ? Lc[j] / Z : Pa * po / Z;
  }
}

/* ------------------------------------------------------------------------ */
/* A13: bootstrap PF over the mixture-of-MRRW motion model                    */
/* (structure of pf2D.cpp:148-210 with my_gmm.cpp:53-58's motion)             */
/* ------------------------------------------------------------------------ */
int mko_pick_component(const float* cumpi, int K, float u) {
  for (int c = 0; c < K; ++c) if (u < cumpi[c]) return c;
  return K - 1;
}

void mko_bpf_prior(const mko_bpf_params* p, const double* eps, float ucomp, double* x) {
  int d = p->d, DD = d * (d + 1) / 2;
  int k = mko_pick_component(p->cumpi, p->K, ucomp);
  const float* Lc = p->S0c + (size_t)k * DD;
  for (int r = 0; r < d; ++r) {
    double s = (double)p->mu[k * d + r];
    for (int c = 0; c <= r; ++c) s += (double)Lc[r * (r + 1) / 2 + c] * eps[c];
    x[r] = s;
  }
}

void mko_bpf_propagate(const mko_bpf_params* p, const double* eps, float ucomp, double* x) {
  int d = p->d, DD = d * (d + 1) / 2;
  int k = mko_pick_component(p->cumpi, p->K, ucomp);
  const float* Lc = p->Lq + (size_t)k * DD;
  double xn[64];
  for (int r = 0; r < d; ++r) {
    double s = (double)p->a[k * d + r] * x[r] + (double)p->mb[k * d + r];
    for (int c = 0; c <= r; ++c) s += (double)Lc[r * (r + 1) / 2 + c] * eps[c];
    xn[r] = s;
  }
  memcpy(x, xn, sizeof(double) * (size_t)d);
}

#define MKO_ZMIN 0.05

double mko_bpf_loglik(const mko_bpf_params* p, const double* x, const int* det_off, const float* det) {
  int d = p->d;
  double s2 = (double)p->sigma * (double)p->sigma;
  double norm = 1.0 / (2.0 * M_PI * s2);
  double floor_ = (1.0 - (double)p->pd) * (double)p->kappa;
  double ll = 0.0;
  for (int j = 0; j < p->J; ++j) {
    const float* Bj = p->Bm + (size_t)j * 3 * d;
    double q[3];
    for (int r = 0; r < 3; ++r) {
      double s = (double)p->mm[j * 3 + r];
      for (int c = 0; c < d; ++c) s += (double)Bj[r * d + c] * x[c];
      q[r] = s;
    }
    if (!(q[2] > MKO_ZMIN)) { ll += log((double)p->kappa); continue; }
    double u = (double)p->fx * q[0] / q[2] + (double)p->cx;
    double v = (double)p->fy * q[1] / q[2] + (double)p->cy;
    double acc = 0.0;
    for (int i = det_off[j]; i < det_off[j + 1]; ++i) {
      double dx = (double)det[2 * i] - u, dy = (double)det[2 * i + 1] - v;
      acc += exp(-0.5 * (dx * dx + dy * dy) / s2);
    }
    ll += log(floor_ + (double)p->pd * norm * acc);
  }
  return ll;
}

void mko_bpf_prior_set(const mko_bpf_params* p, int N, const float* eps, const float* ucomp, double* x,
                       int nthreads) {
  int d = p->d;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
  for (int i = 0; i < N; ++i) {
    double e[64];
    for (int c = 0; c < d; ++c) e[c] = (double)eps[(size_t)i * d + c];
    mko_bpf_prior(p, e, ucomp[i], x + (size_t)i * d);
  }
}

void mko_bpf_forced_frames(const mko_bpf_params* p, int N, int nf, double* x, const int* anc_prev,
                           const float* eps, const float* ucomp, const int* anc, const float* w_dev,
                           const int* det_off, const float* det, double* est, double* loglik,
                           double* ess, double* w_err, int nthreads) {
  int d = p->d, J = p->J;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#endif
  double* xb = (double*)malloc(sizeof(double) * (size_t)N * d);
  double* lw = (double*)malloc(sizeof(double) * (size_t)N);
  const int* ap = anc_prev;
  for (int f = 0; f < nf; ++f) {
    const int* off = det_off + (size_t)f * J;
    const float* ef = eps + (size_t)f * N * d;
    const float* uf = ucomp + (size_t)f * N;
    double mx = -INFINITY;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads) reduction(max : mx)
#endif
    for (int i = 0; i < N; ++i) {
      double e[64];
      double* xi = xb + (size_t)i * d;
      memcpy(xi, x + (size_t)ap[i] * d, sizeof(double) * (size_t)d);
      for (int c = 0; c < d; ++c) e[c] = (double)ef[(size_t)i * d + c];
      mko_bpf_propagate(p, e, uf[i], xi);
      lw[i] = mko_bpf_loglik(p, xi, off, det);
      if (lw[i] > mx) mx = lw[i];
    }
    double S = 0.0, S2 = 0.0, werr = 0.0, e[64];
    int wnan = 0;
    for (int c = 0; c < d; ++c) e[c] = 0.0;
    const float* wd = w_dev ? w_dev + (size_t)f * N : NULL;
    /* fixed-order sums (deterministic for any thread count) */
    for (int i = 0; i < N; ++i) {
      double w = exp(lw[i] - mx);
      S += w;
      S2 += w * w;
      for (int c = 0; c < d; ++c) e[c] += w * xb[(size_t)i * d + c];
      if (wd) {
        double dw = fabs(w - (double)wd[i]);
        if (dw != dw) wnan = 1;          /* a NaN device weight reports NaN */
        else if (dw > werr) werr = dw;
      }
    }
    for (int c = 0; c < d; ++c) est[(size_t)f * d + c] = e[c] / S;
    loglik[f] = mx + log(S) - log((double)N);
    ess[f] = S * S / S2;
    if (w_err) w_err[f] = wd ? (wnan ? NAN : werr) : 0.0;
    memcpy(x, xb, sizeof(double) * (size_t)N * d);
    ap = anc + (size_t)f * N;
  }
  free(xb);
  free(lw);
}

int mko_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void mko_bpf_run_tracks(int n_tracks, const mko_track* tracks, int d, int K, int J,
                        const float* a, const float* mb, const float* mu, const float* Lq,
                        const float* S0c, const float* cumpi, const float* Bm, const float* mm,
                        float fx, float fy, float cx, float cy,
                        const int* det_off, const float* det,
                        float* est, float* loglik, float* ess, int nthreads) {
  int DD = d * (d + 1) / 2;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
  for (int t = 0; t < n_tracks; ++t) {
    const mko_track* tr = &tracks[t];
    int N = tr->n_particles, pi = tr->param_index;
    mko_bpf_params p;
    p.d = d; p.K = K; p.J = J;
    p.a = a + (size_t)pi * K * d; p.mb = mb + (size_t)pi * K * d; p.mu = mu + (size_t)pi * K * d;
    p.Lq = Lq + (size_t)pi * K * DD; p.S0c = S0c + (size_t)pi * K * DD; p.cumpi = cumpi + (size_t)pi * K;
    p.Bm = Bm + (size_t)pi * J * 3 * d; p.mm = mm + (size_t)pi * J * 3;
    p.fx = fx; p.fy = fy; p.cx = cx; p.cy = cy;
    p.kappa = tr->kappa; p.pd = tr->pd; p.sigma = tr->sigma;
    double* xa = (double*)malloc(sizeof(double) * (size_t)N * d);
    double* xb = (double*)malloc(sizeof(double) * (size_t)N * d);
    double* lw = (double*)malloc(sizeof(double) * (size_t)N);
    int* anc = (int*)malloc(sizeof(int) * (size_t)N);
    double eps[64];
    float uc;
    for (int i = 0; i < N; ++i) {
      mko_particle_draws(tr->seed, (uint32_t)tr->track_id, 0xFFFFFFFFu, (uint32_t)i, d, eps, &uc);
      mko_bpf_prior(&p, eps, uc, xa + (size_t)i * d);
      anc[i] = i;
    }
    for (int f = 0; f < tr->n_frames; ++f) {
      long long g = tr->frame_base + f;
      const int* off = det_off + g * J;
      double mx = -INFINITY;
      for (int i = 0; i < N; ++i) {
        double* xi = xb + (size_t)i * d;
        memcpy(xi, xa + (size_t)anc[i] * d, sizeof(double) * (size_t)d);
        mko_particle_draws(tr->seed, (uint32_t)tr->track_id, (uint32_t)f, (uint32_t)i, d, eps, &uc);
        mko_bpf_propagate(&p, eps, uc, xi);
        lw[i] = mko_bpf_loglik(&p, xi, off, det);
        if (lw[i] > mx) mx = lw[i];
      }
      double S = 0.0, S2 = 0.0, e[64];
      for (int c = 0; c < d; ++c) e[c] = 0.0;
      for (int i = 0; i < N; ++i) {
        double w = exp(lw[i] - mx);
        lw[i] = w;
        S += w; S2 += w * w;
        for (int c = 0; c < d; ++c) e[c] += w * xb[(size_t)i * d + c];
      }
      for (int c = 0; c < d; ++c) est[(size_t)g * d + c] = (float)(e[c] / S);
      loglik[g] = (float)(mx + log(S) - log((double)N));
      ess[g] = (float)(S * S / S2);
      uint32_t o[4];
      mko_draw_block(tr->seed, (uint32_t)tr->track_id, (uint32_t)f, 0xFFFFFFFFu, 0x100u, o);
      mko_resample_f64(lw, N, N, o[0], anc);
      double* tmp = xa; xa = xb; xb = tmp;
    }
    free(xa); free(xb); free(lw); free(anc);
  }
}

/* ------------------------------------------------------------------------ */
/* A12: legacy bootstrap PF pf2D (pf2D.cpp:13-268)                            */
/* ------------------------------------------------------------------------ */
void mko_pf2d_load(int d, int K, const double* mean, const double* cov, double* sinv, double* det_s) {
  (void)mean;
  for (int k = 0; k < K; ++k) {
    const double* S = cov + (size_t)k * d * d;
    double Lo[64 * 64];
    chol_lower(d, S, Lo);
    double ld = 0.0;
    for (int i = 0; i < d; ++i) ld += 2.0 * log(Lo[i * d + i]);
    det_s[k] = 1.0 / (pow(2.0 * M_PI, d / 2.0) * sqrt(exp(ld)));   /* pf2D.cpp:35 */
    inv_lu(d, S, sinv + (size_t)k * d * d);                          /* invert(s, .., DECOMP_CHOLESKY) */
  }
}

static void pf2d_uniform_row(const mko_pf2d_model* m, const double* u, double* x) {
  for (int c = 0; c < m->d; ++c) {
    double lo = 1.0, hi;
    if (c == 6) { lo = m->width / 2.0 * m->side + 1.0; hi = m->width / 2.0 + m->width / 2.0 * m->side; }
    else hi = ((c % 2) == 0) * (double)m->width + (((c + 1) % 2) == 0) * (double)m->height;
    x[c] = lo + u[c] * (hi - lo);
  }
}

void mko_pf2d_init(const mko_pf2d_model* m, int N, const double* u, double* particles, double* weights) {
  for (int i = 0; i < N; ++i) {
    pf2d_uniform_row(m, u + (size_t)i * m->d, particles + (size_t)i * m->d);
    weights[i] = 1.0 / (double)N;
  }
}

int mko_pf2d_update(const mko_pf2d_model* m, int N, double* particles, double* weights, const double* z,
                    uint32_t U, const double* reinit_u, const double* eps, double* w_out, int* anc_out) {
  const int d = m->d;
  double sum = 0.0;
  for (int i = 0; i < N; ++i) {
    const double* x = particles + (size_t)i * d;
    double prior = 0.0;
    for (int k = 0; k < m->K; ++k) {
      const double* mu = m->mean + (size_t)k * d;
      const double* Si = m->sinv + (size_t)k * d * d;
      double q = 0.0;
      for (int r = 0; r < d; ++r) {
        double t = 0.0;
        for (int c = 0; c < d; ++c) t += Si[r * d + c] * (x[c] - mu[c]);
        q += (x[r] - mu[r]) * t;
      }
      prior += m->w[k] * m->det_s[k] * (double)expf((float)(-0.5 * q));
    }
    double d0 = x[6] - z[0], d1 = x[7] - z[1], h0 = x[0] - z[2], h1 = x[1] - z[3];
    double lik = (1.0 / (2.0 * M_PI * 15.0)) * exp(-0.5 * (d0 * d0 + d1 * d1) / 15.0) *
                 (1.0 / (2.0 * M_PI * 15.0)) * exp(-0.5 * (h0 * h0 + h1 * h1) / 15.0);
    weights[i] = prior * lik;
    sum += weights[i];
  }
  for (int i = 0; i < N; ++i) weights[i] /= sum;
  if (w_out) memcpy(w_out, weights, sizeof(double) * (size_t)N);
  double mw = 0.0;
  for (int i = 0; i < N; ++i) if (weights[i] > mw) mw = weights[i];
  int reinit = !(mw > 0.0);
  double* old = (double*)malloc(sizeof(double) * (size_t)N * d);
  memcpy(old, particles, sizeof(double) * (size_t)N * d);
  if (reinit) {
    for (int i = 0; i < N; ++i) {
      pf2d_uniform_row(m, reinit_u + (size_t)i * d, particles + (size_t)i * d);
      weights[i] = 1.0 / (double)N;
      if (anc_out) anc_out[i] = -1;
    }
  } else {
    int* anc = (int*)malloc(sizeof(int) * (size_t)N);
    mko_resample_f64(weights, N, N, U, anc);
    for (int i = 0; i < N; ++i) memcpy(particles + (size_t)i * d, old + (size_t)anc[i] * d, sizeof(double) * (size_t)d);
    if (anc_out) memcpy(anc_out, anc, sizeof(int) * (size_t)N);
    free(anc);
  }
  for (int i = 0; i < N; ++i)
    for (int c = 0; c < 8 && c < d; ++c) particles[(size_t)i * d + c] += 5.0 * eps[(size_t)i * 8 + c];
  free(old);
  return reinit;
}

void mko_pf2d_estimate(int N, int d, const double* particles, const double* weights, double* est) {
  for (int c = 0; c < d; ++c) est[c] = 0.0;
  for (int i = 0; i < N; ++i)
    for (int c = 0; c < d; ++c) est[c] += weights[i] * particles[(size_t)i * d + c];
}

/* ------------------------------------------------------------------------ */
/* f2: pose decode and 3-D back-projection (pfPose.cpp:84-127, 173-208)      */
/* ------------------------------------------------------------------------ */
void mko_pose_decode(int d, int F, const double* Hpca, const double* mpca, const double* x, double* e) {
  for (int f = 0; f < F; ++f) {          /* pfPose.cpp:347-348: e = (H_pca^T x + m_pca^T)^T */
    double s = 0.0;
    for (int r = 0; r < d; ++r) s += Hpca[(size_t)r * F + f] * x[r];
    e[f] = s + mpca[f];
  }
}

static void mat3_mul(const double* A, const double* B, double* C) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int k = 0; k < 3; ++k) s += A[i * 3 + k] * B[k * 3 + j];
      C[i * 3 + j] = s;
    }
}

void mko_pose3d(const double* e, const double* Kc, double* pos3d) {
  const double roll = e[16], pitch = e[17], yaw = e[15];       /* pfPose.cpp:104 */
  const double R1[9] = {1, 0, 0, 0, cos(roll), -sin(roll), 0, sin(roll), cos(roll)};
  const double R2[9] = {cos(pitch), 0, sin(pitch), 0, 1, 0, -sin(pitch), 0, cos(pitch)};
  const double R3[9] = {cos(yaw), -sin(yaw), 0, sin(yaw), cos(yaw), 0, 0, 0, 1};
  double T1[9], R[9], P3[9], Pi[9];
  mat3_mul(R3, R2, T1);
  mat3_mul(T1, R1, R);                                          /* rpy: R3 R2 R1 (pfPose.cpp:91) */
  mat3_mul(Kc, R, P3);
  double p4[3];
  for (int i = 0; i < 3; ++i) p4[i] = Kc[i * 3 + 0] * e[18] + Kc[i * 3 + 1] * e[19] + Kc[i * 3 + 2] * e[20];
  inv_lu(3, P3, Pi);                                            /* invert(.., DECOMP_LU) */
  for (int k = 0; k < 5; ++k) {
    const double Z = e[3 * k + 2];
    const double ip[3] = {e[3 * k] * Z - p4[0], e[3 * k + 1] * Z - p4[1], Z - p4[2]};
    for (int i = 0; i < 3; ++i)
      pos3d[i * 5 + k] = Pi[i * 3 + 0] * ip[0] + Pi[i * 3 + 1] * ip[1] + Pi[i * 3 + 2] * ip[2];
  }
}

void mko_pose2d_record(const double* e1, const double* e2, double* p) {
  p[0] = e1[0]; p[1] = e1[1];                                   /* hand1 */
  p[2] = e2[0]; p[3] = e2[1];                                   /* hand2 */
  p[4] = 0.5 * (e1[9] + e2[9]); p[5] = 0.5 * (e1[10] + e2[10]); /* head */
  p[6] = 0.5 * (e1[12] + e2[12]); p[7] = 0.5 * (e1[13] + e2[13]); /* neck */
  p[8] = e1[3]; p[9] = e1[4];                                   /* elbow1 */
  p[10] = e2[3]; p[11] = e2[4];                                 /* elbow2 */
  p[12] = e1[6]; p[13] = e1[7];                                 /* shoulder1 */
  p[14] = e2[6]; p[15] = e2[7];                                 /* shoulder2 */
}

/* ------------------------------------------------------------------------ */
/* f1: likelihood-image front end (pfPose.cpp:210-301)                        */
/* ------------------------------------------------------------------------ */
static int reflect101(int i, int n) {
  if (i < 0) i = -i;
  if (i >= n) i = 2 * n - 2 - i;
  return i;
}

void mko_gaussian_blur_u8(const uint8_t* in, int W, int H, uint8_t* out) {
  float w[15];
  double e[15], sum = 0.0;
  for (int k = 0; k < 15; ++k) { double x = (double)(k - 7); e[k] = exp(-x * x / 18.0); sum += e[k]; }
  for (int k = 0; k < 15; ++k) w[k] = (float)(e[k] / sum);
  float* h = (float*)malloc(sizeof(float) * (size_t)W * H);
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      float acc = 0.0f;
      for (int k = 0; k < 15; ++k) acc = fmaf(w[k], (float)in[(size_t)y * W + reflect101(x + k - 7, W)], acc);
      h[(size_t)y * W + x] = acc;
    }
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      float acc = 0.0f;
      for (int k = 0; k < 15; ++k) acc = fmaf(w[k], h[(size_t)reflect101(y + k - 7, H) * W + x], acc);
      float v = rintf(acc);
      v = v < 0.0f ? 0.0f : (v > 255.0f ? 255.0f : v);
      out[(size_t)y * W + x] = (uint8_t)v;
    }
  free(h);
}

void mko_image_lookup(int M, const double* cand, const uint8_t* img, int W, int H, double* L) {
  for (int j = 0; j < M; ++j) {
    double x = cand[2 * j], y = cand[2 * j + 1];
    L[j] = (y > 0 && y < H && x > 0 && x < W) ? (double)img[(size_t)(int)y * W + (int)x] / 255.0 : 0.0;
  }
}
