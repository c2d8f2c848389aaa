// rbpf.cu -- Rao-Blackwellised particle filter (mixture Kalman filter) of
// pf2DRao (pf2DRao.cpp:125-158) over KF_model (KF_model.cpp:11-25) and the
// my_gmm motion model (my_gmm.cpp:30-75), plus the PDAF association of
// PFTracker::getMeasurementProposal (pfPose.cpp:210-329), in FP64.
//
// Per update: one warp per particle (indicator draw, KF predict, innovation
// Cholesky + Gaussian log-weight, KF update), one block for normalisation and
// exact systematic resampling, one gather of the surviving tracks.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "mkf_common.cuh"

namespace mkf {

constexpr int kMMax = MKF_MAX_M;
constexpr uint32_t kStreamIndicator = 0x102u;
constexpr uint32_t kStreamPdaf = 0x103u;

struct RbpfParams {          // device pointers
  const double *f, *B, *Q, *H, *BH, *R, *w, *mu, *Sigma, *Bm, *mm, *Hd, *hb;
  double fx, fy, cx, cy;
  int d, m, K, N, mode, hand_joint;
};

struct RbpfStepArgs {
  RbpfParams p;
  const double* x;
  const double* P;
  const double* z;
  unsigned mask;
  uint32_t U_ind;
  double* tx;
  double* tP;
  double* logw;
  int* ind;
  int* status;
};

__host__ __device__ inline int rbpf_warp_doubles(int D) {
  return D * D + D + 4 * kMMax * D + 2 * kMMax * kMMax + 2 * kMMax;
}

// systematic indicator of particle j over the K mixture weights, lane c holds w_c
__device__ __forceinline__ int warp_indicator(const double* w, int K, int N, int j, uint32_t U, int lane) {
  double v = (lane < K) ? w[lane] : 0.0;
  double mx = (lane < K && v > 0.0) ? v : 0.0;
  int inf = (lane < K && isinf(v) && v > 0.0) ? 1 : 0;
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    inf |= __shfl_xor_sync(0xffffffffu, inf, o);
  }
  if (inf || !(mx > 0.0)) return resample_fallback_index(U, j, K);
  int e;
  frexp(mx, &e);
  uint64_t q = (lane < K) ? quantize_f64(v, e) : 0ull;
  uint64_t Q = warp_incl_scan_u64(q, lane);
  uint64_t Qt = __shfl_sync(0xffffffffu, Q, K - 1);
  const unsigned __int128 rhs = resample_rhs(j, U, Qt);
  bool ok = (lane < K) && ((((unsigned __int128)(uint64_t)N * (unsigned __int128)Q) << 32) >= rhs);
  unsigned bal = __ballot_sync(0xffffffffu, ok);
  return bal ? (__ffs(bal) - 1) : (K - 1);
}

template <int D>
__global__ void __launch_bounds__(128) rbpf_step_kernel(RbpfStepArgs A) {
  extern __shared__ double rsm[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, wpb = blockDim.x >> 5;
  const int j = blockIdx.x * wpb + wib;
  const RbpfParams& p = A.p;
  if (j >= p.N) return;                      // warp-uniform
  const int m = p.m;
  double* sP = rsm + (size_t)wib * rbpf_warp_doubles(D);
  double* sx = sP + D * D;
  double* sH = sx + D;                        // mm x D
  double* sPHt = sH + kMMax * D;              // D x mm
  double* sHP = sPHt + kMMax * D;             // mm x D
  double* sK = sHP + kMMax * D;               // D x mm
  double* sS = sK + kMMax * D;                // mm x mm (then its Cholesky factor)
  double* sSi = sS + kMMax * kMMax;           // mm x mm inverse
  double* szh = sSi + kMMax * kMMax;          // mm
  double* sy = szh + kMMax;                   // mm
  int rows[kMMax];
  int mm = 0;
  for (int r = 0; r < m; ++r)
    if (A.mask & (1u << r)) rows[mm++] = r;

  for (int i = lane; i < D * D; i += 32) sP[i] = A.P[(size_t)j * D * D + i];
  if (lane < D) sx[lane] = A.x[(size_t)j * D + lane];
  // ---- component indicator: systematic resampling of pi (pf2DRao.cpp:128)
  const int k = warp_indicator(p.w, p.K, p.N, j, A.U_ind, lane);
  __syncwarp();
  // ---- KF_model::predict: x = F x + B, P = F P F^T + Q with F = diag(f)
  const double* f = p.f + k * D;
  for (int i = lane; i < D * D; i += 32) {
    int r = i / D, c = i - r * D;
    sP[i] = (f[r] * sP[i]) * f[c] + p.Q[(size_t)k * D * D + i];
  }
  if (lane < D) sx[lane] = f[lane] * sx[lane] + p.B[k * D + lane];
  __syncwarp();
  // ---- predicted measurement and its Jacobian over the used rows
  if (p.mode == MKF_MEAS_LINEAR) {
    const double* H = p.H + (size_t)k * m * D;
    for (int i = lane; i < mm * D; i += 32) {
      int a = i / D, c = i - a * D;
      sH[a * D + c] = H[rows[a] * D + c];
    }
    if (lane < mm) {
      double s = p.BH[k * m + rows[lane]];
      for (int c = 0; c < D; ++c) s += H[rows[lane] * D + c] * sx[c];
      szh[lane] = s;
    }
  } else if (lane < mm) {
    const int r = rows[lane], jj = r >> 1, comp = r & 1;
    const double* Bj = p.Bm + (size_t)jj * 3 * D;
    double q[3];
    for (int t = 0; t < 3; ++t) {
      double s = p.mm[jj * 3 + t];
      for (int c = 0; c < D; ++c) s += Bj[t * D + c] * sx[c];
      q[t] = s;
    }
    const double iz = 1.0 / q[2];
    double du[3];
    if (comp == 0) {
      szh[lane] = p.fx * q[0] * iz + p.cx;
      du[0] = p.fx * iz; du[1] = 0.0; du[2] = -p.fx * q[0] * iz * iz;
    } else {
      szh[lane] = p.fy * q[1] * iz + p.cy;
      du[0] = 0.0; du[1] = p.fy * iz; du[2] = -p.fy * q[1] * iz * iz;
    }
    for (int c = 0; c < D; ++c)
      sH[lane * D + c] = du[0] * Bj[c] + du[1] * Bj[D + c] + du[2] * Bj[2 * D + c];
  }
  __syncwarp();
  if (lane < mm) sy[lane] = A.z[(size_t)j * m + rows[lane]] - szh[lane];
  // PHt = P H^T  (D x mm), HP = H P (mm x D)
  for (int i = lane; i < D * mm; i += 32) {
    int r = i / mm, a = i - r * mm;
    double s = 0.0;
    for (int c = 0; c < D; ++c) s += sP[r * D + c] * sH[a * D + c];
    sPHt[r * mm + a] = s;
  }
  for (int i = lane; i < mm * D; i += 32) {
    int a = i / D, c = i - a * D;
    double s = 0.0;
    for (int r = 0; r < D; ++r) s += sH[a * D + r] * sP[r * D + c];
    sHP[a * D + c] = s;
  }
  __syncwarp();
  // S = H P H^T + R
  const double* R = p.R + (size_t)k * m * m;
  for (int i = lane; i < mm * mm; i += 32) {
    int a = i / mm, b = i - a * mm;
    double s = 0.0;
    for (int r = 0; r < D; ++r) s += sH[a * D + r] * sPHt[r * mm + b];
    sS[a * mm + b] = s + R[rows[a] * m + rows[b]];
  }
  __syncwarp();
  // ---- lane 0: Cholesky of S, Gaussian log density (pf2DRao.cpp:56-67,
  // exact semantics), and S^-1 from the factor
  int ok = 1;
  double lw = 0.0;
  if (lane == 0 && mm > 0) {
    double L[kMMax * kMMax], Li[kMMax * kMMax], v[kMMax];
    for (int a = 0; a < mm * mm; ++a) { L[a] = 0.0; Li[a] = 0.0; }
    double hld = 0.0, qf = 0.0;
    for (int a = 0; a < mm && ok; ++a) {
      for (int b = 0; b <= a; ++b) {
        double s = sS[a * mm + b];
        for (int c = 0; c < b; ++c) s -= L[a * mm + c] * L[b * mm + c];
        if (a == b) {
          if (!(s > 0.0)) { ok = 0; break; }
          L[a * mm + a] = sqrt(s);
        } else {
          L[a * mm + b] = s / L[b * mm + b];
        }
      }
    }
    // a non-finite measurement (a caller's fault) gives the particle zero
    // weight and no update, so that a frame of them resamples by the uniform
    // fallback instead of turning every state into NaN; flagged MKF_ST_NAN
    bool finite = true;
    for (int a = 0; a < mm; ++a) finite = finite && isfinite(sy[a]);
    if (!finite) {
      ok = 0;
      lw = -INFINITY;
      atomicOr(A.status, MKF_ST_NAN);
    }
    if (ok) {
      for (int a = 0; a < mm; ++a) {
        double s = sy[a];
        for (int c = 0; c < a; ++c) s -= L[a * mm + c] * v[c];
        v[a] = s / L[a * mm + a];
        qf += v[a] * v[a];
        hld += log(L[a * mm + a]);
      }
      lw = -0.5 * qf - hld - 0.5 * (double)mm * 1.8378770664093453;   // log(2 pi)
      for (int a = 0; a < mm; ++a) {            // Li = L^-1 (lower)
        Li[a * mm + a] = 1.0 / L[a * mm + a];
        for (int b = 0; b < a; ++b) {
          double s = 0.0;
          for (int c = b; c < a; ++c) s -= L[a * mm + c] * Li[c * mm + b];
          Li[a * mm + b] = s / L[a * mm + a];
        }
      }
      for (int a = 0; a < mm; ++a)              // S^-1 = Li^T Li
        for (int b = 0; b < mm; ++b) {
          double s = 0.0;
          for (int c = (a > b ? a : b); c < mm; ++c) s += Li[c * mm + a] * Li[c * mm + b];
          sSi[a * mm + b] = s;
        }
    } else if (finite) {
      lw = -INFINITY;
      atomicOr(A.status, MKF_ST_NONPD);
    }
  }
  ok = __shfl_sync(0xffffffffu, ok, 0);
  lw = __shfl_sync(0xffffffffu, lw, 0);
  __syncwarp();
  if (ok && mm > 0) {
    // K = P H^T S^-1; x += K y; P = (I - K H) P = P - K (H P)
    for (int i = lane; i < D * mm; i += 32) {
      int r = i / mm, b = i - r * mm;
      double s = 0.0;
      for (int a = 0; a < mm; ++a) s += sPHt[r * mm + a] * sSi[a * mm + b];
      sK[r * mm + b] = s;
    }
    __syncwarp();
    double xn = 0.0;
    if (lane < D) {
      double s = 0.0;
      for (int a = 0; a < mm; ++a) s += sK[lane * mm + a] * sy[a];
      xn = sx[lane] + s;
    }
    for (int i = lane; i < D * D; i += 32) {
      int r = i / D, c = i - r * D;
      double s = 0.0;
      for (int a = 0; a < mm; ++a) s += sK[r * mm + a] * sHP[a * D + c];
      sP[i] -= s;
    }
    __syncwarp();
    if (lane < D) sx[lane] = xn;
    __syncwarp();
  }
  for (int i = lane; i < D * D; i += 32) A.tP[(size_t)j * D * D + i] = sP[i];
  if (lane < D) A.tx[(size_t)j * D + lane] = sx[lane];
  if (lane == 0) {
    A.logw[j] = lw;
    A.ind[j] = k;
  }
}

// normalise (pf2DRao.cpp:145-148, max-shifted) and resample the tracks (152)
__global__ void __launch_bounds__(1024) rbpf_resample_kernel(const double* logw, int N, uint32_t U,
                                                            double* wn, int* anc, int* status) {
  __shared__ double red[32];
  __shared__ uint64_t red64[34];
  const int tid = threadIdx.x, TB = blockDim.x, lane = tid & 31, w = tid >> 5, nw = TB >> 5;
  double mx = -INFINITY;
  for (int i = tid; i < N; i += TB) mx = fmax(mx, logw[i]);
#pragma unroll
  for (int o = 16; o; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (lane == 0) red[w] = mx;
  __syncthreads();
  mx = lane < nw ? red[lane] : -INFINITY;
#pragma unroll
  for (int o = 16; o; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  __syncthreads();
  const bool fb = !(mx > -INFINITY) || !(mx < INFINITY);
  double s = 0.0;
  if (!fb)
    for (int i = tid; i < N; i += TB) s += exp(logw[i] - mx);
  s = warp_sum_d(s);
  if (lane == 0) red[w] = s;
  __syncthreads();
  if (tid == 0) {
    double t = 0.0;
    for (int q = 0; q < nw; ++q) t += red[q];
    red[0] = t;
  }
  __syncthreads();
  const double sum = red[0];
  double wmax = 0.0;
  for (int i = tid; i < N; i += TB) {
    double v = fb ? 0.0 : exp(logw[i] - mx) / sum;
    if (!(v >= 0.0)) v = 0.0;
    wn[i] = v;
    wmax = fmax(wmax, v);
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) wmax = fmax(wmax, __shfl_xor_sync(0xffffffffu, wmax, o));
  __syncthreads();
  if (lane == 0) red[w] = wmax;
  __syncthreads();
  if (tid == 0) {
    double t = 0.0;
    for (int q = 0; q < nw; ++q) t = fmax(t, red[q]);
    red[0] = t;
  }
  __syncthreads();
  wmax = red[0];
  int e = 0;
  frexp(wmax, &e);
  const int E = (N + TB - 1) / TB;
  const int j0 = min(N, tid * E), j1 = min(N, j0 + E);
  uint64_t cs = 0;
  for (int j = j0; j < j1; ++j) cs += quantize_f64(wn[j], e);
  uint64_t Qt;
  uint64_t P = block_excl_scan_u64(cs, red64, &Qt);
  if (fb || Qt == 0) {
    for (int i = tid; i < N; i += TB) anc[i] = resample_fallback_index(U, i, N);
    if (tid == 0) atomicOr(status, MKF_ST_FALLBACK);
    return;
  }
  scatter_walk(j0, j1, P, N, U, Qt, [&](int j) { return quantize_f64(wn[j], e); }, anc);
}

// tracks[j] = temp[anc[j]] (pf2DRao.cpp:153-156), as independent copies
__global__ void rbpf_gather_kernel(const double* tx, const double* tP, const int* anc, int N, int D,
                                   double* x, double* P) {
  const size_t per = (size_t)D + (size_t)D * D;
  const size_t total = per * N;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
    size_t j = t / per, r = t - j * per;
    int a = anc[j];
    if (r < (size_t)D) x[j * D + r] = tx[(size_t)a * D + r];
    else P[j * D * D + (r - D)] = tP[(size_t)a * D * D + (r - D)];
  }
}

// getEstimator: uniform mean over tracks (pf2DRao.cpp:23-31)
__global__ void __launch_bounds__(256) rbpf_estimate_kernel(const double* x, int N, int D, double* est) {
  __shared__ double red[8];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  for (int r = 0; r < D; ++r) {
    double s = 0.0;
    for (int j = tid; j < N; j += blockDim.x) s += x[(size_t)j * D + r];
    s = warp_sum_d(s);
    if (lane == 0) red[w] = s;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += red[q];
      est[r] = t / (double)N;
    }
    __syncthreads();
  }
}

__global__ void rbpf_reset_kernel(const double* mu, const double* Sigma, const int* bins, int N, int D,
                                  double* x, double* P) {
  const size_t per = (size_t)D + (size_t)D * D;
  const size_t total = per * N;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
    size_t j = t / per, r = t - j * per;
    int k = bins[j];
    if (r < (size_t)D) x[j * D + r] = mu[(size_t)k * D + r];
    else P[j * D * D + (r - D)] = Sigma[(size_t)k * D * D + (r - D)];
  }
}

// ------------------------------------------------------------------ PDAF association
struct PdafArm {
  RbpfParams p;
  const double* x;          // N x d tracks
  double roi[4];
  uint32_t U;
  double* meas;
  int* bins;
  double* w;                // M scratch
  uint64_t p_seed;          // the arm's Philox key
  uint32_t p_track;
};
struct PdafArgs {
  PdafArm arm[2];
  const double* cand;
  int M;
  double Pa, clutter;
};

__device__ void decode_hand(const RbpfParams& p, const double* est, double* hat) {
  const int D = p.d;
  if (p.mode == MKF_MEAS_LINEAR) {
    for (int a = 0; a < 2; ++a) {
      double s = p.hb[a];
      for (int c = 0; c < D; ++c) s += p.Hd[a * D + c] * est[c];
      hat[a] = s;
    }
  } else {
    const double* Bj = p.Bm + (size_t)p.hand_joint * 3 * D;
    double q[3];
    for (int t = 0; t < 3; ++t) {
      double s = p.mm[p.hand_joint * 3 + t];
      for (int c = 0; c < D; ++c) s += Bj[t * D + c] * est[c];
      q[t] = s;
    }
    hat[0] = p.fx * q[0] / q[2] + p.cx;
    hat[1] = p.fy * q[1] / q[2] + p.cy;
  }
}

// both arms' estimates (getEstimator inside getSampleProb, pf2DRao.cpp:111) and
// their decoded hand pixels
__device__ void pdaf_hats(const PdafArm* arm, double (*s_est)[MKF_MAX_D], double (*s_hat)[2], double* red) {
  const int tid = threadIdx.x, TB = blockDim.x, lane = tid & 31, wid = tid >> 5, nw = TB >> 5;
  for (int a = 0; a < 2; ++a) {
    const RbpfParams& p = arm[a].p;
    for (int r = 0; r < p.d; ++r) {
      double s = 0.0;
      for (int j = tid; j < p.N; j += TB) s += arm[a].x[(size_t)j * p.d + r];
      s = warp_sum_d(s);
      if (lane == 0) red[wid] = s;
      __syncthreads();
      if (tid == 0) {
        double t = 0.0;
        for (int q = 0; q < nw; ++q) t += red[q];
        s_est[a][r] = t / (double)p.N;
      }
      __syncthreads();
    }
  }
  if (tid < 2) decode_hand(arm[tid].p, s_est[tid], s_hat[tid]);
  __syncthreads();
}

// weights[j] / sum (pfPose.cpp:294-298), N bins by exact systematic resampling
// of the M candidate weights (the reference's uniform fallback when no weight
// is positive), and the measurement columns [head; candidate; neck]
// (pfPose.cpp:303-323)
__device__ void pdaf_finish(const PdafArm& me, const double* cand, int M, double* red, uint64_t* red64) {
  const int tid = threadIdx.x, TB = blockDim.x, lane = tid & 31, wid = tid >> 5, nw = TB >> 5;
  const int N = me.p.N, m = me.p.m;
  const double* roi = me.roi;
  const double hx = roi[0] + roi[2] / 2.0, hy = roi[1] + 0.5 * roi[3];
  const double nx = roi[0] + roi[2] / 2.0, ny = roi[1] + 1.65 * roi[3];
  double s = 0.0;
  for (int j = tid; j < M; j += TB) s += me.w[j];
  s = warp_sum_d(s);
  if (lane == 0) red[wid] = s;
  __syncthreads();
  if (tid == 0) {
    double t = 0.0;
    for (int q = 0; q < nw; ++q) t += red[q];
    red[0] = t;
  }
  __syncthreads();
  const double sum = red[0];
  __syncthreads();
  double wmax = 0.0;
  int inf = 0;
  for (int j = tid; j < M; j += TB) {
    double v = me.w[j] / sum;
    me.w[j] = v;
    if (isinf(v) && v > 0) inf = 1;
    if (v > 0.0) wmax = fmax(wmax, v);
  }
#pragma unroll
  for (int q = 16; q; q >>= 1) {
    wmax = fmax(wmax, __shfl_xor_sync(0xffffffffu, wmax, q));
    inf |= __shfl_xor_sync(0xffffffffu, inf, q);
  }
  if (lane == 0) red[wid] = inf ? -1.0 : wmax;
  __syncthreads();
  if (tid == 0) {
    double t = 0.0;
    bool bad = false;
    for (int q = 0; q < nw; ++q) { if (red[q] < 0.0) bad = true; else t = fmax(t, red[q]); }
    red[0] = bad ? -1.0 : t;
  }
  __syncthreads();
  wmax = red[0];
  const bool fb = !(wmax > 0.0);
  int e = 0;
  if (!fb) frexp(wmax, &e);
  __syncthreads();
  const int E = (M + TB - 1) / TB;
  const int j0 = min(M, tid * E), j1 = min(M, j0 + E);
  uint64_t cs = 0;
  if (!fb)
    for (int j = j0; j < j1; ++j) cs += quantize_f64(me.w[j], e);
  uint64_t Qt;
  uint64_t P = block_excl_scan_u64(cs, red64, &Qt);
  int* bins = me.bins;
  if (fb || Qt == 0) {
    for (int i = tid; i < N; i += TB) bins[i] = resample_fallback_index(me.U, i, M);
  } else {
    scatter_walk(j0, j1, P, N, me.U, Qt, [&](int j) { return quantize_f64(me.w[j], e); }, bins);
  }
  __syncthreads();
  for (int i = tid; i < N; i += TB) {
    const int bi = bins[i];
    double* z = me.meas + (size_t)i * m;
    z[0] = hx; z[1] = hy;
    z[2] = cand[2 * bi]; z[3] = cand[2 * bi + 1];
    if (m >= 6) { z[4] = nx; z[5] = ny; }
  }
}

__device__ __forceinline__ double gauss2_pdf(double x, double y, const double* hat, double var) {
  const double dx = x - hat[0], dy = y - hat[1];
  return exp(-0.5 * (dx * dx + dy * dy) / var) / (2.0 * 3.14159265358979323846 * var);
}

__global__ void __launch_bounds__(256) pdaf_kernel(PdafArgs A) {
  __shared__ double red[32];
  __shared__ uint64_t red64[34];
  __shared__ double s_est[2][MKF_MAX_D];
  __shared__ double s_hat[2][2];
  const int a = blockIdx.x, o = 1 - a;
  const int tid = threadIdx.x, TB = blockDim.x;
  pdaf_hats(A.arm, s_est, s_hat, red);
  const PdafArm& me = A.arm[a];
  const int N = me.p.N, m = me.p.m, M = A.M;
  const double* roi = me.roi;
  if (M <= 0) {
    const double hx = roi[0] + roi[2] / 2.0, hy = roi[1] + 0.5 * roi[3];
    const double nx = roi[0] + roi[2] / 2.0, ny = roi[1] + 1.65 * roi[3];
    for (int i = tid; i < N; i += TB) {
      double* z = me.meas + (size_t)i * m;
      z[0] = hx; z[1] = hy;
      if (m >= 6) { z[4] = nx; z[5] = ny; }
      if (me.bins) me.bins[i] = -1;
    }
    return;
  }
  const double var = 0.8 * roi[2];               // getSampleProb covariance 0.8 w I
  for (int j = tid; j < M; j += TB) {
    const double cx = A.cand[2 * j], cy = A.cand[2 * j + 1];
    const double po = gauss2_pdf(cx, cy, s_hat[a], var), pt = gauss2_pdf(cx, cy, s_hat[o], var);
    const double Z = po * A.Pa + pt * A.Pa + A.clutter * (1.0 - 2.0 * A.Pa);
    me.w[j] = A.Pa * po / Z;
  }
  __syncthreads();
  pdaf_finish(me, A.cand, M, red, red64);
}

// Likelihood-image proposal (pfPose.cpp:210-301): per arm, M candidates drawn
// uniformly in the box below the face on the first frame after (re)start
// (pfPose.cpp:228-235) or from N(hand, (0.8 w)^2 I) otherwise (getSamples,
// pf2DRao.cpp:85-103), scored by the blurred likelihood L = image / 255 at the
// candidate's pixel over Z = Pa p_own + Pa p_other + clutter (1 - 2 Pa)
// (pfPose.cpp:250-289), then normalised and resampled as above.
struct PdafImageArgs {
  PdafArm arm[2];
  double* cand[2];          // M x 2 per arm (device, written)
  const uint8_t* img;
  int width, height, pitch, M, init;
  double Pa, clutter;
  uint32_t frame;
};
constexpr uint32_t kStreamPropose = 0x104u;

__global__ void __launch_bounds__(256) pdaf_image_kernel(PdafImageArgs A) {
  __shared__ double red[32];
  __shared__ uint64_t red64[34];
  __shared__ double s_est[2][MKF_MAX_D];
  __shared__ double s_hat[2][2];
  const int a = blockIdx.x, o = 1 - a;
  const int tid = threadIdx.x, TB = blockDim.x;
  pdaf_hats(A.arm, s_est, s_hat, red);
  const PdafArm& me = A.arm[a];
  const double* roi = me.roi;
  const double var = 0.8 * roi[2];
  const double sd = 0.8 * roi[2];                // randn with the matrix 0.8 w I as its "stddev"
  const int xo = (int)roi[0], yo = (int)roi[1], wi = (int)roi[2], hi = (int)roi[3];
  const int xmin = max(xo - 4 * wi, 0), xmax = min(xo + 5 * wi, A.width);
  const int ymin = min(yo + hi, A.height), ymax = min(yo + 7 * hi, A.height);
  double* cand = A.cand[a];
  for (int j = tid; j < A.M; j += TB) {
    const u32x4 w = draw_block(me.p_seed, me.p_track, A.frame, (uint32_t)j, kStreamPropose);
    double cx, cy;
    if (A.init) {
      cx = xmin + (double)w.x * (1.0 / 4294967296.0) * (double)(xmax - xmin);
      cy = ymin + (double)w.y * (1.0 / 4294967296.0) * (double)(ymax - ymin);
    } else {
      float n0, n1;
      box_muller(w.x, w.y, n0, n1);
      cx = s_hat[a][0] + sd * (double)n0;
      cy = s_hat[a][1] + sd * (double)n1;
    }
    cand[2 * j] = cx;
    cand[2 * j + 1] = cy;
    double wt = 0.0;
    if (cy > 0.0 && cy < A.height && cx > 0.0 && cx < A.width) {
      const double L = (double)A.img[(size_t)(int)cy * A.pitch + (int)cx] / 255.0;
      if (L != 0.0) {
        const double po = gauss2_pdf(cx, cy, s_hat[a], var), pt = gauss2_pdf(cx, cy, s_hat[o], var);
        wt = L / (po * A.Pa + pt * A.Pa + A.clutter * (1.0 - 2.0 * A.Pa));
      }
    }
    me.w[j] = wt;
  }
  __syncthreads();
  pdaf_finish(me, cand, A.M, red, red64);
}

// GaussianBlur(likelihood, 15x15, sigma 3, BORDER_DEFAULT) (pfPose.cpp:213) as a
// separable float filter: each pass is the fmaf chain over the 15 taps in tap
// order, the border reflects without repeating the edge pixel, and the result
// is rounded to nearest-even and saturated to 8 bits.
constexpr int kBlurR = 7, kBlurTile = 32;
struct BlurArgs {
  const uint8_t* in;
  uint8_t* out;
  int width, height, pitch_in, pitch_out;
  float w[2 * kBlurR + 1];
};
// reflect-101 index for any i (n >= 2): fold with period 2n - 2.  The staged
// tile reaches up to T + R - 1 past its origin, beyond one reflection when the
// image is narrower than a tile; those positions feed no output pixel, but
// they must still be addresses inside the image.
__device__ __forceinline__ int reflect101(int i, int n) {
  const int p = 2 * n - 2;
  i %= p;
  if (i < 0) i += p;
  if (i >= n) i = p - i;
  return i;
}
__global__ void __launch_bounds__(256) blur_kernel(BlurArgs A) {
  constexpr int T = kBlurTile, R = kBlurR, S = T + 2 * R;
  __shared__ float s_in[S][S + 1];
  __shared__ float s_h[S][T + 1];
  const int x0 = blockIdx.x * T, y0 = blockIdx.y * T;
  const int tid = threadIdx.y * blockDim.x + threadIdx.x, nt = blockDim.x * blockDim.y;
  for (int q = tid; q < S * S; q += nt) {
    const int r = q / S, c = q - r * S;
    const int y = reflect101(y0 + r - R, A.height), x = reflect101(x0 + c - R, A.width);
    s_in[r][c] = (float)A.in[(size_t)y * A.pitch_in + x];
  }
  __syncthreads();
  for (int q = tid; q < S * T; q += nt) {          // horizontal pass over every staged row
    const int r = q / T, c = q - r * T;
    float acc = 0.0f;
#pragma unroll
    for (int k = 0; k < 2 * R + 1; ++k) acc = fmaf(A.w[k], s_in[r][c + k], acc);
    s_h[r][c] = acc;
  }
  __syncthreads();
  for (int q = tid; q < T * T; q += nt) {          // vertical pass
    const int r = q / T, c = q - r * T;
    const int y = y0 + r, x = x0 + c;
    if (y >= A.height || x >= A.width) continue;
    float acc = 0.0f;
#pragma unroll
    for (int k = 0; k < 2 * R + 1; ++k) acc = fmaf(A.w[k], s_h[r + k][c], acc);
    const float v = fminf(fmaxf(rintf(acc), 0.0f), 255.0f);
    A.out[(size_t)y * A.pitch_out + x] = (uint8_t)v;
  }
}

}  // namespace mkf

using namespace mkf;

struct mkf_rbpf {
  int d, m, K, N, mode;
  uint64_t seed;
  uint32_t track;
  std::vector<double> f, B, Q, H, BH, R, w, mu, Sigma, Bm, mm, Hd, hb;
  double fx, fy, cx, cy;
  int hand_joint;
  bool dirty, ready;
  double *d_f, *d_B, *d_Q, *d_H, *d_BH, *d_R, *d_w, *d_mu, *d_Sigma, *d_Bm, *d_mm, *d_Hd, *d_hb;
  double *x, *P, *tx, *tP, *logw, *wn, *pw, *pc;
  int *ind, *anc, *bins, *status;
  int pw_cap, pc_cap;
};

// per-arm candidate-weight (M) and candidate (2 M) scratch
static int rbpf_pdaf_scratch(mkf_rbpf* h, int M, bool cand) {
  M = std::max(M, 1);
  if (h->pw_cap < M) {
    if (h->pw) cudaFree(h->pw);
    h->pw = nullptr;
    h->pw_cap = 0;
    MKF_CUDA(cudaMalloc(&h->pw, sizeof(double) * M));
    h->pw_cap = M;
  }
  if (cand && h->pc_cap < M) {
    if (h->pc) cudaFree(h->pc);
    h->pc = nullptr;
    h->pc_cap = 0;
    MKF_CUDA(cudaMalloc(&h->pc, sizeof(double) * 2 * (size_t)M));
    h->pc_cap = M;
  }
  return MKF_OK;
}

static void rbpf_free_params(mkf_rbpf* h) {
  double* ps[] = {h->d_f, h->d_B, h->d_Q, h->d_H, h->d_BH, h->d_R, h->d_w, h->d_mu, h->d_Sigma,
                  h->d_Bm, h->d_mm, h->d_Hd, h->d_hb};
  for (double* p : ps) if (p) cudaFree(p);
  h->d_f = h->d_B = h->d_Q = h->d_H = h->d_BH = h->d_R = h->d_w = h->d_mu = h->d_Sigma = nullptr;
  h->d_Bm = h->d_mm = h->d_Hd = h->d_hb = nullptr;
}

static int up(double** dst, const std::vector<double>& v) {
  MKF_CUDA(cudaMalloc(dst, std::max<size_t>(1, v.size()) * sizeof(double)));
  if (!v.empty()) MKF_CUDA(cudaMemcpy(*dst, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice));
  return MKF_OK;
}

static int rbpf_sync_params(mkf_rbpf* h) {
  if (!h->dirty) return MKF_OK;
  rbpf_free_params(h);
  int st;
  if ((st = up(&h->d_f, h->f)) || (st = up(&h->d_B, h->B)) || (st = up(&h->d_Q, h->Q)) ||
      (st = up(&h->d_H, h->H)) || (st = up(&h->d_BH, h->BH)) || (st = up(&h->d_R, h->R)) ||
      (st = up(&h->d_w, h->w)) || (st = up(&h->d_mu, h->mu)) || (st = up(&h->d_Sigma, h->Sigma)) ||
      (st = up(&h->d_Bm, h->Bm)) || (st = up(&h->d_mm, h->mm)) || (st = up(&h->d_Hd, h->Hd)) ||
      (st = up(&h->d_hb, h->hb)))
    return st;
  h->dirty = false;
  return MKF_OK;
}

static RbpfParams rbpf_params(const mkf_rbpf* h) {
  RbpfParams p;
  p.f = h->d_f; p.B = h->d_B; p.Q = h->d_Q; p.H = h->d_H; p.BH = h->d_BH; p.R = h->d_R; p.w = h->d_w;
  p.mu = h->d_mu; p.Sigma = h->d_Sigma; p.Bm = h->d_Bm; p.mm = h->d_mm; p.Hd = h->d_Hd; p.hb = h->d_hb;
  p.fx = h->fx; p.fy = h->fy; p.cx = h->cx; p.cy = h->cy;
  p.d = h->d; p.m = h->m; p.K = h->K; p.N = h->N; p.mode = h->mode; p.hand_joint = h->hand_joint;
  return p;
}

extern "C" int mkf_rbpf_create(int d, int m, int K, int n_particles, int meas_mode, uint64_t seed,
                               uint32_t track_id, mkf_rbpf_t* out) {
  MKF_ARG(out, "mkf_rbpf_create: null output");
  MKF_ARG(d == 12 || d == 24, "mkf_rbpf_create: d must be 12 or 24");
  MKF_ARG(m >= 1 && m <= kMMax, "mkf_rbpf_create: m out of range");
  MKF_ARG(K >= 1 && K <= MKF_MAX_K, "mkf_rbpf_create: K out of range");
  MKF_ARG(n_particles >= 1 && n_particles <= 65536, "mkf_rbpf_create: n_particles out of range");
  MKF_ARG(meas_mode == MKF_MEAS_LINEAR || meas_mode == MKF_MEAS_PINHOLE, "mkf_rbpf_create: bad meas_mode");
  MKF_ARG(meas_mode == MKF_MEAS_LINEAR || (m % 2 == 0 && m / 2 <= MKF_MAX_J), "mkf_rbpf_create: pinhole needs even m");
  mkf_rbpf* h = new (std::nothrow) mkf_rbpf();
  if (!h) return MKF_ERR_NOMEM;
  h->d = d; h->m = m; h->K = K; h->N = n_particles; h->mode = meas_mode; h->seed = seed; h->track = track_id;
  h->f.assign((size_t)K * d, 0.0); h->B.assign((size_t)K * d, 0.0); h->Q.assign((size_t)K * d * d, 0.0);
  h->H.assign((size_t)K * m * d, 0.0); h->BH.assign((size_t)K * m, 0.0); h->R.assign((size_t)K * m * m, 0.0);
  h->w.assign(K, 0.0); h->mu.assign((size_t)K * d, 0.0); h->Sigma.assign((size_t)K * d * d, 0.0);
  h->Bm.assign((size_t)(m / 2 > 0 ? m / 2 : 1) * 3 * d, 0.0); h->mm.assign((size_t)(m / 2 > 0 ? m / 2 : 1) * 3, 0.0);
  h->Hd.assign((size_t)2 * d, 0.0); h->hb.assign(2, 0.0);
  h->fx = 525.0; h->fy = 525.0; h->cx = 319.5; h->cy = 239.5;
  h->hand_joint = 1;
  h->dirty = true;
  const size_t N = n_particles;
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = cudaMalloc(&h->x, N * d * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&h->P, N * d * d * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&h->tx, N * d * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&h->tP, N * d * d * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&h->logw, N * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&h->wn, N * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&h->ind, N * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&h->anc, N * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&h->bins, N * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&h->status, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(h->status, 0, sizeof(int));
  if (e != cudaSuccess) {
    mkf_rbpf_destroy(h);
    return cuda_fail(e, "mkf_rbpf_create: allocation", __FILE__, __LINE__);
  }
  *out = h;
  return MKF_OK;
}

extern "C" int mkf_rbpf_load_gaussian(mkf_rbpf_t h, int k, const double* u, const double* s,
                                      const double* Hpca, const double* mpca, int F, double w, double g) {
  MKF_ARG(h && u && s && Hpca && mpca, "mkf_rbpf_load_gaussian: null argument");
  MKF_ARG(k >= 0 && k < h->K, "mkf_rbpf_load_gaussian: component index out of range");
  MKF_ARG(h->m == 6 && h->mode == MKF_MEAS_LINEAR, "mkf_rbpf_load_gaussian: reference form needs m == 6, LINEAR");
  static const int sel[6] = {9, 10, 0, 1, 12, 13};     // H1 selector, my_gmm.cpp:59-67
  MKF_ARG(F > 13, "mkf_rbpf_load_gaussian: full-state dimension too small for the H1 selector");
  const int d = h->d;
  for (int r = 0; r < d; ++r) {
    h->f[(size_t)k * d + r] = g;                      // F = g I
    h->B[(size_t)k * d + r] = (1.0 - g) * u[r];       // B = (1 - g) u^T
    h->mu[(size_t)k * d + r] = u[r];
    for (int c = 0; c < d; ++c) {
      h->Q[((size_t)k * d + r) * d + c] = (1.0 - g * g) * s[r * d + c];   // Q = (1 - g^2) s
      h->Sigma[((size_t)k * d + r) * d + c] = s[r * d + c];
    }
  }
  for (int a = 0; a < 6; ++a) {
    for (int c = 0; c < d; ++c) h->H[((size_t)k * 6 + a) * d + c] = Hpca[(size_t)c * F + sel[a]];
    h->BH[(size_t)k * 6 + a] = mpca[sel[a]];
    for (int b = 0; b < 6; ++b) h->R[((size_t)k * 6 + a) * 6 + b] = (a == b) ? 100.0 : 0.0;
  }
  h->w[k] = w;
  h->dirty = true;
  return MKF_OK;
}

extern "C" int mkf_rbpf_set_component(mkf_rbpf_t h, int k, const double* mu, const double* a, const double* Q,
                                      const double* Sigma, const double* R, double w, const double* H,
                                      const double* BH) {
  MKF_ARG(h && mu && a && Q && Sigma && R, "mkf_rbpf_set_component: null argument");
  MKF_ARG(k >= 0 && k < h->K, "mkf_rbpf_set_component: component index out of range");
  MKF_ARG(h->mode == MKF_MEAS_PINHOLE || (H && BH), "mkf_rbpf_set_component: LINEAR needs H and BH");
  const int d = h->d, m = h->m;
  for (int r = 0; r < d; ++r) {
    h->f[(size_t)k * d + r] = a[r];
    h->B[(size_t)k * d + r] = (1.0 - a[r]) * mu[r];
    h->mu[(size_t)k * d + r] = mu[r];
  }
  memcpy(&h->Q[(size_t)k * d * d], Q, sizeof(double) * d * d);
  memcpy(&h->Sigma[(size_t)k * d * d], Sigma, sizeof(double) * d * d);
  memcpy(&h->R[(size_t)k * m * m], R, sizeof(double) * m * m);
  if (H) memcpy(&h->H[(size_t)k * m * d], H, sizeof(double) * m * d);
  if (BH) memcpy(&h->BH[(size_t)k * m], BH, sizeof(double) * m);
  h->w[k] = w;
  h->dirty = true;
  return MKF_OK;
}

extern "C" int mkf_rbpf_set_pinhole(mkf_rbpf_t h, const double* Bm, const double* mm, double fx, double fy,
                                    double cx, double cy) {
  MKF_ARG(h && Bm && mm, "mkf_rbpf_set_pinhole: null argument");
  MKF_ARG(h->mode == MKF_MEAS_PINHOLE, "mkf_rbpf_set_pinhole: filter is not PINHOLE");
  const int J = h->m / 2;
  memcpy(h->Bm.data(), Bm, sizeof(double) * J * 3 * h->d);
  memcpy(h->mm.data(), mm, sizeof(double) * J * 3);
  h->fx = fx; h->fy = fy; h->cx = cx; h->cy = cy;
  h->dirty = true;
  return MKF_OK;
}

extern "C" int mkf_rbpf_set_hand_decode(mkf_rbpf_t h, const double* Hd, const double* hb, int joint) {
  MKF_ARG(h, "mkf_rbpf_set_hand_decode: null handle");
  if (h->mode == MKF_MEAS_LINEAR) {
    MKF_ARG(Hd && hb, "mkf_rbpf_set_hand_decode: LINEAR needs Hd and hb");
    memcpy(h->Hd.data(), Hd, sizeof(double) * 2 * h->d);
    memcpy(h->hb.data(), hb, sizeof(double) * 2);
  } else {
    MKF_ARG(joint >= 0 && joint < h->m / 2, "mkf_rbpf_set_hand_decode: joint out of range");
    h->hand_joint = joint;
  }
  h->dirty = true;
  return MKF_OK;
}

extern "C" int mkf_rbpf_reset(mkf_rbpf_t h, const int* bins, mkf_stream_t stream) {
  MKF_RANGE("mkf_rbpf_reset");
  MKF_ARG(h, "mkf_rbpf_reset: null handle");
  cudaStream_t s = (cudaStream_t)stream;
  int st = rbpf_sync_params(h);
  if (st) return st;
  if (bins) {
    for (int i = 0; i < h->N; ++i)
      MKF_ARG(bins[i] >= 0 && bins[i] < h->K, "mkf_rbpf_reset: bin out of range");
    MKF_CUDA(cudaMemcpyAsync(h->bins, bins, sizeof(int) * h->N, cudaMemcpyHostToDevice, s));
  } else {
    const uint32_t U = draw_block(h->seed, h->track, kFramePrior, kItemFrame, kStreamIndicator).x;
    st = mkf_resample_f64(h->d_w, h->K, h->N, U, h->bins, nullptr, stream);
    if (st) return st;
  }
  const size_t total = (size_t)h->N * (h->d + h->d * h->d);
  int g = (int)std::min<size_t>((total + 255) / 256, 4096);
  rbpf_reset_kernel<<<g, 256, 0, s>>>(h->d_mu, h->d_Sigma, h->bins, h->N, h->d, h->x, h->P);
  MKF_CHECK_LAUNCH("mkf_rbpf_reset");
  MKF_CUDA(cudaMemsetAsync(h->status, 0, sizeof(int), s));
  MKF_CUDA(cudaStreamSynchronize(s));
  h->ready = true;
  return MKF_OK;
}

extern "C" int mkf_rbpf_update_u(mkf_rbpf_t h, const double* d_meas, unsigned mask, uint32_t U_ind,
                                 uint32_t U_anc, mkf_stream_t stream) {
  MKF_RANGE("mkf_rbpf_update_u");
  MKF_ARG(h && d_meas, "mkf_rbpf_update: null argument");
  if (!h->ready) { set_error("mkf_rbpf_update: call mkf_rbpf_reset first"); return MKF_ERR_STATE; }
  int st = rbpf_sync_params(h);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  RbpfStepArgs a;
  a.p = rbpf_params(h);
  a.x = h->x; a.P = h->P; a.z = d_meas;
  a.mask = mask & ((1u << h->m) - 1u);
  a.U_ind = U_ind;
  a.tx = h->tx; a.tP = h->tP; a.logw = h->logw; a.ind = h->ind; a.status = h->status;
  const int wpb = 4;
  const size_t smem = (size_t)wpb * rbpf_warp_doubles(h->d) * sizeof(double);
  const int grid = (h->N + wpb - 1) / wpb;
  if (h->d == 12) {
    MKF_CUDA(cudaFuncSetAttribute(rbpf_step_kernel<12>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    rbpf_step_kernel<12><<<grid, 32 * wpb, smem, s>>>(a);
  } else {
    MKF_CUDA(cudaFuncSetAttribute(rbpf_step_kernel<24>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    rbpf_step_kernel<24><<<grid, 32 * wpb, smem, s>>>(a);
  }
  MKF_CHECK_LAUNCH("mkf_rbpf_update: step kernel");
  rbpf_resample_kernel<<<1, 1024, 0, s>>>(h->logw, h->N, U_anc, h->wn, h->anc, h->status);
  MKF_CHECK_LAUNCH("mkf_rbpf_update: resample kernel");
  const size_t total = (size_t)h->N * (h->d + h->d * h->d);
  int g = (int)std::min<size_t>((total + 255) / 256, 8192);
  rbpf_gather_kernel<<<g, 256, 0, s>>>(h->tx, h->tP, h->anc, h->N, h->d, h->x, h->P);
  MKF_CHECK_LAUNCH("mkf_rbpf_update: gather kernel");
  return MKF_OK;
}

extern "C" int mkf_rbpf_update(mkf_rbpf_t h, uint32_t frame, const double* d_meas, unsigned mask,
                               mkf_stream_t stream) {
  MKF_RANGE("mkf_rbpf_update");
  MKF_ARG(h, "mkf_rbpf_update: null handle");
  const uint32_t U_ind = draw_block(h->seed, h->track, frame, kItemFrame, kStreamIndicator).x;
  const uint32_t U_anc = resample_uniform(h->seed, h->track, frame);
  return mkf_rbpf_update_u(h, d_meas, mask, U_ind, U_anc, stream);
}

extern "C" int mkf_rbpf_estimate(mkf_rbpf_t h, double* d_est, mkf_stream_t stream) {
  MKF_RANGE("mkf_rbpf_estimate");
  MKF_ARG(h && d_est, "mkf_rbpf_estimate: null argument");
  rbpf_estimate_kernel<<<1, 256, 0, (cudaStream_t)stream>>>(h->x, h->N, h->d, d_est);
  MKF_CHECK_LAUNCH("mkf_rbpf_estimate");
  return MKF_OK;
}

extern "C" int mkf_rbpf_read(mkf_rbpf_t h, double* d_x, double* d_P, double* d_logw, double* d_wn, int* d_ind,
                             int* d_anc, mkf_stream_t stream) {
  MKF_ARG(h, "mkf_rbpf_read: null handle");
  cudaStream_t s = (cudaStream_t)stream;
  const size_t N = h->N, d = h->d;
  if (d_x) MKF_CUDA(cudaMemcpyAsync(d_x, h->x, N * d * sizeof(double), cudaMemcpyDeviceToDevice, s));
  if (d_P) MKF_CUDA(cudaMemcpyAsync(d_P, h->P, N * d * d * sizeof(double), cudaMemcpyDeviceToDevice, s));
  if (d_logw) MKF_CUDA(cudaMemcpyAsync(d_logw, h->logw, N * sizeof(double), cudaMemcpyDeviceToDevice, s));
  if (d_wn) MKF_CUDA(cudaMemcpyAsync(d_wn, h->wn, N * sizeof(double), cudaMemcpyDeviceToDevice, s));
  if (d_ind) MKF_CUDA(cudaMemcpyAsync(d_ind, h->ind, N * sizeof(int), cudaMemcpyDeviceToDevice, s));
  if (d_anc) MKF_CUDA(cudaMemcpyAsync(d_anc, h->anc, N * sizeof(int), cudaMemcpyDeviceToDevice, s));
  return MKF_OK;
}

extern "C" int mkf_rbpf_write(mkf_rbpf_t h, const double* d_x, const double* d_P, mkf_stream_t stream) {
  MKF_ARG(h && d_x && d_P, "mkf_rbpf_write: null argument");
  cudaStream_t s = (cudaStream_t)stream;
  int st = rbpf_sync_params(h);
  if (st) return st;
  const size_t N = h->N, d = h->d;
  MKF_CUDA(cudaMemcpyAsync(h->x, d_x, N * d * sizeof(double), cudaMemcpyDeviceToDevice, s));
  MKF_CUDA(cudaMemcpyAsync(h->P, d_P, N * d * d * sizeof(double), cudaMemcpyDeviceToDevice, s));
  h->ready = true;
  return MKF_OK;
}

extern "C" int mkf_rbpf_status(mkf_rbpf_t h, int* status) {
  MKF_ARG(h && status, "mkf_rbpf_status: null argument");
  MKF_CUDA(cudaMemcpy(status, h->status, sizeof(int), cudaMemcpyDeviceToHost));
  return MKF_OK;
}

extern "C" int mkf_rbpf_destroy(mkf_rbpf_t h) {
  if (!h) return MKF_OK;
  rbpf_free_params(h);
  void* ps[] = {h->x, h->P, h->tx, h->tP, h->logw, h->wn, h->pw, h->pc, h->ind, h->anc, h->bins, h->status};
  for (void* p : ps) if (p) cudaFree(p);
  delete h;
  return MKF_OK;
}

extern "C" int mkf_pdaf_associate(mkf_rbpf_t arm0, mkf_rbpf_t arm1, uint32_t frame, const double* roi,
                                  const double* d_cand, int M, double Pa, double clutter, double* d_meas0,
                                  double* d_meas1, int* d_bins0, int* d_bins1, mkf_stream_t stream) {
  MKF_RANGE("mkf_pdaf_associate");
  MKF_ARG(arm0 && arm1 && roi && d_meas0 && d_meas1, "mkf_pdaf_associate: null argument");
  MKF_ARG(M >= 0 && M <= 65536 && (M == 0 || d_cand), "mkf_pdaf_associate: bad candidate list");
  MKF_ARG(arm0->m >= 4 && arm1->m >= 4, "mkf_pdaf_associate: measurement needs head and hand rows");
  MKF_ARG(roi[2] > 0.0 && roi[6] > 0.0, "mkf_pdaf_associate: ROI width must be positive");
  cudaStream_t s = (cudaStream_t)stream;
  mkf_rbpf_t arms[2] = {arm0, arm1};
  double* meas[2] = {d_meas0, d_meas1};
  int* bins[2] = {d_bins0, d_bins1};
  PdafArgs a;
  memset(&a, 0, sizeof(a));
  for (int i = 0; i < 2; ++i) {
    mkf_rbpf_t h = arms[i];
    int st = rbpf_sync_params(h);
    if (st) return st;
    if ((st = rbpf_pdaf_scratch(h, M, false))) return st;
    a.arm[i].p = rbpf_params(h);
    a.arm[i].p_seed = h->seed; a.arm[i].p_track = h->track;
    a.arm[i].x = h->x;
    for (int q = 0; q < 4; ++q) a.arm[i].roi[q] = roi[4 * i + q];
    a.arm[i].U = draw_block(h->seed, h->track, frame, kItemFrame, kStreamPdaf).x;
    a.arm[i].meas = meas[i];
    a.arm[i].bins = bins[i] ? bins[i] : h->bins;
    a.arm[i].w = h->pw;
  }
  a.cand = d_cand; a.M = M; a.Pa = Pa; a.clutter = clutter;
  pdaf_kernel<<<2, 256, 0, s>>>(a);
  MKF_CHECK_LAUNCH("mkf_pdaf_associate");
  return MKF_OK;
}

extern "C" int mkf_pdaf_propose_image(mkf_rbpf_t arm0, mkf_rbpf_t arm1, uint32_t frame, const double* roi,
                                      const uint8_t* d_like, int width, int height, int pitch, int M, int init,
                                      double Pa, double clutter, double* d_meas0, double* d_meas1, int* d_bins0,
                                      int* d_bins1, double* d_cand0, double* d_cand1, mkf_stream_t stream) {
  MKF_RANGE("mkf_pdaf_propose_image");
  MKF_ARG(arm0 && arm1 && roi && d_like && d_meas0 && d_meas1, "mkf_pdaf_propose_image: null argument");
  MKF_ARG(width >= 1 && height >= 1 && pitch >= width, "mkf_pdaf_propose_image: bad image size");
  MKF_ARG(M >= 1 && M <= (1 << 20), "mkf_pdaf_propose_image: M must be in [1, 1048576]");
  MKF_ARG(arm0->m >= 4 && arm1->m >= 4, "mkf_pdaf_propose_image: measurement needs head and hand rows");
  MKF_ARG(roi[2] > 0.0 && roi[6] > 0.0, "mkf_pdaf_propose_image: ROI width must be positive");
  cudaStream_t s = (cudaStream_t)stream;
  mkf_rbpf_t arms[2] = {arm0, arm1};
  double* meas[2] = {d_meas0, d_meas1};
  int* bins[2] = {d_bins0, d_bins1};
  double* cands[2] = {d_cand0, d_cand1};
  PdafImageArgs a;
  memset(&a, 0, sizeof(a));
  for (int i = 0; i < 2; ++i) {
    mkf_rbpf_t h = arms[i];
    int st = rbpf_sync_params(h);
    if (st) return st;
    if ((st = rbpf_pdaf_scratch(h, M, cands[i] == nullptr))) return st;
    a.arm[i].p = rbpf_params(h);
    a.arm[i].p_seed = h->seed; a.arm[i].p_track = h->track;
    a.arm[i].x = h->x;
    for (int q = 0; q < 4; ++q) a.arm[i].roi[q] = roi[4 * i + q];
    a.arm[i].U = draw_block(h->seed, h->track, frame, kItemFrame, kStreamPdaf).x;
    a.arm[i].meas = meas[i];
    a.arm[i].bins = bins[i] ? bins[i] : h->bins;
    a.arm[i].w = h->pw;
    a.cand[i] = cands[i] ? cands[i] : h->pc;
  }
  a.img = d_like; a.width = width; a.height = height; a.pitch = pitch; a.M = M; a.init = init ? 1 : 0;
  a.Pa = Pa; a.clutter = clutter; a.frame = frame;
  pdaf_image_kernel<<<2, 256, 0, s>>>(a);
  MKF_CHECK_LAUNCH("mkf_pdaf_propose_image");
  return MKF_OK;
}

extern "C" int mkf_likelihood_blur(const uint8_t* d_in, int width, int height, int pitch_in, uint8_t* d_out,
                                   int pitch_out, mkf_stream_t stream) {
  MKF_RANGE("mkf_likelihood_blur");
  MKF_ARG(d_in && d_out && d_in != d_out, "mkf_likelihood_blur: null or aliased buffers");
  MKF_ARG(width >= 8 && height >= 8 && pitch_in >= width && pitch_out >= width,
          "mkf_likelihood_blur: image must be at least 8 x 8 with pitches >= width");
  BlurArgs a;
  a.in = d_in; a.out = d_out; a.width = width; a.height = height; a.pitch_in = pitch_in; a.pitch_out = pitch_out;
  double e[2 * kBlurR + 1], sum = 0.0;
  for (int k = 0; k <= 2 * kBlurR; ++k) {
    const double x = (double)(k - kBlurR);
    e[k] = std::exp(-x * x / (2.0 * 3.0 * 3.0));
    sum += e[k];
  }
  for (int k = 0; k <= 2 * kBlurR; ++k) a.w[k] = (float)(e[k] / sum);
  dim3 grid((width + kBlurTile - 1) / kBlurTile, (height + kBlurTile - 1) / kBlurTile), block(32, 8);
  blur_kernel<<<grid, block, 0, (cudaStream_t)stream>>>(a);
  MKF_CHECK_LAUNCH("mkf_likelihood_blur");
  return MKF_OK;
}
