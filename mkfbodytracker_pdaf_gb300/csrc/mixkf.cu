// mixkf.cu -- mixture Kalman filter (GPB1 over the GMM components) with PDAF
// association, its log marginal likelihood, and the hand-written adjoint with
// sqrt(T) checkpointing.
//
// Reference pieces: KF_model::predict/update (KF_model.cpp:11-25), the motion
// model of my_gmm::loadGaussian (my_gmm.cpp:45-75) generalised to
// A_k = diag(a_k), Q_k = Lq_k Lq_k^T, the mixture over components that
// pf2DRao redraws every frame (pf2DRao.cpp:128), and the PDA association
// weights of pfPose.cpp:247-298.
//
// Launch shape: one CTA per track (static round-robin over a persistent grid,
// so every reduction has a fixed order), one lane group per mixture component:
// half a warp at d = 12, a whole warp at d = 24.  A group's
// predict/update/reverse runs lane-parallel over matrix entries; the
// collapse and its reverse are CTA-wide.  Each group's forward scratch (its
// component state and the joint update being formed) is in shared memory; the
// per-frame joint records of a backward segment are in the CTA's global slot
// (sized to stay L2-resident); the per-component adjoint work blocks are in
// shared memory when they fit (STAGE), else in the slot; the collapsed state
// and its adjoint are in shared memory.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "mkf_common.cuh"

namespace mkf {

constexpr int kMixMaxC = MKF_MAX_DET;
constexpr float kMixZMin = 0.05f;

// joint record layout (floats): the 2x2 matrices S, S^-1 and M and the
// scalar groups (VIS, N, B0, ELL) and (NB, IZ, LD) each on a 16-byte boundary,
// so that the reverse reads each with one 16-byte load; float 23 is padding;
// H, U, Kg and W start on a 16-byte boundary
enum {
  R_S = 0, R_SI = 4, R_M = 8, R_VIS = 12, R_N = 13, R_B0 = 14, R_ELL = 15, R_NB = 16, R_IZ = 18, R_LD = 19,
  R_P3 = 20, R_JP = 24, R_ZH = 30, R_NU = 32, R_E = 64, R_BETA = 80, R_H = 96
};
// A record ends at rec_X: it does not keep the covariance entering the update.
// The reverse sweep rebuilds it in the group's scratch (rec_X .. rec_Pin + d^2
// there) from the component's final covariance and the records' gains,
// P_in = P_out + W Kg^T joint by joint backwards: a record is 192 floats
// instead of 348 at d = 12 (288 instead of 888 at d = 24), so that more frames
// of every resident CTA's records fit in L2
__host__ __device__ inline int rec_size(int d) { return (R_H + 8 * d + 3) & ~3; }
__host__ __device__ inline int rec_U(int d) { return R_H + 2 * d; }
__host__ __device__ inline int rec_Kg(int d) { return R_H + 4 * d; }
__host__ __device__ inline int rec_W(int d) { return R_H + 6 * d; }
__host__ __device__ inline int rec_X(int d) { return R_H + 8 * d; }
__host__ __device__ inline int rec_Pin(int d) { return R_H + 9 * d; }

// Per-frame record block (floats): for each component its joint records, its
// updated state (xk, Pk); then the frame's input state, mixture weights and
// collapsed mean.  A backward segment keeps one block per frame.
struct FrameLayout {
  int comp_size, comp_xk, comp_Pk, xin, Pin, w, xo, size;
};
__host__ __device__ inline FrameLayout frame_layout(int d, int K, int J) {
  FrameLayout L;
  L.comp_xk = J * rec_size(d);
  L.comp_Pk = L.comp_xk + d;
  L.comp_size = (L.comp_Pk + d * d + 3) & ~3;
  int o = K * L.comp_size;
  L.xin = o; o += d; L.Pin = o; o += d * d;
  L.w = o; o += 32; L.xo = o; o += d;
  L.size = (o + 31) & ~31;
  return L;
}
// Per-component adjoint work block (floats).  gmu, ga and Sq accumulate over
// one backward segment: the mu and a adjoints, and Sq = the sum of the frames'
// adjoints of the predicted covariance, from which the L_Q adjoint of the
// segment is formed once (L_Q is the same in every frame).
struct WorkLayout {
  int xb, Pb, Xin, Pin, Dkb, tmp, gmu, ga, Sq, size;
};
__host__ __device__ inline WorkLayout work_layout(int d) {
  WorkLayout L;
  int o = 0;
  L.xb = o; o += d; L.Pb = o; o += d * d;
  L.Xin = o; o += d; L.Pin = o; o += d * d;
  L.Dkb = o; o += d;
  L.tmp = o; o += 8 * d;
  L.gmu = o; o += d; L.ga = o; o += d; L.Sq = o; o += d * d;
  L.size = (o + 3) & ~3;
  return L;
}

struct MixDev {
  int d, K, J, DD;
  const float *mu, *a, *Lq, *Q, *logpi, *pi, *S0;
  float sigma, fx, fy, cx, cy;
};

struct MixArgs {
  MixDev M;
  int n_tracks, C;
  const int* n_frames;
  const long long* frame_base;
  const float* Bm;
  const float* mm;
  const float* pd;
  const float* kappa;
  const int* det_off;
  const float2* det;
  const long long* ck_off;     // per track offset (floats) into ck
  float* ck;
  double* ll;                  // per track logL
  float* slots;                // gridDim.x * slot_floats
  long long slot_floats;
  double* gacc;                // gridDim.x * ng (backward)
  int ng;
  int* status;
};

// Lanes per mixture component: half a warp (two components per warp) when a
// component's d-wide work fits in 16 lanes, else the whole warp.  The d-wide
// phases, scalar steps and reductions of the per-component Kalman algebra then
// cost half the warp instructions at d = 12.
template <int D>
__host__ __device__ constexpr int lpc_of() { return D <= 16 ? 16 : 32; }

// The lanes of one component: LPC consecutive lanes of a warp
template <int LPC>
struct Grp {
  int sub;         // lane within the group
  unsigned mask;   // the group's lanes
  __device__ __forceinline__ explicit Grp(int tid)
      : sub(tid & (LPC - 1)), mask(LPC == 32 ? 0xffffffffu : (0xffffu << (tid & 16))) {}
  __device__ __forceinline__ void sync() const { __syncwarp(mask); }
  __device__ __forceinline__ float bcast(float v, int src) const { return __shfl_sync(mask, v, src, LPC); }
  __device__ __forceinline__ float sum(float v) const {
#pragma unroll
    for (int o = LPC / 2; o; o >>= 1) v += __shfl_xor_sync(mask, v, o, LPC);
    return v;
  }
};

// N group sums at once (N = 2, 4 or 8), every lane of the group getting all N
// totals.  Recursive halving: at each xor step a lane keeps half of its current
// values and adds its partner's copy of that half, so the N sums need N - 1 +
// log2 LPC - log2 N exchanges instead of N log2 LPC; lane (i << (log2 LPC -
// log2 N)) ends with total i, which is then broadcast.  The order of the
// additions is fixed (deterministic).
template <int N, int LPC>
__device__ __forceinline__ void wsum_multi(float (&v)[N], const Grp<LPC>& g) {
  constexpr int LG = N == 2 ? 1 : N == 4 ? 2 : 3;
  constexpr int LG5 = LPC == 32 ? 5 : 4;
  static_assert(N == 2 || N == 4 || N == 8, "wsum_multi: N must be 2, 4 or 8");
  float c[N];
#pragma unroll
  for (int i = 0; i < N; ++i) c[i] = v[i];
#pragma unroll
  for (int k = 0; k < LG5; ++k) {
    const int o = (LPC / 2) >> k, h = (N >> k) / 2;   // h values kept at this level (0: the last sums)
    if (h >= 1) {
      const bool upper = (g.sub & o) != 0;
#pragma unroll
      for (int i = 0; i < h; ++i) {
        const float send = upper ? c[i] : c[i + h];
        const float keep = upper ? c[i + h] : c[i];
        c[i] = keep + __shfl_xor_sync(g.mask, send, o, LPC);
      }
    } else {
      c[0] += __shfl_xor_sync(g.mask, c[0], o, LPC);
    }
  }
#pragma unroll
  for (int i = 0; i < N; ++i) v[i] = __shfl_sync(g.mask, c[0], i << (LG5 - LG), LPC);
}

// ---------------------------------------------------------------- forward pieces
// 16-byte loads and stores of four consecutive floats (16-byte aligned: every
// matrix row here starts at a multiple of d floats, d % 4 == 0).  The matrix
// loops below give a lane one row (d <= LPC) and walk its columns four at a
// time, each element with the same operations in the same order as an
// element-per-lane loop, so the results are the same
__device__ __forceinline__ float4 lds4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void sts4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }
__device__ __forceinline__ float4 ldg4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }

// copy N4 16-byte pieces from shared to global memory, a lane's pieces loaded
// two at a time before they are stored (through generic pointers each load
// would otherwise wait for the store before it)
template <int N4, int LPC>
__device__ __forceinline__ void copy_s2g(float4* dst, const float4* src, int lane) {
  constexpr int NIT = (N4 + LPC - 1) / LPC;
#pragma unroll
  for (int u0 = 0; u0 < NIT; u0 += 2) {
    float4 v[2];
#pragma unroll
    for (int u = 0; u < 2; ++u)
      if (u0 + u < NIT && lane + (u0 + u) * LPC < N4) v[u] = src[lane + (u0 + u) * LPC];
#pragma unroll
    for (int u = 0; u < 2; ++u)
      if (u0 + u < NIT && lane + (u0 + u) * LPC < N4) dst[lane + (u0 + u) * LPC] = v[u];
  }
}

// sequential PDAF/EKF update of one joint for one component (its lane group)
// R: this group's scratch record (shared memory, R_H + 8d floats, 16-byte
// aligned); x, P: the component state (shared memory, updated in place, P = x + d,
// 16-byte aligned); Rg: when non-null the global record (16-byte aligned) that
// keeps this update for the reverse sweep
template <int D>
__device__ float joint_fwd(const MixDev& M, float* R, float* x, float* P, const float* Bj, const float* mj,
                           int n, const float2* z, float pd, float kappa, float* Rg, const Grp<lpc_of<D>()>& g) {
  constexpr int d = D, LPC = lpc_of<D>();
  const int lane = g.sub;
  float* H = R + R_H;
  float* U = R + rec_U(d);
  float* Kg = R + rec_Kg(d);
  float* W = R + rec_W(d);
  const bool rec = Rg != nullptr;
  float pt = 0.0f;
  if (lane < 3) {
    pt = mj[lane];
#pragma unroll
    for (int c = 0; c < D; c += 4) {
      const float4 bq = ldg4(Bj + lane * d + c), xq = lds4(x + c);
      pt = fmaf(bq.x, xq.x, pt); pt = fmaf(bq.y, xq.y, pt); pt = fmaf(bq.z, xq.z, pt); pt = fmaf(bq.w, xq.w, pt);
    }
  }
  const float p0 = g.bcast(pt, 0), p1 = g.bcast(pt, 1),
              p2 = g.bcast(pt, 2);
  if (!(p2 > kMixZMin)) {
    if (rec && lane == 0) Rg[R_VIS] = 0.0f;
    g.sync();
    return logf(kappa);
  }
  const float iz = 1.0f / p2;
  const float zh0 = M.fx * p0 * iz + M.cx, zh1 = M.fy * p1 * iz + M.cy;
  const float J00 = M.fx * iz, J02 = -M.fx * p0 * iz * iz, J11 = M.fy * iz, J12 = -M.fy * p1 * iz * iz;
  if (lane < d) {   // H = Jp Bj: column lane of both rows
    const float b2 = __ldg(Bj + 2 * d + lane);
    H[lane] = fmaf(J00, __ldg(Bj + lane), J02 * b2);
    H[d + lane] = fmaf(J11, __ldg(Bj + d + lane), J12 * b2);
  }
  g.sync();
  if (lane < d) {   // U = P H^T, row lane
    float s0 = 0.0f, s1 = 0.0f;
#pragma unroll 1   // (fully unrolled it costs the 80-register backward spills)
    for (int c = 0; c < D; c += 4) {
      const float4 pq = lds4(P + lane * d + c), h0 = lds4(H + c), h1 = lds4(H + d + c);
      s0 = fmaf(pq.x, h0.x, s0); s0 = fmaf(pq.y, h0.y, s0); s0 = fmaf(pq.z, h0.z, s0); s0 = fmaf(pq.w, h0.w, s0);
      s1 = fmaf(pq.x, h1.x, s1); s1 = fmaf(pq.y, h1.y, s1); s1 = fmaf(pq.z, h1.z, s1); s1 = fmaf(pq.w, h1.w, s1);
    }
    *reinterpret_cast<float2*>(U + lane * 2) = make_float2(s0, s1);
  }
  g.sync();
  float sv = 0.0f;
  if (lane < 4) {
    const int a = lane >> 1, b = lane & 1;
    for (int r = 0; r < d; ++r) sv = fmaf(H[a * d + r], U[r * 2 + b], sv);
    if (a == b) sv += M.sigma * M.sigma;
  }
  const float S00 = g.bcast(sv, 0), S01 = g.bcast(sv, 1),
              S10 = g.bcast(sv, 2), S11 = g.bcast(sv, 3);
  const float det = S00 * S11 - S01 * S10;
  const float Si00 = S11 / det, Si01 = -S01 / det, Si10 = -S10 / det, Si11 = S00 / det;
  const float ld = logf(det);
  const float c0 = pd * 0.15915494309189535f, b = (1.0f - pd) * kappa;
  float e = 0.0f, n0 = 0.0f, n1 = 0.0f;
  if (lane < n) {
    n0 = z[lane].x - zh0;
    n1 = z[lane].y - zh1;
    const float q = n0 * (Si00 * n0 + Si01 * n1) + n1 * (Si10 * n0 + Si11 * n1);
    e = c0 * expf(-0.5f * q - 0.5f * ld);
  }
  const float ell = b + g.sum(e);
  const float beta = e / ell, beta0 = b / ell;
  const float nb0 = g.sum(beta * n0), nb1 = g.sum(beta * n1);
  const float C00 = g.sum(beta * n0 * n0) - nb0 * nb0;
  const float C01 = g.sum(beta * n0 * n1) - nb0 * nb1;
  const float C11 = g.sum(beta * n1 * n1) - nb1 * nb1;
  const float M00 = (1.0f - beta0) * S00 - C00, M01 = (1.0f - beta0) * S01 - C01;
  const float M10 = (1.0f - beta0) * S10 - C01, M11 = (1.0f - beta0) * S11 - C11;
  if (lane < d) {   // Kg = U S^-1 and W = Kg M, row lane (W's row needs only Kg's)
    const float2 u = *reinterpret_cast<const float2*>(U + lane * 2);
    const float k0 = u.x * Si00 + u.y * Si10, k1 = u.x * Si01 + u.y * Si11;
    *reinterpret_cast<float2*>(Kg + lane * 2) = make_float2(k0, k1);
    *reinterpret_cast<float2*>(W + lane * 2) = make_float2(k0 * M00 + k1 * M10, k0 * M01 + k1 * M11);
  }
  g.sync();
  if (lane < d) {
    x[lane] += Kg[lane * 2] * nb0 + Kg[lane * 2 + 1] * nb1;
    const float w0 = W[lane * 2], w1 = W[lane * 2 + 1];   // P -= W Kg^T, row lane
#pragma unroll
    for (int c = 0; c < D; c += 4) {
      float4 pq = lds4(P + lane * d + c);
      const float4 k01 = lds4(Kg + 2 * c), k23 = lds4(Kg + 2 * c + 4);
      pq.x -= w0 * k01.x + w1 * k01.y;
      pq.y -= w0 * k01.z + w1 * k01.w;
      pq.z -= w0 * k23.x + w1 * k23.y;
      pq.w -= w0 * k23.z + w1 * k23.w;
      sts4(P + lane * d + c, pq);
    }
  }
  if (lane == 0) {
    R[R_VIS] = 1.0f; R[R_N] = (float)n;
    R[R_P3] = p0; R[R_P3 + 1] = p1; R[R_P3 + 2] = p2; R[R_IZ] = iz;
    R[R_ZH] = zh0; R[R_ZH + 1] = zh1;
    R[R_JP] = J00; R[R_JP + 1] = 0.0f; R[R_JP + 2] = J02; R[R_JP + 3] = 0.0f; R[R_JP + 4] = J11; R[R_JP + 5] = J12;
    R[R_S] = S00; R[R_S + 1] = S01; R[R_S + 2] = S10; R[R_S + 3] = S11;
    R[R_SI] = Si00; R[R_SI + 1] = Si01; R[R_SI + 2] = Si10; R[R_SI + 3] = Si11;
    R[R_LD] = ld; R[R_ELL] = ell; R[R_B0] = beta0; R[R_NB] = nb0; R[R_NB + 1] = nb1;
    R[R_M] = M00; R[R_M + 1] = M01; R[R_M + 2] = M10; R[R_M + 3] = M11;
  }
  if (lane < kMixMaxC) {
    R[R_NU + 2 * lane] = n0; R[R_NU + 2 * lane + 1] = n1;
    R[R_E + lane] = e; R[R_BETA + lane] = beta;
  }
  g.sync();
  if (rec) {
    copy_s2g<(R_H + 8 * D) / 4, LPC>(reinterpret_cast<float4*>(Rg), reinterpret_cast<const float4*>(R), lane);
  }
  g.sync();
  return logf(ell);
}

// ---------------------------------------------------------------- reverse pieces
template <int D>
__device__ void joint_bwd(const MixDev& M, const float* R, const float* Bj, float pd, float kappa, float* xb,
                          float* Pb, float gl, float* tmp, float& sb, const Grp<lpc_of<D>()>& g) {
  const float4 hd = lds4(R + R_VIS);   // VIS, N, B0, ELL
  if (hd.x == 0.0f) return;
  constexpr int d = D, LPC = lpc_of<D>();
  const int lane = g.sub;
  const int n = (int)hd.y;
  const float* H = R + R_H;
  const float* U = R + rec_U(d);
  const float* Kg = R + rec_Kg(d);
  const float* W = R + rec_W(d);
  const float* Pin = R + rec_Pin(d);
  float* Kgb = tmp;
  float* Wb = tmp + 2 * d;
  float* Ub = tmp + 4 * d;
  float* Hb = tmp + 6 * d;
  const float2 nbq = *reinterpret_cast<const float2*>(R + R_NB);
  const float nb0 = nbq.x, nb1 = nbq.y;
  const float4 S4 = lds4(R + R_S), Si4 = lds4(R + R_SI), M4 = lds4(R + R_M);
  const float S[4] = {S4.x, S4.y, S4.z, S4.w};
  const float Si[4] = {Si4.x, Si4.y, Si4.z, Si4.w};
  const float Mm[4] = {M4.x, M4.y, M4.z, M4.w};
  const float beta0 = hd.z, ell = hd.w;
  const float b = (1.0f - pd) * kappa;
  // x' = x + Kg nb
  float t2[2] = {0.0f, 0.0f};
  if (lane < d) { t2[0] = Kg[lane * 2] * xb[lane]; t2[1] = Kg[lane * 2 + 1] * xb[lane]; }
  wsum_multi<2>(t2, g);
  float nbb0 = t2[0], nbb1 = t2[1];
  // P' = P - W Kg^T
  if (lane < d) {   // row lane of Pb against Kg, column lane against W
    float s0 = 0.0f, s1 = 0.0f, t0 = 0.0f, t1 = 0.0f;
#pragma unroll
    for (int c = 0; c < D; c += 2) {
      const float2 pr = *reinterpret_cast<const float2*>(Pb + lane * d + c);
      const float4 kq = lds4(Kg + 2 * c), wq = lds4(W + 2 * c);
      const float pc0 = Pb[c * d + lane], pc1 = Pb[(c + 1) * d + lane];
      s0 = fmaf(pr.x, kq.x, s0); s1 = fmaf(pr.x, kq.y, s1);
      t0 = fmaf(pc0, wq.x, t0); t1 = fmaf(pc0, wq.y, t1);
      s0 = fmaf(pr.y, kq.z, s0); s1 = fmaf(pr.y, kq.w, s1);
      t0 = fmaf(pc1, wq.z, t0); t1 = fmaf(pc1, wq.w, t1);
    }
    *reinterpret_cast<float2*>(Wb + lane * 2) = make_float2(-s0, -s1);
    const float xr = xb[lane];
    *reinterpret_cast<float2*>(Kgb + lane * 2) = make_float2(xr * nb0 - t0, xr * nb1 - t1);
  }
  g.sync();
  // W = Kg M: the M adjoint (partials), and the Kg adjoint's W term; the
  // S^-1 adjoint of Kg = U Si (partials, from the finished Kg adjoint) is
  // reduced together with the M adjoint
  float r8[8] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
  if (lane < d) {
    r8[0] = Kg[lane * 2] * Wb[lane * 2]; r8[1] = Kg[lane * 2] * Wb[lane * 2 + 1];
    r8[2] = Kg[lane * 2 + 1] * Wb[lane * 2]; r8[3] = Kg[lane * 2 + 1] * Wb[lane * 2 + 1];
  }
  if (lane < d) {
    const float2 w = *reinterpret_cast<const float2*>(Wb + lane * 2);
    float2 kb = *reinterpret_cast<const float2*>(Kgb + lane * 2);
    kb.x += w.x * Mm[0] + w.y * Mm[1];
    kb.y += w.x * Mm[2] + w.y * Mm[3];
    *reinterpret_cast<float2*>(Kgb + lane * 2) = kb;
  }
  g.sync();
  if (lane < d) {
    r8[4] = U[lane * 2] * Kgb[lane * 2]; r8[5] = U[lane * 2] * Kgb[lane * 2 + 1];
    r8[6] = U[lane * 2 + 1] * Kgb[lane * 2]; r8[7] = U[lane * 2 + 1] * Kgb[lane * 2 + 1];
  }
  wsum_multi<8>(r8, g);
  const float Mb[4] = {r8[0], r8[1], r8[2], r8[3]};
  // M = (1 - beta0) S - Cn
  float Sb[4], Cnb[4];
  float b0b = 0.0f;
  for (int q = 0; q < 4; ++q) { Sb[q] = (1.0f - beta0) * Mb[q]; b0b -= Mb[q] * S[q]; Cnb[q] = -Mb[q]; }
  const float Cs0 = 2.0f * Cnb[0], Cs1 = Cnb[1] + Cnb[2], Cs3 = 2.0f * Cnb[3];
  float n0 = 0.0f, n1 = 0.0f, be = 0.0f, ee = 0.0f, betab = 0.0f, nub0 = 0.0f, nub1 = 0.0f;
  if (lane < n) {
    const float2 nu = *reinterpret_cast<const float2*>(R + R_NU + 2 * lane);
    n0 = nu.x; n1 = nu.y; be = R[R_BETA + lane]; ee = R[R_E + lane];
    betab = n0 * (Cnb[0] * n0 + Cnb[1] * n1) + n1 * (Cnb[2] * n0 + Cnb[3] * n1);
    nub0 = be * (Cs0 * n0 + Cs1 * n1);
    nub1 = be * (Cs1 * n0 + Cs3 * n1);
  }
  nbb0 -= Cs0 * nb0 + Cs1 * nb1;
  nbb1 -= Cs1 * nb0 + Cs3 * nb1;
  g.sync();
  // Kg = U Si
  if (lane < d) {
    const float2 kb = *reinterpret_cast<const float2*>(Kgb + lane * 2);
    *reinterpret_cast<float2*>(Ub + lane * 2) =
        make_float2(kb.x * Si[0] + kb.y * Si[1], kb.x * Si[2] + kb.y * Si[3]);
  }
  float Sib[4] = {r8[4], r8[5], r8[6], r8[7]};
  // nb = sum beta nu
  if (lane < n) {
    betab += n0 * nbb0 + n1 * nbb1;
    nub0 += be * nbb0;
    nub1 += be * nbb1;
  }
  // beta = e / ell, beta0 = b / ell, log ell
  const float num = b0b * b + g.sum(betab * ee);
  const float ellb = -num / (ell * ell) + gl / ell;
  float ldp = 0.0f, q00 = 0.0f, q01 = 0.0f, q11 = 0.0f;
  if (lane < n) {
    const float eb = betab / ell + ellb;
    const float qb = -0.5f * ee * eb;
    ldp = qb;
    nub0 += qb * (2.0f * Si[0] * n0 + (Si[1] + Si[2]) * n1);
    nub1 += qb * ((Si[2] + Si[1]) * n0 + 2.0f * Si[3] * n1);
    q00 = qb * n0 * n0; q01 = qb * n0 * n1; q11 = qb * n1 * n1;
  }
  float r6[8] = {ldp, q00, q01, q11, nub0, nub1, 0.0f, 0.0f};
  wsum_multi<8>(r6, g);
  const float ldb = r6[0];
  Sib[0] += r6[1];
  Sib[1] += r6[2]; Sib[2] += r6[2];
  Sib[3] += r6[3];
  const float zhb0 = -r6[4], zhb1 = -r6[5];
  // ld = log det S ; Si = S^-1
  Sb[0] += ldb * Si[0]; Sb[1] += ldb * Si[2]; Sb[2] += ldb * Si[1]; Sb[3] += ldb * Si[3];
  {
    float T1[4];
    for (int a = 0; a < 2; ++a)
      for (int c = 0; c < 2; ++c) T1[a * 2 + c] = Si[a] * Sib[c] + Si[2 + a] * Sib[2 + c];
    for (int a = 0; a < 2; ++a)
      for (int c = 0; c < 2; ++c) Sb[a * 2 + c] -= T1[a * 2] * Si[c * 2] + T1[a * 2 + 1] * Si[c * 2 + 1];
  }
  if (lane == 0) sb += 2.0f * M.sigma * (Sb[0] + Sb[3]);
  g.sync();
  // S = H U + sigma^2 I
  if (lane < d) {
    const float2 u = *reinterpret_cast<const float2*>(U + lane * 2);
    Hb[lane] = Sb[0] * u.x + Sb[1] * u.y;
    Hb[d + lane] = Sb[2] * u.x + Sb[3] * u.y;
    const float h0 = H[lane], h1 = H[d + lane];
    float2 ub = *reinterpret_cast<const float2*>(Ub + lane * 2);
    ub.x += h0 * Sb[0] + h1 * Sb[2];
    ub.y += h0 * Sb[1] + h1 * Sb[3];
    *reinterpret_cast<float2*>(Ub + lane * 2) = ub;
  }
  g.sync();
  // U = P H^T
  if (lane < d) {
    const float u0 = Ub[lane * 2], u1 = Ub[lane * 2 + 1];   // Pb += Ub H, row lane
#pragma unroll
    for (int c = 0; c < D; c += 4) {
      float4 pq = lds4(Pb + lane * d + c);
      const float4 h0 = lds4(H + c), h1 = lds4(H + d + c);
      pq.x += u0 * h0.x + u1 * h1.x;
      pq.y += u0 * h0.y + u1 * h1.y;
      pq.z += u0 * h0.z + u1 * h1.z;
      pq.w += u0 * h0.w + u1 * h1.w;
      sts4(Pb + lane * d + c, pq);
    }
    float s0 = 0.0f, s1 = 0.0f;   // Hb += Ub^T Pin, column lane of both rows
#pragma unroll
    for (int r = 0; r < D; ++r) {
      const float2 u = *reinterpret_cast<const float2*>(Ub + r * 2);
      const float pin = Pin[r * d + lane];
      s0 = fmaf(u.x, pin, s0);
      s1 = fmaf(u.y, pin, s1);
    }
    Hb[lane] += s0;
    Hb[d + lane] += s1;
  }
  g.sync();
  // H = Jp Bj
  float jb = 0.0f;
  if (lane < 6) {
    const int a = lane / 3, t = lane - a * 3;
#pragma unroll 1   // (fully unrolled it costs the 80-register backward spills)
    for (int c = 0; c < D; c += 4) {
      const float4 hq = lds4(Hb + a * d + c), bq = ldg4(Bj + t * d + c);
      jb = fmaf(hq.x, bq.x, jb); jb = fmaf(hq.y, bq.y, jb); jb = fmaf(hq.z, bq.z, jb); jb = fmaf(hq.w, bq.w, jb);
    }
  }
  float Jb[6];
  for (int q = 0; q < 6; ++q) Jb[q] = g.bcast(jb, q);
  const float iz = R[R_IZ], iz2 = iz * iz, iz3 = iz2 * iz;
  const float J00 = R[R_JP], J02 = R[R_JP + 2], J11 = R[R_JP + 4], J12 = R[R_JP + 5];
  const float p0 = R[R_P3], p1 = R[R_P3 + 1];
  const float pb0 = J00 * zhb0 + Jb[2] * (-M.fx * iz2);
  const float pb1 = J11 * zhb1 + Jb[5] * (-M.fy * iz2);
  const float pb2 = J02 * zhb0 + J12 * zhb1 + Jb[0] * (-M.fx * iz2) + Jb[2] * (2.0f * M.fx * p0 * iz3) +
                    Jb[4] * (-M.fy * iz2) + Jb[5] * (2.0f * M.fy * p1 * iz3);
  if (lane < d) xb[lane] += Bj[lane] * pb0 + Bj[d + lane] * pb1 + Bj[2 * d + lane] * pb2;
  g.sync();
}

// ---------------------------------------------------------------- CTA-wide frame pieces
constexpr int kDetBlock = 16;     // frames of detection lists prefetched at once

struct Smem {
  float *xh, *Ph, *xo, *Po, *Xb, *Pb, *Pcb, *xt;
  float2* det;          // this frame's lists (points into dblk)
  int* cnt;             // this frame's counts (points into dcnt)
  float2* dblk;         // [kDetBlock][MKF_MAX_J][kMixMaxC]
  int* dcnt;            // [kDetBlock][MKF_MAX_J]
  float *w, *l, *wb, *red;
  double* dred;
  float *stg0, *stg1;   // backward: staged frame records [xin | Pin | w (32) | xo], two buffers
};

// floats of one staged frame record (xin, Pin, the 32 weight slots, xo; the
// same order and offsets as in the global frame record from FL.xin on)
__host__ __device__ inline int stage_floats(int d) { return d + d * d + 32 + d; }

// Prefetch the lists of frames g .. g+n-1 (n <= kDetBlock) into shared memory:
// one coalesced pass instead of two dependent DRAM round trips per frame.
__device__ void load_det_block(const MixArgs& A, long long g, int n, Smem& s, int tid, int TB) {
  const int J = A.M.J;
  __syncthreads();
  for (int q = tid; q < n * J; q += TB) {
    int c = A.det_off[g * J + q + 1] - A.det_off[g * J + q];
    if (c > kMixMaxC) { c = kMixMaxC; atomicOr(A.status, MKF_ST_TRUNC); }
    s.dcnt[(q / J) * MKF_MAX_J + (q % J)] = c < 0 ? 0 : c;
  }
  __syncthreads();
  for (int q = tid; q < n * J * kMixMaxC; q += TB) {
    const int f = q / (J * kMixMaxC), r = q - f * J * kMixMaxC, j = r / kMixMaxC, i = r - j * kMixMaxC;
    if (i < s.dcnt[f * MKF_MAX_J + j])
      s.dblk[(f * MKF_MAX_J + j) * kMixMaxC + i] = A.det[A.det_off[(g + f) * J + j] + i];
  }
  __syncthreads();
}

__device__ __forceinline__ void select_frame_dets(Smem& s, int f) {
  s.det = s.dblk + (size_t)f * MKF_MAX_J * kMixMaxC;
  s.cnt = s.dcnt + f * MKF_MAX_J;
}

// per-group shared scratch of the frame forward: xk (d), Pk (d*d), record (R_H + 8d);
// in the reverse sweep a joint record (R_H + 8d) and the entering covariance
// rebuilt behind it (rec_Pin .. rec_Pin + d*d)
__host__ __device__ inline int fwd_scratch_floats(int d) { return (d + d * d + R_H + 8 * d + 3) & ~3; }

// one frame forward (all groups); each group's component lives in its shared
// scratch (stride SR floats from scr); when frg is non-null the component
// records and states are also kept in the global frame record frg.  Returns
// c_t (valid in every thread); s.w, s.xo, s.Po hold the mixture weights and
// the collapsed posterior
template <int D>
__device__ float frame_forward(const MixArgs& A, float* scr, int SR, float* frg, const FrameLayout& FL,
                               const float* Bm, const float* mm, float pd, float kappa, Smem& s) {
  const MixDev& M = A.M;
  constexpr int d = D, LPC = lpc_of<D>();
  const int K = M.K, J = M.J;
  const int tid = threadIdx.x, TB = blockDim.x, k = tid / LPC;
  const Grp<LPC> g(tid);
  const int lane = g.sub;
  if (k < K) {
    float* xk = scr + (size_t)k * SR;
    float* Pk = xk + d;
    float* R = Pk + d * d;
    float* cg = frg ? frg + (size_t)k * FL.comp_size : nullptr;
    const float* a = M.a + k * d;
    const float* mu = M.mu + k * d;
    // the model is read-only in the kernel: __ldg lets these loads move ahead
    // of the shared stores (generic pointers that could otherwise alias)
    if (lane < d) xk[lane] = fmaf(__ldg(a + lane), s.xh[lane], (1.0f - __ldg(a + lane)) * __ldg(mu + lane));
    const float* Qk = M.Q + (size_t)k * d * d;
    if (lane < d) {   // Pk = A Ph A + Q, row lane
      const float ar = __ldg(a + lane);
#pragma unroll
      for (int c = 0; c < D; c += 4) {
        const float4 ac = ldg4(a + c), ph = lds4(s.Ph + lane * d + c), q = ldg4(Qk + lane * d + c);
        sts4(Pk + lane * d + c, make_float4(fmaf(ar * ac.x, ph.x, q.x), fmaf(ar * ac.y, ph.y, q.y),
                                            fmaf(ar * ac.z, ph.z, q.z), fmaf(ar * ac.w, ph.w, q.w)));
      }
    }
    g.sync();
    float ll = 0.0f;
    for (int j = 0; j < J; ++j)
      ll += joint_fwd<D>(M, R, xk, Pk, Bm + j * 3 * d, mm + j * 3, s.cnt[j], s.det + j * kMixMaxC, pd, kappa,
                         cg ? cg + j * rec_size(d) : nullptr, g);
    if (cg) {   // xk, Pk contiguous in the scratch and in the record (comp_Pk = comp_xk + d)
      const float4* s4 = reinterpret_cast<const float4*>(xk);
      float4* g4 = reinterpret_cast<float4*>(cg + FL.comp_xk);
      for (int i = lane; i < (d + d * d) / 4; i += LPC) g4[i] = s4[i];
    }
    if (lane == 0) s.l[k] = M.logpi[k] + ll;
  }
  __syncthreads();
  if (tid < 32) {   // K <= 32: the softmax over components in the first warp
    const float v = tid < K ? s.l[tid] : -INFINITY;
    const float mx = warp_max(v);
    const float sum = warp_sum(tid < K ? expf(v - mx) : 0.0f);
    const float c = mx + logf(sum);
    if (tid < K) s.w[tid] = expf(v - c);
    if (tid == 0) s.red[0] = c;
  }
  __syncthreads();
  for (int r = tid; r < d; r += TB) {
    float v = 0.0f;
#pragma unroll 4
    for (int q = 0; q < K; ++q) v = fmaf(s.w[q], scr[(size_t)q * SR + r], v);
    s.xo[r] = v;
  }
  __syncthreads();
  for (int i = tid; i < d * d; i += TB) {
    const int r = i / d, c = i - r * d;
    if (r > c) continue;
    float v = 0.0f;
#pragma unroll 4
    for (int q = 0; q < K; ++q) {
      const float* bq = scr + (size_t)q * SR;
      const float Dr = bq[r] - s.xo[r], Dc = bq[c] - s.xo[c];
      v = fmaf(s.w[q], 0.5f * (bq[d + i] + bq[d + c * d + r]) + Dr * Dc, v);
    }
    s.Po[i] = v;
    s.Po[c * d + r] = v;
  }
  __syncthreads();
  return s.red[0];
}

template <int D>
__device__ void prior_state(const MixDev& M, Smem& s, int tid, int TB) {
  constexpr int d = D;
  const int K = M.K;
  for (int r = tid; r < d; r += TB) {
    float v = 0.0f;
    for (int k = 0; k < K; ++k) v = fmaf(M.pi[k], M.mu[k * d + r], v);
    s.xh[r] = v;
  }
  __syncthreads();
  for (int i = tid; i < d * d; i += TB) {
    const int r = i / d, c = i - r * d;
    float v = 0.0f;
    for (int k = 0; k < K; ++k)
      v = fmaf(M.pi[k], M.S0[(size_t)k * d * d + i] + (M.mu[k * d + r] - s.xh[r]) * (M.mu[k * d + c] - s.xh[c]), v);
    s.Ph[i] = v;
  }
  __syncthreads();
}

__device__ float* carve(Smem& s, float* base, int d) {
  float* p = base;
  s.xh = p; p += d; s.Ph = p; p += d * d;
  s.xo = p; p += d; s.Po = p; p += d * d;
  s.Xb = p; p += d; s.Pb = p; p += d * d;
  s.Pcb = p; p += d * d;
  s.xt = p; p += d;
  p = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(p) + 7) & ~uintptr_t(7));
  s.dblk = reinterpret_cast<float2*>(p); p += 2 * kDetBlock * MKF_MAX_J * kMixMaxC;
  s.dcnt = reinterpret_cast<int*>(p); p += kDetBlock * MKF_MAX_J;
  s.det = s.dblk;
  s.cnt = s.dcnt;
  s.w = p; p += 32; s.l = p; p += 32; s.wb = p; p += 32;
  s.red = p; p += 64;
  p = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(p) + 7) & ~uintptr_t(7));
  s.dred = reinterpret_cast<double*>(p);
  p += 2 * 40;
  p = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(p) + 15) & ~uintptr_t(15));
  s.stg0 = p; p += stage_floats(d);
  s.stg1 = p; p += stage_floats(d);
  return reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(p) + 15) & ~uintptr_t(15));
}

// bytes of the shared state carved by carve() (an upper bound, 16-byte multiple)
size_t mix_smem_bytes(int d) {
  size_t b = sizeof(float) * (size_t)(4 * d + 4 * d * d + d + 2 * kDetBlock * MKF_MAX_J * kMixMaxC +
                                      kDetBlock * MKF_MAX_J + 32 * 3 + 64 + 8 + 2 * stage_floats(d)) +
             sizeof(double) * 40 + 96;
  return (b + 15) & ~size_t(15);
}

// ---------------------------------------------------------------- forward kernel
// REGS, the register cap of both kernels: at d = 24 (whole warps, up to 1024
// threads) 64; at d = 12 (half-warp groups, 256 threads for 15 components)
// 128 when every track has its own CTA at two CTAs per SM (faster per CTA),
// else 80, so that three CTAs share an SM (mix_grid chooses).
template <int D, int REGS>
__global__ void __maxnreg__(REGS) mix_forward_kernel(MixArgs A) {
  extern __shared__ __align__(16) float msm[];
  Smem s;
  float* scr = carve(s, msm, D);                 // per-group component scratch follows
  constexpr int d = D;
  const int J = A.M.J;
  const int tid = threadIdx.x, TB = blockDim.x;
  const FrameLayout FL = frame_layout(d, A.M.K, J);
  const int SR = fwd_scratch_floats(d);
  for (int b = blockIdx.x; b < A.n_tracks; b += gridDim.x) {
    const int T = A.n_frames[b];
    const long long g0 = A.frame_base[b];
    const float* Bm = A.Bm + (size_t)b * J * 3 * d;
    const float* mm = A.mm + (size_t)b * J * 3;
    const float pd = A.pd[b], kappa = A.kappa[b];
    float* ck = A.ck + A.ck_off[b];
    prior_state<D>(A.M, s, tid, TB);
    double L = 0.0;
    for (int t = 0; t < T; ++t) {
      if (t % A.C == 0) {
        float* c = ck + (size_t)(t / A.C) * (d + d * d);
        for (int i = tid; i < d; i += TB) c[i] = s.xh[i];
        for (int i = tid; i < d * d; i += TB) c[d + i] = s.Ph[i];
      }
      if (t % kDetBlock == 0) load_det_block(A, g0 + t, min(kDetBlock, T - t), s, tid, TB);
      select_frame_dets(s, t % kDetBlock);
      L += (double)frame_forward<D>(A, scr, SR, nullptr, FL, Bm, mm, pd, kappa, s);
      for (int i = tid; i < d; i += TB) s.xh[i] = s.xo[i];
      for (int i = tid; i < d * d; i += TB) s.Ph[i] = s.Po[i];
      __syncthreads();
    }
    if (tid == 0) A.ll[b] = L;
    __syncthreads();
  }
}

// ---------------------------------------------------------------- backward kernel
// Per segment of C frames: recompute the frames from the segment's checkpoint
// keeping every frame's records (one forward), then reverse them.
// STAGE: the per-component adjoint work blocks live in shared memory (used
// when they fit), so the fixed-order cross-component sums stay on chip;
// otherwise they stay in the global slot.  Records always stay in the slot,
// and the FP64 parameter adjoints (flushed once a segment) in the CTA's
// accumulator row.
template <int D, bool STAGE, int REGS>
__global__ void __maxnreg__(REGS) mix_backward_kernel(MixArgs A) {
  extern __shared__ __align__(16) float msm[];
  Smem s;
  float* scr = carve(s, msm, D);
  const MixDev& M = A.M;
  constexpr int d = D, DD = D * (D + 1) / 2, LPC = lpc_of<D>();
  const int J = M.J, K = M.K;
  const int tid = threadIdx.x, TB = blockDim.x, k = tid / LPC;
  const Grp<LPC> g(tid);
  const int lane = g.sub;
  const bool act = LPC == 32 || k < K;   // a group past the last component (K odd) only joins the barriers
  const FrameLayout FL = frame_layout(d, K, J);
  const WorkLayout WL = work_layout(d);
  const int SR = fwd_scratch_floats(d);
  float* slot = A.slots + (size_t)blockIdx.x * A.slot_floats;
  float* frames = slot + (size_t)K * WL.size;               // C frame records
  // FP64 parameter adjoints (mu, a, Lq, sigma): the CTA's row, zeroed by the host
  double* const gacc = A.gacc + (size_t)blockIdx.x * A.ng;
  float* wb = STAGE ? scr + (size_t)K * SR + (size_t)k * WL.size     // this component's work block
                    : slot + (size_t)k * WL.size;
  float* const wbase = STAGE ? scr + (size_t)K * SR : slot;
  const float* a = M.a + k * d;
  const float* mu = M.mu + k * d;
  const float* Lk = M.Lq + k * DD;
  float sbl = 0.0f;                                         // sigma adjoint of this segment (lane 0)
  double sbd = 0.0;                                         // and its FP64 running sum
  if (act)
    for (int i = lane; i < 2 * d + d * d; i += LPC) wb[WL.gmu + i] = 0.0f;   // gmu, ga, Sq
  // frame record fr's input state, mixture weights and collapsed mean
  // (stage_floats(d) contiguous floats from FL.xin) are copied into a staging
  // buffer with cp.async, and checkpoints (d + d^2 floats) into s.xh, s.Ph; the
  // issuing threads wait for their copies before a barrier
  constexpr int SG4 = (2 * D + D * D + 32) / 4, CK4 = (D + D * D) / 4;
  const int fxin = FL.xin;
  for (int b = blockIdx.x; b < A.n_tracks; b += gridDim.x) {
    const int T = A.n_frames[b];
    const long long g0 = A.frame_base[b];
    const float* Bm = A.Bm + (size_t)b * J * 3 * d;
    const float* mm = A.mm + (size_t)b * J * 3;
    const float pd = A.pd[b], kappa = A.kappa[b];
    const float* ck = A.ck + A.ck_off[b];
    for (int i = tid; i < d; i += TB) s.Xb[i] = 0.0f;
    for (int i = tid; i < d * d; i += TB) s.Pb[i] = 0.0f;
    const int nck = (T + A.C - 1) / A.C;
    // the last segment's checkpoint; each later one is copied while the
    // segment after it is reversed (s.xh, s.Ph are free then)
    if (nck > 0)
      for (int i = tid; i < CK4; i += TB) cp_async16(s.xh + 4 * i, ck + (size_t)(nck - 1) * (d + d * d) + 4 * i);
    cp_async_commit();
    cp_async_wait_all();
    __syncthreads();
    for (int sg = nck - 1; sg >= 0; --sg) {
      const int t0 = sg * A.C, t1 = min(T, t0 + A.C);
      // ---- recompute the segment from its checkpoint (in s.xh, s.Ph), keeping every frame's records
      for (int t = t0; t < t1; ++t) {
        float* fr = frames + (size_t)(t - t0) * FL.size;
        for (int i = tid; i < d; i += TB) fr[FL.xin + i] = s.xh[i];
        for (int i = tid; i < d * d; i += TB) fr[FL.Pin + i] = s.Ph[i];
        if ((t - t0) % kDetBlock == 0) load_det_block(A, g0 + t, min(kDetBlock, t1 - t), s, tid, TB);
        select_frame_dets(s, (t - t0) % kDetBlock);
        frame_forward<D>(A, scr, SR, fr, FL, Bm, mm, pd, kappa, s);
        for (int i = tid; i < K; i += TB) fr[FL.w + i] = s.w[i];
        for (int i = tid; i < d; i += TB) { fr[FL.xo + i] = s.xo[i]; s.xh[i] = s.xo[i]; }
        for (int i = tid; i < d * d; i += TB) s.Ph[i] = s.Po[i];
        __syncthreads();
      }
      // ---- reverse the segment.  Four barriers a frame: the pass that sums
      // frame t's per-component adjoints into Xb, Pb also forms frame t-1's
      // symmetrised covariance adjoint Pcb from the same sums.  Frame t-1's
      // input state, weights and collapsed mean are copied into the other
      // staging buffer while frame t is reversed.
      for (int i = tid; i < SG4; i += TB)
        cp_async16(s.stg0 + 4 * i, frames + (size_t)(t1 - 1 - t0) * FL.size + fxin + 4 * i);
      cp_async_commit();
      for (int i = tid; i < d * d; i += TB) {
        const int r = i / d, c = i - r * d;
        s.Pcb[i] = 0.5f * (s.Pb[i] + s.Pb[c * d + r]);
      }
      cp_async_wait_all();
      __syncthreads();
      if (sg > 0)
        for (int i = tid; i < CK4; i += TB) cp_async16(s.xh + 4 * i, ck + (size_t)(sg - 1) * (d + d * d) + 4 * i);
      cp_async_commit();
      for (int t = t1 - 1; t >= t0; --t) {
        const float* fr = frames + (size_t)(t - t0) * FL.size;
        const float* cb = fr + (size_t)k * FL.comp_size;
        const bool odd = ((t1 - 1 - t) & 1) != 0;   // frame t in stg1, else stg0; frame t-1 in the other
        const float* st = odd ? s.stg1 : s.stg0;
        if (t > t0) {
          float* nx = odd ? s.stg0 : s.stg1;
          for (int i = tid; i < SG4; i += TB) cp_async16(nx + 4 * i, fr - FL.size + fxin + 4 * i);
        }
        cp_async_commit();
        const float* xin = st;
        const float* Pin = st + d;
        const float* wv = st + d + d * d;
        const float* xo = wv + 32;
        const float* xk = cb + FL.comp_xk;
        const float* Pk = cb + FL.comp_Pk;
        const float wk = act ? wv[k] : 0.0f;
        // collapse reverse: P' = sym(sum w (P_k + D D^T)), x' = sum w x_k, softmax (dc = 1)
        float* Dkb = wb + WL.Dkb;
        if (act && lane < d) {
          float v = 0.0f;
#pragma unroll
          for (int c = 0; c < D; c += 4) {   // xk: this frame's record in the slot (written by this kernel)
            const float4 pq = lds4(s.Pcb + lane * d + c), xq = *reinterpret_cast<const float4*>(xk + c);
            const float4 oq = lds4(xo + c);
            v = fmaf(pq.x, xq.x - oq.x, v); v = fmaf(pq.y, xq.y - oq.y, v);
            v = fmaf(pq.z, xq.z - oq.z, v); v = fmaf(pq.w, xq.w - oq.w, v);
          }
          Dkb[lane] = 2.0f * wk * v;
        }
        __syncthreads();
        // xt = Xb - sum_q Dkb_q: every group forms its own copy (lane r), in the same order
        float xt = 0.0f, wbk = 0.0f;
        if (act) {
          if (lane < d) {
            float v = s.Xb[lane];
#pragma unroll 4
            for (int q = 0; q < K; ++q) v -= wbase[(size_t)q * WL.size + WL.Dkb + lane];
            xt = v;
          }
          float wbp = 0.0f;
          if (lane < d) {   // row lane of sum Pcb o (Pk + D D^T), D = xk - xo
            const float xr = xk[lane];
            const float dr = xr - xo[lane];
            wbp = xr * xt;
#pragma unroll
            for (int c = 0; c < D; c += 4) {
              const float4 pq = lds4(s.Pcb + lane * d + c), kq = *reinterpret_cast<const float4*>(Pk + lane * d + c);
              const float4 xq = *reinterpret_cast<const float4*>(xk + c), oq = lds4(xo + c);
              wbp = fmaf(pq.x, kq.x + dr * (xq.x - oq.x), wbp);
              wbp = fmaf(pq.y, kq.y + dr * (xq.y - oq.y), wbp);
              wbp = fmaf(pq.z, kq.z + dr * (xq.z - oq.z), wbp);
              wbp = fmaf(pq.w, kq.w + dr * (xq.w - oq.w), wbp);
            }
          }
          wbk = g.sum(wbp);
          if (lane == 0) s.wb[k] = wbk;
        }
        __syncthreads();
        // sum_q w_q wb_q, formed by every group in the same order
        float swp = 0.0f;
        for (int q = lane; q < K; q += LPC) swp = fmaf(wv[q], s.wb[q], swp);
        const float swb = g.sum(swp);
        const float lb = wk * (wbk - swb) + wk;
        float* xb = wb + WL.xb;
        float* Pb = wb + WL.Pb;
        float* Xin = wb + WL.Xin;
        float* Pinb = wb + WL.Pin;
        if (!act) {
        } else if (wk > 0.0f) {
          if (lane < d) xb[lane] = Dkb[lane] + wk * xt;
          for (int i = lane; i < d * d; i += LPC) Pb[i] = wk * s.Pcb[i];
          g.sync();
          // each joint's record is copied (coalesced, 16 bytes per lane and step)
          // into this group's forward scratch, idle during the reverse sweep, so
          // that the reverse reads it from shared memory instead of L2
          float* Rs = scr + (size_t)k * SR;
          const int RS4 = rec_size(d) / 4;
          for (int j = J - 1; j >= 0; --j) {
            // cp.async: all of a lane's 16-byte pieces in flight at once
            // (plain copies through registers wait out each load before its store)
            const float* src = cb + j * rec_size(d);
            for (int q = lane; q < RS4; q += LPC) cp_async16(Rs + 4 * q, src + 4 * q);
            if (j == J - 1)   // the component's final covariance, rebuilt backwards below
              for (int q = lane; q < D * D / 4; q += LPC) cp_async16(Rs + rec_Pin(d) + 4 * q, Pk + 4 * q);
            cp_async_commit();
            cp_async_wait_all();
            g.sync();
            if (Rs[R_VIS] != 0.0f) {
              // the covariance entering joint j: the forward's P -= W Kg^T undone
              const float* Wr = Rs + rec_W(d);
              const float* Kr = Rs + rec_Kg(d);
              float* Pr = Rs + rec_Pin(d);
              if (lane < d) {
                const float w0 = Wr[lane * 2], w1 = Wr[lane * 2 + 1];
#pragma unroll
                for (int c = 0; c < D; c += 4) {
                  float4 pq = lds4(Pr + lane * d + c);
                  const float4 k01 = lds4(Kr + 2 * c), k23 = lds4(Kr + 2 * c + 4);
                  pq.x += w0 * k01.x + w1 * k01.y;
                  pq.y += w0 * k01.z + w1 * k01.w;
                  pq.z += w0 * k23.x + w1 * k23.y;
                  pq.w += w0 * k23.z + w1 * k23.w;
                  sts4(Pr + lane * d + c, pq);
                }
              }
              g.sync();
            }
            joint_bwd<D>(M, Rs, Bm + j * 3 * d, pd, kappa, xb, Pb, lb, wb + WL.tmp, sbl, g);
            g.sync();
          }
          // predict reverse: x = a*xin + (1-a)*mu ; P = A Pin A + Q (Q = L L^T: its
          // adjoint Pb is summed here and turned into the L adjoint once a segment)
          float* gmu = wb + WL.gmu;
          float* ga = wb + WL.ga;
          float* Sq = wb + WL.Sq;
          if (lane < d) {
            const float al = __ldg(a + lane);
            Xin[lane] = al * xb[lane];
            gmu[lane] += (1.0f - al) * xb[lane];
            float g = (xin[lane] - __ldg(mu + lane)) * xb[lane];
#pragma unroll
            for (int c = 0; c < D; c += 4) {
              const float4 pr = lds4(Pb + lane * d + c), qr = lds4(Pin + lane * d + c), ac = ldg4(a + c);
              g += (pr.x * qr.x + Pb[c * d + lane] * Pin[c * d + lane]) * ac.x;
              g += (pr.y * qr.y + Pb[(c + 1) * d + lane] * Pin[(c + 1) * d + lane]) * ac.y;
              g += (pr.z * qr.z + Pb[(c + 2) * d + lane] * Pin[(c + 2) * d + lane]) * ac.z;
              g += (pr.w * qr.w + Pb[(c + 3) * d + lane] * Pin[(c + 3) * d + lane]) * ac.w;
              // Pin adjoint A Pb A and the segment's Q adjoint sum, row lane
              sts4(Pinb + lane * d + c, make_float4(al * ac.x * pr.x, al * ac.y * pr.y, al * ac.z * pr.z,
                                                    al * ac.w * pr.w));
              float4 sq = lds4(Sq + lane * d + c);
              sq.x += pr.x; sq.y += pr.y; sq.z += pr.z; sq.w += pr.w;
              sts4(Sq + lane * d + c, sq);
            }
            ga[lane] += g;
          }
        } else if (lane < d) {
          Xin[lane] = 0.0f;
#pragma unroll
          for (int c = 0; c < D; c += 4) sts4(Pinb + lane * d + c, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
        }
        __syncthreads();
        for (int r = tid; r < d; r += TB) {
          float v = 0.0f;
#pragma unroll 4
          for (int q = 0; q < K; ++q) v += wbase[(size_t)q * WL.size + WL.Xin + r];
          s.Xb[r] = v;
        }
        for (int i = tid; i < d * d; i += TB) {
          float v = 0.0f;
#pragma unroll 4
          for (int q = 0; q < K; ++q) v += wbase[(size_t)q * WL.size + WL.Pin + i];
          s.Pb[i] = v;
          if (t > t0) {   // the transposed entry's sum, in the same order, for Pcb of frame t-1
            const int r = i / d, c = i - r * d;
            float vt = 0.0f;
#pragma unroll 4
            for (int q = 0; q < K; ++q) vt += wbase[(size_t)q * WL.size + WL.Pin + c * d + r];
            s.Pcb[i] = 0.5f * (v + vt);
          }
        }
        cp_async_wait_all();   // frame t-1's staging buffer (and the next checkpoint)
        __syncthreads();
      }
      // flush this segment's FP32 parameter adjoints into the CTA's FP64
      // accumulators; the L_Q adjoint is tril((Sq + Sq^T) L_Q)
      // (d <= LPC; every group of read-modify-writes loads its accumulators
      // before it stores any, so their L2 round trips overlap)
      if (act) {
        if (lane < d) {
          const float vm = wb[WL.gmu + lane], va = wb[WL.ga + lane];
          double* const pm = gacc + k * d + lane;
          double* const pa = gacc + K * d + k * d + lane;
          const double om = *pm, oa = *pa;
          *pm = om + (double)vm;
          *pa = oa + (double)va;
        }
        const float* Sq = wb + WL.Sq;
        double* const gl = gacc + 2 * K * d + k * DD;
        constexpr int NCH = 2;
        for (int i0 = lane; i0 < DD; i0 += NCH * LPC) {
          float gv[NCH];
#pragma unroll
          for (int u = 0; u < NCH; ++u) {
            const int i = i0 + u * LPC;
            float gs = 0.0f;
            if (i < DD) {
              int r = (int)((sqrtf(8.0f * i + 1.0f) - 1.0f) * 0.5f);
              while (r * (r + 1) / 2 > i) --r;
              while ((r + 1) * (r + 2) / 2 <= i) ++r;
              const int c = i - r * (r + 1) / 2;
              for (int t2 = c; t2 < d; ++t2) gs = fmaf(Sq[r * d + t2] + Sq[t2 * d + r], Lk[t2 * (t2 + 1) / 2 + c], gs);
            }
            gv[u] = gs;
          }
          double ov[NCH];
#pragma unroll
          for (int u = 0; u < NCH; ++u) ov[u] = (i0 + u * LPC < DD) ? gl[i0 + u * LPC] : 0.0;
#pragma unroll
          for (int u = 0; u < NCH; ++u)
            if (i0 + u * LPC < DD) gl[i0 + u * LPC] = ov[u] + (double)gv[u];
        }
        sbd += (double)sbl;
        sbl = 0.0f;
        g.sync();
        for (int i = lane; i < 2 * d + d * d; i += LPC) wb[WL.gmu + i] = 0.0f;
      }
      __syncthreads();
    }
    // prior: x = sum pi mu, P = sum pi (S0 + D D^T)
    for (int r = tid; r < d; r += TB) {
      float v = 0.0f;
      for (int q = 0; q < K; ++q) v = fmaf(M.pi[q], M.mu[q * d + r], v);
      s.xh[r] = v;
    }
    __syncthreads();
    if (act && lane < d) {
      float v = 0.0f;
      for (int c = 0; c < d; ++c) v = fmaf(s.Pb[lane * d + c] + s.Pb[c * d + lane], mu[c] - s.xh[c], v);
      wb[WL.Dkb + lane] = M.pi[k] * v;
    }
    __syncthreads();
    for (int r = tid; r < d; r += TB) {
      float v = s.Xb[r];
      for (int q = 0; q < K; ++q) v -= wbase[(size_t)q * WL.size + WL.Dkb + r];
      s.xt[r] = v;
    }
    __syncthreads();
    if (act && lane < d) gacc[k * d + lane] += (double)(wb[WL.Dkb + lane] + M.pi[k] * s.xt[lane]);
    __syncthreads();
  }
  // sigma: per-group lane 0 partials, fixed-order sum
  if (act && lane == 0) s.dred[k] = sbd;
  __syncthreads();
  if (tid == 0) {
    double v = 0.0;
    for (int q = 0; q < K; ++q) v += s.dred[q];
    gacc[A.ng - 1] += v;
  }
}

// fixed-order reduction of the per-CTA FP64 accumulators
__global__ void mix_reduce_kernel(const double* gacc, int nslots, int ng, double* grad) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < ng; q += gridDim.x * blockDim.x) {
    double v = 0.0;
    for (int s = 0; s < nslots; ++s) v += gacc[(size_t)s * ng + q];
    grad[q] = v;
  }
}

__global__ void mix_total_kernel(const double* ll, int n, double* total) {
  __shared__ double red[32];
  double v = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) v += ll[i];
  v = warp_sum_d(v);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += red[q];
    *total = t;
  }
}

// theta (FP64, flat) -> FP32 device parameters and Q = Lq Lq^T
__global__ void mix_prepare_kernel(const double* theta, int d, int K, float* mu, float* a, float* Lq, float* Q,
                                   float* sigma) {
  const int DD = d * (d + 1) / 2;
  const int n1 = K * d, n2 = 2 * K * d, n3 = n2 + K * DD;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n3 + 1 + K * d * d; i += gridDim.x * blockDim.x) {
    if (i < n1) mu[i] = (float)theta[i];
    else if (i < n2) a[i - n1] = (float)theta[i];
    else if (i < n3) Lq[i - n2] = (float)theta[i];
    else if (i == n3) *sigma = (float)theta[n3];
    else {
      const int q = i - n3 - 1, k = q / (d * d), rc = q - k * d * d, r = rc / d, c = rc - r * d;
      const double* L = theta + n2 + (size_t)k * DD;
      double v = 0.0;
      for (int s2 = 0; s2 <= (r < c ? r : c); ++s2) v += L[r * (r + 1) / 2 + s2] * L[c * (c + 1) / 2 + s2];
      Q[q] = (float)v;
    }
  }
}

__global__ void adam_kernel(double* th, const double* g, double* m, double* v, const uint8_t* mask, int n,
                            double c1, double c2, double lr, double b1, double b2, double eps, double sgn) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (mask && !mask[i]) continue;
    const double gi = g[i];
    m[i] = b1 * m[i] + (1.0 - b1) * gi;
    v[i] = b2 * v[i] + (1.0 - b2) * gi * gi;
    th[i] += sgn * lr * (m[i] / c1) / (sqrt(v[i] / c2) + eps);
  }
}

using MixKernel = void (*)(MixArgs);

}  // namespace mkf

using namespace mkf;

struct mkf_mixkf {
  int d, K, J, DD, n_tracks, C, ng, grid, grid_f, tpb;
  MixKernel fwd_kernel, bwd_kernel;   // chosen instantiations (register caps, STAGE)
  long long G;
  float *mu, *a, *Lq, *Q, *logpi, *pi, *S0, *sigma_d;
  float sigma_h;
  double* theta_dev;
  int *n_frames;
  long long *frame_base, *ck_off;
  float *Bm, *mm, *pd, *kappa, *ck, *slots;
  double *ll, *gacc, *total;
  long long slot_floats;
  int* status;
  double fx, fy, cx, cy;
  bool have_theta;
  bool stage;
  size_t smem_f, smem_b;
  int* h_nf;          // host copy of the tracks' frame counts
  int maxT;
  int fwd_C;          // checkpoint stride of the last forward (0: none yet)
};

// Checkpoint stride C and the buffers that depend on it: the checkpoints
// (every C-th collapsed state of every track) and the per-CTA slot, which holds
// the work arrays and one backward segment of C frames of records.
static int mix_set_stride(mkf_mixkf* h, int C) {
  const FrameLayout FL = frame_layout(h->d, h->K, h->J);
  const WorkLayout WL = work_layout(h->d);
  std::vector<long long> ckoff(h->n_tracks);
  long long ck_total = 0;
  for (int b = 0; b < h->n_tracks; ++b) {
    ckoff[b] = ck_total;
    ck_total += (long long)((h->h_nf[b] + C - 1) / C) * (h->d + h->d * h->d);
  }
  if (h->ck) { cudaFree(h->ck); h->ck = nullptr; }
  if (h->slots) { cudaFree(h->slots); h->slots = nullptr; }
  h->C = C;
  h->fwd_C = 0;
  h->slot_floats = ((long long)h->K * WL.size + (long long)C * FL.size + 63) & ~63LL;
  MKF_CUDA(cudaMalloc(&h->ck, sizeof(float) * (size_t)std::max<long long>(1, ck_total)));
  MKF_CUDA(cudaMemcpy(h->ck_off, ckoff.data(), sizeof(long long) * h->n_tracks, cudaMemcpyHostToDevice));
  MKF_CUDA(cudaMalloc(&h->slots, sizeof(float) * (size_t)h->slot_floats * h->grid));
  return MKF_OK;
}

// ceil(sqrt(T_max)) frames per segment, unless one segment's records of all
// resident CTAs would exceed 60 % of L2; then the longest segment that fits
static int mix_auto_stride(mkf_mixkf* h) {
  const FrameLayout FL = frame_layout(h->d, h->K, h->J);
  int dev = 0, l2 = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev) != cudaSuccess)
    l2 = 0;
  const int c_sqrt = std::max(1, (int)std::ceil(std::sqrt((double)std::max(1, h->maxT))));
  if (l2 <= 0) return c_sqrt;
  const double per_frame = 4.0 * (double)FL.size * h->grid;
  const int c_fit = std::max(1, (int)(0.6 * l2 / per_frame));
  return std::min(c_sqrt, c_fit);
}

static int mix_occ(MixKernel kern, int tpb, size_t smem, int* occ) {
  MKF_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  MKF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, kern, tpb, smem));
  return MKF_OK;
}

// shared-memory sizes, STAGE choice and the persistent grid
static int mix_grid(mkf_mixkf* h) {
  const int d = h->d, K = h->K;
  // the reverse sweep stages one joint record and the rebuilt entering
  // covariance in a group's forward scratch
  if (rec_Pin(d) + d * d > fwd_scratch_floats(d)) {
    set_error("mkf_mixkf: record larger than the group scratch");
    return MKF_ERR_ARG;
  }
  const WorkLayout WL = work_layout(d);
  const size_t base = mix_smem_bytes(d);
  const int SRf = fwd_scratch_floats(d);
  h->smem_f = base + sizeof(float) * (size_t)K * SRf;
  // STAGE: the work blocks in shared memory
  const size_t smem_stage = base + sizeof(float) * (size_t)K * (SRf + WL.size);
  int dev = 0, optin = 0;
  MKF_CUDA(cudaGetDevice(&dev));
  MKF_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  h->stage = smem_stage <= (size_t)optin;
  h->smem_b = h->stage ? smem_stage : h->smem_f;
  if (h->smem_f > (size_t)optin) { set_error("mkf_mixkf: model too large for shared memory"); return MKF_ERR_ARG; }
  // per kernel two register caps at d = 12: the higher one when its resident
  // CTAs already give every track its own CTA, else the lower one for one
  // more CTA per SM; one cap (64) at d = 24
  MixKernel f_hi, f_lo, b_hi, b_lo;
  if (d == 12) {
    f_hi = mix_forward_kernel<12, 128>;
    f_lo = mix_forward_kernel<12, 80>;
    b_hi = h->stage ? mix_backward_kernel<12, true, 128> : mix_backward_kernel<12, false, 128>;
    b_lo = h->stage ? mix_backward_kernel<12, true, 80> : mix_backward_kernel<12, false, 80>;
  } else {
    f_hi = f_lo = mix_forward_kernel<24, 64>;
    b_hi = b_lo = h->stage ? mix_backward_kernel<24, true, 64> : mix_backward_kernel<24, false, 64>;
  }
  int of_hi = 0, of_lo = 0, ob_hi = 0, ob_lo = 0, st;
  if ((st = mix_occ(f_hi, h->tpb, h->smem_f, &of_hi)) || (st = mix_occ(f_lo, h->tpb, h->smem_f, &of_lo)) ||
      (st = mix_occ(b_hi, h->tpb, h->smem_b, &ob_hi)) || (st = mix_occ(b_lo, h->tpb, h->smem_b, &ob_lo)))
    return st;
  const int sms = num_sms();
  const bool fh = h->n_tracks <= sms * of_hi || of_hi >= of_lo;
  const bool bh = h->n_tracks <= sms * ob_hi || ob_hi >= ob_lo;
  h->fwd_kernel = fh ? f_hi : f_lo;
  h->bwd_kernel = bh ? b_hi : b_lo;
  // each kernel its own persistent grid (the forward keeps no per-CTA slot)
  h->grid_f = std::min(h->n_tracks, sms * std::max(1, fh ? of_hi : of_lo));
  h->grid = std::min(h->n_tracks, sms * std::max(1, bh ? ob_hi : ob_lo));
  return MKF_OK;
}

extern "C" int mkf_mixkf_create(const mkf_mix_model* model, int n_tracks, const int* n_frames,
                                const int64_t* frame_base, const double* Bm, const double* mm,
                                const double* p_detect, const double* kappa, int64_t n_frames_total,
                                mkf_mixkf_t* out) {
  MKF_ARG(model && n_frames && frame_base && Bm && mm && p_detect && kappa && out, "mkf_mixkf_create: null argument");
  MKF_ARG(model->d == 12 || model->d == 24, "mkf_mixkf_create: d must be 12 or 24");
  MKF_ARG(model->K >= 1 && model->K <= 32, "mkf_mixkf_create: K must be in [1, 32]");
  MKF_ARG(model->J >= 1 && model->J <= MKF_MAX_J, "mkf_mixkf_create: J out of range");
  MKF_ARG(n_tracks >= 1 && model->pi && model->S0, "mkf_mixkf_create: bad tracks or model");
  const int d = model->d, K = model->K, J = model->J, DD = d * (d + 1) / 2;
  int maxT = 0;
  for (int b = 0; b < n_tracks; ++b) {
    MKF_ARG(n_frames[b] >= 0 && frame_base[b] >= 0 && frame_base[b] + n_frames[b] <= n_frames_total,
            "mkf_mixkf_create: frame range");
    MKF_ARG(p_detect[b] > 0.0 && p_detect[b] < 1.0 && kappa[b] > 0.0, "mkf_mixkf_create: p_detect/kappa");
    maxT = std::max(maxT, n_frames[b]);
  }
  mkf_mixkf* h = new (std::nothrow) mkf_mixkf();
  if (!h) return MKF_ERR_NOMEM;
  memset(h, 0, sizeof(*h));
  h->d = d; h->K = K; h->J = J; h->DD = DD; h->n_tracks = n_tracks; h->G = n_frames_total;
  h->maxT = maxT;
  h->ng = 2 * K * d + K * DD + 1;
  h->tpb = (K * (d <= 16 ? 16 : 32) + 31) / 32 * 32;   // lpc_of<D>() lanes per component, whole warps
  h->fx = model->fx; h->fy = model->fy; h->cx = model->cx; h->cy = model->cy;
  h->h_nf = static_cast<int*>(malloc(sizeof(int) * n_tracks));
  if (!h->h_nf) { delete h; return MKF_ERR_NOMEM; }
  memcpy(h->h_nf, n_frames, sizeof(int) * n_tracks);
  std::vector<float> f_Bm((size_t)n_tracks * J * 3 * d), f_mm((size_t)n_tracks * J * 3), f_pd(n_tracks), f_k(n_tracks);
  for (size_t i = 0; i < f_Bm.size(); ++i) f_Bm[i] = (float)Bm[i];
  for (size_t i = 0; i < f_mm.size(); ++i) f_mm[i] = (float)mm[i];
  for (int b = 0; b < n_tracks; ++b) { f_pd[b] = (float)p_detect[b]; f_k[b] = (float)kappa[b]; }
  std::vector<float> f_pi(K), f_lpi(K), f_S0((size_t)K * d * d);
  for (int k = 0; k < K; ++k) {
    f_pi[k] = (float)model->pi[k];
    f_lpi[k] = model->pi[k] > 0.0 ? (float)std::log(model->pi[k]) : -INFINITY;
  }
  for (size_t i = 0; i < f_S0.size(); ++i) f_S0[i] = (float)model->S0[i];
  std::vector<long long> fb(frame_base, frame_base + n_tracks);
  cudaError_t e = cudaSuccess;
  auto al = [&](void** p, size_t bytes) { if (e == cudaSuccess) e = cudaMalloc(p, std::max<size_t>(bytes, 8)); };
  auto cp = [&](void* dst, const void* src, size_t bytes) {
    if (e == cudaSuccess) e = cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
  };
  al((void**)&h->mu, sizeof(float) * K * d); al((void**)&h->a, sizeof(float) * K * d);
  al((void**)&h->Lq, sizeof(float) * K * DD); al((void**)&h->Q, sizeof(float) * K * d * d);
  al((void**)&h->logpi, sizeof(float) * K); al((void**)&h->pi, sizeof(float) * K);
  al((void**)&h->S0, sizeof(float) * K * d * d); al((void**)&h->sigma_d, sizeof(float));
  al((void**)&h->theta_dev, sizeof(double) * h->ng);
  al((void**)&h->n_frames, sizeof(int) * n_tracks); al((void**)&h->frame_base, sizeof(long long) * n_tracks);
  al((void**)&h->ck_off, sizeof(long long) * n_tracks);
  al((void**)&h->Bm, sizeof(float) * f_Bm.size()); al((void**)&h->mm, sizeof(float) * f_mm.size());
  al((void**)&h->pd, sizeof(float) * n_tracks); al((void**)&h->kappa, sizeof(float) * n_tracks);
  al((void**)&h->ll, sizeof(double) * n_tracks); al((void**)&h->total, sizeof(double));
  al((void**)&h->status, sizeof(int));
  cp(h->pi, f_pi.data(), sizeof(float) * K); cp(h->logpi, f_lpi.data(), sizeof(float) * K);
  cp(h->S0, f_S0.data(), sizeof(float) * f_S0.size());
  cp(h->n_frames, n_frames, sizeof(int) * n_tracks); cp(h->frame_base, fb.data(), sizeof(long long) * n_tracks);
  cp(h->Bm, f_Bm.data(), sizeof(float) * f_Bm.size()); cp(h->mm, f_mm.data(), sizeof(float) * f_mm.size());
  cp(h->pd, f_pd.data(), sizeof(float) * n_tracks); cp(h->kappa, f_k.data(), sizeof(float) * n_tracks);
  if (e == cudaSuccess) e = cudaMemset(h->status, 0, sizeof(int));
  if (e != cudaSuccess) {
    mkf_mixkf_destroy(h);
    return cuda_fail(e, "mkf_mixkf_create: allocation", __FILE__, __LINE__);
  }
  int st = mix_grid(h);
  if (st) { mkf_mixkf_destroy(h); return st; }
  st = mix_set_stride(h, mix_auto_stride(h));
  if (st) { mkf_mixkf_destroy(h); return st; }
  e = cudaMalloc(&h->gacc, sizeof(double) * (size_t)h->ng * h->grid);
  if (e != cudaSuccess) {
    mkf_mixkf_destroy(h);
    return cuda_fail(e, "mkf_mixkf_create: scratch allocation", __FILE__, __LINE__);
  }
  *out = h;
  return MKF_OK;
}

extern "C" int mkf_mixkf_set_checkpoint_stride(mkf_mixkf_t h, int C) {
  MKF_ARG(h && C >= 0, "mkf_mixkf_set_checkpoint_stride: bad argument");
  return mix_set_stride(h, C == 0 ? mix_auto_stride(h) : std::min(C, std::max(1, h->maxT)));
}

extern "C" int mkf_mixkf_checkpoint_stride(mkf_mixkf_t h) { return h ? h->C : 0; }

extern "C" int mkf_mixkf_theta_size(mkf_mixkf_t h) { return h ? h->ng : 0; }

extern "C" int mkf_mixkf_set_theta_device(mkf_mixkf_t h, const double* d_theta, mkf_stream_t stream) {
  MKF_ARG(h && d_theta, "mkf_mixkf_set_theta_device: null argument");
  cudaStream_t s = (cudaStream_t)stream;
  const int n = h->ng + h->K * h->d * h->d;
  mix_prepare_kernel<<<(n + 255) / 256, 256, 0, s>>>(d_theta, h->d, h->K, h->mu, h->a, h->Lq, h->Q, h->sigma_d);
  MKF_CHECK_LAUNCH("mkf_mixkf_set_theta_device");
  MKF_CUDA(cudaMemcpyAsync(&h->sigma_h, h->sigma_d, sizeof(float), cudaMemcpyDeviceToHost, s));
  MKF_CUDA(cudaStreamSynchronize(s));
  h->have_theta = true;
  return MKF_OK;
}

extern "C" int mkf_mixkf_set_theta(mkf_mixkf_t h, const double* theta) {
  MKF_ARG(h && theta, "mkf_mixkf_set_theta: null argument");
  MKF_ARG(theta[h->ng - 1] > 0.0, "mkf_mixkf_set_theta: sigma must be positive");
  MKF_CUDA(cudaMemcpy(h->theta_dev, theta, sizeof(double) * h->ng, cudaMemcpyHostToDevice));
  return mkf_mixkf_set_theta_device(h, h->theta_dev, nullptr);
}

static MixArgs mix_args(mkf_mixkf* h, const int* det_off, const float* det) {
  MixArgs A;
  memset(&A, 0, sizeof(A));
  A.M.d = h->d; A.M.K = h->K; A.M.J = h->J; A.M.DD = h->DD;
  A.M.mu = h->mu; A.M.a = h->a; A.M.Lq = h->Lq; A.M.Q = h->Q; A.M.logpi = h->logpi; A.M.pi = h->pi;
  A.M.S0 = h->S0; A.M.sigma = h->sigma_h;
  A.M.fx = (float)h->fx; A.M.fy = (float)h->fy; A.M.cx = (float)h->cx; A.M.cy = (float)h->cy;
  A.n_tracks = h->n_tracks; A.C = h->C;
  A.n_frames = h->n_frames; A.frame_base = h->frame_base; A.Bm = h->Bm; A.mm = h->mm;
  A.pd = h->pd; A.kappa = h->kappa; A.det_off = det_off; A.det = reinterpret_cast<const float2*>(det);
  A.ck_off = h->ck_off; A.ck = h->ck; A.ll = h->ll; A.slots = h->slots; A.slot_floats = h->slot_floats;
  A.gacc = h->gacc; A.ng = h->ng; A.status = h->status;
  return A;
}

extern "C" int mkf_mixkf_forward(mkf_mixkf_t h, const int* d_det_off, const float* d_det, double* d_loglik,
                                 double* d_total, mkf_stream_t stream) {
  MKF_RANGE("mkf_mixkf_forward");
  MKF_ARG(h && d_det_off && d_det, "mkf_mixkf_forward: null argument");
  if (!h->have_theta) { set_error("mkf_mixkf_forward: set theta first"); return MKF_ERR_STATE; }
  cudaStream_t s = (cudaStream_t)stream;
  MixArgs A = mix_args(h, d_det_off, d_det);
  h->fwd_kernel<<<h->grid_f, h->tpb, h->smem_f, s>>>(A);
  MKF_CHECK_LAUNCH("mkf_mixkf_forward");
  h->fwd_C = h->C;
  if (d_loglik) MKF_CUDA(cudaMemcpyAsync(d_loglik, h->ll, sizeof(double) * h->n_tracks, cudaMemcpyDeviceToDevice, s));
  mix_total_kernel<<<1, 256, 0, s>>>(h->ll, h->n_tracks, d_total ? d_total : h->total);
  MKF_CHECK_LAUNCH("mkf_mixkf_forward: total");
  return MKF_OK;
}

extern "C" int mkf_mixkf_backward(mkf_mixkf_t h, const int* d_det_off, const float* d_det, double* d_grad,
                                  mkf_stream_t stream) {
  MKF_RANGE("mkf_mixkf_backward");
  MKF_ARG(h && d_det_off && d_det && d_grad, "mkf_mixkf_backward: null argument");
  if (!h->have_theta) { set_error("mkf_mixkf_backward: set theta first"); return MKF_ERR_STATE; }
  if (h->fwd_C != h->C) {
    set_error("mkf_mixkf_backward: run mkf_mixkf_forward first (its checkpoints are the backward's input)");
    return MKF_ERR_STATE;
  }
  cudaStream_t s = (cudaStream_t)stream;
  MixArgs A = mix_args(h, d_det_off, d_det);
  MKF_CUDA(cudaMemsetAsync(h->gacc, 0, sizeof(double) * (size_t)h->ng * h->grid, s));
  h->bwd_kernel<<<h->grid, h->tpb, h->smem_b, s>>>(A);
  MKF_CHECK_LAUNCH("mkf_mixkf_backward");
  mix_reduce_kernel<<<(h->ng + 255) / 256, 256, 0, s>>>(h->gacc, h->grid, h->ng, d_grad);
  MKF_CHECK_LAUNCH("mkf_mixkf_backward: reduce");
  return MKF_OK;
}

extern "C" int mkf_mixkf_status(mkf_mixkf_t h, int* status) {
  MKF_ARG(h && status, "mkf_mixkf_status: null argument");
  MKF_CUDA(cudaMemcpy(status, h->status, sizeof(int), cudaMemcpyDeviceToHost));
  return MKF_OK;
}

extern "C" int mkf_mixkf_destroy(mkf_mixkf_t h) {
  if (!h) return MKF_OK;
  void* ps[] = {h->mu, h->a, h->Lq, h->Q, h->logpi, h->pi, h->S0, h->sigma_d, h->theta_dev, h->n_frames,
                h->frame_base, h->ck_off, h->Bm, h->mm, h->pd, h->kappa, h->ck, h->ll, h->total, h->status,
                h->slots, h->gacc};
  for (void* p : ps) if (p) cudaFree(p);
  free(h->h_nf);
  delete h;
  return MKF_OK;
}

extern "C" int mkf_adam_step(double* d_theta, const double* d_grad, double* d_m, double* d_v, const uint8_t* d_mask,
                             int n, int step, double lr, double b1, double b2, double eps, int maximize,
                             mkf_stream_t stream) {
  MKF_RANGE("mkf_adam_step");
  MKF_ARG(d_theta && d_grad && d_m && d_v && n > 0 && step >= 1, "mkf_adam_step: bad argument");
  const double c1 = 1.0 - std::pow(b1, step), c2 = 1.0 - std::pow(b2, step);
  adam_kernel<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(d_theta, d_grad, d_m, d_v, d_mask, n, c1, c2, lr,
                                                                  b1, b2, eps, maximize ? 1.0 : -1.0);
  MKF_CHECK_LAUNCH("mkf_adam_step");
  return MKF_OK;
}
