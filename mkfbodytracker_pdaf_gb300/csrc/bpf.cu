// bpf.cu -- bootstrap particle filter over the mixture-of-MRRW motion model.
//
// Reference structure: pf2D ParticleFilter::update/predict/resample
// (pf2D.cpp:148-210, 90-102, 225-268) with the motion of my_gmm/KF_model
// (my_gmm.cpp:53-58: x' = g x + (1-g) mu, Q = (1-g^2) Sigma, generalised to
// A_k = diag(a_k), Q_k = Lq_k Lq_k^T), and the PDA clutter likelihood whose
// reference analogue is the Pa/clutter-floor mixture at pfPose.cpp:261.
//
// Two launch shapes share the per-particle device code:
//  * batched: one persistent kernel; each CTA owns one track at a time and
//    runs all its frames with the weights, scan and ancestors in shared
//    memory (particle states in a per-CTA global slot, L2-resident);
//  * streaming: one track with up to 2^22 particles, three grid-wide kernels
//    per frame: propagate+score+estimate partials (one wave of resident
//    blocks over contiguous tiles, the model in shared memory, the next
//    ancestor state prefetched with cp.async), quantised tile sums, and the
//    per-tile prefix plus threshold search (tiles in whole waves).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "mkf_common.cuh"

namespace mkf {

constexpr float kZMin = 0.05f;
constexpr float kTwoPi = 6.283185307179586f;

// ------------------------------------------------------------------ model
struct DevModels {
  int n, d, K, J;
  bool diag;          // every Lq_k diagonal
  float *a, *mb, *mu, *Lq, *Ld, *S0c, *cumpi, *Bm, *mm;   // device
  float fx, fy, cx, cy;
};

static void free_models(DevModels& m) {
  float* ps[] = {m.a, m.mb, m.mu, m.Lq, m.Ld, m.S0c, m.cumpi, m.Bm, m.mm};
  for (float* p : ps) if (p) cudaFree(p);
  memset(&m, 0, sizeof(m));
}

static int upload(float** dst, const std::vector<float>& src) {
  MKF_CUDA(cudaMalloc(dst, std::max<size_t>(1, src.size()) * sizeof(float)));
  MKF_CUDA(cudaMemcpy(*dst, src.data(), src.size() * sizeof(float), cudaMemcpyHostToDevice));
  return MKF_OK;
}

static int build_models(const mkf_bpf_models* M, DevModels& out) {
  MKF_ARG(M && M->n_models > 0, "models: n_models must be > 0");
  MKF_ARG(M->d == 12 || M->d == 24, "models: d must be 12 or 24");
  MKF_ARG(M->K >= 1 && M->K <= MKF_MAX_K, "models: K out of range");
  MKF_ARG(M->J >= 1 && M->J <= MKF_MAX_J, "models: J out of range");
  MKF_ARG(M->a && M->mu && M->Lq && M->S0c && M->pi && M->Bm && M->mm, "models: null array");
  const int n = M->n_models, d = M->d, K = M->K, J = M->J, DD = d * (d + 1) / 2;
  const size_t nKd = (size_t)n * K * d;
  std::vector<float> mb(nKd), Ld(nKd), cum((size_t)n * K);
  bool diag = true;
  for (size_t i = 0; i < nKd; ++i)
    mb[i] = (float)((1.0 - (double)M->a[i]) * (double)M->mu[i]);
  for (int p = 0; p < n; ++p)
    for (int k = 0; k < K; ++k) {
      const float* L = M->Lq + ((size_t)p * K + k) * DD;
      for (int r = 0; r < d; ++r) {
        for (int c = 0; c < r; ++c) if (L[r * (r + 1) / 2 + c] != 0.0f) diag = false;
        Ld[((size_t)p * K + k) * d + r] = L[r * (r + 1) / 2 + r];
      }
    }
  for (int p = 0; p < n; ++p) {   // sequential float32 cumulation (the oracle reads this array)
    float acc = 0.0f;
    for (int c = 0; c < K; ++c) { acc += M->pi[(size_t)p * K + c]; cum[(size_t)p * K + c] = acc; }
  }
  memset(&out, 0, sizeof(out));
  out.n = n; out.d = d; out.K = K; out.J = J; out.diag = diag;
  out.fx = M->fx; out.fy = M->fy; out.cx = M->cx; out.cy = M->cy;
  auto vec = [](const float* p, size_t cnt) { return std::vector<float>(p, p + cnt); };
  int st = upload(&out.a, vec(M->a, nKd));   // stops at the first failure
  if (st == MKF_OK) st = upload(&out.mb, mb);
  if (st == MKF_OK) st = upload(&out.mu, vec(M->mu, nKd));
  if (st == MKF_OK) st = upload(&out.Lq, vec(M->Lq, (size_t)n * K * DD));
  if (st == MKF_OK) st = upload(&out.Ld, Ld);
  if (st == MKF_OK) st = upload(&out.S0c, vec(M->S0c, (size_t)n * K * DD));
  if (st == MKF_OK) st = upload(&out.cumpi, cum);
  if (st == MKF_OK) st = upload(&out.Bm, vec(M->Bm, (size_t)n * J * 3 * d));
  if (st == MKF_OK) st = upload(&out.mm, vec(M->mm, (size_t)n * J * 3));
  return st;
}

// ------------------------------------------------------------------ per-particle math
// parameters of one model as seen by one particle (pointers into shared or global)
struct PView {
  const float *a, *mb, *mu, *Lq, *Ld, *S0c, *cumpi, *Bm, *mm;
  const uint8_t* ktab;     // optional component table (kPickBins entries), or null
  int K, J;
  float fx, fy, cx, cy;
};

// mixture component of a particle-frame (mkf_common.cuh: by count, or through
// the track's kPickBins table when the view has one)
__device__ __forceinline__ int pick_component(const PView& p, float u, int ubin) {
  return p.ktab ? pick_component_table_bin(p.ktab, p.cumpi, p.K, u, ubin) : pick_component(p.cumpi, p.K, u);
}

template <int D>
__device__ __forceinline__ void prior_sample(const PView& p, const float* eps, float uc, int ubin, float* x) {
  constexpr int DD = D * (D + 1) / 2;
  int k = pick_component(p, uc, ubin);
  const float* L = p.S0c + k * DD;
#pragma unroll
  for (int r = 0; r < D; ++r) {
    float s = p.mu[k * D + r];
#pragma unroll
    for (int c = 0; c <= r; ++c) s = fmaf(L[r * (r + 1) / 2 + c], eps[c], s);
    x[r] = s;
  }
}

__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }

// x' = A_k x + (I - A_k) mu_k + L_k eps.  VEC: float4 parameter loads (rows of
// a, mb, Ld, Bm are 16-byte aligned since D % 4 == 0); otherwise scalar loads.
template <int D, bool DIAG, bool VEC = true>
__device__ __forceinline__ void propagate(const PView& p, const float* eps, float uc, int ubin, float* x) {
  constexpr int DD = D * (D + 1) / 2;
  int k = pick_component(p, uc, ubin);
  const float* a = p.a + k * D;
  const float* mb = p.mb + k * D;
  if (DIAG) {
    const float* l = p.Ld + k * D;
    if (VEC) {
      // x[r] = fmaf(l[r], eps[r], fmaf(a[r], x[r], mb[r])) two dimensions per instruction
#pragma unroll
      for (int r = 0; r < D; r += 4) {
        float4 av = ld4(a + r), mv = ld4(mb + r), lv = ld4(l + r);
        float2 t0 = pk_fma(make_float2(av.x, av.y), make_float2(x[r], x[r + 1]), make_float2(mv.x, mv.y));
        float2 t1 = pk_fma(make_float2(av.z, av.w), make_float2(x[r + 2], x[r + 3]), make_float2(mv.z, mv.w));
        t0 = pk_fma(make_float2(lv.x, lv.y), make_float2(eps[r], eps[r + 1]), t0);
        t1 = pk_fma(make_float2(lv.z, lv.w), make_float2(eps[r + 2], eps[r + 3]), t1);
        x[r] = t0.x; x[r + 1] = t0.y; x[r + 2] = t1.x; x[r + 3] = t1.y;
      }
    } else {
#pragma unroll
      for (int r = 0; r < D; ++r) x[r] = fmaf(l[r], eps[r], fmaf(a[r], x[r], mb[r]));
    }
  } else {
    const float* L = p.Lq + k * DD;
    float xn[D];
#pragma unroll
    for (int r = 0; r < D; ++r) {
      float s = fmaf(a[r], x[r], mb[r]);
#pragma unroll
      for (int c = 0; c <= r; ++c) s = fmaf(L[r * (r + 1) / 2 + c], eps[c], s);
      xn[r] = s;
    }
#pragma unroll
    for (int r = 0; r < D; ++r) x[r] = xn[r];
  }
}

// Per-track constants of the likelihood.  Detections and the projected joint
// are both scaled by k = sqrt(log2(e) / (2 sigma^2)), so that a detection's
// Gaussian kernel exp(-|z - pi|^2 / (2 sigma^2)) is the single exponential
// 2^(-|k z - k pi|^2).
struct LikConst {
  float k;                          // detection scale
  float fxk, fyk, cxk, cyk;         // camera scaled by k
  float norm, floor_, log_kappa;    // P_D / (2 pi sigma^2), (1 - P_D) kappa, log kappa
};

__device__ __forceinline__ LikConst lik_const(const PView& p, float kappa, float pd, float sigma) {
  LikConst L;
  L.k = sqrtf(0.72134752044448170f / (sigma * sigma));
  L.fxk = p.fx * L.k; L.fyk = p.fy * L.k; L.cxk = p.cx * L.k; L.cyk = p.cy * L.k;
  L.norm = pd / (kTwoPi * sigma * sigma);
  L.floor_ = (1.0f - pd) * kappa;
  L.log_kappa = __logf(kappa);
  return L;
}

__device__ __forceinline__ float ex2_neg(float s) {   // 2^(-s), MUFU.EX2
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(-s));
  return r;
}

// Shared-memory detection layout of one joint (2 MKF_MAX_DET floats): pairs of
// detections as (x_i, x_i+1, y_i, y_i+1), scaled by L.k, so that one 16-byte
// load gives two detections' x and y as packed pairs.
__device__ __forceinline__ void stage_det(float* dj, int i, float2 z, float k) {
  dj[(i >> 1) * 4 + (i & 1)] = z.x * k;
  dj[(i >> 1) * 4 + 2 + (i & 1)] = z.y * k;
}

// Stage slot i of joint j's list for a frame whose list has n entries (clamped
// to MKF_MAX_DET): the detection, scaled by k, or for n <= i < n rounded up to
// a multiple of 4, a +inf padding entry.
__device__ __forceinline__ void stage_list_slot(float* dj, int i, int n, const float2* det, int lo, float k) {
  if (i < n) stage_det(dj, i, det[lo + i], k);
  else if (i < ((n + 3) & ~3)) stage_det(dj, i, make_float2(INFINITY, INFINITY), 1.0f);
}

// log[(1-P_D) kappa + P_D sum_i N(z_i; pi(x), sigma^2 I)] summed over measured
// joints; det holds each joint's detections in the stage_det layout
template <int D, bool VEC = true>
__device__ __forceinline__ float loglik(const PView& p, const float* x, const int* cnt, const float* det,
                                        const LikConst& L) {
  float ll = 0.0f;
  // unrolled to the largest joint count, so that the joints' independent
  // chains (projection, detection sum, logarithm) can overlap
#pragma unroll
  for (int j = 0; j < MKF_MAX_J; ++j) {
    if (j >= p.J) break;
    const float* B = p.Bm + j * 3 * D;
    float q0, q1, q2;
    if (VEC) {
      // two partial sums per row (even and odd dimensions), one packed pair
      float2 p0 = make_float2(p.mm[j * 3 + 0], 0.0f), p1 = make_float2(p.mm[j * 3 + 1], 0.0f);
      float2 p2 = make_float2(p.mm[j * 3 + 2], 0.0f);
#pragma unroll
      for (int c = 0; c < D; c += 4) {
        float4 b0 = ld4(B + c), b1 = ld4(B + D + c), b2 = ld4(B + 2 * D + c);
        const float2 xa = make_float2(x[c], x[c + 1]), xb = make_float2(x[c + 2], x[c + 3]);
        p0 = pk_fma(make_float2(b0.x, b0.y), xa, p0);
        p1 = pk_fma(make_float2(b1.x, b1.y), xa, p1);
        p2 = pk_fma(make_float2(b2.x, b2.y), xa, p2);
        p0 = pk_fma(make_float2(b0.z, b0.w), xb, p0);
        p1 = pk_fma(make_float2(b1.z, b1.w), xb, p1);
        p2 = pk_fma(make_float2(b2.z, b2.w), xb, p2);
      }
      q0 = p0.x + p0.y; q1 = p1.x + p1.y; q2 = p2.x + p2.y;
    } else {
      // the packed path's two partial sums, one lane at a time, so that both
      // load widths give bit-identical log-likelihoods
      float e0 = p.mm[j * 3 + 0], e1 = p.mm[j * 3 + 1], e2 = p.mm[j * 3 + 2];
      float o0 = 0.0f, o1 = 0.0f, o2 = 0.0f;
#pragma unroll
      for (int c = 0; c < D; c += 2) {
        e0 = fmaf(B[c], x[c], e0);
        o0 = fmaf(B[c + 1], x[c + 1], o0);
        e1 = fmaf(B[D + c], x[c], e1);
        o1 = fmaf(B[D + c + 1], x[c + 1], o1);
        e2 = fmaf(B[2 * D + c], x[c], e2);
        o2 = fmaf(B[2 * D + c + 1], x[c + 1], o2);
      }
      q0 = e0 + o0; q1 = e1 + o1; q2 = e2 + o2;
    }
    if (!(q2 > kZMin)) { ll = __fadd_rn(ll, L.log_kappa); continue; }
    const float iz = __fdividef(1.0f, q2);
    const float u = fmaf(L.fxk * q0, iz, L.cxk), v = fmaf(L.fyk * q1, iz, L.cyk);
    // four partial sums (detection i into sum i mod 4) so the exponentials of
    // a list overlap; sums (0, 1) and (2, 3) are packed pairs.  The list is
    // padded with +inf detections to a multiple of four (stage_list): their
    // terms are 2^-inf = +0 exactly, so every group runs the same code.  The
    // loop is unrolled to the longest list, so that the groups' loads and
    // exponentials can be issued ahead of the sums.
    float2 accA = make_float2(0.0f, 0.0f), accB = make_float2(0.0f, 0.0f);
    const float* dj = det + j * 2 * MKF_MAX_DET;
    const float2 uu = make_float2(u, u), vv = make_float2(v, v);
    const int n = (cnt[j] + 3) & ~3;
#pragma unroll
    for (int i = 0; i < MKF_MAX_DET; i += 4) {
      if (i >= n) break;
      const float4 g0 = ld4(dj + 2 * i), g1 = ld4(dj + 2 * i + 4);
      const float2 dxA = pk_sub(make_float2(g0.x, g0.y), uu), dyA = pk_sub(make_float2(g0.z, g0.w), vv);
      const float2 dxB = pk_sub(make_float2(g1.x, g1.y), uu), dyB = pk_sub(make_float2(g1.z, g1.w), vv);
      const float2 sA = pk_fma(dyA, dyA, pk_mul(dxA, dxA)), sB = pk_fma(dyB, dyB, pk_mul(dxB, dxB));
      accA = pk_add(accA, make_float2(ex2_neg(sA.x), ex2_neg(sA.y)));
      accB = pk_add(accB, make_float2(ex2_neg(sB.x), ex2_neg(sB.y)));
    }
    const float acc = (accA.x + accA.y) + (accB.x + accB.y);
    // __fadd_rn: never merged with the multiply inside __logf, so every kernel
    // that inlines this function rounds the log-likelihood the same way
    ll = __fadd_rn(ll, __logf(fmaf(L.norm, acc, L.floor_)));
  }
  return ll;
}

// ------------------------------------------------------------------ batched persistent kernel
struct BatchArgs {
  int n_tracks, K, J, Nmax;
  const int4* meta;                 // n_particles, n_frames, model_index, track_id
  const long long* fbase;
  const unsigned long long* seed;
  const float4* obs;                // kappa, p_detect, sigma, 0
  const int* order;
  int* counter;
  DevModels m;
  const int* det_off;
  const float2* det;
  float* est;
  float* loglik;
  float* ess;
  int* status;
  float* scratch;                   // gridDim.x * 2 * D * Nmax
  int* anc;                         // LOW variant: gridDim.x * Nmax ancestors
  int dbg_track;
  float* dbg_w;
  int* dbg_anc;
};

__host__ __device__ constexpr int pad4(int n) { return (n + 3) & ~3; }

// batched per-CTA state slot: D/4 planes of Nmax float4, particle i's
// dimensions 4g..4g+3 in plane g (a warp's 32 particles read 512 contiguous bytes)
template <int D>
__device__ __forceinline__ void load_state(const float* slot, int Nmax, int i, float* x) {
  const float4* p = reinterpret_cast<const float4*>(slot);
#pragma unroll
  for (int g = 0; g < D / 4; ++g) {
    const float4 v = p[(size_t)g * Nmax + i];
    x[4 * g] = v.x; x[4 * g + 1] = v.y; x[4 * g + 2] = v.z; x[4 * g + 3] = v.w;
  }
}
template <int D>
__device__ __forceinline__ void store_state(float* slot, int Nmax, int i, const float* x) {
  float4* p = reinterpret_cast<float4*>(slot);
#pragma unroll
  for (int g = 0; g < D / 4; ++g) p[(size_t)g * Nmax + i] = make_float4(x[4 * g], x[4 * g + 1], x[4 * g + 2], x[4 * g + 3]);
}

// shared-memory parameter block: a | mb | L | Bm | mm | cumpi, every section 16-byte aligned
template <int D>
__host__ __device__ constexpr int params_floats(int K, int J, bool diag) {
  return 2 * K * D + pad4(diag ? K * D : K * D * (D + 1) / 2) + J * 3 * D + pad4(J * 3) + pad4(K);
}

// Batched persistent kernel: CTAs take tracks from an atomic queue in
// longest-first order, one track at a time.  Particle states live in this
// CTA's global slot (two buffers of D/4 float4 planes of Nmax particles,
// partly L2-resident); per-particle weights, prefix sums and ancestors in
// shared memory (the layout of each variant below), then the track's model.
// Per frame: propagate + score (accumulating the estimate sums), block max,
// weights and ESS, exact systematic resampling, the gather folded into the
// next frame's propagate.  The next frame's detection lists are copied with
// cp.async while a frame resamples, and the Philox words and resampling
// constants that do not depend on the particle are formed once per frame.
// Code variants chosen by the autotuner: VEC (float4 vs scalar parameter loads)
// and SEARCH (ancestors by binary search over the shared prefix sums, 12 Nmax
// bytes of shared memory, vs the scatter walk over each thread's chunk, 8 Nmax).
// LOW (with SEARCH): 8 Nmax bytes of shared memory, so that three CTAs of the
// largest tracks fit on an SM; the log-weights are kept in the prefix array's
// entries, and the ancestors in shared memory behind the N prefix entries
// when 3 N <= 2 Nmax, else in the CTA's global slot (L2).
template <int D, bool DIAG, int TBMAX, int MINB, bool VEC, bool SEARCH, bool PAIR = false, bool LOW = false>
__global__ void __launch_bounds__(TBMAX, MINB) bpf_batched_kernel(BatchArgs A) {
  static_assert(!LOW || (SEARCH && !PAIR), "the LOW layout is a SEARCH variant");
  extern __shared__ __align__(16) unsigned char smem[];
  const int TB = blockDim.x, tid = threadIdx.x;
  constexpr int NV = D + 3;
  const int Nmax = A.Nmax;
  // SEARCH: sQ (u64) | sA (log-weights, weights, then ancestors, as int bits)
  // LOW: sQ (log-weights in the low word, then integer weights, then prefix
  //      sums); sA (ancestors) in global memory
  // scatter: sW (log-weights then weights) | sA (ancestors)
  uint64_t* sQ = reinterpret_cast<uint64_t*>(smem);
  float* sW = reinterpret_cast<float*>(smem);
  int* const sA_slot = LOW ? A.anc + (size_t)blockIdx.x * Nmax : reinterpret_cast<int*>(smem + (SEARCH ? 8 : 4) * (size_t)Nmax);
  float* sP = reinterpret_cast<float*>(smem + (LOW ? 8 : SEARCH ? 12 : 8) * (size_t)Nmax);   // Nmax % 32 == 0
  const int K = A.K, J = A.J;
  const int Lsz = pad4(DIAG ? K * D : K * D * (D + 1) / 2);
  float* s_a = sP;
  float* s_mb = s_a + K * D;
  float* s_L = s_mb + K * D;
  float* s_Bm = s_L + Lsz;
  float* s_mm = s_Bm + J * 3 * D;
  float* s_cum = s_mm + pad4(J * 3);
  float* s_det = sP + params_floats<D>(K, J, DIAG);
  int* s_cnt = reinterpret_cast<int*>(s_det + MKF_MAX_J * 2 * MKF_MAX_DET);
  float* s_red = reinterpret_cast<float*>(s_cnt + 8);                    // 32*NV floats
  uint64_t* s_red64 = reinterpret_cast<uint64_t*>(s_red + 32 * NV + 2);
  s_red64 = reinterpret_cast<uint64_t*>((reinterpret_cast<uintptr_t>(s_red64) + 7) & ~uintptr_t(7));
  uint8_t* s_ktab = reinterpret_cast<uint8_t*>(s_red64 + 34);
  __shared__ int s_item;
  __shared__ int s_flag;
  __shared__ PhiloxPre s_pre[D / 4];   // this frame's item-independent Philox words per stream
  __shared__ PhiloxKeys s_keys;        // this track's round keys
  // the next frame's list offsets and raw detections, copied with cp.async
  // while this frame runs (thread q < J MKF_MAX_DET owns slot q)
  __shared__ int s_offn[MKF_MAX_J + 1];
  __shared__ int s_nn[MKF_MAX_J];   // the next frame's list lengths
  __shared__ int s_lmax;            // this frame's max log-weight, order-preserving int form
  __shared__ uint32_t s_U;          // this frame's resampling uniform
  __shared__ RsThresh s_th;         // and the resampling rule's constants (SEARCH)
  __shared__ RsStep s_st1, s_st4;
  __shared__ __align__(8) float2 s_raw[MKF_MAX_J * MKF_MAX_DET];

  float* xa0 = A.scratch + (size_t)blockIdx.x * 2 * D * Nmax;
  float* xb0 = xa0 + (size_t)D * Nmax;

  for (;;) {
    if (tid == 0) s_item = atomicAdd(A.counter, 1);
    __syncthreads();
    const int item = s_item;
    __syncthreads();
    if (item >= A.n_tracks) break;
    const int b = A.order[item];
    const int4 mt = A.meta[b];
    const int N = mt.x, T = mt.y, mi = mt.z;
    const uint32_t trk = (uint32_t)mt.w;
    const long long g0 = A.fbase[b];
    const unsigned long long seed = A.seed[b];
    const float4 ob = A.obs[b];
    {  // stage this track's model in shared memory
      const float* ga = A.m.a + (size_t)mi * K * D;
      const float* gmb = A.m.mb + (size_t)mi * K * D;
      const float* gL = DIAG ? A.m.Ld + (size_t)mi * K * D : A.m.Lq + (size_t)mi * K * D * (D + 1) / 2;
      const float* gc = A.m.cumpi + (size_t)mi * K;
      const float* gB = A.m.Bm + (size_t)mi * J * 3 * D;
      const float* gm = A.m.mm + (size_t)mi * J * 3;
      for (int i = tid; i < K * D; i += TB) { s_a[i] = ga[i]; s_mb[i] = gmb[i]; }
      for (int i = tid; i < (DIAG ? K * D : K * D * (D + 1) / 2); i += TB) s_L[i] = gL[i];
      for (int i = tid; i < K; i += TB) s_cum[i] = gc[i];
      for (int i = tid; i < J * 3 * D; i += TB) s_Bm[i] = gB[i];
      for (int i = tid; i < J * 3; i += TB) s_mm[i] = gm[i];
      if (tid == 0) { s_flag = 0; s_keys = philox_keys(seed, trk); }
      if (tid < D / 4) s_pre[tid] = philox_pre(seed, trk, kFramePrior, (uint32_t)tid);
      __syncthreads();
      build_pick_table(s_cum, K, s_ktab, tid, TB);
    }
    __syncthreads();
    PView pv;
    pv.a = s_a; pv.mb = s_mb; pv.Lq = s_L; pv.Ld = s_L; pv.cumpi = s_cum; pv.Bm = s_Bm; pv.mm = s_mm;
    pv.ktab = s_ktab;
    pv.mu = A.m.mu + (size_t)mi * K * D;
    pv.S0c = A.m.S0c + (size_t)mi * K * D * (D + 1) / 2;
    pv.K = K; pv.J = J; pv.fx = A.m.fx; pv.fy = A.m.fy; pv.cx = A.m.cx; pv.cy = A.m.cy;
    const bool dbg = (A.dbg_w != nullptr) && (b == A.dbg_track);
    const LikConst LK = lik_const(pv, ob.x, ob.y, ob.z);
    // LOW: the ancestors of a track with 3 N <= 2 Nmax fit in shared memory
    // behind its N prefix entries, else they use the CTA's global slot
    int* const sA = (LOW && 3 * N <= 2 * Nmax) ? reinterpret_cast<int*>(sQ + N) : sA_slot;

    float* xa = xa0;
    float* xb = xb0;
    // prior draw (frame index 0xFFFFFFFF), identity ancestry
    for (int i = tid; i < N; i += TB) {
      float eps[D], x[D];
      int ub;
      float uc = particle_draws_pre<D>(s_pre, s_keys, (uint32_t)i, eps, ub);
      prior_sample<D>(pv, eps, uc, ub, x);
      store_state<D>(xa, Nmax, i, x);
      sA[i] = i;
    }
    __syncthreads();

    // contiguous chunk per thread, an odd number of elements so that a warp's
    // chunk-wise shared-memory accesses fall in distinct banks
    int E = (N + TB - 1) / TB;
    if (E > 1 && !(E & 1)) ++E;
    const int j0 = min(N, tid * E), j1 = min(N, j0 + E);
    // staging slot q = tid of a thread with tid < J MKF_MAX_DET (<= 64 <= TB,
    // so one slot at most): list q / MKF_MAX_DET, entry q % MKF_MAX_DET
    for (int t = 0; t < T; ++t) {
      const long long g = g0 + t;
      // this frame's detection lists: read directly for the first frame (each
      // staging thread reads its list's bounds itself, so one barrier
      // suffices), else from the copies made during the previous frame
      if (tid < J * MKF_MAX_DET) {
        const int qj = tid / MKF_MAX_DET, qi = tid % MKF_MAX_DET;
        int n, nc;
        float2 z = make_float2(0.0f, 0.0f);
        if (t == 0) {
          const int lo = A.det_off[g * J + qj];
          n = A.det_off[g * J + qj + 1] - lo;
          nc = min(max(n, 0), MKF_MAX_DET);
          if (qi < nc) z = A.det[lo + qi];
        } else {
          n = s_nn[qj];
          nc = min(max(n, 0), MKF_MAX_DET);
          if (qi < nc) z = s_raw[tid];
        }
        if (qi == 0) {
          if (n > MKF_MAX_DET) atomicOr(&s_flag, MKF_ST_TRUNC);
          s_cnt[qj] = nc;
        }
        float* dj = s_det + qj * 2 * MKF_MAX_DET;
        if (qi < nc) stage_det(dj, qi, z, LK.k);
        else if (qi < pad4(nc)) stage_det(dj, qi, make_float2(INFINITY, INFINITY), 1.0f);
      }
      // the next frame's offsets, copied while this frame runs
      if (t + 1 < T && tid <= J) cp_async4(&s_offn[tid], A.det_off + (g + 1) * J + tid);
      cp_async_commit();
      if (tid < D / 4) s_pre[tid] = philox_pre(seed, trk, (uint32_t)t, (uint32_t)tid);
      if (tid == 0) s_lmax = float_ordered(-INFINITY);
      if (tid == 32) s_U = resample_uniform(seed, trk, (uint32_t)t);
      __syncthreads();

      // ---- propagate from the resampled set and score.  Besides the
      // log-weights, the non-pair loop accumulates the estimate sums with the
      // frame's upper bound Lub of any log-likelihood (every Gaussian kernel is
      // <= 1) as the shift; they are used when the frame's max M is within 60
      // of Lub (no weight that matters can underflow), else the sums are
      // formed again below with M as the shift.
      float lmax = -INFINITY;
      float Lub = 0.0f;
      for (int j = 0; j < J; ++j) Lub += fmaxf(LK.log_kappa, __logf(fmaf(LK.norm, (float)s_cnt[j], LK.floor_)));
      float fs = 0.0f, fs2 = 0.0f;
      float2 fv[D / 2];
#pragma unroll
      for (int r = 0; r < D / 2; ++r) fv[r] = make_float2(0.0f, 0.0f);
      if (PAIR) {
        // particles i and i + TB of this thread together: two independent
        // dependency chains for the scheduler (same particles, same results)
        for (int i = tid; i < N; i += 2 * TB) {
          const int i2 = i + TB;
          const bool two = i2 < N;
          const int an = sA[i], an2 = two ? sA[i2] : an;
          float x[D], eps[D], y[D], eps2[D];
          load_state<D>(xa, Nmax, an, x);
          load_state<D>(xa, Nmax, an2, y);
          int ub, ub2;
          const float uc = particle_draws_pre<D>(s_pre, s_keys, (uint32_t)i, eps, ub);
          const float uc2 = particle_draws_pre<D>(s_pre, s_keys, (uint32_t)i2, eps2, ub2);
          propagate<D, DIAG, VEC>(pv, eps, uc, ub, x);
          propagate<D, DIAG, VEC>(pv, eps2, uc2, ub2, y);
          store_state<D>(xb, Nmax, i, x);
          const float ll = loglik<D, VEC>(pv, x, s_cnt, s_det, LK);
          if (SEARCH) sA[i] = __float_as_int(ll); else sW[i] = ll;
          lmax = fmaxf(lmax, ll);
          if (two) {
            store_state<D>(xb, Nmax, i2, y);
            const float ll2 = loglik<D, VEC>(pv, y, s_cnt, s_det, LK);
            if (SEARCH) sA[i2] = __float_as_int(ll2); else sW[i2] = ll2;
            lmax = fmaxf(lmax, ll2);
          }
        }
      } else {
        for (int i = tid; i < N; i += TB) {
          const int an = sA[i];
          float x[D], eps[D];
          load_state<D>(xa, Nmax, an, x);
          int ub;
          float uc = particle_draws_pre<D>(s_pre, s_keys, (uint32_t)i, eps, ub);
          propagate<D, DIAG, VEC>(pv, eps, uc, ub, x);
          store_state<D>(xb, Nmax, i, x);
          float ll = loglik<D, VEC>(pv, x, s_cnt, s_det, LK);
          if (LOW) sQ[i] = (uint64_t)__float_as_uint(ll);
          else if (SEARCH) sA[i] = __float_as_int(ll);
          else sW[i] = ll;
          lmax = fmaxf(lmax, ll);
          const float wl = __expf(ll - Lub);
          fs += wl;
          fs2 = fmaf(wl, wl, fs2);
          const float2 ww = make_float2(wl, wl);
#pragma unroll
          for (int r = 0; r < D / 2; ++r) fv[r] = pk_fma(ww, make_float2(x[2 * r], x[2 * r + 1]), fv[r]);
        }
      }
      if (tid <= J) cp_async_wait_all();   // s_offn, visible after the barrier below
      // block max: one shared atomic per warp and one barrier (the max is
      // order independent, so M is the same as any reduction tree's)
      {
        const float wmx = warp_max(lmax);
        if ((tid & 31) == 0) atomicMax(&s_lmax, float_ordered(wmx));
      }
      __syncthreads();
      const float M = float_unordered(s_lmax);
      // the next frame's detections, copied while this frame resamples
      if (tid < J * MKF_MAX_DET && t + 1 < T) {
        const int qj = tid / MKF_MAX_DET, qi = tid % MKF_MAX_DET;
        const int lo = s_offn[qj], n = s_offn[qj + 1] - lo;
        if (qi == 0) s_nn[qj] = n;
        if (qi < min(max(n, 0), MKF_MAX_DET)) cp_async8(&s_raw[tid], A.det + lo + qi);
      }
      cp_async_commit();
      const bool fb = !(M > -INFINITY) || !(M < INFINITY);
      const bool fused = !PAIR && (M - Lub >= -60.0f);

      // ---- weights normalised to the max, weighted-mean estimate, ESS.
      // SEARCH: each thread weights its own contiguous chunk and writes the
      // integer weights straight into the prefix array (the max weight is
      // exactly 1, or every weight is 0, so the quantisation exponent is 1);
      // one combined pass then reduces the estimate sums and scans the chunk sums.
      float acc[NV];
#pragma unroll
      for (int c = 0; c < NV; ++c) acc[c] = 0.0f;   // s, s2, wmax, v[D]
      uint64_t cs = 0;
      if (SEARCH) {
#pragma unroll 4
        for (int j = j0; j < j1; ++j) {
          const float ll = LOW ? __uint_as_float((uint32_t)sQ[j]) : __int_as_float(sA[j]);
          float w = fb ? 0.0f : (ll == M ? 1.0f : __expf(ll - M));
          if (!(w >= 0.0f)) w = 0.0f;
          const uint64_t q = quantize39(w);
          sQ[j] = q;
          cs += q;
          if (dbg) A.dbg_w[(size_t)t * N + j] = w;
          if (!fused) {
            acc[0] += w;
            acc[1] = fmaf(w, w, acc[1]);
            float xi[D];
            load_state<D>(xb, Nmax, j, xi);
#pragma unroll
            for (int r = 0; r < D; ++r) acc[3 + r] = fmaf(w, xi[r], acc[3 + r]);
          }
        }
      } else {
        for (int i = tid; i < N; i += TB) {
          const float ll = sW[i];
          float w = fb ? 0.0f : (ll == M ? 1.0f : __expf(ll - M));
          if (!(w >= 0.0f)) w = 0.0f;
          sW[i] = w;
          if (dbg) A.dbg_w[(size_t)t * N + i] = w;
          acc[2] = fmaxf(acc[2], w);
          if (!fused) {
            acc[0] += w;
            acc[1] = fmaf(w, w, acc[1]);
            float xi[D];
            load_state<D>(xb, Nmax, i, xi);
#pragma unroll
            for (int r = 0; r < D; ++r) acc[3 + r] = fmaf(w, xi[r], acc[3 + r]);
          }
        }
      }
      if (fused) {
        acc[0] = fs;
        acc[1] = fs2;
#pragma unroll
        for (int r = 0; r < D / 2; ++r) { acc[3 + 2 * r] = fv[r].x; acc[4 + 2 * r] = fv[r].y; }
      }
      uint64_t P = 0, Qt = 0;
      {
        const int lane = tid & 31, w = tid >> 5, nw = (TB + 31) >> 5;
        // the warp's sums of acc (column 2, the max weight, is a max and only
        // the scatter variant uses it): lane c << SH ends with column c's sum
        constexpr int NP = NV <= 16 ? 16 : 32, SH = NV <= 16 ? 1 : 0;
        float r[NP];
#pragma unroll
        for (int c = 0; c < NP; ++c) r[c] = (c < NV && c != 2) ? acc[c] : 0.0f;
        const float wm = SEARCH ? 0.0f : warp_max(acc[2]);
        warp_sum_split<NP>(r, lane);
        const uint64_t inc = SEARCH ? warp_incl_scan_u64(cs, lane) : 0ull;
        // (s_red and s_red64 were last read before the previous frame's final barrier)
        if (!(lane & ((1 << SH) - 1)) && (lane >> SH) < NV)
          s_red[w * NV + (lane >> SH)] = (lane >> SH) == 2 ? wm : r[0];
        if (SEARCH && lane == 31) s_red64[w] = inc;
        __syncthreads();
        if (tid < 32) {
          if (SEARCH) {   // warp 0: exclusive scan of the warps' chunk totals
            const uint64_t v = lane < nw ? s_red64[lane] : 0ull;
            const uint64_t vi = warp_incl_scan_u64(v, lane);
            __syncwarp();
            if (lane < nw) s_red64[lane] = vi - v;
            if (lane == 31) s_red64[32] = vi;
          }
          if (tid < NV) {   // thread c alone reads column c, then stores its total in slot c
            float r = 0.0f;
            for (int q = 0; q < nw; ++q) r = (tid == 2) ? fmaxf(r, s_red[q * NV + tid]) : r + s_red[q * NV + tid];
            s_red[tid] = r;
          }
        }
        __syncthreads();
        if (SEARCH) {
          P = s_red64[w] + inc - cs;
          Qt = s_red64[32];
          // the rule's constants (64-bit divisions) once, published by the
          // prefix pass's barrier
          if (tid == 0 && Qt != 0) {
            const RsThresh th = rs_thresh_setup(Qt, N, s_U);
            s_th = th;
            s_st1 = rs_step_setup(th, (uint32_t)TB);
            s_st4 = rs_step_setup(th, 4u * (uint32_t)TB);
          }
        }
      }
      const float S = s_red[0], S2 = s_red[1], Wmax = s_red[2];
      if (tid < D) A.est[(size_t)g * D + tid] = s_red[3 + tid] / S;
      if (tid == 0) {
        A.loglik[g] = (fused ? Lub : M) + __logf(S) - __logf((float)N);
        A.ess[g] = S * S / S2;
        if (fb) s_flag |= MKF_ST_FALLBACK | MKF_ST_NAN;
      }

      // ---- exact systematic resampling: SEARCH: chunk prefix sums in place,
      // then a binary search per target; otherwise chunk sums, block scan and
      // a scatter walk per chunk
      const uint32_t U = s_U;
      if (SEARCH) {
        uint64_t pre = P;
#pragma unroll 4
        for (int j = j0; j < j1; ++j) {
          pre += sQ[j];
          sQ[j] = pre;
        }
        __syncthreads();
        if (fb || Qt == 0) {
          for (int i = tid; i < N; i += TB) sA[i] = resample_fallback_index(U, i, N);
        } else {
          // four targets per thread at a time (i, i + TB, i + 2 TB, i + 3 TB),
          // their thresholds walked along the stride (one 32-bit division per
          // thread and frame); a target past N - 1 is searched (in bounds) but
          // not stored
          const RsThresh th = s_th;
          const RsStep st4 = s_st4;
          RsWalk wk[4];
          wk[0] = rs_walk_init(th, (uint32_t)tid);
          {
            const RsStep st1 = s_st1;
#pragma unroll
            for (int g = 1; g < 4; ++g) { wk[g] = wk[g - 1]; rs_walk_next(th, st1, wk[g]); }
          }
          for (int i0 = tid; i0 < N; i0 += 4 * TB) {
            uint64_t T4[4];
            int r4[4];
#pragma unroll
            for (int g = 0; g < 4; ++g) {
              T4[g] = rs_walk_threshold(th, wk[g]);
              rs_walk_next(th, st4, wk[g]);
            }
            search_u64_pow2<4>(sQ, N, T4, r4);
#pragma unroll
            for (int g = 0; g < 4; ++g)
              if (i0 + g * TB < N) sA[i0 + g * TB] = r4[g];
          }
        }
      } else {
        int e = 0;
        frexpf(Wmax, &e);
        for (int j = j0; j < j1; ++j) cs += quantize_f32(sW[j], e);
        P = block_excl_scan_u64(cs, s_red64, &Qt);   // includes barriers
        if (fb || Qt == 0) {
          for (int i = tid; i < N; i += TB) sA[i] = resample_fallback_index(U, i, N);
        } else if (j0 < j1) {
          int i = (j0 == 0) ? 0 : count_targets_le(P, N, U, Qt);
          uint64_t Qj = P;
          for (int j = j0; j < j1; ++j) {
            Qj += quantize_f32(sW[j], e);
            const unsigned __int128 lim = ((unsigned __int128)(uint64_t)N * (unsigned __int128)Qj) << 32;
            while (i < N && resample_rhs(i, U, Qt) <= lim) sA[i++] = j;
          }
        }
      }
      cp_async_wait_all();   // this thread's s_raw slot for the next frame
      __syncthreads();
      if (dbg)
        for (int i = tid; i < N; i += TB) A.dbg_anc[(size_t)t * N + i] = sA[i];
      float* tmp = xa; xa = xb; xb = tmp;
    }
    if (tid == 0) A.status[b] = s_flag;
    __syncthreads();
  }
}

static size_t batched_smem_bytes(int D, int Nmax, int K, int J, bool diag, bool search, bool low) {
  size_t pf = (D == 12) ? params_floats<12>(K, J, diag) : params_floats<24>(K, J, diag);
  size_t bytes = (low ? 8 : search ? 12 : 8) * (size_t)Nmax + 4 * pf + 8 * MKF_MAX_J * MKF_MAX_DET + 32 +
                 4 * (32 * (D + 3) + 2) + 8 * 34 + 16 + kPickBins;
  return (bytes + 15) & ~size_t(15);
}

// ------------------------------------------------------------------ streaming kernels (one track)
struct FrameScalars {
  float M;
  int fb;
  unsigned int ticket_a;
  int status;
};

struct StreamArgs {
  int N, tile_a, tile_b;
  uint64_t seed;
  uint32_t track, frame, U;
  float kappa, pd, sigma;
  PView pv;
  const int* det_off;
  const float2* det;
  const int* anc;
  const float* xa;
  float* xb;
  float* logw;
  float* partial;         // nb_a * (D+3): m, s, s2, v[D]
  unsigned long long* bsum;  // nb_b
  FrameScalars* fs;
  float* est;
  float* out_loglik;
  float* out_ess;
  float* dbg_w;
  int* anc_out;
  const uint32_t* frame_base;   // device frame offset (graph replays), or null
  bool prior;
};

// frame index of this step: a.frame, plus the device offset when replayed from a graph
__device__ __forceinline__ uint32_t step_frame(const StreamArgs& A) {
  return A.frame_base ? A.frame + *A.frame_base : A.frame;
}
__device__ __forceinline__ uint32_t step_uniform(const StreamArgs& A) {
  return A.frame_base ? resample_uniform(A.seed, A.track, step_frame(A)) : A.U;
}

// online merge of (m, s, s2, v) accumulators
template <int D>
__device__ __forceinline__ void merge_acc(float& m, float& s, float& s2, float* v, float m2, float t,
                                          float t2, const float* v2) {
  if (!(m2 > -INFINITY)) return;
  if (!(m > -INFINITY)) {
    m = m2; s = t; s2 = t2;
#pragma unroll
    for (int r = 0; r < D; ++r) v[r] = v2[r];
    return;
  }
  float M = fmaxf(m, m2);
  float f1 = __expf(m - M), f2 = __expf(m2 - M);
  s = s * f1 + t * f2;
  s2 = s2 * f1 * f1 + t2 * f2 * f2;
#pragma unroll
  for (int r = 0; r < D; ++r) v[r] = v[r] * f1 + v2[r] * f2;
  m = M;
}

template <int D>
__device__ void block_merge(float& m, float& s, float& s2, float* v, float* red) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  constexpr int NV = D + 3;
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    float m2 = __shfl_xor_sync(0xffffffffu, m, o);
    float t = __shfl_xor_sync(0xffffffffu, s, o);
    float t2 = __shfl_xor_sync(0xffffffffu, s2, o);
    float v2[D];
#pragma unroll
    for (int r = 0; r < D; ++r) v2[r] = __shfl_xor_sync(0xffffffffu, v[r], o);
    // symmetric merge so all lanes agree
    float mm = m, ss = s, ss2 = s2, vv[D];
#pragma unroll
    for (int r = 0; r < D; ++r) vv[r] = v[r];
    if (lane & o) {   // put the lower lane's value first for a fixed order
      m = m2; s = t; s2 = t2;
#pragma unroll
      for (int r = 0; r < D; ++r) v[r] = v2[r];
      merge_acc<D>(m, s, s2, v, mm, ss, ss2, vv);
    } else {
      merge_acc<D>(m, s, s2, v, m2, t, t2, v2);
    }
  }
  __syncthreads();
  if (lane == 0) {
    red[w * NV + 0] = m; red[w * NV + 1] = s; red[w * NV + 2] = s2;
#pragma unroll
    for (int r = 0; r < D; ++r) red[w * NV + 3 + r] = v[r];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    m = red[0]; s = red[1]; s2 = red[2];
#pragma unroll
    for (int r = 0; r < D; ++r) v[r] = red[3 + r];
    for (int q = 1; q < nw; ++q) merge_acc<D>(m, s, s2, v, red[q * NV], red[q * NV + 1], red[q * NV + 2], red + q * NV + 3);
  }
}


// Dynamic shared memory of bpf_stream_a: the model's parameter block
// (params_floats: a | mb | L | Bm | mm | cumpi) and a two-slot ring holding
// each thread's next ancestor state (slot r, plane g at (r D/4 + g) TB + tid).
template <int D>
__host__ __device__ constexpr size_t stream_a_smem_floats(int K, int J, bool diag, int TB) {
  return (size_t)params_floats<D>(K, J, diag) + 2 * (size_t)TB * D;
}

// the float4 planes of ancestor an's state into ring slot r of this thread
template <int D>
__device__ __forceinline__ void gather_state_async(float4* ring, int r, int tid, int TB, const float* xa, int N,
                                                   int an) {
  const float4* src = reinterpret_cast<const float4*>(xa);
#pragma unroll
  for (int g = 0; g < D / 4; ++g) cp_async16(ring + (size_t)(r * (D / 4) + g) * TB + tid, src + (size_t)g * N + an);
}

template <int D, bool DIAG>
__global__ void __launch_bounds__(256) bpf_stream_a(StreamArgs A) {
  extern __shared__ __align__(16) float s_dyn[];
  __shared__ __align__(16) float s_det[MKF_MAX_J * 2 * MKF_MAX_DET];
  __shared__ int s_cnt[MKF_MAX_J];
  __shared__ float s_red[32 * (D + 3)];
  __shared__ bool s_last;
  __shared__ uint8_t s_ktab[kPickBins];
  __shared__ PhiloxPre s_pre[D / 4];
  __shared__ PhiloxKeys s_keys;
  const int tid = threadIdx.x, TB = blockDim.x;
  const int K = A.pv.K, J = A.pv.J;
  const uint32_t frame = A.prior ? kFramePrior : step_frame(A);
  const LikConst LK = lik_const(A.pv, A.kappa, A.pd, A.sigma);
  // this block's copy of the model (the propagate and likelihood read it per
  // particle) and its component pick table; the prior's mu and S0c stay global
  const int Lsz = pad4(DIAG ? K * D : K * D * (D + 1) / 2);
  float* s_a = s_dyn;
  float* s_mb = s_a + K * D;
  float* s_L = s_mb + K * D;
  float* s_Bm = s_L + Lsz;
  float* s_mm = s_Bm + J * 3 * D;
  float* s_cum = s_mm + pad4(J * 3);
  float4* ring = reinterpret_cast<float4*>(s_dyn + params_floats<D>(K, J, DIAG));
  PView pv = A.pv;
  for (int q = tid; q < K * D; q += TB) { s_a[q] = pv.a[q]; s_mb[q] = pv.mb[q]; }
  for (int q = tid; q < (DIAG ? K * D : K * D * (D + 1) / 2); q += TB) s_L[q] = DIAG ? pv.Ld[q] : pv.Lq[q];
  for (int q = tid; q < J * 3 * D; q += TB) s_Bm[q] = pv.Bm[q];
  for (int q = tid; q < J * 3; q += TB) s_mm[q] = pv.mm[q];
  for (int q = tid; q < K; q += TB) s_cum[q] = pv.cumpi[q];
  if (tid == 0) s_keys = philox_keys(A.seed, A.track);
  if (tid < D / 4) s_pre[tid] = philox_pre(A.seed, A.track, frame, (uint32_t)tid);
  __syncthreads();
  build_pick_table(s_cum, K, s_ktab, tid, TB);
  pv.a = s_a; pv.mb = s_mb; pv.Lq = s_L; pv.Ld = s_L; pv.Bm = s_Bm; pv.mm = s_mm;
  pv.cumpi = s_cum;
  pv.ktab = s_ktab;
  __syncthreads();
  if (!A.prior) {
    for (int q = tid; q < J * MKF_MAX_DET; q += TB) {
      const int j = q / MKF_MAX_DET, i = q - j * MKF_MAX_DET;
      const int lo = A.det_off[j], n = A.det_off[j + 1] - lo;
      const int nc = min(max(n, 0), MKF_MAX_DET);
      if (i == 0) {
        if (n > MKF_MAX_DET && blockIdx.x == 0) atomicOr(&A.fs->status, MKF_ST_TRUNC);
        s_cnt[j] = nc;
      }
      stage_list_slot(s_det + j * 2 * MKF_MAX_DET, i, nc, A.det, lo, LK.k);
    }
    __syncthreads();
  }
  float m = -INFINITY, s = 0.0f, s2 = 0.0f, v[D];
#pragma unroll
  for (int r = 0; r < D; ++r) v[r] = 0.0f;
  const int base = blockIdx.x * A.tile_a;
  const int end = min(A.N, base + A.tile_a);
  if (A.prior) {
    for (int i = base + tid; i < end; i += TB) {
      float x[D], eps[D];
      int ub;
      float uc = particle_draws_pre<D>(s_pre, s_keys, (uint32_t)i, eps, ub);
      prior_sample<D>(pv, eps, uc, ub, x);
      store_state<D>(A.xb, A.N, i, x);
    }
    return;
  }
  // software pipeline over this thread's particles i, i + TB, ...: the state
  // of the next particle's ancestor is copied into the ring while this one is
  // computed, and the ancestor index after that is loaded a step ahead
  int an_next = 0;
  if (base + tid < end) {
    gather_state_async<D>(ring, 0, tid, TB, A.xa, A.N, A.anc[base + tid]);
    if (base + tid + TB < end) an_next = A.anc[base + tid + TB];
  }
  cp_async_commit();
  int slot = 0;
  for (int i = base + tid; i < end; i += TB) {
    float x[D], eps[D];
    cp_async_wait_all();
#pragma unroll
    for (int g = 0; g < D / 4; ++g) {
      const float4 q = ring[(size_t)(slot * (D / 4) + g) * TB + tid];
      x[4 * g] = q.x; x[4 * g + 1] = q.y; x[4 * g + 2] = q.z; x[4 * g + 3] = q.w;
    }
    slot ^= 1;
    if (i + TB < end) gather_state_async<D>(ring, slot, tid, TB, A.xa, A.N, an_next);
    cp_async_commit();
    if (i + 2 * TB < end) an_next = A.anc[i + 2 * TB];
    int ub;
    float uc = particle_draws_pre<D>(s_pre, s_keys, (uint32_t)i, eps, ub);
    propagate<D, DIAG>(pv, eps, uc, ub, x);
    store_state<D>(A.xb, A.N, i, x);
    float ll = loglik<D>(pv, x, s_cnt, s_det, LK);
    A.logw[i] = ll;
    // online accumulation
    if (ll > m) {
      float f = (m > -INFINITY) ? __expf(m - ll) : 0.0f;
      s = s * f + 1.0f;
      s2 = s2 * f * f + 1.0f;
#pragma unroll
      for (int r = 0; r < D; ++r) v[r] = fmaf(v[r], f, x[r]);
      m = ll;
    } else if (ll > -INFINITY) {
      float w = __expf(ll - m);
      s += w;
      s2 = fmaf(w, w, s2);
#pragma unroll
      for (int r = 0; r < D; ++r) v[r] = fmaf(w, x[r], v[r]);
    }
  }
  block_merge<D>(m, s, s2, v, s_red);
  constexpr int NV = D + 3;
  if (tid == 0) {
    float* p = A.partial + (size_t)blockIdx.x * NV;
    p[0] = m; p[1] = s; p[2] = s2;
#pragma unroll
    for (int r = 0; r < D; ++r) p[3 + r] = v[r];
    __threadfence();
    unsigned t = atomicAdd(&A.fs->ticket_a, 1u);
    s_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  // last block: combine every block's partial in a fixed order
  m = -INFINITY; s = 0.0f; s2 = 0.0f;
#pragma unroll
  for (int r = 0; r < D; ++r) v[r] = 0.0f;
  for (int q = tid; q < (int)gridDim.x; q += TB) {
    const volatile float* p = A.partial + (size_t)q * NV;
    float v2[D];
#pragma unroll
    for (int r = 0; r < D; ++r) v2[r] = p[3 + r];
    merge_acc<D>(m, s, s2, v, p[0], p[1], p[2], v2);
  }
  block_merge<D>(m, s, s2, v, s_red);
  if (tid == 0) {
    bool fb = !(m > -INFINITY) || !(m < INFINITY);
    A.fs->M = m;
    A.fs->fb = fb ? 1 : 0;
    if (fb) A.fs->status |= MKF_ST_FALLBACK | MKF_ST_NAN;
    A.fs->ticket_a = 0u;
    if (A.est)
      for (int r = 0; r < D; ++r) A.est[r] = v[r] / s;
    if (A.out_loglik) *A.out_loglik = m + logf(s) - logf((float)A.N);
    if (A.out_ess) *A.out_ess = s * s / s2;
  }
}

__device__ __forceinline__ float stream_weight(float ll, float M, int fb) {
  float w = fb ? 0.0f : (ll == M ? 1.0f : __expf(ll - M));
  return (w >= 0.0f) ? w : 0.0f;
}

// block sums of quantised weights; the last block scans them (exclusive)
__global__ void __launch_bounds__(256) bpf_stream_b(StreamArgs A) {
  __shared__ uint64_t s_red64[34];
  const int tid = threadIdx.x, TB = blockDim.x;
  const float M = A.fs->M;
  const int fb = A.fs->fb;
  const int base = blockIdx.x * A.tile_b, end = min(A.N, base + A.tile_b);
  // integer sums are order-free: coalesced 16-byte reads, four in flight per
  // thread (base is a multiple of 4: tile_b is a multiple of the block size)
  uint64_t cs = 0;
  const int n4 = (end - base) >> 2;
  const float4* l4 = reinterpret_cast<const float4*>(A.logw + base);
#pragma unroll 4
  for (int q = tid; q < n4; q += TB) {
    const float4 lw = l4[q];
    const float w0 = stream_weight(lw.x, M, fb), w1 = stream_weight(lw.y, M, fb);
    const float w2 = stream_weight(lw.z, M, fb), w3 = stream_weight(lw.w, M, fb);
    if (A.dbg_w) reinterpret_cast<float4*>(A.dbg_w + base)[q] = make_float4(w0, w1, w2, w3);
    cs += quantize39(w0) + quantize39(w1) + quantize39(w2) + quantize39(w3);
  }
  for (int j = base + 4 * n4 + tid; j < end; j += TB) {
    float w = stream_weight(A.logw[j], M, fb);
    if (A.dbg_w) A.dbg_w[j] = w;
    cs += quantize39(w);
  }
  uint64_t tot;
  block_excl_scan_u64(cs, s_red64, &tot);
  if (tid == 0) A.bsum[blockIdx.x] = tot;
}

// Number of targets i in [0, N) with T_i <= X, by one warp: a float estimate
// of N X / Qt (within a few of the count) settled by exact 64-bit thresholds
// at 32 candidates around it (T_i is nondecreasing, so the candidates at or
// below X are the lanes under the count); the 128-bit count when the estimate
// misses by 16 or more.
__device__ __forceinline__ int count_targets_le_warp(const RsThresh& th, uint64_t X, int N, uint32_t U, uint64_t Qt,
                                                     int lane) {
  const float xf = fmaf((float)(uint32_t)(X >> 32), 4294967296.0f, (float)(uint32_t)X);
  const float qf = fmaf((float)(uint32_t)(Qt >> 32), 4294967296.0f, (float)(uint32_t)Qt);
  const int est = (int)fminf(fmaxf(xf / qf * (float)N, 0.0f), (float)N);
  const int i = est - 16 + lane;
  const bool le = (i < 0) || (i < N && rs_threshold64(th, (uint32_t)i) <= X);
  const int c = __popc(__ballot_sync(0xffffffffu, le));
  if (c > 0 && c < 32) return est - 16 + c;
  return count_targets_le(X, N, U, Qt);
}

__global__ void __launch_bounds__(256, 5) bpf_stream_c(StreamArgs A, int tile_c) {
  extern __shared__ __align__(16) unsigned char smem_c[];
  uint64_t* sQ = reinterpret_cast<uint64_t*>(smem_c);
  __shared__ uint64_t s_red64[34];
  __shared__ int s_lo, s_hi;
  __shared__ RsThresh s_th;
  __shared__ RsStep s_st[2];
  const int tid = threadIdx.x, TB = blockDim.x, lane = tid & 31, w = tid >> 5;
  const float M = A.fs->M;
  const int fbM = A.fs->fb;
  const int base = blockIdx.x * tile_c, end = min(A.N, base + tile_c), n = end - base;
  // the tile's integer weights (they need M only), read coalesced; issued
  // first, so that their loads overlap the tile-sum loads below
  {
    const int n4 = n >> 2;
    const float4* l4 = reinterpret_cast<const float4*>(A.logw + base);
#pragma unroll 4
    for (int q = tid; q < n4; q += TB) {
      const float4 lw = l4[q];
      ulonglong2* d2 = reinterpret_cast<ulonglong2*>(sQ) + 2 * q;
      d2[0] = make_ulonglong2(quantize39(stream_weight(lw.x, M, fbM)), quantize39(stream_weight(lw.y, M, fbM)));
      d2[1] = make_ulonglong2(quantize39(stream_weight(lw.z, M, fbM)), quantize39(stream_weight(lw.w, M, fbM)));
    }
    for (int j = 4 * n4 + tid; j < n; j += TB) sQ[j] = quantize39(stream_weight(A.logw[base + j], M, fbM));
  }
  // the total Qt and this tile's exclusive prefix, from the tile sums of
  // bpf_stream_b (every block forms them: a few thousand L2-resident words);
  // block totals of two integer sums, one barrier (which also publishes sQ)
  uint64_t all = 0, before = 0;
  for (int q = tid; q < (int)gridDim.x; q += TB) {
    const uint64_t v = A.bsum[q];
    all += v;
    before += (q < (int)blockIdx.x) ? v : 0ull;
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    all += __shfl_xor_sync(0xffffffffu, all, o);
    before += __shfl_xor_sync(0xffffffffu, before, o);
  }
  if (lane == 0) { s_red64[w] = all; s_red64[16 + w] = before; }
  __syncthreads();
  uint64_t Qt = 0, Xprev = 0;
  for (int q = 0; q < (TB >> 5); ++q) { Qt += s_red64[q]; Xprev += s_red64[16 + q]; }
  const int fb = fbM || Qt == 0ull;
  if (blockIdx.x == 0 && tid == 0 && Qt == 0ull && !fbM) atomicOr(&A.fs->status, MKF_ST_FALLBACK);
  const uint32_t U = step_uniform(A);
  if (fb) {
    for (int i = base + tid; i < end; i += TB) A.anc_out[i] = resample_fallback_index(U, i, A.N);
    return;
  }
  // the resampling rule's constants (64-bit divisions), once per block (read
  // after the chunk scan's barriers)
  if (tid == 0) {
    const RsThresh th = rs_thresh_setup(Qt, A.N, U);
    s_th = th;
    s_st[0] = rs_step_setup(th, (uint32_t)TB);
    s_st[1] = rs_step_setup(th, 4u * (uint32_t)TB);
  }
  // prefix sums over contiguous chunks of an odd length (distinct banks across a warp)
  int E = (n + TB - 1) / TB;
  if (E > 1 && !(E & 1)) ++E;
  const int j0 = min(n, tid * E), j1 = min(n, j0 + E);
  uint64_t cs = 0;
  for (int j = j0; j < j1; ++j) cs += sQ[j];
  uint64_t tot;
  uint64_t pre = block_excl_scan_u64(cs, s_red64, &tot) + Xprev;
  for (int j = j0; j < j1; ++j) {
    pre += sQ[j];
    sQ[j] = pre;
  }
  // the tile's target range [lo, hi): warp 0 and warp 1 count the targets at
  // or below each end of the tile's prefix range
  {
    if (w < 2) {
      const RsThresh th = s_th;
      const bool first = (w == 0) ? (blockIdx.x == 0) : (blockIdx.x == gridDim.x - 1);
      const int c = first ? (w == 0 ? 0 : A.N)
                          : count_targets_le_warp(th, w == 0 ? Xprev : Xprev + tot, A.N, U, Qt, tid & 31);
      if ((tid & 31) == 0) (w == 0 ? s_lo : s_hi) = c;
    }
  }
  __syncthreads();
  // targets of this tile by 64-bit thresholds walked along each thread's
  // stride (one division estimate per thread, not per target), four
  // interleaved searches per thread; targets past hi are formed and dropped
  const RsThresh th = s_th;
  const int lo = s_lo, hi = s_hi;
  const RsStep st1 = s_st[0], st4 = s_st[1];
  RsWalk wk[4];
  wk[0] = rs_walk_init64(th, (uint32_t)(lo + tid));
#pragma unroll
  for (int g = 1; g < 4; ++g) { wk[g] = wk[g - 1]; rs_walk_next(th, st1, wk[g]); }
  for (int i0 = lo + tid; i0 < hi; i0 += 4 * TB) {
    uint64_t T4[4];
    int r4[4];
#pragma unroll
    for (int g = 0; g < 4; ++g) {
      T4[g] = rs_walk_threshold(th, wk[g]);
      rs_walk_next(th, st4, wk[g]);
    }
    search_u64_pow2<4>(sQ, n, T4, r4);
#pragma unroll
    for (int g = 0; g < 4; ++g)
      if (i0 + g * TB < hi) A.anc_out[i0 + g * TB] = base + r4[g];
  }
}

// ------------------------------------------------------------------ handles
struct BpfHandle {
  DevModels m;
  mkf_bpf_track tr;
  int N, d;
  float *xa, *xb, *logw, *w, *partial;
  int* anc;
  unsigned long long* bsum;
  FrameScalars* fs;
  int nb_a, nb_b, tile_a, tile_b;
  bool ready;
  bool debug;
};

constexpr int kStreamTB = 256;
constexpr int kTileB = 4096;

}  // namespace mkf

using namespace mkf;

struct mkf_bpf { BpfHandle h; };
// Host-buffer runs keep the device run's longest-first track order and split it
// in two launches: the head (the first grid-size tracks of that order, one per
// persistent CTA) starts as soon as its own tracks' lists are copied (one small
// copy per track, into buffer 0), while the whole input is copied in bulk
// (buffer 1) for the tail launch, whose CTAs take the SMs that head CTAs free.
struct HostRun {
  bool ready;
  int head;                                  // tracks in the head launch
  int* counters;                             // device, 2 work counters
  int* h_det_off_dev[2];
  float* h_det_dev[2];
  size_t det_cap;
  cudaStream_t copy, comp[2];
  cudaEvent_t start, copied[2], done[2];
};

struct mkf_bpf_batch {
  mkf_bpf_batch() : m(), n_tracks(0), Nmax(0), d(0), K(0), J(0), G(0), tb(0), ctas_per_sm(0), meta(nullptr),
                    fbase(nullptr), seed(nullptr), obs(nullptr), order(nullptr), counter(nullptr), scratch(nullptr),
                    scratch_slots(0), scratch_sets(1), last_grid(0), variant(0), dbg_track(-1), dbg_w(nullptr),
                    dbg_anc(nullptr), d_est(nullptr),
                    d_ll(nullptr), d_ess(nullptr), d_status(nullptr), hr() {}
  DevModels m;
  int n_tracks, Nmax, d, K, J;
  long long G;
  int tb, ctas_per_sm;
  int4* meta;
  long long* fbase;
  unsigned long long* seed;
  float4* obs;
  int* order;
  int* counter;
  float* scratch;
  size_t scratch_slots;
  int scratch_sets;                          // slot sets of concurrent launches (1, or 2 for host-buffer runs)
  int last_grid;
  int variant;
  int dbg_track;
  float* dbg_w;
  int* dbg_anc;
  // host-run staging of outputs (when the caller's buffers are not mapped)
  float *d_est, *d_ll, *d_ess;
  int* d_status;
  HostRun hr;
  std::vector<mkf_bpf_track> tracks;         // host copy: the head tracks' frame ranges
  std::vector<int> order_h;                  // host copy of order
};

static PView make_view(const DevModels& m, int mi) {
  PView p;
  const int d = m.d, K = m.K, J = m.J, DD = d * (d + 1) / 2;
  p.a = m.a + (size_t)mi * K * d; p.mb = m.mb + (size_t)mi * K * d; p.mu = m.mu + (size_t)mi * K * d;
  p.Lq = m.Lq + (size_t)mi * K * DD; p.Ld = m.Ld + (size_t)mi * K * d;
  p.S0c = m.S0c + (size_t)mi * K * DD; p.cumpi = m.cumpi + (size_t)mi * K;
  p.Bm = m.Bm + (size_t)mi * J * 3 * d; p.mm = m.mm + (size_t)mi * J * 3;
  p.ktab = nullptr;
  p.K = K; p.J = J; p.fx = m.fx; p.fy = m.fy; p.cx = m.cx; p.cy = m.cy;
  return p;
}

template <int D, bool DIAG>
static size_t stream_a_smem_bytes(const DevModels& m) {
  return stream_a_smem_floats<D>(m.K, m.J, DIAG, kStreamTB) * sizeof(float);
}
static size_t stream_a_smem(const DevModels& m) {
  if (m.d == 12) return m.diag ? stream_a_smem_bytes<12, true>(m) : stream_a_smem_bytes<12, false>(m);
  return m.diag ? stream_a_smem_bytes<24, true>(m) : stream_a_smem_bytes<24, false>(m);
}
// opt the instance this model launches into its dynamic shared memory size
// (above the default 48 KB only for d = 24 with a full noise factor) and
// report its resident blocks per SM
template <typename Kern>
static cudaError_t kernel_smem_occ(Kern kern, int bytes, int* occ) {
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, kern, kStreamTB, bytes);
  return e;
}
static cudaError_t stream_a_attr(const DevModels& m, int* occ) {
  const int bytes = (int)stream_a_smem(m);
  if (m.d == 12)
    return m.diag ? kernel_smem_occ(bpf_stream_a<12, true>, bytes, occ) : kernel_smem_occ(bpf_stream_a<12, false>, bytes, occ);
  return m.diag ? kernel_smem_occ(bpf_stream_a<24, true>, bytes, occ) : kernel_smem_occ(bpf_stream_a<24, false>, bytes, occ);
}

static void stream_a(const DevModels& m, const StreamArgs& a, int nb, cudaStream_t s) {
  const size_t smem = stream_a_smem(m);
  if (m.d == 12) {
    if (m.diag) bpf_stream_a<12, true><<<nb, kStreamTB, smem, s>>>(a);
    else bpf_stream_a<12, false><<<nb, kStreamTB, smem, s>>>(a);
  } else {
    if (m.diag) bpf_stream_a<24, true><<<nb, kStreamTB, smem, s>>>(a);
    else bpf_stream_a<24, false><<<nb, kStreamTB, smem, s>>>(a);
  }
}

extern "C" int mkf_bpf_create(const mkf_bpf_models* models, const mkf_bpf_track* track, mkf_bpf_t* out) {
  MKF_ARG(models && track && out, "mkf_bpf_create: null argument");
  MKF_ARG(track->n_particles >= 1 && track->n_particles <= (1 << 22), "mkf_bpf_create: n_particles out of range");
  MKF_ARG(track->model_index >= 0 && track->model_index < models->n_models, "mkf_bpf_create: bad model_index");
  MKF_ARG(track->kappa > 0.0f && track->p_detect > 0.0f && track->p_detect < 1.0f && track->sigma_px > 0.0f,
          "mkf_bpf_create: kappa, p_detect, sigma_px out of range");
  mkf_bpf* H = new (std::nothrow) mkf_bpf();
  if (!H) return MKF_ERR_NOMEM;
  BpfHandle& h = H->h;
  memset(&h, 0, sizeof(h));
  int st = build_models(models, h.m);
  if (st) { free_models(h.m); delete H; return st; }
  h.tr = *track;
  h.N = track->n_particles;
  h.d = models->d;
  // tiles.  Propagate/score: one wave of resident blocks, each over one
  // contiguous tile (its fixed cost -- model staging, pick table, the block's
  // estimate merge -- is paid once per block, and no partial last wave).  Sums
  // and search: tiles of at most kTileB particles in a whole number of waves of
  // the search kernel's resident blocks.
  const int sms = num_sms();
  int occ_a = 0, occ_c = 0;
  cudaError_t e = stream_a_attr(h.m, &occ_a);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_c, bpf_stream_c, kStreamTB, kTileB * sizeof(uint64_t));
  if (e != cudaSuccess) {
    free_models(h.m);
    delete H;
    return cuda_fail(e, "mkf_bpf_create: kernel attributes", __FILE__, __LINE__);
  }
  auto round_tb = [](long long t) { return (int)std::max<long long>(kStreamTB, (t + kStreamTB - 1) / kStreamTB * kStreamTB); };
  const long long wave_a = (long long)sms * std::max(1, occ_a), wave_c = (long long)sms * std::max(1, occ_c);
  h.tile_a = round_tb((h.N + wave_a - 1) / wave_a);
  const long long waves_c = std::max(1LL, (h.N + wave_c * kTileB - 1) / (wave_c * kTileB));
  h.tile_b = std::min(kTileB, round_tb((h.N + waves_c * wave_c - 1) / (waves_c * wave_c)));
  h.nb_a = (h.N + h.tile_a - 1) / h.tile_a;
  h.nb_b = (h.N + h.tile_b - 1) / h.tile_b;
  const size_t N = h.N, d = h.d;
  if (e == cudaSuccess) e = cudaMalloc(&h.xa, N * d * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&h.xb, N * d * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&h.logw, N * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&h.w, N * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&h.anc, N * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&h.partial, (size_t)h.nb_a * (d + 3) * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&h.bsum, (size_t)h.nb_b * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMalloc(&h.fs, sizeof(FrameScalars));
  if (e == cudaSuccess) e = cudaMemset(h.fs, 0, sizeof(FrameScalars));
  if (e != cudaSuccess) {
    mkf_bpf_destroy(H);
    return cuda_fail(e, "mkf_bpf_create: allocation", __FILE__, __LINE__);
  }
  *out = H;
  return MKF_OK;
}

static StreamArgs stream_args(BpfHandle& h) {
  StreamArgs a;
  memset(&a, 0, sizeof(a));
  a.N = h.N; a.tile_a = h.tile_a; a.tile_b = h.tile_b;
  a.seed = h.tr.seed; a.track = h.tr.track_id;
  a.kappa = h.tr.kappa; a.pd = h.tr.p_detect; a.sigma = h.tr.sigma_px;
  a.pv = make_view(h.m, h.tr.model_index);
  a.partial = h.partial; a.bsum = h.bsum; a.fs = h.fs;
  return a;
}

extern "C" int mkf_bpf_reset(mkf_bpf_t H, mkf_stream_t stream) {
  MKF_RANGE("mkf_bpf_reset");
  MKF_ARG(H, "mkf_bpf_reset: null handle");
  BpfHandle& h = H->h;
  cudaStream_t s = (cudaStream_t)stream;
  StreamArgs a = stream_args(h);
  a.prior = true;
  a.xb = h.xa;
  stream_a(h.m, a, h.nb_a, s);
  MKF_CHECK_LAUNCH("mkf_bpf_reset: prior kernel");
  // identity ancestry: sequence 0..N-1
  std::vector<int> iota(h.N);
  for (int i = 0; i < h.N; ++i) iota[i] = i;
  MKF_CUDA(cudaMemcpyAsync(h.anc, iota.data(), sizeof(int) * h.N, cudaMemcpyHostToDevice, s));
  MKF_CUDA(cudaMemsetAsync(h.fs, 0, sizeof(FrameScalars), s));
  MKF_CUDA(cudaStreamSynchronize(s));
  h.ready = true;
  return MKF_OK;
}

// one frame: propagate+score, block sums, ancestor search (three launches on s)
static int enqueue_update(BpfHandle& h, uint32_t frame, const uint32_t* frame_base, const int* d_det_off,
                          const float* d_det, float* d_est, float* d_loglik, float* d_ess, cudaStream_t s) {
  StreamArgs a = stream_args(h);
  a.frame = frame;
  a.frame_base = frame_base;
  a.U = frame_base ? 0u : resample_uniform(h.tr.seed, h.tr.track_id, frame);
  a.det_off = d_det_off;
  a.det = reinterpret_cast<const float2*>(d_det);
  a.anc = h.anc; a.xa = h.xa; a.xb = h.xb; a.logw = h.logw;
  a.est = d_est; a.out_loglik = d_loglik; a.out_ess = d_ess;
  a.dbg_w = h.debug ? h.w : nullptr;
  a.anc_out = h.anc;
  stream_a(h.m, a, h.nb_a, s);
  MKF_CHECK_LAUNCH("mkf_bpf_update: propagate/score kernel");
  bpf_stream_b<<<h.nb_b, kStreamTB, 0, s>>>(a);
  MKF_CHECK_LAUNCH("mkf_bpf_update: block-sum kernel");
  bpf_stream_c<<<h.nb_b, kStreamTB, (size_t)h.tile_b * sizeof(uint64_t), s>>>(a, h.tile_b);
  MKF_CHECK_LAUNCH("mkf_bpf_update: search kernel");
  std::swap(h.xa, h.xb);
  return MKF_OK;
}

extern "C" int mkf_bpf_update(mkf_bpf_t H, uint32_t frame, const int* d_det_off, const float* d_det,
                              float* d_est, float* d_loglik, float* d_ess, mkf_stream_t stream) {
  MKF_RANGE("mkf_bpf_update");
  MKF_ARG(H && d_det_off, "mkf_bpf_update: null argument");
  BpfHandle& h = H->h;
  if (!h.ready) { set_error("mkf_bpf_update: call mkf_bpf_reset first"); return MKF_ERR_STATE; }
  return enqueue_update(h, frame, nullptr, d_det_off, d_det, d_est, d_loglik, d_ess, (cudaStream_t)stream);
}

// ------------------------------------------------------------- captured frame loops
struct mkf_bpf_graph {
  mkf_bpf_t owner;
  int n_frames;
  uint32_t* frame_base;          // device
  cudaGraphExec_t exec;
};

__global__ void set_frame_base_kernel(uint32_t* p, uint32_t v) { *p = v; }

extern "C" int mkf_bpf_graph_create(mkf_bpf_t H, int n_frames, const int* d_det_off, const float* d_det,
                                    float* d_est, float* d_loglik, float* d_ess, mkf_bpf_graph_t* out) {
  MKF_ARG(H && out && d_det_off && n_frames >= 1, "mkf_bpf_graph_create: bad argument");
  BpfHandle& h = H->h;
  if (!h.ready) { set_error("mkf_bpf_graph_create: call mkf_bpf_reset first"); return MKF_ERR_STATE; }
  mkf_bpf_graph* g = new (std::nothrow) mkf_bpf_graph();
  if (!g) return MKF_ERR_NOMEM;
  g->owner = H; g->n_frames = n_frames; g->frame_base = nullptr; g->exec = nullptr;
  cudaError_t e = cudaMalloc(&g->frame_base, sizeof(uint32_t));
  if (e != cudaSuccess) { delete g; return cuda_fail(e, "mkf_bpf_graph_create: allocation", __FILE__, __LINE__); }
  cudaStream_t cs = nullptr;
  e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    if (cs) cudaStreamDestroy(cs);
    cudaFree(g->frame_base); delete g;
    return cuda_fail(e, "mkf_bpf_graph_create: capture start", __FILE__, __LINE__);
  }
  float* const x0 = h.xa;
  const int J = h.m.J;
  int rc = MKF_OK;
  for (int t = 0; t < n_frames && rc == MKF_OK; ++t)
    rc = enqueue_update(h, (uint32_t)t, g->frame_base, d_det_off + (size_t)t * J, d_det,
                        d_est ? d_est + (size_t)t * h.d : nullptr, d_loglik ? d_loglik + t : nullptr,
                        d_ess ? d_ess + t : nullptr, cs);
  // an odd number of frames ends in the other buffer: copy back so that launches chain
  if (h.xa != x0) {
    if (rc == MKF_OK) {
      cudaError_t ce = cudaMemcpyAsync(x0, h.xa, sizeof(float) * (size_t)h.N * h.d, cudaMemcpyDeviceToDevice, cs);
      if (ce != cudaSuccess) rc = cuda_fail(ce, "mkf_bpf_graph_create: copy-back", __FILE__, __LINE__);
    }
    std::swap(h.xa, h.xb);
  }
  cudaGraph_t graph = nullptr;
  e = cudaStreamEndCapture(cs, &graph);
  if (rc == MKF_OK && e != cudaSuccess) rc = cuda_fail(e, "mkf_bpf_graph_create: capture end", __FILE__, __LINE__);
  if (rc == MKF_OK) {
    e = cudaGraphInstantiate(&g->exec, graph, 0);
    if (e != cudaSuccess) rc = cuda_fail(e, "mkf_bpf_graph_create: instantiate", __FILE__, __LINE__);
  }
  if (graph) cudaGraphDestroy(graph);
  cudaStreamDestroy(cs);
  if (rc != MKF_OK) {
    cudaGetLastError();
    cudaFree(g->frame_base); delete g;
    return rc;
  }
  *out = g;
  return MKF_OK;
}

extern "C" int mkf_bpf_graph_launch(mkf_bpf_graph_t g, uint32_t frame0, mkf_stream_t stream) {
  MKF_RANGE("mkf_bpf_graph_launch");
  MKF_ARG(g && g->exec, "mkf_bpf_graph_launch: null graph");
  cudaStream_t s = (cudaStream_t)stream;
  set_frame_base_kernel<<<1, 1, 0, s>>>(g->frame_base, frame0);
  MKF_CHECK_LAUNCH("mkf_bpf_graph_launch: frame offset");
  MKF_CUDA(cudaGraphLaunch(g->exec, s));
  return MKF_OK;
}

extern "C" int mkf_bpf_graph_destroy(mkf_bpf_graph_t g) {
  if (!g) return MKF_OK;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->frame_base) cudaFree(g->frame_base);
  delete g;
  return MKF_OK;
}

// particle i's dimension r lives at plane r / 4, lane r % 4 of the state buffer
__global__ void soa_from_planes_kernel(const float* planes, int N, int d, float* soa) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < (size_t)N * d; q += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(q / N), i = (int)(q - (size_t)r * N);
    soa[q] = planes[((size_t)(r >> 2) * N + i) * 4 + (r & 3)];
  }
}

extern "C" int mkf_bpf_read_debug(mkf_bpf_t H, float* d_x, float* d_logw, float* d_w, int* d_anc,
                                  mkf_stream_t stream) {
  MKF_ARG(H, "mkf_bpf_read_debug: null handle");
  BpfHandle& h = H->h;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t N = h.N;
  if (d_x) {   // float4 planes -> the documented SoA (d, N)
    soa_from_planes_kernel<<<(int)std::min<size_t>((N * h.d + 255) / 256, 65535), 256, 0, s>>>(h.xa, h.N, h.d, d_x);
    MKF_CHECK_LAUNCH("mkf_bpf_read_debug: layout");
  }
  if (d_logw) MKF_CUDA(cudaMemcpyAsync(d_logw, h.logw, N * sizeof(float), cudaMemcpyDeviceToDevice, s));
  if (d_w) MKF_CUDA(cudaMemcpyAsync(d_w, h.w, N * sizeof(float), cudaMemcpyDeviceToDevice, s));
  if (d_anc) MKF_CUDA(cudaMemcpyAsync(d_anc, h.anc, N * sizeof(int), cudaMemcpyDeviceToDevice, s));
  return MKF_OK;
}

extern "C" int mkf_bpf_set_debug(mkf_bpf_t H, int enable) {
  MKF_ARG(H, "mkf_bpf_set_debug: null handle");
  H->h.debug = enable != 0;
  return MKF_OK;
}

extern "C" int mkf_bpf_status(mkf_bpf_t H, int* status) {
  MKF_ARG(H && status, "mkf_bpf_status: null argument");
  FrameScalars fs;
  MKF_CUDA(cudaMemcpy(&fs, H->h.fs, sizeof(fs), cudaMemcpyDeviceToHost));
  *status = fs.status;
  return MKF_OK;
}

extern "C" int mkf_bpf_destroy(mkf_bpf_t H) {
  if (!H) return MKF_OK;
  BpfHandle& h = H->h;
  void* ps[] = {h.xa, h.xb, h.logw, h.w, h.anc, h.partial, h.bsum, h.fs};
  for (void* p : ps) if (p) cudaFree(p);
  free_models(h.m);
  delete H;
  return MKF_OK;
}

// ------------------------------------------------------------------ batched C ABI
extern "C" int mkf_bpf_batch_create(const mkf_bpf_models* models, int n_tracks, const mkf_bpf_track* tracks,
                                    int64_t n_frames_total, mkf_bpf_batch_t* out) {
  MKF_ARG(models && tracks && out && n_tracks > 0, "mkf_bpf_batch_create: bad argument");
  int Nmax = 0;
  long long sumT = 0;
  for (int b = 0; b < n_tracks; ++b) {
    const mkf_bpf_track& t = tracks[b];
    MKF_ARG(t.n_particles >= 1 && t.n_particles <= 8192, "mkf_bpf_batch_create: n_particles must be in [1, 8192]");
    MKF_ARG(t.n_frames >= 0, "mkf_bpf_batch_create: n_frames < 0");
    MKF_ARG(t.model_index >= 0 && t.model_index < models->n_models, "mkf_bpf_batch_create: bad model_index");
    MKF_ARG(t.frame_base >= 0 && t.frame_base + t.n_frames <= n_frames_total, "mkf_bpf_batch_create: frame range");
    MKF_ARG(t.kappa > 0.0f && t.p_detect > 0.0f && t.p_detect < 1.0f && t.sigma_px > 0.0f,
            "mkf_bpf_batch_create: kappa, p_detect, sigma_px out of range");
    Nmax = std::max(Nmax, t.n_particles);
    sumT += t.n_frames;
  }
  mkf_bpf_batch* B = new (std::nothrow) mkf_bpf_batch();
  if (!B) return MKF_ERR_NOMEM;
  int st = build_models(models, B->m);
  if (st) { free_models(B->m); delete B; return st; }
  B->n_tracks = n_tracks; B->Nmax = (Nmax + 31) & ~31; B->d = models->d; B->K = models->K; B->J = models->J;
  B->G = n_frames_total;
  // the fastest shape measured on GB300 for the uneven-track workload
  B->tb = 256; B->ctas_per_sm = 3; B->variant = MKF_BPF_VEC_LOADS | MKF_BPF_SEARCH | MKF_BPF_LOWSMEM;
  B->scratch_sets = 1;
  B->dbg_track = -1;
  B->tracks.assign(tracks, tracks + n_tracks);
  std::vector<int4> meta(n_tracks);
  std::vector<long long> fb(n_tracks);
  std::vector<unsigned long long> sd(n_tracks);
  std::vector<float4> ob(n_tracks);
  std::vector<int> order(n_tracks);
  for (int b = 0; b < n_tracks; ++b) {
    const mkf_bpf_track& t = tracks[b];
    meta[b] = make_int4(t.n_particles, t.n_frames, t.model_index, (int)t.track_id);
    fb[b] = t.frame_base; sd[b] = t.seed;
    ob[b] = make_float4(t.kappa, t.p_detect, t.sigma_px, 0.0f);
    order[b] = b;
  }
  // longest-processing-time-first schedule over the persistent CTAs
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    return (long long)tracks[x].n_particles * tracks[x].n_frames > (long long)tracks[y].n_particles * tracks[y].n_frames;
  });
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = cudaMalloc(&B->meta, n_tracks * sizeof(int4));
  if (e == cudaSuccess) e = cudaMalloc(&B->fbase, n_tracks * sizeof(long long));
  if (e == cudaSuccess) e = cudaMalloc(&B->seed, n_tracks * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMalloc(&B->obs, n_tracks * sizeof(float4));
  if (e == cudaSuccess) e = cudaMalloc(&B->order, n_tracks * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&B->counter, sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpy(B->meta, meta.data(), n_tracks * sizeof(int4), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(B->fbase, fb.data(), n_tracks * sizeof(long long), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(B->seed, sd.data(), n_tracks * sizeof(unsigned long long), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(B->obs, ob.data(), n_tracks * sizeof(float4), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(B->order, order.data(), n_tracks * sizeof(int), cudaMemcpyHostToDevice);
  B->order_h = order;
  if (e != cudaSuccess) {
    mkf_bpf_batch_destroy(B);
    return cuda_fail(e, "mkf_bpf_batch_create: allocation", __FILE__, __LINE__);
  }
  (void)sumT;
  *out = B;
  return MKF_OK;
}

extern "C" int mkf_bpf_batch_set_tuning(mkf_bpf_batch_t B, int block_threads, int ctas_per_sm) {
  MKF_ARG(B, "mkf_bpf_batch_set_tuning: null handle");
  MKF_ARG(block_threads >= 64 && block_threads <= 512 && block_threads % 32 == 0,
          "mkf_bpf_batch_set_tuning: block_threads must be a multiple of 32 in [64, 512]");
  MKF_ARG(ctas_per_sm >= 0 && ctas_per_sm <= 32, "mkf_bpf_batch_set_tuning: ctas_per_sm out of range");
  B->tb = block_threads;
  B->ctas_per_sm = ctas_per_sm;
  return MKF_OK;
}

extern "C" int mkf_bpf_batch_last_grid(mkf_bpf_batch_t B, int* grid) {
  MKF_ARG(B && grid, "mkf_bpf_batch_last_grid: null argument");
  *grid = B->last_grid;
  return MKF_OK;
}

extern "C" int mkf_bpf_batch_set_debug(mkf_bpf_batch_t B, int track, float* d_w, int* d_anc) {
  MKF_ARG(B, "mkf_bpf_batch_set_debug: null handle");
  B->dbg_track = track; B->dbg_w = d_w; B->dbg_anc = d_anc;
  return MKF_OK;
}

// One launch of the persistent kernel over a.n_tracks tracks (a.order,
// a.counter set by the caller).  slot_set selects one of B->scratch_sets
// disjoint sets of per-CTA slots, so that launches that may overlap on the
// GPU never share a slot.
template <int D, bool DIAG, int TBMAX, int MINB, bool VEC, bool SEARCH, bool PAIR, bool LOW>
static int launch_batched_v(mkf_bpf_batch* B, BatchArgs& a, cudaStream_t s, int slot_set) {
  auto kern = bpf_batched_kernel<D, DIAG, TBMAX, MINB, VEC, SEARCH, PAIR, LOW>;
  size_t smem = batched_smem_bytes(D, B->Nmax, B->K, B->J, DIAG, SEARCH, LOW);
  MKF_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  // the largest shared-memory carveout: residency is bounded by shared memory
  MKF_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                (int)cudaSharedmemCarveoutMaxShared));
  int occ = 0;
  MKF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, B->tb, smem));
  if (occ < 1) { set_error("mkf_bpf_batch_run: block shape does not fit on an SM"); return MKF_ERR_ARG; }
  int per_sm = B->ctas_per_sm > 0 ? std::min(B->ctas_per_sm, occ) : occ;
  const long long full = (long long)num_sms() * per_sm;
  // per CTA: two state buffers (2 D Nmax floats); LOW adds Nmax ancestors.
  // Every set is sized for the full grid of the whole batch.
  const size_t per_set = (size_t)std::min<long long>(full, B->n_tracks) * (2 * D + (LOW ? 1 : 0)) * B->Nmax;
  const size_t need = per_set * (size_t)B->scratch_sets;
  if (need > B->scratch_slots) {
    if (B->scratch) cudaFree(B->scratch);
    B->scratch = nullptr;
    B->scratch_slots = 0;
    MKF_CUDA(cudaMalloc(&B->scratch, need * sizeof(float)));
    B->scratch_slots = need;
  }
  const long long grid = std::min<long long>(full, a.n_tracks);
  if (grid < 1) return MKF_OK;
  float* base = B->scratch + (size_t)slot_set * per_set;
  a.scratch = base;
  a.anc = LOW ? reinterpret_cast<int*>(base + (size_t)grid * 2 * D * B->Nmax) : nullptr;
  B->last_grid = (int)grid;
  MKF_CUDA(cudaMemsetAsync(a.counter, 0, sizeof(int), s));
  kern<<<(int)grid, B->tb, smem, s>>>(a);
  MKF_CHECK_LAUNCH("mkf_bpf_batch_run: batched kernel");
  return MKF_OK;
}

// Launch bounds by block size and requested residency.  ALL: up to 256
// threads at 2 (128 registers) or 3 (80 registers) CTAs per SM, up to 384
// threads at 2 CTAs per SM (80 registers), up to 512 threads at 1.  Otherwise
// (the variants the autotuner ranks below float4 loads + search): up to 256
// threads at 2 CTAs per SM, up to 512 at 1, which keeps the number of compiled
// kernels, and the build time, down.
template <int D, bool DIAG, bool VEC, bool SEARCH, bool PAIR = false, bool LOW = false, bool ALL = false>
static int launch_shape(mkf_bpf_batch* B, BatchArgs& a, cudaStream_t s, int set) {
  if constexpr (ALL) {
    if (B->tb > 384) return launch_batched_v<D, DIAG, 512, 1, VEC, SEARCH, PAIR, LOW>(B, a, s, set);
    if (B->tb > 256) return launch_batched_v<D, DIAG, 384, 2, VEC, SEARCH, PAIR, LOW>(B, a, s, set);
    if (B->ctas_per_sm >= 3) return launch_batched_v<D, DIAG, 256, 3, VEC, SEARCH, PAIR, LOW>(B, a, s, set);
    return launch_batched_v<D, DIAG, 256, 2, VEC, SEARCH, PAIR, LOW>(B, a, s, set);
  }
  if (B->tb > 256) return launch_batched_v<D, DIAG, 512, 1, VEC, SEARCH, PAIR, LOW>(B, a, s, set);
  return launch_batched_v<D, DIAG, 256, 2, VEC, SEARCH, PAIR, LOW>(B, a, s, set);
}

// the load-width and resampler variants are compiled for the diagonal-noise
// d = 12 model only
template <int D, bool DIAG>
static int launch_batched(mkf_bpf_batch* B, BatchArgs& a, cudaStream_t s, int set) {
  if constexpr (D == 12 && DIAG) {
    const bool vec = (B->variant & MKF_BPF_VEC_LOADS) != 0, search = (B->variant & MKF_BPF_SEARCH) != 0;
    if (B->variant & MKF_BPF_PAIR) return launch_shape<D, DIAG, true, true, true>(B, a, s, set);
    if (B->variant & MKF_BPF_LOWSMEM) return launch_shape<D, DIAG, true, true, false, true, true>(B, a, s, set);
    if (vec && search) return launch_shape<D, DIAG, true, true, false, false, true>(B, a, s, set);
    if (vec) return launch_shape<D, DIAG, true, false>(B, a, s, set);
    if (search) return launch_shape<D, DIAG, false, true>(B, a, s, set);
    return launch_shape<D, DIAG, false, false>(B, a, s, set);
  } else {
    return launch_shape<D, DIAG, true, false>(B, a, s, set);
  }
}

static int launch_any(mkf_bpf_batch* B, BatchArgs& a, cudaStream_t s, int set) {
  if (B->d == 12) return B->m.diag ? launch_batched<12, true>(B, a, s, set) : launch_batched<12, false>(B, a, s, set);
  return B->m.diag ? launch_batched<24, true>(B, a, s, set) : launch_batched<24, false>(B, a, s, set);
}

static BatchArgs batch_args(const mkf_bpf_batch* B, const int* d_det_off, const float* d_det, float* d_est,
                            float* d_loglik, float* d_ess, int* d_status) {
  BatchArgs a;
  memset(&a, 0, sizeof(a));
  a.n_tracks = B->n_tracks; a.K = B->K; a.J = B->J; a.Nmax = B->Nmax;
  a.meta = B->meta; a.fbase = B->fbase; a.seed = B->seed; a.obs = B->obs;
  a.order = B->order; a.counter = B->counter; a.m = B->m;
  a.det_off = d_det_off; a.det = reinterpret_cast<const float2*>(d_det);
  a.est = d_est; a.loglik = d_loglik; a.ess = d_ess; a.status = d_status;
  a.dbg_track = B->dbg_track; a.dbg_w = B->dbg_w; a.dbg_anc = B->dbg_anc;
  return a;
}

extern "C" int mkf_bpf_batch_set_variant(mkf_bpf_batch_t B, int flags) {
  MKF_ARG(B, "mkf_bpf_batch_set_variant: null handle");
  MKF_ARG((flags & ~(MKF_BPF_VEC_LOADS | MKF_BPF_SEARCH | MKF_BPF_PAIR | MKF_BPF_LOWSMEM)) == 0,
          "mkf_bpf_batch_set_variant: unknown flag");
  MKF_ARG(!(flags & MKF_BPF_LOWSMEM) ||
              ((flags & (MKF_BPF_VEC_LOADS | MKF_BPF_SEARCH)) == (MKF_BPF_VEC_LOADS | MKF_BPF_SEARCH) &&
               !(flags & MKF_BPF_PAIR)),
          "mkf_bpf_batch_set_variant: MKF_BPF_LOWSMEM needs MKF_BPF_VEC_LOADS | MKF_BPF_SEARCH, without MKF_BPF_PAIR");
  B->variant = flags;
  return MKF_OK;
}

extern "C" int mkf_bpf_batch_run(mkf_bpf_batch_t B, const int* d_det_off, const float* d_det,
                                 float* d_est, float* d_loglik, float* d_ess, int* d_status,
                                 mkf_stream_t stream) {
  MKF_RANGE("mkf_bpf_batch_run");
  MKF_ARG(B && d_det_off && d_est && d_loglik && d_ess && d_status, "mkf_bpf_batch_run: null argument");
  BatchArgs a = batch_args(B, d_det_off, d_det, d_est, d_loglik, d_ess, d_status);
  return launch_any(B, a, (cudaStream_t)stream, 0);
}

static void free_host_run(HostRun& r) {
  void* ps[] = {r.counters, r.h_det_off_dev[0], r.h_det_off_dev[1], r.h_det_dev[0], r.h_det_dev[1]};
  for (void* p : ps) if (p) cudaFree(p);
  cudaStream_t ss[] = {r.copy, r.comp[0], r.comp[1]};
  for (cudaStream_t x : ss) if (x) cudaStreamDestroy(x);
  cudaEvent_t es[] = {r.start, r.copied[0], r.copied[1], r.done[0], r.done[1]};
  for (cudaEvent_t x : es) if (x) cudaEventDestroy(x);
  r = HostRun();
}

static int setup_host_run(mkf_bpf_batch* B) {
  HostRun& r = B->hr;
  const size_t G = (size_t)B->G, J = (size_t)B->J, d = (size_t)B->d;
  MKF_CUDA(cudaMalloc(&r.counters, 2 * sizeof(int)));
  for (int k = 0; k < 2; ++k) MKF_CUDA(cudaMalloc(&r.h_det_off_dev[k], (G * J + 1) * sizeof(int)));
  if (!B->d_est) MKF_CUDA(cudaMalloc(&B->d_est, G * d * sizeof(float)));
  if (!B->d_ll) MKF_CUDA(cudaMalloc(&B->d_ll, G * sizeof(float)));
  if (!B->d_ess) MKF_CUDA(cudaMalloc(&B->d_ess, G * sizeof(float)));
  if (!B->d_status) MKF_CUDA(cudaMalloc(&B->d_status, B->n_tracks * sizeof(int)));
  MKF_CUDA(cudaStreamCreateWithFlags(&r.copy, cudaStreamNonBlocking));
  for (int k = 0; k < 2; ++k) {
    MKF_CUDA(cudaStreamCreateWithFlags(&r.comp[k], cudaStreamNonBlocking));
    MKF_CUDA(cudaEventCreateWithFlags(&r.copied[k], cudaEventDisableTiming));
    MKF_CUDA(cudaEventCreateWithFlags(&r.done[k], cudaEventDisableTiming));
  }
  MKF_CUDA(cudaEventCreateWithFlags(&r.start, cudaEventDisableTiming));
  // the head: one track per CTA of the persistent grid (an upper bound of it)
  r.head = std::min(B->n_tracks, num_sms() * std::max(1, B->ctas_per_sm > 0 ? B->ctas_per_sm : 3));
  B->scratch_sets = 2;
  r.ready = true;
  return MKF_OK;
}

// device address of a host buffer that the GPU can write directly (pinned and
// mapped), or null
static void* mapped_device_ptr(void* host) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, host) != cudaSuccess) { cudaGetLastError(); return nullptr; }
  return (at.type == cudaMemoryTypeHost) ? at.devicePointer : nullptr;
}

extern "C" int mkf_bpf_batch_run_host(mkf_bpf_batch_t B, const int* det_off, const float* det, int64_t n_det,
                                      float* est, float* loglik, float* ess, int* status,
                                      mkf_stream_t stream) {
  MKF_RANGE("mkf_bpf_batch_run_host");
  MKF_ARG(B && det_off && det && est && loglik && ess && status && n_det >= 0, "mkf_bpf_batch_run_host: null argument");
  MKF_ARG(n_det <= 0x7FFFFFFFLL, "mkf_bpf_batch_run_host: more than 2^31 - 1 detections (int32 offsets)");
  cudaStream_t s = (cudaStream_t)stream;
  const size_t G = (size_t)B->G, J = (size_t)B->J, d = (size_t)B->d;
  MKF_ARG(det_off[0] >= 0 && (int64_t)det_off[G * J] <= n_det, "mkf_bpf_batch_run_host: det_off outside [0, n_det]");
  HostRun& r = B->hr;
  if (!r.ready) {
    int st = setup_host_run(B);
    if (st) { free_host_run(r); return st; }
  }
  if ((size_t)n_det > r.det_cap || !r.h_det_dev[0]) {
    for (int k = 0; k < 2; ++k) {
      if (r.h_det_dev[k]) cudaFree(r.h_det_dev[k]);
      r.h_det_dev[k] = nullptr;
    }
    r.det_cap = 0;
    for (int k = 0; k < 2; ++k)
      MKF_CUDA(cudaMalloc(&r.h_det_dev[k], std::max<size_t>(1, (size_t)n_det) * 2 * sizeof(float)));
    r.det_cap = (size_t)n_det;
  }
  // outputs: written by the kernels straight into the caller's buffers when
  // those are pinned and mapped, else staged on the device and copied after
  float* o_est = static_cast<float*>(mapped_device_ptr(est));
  float* o_ll = static_cast<float*>(mapped_device_ptr(loglik));
  float* o_ess = static_cast<float*>(mapped_device_ptr(ess));
  int* o_st = static_cast<int*>(mapped_device_ptr(status));
  const bool direct = o_est && o_ll && o_ess && o_st;
  if (!direct) { o_est = B->d_est; o_ll = B->d_ll; o_ess = B->d_ess; o_st = B->d_status; }

  MKF_CUDA(cudaEventRecord(r.start, s));
  for (cudaStream_t x : {r.copy, r.comp[0], r.comp[1]}) MKF_CUDA(cudaStreamWaitEvent(x, r.start, 0));
  // head tracks' lists into buffer 0, track by track
  for (int q = 0; q < r.head; ++q) {
    const mkf_bpf_track& t = B->tracks[B->order_h[q]];
    if (t.n_frames <= 0) continue;
    const size_t e0 = (size_t)t.frame_base * J, e1 = (size_t)(t.frame_base + t.n_frames) * J + 1;
    MKF_CUDA(cudaMemcpyAsync(r.h_det_off_dev[0] + e0, det_off + e0, (e1 - e0) * sizeof(int), cudaMemcpyHostToDevice, r.copy));
    const size_t o0 = (size_t)det_off[e0], o1 = (size_t)det_off[e1 - 1];
    if (o1 > o0)
      MKF_CUDA(cudaMemcpyAsync(r.h_det_dev[0] + 2 * o0, det + 2 * o0, (o1 - o0) * 2 * sizeof(float),
                               cudaMemcpyHostToDevice, r.copy));
  }
  MKF_CUDA(cudaEventRecord(r.copied[0], r.copy));
  // everything into buffer 1, for the tail
  if (r.head < B->n_tracks) {
    MKF_CUDA(cudaMemcpyAsync(r.h_det_off_dev[1], det_off, (G * J + 1) * sizeof(int), cudaMemcpyHostToDevice, r.copy));
    MKF_CUDA(cudaMemcpyAsync(r.h_det_dev[1], det, (size_t)n_det * 2 * sizeof(float), cudaMemcpyHostToDevice, r.copy));
  }
  MKF_CUDA(cudaEventRecord(r.copied[1], r.copy));
  for (int k = 0; k < 2; ++k) {
    const int n = k == 0 ? r.head : B->n_tracks - r.head;
    cudaStream_t cs = r.comp[k];
    MKF_CUDA(cudaStreamWaitEvent(cs, r.copied[k], 0));
    if (n > 0) {
      BatchArgs a = batch_args(B, r.h_det_off_dev[k], r.h_det_dev[k], o_est, o_ll, o_ess, o_st);
      a.order = B->order + (k == 0 ? 0 : r.head);
      a.n_tracks = n;
      a.counter = r.counters + k;
      int st = launch_any(B, a, cs, k);
      if (st) return st;
    }
    MKF_CUDA(cudaEventRecord(r.done[k], cs));
    MKF_CUDA(cudaStreamWaitEvent(s, r.done[k], 0));
  }
  if (!direct) {
    MKF_CUDA(cudaMemcpyAsync(est, B->d_est, G * d * sizeof(float), cudaMemcpyDeviceToHost, s));
    MKF_CUDA(cudaMemcpyAsync(loglik, B->d_ll, G * sizeof(float), cudaMemcpyDeviceToHost, s));
    MKF_CUDA(cudaMemcpyAsync(ess, B->d_ess, G * sizeof(float), cudaMemcpyDeviceToHost, s));
    MKF_CUDA(cudaMemcpyAsync(status, B->d_status, B->n_tracks * sizeof(int), cudaMemcpyDeviceToHost, s));
  }
  MKF_CUDA(cudaStreamSynchronize(s));
  return MKF_OK;
}

extern "C" int mkf_bpf_batch_destroy(mkf_bpf_batch_t B) {
  if (!B) return MKF_OK;
  void* ps[] = {B->meta, B->fbase, B->seed, B->obs, B->order, B->counter, B->scratch,
                B->d_est, B->d_ll, B->d_ess, B->d_status};
  for (void* p : ps) if (p) cudaFree(p);
  free_host_run(B->hr);
  free_models(B->m);
  delete B;
  return MKF_OK;
}
