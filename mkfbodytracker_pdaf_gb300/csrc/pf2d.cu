// pf2d.cu -- the legacy bootstrap particle filter pf2D (pf2D.cpp:13-268) with
// its own my_gmm prior (pf2D.h:12-23), FP64, literal semantics: float expf in
// the GMM prior density, stale weights after resampling, uniform
// re-initialisation when every weight is zero, N(0, 5^2) random walk on
// columns 0..7.  Draws come from Philox instead of rand()/cv::randu/randn.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "mkf_common.cuh"

namespace mkf {

constexpr uint32_t kStreamPf2dUniform = 0x200u;   // + c/4 for column c
constexpr uint32_t kStreamPf2dNormal = 0x210u;    // two blocks: 8 normals

// uniform of particle i, column c at this frame (53-bit-exact double from one word)
__device__ __forceinline__ double pf2d_uniform(uint64_t seed, uint32_t track, uint32_t frame, int i, int c) {
  u32x4 w = draw_block(seed, track, frame, (uint32_t)i, kStreamPf2dUniform + (uint32_t)(c >> 2));
  const uint32_t v = (c & 3) == 0 ? w.x : (c & 3) == 1 ? w.y : (c & 3) == 2 ? w.z : w.w;
  return (double)v * (1.0 / 4294967296.0);
}

__device__ __forceinline__ void pf2d_normals(uint64_t seed, uint32_t track, uint32_t frame, int i, double* e) {
  for (int b = 0; b < 2; ++b) {
    u32x4 w = draw_block(seed, track, frame, (uint32_t)i, kStreamPf2dNormal + (uint32_t)b);
    float z0, z1, z2, z3;
    box_muller(w.x, w.y, z0, z1);
    box_muller(w.z, w.w, z2, z3);
    e[4 * b] = z0; e[4 * b + 1] = z1; e[4 * b + 2] = z2; e[4 * b + 3] = z3;
  }
}

struct Pf2dArgs {
  int N, d, K, side, width, height;
  uint64_t seed;
  uint32_t track, frame, U;
  const double *mean, *sinv, *det_s, *w;
  double z[4];
  double *x, *xold, *wts;
  int* anc;
  int* flag;       // [0] re-initialised this frame
  int* status;
};

// column ranges of the constructor's cv::randu (pf2D.cpp:57-70)
__device__ __forceinline__ void pf2d_range(const Pf2dArgs& A, int c, double* lo, double* hi) {
  if (c == 6) {
    *lo = A.width / 2.0 * A.side + 1.0;
    *hi = A.width / 2.0 + A.width / 2.0 * A.side;
  } else {
    *lo = 1.0;
    *hi = ((c % 2) == 0) * (double)A.width + (((c + 1) % 2) == 0) * (double)A.height;
  }
}

__global__ void pf2d_init_kernel(Pf2dArgs A) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < A.N * A.d; t += gridDim.x * blockDim.x) {
    const int i = t / A.d, c = t - i * A.d;
    double lo, hi;
    pf2d_range(A, c, &lo, &hi);
    A.x[t] = lo + pf2d_uniform(A.seed, A.track, kFramePrior, i, c) * (hi - lo);
    if (c == 0) A.wts[i] = 1.0 / (double)A.N;
  }
}

// prior (GMM with float expf, pf2D.cpp:157-164) x likelihood (pf2D.cpp:168)
__global__ void pf2d_weight_kernel(Pf2dArgs A) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.N) return;
  const int d = A.d;
  const double* x = A.x + (size_t)i * d;
  double prior = 0.0;
  for (int k = 0; k < A.K; ++k) {
    const double* mu = A.mean + (size_t)k * d;
    const double* Si = A.sinv + (size_t)k * d * d;
    double q = 0.0;
    for (int r = 0; r < d; ++r) {
      double t = 0.0;
      for (int c = 0; c < d; ++c) t += Si[r * d + c] * (x[c] - mu[c]);
      q += (x[r] - mu[r]) * t;
    }
    prior += A.w[k] * A.det_s[k] * (double)expf((float)(-0.5 * q));
  }
  const double d0 = x[6] - A.z[0], d1 = x[7] - A.z[1], h0 = x[0] - A.z[2], h1 = x[1] - A.z[3];
  const double c15 = 1.0 / (2.0 * 3.14159265358979323846 * 15.0);
  const double lik = c15 * exp(-0.5 * (d0 * d0 + d1 * d1) / 15.0) * c15 * exp(-0.5 * (h0 * h0 + h1 * h1) / 15.0);
  A.wts[i] = prior * lik;
}

// normalise by the sum (pf2D.cpp:171-177), then resample (pf2D.cpp:225-268)
__global__ void __launch_bounds__(1024) pf2d_resample_kernel(Pf2dArgs A) {
  __shared__ double red[32];
  __shared__ uint64_t red64[34];
  const int tid = threadIdx.x, TB = blockDim.x, lane = tid & 31, wid = tid >> 5, nw = TB >> 5;
  const int N = A.N;
  double s = 0.0;
  for (int i = tid; i < N; i += TB) s += A.wts[i];
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
  double mw = 0.0;
  for (int i = tid; i < N; i += TB) {
    const double v = A.wts[i] / sum;
    A.wts[i] = v;
    if (v > mw) mw = v;              // maxWeight ignores NaN (pf2D.cpp:212-223)
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) mw = fmax(mw, __shfl_xor_sync(0xffffffffu, mw, o));
  if (lane == 0) red[wid] = mw;
  __syncthreads();
  if (tid == 0) {
    double t = 0.0;
    for (int q = 0; q < nw; ++q) t = fmax(t, red[q]);
    red[0] = t;
    A.flag[0] = (t > 0.0) ? 0 : 1;
  }
  __syncthreads();
  mw = red[0];
  if (!(mw > 0.0)) {
    if (tid == 0) atomicOr(A.status, MKF_ST_FALLBACK);
    for (int i = tid; i < N; i += TB) A.anc[i] = -1;
    return;
  }
  int e;
  frexp(mw, &e);
  const int E = (N + TB - 1) / TB;
  const int j0 = min(N, tid * E), j1 = min(N, j0 + E);
  uint64_t cs = 0;
  for (int j = j0; j < j1; ++j) cs += quantize_f64(A.wts[j], e);
  uint64_t Qt;
  const uint64_t P = block_excl_scan_u64(cs, red64, &Qt);
  scatter_walk(j0, j1, P, N, A.U, Qt, [&](int j) { return quantize_f64(A.wts[j], e); }, A.anc);
}

// particles <- old[anc] (or uniform re-init), then predict: cols 0..7 += N(0, 5^2)
__global__ void pf2d_move_kernel(Pf2dArgs A) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.N) return;
  const int d = A.d;
  const bool reinit = A.flag[0] != 0;
  double* x = A.x + (size_t)i * d;
  if (reinit) {
    for (int c = 0; c < d; ++c) {
      double lo, hi;
      pf2d_range(A, c, &lo, &hi);
      x[c] = lo + pf2d_uniform(A.seed, A.track, A.frame, i, c) * (hi - lo);
    }
    A.wts[i] = 1.0 / (double)A.N;
  } else {
    const double* src = A.xold + (size_t)A.anc[i] * d;
    for (int c = 0; c < d; ++c) x[c] = src[c];
  }
  double e[8];
  pf2d_normals(A.seed, A.track, A.frame, i, e);
  for (int c = 0; c < 8 && c < d; ++c) x[c] += 5.0 * e[c];
}

// getEstimator: sum_i weights[i] * particles.row(i) (pf2D.cpp:79-87)
__global__ void __launch_bounds__(256) pf2d_estimate_kernel(const double* x, const double* w, int N, int d, double* est) {
  __shared__ double red[8];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  for (int c = 0; c < d; ++c) {
    double s = 0.0;
    for (int i = tid; i < N; i += blockDim.x) s += w[i] * x[(size_t)i * d + c];
    s = warp_sum_d(s);
    if (lane == 0) red[wid] = s;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += red[q];
      est[c] = t;
    }
    __syncthreads();
  }
}

__global__ void pf2d_draws_kernel(uint64_t seed, uint32_t track, uint32_t frame, int N, int d, double* eps, double* u) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  double e[8];
  pf2d_normals(seed, track, frame, i, e);
  for (int c = 0; c < 8; ++c) eps[(size_t)i * 8 + c] = e[c];
  for (int c = 0; c < d; ++c) u[(size_t)i * d + c] = pf2d_uniform(seed, track, frame, i, c);
}

// host: Cholesky-based inverse and normaliser of one covariance (my_gmm::loadGaussian, pf2D.cpp:26-37)
static bool host_spd_inverse(int d, const double* S, double* Si, double* det_s) {
  std::vector<double> L((size_t)d * d, 0.0), Li((size_t)d * d, 0.0);
  double ld = 0.0;
  for (int i = 0; i < d; ++i)
    for (int j = 0; j <= i; ++j) {
      double s = S[i * d + j];
      for (int k = 0; k < j; ++k) s -= L[i * d + k] * L[j * d + k];
      if (i == j) {
        if (!(s > 0.0)) return false;
        L[i * d + i] = std::sqrt(s);
        ld += 2.0 * std::log(L[i * d + i]);
      } else {
        L[i * d + j] = s / L[j * d + j];
      }
    }
  for (int i = 0; i < d; ++i) {
    Li[i * d + i] = 1.0 / L[i * d + i];
    for (int j = 0; j < i; ++j) {
      double s = 0.0;
      for (int k = j; k < i; ++k) s -= L[i * d + k] * Li[k * d + j];
      Li[i * d + j] = s / L[i * d + i];
    }
  }
  for (int a = 0; a < d; ++a)
    for (int b = 0; b < d; ++b) {
      double s = 0.0;
      for (int k = std::max(a, b); k < d; ++k) s += Li[k * d + a] * Li[k * d + b];
      Si[a * d + b] = s;
    }
  *det_s = 1.0 / (std::pow(2.0 * 3.14159265358979323846, d / 2.0) * std::sqrt(std::exp(ld)));
  return true;
}

}  // namespace mkf

using namespace mkf;

struct mkf_pf2d {
  int N, d, K, side, width, height;
  uint64_t seed;
  uint32_t track;
  double *mean, *sinv, *det_s, *w, *x, *xold, *wts;
  int *anc, *flag, *status;
};

static Pf2dArgs pf2d_args(mkf_pf2d* h) {
  Pf2dArgs a;
  memset(&a, 0, sizeof(a));
  a.N = h->N; a.d = h->d; a.K = h->K; a.side = h->side; a.width = h->width; a.height = h->height;
  a.seed = h->seed; a.track = h->track;
  a.mean = h->mean; a.sinv = h->sinv; a.det_s = h->det_s; a.w = h->w;
  a.x = h->x; a.xold = h->xold; a.wts = h->wts; a.anc = h->anc; a.flag = h->flag; a.status = h->status;
  return a;
}

extern "C" int mkf_pf2d_create(int n_particles, int d, int side, int K, const double* mean, const double* cov,
                               const double* w, int width, int height, uint64_t seed, uint32_t track_id,
                               mkf_pf2d_t* out) {
  MKF_ARG(out && mean && cov && w, "mkf_pf2d_create: null argument");
  MKF_ARG(n_particles >= 1 && n_particles <= 65536, "mkf_pf2d_create: n_particles out of range");
  MKF_ARG(d >= 8 && d <= 32, "mkf_pf2d_create: d must be in [8, 32] (columns 0..7 are image coordinates)");
  MKF_ARG(K >= 1 && K <= 64 && width > 1 && height > 1, "mkf_pf2d_create: bad K or image size");
  std::vector<double> sinv((size_t)K * d * d), det((size_t)K);
  for (int k = 0; k < K; ++k)
    if (!host_spd_inverse(d, cov + (size_t)k * d * d, &sinv[(size_t)k * d * d], &det[k])) {
      set_error("mkf_pf2d_create: a component covariance is not positive definite");
      return MKF_ERR_NONPD;
    }
  mkf_pf2d* h = new (std::nothrow) mkf_pf2d();
  if (!h) return MKF_ERR_NOMEM;
  memset(h, 0, sizeof(*h));
  h->N = n_particles; h->d = d; h->K = K; h->side = side ? 1 : 0; h->width = width; h->height = height;
  h->seed = seed; h->track = track_id;
  cudaError_t e = cudaSuccess;
  auto al = [&](void** p, size_t b) { if (e == cudaSuccess) e = cudaMalloc(p, std::max<size_t>(b, 8)); };
  auto cp = [&](void* dst, const void* src, size_t b) { if (e == cudaSuccess) e = cudaMemcpy(dst, src, b, cudaMemcpyHostToDevice); };
  const size_t N = n_particles;
  al((void**)&h->mean, sizeof(double) * K * d); al((void**)&h->sinv, sizeof(double) * K * d * d);
  al((void**)&h->det_s, sizeof(double) * K); al((void**)&h->w, sizeof(double) * K);
  al((void**)&h->x, sizeof(double) * N * d); al((void**)&h->xold, sizeof(double) * N * d);
  al((void**)&h->wts, sizeof(double) * N); al((void**)&h->anc, sizeof(int) * N);
  al((void**)&h->flag, sizeof(int)); al((void**)&h->status, sizeof(int));
  cp(h->mean, mean, sizeof(double) * K * d); cp(h->sinv, sinv.data(), sizeof(double) * K * d * d);
  cp(h->det_s, det.data(), sizeof(double) * K); cp(h->w, w, sizeof(double) * K);
  if (e == cudaSuccess) e = cudaMemset(h->status, 0, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(h->flag, 0, sizeof(int));
  if (e != cudaSuccess) {
    mkf_pf2d_destroy(h);
    return cuda_fail(e, "mkf_pf2d_create: allocation", __FILE__, __LINE__);
  }
  Pf2dArgs a = pf2d_args(h);
  pf2d_init_kernel<<<(int)std::min<size_t>((N * d + 255) / 256, 4096), 256>>>(a);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    mkf_pf2d_destroy(h);
    return cuda_fail(e, "mkf_pf2d_create: init", __FILE__, __LINE__);
  }
  *out = h;
  return MKF_OK;
}

extern "C" int mkf_pf2d_update(mkf_pf2d_t h, uint32_t frame, const double* z, mkf_stream_t stream) {
  MKF_RANGE("mkf_pf2d_update");
  MKF_ARG(h && z, "mkf_pf2d_update: null argument");
  cudaStream_t s = (cudaStream_t)stream;
  Pf2dArgs a = pf2d_args(h);
  a.frame = frame;
  a.U = resample_uniform(h->seed, h->track, frame);
  for (int q = 0; q < 4; ++q) a.z[q] = z[q];
  const int g = (h->N + 127) / 128;
  pf2d_weight_kernel<<<g, 128, 0, s>>>(a);
  MKF_CHECK_LAUNCH("mkf_pf2d_update: weight kernel");
  pf2d_resample_kernel<<<1, 1024, 0, s>>>(a);
  MKF_CHECK_LAUNCH("mkf_pf2d_update: resample kernel");
  MKF_CUDA(cudaMemcpyAsync(h->xold, h->x, sizeof(double) * (size_t)h->N * h->d, cudaMemcpyDeviceToDevice, s));
  pf2d_move_kernel<<<g, 128, 0, s>>>(a);
  MKF_CHECK_LAUNCH("mkf_pf2d_update: move kernel");
  return MKF_OK;
}

extern "C" int mkf_pf2d_estimate(mkf_pf2d_t h, double* d_est, mkf_stream_t stream) {
  MKF_ARG(h && d_est, "mkf_pf2d_estimate: null argument");
  pf2d_estimate_kernel<<<1, 256, 0, (cudaStream_t)stream>>>(h->x, h->wts, h->N, h->d, d_est);
  MKF_CHECK_LAUNCH("mkf_pf2d_estimate");
  return MKF_OK;
}

extern "C" int mkf_pf2d_read(mkf_pf2d_t h, double* d_particles, double* d_weights, int* d_anc, int* reinit,
                             mkf_stream_t stream) {
  MKF_ARG(h, "mkf_pf2d_read: null handle");
  cudaStream_t s = (cudaStream_t)stream;
  const size_t N = h->N;
  if (d_particles) MKF_CUDA(cudaMemcpyAsync(d_particles, h->x, sizeof(double) * N * h->d, cudaMemcpyDeviceToDevice, s));
  if (d_weights) MKF_CUDA(cudaMemcpyAsync(d_weights, h->wts, sizeof(double) * N, cudaMemcpyDeviceToDevice, s));
  if (d_anc) MKF_CUDA(cudaMemcpyAsync(d_anc, h->anc, sizeof(int) * N, cudaMemcpyDeviceToDevice, s));
  if (reinit) {
    MKF_CUDA(cudaMemcpyAsync(reinit, h->flag, sizeof(int), cudaMemcpyDeviceToHost, s));
    MKF_CUDA(cudaStreamSynchronize(s));
  }
  return MKF_OK;
}

extern "C" int mkf_pf2d_draws(uint64_t seed, uint32_t track, uint32_t frame, int n, int d, double* d_eps,
                              double* d_u, mkf_stream_t stream) {
  MKF_ARG(d_eps && d_u && n >= 1 && d >= 8 && d <= 32, "mkf_pf2d_draws: bad argument");
  pf2d_draws_kernel<<<(n + 127) / 128, 128, 0, (cudaStream_t)stream>>>(seed, track, frame, n, d, d_eps, d_u);
  MKF_CHECK_LAUNCH("mkf_pf2d_draws");
  return MKF_OK;
}

extern "C" int mkf_pf2d_destroy(mkf_pf2d_t h) {
  if (!h) return MKF_OK;
  void* ps[] = {h->mean, h->sinv, h->det_s, h->w, h->x, h->xold, h->wts, h->anc, h->flag, h->status};
  for (void* p : ps) if (p) cudaFree(p);
  delete h;
  return MKF_OK;
}
