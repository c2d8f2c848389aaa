// util.cu -- error plumbing, draws, and the standalone systematic resampler
// (ParticleFilter::resample, pf2DRao.cpp:175-210).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "mkf_common.cuh"

namespace mkf {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

int cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
  char buf[512];
  snprintf(buf, sizeof(buf), "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
  g_last_error = buf;
  return e == cudaErrorMemoryAllocation ? MKF_ERR_NOMEM : MKF_ERR_CUDA;
}

int num_sms() {
  int dev = 0, n = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  return n > 0 ? n : 1;
}

// ------------------------------------------------------------------ draws
template <int D>
__global__ void draw_particles_kernel(uint64_t seed, uint32_t track, uint32_t frame, int n,
                                      float* eps, float* ucomp) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float e[D];
  float u = particle_draws<D>(seed, track, frame, (uint32_t)i, e);
#pragma unroll
  for (int r = 0; r < D; ++r) eps[(size_t)i * D + r] = e[r];
  ucomp[i] = u;
}

// ------------------------------------------------------------------ standalone resampler
// Scratch: per-device cache grown on demand (block sums + frame scalars).
struct RsScratch {
  unsigned long long* bsum = nullptr;
  unsigned long long* wmax_bits = nullptr;   // [0] max bits (f32 or f64), [1] +inf flag
  unsigned int* ticket = nullptr;
  unsigned long long* qt = nullptr;
  int cap = 0;
};
static std::mutex g_rs_mu;
static RsScratch g_rs[64];

static int rs_get(int nb, RsScratch** out) {
  int dev = 0;
  MKF_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) { set_error("resample: device index out of range"); return MKF_ERR_ARG; }
  std::lock_guard<std::mutex> lk(g_rs_mu);
  RsScratch& s = g_rs[dev];
  if (s.cap < nb) {
    if (s.bsum) cudaFree(s.bsum);
    s.bsum = nullptr;
    s.cap = 0;
    MKF_CUDA(cudaMalloc(&s.bsum, sizeof(unsigned long long) * (size_t)nb));
    s.cap = nb;
  }
  if (!s.wmax_bits) {
    MKF_CUDA(cudaMalloc(&s.wmax_bits, sizeof(unsigned long long) * 4));
    s.ticket = reinterpret_cast<unsigned int*>(s.wmax_bits + 2);
    s.qt = s.wmax_bits + 3;
  }
  *out = &s;
  return MKF_OK;
}

template <typename T> struct WTraits;
template <> struct WTraits<float> {
  static __device__ __forceinline__ unsigned long long bits(float v) { return (unsigned long long)__float_as_uint(v); }
  static __device__ __forceinline__ float from(unsigned long long b) { return __uint_as_float((unsigned)b); }
  static __device__ __forceinline__ int expo(float m) { int e; frexpf(m, &e); return e; }
  static __device__ __forceinline__ uint64_t q(float w, int e) { return quantize_f32(w, e); }
};
template <> struct WTraits<double> {
  static __device__ __forceinline__ unsigned long long bits(double v) { return (unsigned long long)__double_as_longlong(v); }
  static __device__ __forceinline__ double from(unsigned long long b) { return __longlong_as_double((long long)b); }
  static __device__ __forceinline__ int expo(double m) { int e; frexp(m, &e); return e; }
  static __device__ __forceinline__ uint64_t q(double w, int e) { return quantize_f64(w, e); }
};

constexpr int kRsTB = 256;
constexpr int kRsTile = 4096;

// pass 1: max of the sanitised weights (nonnegative floats order like their bits)
template <typename T>
__global__ void __launch_bounds__(kRsTB) rs_max(const T* w, int L, unsigned long long* wm) {
  __shared__ unsigned long long s[kRsTB / 32];
  unsigned long long m = 0;
  int inf = 0;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < L; j += gridDim.x * blockDim.x) {
    T v = w[j];
    if (isinf(v) && v > 0) inf = 1;
    else if (v > (T)0) m = max(m, WTraits<T>::bits(v));
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    inf |= __shfl_xor_sync(0xffffffffu, inf, o);
  }
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long r = 0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) r = max(r, s[q]);
    atomicMax(&wm[0], r);
  }
  if (inf && (threadIdx.x & 31) == 0) atomicOr(&wm[1], 1ull);
}

template <typename T>
__device__ __forceinline__ bool rs_state(const unsigned long long* wm, int* e) {
  T mx = WTraits<T>::from(wm[0]);
  bool fb = (wm[1] != 0ull) || !(mx > (T)0);
  *e = fb ? 0 : WTraits<T>::expo(mx);
  return fb;
}

// pass 2: block sums of quantised weights, last block scans them (exclusive)
template <typename T>
__global__ void __launch_bounds__(kRsTB) rs_sum(const T* w, int L, unsigned long long* wm,
                                               unsigned long long* bsum, unsigned int* ticket,
                                               unsigned long long* qt) {
  __shared__ uint64_t red[34];
  __shared__ bool last;
  int e;
  bool fb = rs_state<T>(wm, &e);
  const int base = blockIdx.x * kRsTile, end = min(L, base + kRsTile);
  const int E = kRsTile / kRsTB;
  const int j0 = min(end, base + threadIdx.x * E), j1 = min(end, j0 + E);
  uint64_t cs = 0;
  if (!fb)
    for (int j = j0; j < j1; ++j) cs += WTraits<T>::q(w[j], e);
  uint64_t tot;
  block_excl_scan_u64(cs, red, &tot);
  if (threadIdx.x == 0) {
    bsum[blockIdx.x] = tot;
    __threadfence();
    last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  const int nb = gridDim.x, E2 = (nb + kRsTB - 1) / kRsTB;
  const int q0 = min(nb, (int)threadIdx.x * E2), q1 = min(nb, q0 + E2);
  uint64_t c2 = 0;
  for (int q = q0; q < q1; ++q) c2 += ((volatile unsigned long long*)bsum)[q];
  uint64_t Qt;
  uint64_t pre = block_excl_scan_u64(c2, red, &Qt);
  __syncthreads();
  for (int q = q0; q < q1; ++q) {
    uint64_t v = ((volatile unsigned long long*)bsum)[q];
    bsum[q] = pre;
    pre += v;
  }
  if (threadIdx.x == 0) { *qt = Qt; *ticket = 0u; }
}

__device__ __forceinline__ int rs_count_le(uint64_t X, int N, uint32_t U, uint64_t Qt) {
  const unsigned __int128 lim = ((unsigned __int128)(uint64_t)N * (unsigned __int128)X) << 32;
  long long lo = 0, hi = N;
  while (lo < hi) {
    long long mid = (lo + hi) >> 1;
    if (resample_rhs((int)mid, U, Qt) <= lim) lo = mid + 1; else hi = mid;
  }
  return (int)lo;
}

// pass 3: each weight tile emits the ancestors of the targets that fall in it
template <typename T>
__global__ void __launch_bounds__(kRsTB) rs_search(const T* w, int L, int N, uint32_t U,
                                                  const unsigned long long* wm,
                                                  const unsigned long long* bsum,
                                                  const unsigned long long* qt, int* idx,
                                                  int* fallback) {
  __shared__ uint64_t sQ[kRsTile];
  __shared__ uint64_t red[34];
  __shared__ int s_lo, s_hi;
  int e;
  bool fb = rs_state<T>(wm, &e);
  const uint64_t Qt = *qt;
  if (fb || Qt == 0ull) {
    // uniform-random indices (pf2DRao.cpp:184-192): block b covers targets [b*ceil(N/nb) ..)
    const int per = (N + gridDim.x - 1) / gridDim.x;
    const int i0 = blockIdx.x * per, i1 = min(N, i0 + per);
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) idx[i] = resample_fallback_index(U, i, L);
    if (fallback && blockIdx.x == 0 && threadIdx.x == 0) *fallback = 1;
    return;
  }
  if (fallback && blockIdx.x == 0 && threadIdx.x == 0) *fallback = 0;
  const int base = blockIdx.x * kRsTile, end = min(L, base + kRsTile), n = end - base;
  const int E = kRsTile / kRsTB;
  const int j0 = min(end, base + (int)threadIdx.x * E), j1 = min(end, j0 + E);
  uint64_t cs = 0;
  for (int j = j0; j < j1; ++j) cs += WTraits<T>::q(w[j], e);
  uint64_t tot;
  uint64_t pre = block_excl_scan_u64(cs, red, &tot) + bsum[blockIdx.x];
  for (int j = j0; j < j1; ++j) {
    pre += WTraits<T>::q(w[j], e);
    sQ[j - base] = pre;
  }
  if (threadIdx.x == 0) {
    uint64_t Xprev = bsum[blockIdx.x];
    s_lo = (blockIdx.x == 0) ? 0 : rs_count_le(Xprev, N, U, Qt);
    s_hi = (blockIdx.x == gridDim.x - 1) ? N : rs_count_le(Xprev + tot, N, U, Qt);
  }
  __syncthreads();
  for (int i = s_lo + (int)threadIdx.x; i < s_hi; i += blockDim.x)
    idx[i] = base + resample_search(sQ, n, N, resample_rhs(i, U, Qt));
}

template <typename T>
static int resample_impl(const T* d_w, int L, int N, uint32_t U, int* d_idx, int* d_fb, cudaStream_t s) {
  MKF_ARG(d_w && d_idx, "mkf_resample: null pointer");
  MKF_ARG(L >= 1 && L <= (1 << 23) && N >= 1 && N <= (1 << 23), "mkf_resample: L and N must be in [1, 2^23]");
  const int nb = (L + kRsTile - 1) / kRsTile;
  RsScratch* sc;
  int st = rs_get(nb, &sc);
  if (st) return st;
  MKF_CUDA(cudaMemsetAsync(sc->wmax_bits, 0, sizeof(unsigned long long) * 4, s));
  const int g1 = std::min(std::max(1, (L + kRsTB - 1) / kRsTB), 4 * num_sms());
  rs_max<T><<<g1, kRsTB, 0, s>>>(d_w, L, sc->wmax_bits);
  MKF_CHECK_LAUNCH("mkf_resample: max kernel");
  rs_sum<T><<<nb, kRsTB, 0, s>>>(d_w, L, sc->wmax_bits, sc->bsum, sc->ticket, sc->qt);
  MKF_CHECK_LAUNCH("mkf_resample: sum kernel");
  rs_search<T><<<nb, kRsTB, 0, s>>>(d_w, L, N, U, sc->wmax_bits, sc->bsum, sc->qt, d_idx, d_fb);
  MKF_CHECK_LAUNCH("mkf_resample: search kernel");
  return MKF_OK;
}

}  // namespace mkf

using namespace mkf;

extern "C" const char* mkf_version(void) { return "mkfbodytracker_pdaf_gb300 0.1.0 (sm_103a)"; }
extern "C" const char* mkf_last_error(void) { return g_last_error.c_str(); }

extern "C" int mkf_philox_block(uint64_t seed, uint32_t track, uint32_t frame, uint32_t item,
                                uint32_t stream, uint32_t out[4]) {
  MKF_ARG(out, "mkf_philox_block: null output");
  u32x4 o = draw_block(seed, track, frame, item, stream);
  out[0] = o.x; out[1] = o.y; out[2] = o.z; out[3] = o.w;
  return MKF_OK;
}

extern "C" int mkf_draw_particles(uint64_t seed, uint32_t track, uint32_t frame, int n, int d,
                                  float* d_eps, float* d_ucomp, mkf_stream_t stream) {
  MKF_ARG(d_eps && d_ucomp && n >= 0, "mkf_draw_particles: bad argument");
  MKF_ARG(d == 12 || d == 24, "mkf_draw_particles: d must be 12 or 24");
  if (n == 0) return MKF_OK;
  cudaStream_t s = (cudaStream_t)stream;
  int g = (n + 255) / 256;
  if (d == 12) draw_particles_kernel<12><<<g, 256, 0, s>>>(seed, track, frame, n, d_eps, d_ucomp);
  else draw_particles_kernel<24><<<g, 256, 0, s>>>(seed, track, frame, n, d_eps, d_ucomp);
  MKF_CHECK_LAUNCH("mkf_draw_particles");
  return MKF_OK;
}

extern "C" int mkf_resample_f64(const double* d_w, int L, int N, uint32_t U, int* d_idx, int* d_fallback,
                                mkf_stream_t stream) {
  MKF_RANGE("mkf_resample_f64");
  return resample_impl<double>(d_w, L, N, U, d_idx, d_fallback, (cudaStream_t)stream);
}
extern "C" int mkf_resample_f32(const float* d_w, int L, int N, uint32_t U, int* d_idx, int* d_fallback,
                                mkf_stream_t stream) {
  MKF_RANGE("mkf_resample_f32");
  return resample_impl<float>(d_w, L, N, U, d_idx, d_fallback, (cudaStream_t)stream);
}

// ------------------------------------------------------------------ allocation-free resampler
// mkf_resample_f32_noalloc: the same exact systematic resampler as
// mkf_resample_f32, for callers that must not allocate device memory -- for
// example a per-frame tracking loop with a hard latency budget (cudaMalloc and
// cudaFree can synchronise the whole device) or an application that budgets
// all of its device memory up front.  Its scratch (per-block integer sums and
// four control words) lives in the fixed file-scope array below, sized for at
// most kNoAllocMaxWeights weights; every GPU that loads this library holds the
// array until the process exits.
namespace mkf {

constexpr int kNoAllocMaxWeights = 1 << 20;
constexpr int kNoAllocMaxBlocks = kNoAllocMaxWeights / kRsTile;      // 256 weight tiles
// [0] max-weight bits, [1] +inf flag, [2] ticket (as two u32), [3] total, then block sums
static __device__ __align__(256) unsigned long long g_resample_noalloc_scratch[4 + kNoAllocMaxBlocks];

static std::mutex g_noalloc_mu;
static unsigned long long* g_noalloc_ptr[64];

// Host code cannot use the array's name as a device address, so the address is
// looked up once per device (with that device current) on its first call.
static int noalloc_scratch(unsigned long long** out) {
  int dev = 0;
  MKF_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) { set_error("mkf_resample_f32_noalloc: device index out of range"); return MKF_ERR_ARG; }
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_resample_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "mkf_resample_f32_noalloc: cudaGetSymbolAddress", __FILE__, __LINE__);
    g_noalloc_ptr[dev] = static_cast<unsigned long long*>(p);
  }
  *out = g_noalloc_ptr[dev];
  return MKF_OK;
}

}  // namespace mkf

extern "C" int mkf_resample_f32_noalloc(const float* d_w, int L, int N, uint32_t U, int* d_idx,
                                        int* d_fallback, mkf_stream_t stream) {
  MKF_RANGE("mkf_resample_f32_noalloc");
  MKF_ARG(d_w && d_idx, "mkf_resample_f32_noalloc: null pointer");
  if (L < 1 || L > kNoAllocMaxWeights) {
    set_error("mkf_resample_f32_noalloc: L must be in [1, 1048576] (the fixed scratch holds 256 tiles "
              "of 4096 weights); use mkf_resample_f32 for larger inputs");
    return MKF_ERR_ARG;
  }
  MKF_ARG(N >= 1 && N <= (1 << 23), "mkf_resample_f32_noalloc: N must be in [1, 2^23]");
  unsigned long long* sc = nullptr;
  int st = noalloc_scratch(&sc);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const int nb = (L + kRsTile - 1) / kRsTile;
  // the max bits, the +inf flag and the ticket must start at zero on every call
  MKF_CUDA(cudaMemsetAsync(sc, 0, sizeof(unsigned long long) * 4, s));
  unsigned long long* wm = sc;
  unsigned int* ticket = reinterpret_cast<unsigned int*>(sc + 2);
  unsigned long long* qt = sc + 3;
  unsigned long long* bsum = sc + 4;
  const int g1 = std::min(std::max(1, (L + kRsTB - 1) / kRsTB), 4 * num_sms());
  rs_max<float><<<g1, kRsTB, 0, s>>>(d_w, L, wm);
  MKF_CHECK_LAUNCH("mkf_resample_f32_noalloc: max kernel");
  rs_sum<float><<<nb, kRsTB, 0, s>>>(d_w, L, wm, bsum, ticket, qt);
  MKF_CHECK_LAUNCH("mkf_resample_f32_noalloc: sum kernel");
  rs_search<float><<<nb, kRsTB, 0, s>>>(d_w, L, N, U, wm, bsum, qt, d_idx, d_fallback);
  MKF_CHECK_LAUNCH("mkf_resample_f32_noalloc: search kernel");
  return MKF_OK;
}
