// mkf_common.cuh -- shared device/host pieces of the GB300 filtering hot path.
#pragma once
#include <cuda_runtime.h>
#include <math.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>
#include <string.h>
#include <string>
#include "../../include/mkf_gb300.h"

#define MKF_HD __host__ __device__ __forceinline__
// loop unrolling in host-and-device functions (the host compiler has no such pragma)
#ifdef __CUDA_ARCH__
#define MKF_UNROLL _Pragma("unroll")
#else
#define MKF_UNROLL
#endif

namespace mkf {

// ---------------------------------------------------------------- errors
void set_error(const std::string& msg);
int cuda_fail(cudaError_t e, const char* what, const char* file, int line);
#define MKF_CUDA(call)                                                   \
  do {                                                                   \
    cudaError_t _e = (call);                                             \
    if (_e != cudaSuccess) return ::mkf::cuda_fail(_e, #call, __FILE__, __LINE__); \
  } while (0)
#define MKF_CHECK_LAUNCH(what)                                           \
  do {                                                                   \
    cudaError_t _e = cudaGetLastError();                                 \
    if (_e != cudaSuccess) return ::mkf::cuda_fail(_e, what, __FILE__, __LINE__); \
  } while (0)
#define MKF_ARG(cond, msg)                                               \
  do {                                                                   \
    if (!(cond)) { ::mkf::set_error(msg); return MKF_ERR_ARG; }          \
  } while (0)

int num_sms();

// NVTX range around the host side of one C-ABI call (named on Nsight
// timelines; a no-op unless a tool is attached)
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};
#define MKF_RANGE(name) ::mkf::NvtxRange mkf_nvtx_range_(name)

// ---------------------------------------------------------------- Philox4x32-10
// Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3",
// SC'11.  Replaces cv::RNG / randn / rand() (pf2DRao.cpp:96,179; pf2D.cpp:228,255).
struct u32x4 { uint32_t x, y, z, w; };

MKF_HD u32x4 philox4x32_10(u32x4 c, uint32_t k0, uint32_t k1) {
  MKF_UNROLL
  for (int r = 0; r < 10; ++r) {
    if (r) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
#ifdef __CUDA_ARCH__
    uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
    uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
#else
    uint64_t p0 = (uint64_t)0xD2511F53u * c.x, p1 = (uint64_t)0xCD9E8D57u * c.z;
    uint32_t lo0 = (uint32_t)p0, hi0 = (uint32_t)(p0 >> 32);
    uint32_t lo1 = (uint32_t)p1, hi1 = (uint32_t)(p1 >> 32);
#endif
    u32x4 n;
    n.x = hi1 ^ c.y ^ k0;
    n.y = lo1;
    n.z = hi0 ^ c.w ^ k1;
    n.w = lo0;
    c = n;
  }
  return c;
}

MKF_HD u32x4 draw_block(uint64_t seed, uint32_t track, uint32_t frame, uint32_t item,
                        uint32_t stream) {
  u32x4 c{frame, item, stream, 0u};
  return philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32) ^ track);
}

constexpr uint32_t kFramePrior = 0xFFFFFFFFu;
constexpr uint32_t kItemFrame = 0xFFFFFFFFu;
constexpr uint32_t kStreamResample = 0x100u;

MKF_HD uint32_t resample_uniform(uint64_t seed, uint32_t track, uint32_t frame) {
  return draw_block(seed, track, frame, kItemFrame, kStreamResample).x;
}

// ---------------------------------------------------------------- Philox, split by item
// The particle draws are draw_block(seed, track, frame, item, stream) for the
// items of one frame: the counter {frame, item, stream, 0} varies only in its
// second word, which enters round 0 through one XOR.  Everything that does not
// depend on the item is therefore computed once per frame and stream:
//  round 0: both products (frame, stream) and three of the four output words;
//  round 1: the product of word 2 and word 0's output (x1 below);
//  round 2: the product of x1 and word 3's output (w2);
// and the round keys once per track.  Per item that leaves one XOR, one product
// and one XOR, then one product and two XORs, then seven full rounds: 34
// operations instead of 60.  philox_item equals philox4x32_10 bit for bit
// (checked on the host against the direct form).
struct alignas(16) PhiloxPre {
  uint32_t x0;   // round 0: word 0 = x0 ^ item
  uint32_t z1;   // round 1: word 2 = hi(M0 (x0 ^ item)) ^ z1
  uint32_t x2;   // round 2: word 0 = hi(M1 word2) ^ x2
  uint32_t z2;   // round 2: word 2 = lo(M0 (x0 ^ item)) ^ z2
  uint32_t w2;   // round 2: word 3
  uint32_t pad[3];
};
struct alignas(16) PhiloxKeys { uint32_t k[14]; uint32_t pad[2]; };   // (k0, k1) of rounds 3..9

MKF_HD void philox_mulhilo(uint32_t m, uint32_t a, uint32_t& lo, uint32_t& hi) {
#ifdef __CUDA_ARCH__
  lo = m * a;
  hi = __umulhi(m, a);
#else
  const uint64_t p = (uint64_t)m * a;
  lo = (uint32_t)p;
  hi = (uint32_t)(p >> 32);
#endif
}

MKF_HD PhiloxKeys philox_keys(uint64_t seed, uint32_t track) {
  PhiloxKeys ks;
  uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32) ^ track;
  for (int r = 1; r < 10; ++r) {
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    if (r >= 3) { ks.k[2 * (r - 3)] = k0; ks.k[2 * (r - 3) + 1] = k1; }
  }
  ks.pad[0] = ks.pad[1] = 0u;
  return ks;
}

MKF_HD PhiloxPre philox_pre(uint64_t seed, uint32_t track, uint32_t frame, uint32_t stream) {
  const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32) ^ track;
  uint32_t l0, h0, l1, h1;
  // round 0 on {frame, item, stream, 0}
  philox_mulhilo(0xD2511F53u, frame, l0, h0);
  philox_mulhilo(0xCD9E8D57u, stream, l1, h1);
  const uint32_t y0 = l1, z0 = h0 ^ k1, w0 = l0;
  PhiloxPre p;
  p.x0 = h1 ^ k0;
  // round 1: words 0 and 1 of the output depend only on z0 and y0
  philox_mulhilo(0xCD9E8D57u, z0, l1, h1);
  const uint32_t x1 = h1 ^ y0 ^ (k0 + 0x9E3779B9u), y1 = l1;
  p.z1 = w0 ^ (k1 + 0xBB67AE85u);
  // round 2: the product of x1
  philox_mulhilo(0xD2511F53u, x1, l0, h0);
  p.x2 = y1 ^ (k0 + 2u * 0x9E3779B9u);
  p.z2 = h0 ^ (k1 + 2u * 0xBB67AE85u);
  p.w2 = l0;
  p.pad[0] = p.pad[1] = p.pad[2] = 0u;
  return p;
}

// one round of philox4x32_10 with round key (k0, k1)
MKF_HD u32x4 philox_round(u32x4 c, uint32_t k0, uint32_t k1) {
  uint32_t lo0, hi0, lo1, hi1;
  philox_mulhilo(0xD2511F53u, c.x, lo0, hi0);
  philox_mulhilo(0xCD9E8D57u, c.z, lo1, hi1);
  return u32x4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
}

// rounds 0..2 of the split form: the counter words entering round 3
MKF_HD u32x4 philox_item_head(const PhiloxPre& p, uint32_t item) {
  uint32_t la, ha, lb, hb;
  philox_mulhilo(0xD2511F53u, p.x0 ^ item, la, ha);   // round 1, word 0's product
  const uint32_t z1 = ha ^ p.z1;                       // round 1 output: {x1, y1, z1, la}
  philox_mulhilo(0xCD9E8D57u, z1, lb, hb);             // round 2, word 2's product
  return u32x4{hb ^ p.x2, lb, la ^ p.z2, p.w2};
}

MKF_HD u32x4 philox_item(const PhiloxPre& p, const PhiloxKeys& ks, uint32_t item) {
  u32x4 c = philox_item_head(p, item);
  MKF_UNROLL
  for (int r = 0; r < 7; ++r) c = philox_round(c, ks.k[2 * r], ks.k[2 * r + 1]);
  return c;
}

#ifdef __CUDACC__
// global -> shared copies that complete asynchronously (cp.async: no registers
// held while in flight); the issuing thread waits for its own groups
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// 16 bytes from shared memory on every call (volatile: never hoisted into
// registers across a loop, which would cost the particle loops their registers)
__device__ __forceinline__ uint4 lds_u4(const void* p) {
  uint4 v;
  asm volatile("ld.shared.v4.u32 {%0, %1, %2, %3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "r"((uint32_t)__cvta_generic_to_shared(p)));
  return v;
}

// philox_item for NB streams of one item, the blocks advanced round by round
// (each round key read once for all of them); pre and ks in shared memory
template <int NB>
__device__ __forceinline__ void philox_items_smem(const PhiloxPre* pre, const PhiloxKeys* ks, uint32_t item,
                                                  u32x4* out) {
#pragma unroll
  for (int b = 0; b < NB; ++b) {
    const uint4 a = lds_u4(&pre[b].x0);
    const uint4 w = lds_u4(&pre[b].w2);
    PhiloxPre p;
    p.x0 = a.x; p.z1 = a.y; p.x2 = a.z; p.z2 = a.w; p.w2 = w.x;
    out[b] = philox_item_head(p, item);
  }
#pragma unroll
  for (int r = 0; r < 7; r += 2) {
    const uint4 k = lds_u4(&ks->k[2 * r]);
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      out[b] = philox_round(out[b], k.x, k.y);
      if (r + 1 < 7) out[b] = philox_round(out[b], k.z, k.w);
    }
  }
}
#endif

// ---------------------------------------------------------------- component pick
// First k with u < cumpi[k] (the last component if none): with cumpi
// nondecreasing that is the number of c < K-1 with cumpi[c] <= u, counted with
// independent loads instead of a dependent walk.
MKF_HD int pick_component(const float* cumpi, int K, float u) {
  int k = 0;
  for (int c = 0; c < K - 1; ++c) k += (u >= cumpi[c]) ? 1 : 0;
  return k;
}

// The same count from a table over kPickBins equal bins of [0, 1): entry b holds
// #{c < K-1 : cumpi[c] <= b / kPickBins} in its low 7 bits (K <= 128) and, in
// bit 7, whether some cumpi[c] falls strictly inside the bin; only then does the
// count continue past the bin's lower edge.  u is a multiple of 2^-23 in [0, 1),
// so u * kPickBins and its floor are exact.  build_pick_table fills entries
// tid, tid + TB, ... (a block fills it cooperatively).
constexpr int kPickBins = 1024;
MKF_HD void build_pick_table(const float* cumpi, int K, uint8_t* tab, int tid, int TB) {
  for (int b = tid; b < kPickBins; b += TB) {
    const float lo = (float)b * (1.0f / kPickBins), hi = (float)(b + 1) * (1.0f / kPickBins);
    int s = 0, s2 = 0;
    for (int c = 0; c < K - 1; ++c) {
      s += (cumpi[c] <= lo) ? 1 : 0;
      s2 += (cumpi[c] < hi) ? 1 : 0;
    }
    tab[b] = (uint8_t)(s | ((s2 > s) ? 0x80 : 0));
  }
}
MKF_HD int pick_component_table(const uint8_t* tab, const float* cumpi, int K, float u) {
#ifdef __CUDA_ARCH__
  const int e = tab[__float2int_rz(u * (float)kPickBins)];
#else
  const int e = tab[(int)(u * (float)kPickBins)];   // truncation, as __float2int_rz
#endif
  int k = e & 0x7F;
  if (e & 0x80)
    while (k < K - 1 && u >= cumpi[k]) ++k;
  return k;
}
// the same with u's bin floor(u kPickBins) given (the particle draws form it
// from the uniform's bits without a float-to-int conversion)
MKF_HD int pick_component_table_bin(const uint8_t* tab, const float* cumpi, int K, float u, int bin) {
  const int e = tab[bin];
  int k = e & 0x7F;
  if (e & 0x80)
    while (k < K - 1 && u >= cumpi[k]) ++k;
  return k;
}
// u = ((lowb << 8) >> 9) 2^-23 for the 24-bit value lowb of the particle
// draws, so floor(u kPickBins) = lowb >> 14 exactly (kPickBins = 2^10)
MKF_HD int pick_bin_of(uint32_t lowb) { return (int)(lowb >> 14); }

#ifdef __CUDACC__
// ---------------------------------------------------------------- packed FP32 pairs
// Blackwell f32x2 instructions: one issue for two lanes, each lane rounded as
// the scalar operation would be (so results equal the scalar code's).
union F2U { float2 f; unsigned long long u; };
__device__ __forceinline__ float2 pk_fma(float2 a, float2 b, float2 c) {
  F2U x, y, z, d;
  x.f = a; y.f = b; z.f = c;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d.u) : "l"(x.u), "l"(y.u), "l"(z.u));
  return d.f;
}
__device__ __forceinline__ float2 pk_add(float2 a, float2 b) {
  F2U x, y, d;
  x.f = a; y.f = b;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d.u) : "l"(x.u), "l"(y.u));
  return d.f;
}
__device__ __forceinline__ float2 pk_sub(float2 a, float2 b) {
  F2U x, y, d;
  x.f = a; y.f = b;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d.u) : "l"(x.u), "l"(y.u));
  return d.f;
}
__device__ __forceinline__ float2 pk_mul(float2 a, float2 b) {
  F2U x, y, d;
  x.f = a; y.f = b;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d.u) : "l"(x.u), "l"(y.u));
  return d.f;
}

// Box-Muller pair from two words (top 24 bits): u1 in (0,1], u2 in [0,1).
// MUFU intrinsics: the CPU oracle consumes these values dumped by
// mkf_draw_particles, so libm-vs-device rounding never enters parity.
__device__ __forceinline__ void box_muller(uint32_t w0, uint32_t w1, float& z0, float& z1) {
  float u1 = (float)((w0 >> 8) + 1u) * (1.0f / 16777216.0f);
  float u2 = (float)(w1 >> 8) * (1.0f / 16777216.0f);
  const float y = -2.0f * __logf(u1);                 // >= 0; y * rsqrt(y) is the MUFU square root
  float r = y * rsqrtf(fmaxf(y, 1e-30f));
  float s, c;
  __sincosf(3.14159265358979f * (2.0f * u2 - 1.0f), &s, &c);
  z0 = r * c;
  z1 = r * s;
}

__device__ __forceinline__ float lg2_approx(float x) {
  float r;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// A float in [1, 2) whose 23 mantissa bits are the word's top 23 bits (no
// integer-to-float conversion, which runs at a fraction of the FP32 rate).
__device__ __forceinline__ float unit_bits(uint32_t w) { return __uint_as_float(0x3F800000u | (w >> 9)); }

// Both Box-Muller pairs of one Philox block, (w.x, w.y) -> z[0], z[1] and
// (w.z, w.w) -> z[2], z[3], with the two pairs' arithmetic in packed f32x2
// instructions.  Uniforms of 23 bits: u1 = 2 - [1, 2) in (0, 1], u2 = [1, 2) - 1
// in [0, 1), both exact.  r = sqrt(-2 ln u1) with -2 ln u1 = lg2(u1) (-2 ln 2)
// and sqrt.approx, angle pi (2 u2 - 1) as fma(2 pi, u2, -pi) (the same single
// rounding), z = r (cos, sin).
__device__ __forceinline__ void box_muller2(u32x4 w, float* z) {
  const float2 u1 = pk_sub(make_float2(2.0f, 2.0f), make_float2(unit_bits(w.x), unit_bits(w.z)));
  const float2 u2 = pk_sub(make_float2(unit_bits(w.y), unit_bits(w.w)), make_float2(1.0f, 1.0f));
  const float2 y = pk_mul(make_float2(lg2_approx(u1.x), lg2_approx(u1.y)),
                          make_float2(-1.3862943611198906f, -1.3862943611198906f));
  float r0, r1;   // MUFU square roots (y >= 0; y = 0 gives 0)
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r0) : "f"(y.x));
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r1) : "f"(y.y));
  const float2 r = make_float2(r0, r1);
  const float2 ang = pk_fma(make_float2(6.283185307179586f, 6.283185307179586f), u2,
                            make_float2(-3.14159265358979f, -3.14159265358979f));
  float s0, c0, s1, c1;
  __sincosf(ang.x, &s0, &c0);
  __sincosf(ang.y, &s1, &c1);
  const float2 z01 = pk_mul(make_float2(r.x, r.x), make_float2(c0, s0));
  const float2 z23 = pk_mul(make_float2(r.y, r.y), make_float2(c1, s1));
  z[0] = z01.x; z[1] = z01.y; z[2] = z23.x; z[3] = z23.y;
}

// All draws of one particle-frame: D normals (D / 4 Philox blocks at streams
// 0, 1, ...) and the component uniform, 23 bits from the low bytes of words
// 0..2 of block 0 ((24-bit value) >> 1, times 2^-23).
template <int D>
__device__ __forceinline__ float particle_draws(uint64_t seed, uint32_t track, uint32_t frame,
                                                uint32_t item, float* eps) {
  static_assert(D % 4 == 0, "particle_draws: D must be a multiple of 4");
  uint32_t lowb = 0;
#pragma unroll
  for (int b = 0; b < D / 4; ++b) {
    u32x4 w = draw_block(seed, track, frame, item, (uint32_t)b);
    if (b == 0) lowb = (w.x & 0xFFu) | ((w.y & 0xFFu) << 8) | ((w.z & 0xFFu) << 16);
    box_muller2(w, eps + 4 * b);
  }
  return unit_bits(lowb << 8) - 1.0f;
}

// particle_draws with the item-independent Philox work done beforehand:
// pre[b] = philox_pre(seed, track, frame, b) for b < D / 4, ks =
// philox_keys(seed, track), both in shared memory.  Same values; ubin is the
// component uniform's bin of the pick table.
template <int D>
__device__ __forceinline__ float particle_draws_pre(const PhiloxPre* pre, const PhiloxKeys& ks, uint32_t item,
                                                    float* eps, int& ubin) {
  static_assert(D % 4 == 0, "particle_draws_pre: D must be a multiple of 4");
  // every block's Philox first (independent chains the scheduler can
  // interleave), then the Box-Muller pairs
  u32x4 w[D / 4];
#pragma unroll
  for (int b = 0; b < D / 4; ++b) philox_items_smem<1>(pre + b, &ks, item, &w[b]);
  const uint32_t lowb = (w[0].x & 0xFFu) | ((w[0].y & 0xFFu) << 8) | ((w[0].z & 0xFFu) << 16);
#pragma unroll
  for (int b = 0; b < D / 4; ++b) box_muller2(w[b], eps + 4 * b);
  ubin = pick_bin_of(lowb);
  return unit_bits(lowb << 8) - 1.0f;
}

// ---------------------------------------------------------------- block helpers
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ uint64_t warp_incl_scan_u64(uint64_t v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint64_t t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// Sums of N values (N = 16 or 32) over the warp with 2 N - 1 exchanges instead
// of 5 N: at each level a lane keeps half of its values and receives the other
// lane's copy of that half.  Afterwards lane i << (5 - log2 N) holds total i in
// v[0] (other entries are scratch).  The order of the additions is fixed.
template <int N>
__device__ __forceinline__ void warp_sum_split(float (&v)[N], int lane) {
  static_assert(N == 16 || N == 32, "warp_sum_split: N must be 16 or 32");
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const int o = 16 >> k, h = (N >> k) / 2;   // h values kept at this level (0: the last sums)
    if (h >= 1) {
      const bool upper = (lane & o) != 0;
#pragma unroll
      for (int i = 0; i < h; ++i) {
        const float send = upper ? v[i] : v[i + h];
        const float keep = upper ? v[i + h] : v[i];
        v[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
      }
    } else {
      v[0] += __shfl_xor_sync(0xffffffffu, v[0], o);
    }
  }
}

// An int whose signed order is the float order (any non-NaN float), so that
// atomicMax on it is a float max; float_unordered inverts it.
__device__ __forceinline__ int float_ordered(float f) {
  const int i = __float_as_int(f);
  return i ^ ((i >> 31) & 0x7FFFFFFF);
}
__device__ __forceinline__ float float_unordered(int i) { return __int_as_float(i ^ ((i >> 31) & 0x7FFFFFFF)); }

// exclusive block scan of one uint64 per thread; red holds >= 33 uint64
__device__ __forceinline__ uint64_t block_excl_scan_u64(uint64_t v, uint64_t* red, uint64_t* total) {
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  uint64_t inc = warp_incl_scan_u64(v, lane);
  __syncthreads();
  if (lane == 31) red[w] = inc;
  __syncthreads();
  if (w == 0) {
    uint64_t t = lane < nw ? red[lane] : 0;
    uint64_t ti = warp_incl_scan_u64(t, lane);
    if (lane < nw) red[lane] = ti - t;
    if (lane == 31) red[32] = ti;
  }
  __syncthreads();
  uint64_t r = red[w] + inc - v;
  if (total) *total = red[32];
  return r;
}

#endif  // __CUDACC__

// ---------------------------------------------------------------- exact resampler
// Weights -> 64-bit integers with 40 bits below the max (exact power-of-two
// scaling then truncation; e is the max weight's binary exponent, frexp
// convention); systematic resampling in exact integer arithmetic.
constexpr int kQBits = 40;

MKF_HD uint64_t quantize_f32(float w, int e) {
#ifdef __CUDA_ARCH__
  return (w > 0.0f) ? (uint64_t)__float2ull_rz(ldexpf(w, kQBits - e)) : 0ull;
#else
  return (w > 0.0f) ? (uint64_t)ldexpf(w, kQBits - e) : 0ull;   // the cast truncates
#endif
}
MKF_HD uint64_t quantize_f64(double w, int e) {
#ifdef __CUDA_ARCH__
  return (w > 0.0) ? (uint64_t)__double2ull_rz(ldexp(w, kQBits - e)) : 0ull;
#else
  return (w > 0.0) ? (uint64_t)ldexp(w, kQBits - e) : 0ull;
#endif
}

// target of particle i: (i 2^32 + U) * Qt  (128-bit)
MKF_HD unsigned __int128 resample_rhs(int i, uint32_t U, uint64_t Qt) {
  return (unsigned __int128)((((uint64_t)(uint32_t)i) << 32) | (uint64_t)U) * (unsigned __int128)Qt;
}
// first j in [0, n) with N Q[j] 2^32 >= rhs; Q nondecreasing; returns n-1 if none
MKF_HD int resample_search(const uint64_t* Q, int n, int N, unsigned __int128 rhs) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    unsigned __int128 lhs = ((unsigned __int128)(uint64_t)N * (unsigned __int128)Q[mid]) << 32;
    if (lhs < rhs) lo = mid + 1; else hi = mid;
  }
  return lo;
}
MKF_HD int resample_fallback_index(uint32_t U, int i, int L) {
  u32x4 o = philox4x32_10(u32x4{(uint32_t)i, 0u, 0u, 0u}, U, 0x5EEDu);
  return (int)(((uint64_t)o.x * (uint64_t)L) >> 32);
}
// number of targets i in [0, N) with (i 2^32 + U) Qt <= N X 2^32
MKF_HD int count_targets_le(uint64_t X, int N, uint32_t U, uint64_t Qt) {
  const unsigned __int128 lim = ((unsigned __int128)(uint64_t)N * (unsigned __int128)X) << 32;
  double est = (double)N * ((double)X / (double)Qt);
  long long i = (long long)est;
  if (i < 0) i = 0;
  if (i > N) i = N;
  for (int it = 0; it < 64 && i < N && resample_rhs((int)i, U, Qt) <= lim; ++it) ++i;
  for (int it = 0; it < 64 && i > 0 && resample_rhs((int)(i - 1), U, Qt) > lim; ++it) --i;
  bool ok = (i == N || resample_rhs((int)i, U, Qt) > lim) && (i == 0 || resample_rhs((int)(i - 1), U, Qt) <= lim);
  if (!ok) {
    long long lo = 0, hi = N;
    while (lo < hi) {
      long long mid = (lo + hi) >> 1;
      if (resample_rhs((int)mid, U, Qt) <= lim) lo = mid + 1; else hi = mid;
    }
    i = lo;
  }
  return (int)i;
}

// Scatter walk of exact systematic resampling for one thread's contiguous chunk
// [j0, j1) of integer weights q_j (get(j)), whose exclusive prefix is P: emits
// ancestors j for every target i whose rule "first j with N Q_j 2^32 >=
// (i 2^32 + U) Qt" lands in the chunk.
template <typename GetQ>
MKF_HD void scatter_walk(int j0, int j1, uint64_t P, int N, uint32_t U, uint64_t Qt, GetQ get, int* anc) {
  if (j0 >= j1) return;
  int i = (j0 == 0) ? 0 : count_targets_le(P, N, U, Qt);
  uint64_t Qj = P;
  for (int j = j0; j < j1; ++j) {
    Qj += get(j);
    const unsigned __int128 lim = ((unsigned __int128)(uint64_t)N * (unsigned __int128)Qj) << 32;
    while (i < N && resample_rhs(i, U, Qt) <= lim) anc[i++] = j;
  }
}

// The same rule with 64-bit thresholds (integer only, host and device): target
// i takes the first j whose inclusive prefix Q_j >= T_i = ceil((i 2^32 + U) Qt /
// (N 2^32)), the 128-bit comparison N Q_j 2^32 >= (i 2^32 + U) Qt restated
// exactly.  With Qt = A N + r and floor(U Qt / 2^32) = C N + s, and V_i = i r + s:
//   T_i = i A + C + floor(V_i / N) + [V_i mod N > 0 or (U Qt mod 2^32) > 0].
// Needs N <= 65536 (V_i < N^2 fits 32 bits) and i A + C < 2^64.
struct RsThresh {
  uint64_t A, C;
  uint32_t r, s, N, low;
  float invN;
};
MKF_HD RsThresh rs_thresh_setup(uint64_t Qt, int N, uint32_t U) {
  RsThresh t;
  t.N = (uint32_t)N;
  t.A = Qt / t.N;
  t.r = (uint32_t)(Qt - t.A * t.N);
  const unsigned __int128 UQ = (unsigned __int128)U * Qt;
  const uint64_t UQh = (uint64_t)(UQ >> 32);
  t.low = (uint32_t)UQ;
  t.C = UQh / t.N;
  t.s = (uint32_t)(UQh - t.C * t.N);
  t.invN = 1.0f / (float)N;
  return t;
}
MKF_HD uint64_t rs_threshold(const RsThresh& t, uint32_t i) {
  const uint32_t V = i * t.r + t.s;
  const uint32_t g = V / t.N, h = V - g * t.N;
  return (uint64_t)i * t.A + t.C + g + (((h | t.low) != 0u) ? 1u : 0u);
}
// rs_threshold along a stride of targets i, i + S, i + 2S, ... without a
// division per target: with S r = dq N + dr, V_{i+S} = V_i + S r, so
// floor(V / N) grows by dq plus the carry of (V_i mod N) + dr.  The walk keeps
// base = i A + C + floor(V_i / N) and h = V_i mod N (< N), so any target index
// (also past N - 1) stays in 32-bit arithmetic; needs S r < 2^32 and N <= 65536.
struct RsStep {
  uint64_t dA;
  uint32_t dq, dr;
};
struct RsWalk {
  uint64_t base;
  uint32_t h;
};
MKF_HD RsStep rs_step_setup(const RsThresh& t, uint32_t S) {
  RsStep st;
  const uint32_t v = S * t.r;
  st.dq = v / t.N;
  st.dr = v - st.dq * t.N;
  st.dA = (uint64_t)S * t.A;
  return st;
}
MKF_HD RsWalk rs_walk_init(const RsThresh& t, uint32_t i) {
  const uint32_t V = i * t.r + t.s;
  const uint32_t g = V / t.N;
  RsWalk w;
  w.h = V - g * t.N;
  w.base = (uint64_t)i * t.A + t.C + g;
  return w;
}
MKF_HD uint64_t rs_walk_threshold(const RsThresh& t, const RsWalk& w) {
  return w.base + (((w.h | t.low) != 0u) ? 1u : 0u);
}
MKF_HD void rs_walk_next(const RsThresh& t, const RsStep& st, RsWalk& w) {
  uint32_t h = w.h + st.dr;
  const uint32_t c = (h >= t.N) ? 1u : 0u;
  w.h = h - (c ? t.N : 0u);
  w.base += st.dA + st.dq + c;
}

// floor(V_i / N) and V_i mod N for any N <= 2^22 and i < 2^23 (V_i < 2^45):
// a float estimate (relative error <= 4 2^-24, so within one of the truth)
// and exact integer correction.
MKF_HD void rs_divmod64(const RsThresh& t, uint32_t i, uint32_t& g, uint32_t& hq) {
  const uint64_t V = (uint64_t)i * t.r + t.s;
  // float(V) from two 32-bit conversions (V < 2^45); the 64-bit one runs on the FP64 pipe
  const float vf = fmaf((float)(uint32_t)(V >> 20), 1048576.0f, (float)(uint32_t)(V & 0xFFFFFu));
#ifdef __CUDA_ARCH__
  g = __float2uint_rz(vf * t.invN);
#else
  g = (uint32_t)(vf * t.invN);   // truncation, as __float2uint_rz
#endif
  long long h = (long long)V - (long long)g * (long long)t.N;
  for (int k = 0; k < 2; ++k)
    if (h < 0) { --g; h += t.N; }
  for (int k = 0; k < 2; ++k)
    if (h >= (long long)t.N) { ++g; h -= t.N; }
  hq = (uint32_t)h;
}
// The threshold T_i for any N <= 2^22.
MKF_HD uint64_t rs_threshold64(const RsThresh& t, uint32_t i) {
  uint32_t g, h;
  rs_divmod64(t, i, g, h);
  return (uint64_t)i * t.A + t.C + g + (((h | t.low) != 0u) ? 1u : 0u);
}
// Start of a strided walk (rs_walk_next) for any N <= 2^22 and i < 2^23; the
// walk itself stays exact while S r < 2^32 (S <= 1024 for every such N).
MKF_HD RsWalk rs_walk_init64(const RsThresh& t, uint32_t i) {
  uint32_t g, h;
  rs_divmod64(t, i, g, h);
  RsWalk w;
  w.h = h;
  w.base = (uint64_t)i * t.A + t.C + g;
  return w;
}

// quantize_f32(w, 1) (the device's 64-bit conversion path) for a weight
// normalised to max 1 (w <= 1), without the 64-bit conversion (which runs on
// GB300's small FP64 pipe): floor(w 2^39) from the float's fields with integer
// shifts; 0 for zero, negative, NaN and subnormal w
MKF_HD uint64_t quantize39(float w) {
#ifdef __CUDA_ARCH__
  const uint32_t b = __float_as_uint(w);
#else
  uint32_t b;
  memcpy(&b, &w, sizeof(b));
  if (!(w > 0.0f)) b = 0;   // keeps the host's shifts in range (the device's shl clamps)
#endif
  const int e = (int)(b >> 23) - 111;
  const uint64_t m = (uint64_t)((b & 0x7FFFFFu) | 0x800000u);
  const uint64_t q = e >= 0 ? (m << e) : (e > -24 ? (m >> -e) : 0ull);
  return (w > 0.0f) ? q : 0ull;
}

// First j in [0, n) with Q[j] >= T (Q nondecreasing) for G targets at once: a
// branch-free lower bound whose halving steps depend on n only, so the G
// searches run interleaved.  Needs T[g] <= Q[n-1] (else the result is n).
template <int G>
MKF_HD void search_u64_multi(const uint64_t* Q, int n, const uint64_t* T, int* out) {
  int base[G];
  MKF_UNROLL
  for (int g = 0; g < G; ++g) base[g] = 0;
  int len = n;
  while (len > 1) {
    const int half = len >> 1;
    MKF_UNROLL
    for (int g = 0; g < G; ++g) base[g] = (Q[base[g] + half] < T[g]) ? base[g] + half : base[g];
    len -= half;
  }
  MKF_UNROLL
  for (int g = 0; g < G; ++g) out[g] = base[g] + ((Q[base[g]] < T[g]) ? 1 : 0);
}

// The same lower bound by power-of-two steps (Shar's form of binary search):
// with p the largest power of two <= n, one compare at n - p - 1 places the
// answer in a window of p entries starting at 0 or n - p, and log2(p) steps of
// h = p/2 .. 1 ("base += h if Q[base + h - 1] < T") finish it, with no final
// compare.  Every index read is < n.  Needs T[g] <= Q[n-1], else the result is
// some j < n (which callers discard).
template <int G>
MKF_HD void search_u64_pow2(const uint64_t* Q, int n, const uint64_t* T, int* out) {
#ifdef __CUDA_ARCH__
  const int p = 1 << (31 - __clz(n));
#else
  const int p = 1 << (31 - __builtin_clz((unsigned)n));
#endif
  int base[G];
  MKF_UNROLL
  for (int g = 0; g < G; ++g) base[g] = (p != n && Q[n - p - 1] < T[g]) ? n - p : 0;
  for (int h = p >> 1; h; h >>= 1) {
    MKF_UNROLL
    for (int g = 0; g < G; ++g) base[g] += (Q[base[g] + h - 1] < T[g]) ? h : 0;
  }
  MKF_UNROLL
  for (int g = 0; g < G; ++g) out[g] = base[g];
}

}  // namespace mkf
