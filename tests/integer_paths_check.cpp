// The integer paths of the particle kernels, from mkf_common.cuh compiled here
// for the host, against independent restatements:
//  - thresholds: rs_thresh_setup with rs_threshold (N <= 65536) and
//    rs_threshold64 (N <= 2^22) against T_i = ceil((i 2^32 + U) Qt / (N 2^32))
//    in 128-bit integers; random N, Qt in [1, 2^62) (at most 2^22 weights of
//    40 bits each), U and i, plus the extremes of each;
//  - stride: the division-free walk of those thresholds along a stride of
//    targets (rs_walk_*, started by rs_walk_init for N <= 65536 and by
//    rs_walk_init64 for N <= 2^22) against the same 128-bit T_i, past N - 1
//    included;
//  - quantize: quantize39(w) against floor(w 2^39) in double (exact: a float
//    times a power of two) for weights w <= 1 (its domain): random, boundary,
//    subnormal, zero, negative, -inf and NaN; quantize_f32 / quantize_f64 (the
//    general-exponent forms) against floor(w 2^(40-e)) in long double for
//    weights up to their max 2^e;
//  - search: search_u64_multi<4> and search_u64_pow2<4> against std::lower_bound on random
//    nondecreasing prefix arrays (with runs of equal values) of 1 .. 2^22 entries;
//  - pick: the particle kernels' component pick through the 1024-bin table
//    (build_pick_table / pick_component_table) against the direct count, for
//    K in [1, 32], cumulative weights with zero-weight components, sums short of
//    or past 1, cumulative values on bin edges, and every uniform u = m 2^-24 of
//    a sample.  (The weights cover the picks that the random-mixture workloads
//    and the shipped models make.)  pickbin: the table bin that the particle
//    draws take from their 24-bit value (pick_bin_of) against floor(u 1024) of
//    the uniform passed beside it, for every 24-bit value, and the table pick
//    with that bin against the count;
//  - philox: philox4x32_10 (every draw of the kernels) against the Random123
//    known-answer vectors; philox_split: the particle kernels' per-item form
//    (philox_pre + philox_keys + philox_item) against the direct form;
//  - walk: the scatter walk over per-thread chunks (scatter_walk with
//    count_targets_le, the RBPF, PDAF, pf2D and scatter-variant resampler) and
//    the 128-bit binary search (resample_search) against a direct two-pointer
//    evaluation of the rule "first j with N Q_j 2^32 >= (i 2^32 + U) Qt", on
//    random integer weights (with zeros and a dominant weight) and chunkings.
// Prints one "name mismatches cases" line per piece.
#include "mkf_common.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <random>
#include <vector>

static bool check(uint64_t Qt, int N, uint32_t U, uint32_t i) {
  const mkf::RsThresh th = mkf::rs_thresh_setup(Qt, N, U);
  const unsigned __int128 num = ((((unsigned __int128)i) << 32) + U) * (unsigned __int128)Qt;
  const unsigned __int128 den = ((unsigned __int128)(uint64_t)N) << 32;
  const unsigned __int128 ref = (num + den - 1) / den;
  bool ok = mkf::rs_threshold64(th, i) == (uint64_t)ref && ref >> 64 == 0;
  if (N <= 65536) ok = ok && mkf::rs_threshold(th, i) == (uint64_t)ref;
  return ok;
}

static void thresholds(std::mt19937_64& rng) {
  long long bad = 0, n = 0;
  for (int it = 0; it < 400000; ++it) {
    const int N = 1 + (int)(rng() % (it & 1 ? 65536 : 4194304));
    const uint64_t Qt = 1 + (rng() >> (2 + rng() % 60));
    const uint32_t U = (uint32_t)rng();
    const uint32_t i = (uint32_t)(rng() % N);
    bad += !check(Qt, N, U, i);
    ++n;
  }
  const int Ns[] = {1, 2, 3, 255, 256, 4097, 65535, 65536, 65537, 1048575, 4194303, 4194304};
  const uint64_t Qs[] = {1, 2, 3, (1ull << 40) - 1, 1ull << 40, (1ull << 62) - 1};
  const uint32_t Us[] = {0u, 1u, 0x80000000u, 0xFFFFFFFFu};
  for (int N : Ns)
    for (uint64_t Qt : Qs)
      for (uint32_t U : Us)
        for (uint32_t i : {0u, 1u, (uint32_t)N / 2, (uint32_t)N - 1}) {
          if (i >= (uint32_t)N) continue;
          bad += !check(Qt, N, U, i);
          ++n;
        }
  std::printf("thresholds %lld %lld\n", bad, n);
}

// the strided walk (rs_walk_*) against T_i at every target of the stride,
// including targets past N - 1 (they are formed, then left unused, by the kernels)
static void stride_walk(std::mt19937_64& rng) {
  long long bad = 0, n = 0;
  for (int it = 0; it < 3000; ++it) {
    const int N = 1 + (int)(rng() % (it % 3 == 0 ? 65536 : 8192));
    const uint64_t Qt = 1 + (rng() >> (2 + rng() % 60));
    const uint32_t U = (uint32_t)rng();
    const uint32_t S = 32u * (1u + (uint32_t)(rng() % 64));       // 32 .. 2048
    const uint32_t i0 = (uint32_t)(rng() % S);
    const mkf::RsThresh th = mkf::rs_thresh_setup(Qt, N, U);
    const mkf::RsStep st = mkf::rs_step_setup(th, S);
    mkf::RsWalk w = mkf::rs_walk_init(th, i0);
    for (uint32_t i = i0; i < (uint32_t)N + 4 * S; i += S) {
      const unsigned __int128 num = ((((unsigned __int128)i) << 32) + U) * (unsigned __int128)Qt;
      const unsigned __int128 den = ((unsigned __int128)(uint64_t)N) << 32;
      const unsigned __int128 ref = (num + den - 1) / den;
      bad += mkf::rs_walk_threshold(th, w) != (uint64_t)ref;
      ++n;
      mkf::rs_walk_next(th, st, w);
    }
  }
  // the 64-bit start (rs_walk_init64) for N up to 2^22, with S r < 2^32
  for (int it = 0; it < 3000; ++it) {
    const int N = 1 + (int)(rng() % (it % 2 == 0 ? (1 << 22) : 70000));
    const uint64_t Qt = 1 + (rng() >> (2 + rng() % 60));
    const uint32_t U = (uint32_t)rng();
    const uint32_t S = 32u * (1u + (uint32_t)(rng() % 32));       // 32 .. 1024
    const uint32_t i0 = (uint32_t)(rng() % (uint64_t)(N + S));
    const mkf::RsThresh th = mkf::rs_thresh_setup(Qt, N, U);
    const mkf::RsStep st = mkf::rs_step_setup(th, S);
    mkf::RsWalk w = mkf::rs_walk_init64(th, i0);
    int steps = 0;
    for (uint32_t i = i0; i < (uint32_t)N + 4 * S && steps < 64; i += S, ++steps) {
      const unsigned __int128 num = ((((unsigned __int128)i) << 32) + U) * (unsigned __int128)Qt;
      const unsigned __int128 den = ((unsigned __int128)(uint64_t)N) << 32;
      const unsigned __int128 ref = (num + den - 1) / den;
      bad += mkf::rs_walk_threshold(th, w) != (uint64_t)ref;
      bad += i < (uint32_t)N && mkf::rs_threshold64(th, i) != (uint64_t)ref;
      n += 2;
      mkf::rs_walk_next(th, st, w);
    }
  }
  std::printf("stride %lld %lld\n", bad, n);
}

static uint64_t quantize_ref(float w) {
  if (!(w > 0.0f) || !std::isfinite(w) || w < std::numeric_limits<float>::min()) return 0;
  return (uint64_t)std::floor(std::ldexp((double)w, 39));
}

static void quantize(std::mt19937_64& rng) {
  long long bad = 0, n = 0;
  std::uniform_real_distribution<float> u01(0.0f, 1.0f);
  std::vector<float> ws = {0.0f, -0.0f, 1.0f, -1.0f, 0.5f, std::nextafter(1.0f, 0.0f),
                           std::ldexp(1.0f, -39), std::ldexp(1.0f, -40), std::ldexp(1.5f, -39),
                           std::ldexp(1.0f, -63), std::ldexp(1.0f, -126), std::ldexp(1.0f, -130),
                           -std::numeric_limits<float>::infinity(), std::numeric_limits<float>::quiet_NaN()};
  for (int k = 0; k < 1000000; ++k) {
    const float w = u01(rng);
    ws.push_back(k & 1 ? w : std::ldexp(w, -(int)(rng() % 64)));
  }
  for (float w : ws) {
    bad += mkf::quantize39(w) != quantize_ref(w);
    bad += (w <= 1.0f && w > 0.0f) && mkf::quantize_f32(w, 1) != quantize_ref(w);   // the same value
    ++n;
  }
  // general exponents: w in (0, 2^e), e = max weight's frexp exponent
  for (int k = 0; k < 200000; ++k) {
    const int e = (int)(rng() % 200) - 100;
    const double wd = std::ldexp(std::uniform_real_distribution<double>(0.0, 1.0)(rng), e);
    const float wf = (float)wd;
    const long double rf = std::floor(std::ldexp((long double)wf, 40 - e));
    const long double rd = std::floor(std::ldexp((long double)wd, 40 - e));
    bad += wf > 0.0f && wf < std::ldexp(1.0f, e) && mkf::quantize_f32(wf, e) != (uint64_t)rf;
    bad += wd > 0.0 && mkf::quantize_f64(wd, e) != (uint64_t)rd;
    n += 2;
  }
  bad += mkf::quantize_f64(0.0, 1) != 0 || mkf::quantize_f64(-1.0, 1) != 0 || mkf::quantize_f32(-0.5f, 0) != 0;
  n += 3;
  std::printf("quantize %lld %lld\n", bad, n);
}

static void search(std::mt19937_64& rng) {
  long long bad = 0, n = 0;
  for (int it = 0; it < 400; ++it) {
    const int len = 1 + (int)(rng() % (it < 100 ? 64 : it < 390 ? 65536 : 4194304));
    std::vector<uint64_t> Q(len);
    uint64_t acc = 0;
    for (int j = 0; j < len; ++j) {
      acc += (rng() % 4 == 0) ? 0 : (rng() >> 30);     // runs of equal prefix values
      Q[j] = acc;
    }
    for (int k = 0; k < 256; ++k) {
      uint64_t T[4];
      int out[4];
      for (int g = 0; g < 4; ++g) {
        const int pick = (int)(rng() % len);
        T[g] = (rng() & 1) ? Q[pick] : (Q[pick] == 0 ? 0 : Q[pick] - rng() % (Q[pick] + 1) / 2);
        if (T[g] > Q[len - 1]) T[g] = Q[len - 1];
      }
      mkf::search_u64_multi<4>(Q.data(), len, T, out);
      int out2[4];
      mkf::search_u64_pow2<4>(Q.data(), len, T, out2);
      for (int g = 0; g < 4; ++g) {
        const int ref = (int)(std::lower_bound(Q.begin(), Q.end(), T[g]) - Q.begin());
        bad += out[g] != ref;
        bad += out2[g] != ref;
        n += 2;
      }
    }
  }
  std::printf("search %lld %lld\n", bad, n);
}

static void pick(std::mt19937_64& rng) {
  long long bad = 0, n = 0;
  std::uniform_real_distribution<float> u01(0.0f, 1.0f);
  std::vector<uint8_t> tab(mkf::kPickBins);
  for (int it = 0; it < 3000; ++it) {
    const int K = 1 + (int)(rng() % 32);
    std::vector<float> pi(K), cum(K);
    float tot = 0.0f;
    for (int k = 0; k < K; ++k) {
      pi[k] = (rng() % 5 == 0) ? 0.0f : u01(rng);
      tot += pi[k];
    }
    const float scale = (it % 3 == 0) ? 1.0f : (it % 3 == 1 ? 0.999f : 1.001f);
    float acc = 0.0f;
    for (int k = 0; k < K; ++k) {
      acc += tot > 0.0f ? pi[k] / tot * scale : 1.0f / K;
      cum[k] = acc;
    }
    if (it % 7 == 0)   // cumulative values exactly on bin edges
      for (int k = 0; k + 1 < K; ++k) cum[k] = std::floor(cum[k] * mkf::kPickBins) / mkf::kPickBins;
    for (int k = 1; k < K; ++k) cum[k] = std::max(cum[k], cum[k - 1]);
    for (int b = 0; b < mkf::kPickBins; ++b) tab[b] = 0xFF;
    mkf::build_pick_table(cum.data(), K, tab.data(), 0, 1);
    for (int q = 0; q < 2000; ++q) {
      uint32_t m = (uint32_t)(rng() >> 40);                          // 24 bits
      if (q < 64 && K > 1) {                                         // u on a cumulative value or a bin edge
        const float c = (q & 1) ? cum[rng() % (K - 1)] : (float)(rng() % mkf::kPickBins) / mkf::kPickBins;
        m = (uint32_t)std::min(std::max(0.0, std::ldexp((double)c, 24)), 16777215.0);
      }
      const float u = (float)m * (1.0f / 16777216.0f);
      bad += mkf::pick_component_table(tab.data(), cum.data(), K, u) != mkf::pick_component(cum.data(), K, u);
      ++n;
    }
  }
  std::printf("pick %lld %lld\n", bad, n);
}

// the pick table's bin from the particle draws' 24-bit value lowb, without a
// float conversion (pick_bin_of), against floor(u kPickBins) of the uniform
// u = ((lowb << 8) >> 9) 2^-23 that the kernels pass beside it, for every lowb;
// and the table pick with that bin against the count
static void pickbin(std::mt19937_64& rng) {
  long long bad = 0, n = 0;
  for (uint32_t lowb = 0; lowb < (1u << 24); ++lowb) {
    uint32_t bits = 0x3F800000u | ((lowb << 8) >> 9);
    float f;
    std::memcpy(&f, &bits, 4);
    const float u = f - 1.0f;
    bad += mkf::pick_bin_of(lowb) != (int)(u * (float)mkf::kPickBins);
    ++n;
  }
  std::uniform_real_distribution<float> u01(0.0f, 1.0f);
  std::vector<uint8_t> tab(mkf::kPickBins);
  for (int it = 0; it < 200; ++it) {
    const int K = 1 + (int)(rng() % 32);
    std::vector<float> cum(K);
    float tot = 0.0f;
    for (int k = 0; k < K; ++k) { tot += (rng() % 5 == 0) ? 0.0f : u01(rng); cum[k] = tot; }
    for (int k = 0; k < K; ++k) cum[k] /= tot > 0.0f ? tot : 1.0f;
    mkf::build_pick_table(cum.data(), K, tab.data(), 0, 1);
    for (int q = 0; q < 20000; ++q) {
      const uint32_t lowb = (uint32_t)(rng() & 0xFFFFFFu);
      uint32_t bits = 0x3F800000u | ((lowb << 8) >> 9);
      float f;
      std::memcpy(&f, &bits, 4);
      const float u = f - 1.0f;
      bad += mkf::pick_component_table_bin(tab.data(), cum.data(), K, u, mkf::pick_bin_of(lowb)) !=
             mkf::pick_component(cum.data(), K, u);
      ++n;
    }
  }
  std::printf("pickbin %lld %lld\n", bad, n);
}

static void philox() {
  struct Kat { mkf::u32x4 ctr; uint32_t k0, k1; mkf::u32x4 out; };
  const Kat kats[] = {
      {{0u, 0u, 0u, 0u}, 0u, 0u, {0x6627e8d5u, 0xe169c58du, 0xbc57ac4cu, 0x9b00dbd8u}},
      {{0xffffffffu, 0xffffffffu, 0xffffffffu, 0xffffffffu}, 0xffffffffu, 0xffffffffu,
       {0x408f276du, 0x41c83b0eu, 0xa20bc7c6u, 0x6d5451fdu}},
      {{0x243f6a88u, 0x85a308d3u, 0x13198a2eu, 0x03707344u}, 0xa4093822u, 0x299f31d0u,
       {0xd16cfe09u, 0x94fdccebu, 0x5001e420u, 0x24126ea1u}}};
  long long bad = 0, n = 0;
  for (const Kat& k : kats) {
    const mkf::u32x4 o = mkf::philox4x32_10(k.ctr, k.k0, k.k1);
    bad += o.x != k.out.x || o.y != k.out.y || o.z != k.out.z || o.w != k.out.w;
    ++n;
  }
  std::printf("philox %lld %lld\n", bad, n);
}

// the per-item split (philox_pre / philox_keys / philox_item, used by the
// particle kernels) against the direct philox4x32_10 of draw_block
static void philox_split(std::mt19937_64& rng) {
  long long bad = 0, n = 0;
  for (int it = 0; it < 20000; ++it) {
    const uint64_t seed = it < 4 ? (it & 1 ? ~0ull : 0ull) : rng();
    const uint32_t track = it < 4 ? (it & 2 ? ~0u : 0u) : (uint32_t)rng();
    const uint32_t frame = it % 7 == 0 ? mkf::kFramePrior : (uint32_t)(rng() % 4096);
    const uint32_t stream = (uint32_t)(rng() % 8);
    const mkf::PhiloxPre pre = mkf::philox_pre(seed, track, frame, stream);
    const mkf::PhiloxKeys ks = mkf::philox_keys(seed, track);
    for (int q = 0; q < 50; ++q) {
      const uint32_t item = q < 2 ? (q ? ~0u : 0u) : (uint32_t)rng();
      const mkf::u32x4 a = mkf::philox_item(pre, ks, item);
      const mkf::u32x4 b = mkf::draw_block(seed, track, frame, item, stream);
      bad += a.x != b.x || a.y != b.y || a.z != b.z || a.w != b.w;
      ++n;
    }
  }
  std::printf("philox_split %lld %lld\n", bad, n);
}

static void walk(std::mt19937_64& rng) {
  long long bad = 0, n = 0;
  for (int it = 0; it < 600; ++it) {
    const int L = 1 + (int)(rng() % 3000), N = 1 + (int)(rng() % 3000);
    std::vector<uint64_t> q(L), Q(L);
    uint64_t acc = 0;
    for (int j = 0; j < L; ++j) {
      const int kind = (int)(rng() % 8);
      q[j] = kind == 0 ? 0 : kind == 1 ? (1ull << 40) : (rng() >> (24 + rng() % 30));
      acc += q[j];
      Q[j] = acc;
    }
    if (acc == 0) { q[L - 1] = 1; Q[L - 1] = acc = 1; }
    const uint64_t Qt = acc;
    const uint32_t U = (uint32_t)rng();
    // direct evaluation of the rule, one pointer per side
    std::vector<int> ref(N);
    int j = 0;
    for (int i = 0; i < N; ++i) {
      const unsigned __int128 rhs = mkf::resample_rhs(i, U, Qt);
      while ((((unsigned __int128)(uint64_t)N * (unsigned __int128)Q[j]) << 32) < rhs) ++j;
      ref[i] = j;
    }
    // the scatter walk over chunks of E weights, as the kernels' threads run it
    const int E = 1 + (int)(rng() % 64);
    std::vector<int> anc(N, -1);
    for (int j0 = 0; j0 < L; j0 += E) {
      const int j1 = std::min(L, j0 + E);
      const uint64_t P = j0 ? Q[j0 - 1] : 0;
      mkf::scatter_walk(j0, j1, P, N, U, Qt, [&](int k) { return q[k]; }, anc.data());
    }
    for (int i = 0; i < N; ++i) {
      bad += anc[i] != ref[i];
      bad += mkf::resample_search(Q.data(), L, N, mkf::resample_rhs(i, U, Qt)) != ref[i];
      n += 2;
    }
  }
  std::printf("walk %lld %lld\n", bad, n);
}

int main() {
  std::mt19937_64 rng(20140601);
  philox();
  philox_split(rng);
  walk(rng);
  thresholds(rng);
  stride_walk(rng);
  quantize(rng);
  search(rng);
  pick(rng);
  pickbin(rng);
  return 0;
}
