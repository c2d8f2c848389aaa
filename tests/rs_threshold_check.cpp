// The resampler's 64-bit threshold forms (rs_thresh_setup with rs_threshold,
// N <= 65536, and rs_threshold64, N <= 2^22, from mkf_common.cuh compiled here
// for the host) against the exact rule T_i = ceil((i 2^32 + U) Qt / (N 2^32))
// in 128-bit integers.  Cases: random N, Qt in [1, 2^62) (at most 2^22 weights
// of 40 bits each), U and i; plus the extremes of each.  Prints "mismatches cases".
#include "mkf_common.cuh"

#include <cstdio>
#include <random>

static bool check(uint64_t Qt, int N, uint32_t U, uint32_t i) {
  const mkf::RsThresh th = mkf::rs_thresh_setup(Qt, N, U);
  const unsigned __int128 num = ((((unsigned __int128)i) << 32) + U) * (unsigned __int128)Qt;
  const unsigned __int128 den = ((unsigned __int128)(uint64_t)N) << 32;
  const unsigned __int128 ref = (num + den - 1) / den;
  bool ok = mkf::rs_threshold64(th, i) == (uint64_t)ref && ref >> 64 == 0;
  if (N <= 65536) ok = ok && mkf::rs_threshold(th, i) == (uint64_t)ref;
  return ok;
}

int main() {
  std::mt19937_64 rng(20140601);
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
  std::printf("%lld %lld\n", bad, n);
  return 0;
}
