/*
 * ORACLE timing driver (test and benchmark infrastructure only).
 *
 * Times scpp/gfft's own transform objects, compiled from the reference's
 * headers, on the host cores: the CPU arm of the benchmark.  One object of
 * GenerateTransform's serial policy per configuration, obtained the way the
 * reference's own harness obtains it (Transform<...>::Instance,
 * test/gfft_performance.h:95), shared by every OpenMP thread of a
 * `parallel for` over the batch: fft() is re-entrant on distinct data (its
 * temporaries live on the stack, src/gfftspec_inp.h:94).
 *
 * The reference's own OpenMP<NT> policy (src/gfftpolicy.h:403-453,
 * src/gfftomp.h) is not timed: it does not compile.  Its recursion stops at
 * partial specialisations of DFTk_inp_adapter that take `ulong_t K`
 * (src/gfftomp.h:287-293), while the serial recursion's stop at ones taking
 * `long_t K` (src/gfftalg.h:447-450, 494-496); a non-type template argument
 * deduces only against a parameter of its own type, so with either type for
 * the integral constant `ulong_` one of the two recursions never terminates.
 *
 * Usage: ref_bench N BATCH STEPS WARMUP   (N = 4096: FLOAT complex, out of place)
 * Prints one JSON line: seconds per step (min and mean), threads, a checksum.
 * Inputs: uniform [-1, 1) from splitmix64 (seed 0x5EED0003), as the
 * benchmark's synthetic data.
 */
#include <omp.h>

#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "gfft.h"

using namespace GFFT;

static uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

template <long N>
static int run(long batch, int steps, int warmup) {
  typedef typename Transform<ulong_<N>, FLOAT, DFT, ulong_<1>, Serial, OUT_OF_PLACE, 0>::Instance Obj;
  static Obj obj;
  const size_t m = (size_t)2 * N * (size_t)batch;
  std::vector<float> x(m), y(m);
  uint64_t s = 0x5EED0003ull;
  for (size_t i = 0; i < m; ++i) x[i] = (float)((double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0);
  auto step = [&]() {
#pragma omp parallel for schedule(static)
    for (long t = 0; t < batch; ++t) obj.fft(&x[(size_t)t * 2 * N], &y[(size_t)t * 2 * N]);
  };
  for (int i = 0; i < warmup; ++i) step();
  double best = 1e30, total = 0;
  for (int i = 0; i < steps; ++i) {
    auto t0 = std::chrono::steady_clock::now();
    step();
    const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    total += dt;
    if (dt < best) best = dt;
  }
  double cs = 0;
  for (size_t i = 0; i < m; i += 997) cs += std::fabs((double)y[i]);
  std::printf(
      "{\"n\": %ld, \"batch\": %ld, \"steps\": %d, \"warmup\": %d, \"s_min\": %.9g, \"s_mean\": %.9g, "
      "\"threads\": %d, \"checksum\": %.9g, \"objects\": \"Transform<ulong_<%ld>, FLOAT, DFT, ulong_<1>, Serial, "
      "OUT_OF_PLACE>::Instance\"}\n",
      (long)N, batch, steps, warmup, best, total / (steps > 0 ? steps : 1), omp_get_max_threads(), cs, (long)N);
  return 0;
}

int main(int argc, char** argv) {
  if (argc < 5) {
    std::fprintf(stderr, "usage: %s N BATCH STEPS WARMUP\n", argv[0]);
    return 2;
  }
  const long n = std::atol(argv[1]), batch = std::atol(argv[2]);
  const int steps = std::atoi(argv[3]), warmup = std::atoi(argv[4]);
  if (batch < 1 || steps < 0 || warmup < 0) return 2;
  switch (n) {
    case 4096: return run<4096>(batch, steps, warmup);
    case 1024: return run<1024>(batch, steps, warmup);
    default: std::fprintf(stderr, "length %ld not compiled\n", n); return 2;
  }
}
