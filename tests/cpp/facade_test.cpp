// Drop-in test of include/gfft.h: user code written the way the reference's
// sample program is (src/gfft.cpp:40-97), against the GB300 library.
//   facade_test          factory errors only (no GPU needed)
//   facade_test gpu      transforms on host arrays vs a long-double direct DFT
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "gfft.h"

using namespace GFFT;

static int fail(const char* m) {
  std::printf("FAIL: %s\n", m);
  return 1;
}

int main(int argc, char** argv) {
  const bool gpu = argc > 1 && std::strcmp(argv[1], "gpu") == 0;
  typedef TYPELIST_2(ulong_<16>, ulong_<1024>) NList;
  typedef GenerateTransform<NList, DOUBLE, TYPELIST_2(DFT, IDFT), ulong_<1>, Serial, OUT_OF_PLACE> TransformSet;
  TransformSet gfft;
  // unknown combinations throw the reference's exception
  const unsigned long bad[][5] = {{32, DOUBLE::ID, DFT::ID, Serial::ID, OUT_OF_PLACE::ID},
                                  {16, FLOAT::ID, DFT::ID, Serial::ID, OUT_OF_PLACE::ID},
                                  {16, DOUBLE::ID, RDFT::ID, Serial::ID, OUT_OF_PLACE::ID},
                                  {16, DOUBLE::ID, DFT::ID, OpenMP<4>::ID, OUT_OF_PLACE::ID},
                                  {16, DOUBLE::ID, DFT::ID, Serial::ID, IN_PLACE::ID}};
  for (auto& b : bad) {
    bool thrown = false;
    try {
      delete gfft.CreateTransformObject(b[0], b[1], b[2], 1, b[3], b[4]);
    } catch (TransformFactoryError<unsigned long, TransformSet::ObjectType>::Exception& e) {
      thrown = std::strcmp(e.what(),
                           "Requested transform is not compiled! Check your instantiation of GenerateTransform "
                           "class!") == 0;
    }
    if (!thrown) return fail("expected TransformFactoryError");
  }
  if (DOUBLE::ID != 0 || COMPLEX_FLOAT::ID != 3 || IRDFT::ID != 3 || OpenMP<8>::ID != 7 || IN_PLACE::ID != 0)
    return fail("tag ids");
  // the cosine-transform tags keep the reference's IDs (src/gfftpolicy.h:302-365)
  if (DCT1::ID != 4 || IDCT1::ID != 5 || DCT2::ID != 6 || IDCT2::ID != 7 || DCT2::Inverse::ID != 7)
    return fail("cosine tag ids");
  typedef GenerateTransform<TYPELIST_1(ulong_<100>), DOUBLE, TYPELIST_2(DCT2, IDCT2), ulong_<1>, Serial, OUT_OF_PLACE>
      CosineSet;
  CosineSet cosines;
  if (!gpu) {
    std::printf("facade ok (cpu)\n");
    return 0;
  }
  const long N = 1024;
  std::vector<double> x(2 * N), y(2 * N), z(2 * N);
  for (long i = 0; i < N; ++i) {  // GenInput::seq (src/direct.h:52-56)
    x[2 * i] = 2.0 * i;
    x[2 * i + 1] = 2.0 * i + 1;
  }
  TransformSet::ObjectType* f = gfft.CreateTransformObject(N, DOUBLE::ID, DFT::ID, 1, Serial::ID, OUT_OF_PLACE::ID);
  TransformSet::ObjectType* fi = gfft.CreateTransformObject(N, DOUBLE::ID, IDFT::ID, 1, Serial::ID, OUT_OF_PLACE::ID);
  f->fft(x.data(), y.data());
  fi->fft(y.data(), z.data());
  double err = 0, mag = 0, rt = 0;
  for (long k = 0; k < N; ++k) {
    long double sr = 0, si = 0;
    for (long n = 0; n < N; ++n) {
      long double a = -2.0L * 3.14159265358979323846264338327950288L * (long double)((k * n) % N) / N;
      sr += x[2 * n] * cosl(a) - x[2 * n + 1] * sinl(a);
      si += x[2 * n] * sinl(a) + x[2 * n + 1] * cosl(a);
    }
    err = std::fmax(err, std::fabs((double)(sr - y[2 * k])) + std::fabs((double)(si - y[2 * k + 1])));
    mag = std::fmax(mag, std::fabs((double)sr) + std::fabs((double)si));
  }
  for (long i = 0; i < 2 * N; ++i) rt = std::fmax(rt, std::fabs(z[i] - x[i]));
  delete f;
  delete fi;
  // in place via Transform<...>::Instance and the added ifft()
  Transform<ulong_<N>, DOUBLE, DFT, ulong_<1>, Serial, IN_PLACE>::Instance inp(N, DOUBLE::ID, DFT::ID, Serial::ID);
  std::vector<double> w = x;
  inp.fft(w.data());
  double d = 0;
  for (long i = 0; i < 2 * N; ++i) d = std::fmax(d, std::fabs(w[i] - y[i]));
  inp.ifft(w.data());
  double rt2 = 0;
  for (long i = 0; i < 2 * N; ++i) rt2 = std::fmax(rt2, std::fabs(w[i] - x[i]));
  std::printf("max|dft err|/max|X| = %.3g, roundtrip %.3g, inplace-vs-oop %.3g, inplace roundtrip %.3g\n",
              err / mag, rt, d, rt2);
  if (err / mag > 1e-14 || rt > 1e-10 || d != 0 || rt2 > 1e-10) return fail("accuracy");
  // DCT2 of 100 reals (the reference's direct.h sum) through the factory
  {
    const long M = 100;
    std::vector<double> a(M), b(M);
    for (long i = 0; i < M; ++i) a[i] = std::sin(0.37 * i) + 0.25 * i / M;
    CosineSet::ObjectType* dct = cosines.CreateTransformObject(M, DOUBLE::ID, DCT2::ID, 1, Serial::ID,
                                                                OUT_OF_PLACE::ID);
    dct->fft(a.data(), b.data());
    delete dct;
    double e2 = 0, m2 = 0;
    for (long k = 0; k < M; ++k) {
      long double s2 = 0;
      for (long l = 0; l < M; ++l)
        s2 += a[l] * cosl(3.14159265358979323846264338327950288L * (long double)((k * l) % (2 * M)) / M);
      e2 = std::fmax(e2, std::fabs((double)(s2 - b[k])));
      m2 = std::fmax(m2, std::fabs((double)s2));
    }
    std::printf("dct2 max err / max = %.3g\n", e2 / m2);
    if (e2 / m2 > 1e-13) return fail("dct2 accuracy");
  }
  std::printf("facade ok (gpu)\n");
  return 0;
}
