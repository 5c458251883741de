/*
 * ORACLE build helper (test infrastructure only).
 *
 * Compiles scpp/gfft's own transform objects, from the reference's headers
 * where they lie, into a shared library with one C entry point, so that the
 * reference's outputs can be recorded as golden fixtures and used to pin the
 * CPU restatement (gfft_restate.cpp).  The reference resolves N at compile
 * time, so every (N, value type, transform, place) combination needed is
 * instantiated here; unsupported combinations (in-place composite N, real
 * transforms out of place or of non-power-of-two N: src/gfftalg.h:386-395,
 * src/gfftswap.h:282-286) are not instantiated and report -1.
 *
 * Objects are obtained the way the reference's own harnesses obtain them
 * (Transform<...>::Instance, test/gfft_accuracy.h:163), each ID-free.
 *
 * Build: oracle/build.py build_ref() (outputs only into oracle/_ref/).
 */
#include <complex>
#include <cstdint>
#include <cstring>
#include <map>
#include <tuple>

#include "gfft.h"

using namespace GFFT;

typedef void (*exec_fn)(const void*, void*);
typedef std::tuple<long, int, int, int> Key; /* n, vtype, trans, place */

static std::map<Key, exec_fn>& table() {
  static std::map<Key, exec_fn> t;
  return t;
}

constexpr long smallest_prime(long n, long p = 2) {
  return (p * p > n) ? n : (n % p == 0 ? p : smallest_prime(n, p + 1));
}
constexpr bool is_power_of(long n, long p) { return n == 1 ? true : (n % p == 0 && is_power_of(n / p, p)); }
constexpr bool prime_power(long n) { return n > 1 && is_power_of(n, smallest_prime(n)); }
constexpr bool power_of_two(long n) { return n > 1 && is_power_of(n, 2); }

template <class VT, class TT, class PL>
struct Runner;

template <class VT, class TT>
struct Runner<VT, TT, IN_PLACE> {
  template <long N>
  static void run(const void* s, void* d) {
    typedef typename VT::ValueType T;
    typedef typename Transform<ulong_<N>, VT, TT, ulong_<1>, Serial, IN_PLACE, 0>::Instance Obj;
    static Obj obj;
    if (s != d) std::memcpy(d, s, sizeof(T) * (Loki::TypeTraits<T>::isStdFundamental ? 2 : 1) * N);
    obj.fft(static_cast<T*>(d));
  }
};
template <class VT, class TT>
struct Runner<VT, TT, OUT_OF_PLACE> {
  template <long N>
  static void run(const void* s, void* d) {
    typedef typename VT::ValueType T;
    typedef typename Transform<ulong_<N>, VT, TT, ulong_<1>, Serial, OUT_OF_PLACE, 0>::Instance Obj;
    static Obj obj;
    obj.fft(static_cast<const T*>(s), static_cast<T*>(d));
  }
};

template <long N, class VT, class TT, class PL, bool OK>
struct Reg {
  static void apply() {}
};
template <long N, class VT, class TT, class PL>
struct Reg<N, VT, TT, PL, true> {
  static void apply() {
    table()[Key(N, (int)VT::ID, (int)TT::ID, (int)PL::ID)] = &Runner<VT, TT, PL>::template run<N>;
  }
};

/* Combinations the reference itself does not compile, left out:
 *  - FLOAT / COMPLEX_FLOAT at N = 12: Sub<> of two SDecimal with different
 *    digit counts is undefined (src/metacomplex.h:57);
 *  - COMPLEX_* in place at N = 2: GFFTswap2<2,1,std::complex<T>,0> is an
 *    ambiguous specialization (src/gfftswap.h:119-124, 218-224). */
template <class VT>
constexpr bool compiles(long n) {
  return !(VT::Accuracy == 1 && n == 12);
}
template <class VT>
constexpr bool compiles_inp(long n) {
  return compiles<VT>(n) && !(VT::ID >= 2 && n == 2);
}

template <class VT, long N>
struct RegAll {
  static const bool C = compiles<VT>(N);
  static const bool CI = compiles_inp<VT>(N);
  static void apply() {
    Reg<N, VT, DFT, OUT_OF_PLACE, C>::apply();
    Reg<N, VT, IDFT, OUT_OF_PLACE, C>::apply();
    Reg<N, VT, DFT, IN_PLACE, CI && prime_power(N)>::apply();
    Reg<N, VT, IDFT, IN_PLACE, CI && prime_power(N)>::apply();
    Reg<N, VT, RDFT, IN_PLACE, CI && power_of_two(N)>::apply();
    Reg<N, VT, IRDFT, IN_PLACE, CI && power_of_two(N)>::apply();
  }
};

template <class VT, long... Ns>
struct RegList;
template <class VT>
struct RegList<VT> {
  static void apply() {}
};
template <class VT, long N, long... Ns>
struct RegList<VT, N, Ns...> {
  static void apply() {
    RegAll<VT, N>::apply();
    RegList<VT, Ns...>::apply();
  }
};

#ifndef REF_VTYPE
#define REF_VTYPE DOUBLE
#endif

/* The size list: the reference's accuracy sweep (test_accuracy.sh:4-28:
 * 2^2..2^11, 3^2..3^7, 5^2..5^4, 7^2..7^3) widened by a few, mixed sizes for
 * the out-of-place path, and the benchmark sizes 1024, 4096, 2^19 (the real
 * transform of 2^20 reals), 3*2^18, 5^8 and 2^10*3^5. */
#define REF_SIZES                                                                                  \
  2, 4, 8, 16, 32, 64, 128, 256, 512, 1024, 2048, 4096, 3, 9, 27, 81, 243, 729, 2187, 5, 25, 125, 625, \
      3125, 7, 49, 343, 2401, 11, 13, 121, 6, 10, 12, 15, 18, 20, 24, 30, 36, 45, 48, 60, 72, 96, 100, \
      120, 144, 192, 210, 240, 360, 384, 480, 500, 768, 1000, 1536, 2000, 3000, 3072, 524288, 786432,   \
      390625, 248832


/* Root-of-unity constants of every recursion level, exactly as the
 * reference's objects use them: the top level takes GetFirstRoot<N,S,Acc>
 * (src/gfftpolicy.h:155, 196), each next level IPowBig<W1,K>
 * (src/gfftalg.h:408, 475), and a level reads its root through
 * Compute<W::Re/Im, Accuracy>::value() (src/gfftalg.h:237-238,
 * src/twiddles.h:294-295).  Recorded top-down, one (re, im) pair per level of
 * length >= 2 that has a combine pass. */
template <long N, class NFact, class VT, int S, class W1>
struct RootChain;

template <long N, long K, long P, class Tail, class VT, int S, class W1>
struct RootChain<N, Loki::Typelist<pair_<ulong_<K>, ulong_<P> >, Tail>, VT, S, W1> {
  static const long M = N / K;
  typedef typename IPowBig<W1, K>::Result WK;
  typedef Loki::Typelist<pair_<ulong_<K>, ulong_<P - 1> >, Tail> Next;
  static int apply(double* re, double* im) {
    re[0] = Compute<typename W1::Re, VT::Accuracy>::value();
    im[0] = Compute<typename W1::Im, VT::Accuracy>::value();
    return 1 + RootChain<M, Next, VT, S, WK>::apply(re + 1, im + 1);
  }
};
template <long N, long K, class Tail, class VT, int S, class W1>
struct RootChain<N, Loki::Typelist<pair_<ulong_<K>, ulong_<0> >, Tail>, VT, S, W1>
    : public RootChain<N, Tail, VT, S, W1> {};
template <long N, class VT, int S, class W1>
struct RootChain<N, Loki::Typelist<pair_<ulong_<N>, ulong_<1> >, Loki::NullType>, VT, S, W1> {
  static int apply(double*, double*) { return 0; }
};

typedef int (*roots_fn)(double*, double*);
static std::map<std::tuple<long, int>, roots_fn>& roots_table() {
  static std::map<std::tuple<long, int>, roots_fn> t;
  return t;
}
template <class VT, long N, int S>
static int roots_of(double* re, double* im) {
  typedef typename Factorize<ulong_<N> >::Result F;
  typedef typename GetFirstRoot<N, S, VT::Accuracy>::Result W1;
  return RootChain<N, F, VT, S, W1>::apply(re, im);
}
template <class VT, long N, bool C>
struct RootReg {
  static void apply() {}
};
template <class VT, long N>
struct RootReg<VT, N, true> {
  static void apply() {
    roots_table()[std::make_tuple(N, 1)] = &roots_of<VT, N, 1>;
    roots_table()[std::make_tuple(N, -1)] = &roots_of<VT, N, -1>;
  }
};
template <class VT, long... Ns>
struct RootList;
template <class VT>
struct RootList<VT> {
  static void apply() {}
};
template <class VT, long N, long... Ns>
struct RootList<VT, N, Ns...> {
  static void apply() {
    RootReg<VT, N, compiles<VT>(N)>::apply();
    RootList<VT, Ns...>::apply();
  }
};

namespace {
struct Init {
  Init() {
    RegList<REF_VTYPE, REF_SIZES>::apply();
#if REF_ROOTS
    RootList<REF_VTYPE, REF_SIZES>::apply();
#endif
  }
};
static Init init_;
}  // namespace

#define CAT2(a, b) a##b
#define CAT(a, b) CAT2(a, b)

#if REF_ROOTS
/* Level roots (top-down) of the object of length n and sign s; returns the
 * number of levels, or -1 if n was not compiled. */
extern "C" int CAT(ref_roots_, REF_VTYPE)(long n, int s, double* re, double* im) {
  auto it = roots_table().find(std::make_tuple(n, s));
  if (it == roots_table().end()) return -1;
  return it->second(re, im);
}
#endif

extern "C" int CAT(ref_exec_, REF_VTYPE)(long n, int trans, int place, const void* src, void* dst) {
  auto it = table().find(Key(n, (int)REF_VTYPE::ID, trans, place));
  if (it == table().end()) return -1;
  it->second(src, dst);
  return 0;
}
