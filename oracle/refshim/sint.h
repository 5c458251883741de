/*
 * Stand-in for the missing `metafactor/sint.h` of scpp/gfft (the `metafactor`
 * git submodule, https://github.com/scpp/metafactor, is an empty directory in
 * the reference tree and its commit is unrecoverable).
 *
 * Written from scratch from how the reference USES these names:
 *   - long_t / ulong_t / short_t          (src/sbigint.h:34, src/gfftomp.h:552)
 *   - long_<N>::value, ulong_<N>::value   (src/gfftgen.h:76, src/gfftfactor.h:147)
 *   - pair_<A,B>::first / ::second        (src/gfftalg.h:415, src/gfftfactor.h:147)
 *   - SIntID<N>                           (src/gfftgen.h:178 documentation)
 *
 * This is test infrastructure: it only lets the reference's own headers
 * compile so that the oracle can be pinned against the reference's outputs.
 */
#ifndef GFFT_REFSHIM_SINT_H
#define GFFT_REFSHIM_SINT_H

typedef long long_t;
typedef unsigned long ulong_t;
typedef int int_t;
typedef short short_t;

template <long_t N>
struct long_ {
  typedef long_t value_type;
  static const long_t value = N;
  static const long_t ID = N - 1;
};

// The reference matches `ulong_<K>` against `long_t K` in partial
// specializations (src/gfftalg.h:447-450, 494-496): the parameter is long_t.
template <long_t N>
struct ulong_ {
  typedef ulong_t value_type;
  static const ulong_t value = N;
  static const ulong_t ID = N - 1;
};

template <class A, class B>
struct pair_ {
  typedef A first;
  typedef B second;
};

template <long_t N>
struct SIntID : public ulong_<N> {};

#endif
