/*
 * Stand-in for the missing `metafactor/metafactor.h` of scpp/gfft (submodule
 * https://github.com/scpp/metafactor, absent from the reference tree).
 *
 * Provides exactly what the reference's call sites need:
 *   - Factorization<ulong_<N>>::Result : Loki typelist of
 *       pair_<ulong_<p>, ulong_<k>>, primes ascending, found by trial division
 *       (src/gfftfactor.h:160-169, src/gfftpolicy.h:388-389, 426-431)
 *   - GCD<long_<a>, long_<b>>::Result::value (src/gfftpolicy.h:426)
 *
 * The published algorithm is plain trial division in ascending order, which is
 * what the reference's own commented-out copy does (src/gfftfactor.h:55-136):
 * the factor ORDER, not the method, is what fixes the butterfly sequence.
 * Test infrastructure only.
 */
#ifndef GFFT_REFSHIM_METAFACTOR_H
#define GFFT_REFSHIM_METAFACTOR_H

#include "sint.h"
#include "Typelist.h"

namespace refshim {

// multiplicity of prime p in n
template <ulong_t N, ulong_t P, bool Div = (N % P == 0)>
struct Mult {
  static const ulong_t value = 0;
  static const ulong_t rest = N;
};
template <ulong_t N, ulong_t P>
struct Mult<N, P, true> {
  static const ulong_t value = Mult<N / P, P>::value + 1;
  static const ulong_t rest = Mult<N / P, P>::rest;
};

// trial division starting at candidate P
template <ulong_t N, ulong_t P, bool Done = (N == 1), bool Prime = (P * P > N)>
struct Trial;

template <ulong_t N, ulong_t P, bool Prime>
struct Trial<N, P, true, Prime> {
  typedef Loki::NullType Result;
};

// P*P > N and N > 1: N itself is prime
template <ulong_t N, ulong_t P>
struct Trial<N, P, false, true> {
  typedef Loki::Typelist<pair_<ulong_<N>, ulong_<1> >, Loki::NullType> Result;
};

template <ulong_t N, ulong_t P>
struct Trial<N, P, false, false> {
  typedef Mult<N, P> M;
  typedef typename Trial<M::rest, (P == 2 ? 3 : P + 2)>::Result Next;
  typedef typename Loki::Select<(M::value > 0),
                                Loki::Typelist<pair_<ulong_<P>, ulong_<M::value> >, Next>,
                                Next>::Result Result;
};

}  // namespace refshim

template <typename Num>
struct Factorization;

template <long_t N>
struct Factorization<ulong_<N> > {
  typedef typename refshim::Trial<(ulong_t)N, 2>::Result Result;
};


template <class A, class B>
struct GCD;

template <long_t A, long_t B>
struct GCD<long_<A>, long_<B> > {
  typedef typename GCD<long_<B>, long_<A % B> >::Result Result;
};

template <long_t A>
struct GCD<long_<A>, long_<0> > {
  typedef long_<A> Result;
};

#endif
