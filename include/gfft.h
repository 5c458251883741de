/*
 * gfft.h — C++ drop-in facade of GFFT's factory and transform objects over
 * the gfft_gb300 C ABI (gfft_gb300.h).
 *
 * Mirrors, name for name, what user code of the reference (scpp/gfft) writes
 * (pattern of src/gfft.cpp:40-97):
 *
 *   typedef TYPELIST_1(ulong_<1024>) NList;
 *   typedef GFFT::GenerateTransform<NList, GFFT::DOUBLE, TYPELIST_2(GFFT::DFT, GFFT::IDFT),
 *                                   ulong_<1>, GFFT::Serial, GFFT::IN_PLACE> TransformSet;
 *   TransformSet gfft;
 *   TransformSet::ObjectType* obj = gfft.CreateTransformObject(1024, GFFT::DOUBLE::ID, GFFT::DFT::ID,
 *                                                              1, GFFT::Serial::ID, GFFT::IN_PLACE::ID);
 *   obj->fft(data);            // IN_PLACE: AbstractFFT_inp<T>::fft(T*)
 *   delete obj;
 *
 * Reference interfaces replaced:
 *   GenerateTransform / CreateTransformObject   src/gfftgen.h:189-231
 *   TransformFactoryError::Exception            src/gfftgen.h:133-145
 *   AbstractFFT_inp / AbstractFFT_oop           src/gfftpolicy.h:46-58
 *   tags DOUBLE..COMPLEX_FLOAT, DFT..IRDFT (and DCT1..IDCT2),
 *   IN_PLACE/OUT_OF_PLACE, Serial/OpenMP<NT>    src/gfftpolicy.h:78-453
 *   groups (Default / FullList)                 src/gfftparamgroups.h:30-78
 *   Transform<...>::Instance                    src/gfftgen.h:46-87
 *
 * fft() takes HOST pointers here, exactly like the reference (it copies in,
 * transforms on the GPU, copies out); fft_device() takes device pointers and
 * a stream and does not synchronise.  Typelists: a small variadic stand-in
 * for Loki's (TYPELIST_n macros kept).  Differences: sizes are checked at
 * run time against NList (the reference compiles one class per size), and
 * an added ifft() runs the inverse transform type.
 */
#ifndef GFFT_GB300_FACADE_H
#define GFFT_GB300_FACADE_H

#include <complex>
#include <cstdint>
#include <exception>
#include <vector>

#include "gfft_gb300.h"

#ifndef GFFT_GB300_NO_INT_TYPES
/* integral constants as in the reference's metafactor sint.h */
template <unsigned long N>
struct ulong_ {
  static const unsigned long value = N;
};
template <long N>
struct long_ {
  static const long value = N;
};
template <unsigned long N>
struct SIntID : ulong_<N> {};
#endif

namespace GFFT {

/* ---- type lists ---------------------------------------------------------- */
template <class... T>
struct TypeList {};

template <class T>
struct AsList {
  typedef TypeList<T> type;
};
template <class... T>
struct AsList<TypeList<T...> > {
  typedef TypeList<T...> type;
};

#define TYPELIST_1(a) ::GFFT::TypeList<a>
#define TYPELIST_2(a, b) ::GFFT::TypeList<a, b>
#define TYPELIST_3(a, b, c) ::GFFT::TypeList<a, b, c>
#define TYPELIST_4(a, b, c, d) ::GFFT::TypeList<a, b, c, d>
#define TYPELIST_5(a, b, c, d, e) ::GFFT::TypeList<a, b, c, d, e>
#define TYPELIST_6(a, b, c, d, e, f) ::GFFT::TypeList<a, b, c, d, e, f>

template <class L>
struct Values;
template <class... T>
struct Values<TypeList<T...> > {
  static std::vector<unsigned long> ids() { return {static_cast<unsigned long>(T::ID)...}; }
  static std::vector<unsigned long> nums() { return {static_cast<unsigned long>(T::value)...}; }
};

/* ---- tags (IDs identical to the reference) ------------------------------- */
typedef unsigned int id_t;

struct DOUBLE {
  static const id_t ID = 0;
  typedef double base_type;
  typedef double ValueType;
  static const char* name() { return "double"; }
};
struct FLOAT {
  static const id_t ID = 1;
  typedef float base_type;
  typedef float ValueType;
  static const char* name() { return "float"; }
};
struct COMPLEX_DOUBLE {
  static const id_t ID = 2;
  typedef double base_type;
  typedef std::complex<double> ValueType;
  static const char* name() { return "std::complex<double>"; }
};
struct COMPLEX_FLOAT {
  static const id_t ID = 3;
  typedef float base_type;
  typedef std::complex<float> ValueType;
  static const char* name() { return "std::complex<float>"; }
};

struct IDFT;
struct IRDFT;
struct DFT {
  static const id_t ID = 0;
  static const int Sign = 1;
  typedef IDFT Inverse;
};
struct IDFT {
  static const id_t ID = 1;
  static const int Sign = -1;
  typedef DFT Inverse;
};
struct RDFT {
  static const id_t ID = 2;
  static const int Sign = 1;
  typedef IRDFT Inverse;
};
struct IRDFT {
  static const id_t ID = 3;
  static const int Sign = -1;
  typedef RDFT Inverse;
};
/* Cosine transforms of n reals (DOUBLE / FLOAT): the sums of the reference's
 * direct.h (src/direct.h:270-312); the I* tags divide by n (Backward). */
struct IDCT1;
struct IDCT2;
struct DCT1 {
  static const id_t ID = 4;
  static const int Sign = 1;
  typedef IDCT1 Inverse;
};
struct IDCT1 {
  static const id_t ID = 5;
  static const int Sign = -1;
  typedef DCT1 Inverse;
};
struct DCT2 {
  static const id_t ID = 6;
  static const int Sign = 1;
  typedef IDCT2 Inverse;
};
struct IDCT2 {
  static const id_t ID = 7;
  static const int Sign = -1;
  typedef DCT2 Inverse;
};

struct Serial {
  static const id_t ID = 0;
  static const unsigned long NParProc = 1;
};
template <unsigned int NT>
struct OpenMP {
  static const id_t ID = NT - 1;
  static const unsigned long NParProc = NT;
};
template <>
struct OpenMP<0> : Serial {};
template <>
struct OpenMP<1> : Serial {};

template <class T>
class AbstractFFT_inp {
 public:
  virtual void fft(T*) = 0;
  virtual ~AbstractFFT_inp() {}
};
template <class T>
class AbstractFFT_oop {
 public:
  virtual void fft(const T*, T*) = 0;
  virtual ~AbstractFFT_oop() {}
};

struct IN_PLACE {
  static const id_t ID = 0;
  template <class T>
  struct Interface {
    typedef AbstractFFT_inp<T> Result;
  };
  static const char* name() { return "in-place"; }
};
struct OUT_OF_PLACE {
  static const id_t ID = 1;
  template <class T>
  struct Interface {
    typedef AbstractFFT_oop<T> Result;
  };
  static const char* name() { return "out-of-place"; }
};

struct ValueTypeGroup {
  typedef TYPELIST_4(DOUBLE, FLOAT, COMPLEX_DOUBLE, COMPLEX_FLOAT) FullList;
  typedef DOUBLE Default;
};
struct TransformTypeGroup {
  typedef TYPELIST_4(DFT, IDFT, RDFT, IRDFT) FullList;
  typedef DFT Default;
};
struct ParallelizationGroup {
  typedef TYPELIST_4(OpenMP<1>, OpenMP<2>, OpenMP<4>, OpenMP<8>) FullList;
  typedef Serial Default;
};
struct PlaceGroup {
  typedef TYPELIST_2(IN_PLACE, OUT_OF_PLACE) FullList;
  typedef OUT_OF_PLACE Default;
};

/* ---- errors -------------------------------------------------------------- */
template <typename IdentifierType, class AbstractProduct>
struct TransformFactoryError {
  struct Exception : public std::exception {
    const char* what() const throw() {
      return "Requested transform is not compiled! Check your instantiation of GenerateTransform class!";
    }
  };
};

/* A failing C-ABI call (allocation, CUDA, invalid argument). */
struct GpuError : public std::exception {
  int status;
  explicit GpuError(int s) : status(s) {}
  const char* what() const throw() { return gfft_strerror(status); }
};

inline void check(int st) {
  if (st != GFFT_OK) throw GpuError(st);
}

/* ---- transform objects --------------------------------------------------- */
namespace detail {

class Handle {
 public:
  Handle(unsigned long n, int vt, int tr, int par, int pl, unsigned long batch) : h_(nullptr) {
    check(gfft_create(&h_, n, vt, tr, 1, par, pl, batch));
  }
  ~Handle() {
    if (h_) gfft_destroy(h_);
  }
  gfft_handle get() const { return h_; }

 private:
  Handle(const Handle&);
  Handle& operator=(const Handle&);
  gfft_handle h_;
};

template <class T, class Base>
class ObjectBase : public Base {
 public:
  ObjectBase(unsigned long n, int vt, int tr, int par, int pl, unsigned long batch)
      : n_(n), vt_(vt), tr_(tr), par_(par), pl_(pl), batch_(batch), h_(n, vt, tr, par, pl, batch), inv_(nullptr) {}
  ~ObjectBase() { delete inv_; }
  /* device pointers, asynchronous on `stream` */
  void fft_device(const void* src, void* dst, gfft_stream stream = nullptr) {
    check(gfft_exec(h_.get(), src, dst, stream));
  }
  gfft_handle handle() const { return h_.get(); }

 protected:
  void run_host(const T* src, T* dst) { check(gfft_exec_host(h_.get(), src, dst, nullptr)); }
  detail::Handle& inverse() {
    if (!inv_) {
      static const int inv_of[8] = {1, 0, 3, 2, 5, 4, 7, 6};
      inv_ = new Handle(n_, vt_, inv_of[tr_], par_, pl_, batch_);
    }
    return *inv_;
  }
  unsigned long n_;
  int vt_, tr_, par_, pl_;
  unsigned long batch_;
  Handle h_;
  Handle* inv_;
};

}  // namespace detail

template <class T>
class InPlaceObject : public detail::ObjectBase<T, AbstractFFT_inp<T> > {
  typedef detail::ObjectBase<T, AbstractFFT_inp<T> > B;

 public:
  InPlaceObject(unsigned long n, int vt, int tr, int par, unsigned long batch = 1) : B(n, vt, tr, par, 0, batch) {}
  void fft(T* data) { this->run_host(data, data); }
  void ifft(T* data) { check(gfft_exec_host(this->inverse().get(), data, data, nullptr)); }
};

template <class T>
class OutOfPlaceObject : public detail::ObjectBase<T, AbstractFFT_oop<T> > {
  typedef detail::ObjectBase<T, AbstractFFT_oop<T> > B;

 public:
  OutOfPlaceObject(unsigned long n, int vt, int tr, int par, unsigned long batch = 1) : B(n, vt, tr, par, 1, batch) {}
  void fft(const T* src, T* dst) { this->run_host(src, dst); }
  void ifft(const T* src, T* dst) { check(gfft_exec_host(this->inverse().get(), src, dst, nullptr)); }
};

template <class Place, class T>
struct ObjectFor;
template <class T>
struct ObjectFor<IN_PLACE, T> {
  typedef InPlaceObject<T> type;
};
template <class T>
struct ObjectFor<OUT_OF_PLACE, T> {
  typedef OutOfPlaceObject<T> type;
};

/* Transform<N, VType, Type, Dim, Parall, Place>::Instance (src/gfftgen.h:46-87) */
template <class N, class VType, class Type, class Dim = ulong_<1>, class Parall = Serial, class Place = OUT_OF_PLACE>
class Transform {
 public:
  typedef typename VType::ValueType T;
  typedef typename ObjectFor<Place, T>::type Instance;
  typedef typename Place::template Interface<T>::Result ReturnType;
  static const unsigned long Len = N::value;
  static ReturnType* Create() { return new Instance(N::value, VType::ID, Type::ID, Parall::ID); }
};

/* GenerateTransform<NList, VType, TransType, Dim, Parall, Place>
 * (src/gfftgen.h:189-231).  NList holds ulong_<N> sizes; the other
 * parameters are one tag or a TYPELIST of tags.  ObjectType is the abstract
 * interface of the (single) place; VType fixes the element type. */
template <class NList, class VType, class TransType = TransformTypeGroup::Default, class Dim = ulong_<1>,
          class Parall = ParallelizationGroup::Default, class Place = PlaceGroup::Default>
class GenerateTransform {
 public:
  typedef typename VType::ValueType T;
  typedef Place PlaceType;
  typedef typename Place::template Interface<T>::Result ObjectType;

  ObjectType* CreateTransformObject(unsigned long n, unsigned long vtype_id,
                                    unsigned long trans_id = TransformTypeGroup::Default::ID, unsigned long dim = 1,
                                    unsigned long parall_id = ParallelizationGroup::Default::ID,
                                    unsigned long place_id = PlaceGroup::Default::ID, unsigned long batch = 1) {
    if (!contains(Values<typename AsList<NList>::type>::nums(), n) || vtype_id != VType::ID ||
        !contains(Values<typename AsList<TransType>::type>::ids(), trans_id) || dim != Dim::value ||
        !contains(Values<typename AsList<Parall>::type>::ids(), parall_id) || place_id != Place::ID)
      throw typename TransformFactoryError<unsigned long, ObjectType>::Exception();
    return new typename ObjectFor<Place, T>::type(n, (int)vtype_id, (int)trans_id, (int)parall_id, batch);
  }

 private:
  static bool contains(const std::vector<unsigned long>& v, unsigned long x) {
    for (unsigned long e : v)
      if (e == x) return true;
    return false;
  }
};

}  // namespace GFFT

#endif /* GFFT_GB300_FACADE_H */
