// Shared device definitions for the GB300 CSEM kernels.
//
// Two arithmetic "precisions" drive every kernel template:
//   F64  bit-faithful complex128: each add/sub/mul/div is an explicitly rounded
//        __d*_rn intrinsic (never contracted into an FMA), divisions by grid spacings
//        are true IEEE divisions, complex products are (ar*br - ai*bi, ar*bi + ai*br)
//        and complex quotients use Smith's method (R. L. Smith, CACM 5(8) 1962).
//        Evaluated in the same order as the reference C (fdfd.c, solver.c), this gives
//        the reference's results bit for bit.
//   F32  fast complex64 for the inner solves of the mixed-precision solver: spacings
//        enter as precomputed reciprocals, FMA contraction is allowed.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "prof.h"

namespace csem {

struct F64 {
  typedef double R;
  typedef double2 C;
  static __device__ __forceinline__ R add(R a, R b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ R sub(R a, R b) { return __dsub_rn(a, b); }
  static __device__ __forceinline__ R mul(R a, R b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ R div(R a, R b) { return __ddiv_rn(a, b); }
  // a / d for a grid spacing d with reciprocal rinv: exact division here
  static __device__ __forceinline__ R divs(R a, R d, R rinv) { (void)rinv; return __ddiv_rn(a, d); }
  static __device__ __forceinline__ C mk(R x, R y) { return make_double2(x, y); }
  static constexpr bool exact = true;
};

struct F32 {
  typedef float R;
  typedef float2 C;
  static __device__ __forceinline__ R add(R a, R b) { return a + b; }
  static __device__ __forceinline__ R sub(R a, R b) { return a - b; }
  static __device__ __forceinline__ R mul(R a, R b) { return a * b; }
  static __device__ __forceinline__ R div(R a, R b) { return __fdiv_rn(a, b); }
  static __device__ __forceinline__ R divs(R a, R d, R rinv) { (void)d; return a * rinv; }
  static __device__ __forceinline__ C mk(R x, R y) { return make_float2(x, y); }
  static constexpr bool exact = false;
};

// F64Q: complex128 arithmetic without the reference's rounding, for the mixed solver's
// defect-correction residual r = b - A x, which needs complex128 accuracy but not the
// reference's bits: spacings enter as reciprocals and FMA contraction is allowed, as in
// F32. Its grids and per-system scalars have F64's layout (same R and C).
struct F64Q {
  typedef double R;
  typedef double2 C;
  static __device__ __forceinline__ R add(R a, R b) { return a + b; }
  static __device__ __forceinline__ R sub(R a, R b) { return a - b; }
  static __device__ __forceinline__ R mul(R a, R b) { return a * b; }
  static __device__ __forceinline__ R div(R a, R b) { return a / b; }
  static __device__ __forceinline__ R divs(R a, R d, R rinv) { (void)d; return a * rinv; }
  static __device__ __forceinline__ C mk(R x, R y) { return make_double2(x, y); }
  static constexpr bool exact = false;
};

// complex helpers over a precision P
template <class P> __device__ __forceinline__ typename P::C cadd(typename P::C a, typename P::C b)
{ return P::mk(P::add(a.x, b.x), P::add(a.y, b.y)); }
template <class P> __device__ __forceinline__ typename P::C csub(typename P::C a, typename P::C b)
{ return P::mk(P::sub(a.x, b.x), P::sub(a.y, b.y)); }
template <class P> __device__ __forceinline__ typename P::C cmul(typename P::C a, typename P::C b)
{ return P::mk(P::sub(P::mul(a.x, b.x), P::mul(a.y, b.y)), P::add(P::mul(a.x, b.y), P::mul(a.y, b.x))); }
template <class P> __device__ __forceinline__ typename P::C cconj(typename P::C a) { return P::mk(a.x, -a.y); }
template <class P> __device__ __forceinline__ typename P::C cneg(typename P::C a) { return P::mk(-a.x, -a.y); }
// real * complex (componentwise)
template <class P> __device__ __forceinline__ typename P::C rmul(typename P::R s, typename P::C a)
{ return P::mk(P::mul(s, a.x), P::mul(s, a.y)); }
// complex / real (componentwise true division)
template <class P> __device__ __forceinline__ typename P::C cdivr(typename P::C a, typename P::R d)
{ return P::mk(P::div(a.x, d), P::div(a.y, d)); }
// complex / grid spacing (exact in F64, reciprocal multiply in F32)
template <class P> __device__ __forceinline__ typename P::C cdivs(typename P::C a, typename P::R d, typename P::R r)
{ return P::mk(P::divs(a.x, d, r), P::divs(a.y, d, r)); }
// complex / complex, Smith 1962
template <class P> __device__ __forceinline__ typename P::C cdiv(typename P::C a, typename P::C b)
{
  typedef typename P::R R;
  if (fabs(b.x) < fabs(b.y)) {
    R r = P::div(b.x, b.y);
    R den = P::add(P::mul(b.x, r), b.y);
    return P::mk(P::div(P::add(P::mul(a.x, r), a.y), den), P::div(P::sub(P::mul(a.y, r), a.x), den));
  }
  R r = P::div(b.y, b.x);
  R den = P::add(P::mul(b.y, r), b.x);
  return P::mk(P::div(P::add(P::mul(a.y, r), a.x), den), P::div(P::sub(a.y, P::mul(a.x, r)), den));
}

template <class P> __device__ __forceinline__ typename P::C czero() { return P::mk(0, 0); }

// Geometry and conductivity of one padded model as one precision sees it.
// 1-D arrays are on the FULL padded grid (length n+1); r* are reciprocals.
// sigma* are full-grid flat arrays in the reference's index order.
template <class P> struct GridP {
  typedef typename P::R R;
  int n1, n2, n3;      // operator grid (n3 = nz+nb when airbc, else full depth)
  int n3f, nb, airbc, fvm;
  int kstart;          // nb when airbc else 0: operator plane k is full-grid plane k+kstart
  long lEx, lEy, lEz, lE;
  const R *d1, *d2, *d3, *d1s, *d2s, *d3s;
  const R *r1, *r2, *r3, *r1s, *r2s, *r3s;
  const R *s11, *s22, *s33;
};

// the same grid seen by another precision with the same real type (F64 -> F64Q)
template <class Q, class P> inline GridP<Q> grid_as(const GridP<P>& g)
{
  static_assert(sizeof(typename Q::R) == sizeof(typename P::R), "grid_as: same real type only");
  GridP<Q> q;
  q.n1 = g.n1; q.n2 = g.n2; q.n3 = g.n3; q.n3f = g.n3f; q.nb = g.nb; q.airbc = g.airbc; q.fvm = g.fvm;
  q.kstart = g.kstart;
  q.lEx = g.lEx; q.lEy = g.lEy; q.lEz = g.lEz; q.lE = g.lE;
  q.d1 = g.d1; q.d2 = g.d2; q.d3 = g.d3; q.d1s = g.d1s; q.d2s = g.d2s; q.d3s = g.d3s;
  q.r1 = g.r1; q.r2 = g.r2; q.r3 = g.r3; q.r1s = g.r1s; q.r2s = g.r2s; q.r3s = g.r3s;
  q.s11 = g.s11; q.s22 = g.s22; q.s33 = g.s33;
  return q;
}

// index maps of the reference layout (fdfd.c:13-21)
__device__ __forceinline__ long ix1(int n1, int n2, int k, int j, int i) { return i + (long)n1 * (j + (long)(n2 + 1) * k); }
__device__ __forceinline__ long ix2(int n1, int n2, int k, int j, int i) { return i + (long)(n1 + 1) * (j + (long)n2 * k); }
__device__ __forceinline__ long ix3(int n1, int n2, int k, int j, int i) { return i + (long)(n1 + 1) * (j + (long)(n2 + 1) * k); }

// Per-system scalars: I*omega*mu0 and its reciprocal 1/(I*omega*mu0), as complex.
template <class P> struct SysScal {
  typename P::C iom;
  typename P::C iwmu;
};

}  // namespace csem
