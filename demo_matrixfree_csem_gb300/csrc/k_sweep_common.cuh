// Helpers shared by the LU-SGS component sweeps (k_lusgs2.cu: lockstep row pipelines,
// k_lusgs3.cu: line-tiled complex64 sweeps): the view of one system's vector on the
// sweep grid, 1-D spacings, read-only loads and the complex64 linear-form point update.
#pragma once
#include "csem_cuda.cuh"
#include "engine.h"

namespace csem {
namespace sweep {
namespace {

template <class P> struct View {
  typedef typename P::C C;
  int n1, n2, vshift;
  C* Y[3];
  C* CAP[3];
  const C* X[3];
  __device__ __forceinline__ long idx(int c, int k, int j, int i) const
  {
    return c == 0 ? ix1(n1, n2, k, j, i) : (c == 1 ? ix2(n1, n2, k, j, i) : ix3(n1, n2, k, j, i));
  }
  __device__ __forceinline__ C* at(int c, int k, int j, int i) const
  {
    return k >= vshift ? Y[c] + idx(c, k - vshift, j, i) : CAP[c] + idx(c, k, j, i);
  }
  __device__ __forceinline__ C ld(int c, int k, int j, int i) const { return *at(c, k, j, i); }
  // start of row (k, j) of component c (element i of the row is row[i]); rows of one
  // plane are row_len(c) elements apart
  __device__ __forceinline__ C* row(int c, int k, int j) const { return at(c, k, j, 0); }
  __device__ __forceinline__ const C* brow(int c, int k, int j) const
  {
    return k >= vshift ? X[c] + idx(c, k - vshift, j, 0) : nullptr;
  }
  __device__ __forceinline__ int row_len(int c) const { return c == 0 ? n1 : n1 + 1; }
};

template <class P>
__device__ __forceinline__ View<P> view_of(const SweepP<P>& s, int slot, int sys)
{
  View<P> v;
  v.n1 = s.g.n1;
  v.n2 = s.g.n2;
  v.vshift = s.vshift;
  typename P::C* y = s.Y + (size_t)sys * s.g.lE;
  v.Y[0] = y;
  v.Y[1] = y + s.g.lEx;
  v.Y[2] = y + s.g.lEx + s.g.lEy;
  const typename P::C* x = s.X + (size_t)sys * s.g.lE;
  v.X[0] = x;
  v.X[1] = x + s.g.lEx;
  v.X[2] = x + s.g.lEx + s.g.lEy;
  typename P::C* cp = s.CAP ? s.CAP + (size_t)slot * s.capE : nullptr;
  v.CAP[0] = cp;
  v.CAP[1] = cp ? cp + s.capEx : nullptr;
  v.CAP[2] = cp ? cp + s.capEx + s.capEy : nullptr;
  return v;
}

// read-only loads (nothing a sweep reads through these is written during the launch)
template <class T> __device__ __forceinline__ T ro(const T* p) { return __ldg(p); }

// 1-D spacings of one axis at index n: staggered d*s[n], d*s[n-1], cell d*[n] and their
// reciprocals (the F32 path divides by multiplying)
template <class P> struct Ax {
  typename P::R ds, rs, dsm, rsm, d, r;
};
// all six values at n >= 1
template <class P>
__device__ __forceinline__ Ax<P> axis(const typename P::R* d, const typename P::R* ds, const typename P::R* r,
                                      const typename P::R* rs, int n)
{
  Ax<P> a;
  a.ds = ro(ds + n);
  a.rs = ro(rs + n);
  a.dsm = ro(ds + n - 1);
  a.rsm = ro(rs + n - 1);
  a.d = ro(d + n);
  a.r = ro(r + n);
  return a;
}
// the values at n only (n may be 0; dsm/rsm are not used by the caller)
template <class P>
__device__ __forceinline__ Ax<P> axis_at(const typename P::R* d, const typename P::R* ds, const typename P::R* r,
                                         const typename P::R* rs, int n)
{
  Ax<P> a;
  a.ds = ro(ds + n);
  a.rs = ro(rs + n);
  a.dsm = 0;
  a.rsm = 0;
  a.d = ro(d + n);
  a.r = ro(r + n);
  return a;
}

struct Lin32 {
  float2 B, w;
  float gp, gn;
};

__device__ __forceinline__ float2 mul32(float2 a, float2 b)
{
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 sub32(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 scl32(float s, float2 a) { return make_float2(s * a.x, s * a.y); }

// the chain part: v = B + w (gp prev + gn nb)
__device__ __forceinline__ float2 lin_apply(const Lin32& L, float2 prev, float2 nb)
{
  const float2 u = make_float2(L.gp * prev.x + L.gn * nb.x, L.gp * prev.y + L.gn * nb.y);
  return make_float2(L.B.x + L.w.x * u.x - L.w.y * u.y, L.B.y + L.w.x * u.y + L.w.y * u.x);
}

// aii = gg iwmu - sg (fdfd.c fin); kc = known - cross
__device__ __forceinline__ Lin32 lin_make(const SysScal<F32>& sc, int fvm, float gg, float sg, float vol,
                                          float2 b, float2 kc, float gp, float gn)
{
  const float2 aii = make_float2(gg * sc.iwmu.x - sg, gg * sc.iwmu.y);
  const float r = __frcp_rn(aii.x * aii.x + aii.y * aii.y);
  const float2 inv = make_float2(aii.x * r, -aii.y * r);
  Lin32 L;
  L.w = mul32(sc.iwmu, inv);
  float2 bt = mul32(b, inv);
  if (fvm) {
    const float2 f = make_float2(vol * sc.iom.x, vol * sc.iom.y);
    const float rf = __frcp_rn(f.x * f.x + f.y * f.y);
    bt = mul32(bt, make_float2(f.x * rf, -f.y * rf));
  }
  const float2 wk = mul32(L.w, kc);
  L.B = make_float2(bt.x + wk.x, bt.y + wk.y);
  L.gp = gp;
  L.gn = gn;
  return L;
}

}  // namespace
}  // namespace sweep
}  // namespace csem
