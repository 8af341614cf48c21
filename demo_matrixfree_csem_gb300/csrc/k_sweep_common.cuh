// Helpers shared by the LU-SGS component sweeps (k_lusgs2.cu: lockstep row pipelines,
// k_lusgs3.cu: line-tiled complex64 sweeps, k_lusgs4.cu: row pipelines over several
// systems at one frequency): the view of one system's vector on the sweep grid, 1-D
// spacings, read-only loads, the hand-over between warps and the complex64 linear-form
// point update.
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

constexpr int MAXROWS = 512;  // rows of one sweep handled by one CTA (a thread each)
constexpr int NB_ROWS = 256;  // up to this many rows the warps hand over through named barriers

template <class C> __device__ __forceinline__ C shfl_up(C v)
{
  C r;
  r.x = __shfl_up_sync(0xffffffffu, v.x, 1);
  r.y = __shfl_up_sync(0xffffffffu, v.y, 1);
  return r;
}

// Hand-over between warps. Warp w's last row feeds warp w+1's first row one step later
// through a one-slot buffer in shared memory, synchronised pairwise with named barriers
// (ids 1 + 2w "full" and 2 + 2w "empty", 64 threads each: the producing and the
// consuming warp), so a warp waits only for its neighbours, never for the whole CTA.
// At each step T >= 1 the consumer waits on "full", reads and signals "empty"; at each
// step the producer (from T >= 1 after waiting on "empty", i.e. once the previous value
// has been read) writes and signals "full". Each barrier generation therefore holds
// exactly one producer and one consumer operation, and a final wait on "full" after
// the loop completes the last one (this protocol was checked exhaustively over warp
// counts and step counts, under arbitrary interleavings, before use).
__device__ __forceinline__ void nbar_sync(int id) { asm volatile("bar.sync %0, 64;" ::"r"(id) : "memory"); }
__device__ __forceinline__ void nbar_arrive(int id) { asm volatile("bar.arrive %0, 64;" ::"r"(id) : "memory"); }

// Hand-over state of one CTA. Up to 256 rows (8 warps): the one-slot buffer with the
// pairwise named barriers described above. Larger CTAs (up to 16 warps; there are only
// 16 named barriers) use a two-slot buffer and one CTA barrier per step instead.
template <int VW, class C, bool NAMED> struct HandOff;

template <int VW, class C> struct HandOff<VW, C, true> {
  C slot[NB_ROWS / 32][VW];
  // the value the row before this thread's row produced at the previous step: a shuffle
  // from the previous lane, or the slot for lane 0; the first row reads the zero boundary
  __device__ __forceinline__ void get(const C (&res)[VW], C (&nb)[VW], int T)
  {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < VW; q++) nb[q] = shfl_up(res[q]);
    if (w > 0 && T > 0) {
      nbar_sync(1 + 2 * (w - 1));  // warp w-1 has written step T-1
      if (lane == 0) {
#pragma unroll
        for (int q = 0; q < VW; q++) nb[q] = slot[w - 1][q];
      }
      nbar_arrive(2 + 2 * (w - 1));  // the slot may be rewritten
    } else if (lane == 0) {
#pragma unroll
      for (int q = 0; q < VW; q++) {
        nb[q].x = 0;
        nb[q].y = 0;
      }
    }
  }
  __device__ __forceinline__ void put(const C (&res)[VW], int T)
  {
    const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (w + 1 >= nw) return;  // the last warp feeds nobody
    if (T >= 1) nbar_sync(2 + 2 * w);  // warp w+1 has read step T-1
    if ((threadIdx.x & 31) == 31) {
#pragma unroll
      for (int q = 0; q < VW; q++) slot[w][q] = res[q];
    }
    nbar_arrive(1 + 2 * w);
  }
  // completes the last generation of the "full" barriers after the step loop
  __device__ __forceinline__ void finish(int nsteps)
  {
    const int w = threadIdx.x >> 5;
    if (w > 0 && nsteps > 0) nbar_sync(1 + 2 * (w - 1));
  }
};

template <int VW, class C> struct HandOff<VW, C, false> {
  C slot[2][MAXROWS / 32][VW];
  __device__ __forceinline__ void get(const C (&res)[VW], C (&nb)[VW], int T)
  {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < VW; q++) nb[q] = shfl_up(res[q]);
    if (lane == 0) {
#pragma unroll
      for (int q = 0; q < VW; q++) {
        C v;
        v.x = 0;
        v.y = 0;
        if (w > 0 && T > 0) v = slot[(T - 1) & 1][w - 1][q];
        nb[q] = v;
      }
    }
  }
  __device__ __forceinline__ void put(const C (&res)[VW], int T)
  {
    if ((threadIdx.x & 31) == 31) {
#pragma unroll
      for (int q = 0; q < VW; q++) slot[T & 1][threadIdx.x >> 5][q] = res[q];
    }
    __syncthreads();
  }
  __device__ __forceinline__ void finish(int) {}
};

// The same hand-over for CTAs of exactly NW warps (NW <= 8) with the barrier ids as
// immediates: the pairs use ids 1 .. 2 NW - 2 only, so a CTA holds 2 NW - 1 hardware
// barriers instead of 16 and more CTAs fit on an SM (a runtime id makes the compiler
// reserve all 16).
template <int ID> __device__ __forceinline__ void nbar_sync_i() { asm volatile("bar.sync %0, 64;" ::"n"(ID) : "memory"); }
template <int ID> __device__ __forceinline__ void nbar_arrive_i() { asm volatile("bar.arrive %0, 64;" ::"n"(ID) : "memory"); }

#define CSEM_NBAR_CASE(K, F)            \
  case K:                               \
    if constexpr (K <= MAXID) F<K>();   \
    break;
template <int MAXID> __device__ __forceinline__ void nbar_sync_n(int id)
{
  switch (id) {
    CSEM_NBAR_CASE(1, nbar_sync_i) CSEM_NBAR_CASE(2, nbar_sync_i) CSEM_NBAR_CASE(3, nbar_sync_i)
    CSEM_NBAR_CASE(4, nbar_sync_i) CSEM_NBAR_CASE(5, nbar_sync_i) CSEM_NBAR_CASE(6, nbar_sync_i)
    CSEM_NBAR_CASE(7, nbar_sync_i) CSEM_NBAR_CASE(8, nbar_sync_i) CSEM_NBAR_CASE(9, nbar_sync_i)
    CSEM_NBAR_CASE(10, nbar_sync_i) CSEM_NBAR_CASE(11, nbar_sync_i) CSEM_NBAR_CASE(12, nbar_sync_i)
    CSEM_NBAR_CASE(13, nbar_sync_i) CSEM_NBAR_CASE(14, nbar_sync_i)
    default: break;
  }
}
template <int MAXID> __device__ __forceinline__ void nbar_arrive_n(int id)
{
  switch (id) {
    CSEM_NBAR_CASE(1, nbar_arrive_i) CSEM_NBAR_CASE(2, nbar_arrive_i) CSEM_NBAR_CASE(3, nbar_arrive_i)
    CSEM_NBAR_CASE(4, nbar_arrive_i) CSEM_NBAR_CASE(5, nbar_arrive_i) CSEM_NBAR_CASE(6, nbar_arrive_i)
    CSEM_NBAR_CASE(7, nbar_arrive_i) CSEM_NBAR_CASE(8, nbar_arrive_i) CSEM_NBAR_CASE(9, nbar_arrive_i)
    CSEM_NBAR_CASE(10, nbar_arrive_i) CSEM_NBAR_CASE(11, nbar_arrive_i) CSEM_NBAR_CASE(12, nbar_arrive_i)
    CSEM_NBAR_CASE(13, nbar_arrive_i) CSEM_NBAR_CASE(14, nbar_arrive_i)
    default: break;
  }
}
#undef CSEM_NBAR_CASE

template <int VW, class C, int NW> struct HandOffN {
  static constexpr int MAXID = 2 * NW - 2;
  C slot[NW > 1 ? NW - 1 : 1][VW];
  __device__ __forceinline__ void get(const C (&res)[VW], C (&nb)[VW], int T)
  {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < VW; q++) nb[q] = shfl_up(res[q]);
    if (w > 0 && T > 0) {
      nbar_sync_n<MAXID>(1 + 2 * (w - 1));  // warp w-1 has written step T-1
      if (lane == 0) {
#pragma unroll
        for (int q = 0; q < VW; q++) nb[q] = slot[w - 1][q];
      }
      nbar_arrive_n<MAXID>(2 + 2 * (w - 1));  // the slot may be rewritten
    } else if (lane == 0) {
#pragma unroll
      for (int q = 0; q < VW; q++) {
        nb[q].x = 0;
        nb[q].y = 0;
      }
    }
  }
  __device__ __forceinline__ void put(const C (&res)[VW], int T)
  {
    const int w = threadIdx.x >> 5;
    if (w + 1 >= NW) return;  // the last warp feeds nobody
    if (T >= 1) nbar_sync_n<MAXID>(2 + 2 * w);  // warp w+1 has read step T-1
    if ((threadIdx.x & 31) == 31) {
#pragma unroll
      for (int q = 0; q < VW; q++) slot[w][q] = res[q];
    }
    nbar_arrive_n<MAXID>(1 + 2 * w);
  }
  __device__ __forceinline__ void finish(int nsteps)
  {
    const int w = threadIdx.x >> 5;
    if (w > 0 && nsteps > 0) nbar_sync_n<MAXID>(1 + 2 * (w - 1));
  }
};

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

// The parts of the linear form that depend only on the point and the frequency (shared
// by every system at that frequency): 1/aii with aii = gg iwmu - sg (fdfd.c fin), w =
// iwmu/aii and, with fvm, 1/(vol iom)
struct Coef32 {
  float2 inv, w, finv;
};

__device__ __forceinline__ Coef32 lin_coef(const SysScal<F32>& sc, int fvm, float gg, float sg, float vol)
{
  const float2 aii = make_float2(gg * sc.iwmu.x - sg, gg * sc.iwmu.y);
  const float r = __frcp_rn(aii.x * aii.x + aii.y * aii.y);
  Coef32 c;
  c.inv = make_float2(aii.x * r, -aii.y * r);
  c.w = mul32(sc.iwmu, c.inv);
  c.finv = make_float2(0.f, 0.f);
  if (fvm) {
    const float2 f = make_float2(vol * sc.iom.x, vol * sc.iom.y);
    const float rf = __frcp_rn(f.x * f.x + f.y * f.y);
    c.finv = make_float2(f.x * rf, -f.y * rf);
  }
  return c;
}

// the system's part: B = b/(f aii) + w kc, kc = known - cross
__device__ __forceinline__ float2 lin_B(const Coef32& c, int fvm, float2 b, float2 kc)
{
  float2 bt = mul32(b, c.inv);
  if (fvm) bt = mul32(bt, c.finv);
  const float2 wk = mul32(c.w, kc);
  return make_float2(bt.x + wk.x, bt.y + wk.y);
}

__device__ __forceinline__ Lin32 lin_make(const SysScal<F32>& sc, int fvm, float gg, float sg, float vol,
                                          float2 b, float2 kc, float gp, float gn)
{
  const Coef32 c = lin_coef(sc, fvm, gg, sg, vol);
  Lin32 L;
  L.w = c.w;
  L.B = lin_B(c, fvm, b, kc);
  L.gp = gp;
  L.gn = gn;
  return L;
}

}  // namespace
}  // namespace sweep
}  // namespace csem
