// LU-SGS component sweeps as pipelined warps: one launch per sweep.
//
// A sweep updates one field component in the reference's lexicographic Gauss-Seidel
// order (fdfd.c:347-503). In the coupled plane (r, m) a point depends on (r-1, m) and
// (r, m-1) (forward; (r+1, m), (r, m+1) backward); the third axis is independent:
//   Ex: rows r = k, march m = j, independent i      (k_sweep_x, 4 i per lane)
//   Ey: rows r = k, march m = i, independent j      (k_sweep_yz, 4 i per step)
//   Ez: rows r = j, march m = i, independent k      (k_sweep_yz, 4 i per step)
// One warp owns one independent line (Ex: 4 consecutive i) of one system. Its 32 lanes
// take 32 consecutive rows and run skewed by one step: at macro-step T lane l works at
// march position T - l, so the row above (lane l-1) finished that position one step
// earlier and hands its new values over with a warp shuffle; the own-row dependency is
// a register. Row blocks of 32 follow one another; the row just above a block is read
// back from memory. Every point is computed with the same arithmetic and the same
// neighbour values as the reference, so complex128 results are bit-identical.
// In Ey/Ez sweeps each lane advances 4 consecutive i per macro-step (one 32-byte
// sector of complex64 per row and array).
#include "csem_cuda.cuh"
#include "engine.h"

namespace csem {

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
  __device__ __forceinline__ C ld(int c, int k, int j, int i) const
  {
    return k >= vshift ? Y[c][idx(c, k - vshift, j, i)] : CAP[c][idx(c, k, j, i)];
  }
  __device__ __forceinline__ void st(int c, int k, int j, int i, C v) const
  {
    if (k >= vshift) Y[c][idx(c, k - vshift, j, i)] = v;
    else CAP[c][idx(c, k, j, i)] = v;
  }
  __device__ __forceinline__ C ldb(int c, int k, int j, int i) const
  {
    return k >= vshift ? X[c][idx(c, k - vshift, j, i)] : P::mk(0, 0);
  }
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

template <class P>
__device__ __forceinline__ typename P::R geo(typename P::R a0, typename P::R a1, typename P::R A, typename P::R b0,
                                             typename P::R b1, typename P::R B)
{
  typedef typename P::R R;
  const R one = 1;
  return P::add(P::div(P::add(P::div(one, a0), P::div(one, a1)), A),
                P::div(P::add(P::div(one, b0), P::div(one, b1)), B));
}

template <class P>
__device__ __forceinline__ typename P::C fin(typename P::C b, typename P::C aij, typename P::R gg, typename P::R sg,
                                             typename P::R vol, const SysScal<P>& sc, int fvm)
{
  typename P::C aii = rmul<P>(gg, sc.iwmu);
  aii.x = P::sub(aii.x, sg);
  if (fvm) {
    typename P::C f = rmul<P>(vol, sc.iom);
    aij = cmul<P>(aij, f);
    aii = cmul<P>(aii, f);
  }
  return cdiv<P>(csub<P>(b, aij), aii);
}

// --- per-point updates with the reference's operation order; the component being
// updated is zero at its own point while its row is evaluated (fdfd.c:357,383,409)

// Ex at (k,j,i): fdfd.c:358-369
template <class P>
__device__ __forceinline__ typename P::C upd_ex(const GridP<P>& g, const SysScal<P>& sc, int k, int j, int i,
                                                typename P::C eyA, typename P::C eyB, typename P::C eyC,
                                                typename P::C eyD, typename P::C exjp, typename P::C exjm,
                                                typename P::C exkp, typename P::C exkm, typename P::C ezA,
                                                typename P::C ezB, typename P::C ezC, typename P::C ezD,
                                                typename P::C b)
{
  typedef typename P::C C;
  const C own = czero<P>();
  C t1 = csub<P>(cdivs<P>(csub<P>(eyA, eyB), g.d1s[i], g.r1s[i]), cdivs<P>(csub<P>(exjp, own), g.d2s[j], g.r2s[j]));
  C t2 = csub<P>(cdivs<P>(csub<P>(eyC, eyD), g.d1s[i], g.r1s[i]), cdivs<P>(csub<P>(own, exjm), g.d2s[j - 1], g.r2s[j - 1]));
  C t3 = csub<P>(cdivs<P>(csub<P>(exkp, own), g.d3s[k], g.r3s[k]), cdivs<P>(csub<P>(ezA, ezB), g.d1s[i], g.r1s[i]));
  C t4 = csub<P>(cdivs<P>(csub<P>(own, exkm), g.d3s[k - 1], g.r3s[k - 1]), cdivs<P>(csub<P>(ezC, ezD), g.d1s[i], g.r1s[i]));
  const typename P::R sg = g.s11[ix1(g.n1, g.n2, k, j, i)];
  C aij = csub<P>(cmul<P>(csub<P>(cdivs<P>(csub<P>(t1, t2), g.d2[j], g.r2[j]), cdivs<P>(csub<P>(t3, t4), g.d3[k], g.r3[k])),
                          sc.iwmu),
                  rmul<P>(sg, own));
  typename P::R gg = geo<P>(g.d2s[j], g.d2s[j - 1], g.d2[j], g.d3s[k], g.d3s[k - 1], g.d3[k]);
  typename P::R vol = g.fvm ? P::mul(P::mul(g.d1s[i], g.d2[j]), g.d3[k]) : 0;
  return fin<P>(b, aij, gg, sg, vol, sc, g.fvm);
}

// Ey at (k,j,i): fdfd.c:384-395
template <class P>
__device__ __forceinline__ typename P::C upd_ey(const GridP<P>& g, const SysScal<P>& sc, int k, int j, int i,
                                                typename P::C ezA, typename P::C ezB, typename P::C ezC,
                                                typename P::C ezD, typename P::C eykp, typename P::C eykm,
                                                typename P::C eyip, typename P::C eyim, typename P::C exA,
                                                typename P::C exB, typename P::C exC, typename P::C exD,
                                                typename P::C b)
{
  typedef typename P::C C;
  const C own = czero<P>();
  C t1 = csub<P>(cdivs<P>(csub<P>(ezA, ezB), g.d2s[j], g.r2s[j]), cdivs<P>(csub<P>(eykp, own), g.d3s[k], g.r3s[k]));
  C t2 = csub<P>(cdivs<P>(csub<P>(ezC, ezD), g.d2s[j], g.r2s[j]), cdivs<P>(csub<P>(own, eykm), g.d3s[k - 1], g.r3s[k - 1]));
  C t3 = csub<P>(cdivs<P>(csub<P>(eyip, own), g.d1s[i], g.r1s[i]), cdivs<P>(csub<P>(exA, exB), g.d2s[j], g.r2s[j]));
  C t4 = csub<P>(cdivs<P>(csub<P>(own, eyim), g.d1s[i - 1], g.r1s[i - 1]), cdivs<P>(csub<P>(exC, exD), g.d2s[j], g.r2s[j]));
  const typename P::R sg = g.s22[ix2(g.n1, g.n2, k, j, i)];
  C aij = csub<P>(cmul<P>(csub<P>(cdivs<P>(csub<P>(t1, t2), g.d3[k], g.r3[k]), cdivs<P>(csub<P>(t3, t4), g.d1[i], g.r1[i])),
                          sc.iwmu),
                  rmul<P>(sg, own));
  typename P::R gg = geo<P>(g.d3s[k], g.d3s[k - 1], g.d3[k], g.d1s[i], g.d1s[i - 1], g.d1[i]);
  typename P::R vol = g.fvm ? P::mul(P::mul(g.d1s[i], g.d2[j]), g.d3[k]) : 0;  // Ex's volume (fdfd.c:391)
  return fin<P>(b, aij, gg, sg, vol, sc, g.fvm);
}

// Ez at (k,j,i): fdfd.c:410-421
template <class P>
__device__ __forceinline__ typename P::C upd_ez(const GridP<P>& g, const SysScal<P>& sc, int k, int j, int i,
                                                typename P::C exA, typename P::C exB, typename P::C exC,
                                                typename P::C exD, typename P::C ezip, typename P::C ezim,
                                                typename P::C ezjp, typename P::C ezjm, typename P::C eyA,
                                                typename P::C eyB, typename P::C eyC, typename P::C eyD,
                                                typename P::C b)
{
  typedef typename P::C C;
  const C own = czero<P>();
  C t1 = csub<P>(cdivs<P>(csub<P>(exA, exB), g.d3s[k], g.r3s[k]), cdivs<P>(csub<P>(ezip, own), g.d1s[i], g.r1s[i]));
  C t2 = csub<P>(cdivs<P>(csub<P>(exC, exD), g.d3s[k], g.r3s[k]), cdivs<P>(csub<P>(own, ezim), g.d1s[i - 1], g.r1s[i - 1]));
  C t3 = csub<P>(cdivs<P>(csub<P>(ezjp, own), g.d2s[j], g.r2s[j]), cdivs<P>(csub<P>(eyA, eyB), g.d3s[k], g.r3s[k]));
  C t4 = csub<P>(cdivs<P>(csub<P>(own, ezjm), g.d2s[j - 1], g.r2s[j - 1]), cdivs<P>(csub<P>(eyC, eyD), g.d3s[k], g.r3s[k]));
  const typename P::R sg = g.s33[ix3(g.n1, g.n2, k, j, i)];
  C aij = csub<P>(cmul<P>(csub<P>(cdivs<P>(csub<P>(t1, t2), g.d1[i], g.r1[i]), cdivs<P>(csub<P>(t3, t4), g.d2[j], g.r2[j])),
                          sc.iwmu),
                  rmul<P>(sg, own));
  typename P::R gg = geo<P>(g.d1s[i], g.d1s[i - 1], g.d1[i], g.d2s[j], g.d2s[j - 1], g.d2[j]);
  typename P::R vol = g.fvm ? P::mul(P::mul(g.d1s[i], g.d2[j]), g.d3[k]) : 0;  // Ex's volume (fdfd.c:417)
  return fin<P>(b, aij, gg, sg, vol, sc, g.fvm);
}

template <class C> __device__ __forceinline__ C shfl_up(C v, int d)
{
  C r;
  r.x = __shfl_up_sync(0xffffffffu, v.x, d);
  r.y = __shfl_up_sync(0xffffffffu, v.y, d);
  return r;
}

constexpr int XV = 4;  // i per lane in the Ex sweep
constexpr int YV = 4;  // i per macro-step in the Ey/Ez sweeps

}  // namespace

// Ex sweep: lanes = k rows, march j, XV consecutive i per lane.
template <class P, bool FWD>
__global__ void __launch_bounds__(128) k_sweep_x(SweepP<P> s)
{
  typedef typename P::C C;
  const int lane = threadIdx.x & 31;
  const int grp = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int slot = blockIdx.z;
  const int sys = s.sys_list ? s.sys_list[slot] : slot;
  const GridP<P>& g = s.g;
  const int n1 = g.n1, n2 = g.n2, nK = s.nK;
  const int i0 = grp * XV;
  if (i0 >= n1) return;  // whole warp leaves together
  const View<P> V = view_of<P>(s, slot, sys);
  const SysScal<P> sc = s.scal[sys];
  const C z = czero<P>();
  const int R = nK - 1, M = n2 - 1;  // rows k = 1..R, march j = 1..M
  for (int rb = 0; rb < R; rb += 32) {
    const int rr = rb + lane;                          // row ordinal in sweep order
    const bool rowok = rr < R;
    const int k = FWD ? 1 + rr : R - rr;
    const int kprev = FWD ? k - 1 : k + 1;            // the row this row depends on
    C res[XV], own[XV];
#pragma unroll
    for (int q = 0; q < XV; q++) res[q] = own[q] = z;  // own: Ex(k, j-/+1) new; boundary rows are 0
    for (int T = 0; T < M + 31; T++) {
      C nb[XV];
#pragma unroll
      for (int q = 0; q < XV; q++) nb[q] = shfl_up(res[q], 1);
      const int c = T - lane;
      if (rowok && c >= 0 && c < M) {
        const int j = FWD ? 1 + c : M - c;
        if (lane == 0) {
#pragma unroll
          for (int q = 0; q < XV; q++) nb[q] = (i0 + q < n1) ? V.ld(0, kprev, j, i0 + q) : z;
        }
#pragma unroll
        for (int q = 0; q < XV; q++) {
          const int i = i0 + q;
          if (i >= n1) { res[q] = z; continue; }
          C v;
          if (FWD) {
            v = upd_ex<P>(g, sc, k, j, i, z, z, z, z, z, own[q], z, nb[q], z, z, z, z, V.ldb(0, k, j, i));
          } else {
            v = upd_ex<P>(g, sc, k, j, i, V.ld(1, k, j, i + 1), V.ld(1, k, j, i), V.ld(1, k, j - 1, i + 1),
                          V.ld(1, k, j - 1, i), own[q], V.ld(0, k, j - 1, i), nb[q], V.ld(0, k - 1, j, i),
                          V.ld(2, k, j, i + 1), V.ld(2, k, j, i), V.ld(2, k - 1, j, i + 1), V.ld(2, k - 1, j, i),
                          V.ldb(0, k, j, i));
          }
          V.st(0, k, j, i, v);
          res[q] = v;
          own[q] = v;
        }
      } else {
#pragma unroll
        for (int q = 0; q < XV; q++) res[q] = z;
      }
    }
    __syncwarp();
  }
}

// Ey (COMP 1) / Ez (COMP 2) sweeps: march i in chunks of YV, lanes = rows.
template <class P, int COMP, bool FWD>
__global__ void __launch_bounds__(128) k_sweep_yz(SweepP<P> s)
{
  typedef typename P::C C;
  const int lane = threadIdx.x & 31;
  const int ind = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);  // j (Ey) or k (Ez)
  const int slot = blockIdx.z;
  const int sys = s.sys_list ? s.sys_list[slot] : slot;
  const GridP<P>& g = s.g;
  const int n1 = g.n1, n2 = g.n2, nK = s.nK;
  const int NI = COMP == 1 ? n2 : nK;
  if (ind >= NI) return;
  const View<P> V = view_of<P>(s, slot, sys);
  const SysScal<P> sc = s.scal[sys];
  const C z = czero<P>();
  const int R = COMP == 1 ? nK - 1 : n2 - 1;  // rows k (Ey) or j (Ez) = 1..R
  const int M = n1 - 1;                       // march i = 1..M
  const int NC = (M + YV - 1) / YV;
  for (int rb = 0; rb < R; rb += 32) {
    const int rr = rb + lane;
    const bool rowok = rr < R;
    const int r = FWD ? 1 + rr : R - rr;
    const int rprev = FWD ? r - 1 : r + 1;
    C res[YV];
#pragma unroll
    for (int q = 0; q < YV; q++) res[q] = z;
    C prev = z;  // own row at the previous march point (boundary i = 0 / n1 is 0)
    for (int T = 0; T < NC + 31; T++) {
      C nb[YV];
#pragma unroll
      for (int q = 0; q < YV; q++) nb[q] = shfl_up(res[q], 1);
      const int c = T - lane;
      if (rowok && c >= 0 && c < NC) {
#pragma unroll
        for (int q = 0; q < YV; q++) {
          const int m = c * YV + q;
          if (m >= M) { res[q] = z; continue; }
          const int i = FWD ? 1 + m : M - m;
          C nbq = nb[q];
          if (lane == 0) nbq = COMP == 1 ? V.ld(1, rprev, ind, i) : V.ld(2, ind, rprev, i);
          C v;
          if (COMP == 1) {  // Ey at (k=r, j=ind, i)
            const int k = r, j = ind;
            if (FWD)
              v = upd_ey<P>(g, sc, k, j, i, z, z, z, z, z, nbq, z, prev, V.ld(0, k, j + 1, i), V.ld(0, k, j, i),
                            V.ld(0, k, j + 1, i - 1), V.ld(0, k, j, i - 1), V.ldb(1, k, j, i));
            else
              v = upd_ey<P>(g, sc, k, j, i, V.ld(2, k, j + 1, i), V.ld(2, k, j, i), V.ld(2, k - 1, j + 1, i),
                            V.ld(2, k - 1, j, i), nbq, V.ld(1, k - 1, j, i), prev, V.ld(1, k, j, i - 1),
                            V.ld(0, k, j + 1, i), V.ld(0, k, j, i), V.ld(0, k, j + 1, i - 1), V.ld(0, k, j, i - 1),
                            V.ldb(1, k, j, i));
            V.st(1, k, j, i, v);
          } else {  // Ez at (k=ind, j=r, i)
            const int k = ind, j = r;
            if (FWD)
              v = upd_ez<P>(g, sc, k, j, i, V.ld(0, k + 1, j, i), V.ld(0, k, j, i), V.ld(0, k + 1, j, i - 1),
                            V.ld(0, k, j, i - 1), z, prev, z, nbq, V.ld(1, k + 1, j, i), V.ld(1, k, j, i),
                            V.ld(1, k + 1, j - 1, i), V.ld(1, k, j - 1, i), V.ldb(2, k, j, i));
            else
              v = upd_ez<P>(g, sc, k, j, i, V.ld(0, k + 1, j, i), V.ld(0, k, j, i), V.ld(0, k + 1, j, i - 1),
                            V.ld(0, k, j, i - 1), prev, V.ld(2, k, j, i - 1), nbq, V.ld(2, k, j - 1, i),
                            V.ld(1, k + 1, j, i), V.ld(1, k, j, i), V.ld(1, k + 1, j - 1, i), V.ld(1, k, j - 1, i),
                            V.ldb(2, k, j, i));
            V.st(2, k, j, i, v);
          }
          res[q] = v;
          prev = v;
        }
      } else {
#pragma unroll
        for (int q = 0; q < YV; q++) res[q] = z;
      }
    }
    __syncwarp();
  }
}

template <class P>
void launch_sweep_pipelined(const SweepP<P>& s, int comp, bool fwd, int nslot, cudaStream_t st)
{
  const int WPB = 4;  // warps per block
  if (comp == 0) {
    const int ngrp = (s.g.n1 + XV - 1) / XV;
    dim3 grd((ngrp + WPB - 1) / WPB, 1, nslot);
    if (fwd) count_launch(), k_sweep_x<P, true><<<grd, 32 * WPB, 0, st>>>(s);
    else count_launch(), k_sweep_x<P, false><<<grd, 32 * WPB, 0, st>>>(s);
  } else {
    const int NI = comp == 1 ? s.g.n2 : s.nK;
    dim3 grd((NI + WPB - 1) / WPB, 1, nslot);
    if (comp == 1) {
      if (fwd) count_launch(), k_sweep_yz<P, 1, true><<<grd, 32 * WPB, 0, st>>>(s);
      else count_launch(), k_sweep_yz<P, 1, false><<<grd, 32 * WPB, 0, st>>>(s);
    } else {
      if (fwd) count_launch(), k_sweep_yz<P, 2, true><<<grd, 32 * WPB, 0, st>>>(s);
      else count_launch(), k_sweep_yz<P, 2, false><<<grd, 32 * WPB, 0, st>>>(s);
    }
  }
}

template void launch_sweep_pipelined<F64>(const SweepP<F64>&, int, bool, int, cudaStream_t);
template void launch_sweep_pipelined<F32>(const SweepP<F32>&, int, bool, int, cudaStream_t);

}  // namespace csem
