// LU-SGS component sweeps as lockstep row pipelines: one launch per sweep.
//
// A sweep updates one field component in the reference's lexicographic Gauss-Seidel
// order (fdfd.c:347-503). In the coupled plane (r, m) a point depends on (r-1, m) and
// (r, m-1) (forward; (r+1, m), (r, m+1) backward); the third axis is independent:
//   Ex: rows r = k, march m = j, independent i  (VW consecutive i per lane)
//   Ey: rows r = k, march m = i, independent j  (VW consecutive i per step)
//   Ez: rows r = j, march m = i, independent k  (VW consecutive i per step)
// One CTA owns one independent line of one system and gives every row of the sweep a
// thread: thread t takes the t-th row in sweep order. All rows advance together, one
// march step per iteration, skewed by one step per row: at step T row t works at march
// position T - t, so the row before it finished that position at step T - 1. That value
// arrives by warp shuffle, or through shared memory from the last lane of the previous
// warp (one __syncthreads per step). The own-row dependency stays in registers and the
// sweep's first row depends on the boundary, which is zero. A sweep takes
// (march positions + rows - 1) steps.
//
// Inside a step a thread first issues every load it needs for its VW points (none of
// them is written in this step), then computes and stores, so one memory round trip
// is exposed per step instead of one per point.
//
// Every point is evaluated with the same operations, operands and order as the
// reference (the F64 instantiation is bit-identical to it and to the one-launch-per-
// diagonal kernels of k_lusgs.cu); F32 uses reciprocal spacings and a reciprocal-based
// complex quotient.
#include "csem_cuda.cuh"
#include "engine.h"

namespace csem {

namespace {

constexpr int MAXROWS = 256;  // rows of one sweep handled by one CTA (a thread each)

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

// (1/a0 + 1/a1)/A + (1/b0 + 1/b1)/B; F64 divides exactly, F32 uses the reciprocals
template <class P>
__device__ __forceinline__ typename P::R geo(typename P::R a0, typename P::R ra0, typename P::R a1,
                                             typename P::R ra1, typename P::R A, typename P::R rA, typename P::R b0,
                                             typename P::R rb0, typename P::R b1, typename P::R rb1, typename P::R B,
                                             typename P::R rB)
{
  typedef typename P::R R;
  const R one = 1;
  return P::add(P::divs(P::add(P::divs(one, a0, ra0), P::divs(one, a1, ra1)), A, rA),
                P::divs(P::add(P::divs(one, b0, rb0), P::divs(one, b1, rb1)), B, rB));
}

// (b - aij) / aii: Smith's quotient in F64, a * conj(d) / |d|^2 in F32
template <class P>
__device__ __forceinline__ typename P::C quot(typename P::C a, typename P::C d)
{
  if constexpr (P::exact) {
    return cdiv<P>(a, d);
  } else {
    const float inv = __frcp_rn(d.x * d.x + d.y * d.y);
    return P::mk((a.x * d.x + a.y * d.y) * inv, (a.y * d.x - a.x * d.y) * inv);
  }
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
  return quot<P>(csub<P>(b, aij), aii);
}

// --- per-point updates in the reference's operation order; the component being
// updated is zero at its own point while its row is evaluated (fdfd.c:357,383,409)

// Ex at (k,j,i): fdfd.c:358-369
template <class P>
__device__ __forceinline__ typename P::C upd_ex(const GridP<P>& g, const SysScal<P>& sc, int k, int j, int i,
                                                typename P::C eyA, typename P::C eyB, typename P::C eyC,
                                                typename P::C eyD, typename P::C exjp, typename P::C exjm,
                                                typename P::C exkp, typename P::C exkm, typename P::C ezA,
                                                typename P::C ezB, typename P::C ezC, typename P::C ezD,
                                                typename P::C b, typename P::R sg)
{
  typedef typename P::C C;
  const C own = czero<P>();
  C t1 = csub<P>(cdivs<P>(csub<P>(eyA, eyB), g.d1s[i], g.r1s[i]), cdivs<P>(csub<P>(exjp, own), g.d2s[j], g.r2s[j]));
  C t2 = csub<P>(cdivs<P>(csub<P>(eyC, eyD), g.d1s[i], g.r1s[i]), cdivs<P>(csub<P>(own, exjm), g.d2s[j - 1], g.r2s[j - 1]));
  C t3 = csub<P>(cdivs<P>(csub<P>(exkp, own), g.d3s[k], g.r3s[k]), cdivs<P>(csub<P>(ezA, ezB), g.d1s[i], g.r1s[i]));
  C t4 = csub<P>(cdivs<P>(csub<P>(own, exkm), g.d3s[k - 1], g.r3s[k - 1]), cdivs<P>(csub<P>(ezC, ezD), g.d1s[i], g.r1s[i]));
  C aij = csub<P>(cmul<P>(csub<P>(cdivs<P>(csub<P>(t1, t2), g.d2[j], g.r2[j]), cdivs<P>(csub<P>(t3, t4), g.d3[k], g.r3[k])),
                          sc.iwmu),
                  rmul<P>(sg, own));
  typename P::R gg = geo<P>(g.d2s[j], g.r2s[j], g.d2s[j - 1], g.r2s[j - 1], g.d2[j], g.r2[j], g.d3s[k], g.r3s[k],
                            g.d3s[k - 1], g.r3s[k - 1], g.d3[k], g.r3[k]);
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
                                                typename P::C b, typename P::R sg)
{
  typedef typename P::C C;
  const C own = czero<P>();
  C t1 = csub<P>(cdivs<P>(csub<P>(ezA, ezB), g.d2s[j], g.r2s[j]), cdivs<P>(csub<P>(eykp, own), g.d3s[k], g.r3s[k]));
  C t2 = csub<P>(cdivs<P>(csub<P>(ezC, ezD), g.d2s[j], g.r2s[j]), cdivs<P>(csub<P>(own, eykm), g.d3s[k - 1], g.r3s[k - 1]));
  C t3 = csub<P>(cdivs<P>(csub<P>(eyip, own), g.d1s[i], g.r1s[i]), cdivs<P>(csub<P>(exA, exB), g.d2s[j], g.r2s[j]));
  C t4 = csub<P>(cdivs<P>(csub<P>(own, eyim), g.d1s[i - 1], g.r1s[i - 1]), cdivs<P>(csub<P>(exC, exD), g.d2s[j], g.r2s[j]));
  C aij = csub<P>(cmul<P>(csub<P>(cdivs<P>(csub<P>(t1, t2), g.d3[k], g.r3[k]), cdivs<P>(csub<P>(t3, t4), g.d1[i], g.r1[i])),
                          sc.iwmu),
                  rmul<P>(sg, own));
  typename P::R gg = geo<P>(g.d3s[k], g.r3s[k], g.d3s[k - 1], g.r3s[k - 1], g.d3[k], g.r3[k], g.d1s[i], g.r1s[i],
                            g.d1s[i - 1], g.r1s[i - 1], g.d1[i], g.r1[i]);
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
                                                typename P::C b, typename P::R sg)
{
  typedef typename P::C C;
  const C own = czero<P>();
  C t1 = csub<P>(cdivs<P>(csub<P>(exA, exB), g.d3s[k], g.r3s[k]), cdivs<P>(csub<P>(ezip, own), g.d1s[i], g.r1s[i]));
  C t2 = csub<P>(cdivs<P>(csub<P>(exC, exD), g.d3s[k], g.r3s[k]), cdivs<P>(csub<P>(own, ezim), g.d1s[i - 1], g.r1s[i - 1]));
  C t3 = csub<P>(cdivs<P>(csub<P>(ezjp, own), g.d2s[j], g.r2s[j]), cdivs<P>(csub<P>(eyA, eyB), g.d3s[k], g.r3s[k]));
  C t4 = csub<P>(cdivs<P>(csub<P>(own, ezjm), g.d2s[j - 1], g.r2s[j - 1]), cdivs<P>(csub<P>(eyC, eyD), g.d3s[k], g.r3s[k]));
  C aij = csub<P>(cmul<P>(csub<P>(cdivs<P>(csub<P>(t1, t2), g.d1[i], g.r1[i]), cdivs<P>(csub<P>(t3, t4), g.d2[j], g.r2[j])),
                          sc.iwmu),
                  rmul<P>(sg, own));
  typename P::R gg = geo<P>(g.d1s[i], g.r1s[i], g.d1s[i - 1], g.r1s[i - 1], g.d1[i], g.r1[i], g.d2s[j], g.r2s[j],
                            g.d2s[j - 1], g.r2s[j - 1], g.d2[j], g.r2[j]);
  typename P::R vol = g.fvm ? P::mul(P::mul(g.d1s[i], g.d2[j]), g.d3[k]) : 0;  // Ex's volume (fdfd.c:417)
  return fin<P>(b, aij, gg, sg, vol, sc, g.fvm);
}

template <class C> __device__ __forceinline__ C shfl_up(C v)
{
  C r;
  r.x = __shfl_up_sync(0xffffffffu, v.x, 1);
  r.y = __shfl_up_sync(0xffffffffu, v.y, 1);
  return r;
}

// Value the row before this thread's row produced at the previous step: a shuffle from
// the previous lane, or shared memory for lane 0 (written by the previous warp's last
// lane before the barrier); the sweep's first row reads the zero boundary.
template <int VW, class C>
__device__ __forceinline__ void neighbours(const C (&res)[VW], C (&nb)[VW], const C (*hand)[2][VW], int T)
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
      if (w > 0 && T > 0) v = hand[w - 1][(T - 1) & 1][q];
      nb[q] = v;
    }
  }
}

template <int VW, class C>
__device__ __forceinline__ void hand_over(const C (&res)[VW], C (*hand)[2][VW], int T)
{
  if ((threadIdx.x & 31) == 31) {
#pragma unroll
    for (int q = 0; q < VW; q++) hand[threadIdx.x >> 5][T & 1][q] = res[q];
  }
  __syncthreads();
}

}  // namespace

// Ex sweep: rows k, march j, VW consecutive i per thread. grid (i groups, systems)
template <class P, bool FWD, int VW>
__global__ void __launch_bounds__(MAXROWS) k_sweep_ex(SweepP<P> s)
{
  typedef typename P::C C;
  typedef typename P::R R;
  __shared__ C hand[MAXROWS / 32][2][VW];
  const int slot = blockIdx.y;
  const int sys = s.sys_list ? s.sys_list[slot] : slot;
  const GridP<P>& g = s.g;
  const int n1 = g.n1, nK = s.nK;
  const int i0 = blockIdx.x * VW;
  const View<P> V = view_of<P>(s, slot, sys);
  const SysScal<P> sc = s.scal[sys];
  const C z = czero<P>();
  const int R_ = nK - 1, M = g.n2 - 1;  // rows k = 1..R_, march j = 1..M
  const int rr = threadIdx.x;
  const bool rowok = rr < R_;
  const int k = FWD ? 1 + rr : R_ - rr;
  C res[VW];
#pragma unroll
  for (int q = 0; q < VW; q++) res[q] = z;
  for (int T = 0; T < M + R_ - 1; T++) {
    C nb[VW];
    neighbours<VW, C>(res, nb, hand, T);
    const int c = T - rr;
    if (rowok && c >= 0 && c < M) {
      const int j = FWD ? 1 + c : M - c;
      C exjm[VW], exkm[VW], b[VW], eyA[VW], eyB[VW], eyC[VW], eyD[VW], ezA[VW], ezB[VW], ezC[VW], ezD[VW];
      R sg[VW];
#pragma unroll
      for (int q = 0; q < VW; q++) {  // loads: nothing read here is written in this step
        const int i = i0 + q;
        if (i < n1) {
          b[q] = V.ldb(0, k, j, i);
          sg[q] = g.s11[ix1(g.n1, g.n2, k, j, i)];
          if (!FWD) {
            exjm[q] = V.ld(0, k, j - 1, i);
            exkm[q] = V.ld(0, k - 1, j, i);
            eyA[q] = V.ld(1, k, j, i + 1);
            eyB[q] = V.ld(1, k, j, i);
            eyC[q] = V.ld(1, k, j - 1, i + 1);
            eyD[q] = V.ld(1, k, j - 1, i);
            ezA[q] = V.ld(2, k, j, i + 1);
            ezB[q] = V.ld(2, k, j, i);
            ezC[q] = V.ld(2, k - 1, j, i + 1);
            ezD[q] = V.ld(2, k - 1, j, i);
          }
        }
      }
#pragma unroll
      for (int q = 0; q < VW; q++) {
        const int i = i0 + q;
        if (i >= n1) {
          res[q] = z;
          continue;
        }
        C v;
        if (FWD)  // own row: j-1 is the previous step's value; row k-1 is the neighbour
          v = upd_ex<P>(g, sc, k, j, i, z, z, z, z, z, res[q], z, nb[q], z, z, z, z, b[q], sg[q]);
        else      // own row: j+1 is the previous step's value; row k+1 is the neighbour
          v = upd_ex<P>(g, sc, k, j, i, eyA[q], eyB[q], eyC[q], eyD[q], res[q], exjm[q], nb[q], exkm[q], ezA[q],
                        ezB[q], ezC[q], ezD[q], b[q], sg[q]);
        *V.at(0, k, j, i) = v;
        res[q] = v;
      }
    } else {
#pragma unroll
      for (int q = 0; q < VW; q++) res[q] = z;
    }
    hand_over<VW, C>(res, hand, T);
  }
}

// Ey (COMP 1: line j, rows k) / Ez (COMP 2: line k, rows j) sweeps, march i in chunks
// of VW. grid (lines, systems)
template <class P, int COMP, bool FWD, int VW>
__global__ void __launch_bounds__(MAXROWS) k_sweep_eyz(SweepP<P> s)
{
  typedef typename P::C C;
  typedef typename P::R R;
  __shared__ C hand[MAXROWS / 32][2][VW];
  const int slot = blockIdx.y;
  const int sys = s.sys_list ? s.sys_list[slot] : slot;
  const GridP<P>& g = s.g;
  const int n1 = g.n1, n2 = g.n2, nK = s.nK;
  const int line = blockIdx.x;  // j (Ey) or k (Ez)
  const View<P> V = view_of<P>(s, slot, sys);
  const SysScal<P> sc = s.scal[sys];
  const C z = czero<P>();
  const int R_ = COMP == 1 ? nK - 1 : n2 - 1;  // rows k (Ey) or j (Ez) = 1..R_
  const int M = n1 - 1;                         // march i = 1..M
  const int NC = (M + VW - 1) / VW;
  const int rr = threadIdx.x;
  const bool rowok = rr < R_;
  const int r = FWD ? 1 + rr : R_ - rr;
  const int k = COMP == 1 ? r : line;
  const int j = COMP == 1 ? line : r;
  C res[VW];
#pragma unroll
  for (int q = 0; q < VW; q++) res[q] = z;
  for (int T = 0; T < NC + R_ - 1; T++) {
    C nb[VW];
    neighbours<VW, C>(res, nb, hand, T);
    const int c = T - rr;
    if (rowok && c >= 0 && c < NC) {
      C prev = c > 0 ? res[VW - 1] : z;  // own row at the previous march position
      C b[VW], xA[VW], xB[VW], xC[VW], xD[VW], yA[VW], yB[VW], yC[VW], yD[VW], own2[VW];
      R sg[VW];
#pragma unroll
      for (int q = 0; q < VW; q++) {  // loads
        const int m = c * VW + q;
        if (m < M) {
          const int i = FWD ? 1 + m : M - m;
          if (COMP == 1) {
            b[q] = V.ldb(1, k, j, i);
            sg[q] = g.s22[ix2(g.n1, g.n2, k, j, i)];
            xA[q] = V.ld(0, k, j + 1, i);
            xB[q] = V.ld(0, k, j, i);
            xC[q] = V.ld(0, k, j + 1, i - 1);
            xD[q] = V.ld(0, k, j, i - 1);
            if (!FWD) {
              yA[q] = V.ld(2, k, j + 1, i);
              yB[q] = V.ld(2, k, j, i);
              yC[q] = V.ld(2, k - 1, j + 1, i);
              yD[q] = V.ld(2, k - 1, j, i);
              own2[q] = V.ld(1, k, j, i - 1);  // Ey(i-1): not yet swept backward
              // Ey(k-1): the next row's old value
            }
          } else {
            b[q] = V.ldb(2, k, j, i);
            sg[q] = g.s33[ix3(g.n1, g.n2, k, j, i)];
            xA[q] = V.ld(0, k + 1, j, i);
            xB[q] = V.ld(0, k, j, i);
            xC[q] = V.ld(0, k + 1, j, i - 1);
            xD[q] = V.ld(0, k, j, i - 1);
            yA[q] = V.ld(1, k + 1, j, i);
            yB[q] = V.ld(1, k, j, i);
            yC[q] = V.ld(1, k + 1, j - 1, i);
            yD[q] = V.ld(1, k, j - 1, i);
            if (!FWD) own2[q] = V.ld(2, k, j, i - 1);  // Ez(i-1): not yet swept backward
          }
        }
      }
      C rowold[VW];  // backward: the next row's forward value at this position
      if (!FWD) {
#pragma unroll
        for (int q = 0; q < VW; q++) {
          const int m = c * VW + q;
          if (m < M) {
            const int i = M - m;
            rowold[q] = COMP == 1 ? V.ld(1, k - 1, j, i) : V.ld(2, k, j - 1, i);
          }
        }
      }
#pragma unroll
      for (int q = 0; q < VW; q++) {
        const int m = c * VW + q;
        if (m >= M) {
          res[q] = z;
          continue;
        }
        const int i = FWD ? 1 + m : M - m;
        C v;
        if (COMP == 1) {
          if (FWD)
            v = upd_ey<P>(g, sc, k, j, i, z, z, z, z, z, nb[q], z, prev, xA[q], xB[q], xC[q], xD[q], b[q], sg[q]);
          else
            v = upd_ey<P>(g, sc, k, j, i, yA[q], yB[q], yC[q], yD[q], nb[q], rowold[q], prev, own2[q], xA[q], xB[q],
                          xC[q], xD[q], b[q], sg[q]);
          *V.at(1, k, j, i) = v;
        } else {
          if (FWD)
            v = upd_ez<P>(g, sc, k, j, i, xA[q], xB[q], xC[q], xD[q], z, prev, z, nb[q], yA[q], yB[q], yC[q], yD[q],
                          b[q], sg[q]);
          else
            v = upd_ez<P>(g, sc, k, j, i, xA[q], xB[q], xC[q], xD[q], prev, own2[q], nb[q], rowold[q], yA[q], yB[q],
                          yC[q], yD[q], b[q], sg[q]);
          *V.at(2, k, j, i) = v;
        }
        res[q] = v;
        prev = v;
      }
    } else {
#pragma unroll
      for (int q = 0; q < VW; q++) res[q] = z;
    }
    hand_over<VW, C>(res, hand, T);
  }
}

bool sweep_pipelined_fits(int comp, int n1, int n2, int nK)
{
  const int rows = comp == 2 ? n2 - 1 : nK - 1;
  return rows >= 1 && rows <= MAXROWS && n1 >= 2 && n2 >= 2;
}

template <class P>
void launch_sweep_pipelined(const SweepP<P>& s, int comp, bool fwd, int nslot, cudaStream_t st)
{
  // points per thread and step: 4 complex64 (one 32-byte sector), 2 complex128
  constexpr int VW = P::exact ? 2 : 4;
  const int n1 = s.g.n1, n2 = s.g.n2, nK = s.nK;
  const int rows = comp == 2 ? n2 - 1 : nK - 1;
  const int threads = (rows + 31) / 32 * 32;
  if (comp == 0) {
    dim3 grd((n1 + VW - 1) / VW, nslot);
    if (fwd) count_launch(), k_sweep_ex<P, true, VW><<<grd, threads, 0, st>>>(s);
    else count_launch(), k_sweep_ex<P, false, VW><<<grd, threads, 0, st>>>(s);
  } else if (comp == 1) {
    dim3 grd(n2, nslot);
    if (fwd) count_launch(), k_sweep_eyz<P, 1, true, VW><<<grd, threads, 0, st>>>(s);
    else count_launch(), k_sweep_eyz<P, 1, false, VW><<<grd, threads, 0, st>>>(s);
  } else {
    dim3 grd(nK, nslot);
    if (fwd) count_launch(), k_sweep_eyz<P, 2, true, VW><<<grd, threads, 0, st>>>(s);
    else count_launch(), k_sweep_eyz<P, 2, false, VW><<<grd, threads, 0, st>>>(s);
  }
}

template void launch_sweep_pipelined<F64>(const SweepP<F64>&, int, bool, int, cudaStream_t);
template void launch_sweep_pipelined<F32>(const SweepP<F32>&, int, bool, int, cudaStream_t);

}  // namespace csem
