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
// warp (pairwise named barriers between neighbouring warps). The own-row dependency stays
// in registers and the sweep's first row depends on the boundary, which is zero. A sweep
// takes (march positions + rows - 1) steps.
//
// Inside a step a thread first issues every load it needs for its VW points (none of
// them is written in this step), then computes and stores, so one memory round trip
// is exposed per step instead of one per point.
//
// In k_sweep_ex / k_sweep_eyz every point is evaluated with the same operations, operands
// and order as the reference (the complex128 instantiation is bit-identical to it and to
// the one-launch-per-diagonal kernels of k_lusgs.cu). complex64 runs k_sweep_ex32 /
// k_sweep_eyz32 below: the same update in linear form, with reciprocal spacings.
#include "csem_cuda.cuh"
#include "engine.h"
#include "k_sweep_common.cuh"

namespace csem {

using namespace sweep;

namespace {

// resident CTAs per SM the register budget is sized for, by points per thread and step
// (complex128 at one point per thread keeps 2, whose 128 registers avoid spilling)
template <class P, int VW> struct MinBlocks {
  static constexpr int value = VW >= 4 ? 1 : (VW == 2 ? 2 : (P::exact ? 2 : 3));
};
// Register budget of the sweeps: by default from MinBlocks for a full CTA; a build may set
// explicit caps per width (CSEM_SWEEP_MAXNREG1 / 2 / 4) for CTAs of up to 256 rows instead.
#if defined(CSEM_SWEEP_MAXNREG1) && defined(CSEM_SWEEP_MAXNREG2) && defined(CSEM_SWEEP_MAXNREG4)
template <int VW> struct RegCap {
  static constexpr int value = VW == 1 ? CSEM_SWEEP_MAXNREG1 : (VW == 2 ? CSEM_SWEEP_MAXNREG2 : CSEM_SWEEP_MAXNREG4);
};
#define CSEM_SWEEP_BOUNDS(VW, MAXR) __launch_bounds__(MAXR) __maxnreg__(MAXR > NB_ROWS ? 128 : RegCap<VW>::value)
#define CSEM_SWEEP_BOUNDS32(VW, MAXR) __launch_bounds__(MAXR) __maxnreg__(MAXR > NB_ROWS ? 128 : RegCap<VW>::value)
#else
#define CSEM_SWEEP_BOUNDS(VW, MAXR) __launch_bounds__(MAXR, MAXR > NB_ROWS ? 1 : MinBlocks<P, VW>::value)
#define CSEM_SWEEP_BOUNDS32(VW, MAXR) __launch_bounds__(MAXR, MAXR > NB_ROWS ? 1 : MinBlocks<F32, VW>::value)
#endif

// (1/a.ds + 1/a.dsm)/a.d + (1/b.ds + 1/b.dsm)/b.d; F64 divides exactly, F32 multiplies
// by the reciprocals
template <class P>
__device__ __forceinline__ typename P::R geo(const Ax<P>& a, const Ax<P>& b)
{
  typedef typename P::R R;
  const R one = 1;
  return P::add(P::divs(P::add(P::divs(one, a.ds, a.rs), P::divs(one, a.dsm, a.rsm)), a.d, a.r),
                P::divs(P::add(P::divs(one, b.ds, b.rs), P::divs(one, b.dsm, b.rsm)), b.d, b.r));
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
// updated is zero at its own point while its row is evaluated (fdfd.c:357,383,409).
// X, Y, Z are the spacings at the point's i, j, k.

// Ex at (k,j,i): fdfd.c:358-369
template <class P>
__device__ __forceinline__ typename P::C upd_ex(const SysScal<P>& sc, int fvm, const Ax<P>& X, const Ax<P>& Y,
                                                const Ax<P>& Z, typename P::C eyA, typename P::C eyB,
                                                typename P::C eyC, typename P::C eyD, typename P::C exjp,
                                                typename P::C exjm, typename P::C exkp, typename P::C exkm,
                                                typename P::C ezA, typename P::C ezB, typename P::C ezC,
                                                typename P::C ezD, typename P::C b, typename P::R sg)
{
  typedef typename P::C C;
  const C own = czero<P>();
  C t1 = csub<P>(cdivs<P>(csub<P>(eyA, eyB), X.ds, X.rs), cdivs<P>(csub<P>(exjp, own), Y.ds, Y.rs));
  C t2 = csub<P>(cdivs<P>(csub<P>(eyC, eyD), X.ds, X.rs), cdivs<P>(csub<P>(own, exjm), Y.dsm, Y.rsm));
  C t3 = csub<P>(cdivs<P>(csub<P>(exkp, own), Z.ds, Z.rs), cdivs<P>(csub<P>(ezA, ezB), X.ds, X.rs));
  C t4 = csub<P>(cdivs<P>(csub<P>(own, exkm), Z.dsm, Z.rsm), cdivs<P>(csub<P>(ezC, ezD), X.ds, X.rs));
  C aij = csub<P>(cmul<P>(csub<P>(cdivs<P>(csub<P>(t1, t2), Y.d, Y.r), cdivs<P>(csub<P>(t3, t4), Z.d, Z.r)), sc.iwmu),
                  rmul<P>(sg, own));
  typename P::R vol = fvm ? P::mul(P::mul(X.ds, Y.d), Z.d) : 0;
  return fin<P>(b, aij, geo<P>(Y, Z), sg, vol, sc, fvm);
}

// Ey at (k,j,i): fdfd.c:384-395
template <class P>
__device__ __forceinline__ typename P::C upd_ey(const SysScal<P>& sc, int fvm, const Ax<P>& X, const Ax<P>& Y,
                                                const Ax<P>& Z, typename P::C ezA, typename P::C ezB,
                                                typename P::C ezC, typename P::C ezD, typename P::C eykp,
                                                typename P::C eykm, typename P::C eyip, typename P::C eyim,
                                                typename P::C exA, typename P::C exB, typename P::C exC,
                                                typename P::C exD, typename P::C b, typename P::R sg)
{
  typedef typename P::C C;
  const C own = czero<P>();
  C t1 = csub<P>(cdivs<P>(csub<P>(ezA, ezB), Y.ds, Y.rs), cdivs<P>(csub<P>(eykp, own), Z.ds, Z.rs));
  C t2 = csub<P>(cdivs<P>(csub<P>(ezC, ezD), Y.ds, Y.rs), cdivs<P>(csub<P>(own, eykm), Z.dsm, Z.rsm));
  C t3 = csub<P>(cdivs<P>(csub<P>(eyip, own), X.ds, X.rs), cdivs<P>(csub<P>(exA, exB), Y.ds, Y.rs));
  C t4 = csub<P>(cdivs<P>(csub<P>(own, eyim), X.dsm, X.rsm), cdivs<P>(csub<P>(exC, exD), Y.ds, Y.rs));
  C aij = csub<P>(cmul<P>(csub<P>(cdivs<P>(csub<P>(t1, t2), Z.d, Z.r), cdivs<P>(csub<P>(t3, t4), X.d, X.r)), sc.iwmu),
                  rmul<P>(sg, own));
  typename P::R vol = fvm ? P::mul(P::mul(X.ds, Y.d), Z.d) : 0;  // Ex's volume (fdfd.c:391)
  return fin<P>(b, aij, geo<P>(Z, X), sg, vol, sc, fvm);
}

// Ez at (k,j,i): fdfd.c:410-421
template <class P>
__device__ __forceinline__ typename P::C upd_ez(const SysScal<P>& sc, int fvm, const Ax<P>& X, const Ax<P>& Y,
                                                const Ax<P>& Z, typename P::C exA, typename P::C exB,
                                                typename P::C exC, typename P::C exD, typename P::C ezip,
                                                typename P::C ezim, typename P::C ezjp, typename P::C ezjm,
                                                typename P::C eyA, typename P::C eyB, typename P::C eyC,
                                                typename P::C eyD, typename P::C b, typename P::R sg)
{
  typedef typename P::C C;
  const C own = czero<P>();
  C t1 = csub<P>(cdivs<P>(csub<P>(exA, exB), Z.ds, Z.rs), cdivs<P>(csub<P>(ezip, own), X.ds, X.rs));
  C t2 = csub<P>(cdivs<P>(csub<P>(exC, exD), Z.ds, Z.rs), cdivs<P>(csub<P>(own, ezim), X.dsm, X.rsm));
  C t3 = csub<P>(cdivs<P>(csub<P>(ezjp, own), Y.ds, Y.rs), cdivs<P>(csub<P>(eyA, eyB), Z.ds, Z.rs));
  C t4 = csub<P>(cdivs<P>(csub<P>(own, ezjm), Y.dsm, Y.rsm), cdivs<P>(csub<P>(eyC, eyD), Z.ds, Z.rs));
  C aij = csub<P>(cmul<P>(csub<P>(cdivs<P>(csub<P>(t1, t2), X.d, X.r), cdivs<P>(csub<P>(t3, t4), Y.d, Y.r)), sc.iwmu),
                  rmul<P>(sg, own));
  typename P::R vol = fvm ? P::mul(P::mul(X.ds, Y.d), Z.d) : 0;  // Ex's volume (fdfd.c:417)
  return fin<P>(b, aij, geo<P>(X, Y), sg, vol, sc, fvm);
}

}  // namespace

// Ex sweep: rows k, march j, VW consecutive i per thread. grid (i groups, systems)
template <class P, bool FWD, int VW, int MAXR>
__global__ void CSEM_SWEEP_BOUNDS(VW, MAXR) k_sweep_ex(SweepP<P> s)
{
  typedef typename P::C C;
  typedef typename P::R R;
  __shared__ HandOff<VW, C, (MAXR <= NB_ROWS)> hand;
  const int slot = blockIdx.y;
  const int sys = s.sys_list ? s.sys_list[slot] : slot;
  const GridP<P>& g = s.g;
  const int n1 = g.n1, n2 = g.n2, nK = s.nK;
  const int i0 = blockIdx.x * VW;
  const View<P> V = view_of<P>(s, slot, sys);
  const SysScal<P> sc = s.scal[sys];
  const C z = czero<P>();
  const int R_ = nK - 1, M = n2 - 1;  // rows k = 1..R_, march j = 1..M
  const int rr = threadIdx.x;
  const bool rowok = rr < R_;
  const int k = FWD ? 1 + rr : R_ - rr;
  // spacings fixed for this thread: k (row) and the VW i's
  const Ax<P> Z = rowok ? axis<P>(g.d3, g.d3s, g.r3, g.r3s, k) : Ax<P>{};
  Ax<P> X[VW];
#pragma unroll
  for (int q = 0; q < VW; q++)
    X[q] = i0 + q < n1 ? axis_at<P>(g.d1, g.d1s, g.r1, g.r1s, i0 + q) : Ax<P>{};
  // planes this thread reads and writes, offset to its first i; row j is j * row_len
  C* ex0 = nullptr;
  const C *ex1 = nullptr, *ey0 = nullptr, *ez0 = nullptr, *ez1 = nullptr, *bb = nullptr;
  const R* sg0 = nullptr;
  if (rowok) {
    ex0 = V.row(0, k, 0) + i0;
    ex1 = V.row(0, k - 1, 0) + i0;
    ey0 = V.row(1, k, 0) + i0;
    ez0 = V.row(2, k, 0) + i0;
    ez1 = V.row(2, k - 1, 0) + i0;
    bb = V.brow(0, k, 0);
    if (bb) bb += i0;
    sg0 = g.s11 + ix1(n1, n2, k, 0, i0);
  }
  const int L1 = n1 + 1;
  C res[VW];
#pragma unroll
  for (int q = 0; q < VW; q++) res[q] = z;
  for (int T = 0; T < M + R_ - 1; T++) {
    C nb[VW];
    hand.get(res, nb, T);
    const int c = T - rr;
    if (rowok && c >= 0 && c < M) {
      const int j = FWD ? 1 + c : M - c;
      const Ax<P> Y = axis<P>(g.d2, g.d2s, g.r2, g.r2s, j);
      const int ox = j * n1, oy = j * L1;
      C exjm[VW], exkm[VW], b[VW], eyA[VW], eyB[VW], eyC[VW], eyD[VW], ezA[VW], ezB[VW], ezC[VW], ezD[VW];
      R sg[VW];
#pragma unroll
      for (int q = 0; q < VW; q++) {  // loads: nothing read here is written in this step
        if (i0 + q < n1) {
          b[q] = bb ? ro(bb + ox + q) : z;
          sg[q] = ro(sg0 + ox + q);
          if (!FWD) {
            exjm[q] = ex0[ox - n1 + q];
            exkm[q] = ex1[ox + q];
            eyA[q] = ro(ey0 + oy + q + 1);
            eyB[q] = ro(ey0 + oy + q);
            eyC[q] = ro(ey0 + oy - L1 + q + 1);
            eyD[q] = ro(ey0 + oy - L1 + q);
            ezA[q] = ro(ez0 + oy + q + 1);
            ezB[q] = ro(ez0 + oy + q);
            ezC[q] = ro(ez1 + oy + q + 1);
            ezD[q] = ro(ez1 + oy + q);
          }
        }
      }
#pragma unroll
      for (int q = 0; q < VW; q++) {
        if (i0 + q >= n1) {
          res[q] = z;
          continue;
        }
        C v;
        if (FWD)  // own row: j-1 is the previous step's value; row k-1 is the neighbour
          v = upd_ex<P>(sc, g.fvm, X[q], Y, Z, z, z, z, z, z, res[q], z, nb[q], z, z, z, z, b[q], sg[q]);
        else      // own row: j+1 is the previous step's value; row k+1 is the neighbour
          v = upd_ex<P>(sc, g.fvm, X[q], Y, Z, eyA[q], eyB[q], eyC[q], eyD[q], res[q], exjm[q], nb[q], exkm[q],
                        ezA[q], ezB[q], ezC[q], ezD[q], b[q], sg[q]);
        ex0[ox + q] = v;
        res[q] = v;
      }
    } else {
#pragma unroll
      for (int q = 0; q < VW; q++) res[q] = z;
    }
    hand.put(res, T);
  }
  hand.finish(M + R_ - 1);
}

// Ey (COMP 1: line j, rows k) / Ez (COMP 2: line k, rows j) sweeps, march i in chunks
// of VW. grid (lines, systems)
template <class P, int COMP, bool FWD, int VW, int MAXR>
__global__ void CSEM_SWEEP_BOUNDS(VW, MAXR) k_sweep_eyz(SweepP<P> s)
{
  typedef typename P::C C;
  typedef typename P::R R;
  __shared__ HandOff<VW, C, (MAXR <= NB_ROWS)> hand;
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
  // spacings fixed for this thread: the line's and the row's
  Ax<P> Y, Z;
  if (COMP == 1) {
    Y = axis_at<P>(g.d2, g.d2s, g.r2, g.r2s, j);
    Z = rowok ? axis<P>(g.d3, g.d3s, g.r3, g.r3s, k) : Ax<P>{};
  } else {
    Y = rowok ? axis<P>(g.d2, g.d2s, g.r2, g.r2s, j) : Ax<P>{};
    Z = axis_at<P>(g.d3, g.d3s, g.r3, g.r3s, k);
  }
  // the rows this thread reads and writes (element i is row[i])
  C* own = nullptr;                                 // this component at (k, j)
  const C *nxt = nullptr;                           // this component on the next row
  const C *xa = nullptr, *xb = nullptr;             // Ex rows
  const C *ya = nullptr, *yb = nullptr, *yc = nullptr, *yd = nullptr;  // the other component's rows
  const C* bb = nullptr;
  const R* sg0 = nullptr;
  if (rowok) {
    if (COMP == 1) {
      own = V.row(1, k, j);
      nxt = V.row(1, k - 1, j);
      xa = V.row(0, k, j + 1);
      xb = V.row(0, k, j);
      ya = V.row(2, k, j + 1);
      yb = V.row(2, k, j);
      yc = V.row(2, k - 1, j + 1);
      yd = V.row(2, k - 1, j);
      sg0 = g.s22 + ix2(n1, n2, k, j, 0);
    } else {
      own = V.row(2, k, j);
      nxt = V.row(2, k, j - 1);
      xa = V.row(0, k + 1, j);
      xb = V.row(0, k, j);
      ya = V.row(1, k + 1, j);
      yb = V.row(1, k, j);
      yc = V.row(1, k + 1, j - 1);
      yd = V.row(1, k, j - 1);
      sg0 = g.s33 + ix3(n1, n2, k, j, 0);
    }
    bb = V.brow(COMP, k, j);
  }
  C res[VW];
#pragma unroll
  for (int q = 0; q < VW; q++) res[q] = z;
  for (int T = 0; T < NC + R_ - 1; T++) {
    C nb[VW];
    hand.get(res, nb, T);
    const int c = T - rr;
    if (rowok && c >= 0 && c < NC) {
      C prev = c > 0 ? res[VW - 1] : z;  // own row at the previous march position
      C b[VW], xA[VW], xB[VW], xC[VW], xD[VW], yA[VW], yB[VW], yC[VW], yD[VW], own2[VW], rowold[VW];
      R sg[VW];
      Ax<P> X[VW];
#pragma unroll
      for (int q = 0; q < VW; q++) {  // loads: nothing read here is written in this step
        const int m = c * VW + q;
        if (m < M) {
          const int i = FWD ? 1 + m : M - m;
          X[q] = axis<P>(g.d1, g.d1s, g.r1, g.r1s, i);
          b[q] = bb ? ro(bb + i) : z;
          sg[q] = ro(sg0 + i);
          xA[q] = ro(xa + i);
          xB[q] = ro(xb + i);
          xC[q] = ro(xa + i - 1);
          xD[q] = ro(xb + i - 1);
          if (COMP == 2 || !FWD) {  // the other component: Ey for Ez, Ez backward for Ey
            yA[q] = ro(ya + i);
            yB[q] = ro(yb + i);
            yC[q] = ro(yc + i);
            yD[q] = ro(yd + i);
          }
          if (!FWD) {  // this row at the next position and the next row: not yet swept
            own2[q] = own[i - 1];
            rowold[q] = nxt[i];
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
            v = upd_ey<P>(sc, g.fvm, X[q], Y, Z, z, z, z, z, z, nb[q], z, prev, xA[q], xB[q], xC[q], xD[q], b[q],
                          sg[q]);
          else
            v = upd_ey<P>(sc, g.fvm, X[q], Y, Z, yA[q], yB[q], yC[q], yD[q], nb[q], rowold[q], prev, own2[q], xA[q],
                          xB[q], xC[q], xD[q], b[q], sg[q]);
        } else {
          if (FWD)
            v = upd_ez<P>(sc, g.fvm, X[q], Y, Z, xA[q], xB[q], xC[q], xD[q], z, prev, z, nb[q], yA[q], yB[q], yC[q],
                          yD[q], b[q], sg[q]);
          else
            v = upd_ez<P>(sc, g.fvm, X[q], Y, Z, xA[q], xB[q], xC[q], xD[q], prev, own2[q], nb[q], rowold[q], yA[q],
                          yB[q], yC[q], yD[q], b[q], sg[q]);
        }
        own[i] = v;
        res[q] = v;
        prev = v;
      }
    } else {
#pragma unroll
      for (int q = 0; q < VW; q++) res[q] = z;
    }
    hand.put(res, T);
  }
  hand.finish(NC + R_ - 1);
}

// ---------------------------------------------------------------------------------------
// complex64 sweeps: linear form, operands one step ahead.
//
// The update of a point is linear in the values it takes from the chain: its own row at
// the previous march position (prev) and the previous row at this position (nb). With
// the component's own point zero while its row is evaluated (fdfd.c:357,383,409), the
// reference's update (b - aij) / aii rearranges to
//   v = B + w (gp prev + gn nb),  w = iwmu / aii,
//   B = b / (f aii) + w (known - cross),
// where cross is the coupling to the other two components (read-only during the sweep),
// known the own-component neighbours already fixed when the point is reached (the
// not-yet-swept values of the backward sweep), gp and gn the spacing products of the two
// chain neighbours and f = vol iom with fvm (1 otherwise). B, w, gp, gn depend only on
// operands no other thread of the sweep writes before the point is reached, so each step
// loads the next step's operands first, runs the short chain part (a real and a complex
// multiply-add after nb arrives), hands over, and only then folds the loaded operands
// into the next step's B and w while the loads were in flight. Same operations as the
// reference up to the order of rounding (complex64 only; complex128 keeps the reference's
// order in k_sweep_ex / k_sweep_eyz).
namespace {

// operands of one Ex step (the backward-only ones are dropped by the compiler forward)
template <int VW> struct RawEx {
  float2 b[VW], exjm[VW], exkm[VW], eyA[VW], eyB[VW], eyC[VW], eyD[VW], ezA[VW], ezB[VW], ezC[VW], ezD[VW];
  float sg[VW];
  Ax<F32> Y;
};

template <int VW> struct RawEyz {
  float2 b[VW], xA[VW], xB[VW], xC[VW], xD[VW], yA[VW], yB[VW], yC[VW], yD[VW], own2[VW], rowold[VW];
  float sg[VW];
  Ax<F32> X[VW];
};

}  // namespace

// Ex, complex64: rows k, march j, VW consecutive i per thread. grid (line groups, systems).
//
// A CTA may carry several lines one after the other (lpc lines, a conveyor): a row that
// finishes its march on one line starts the next line at the next step, while the rows
// behind it are still on the previous one. Row t works at step T on conveyor position
// u = T - t, i.e. line u / M, march position u % M, so the row before it finished the
// same line and position at step T - 1 and the hand-over is unchanged. The pipeline
// fills and drains once per CTA instead of once per line.
template <bool FWD, int VW, int MAXR>
__global__ void CSEM_SWEEP_BOUNDS32(VW, MAXR) k_sweep_ex32(SweepP<F32> s, int lpc)
{
  typedef float2 C;
  __shared__ HandOff<VW, C, (MAXR <= NB_ROWS)> hand;
  const int slot = blockIdx.y;
  const int sys = s.sys_list ? s.sys_list[slot] : slot;
  const GridP<F32>& g = s.g;
  const int n1 = g.n1, n2 = g.n2, nK = s.nK;
  const int nlines = (n1 + VW - 1) / VW;
  const int line0 = blockIdx.x * lpc;
  const int nl = min(lpc, nlines - line0);
  const View<F32> V = view_of<F32>(s, slot, sys);
  const SysScal<F32> sc = s.scal[sys];
  const C z = make_float2(0.f, 0.f);
  const int R_ = nK - 1, M = n2 - 1;  // rows k = 1..R_, march j = 1..M
  const int U = nl * M;               // conveyor positions
  const int rr = threadIdx.x;
  const bool rowok = rr < R_;
  const int k = FWD ? 1 + rr : R_ - rr;
  const Ax<F32> Z = rowok ? axis<F32>(g.d3, g.d3s, g.r3, g.r3s, k) : Ax<F32>{};
  // the row's planes at i = 0; a line adds its first i
  C* ex0 = nullptr;
  const C *ex1 = nullptr, *ey0 = nullptr, *ez0 = nullptr, *ez1 = nullptr, *bb = nullptr;
  const float* sg0 = nullptr;
  if (rowok) {
    ex0 = V.row(0, k, 0);
    ex1 = V.row(0, k - 1, 0);
    ey0 = V.row(1, k, 0);
    ez0 = V.row(2, k, 0);
    ez1 = V.row(2, k - 1, 0);
    bb = V.brow(0, k, 0);
    sg0 = g.s11 + ix1(n1, n2, k, 0, 0);
  }
  const int L1 = n1 + 1;
  const float gn = Z.r * (FWD ? Z.rsm : Z.rs);
  int il = line0 * VW;  // first i of the line the loads are on
  int is = il;          // first i of the line the stores are on
  Ax<F32> X[VW];        // spacings of the load line's i's
  auto set_line = [&](int i0) {
    il = i0;
#pragma unroll
    for (int q = 0; q < VW; q++) X[q] = i0 + q < n1 ? axis_at<F32>(g.d1, g.d1s, g.r1, g.r1s, i0 + q) : Ax<F32>{};
  };
  set_line(il);
  RawEx<VW> raw;
  Lin32 lin[VW];
  // loads of march position c of the load line (nothing read here is written before that step)
  auto load = [&](int c) {
    const int j = FWD ? 1 + c : M - c;
    raw.Y = axis<F32>(g.d2, g.d2s, g.r2, g.r2s, j);
    const int ox = j * n1 + il, oy = j * L1 + il;
#pragma unroll
    for (int q = 0; q < VW; q++) {
      if (il + q < n1) {
        raw.b[q] = bb ? ro(bb + ox + q) : z;
        raw.sg[q] = ro(sg0 + ox + q);
        if (!FWD) {
          raw.exjm[q] = ex0[ox - n1 + q];
          raw.exkm[q] = ex1[ox + q];
          raw.eyA[q] = ro(ey0 + oy + q + 1);
          raw.eyB[q] = ro(ey0 + oy + q);
          raw.eyC[q] = ro(ey0 + oy - L1 + q + 1);
          raw.eyD[q] = ro(ey0 + oy - L1 + q);
          raw.ezA[q] = ro(ez0 + oy + q + 1);
          raw.ezB[q] = ro(ez0 + oy + q);
          raw.ezC[q] = ro(ez1 + oy + q + 1);
          raw.ezD[q] = ro(ez1 + oy + q);
        }
      }
    }
  };
  auto make = [&]() {
    const Ax<F32>& Y = raw.Y;
    const float gg = (Y.rs + Y.rsm) * Y.r + (Z.rs + Z.rsm) * Z.r;  // geo(Y, Z)
    const float gp = Y.r * (FWD ? Y.rsm : Y.rs);
#pragma unroll
    for (int q = 0; q < VW; q++) {
      if (il + q >= n1) continue;
      C kc = z;
      if (!FWD) {
        const C dy = sub32(sub32(raw.eyA[q], raw.eyB[q]), sub32(raw.eyC[q], raw.eyD[q]));
        const C dz = sub32(sub32(raw.ezA[q], raw.ezB[q]), sub32(raw.ezC[q], raw.ezD[q]));
        const C cross = scl32(X[q].rs, make_float2(Y.r * dy.x + Z.r * dz.x, Y.r * dy.y + Z.r * dz.y));
        const C known = make_float2(Y.r * Y.rsm * raw.exjm[q].x + Z.r * Z.rsm * raw.exkm[q].x,
                                    Y.r * Y.rsm * raw.exjm[q].y + Z.r * Z.rsm * raw.exkm[q].y);
        kc = sub32(known, cross);
      }
      lin[q] = lin_make(sc, g.fvm, gg, raw.sg[q], X[q].ds * Y.d * Z.d, raw.b[q], kc, gp, gn);
    }
  };
  C res[VW];
#pragma unroll
  for (int q = 0; q < VW; q++) res[q] = z;
  if (rowok && rr == 0 && U > 0) {
    load(0);
    make();
  }
  for (int T = 0; T < U + R_ - 1; T++) {
    const int u = T - rr;
    const bool act = rowok && u >= 0 && u < U;
    const bool nxt = rowok && u + 1 >= 0 && u + 1 < U;
    int cn = 0;
    if (nxt) {
      cn = (u + 1) % M;
      if (cn == 0 && u + 1 > 0) set_line((line0 + (u + 1) / M) * VW);  // the loads move to the next line
      load(cn);
    }
    C nb[VW];
    hand.get(res, nb, T);
    if (act) {
      const int c = u % M;
      const int ox = (FWD ? 1 + c : M - c) * n1 + is;
#pragma unroll
      for (int q = 0; q < VW; q++) {
        if (is + q >= n1) {
          res[q] = z;
          continue;
        }
        const C v = lin_apply(lin[q], c > 0 ? res[q] : z, nb[q]);  // prev: own row, previous j
        ex0[ox + q] = v;
        res[q] = v;
      }
      if (c == M - 1) is = il;  // the stores follow the loads onto the next line
    } else {
#pragma unroll
      for (int q = 0; q < VW; q++) res[q] = z;
    }
    hand.put(res, T);
    if (nxt) make();
  }
  hand.finish(U + R_ - 1);
}

// Ey (COMP 1: line j, rows k) / Ez (COMP 2: line k, rows j), complex64: march i in
// chunks of VW, lpc lines per CTA as a conveyor (see k_sweep_ex32). grid (line groups,
// systems)
template <int COMP, bool FWD, int VW, int MAXR>
__global__ void CSEM_SWEEP_BOUNDS32(VW, MAXR) k_sweep_eyz32(SweepP<F32> s, int lpc)
{
  typedef float2 C;
  __shared__ HandOff<VW, C, (MAXR <= NB_ROWS)> hand;
  const int slot = blockIdx.y;
  const int sys = s.sys_list ? s.sys_list[slot] : slot;
  const GridP<F32>& g = s.g;
  const int n1 = g.n1, n2 = g.n2, nK = s.nK;
  const int nlines = COMP == 1 ? n2 : nK;
  const int line0 = blockIdx.x * lpc;
  const int nl = min(lpc, nlines - line0);
  const View<F32> V = view_of<F32>(s, slot, sys);
  const SysScal<F32> sc = s.scal[sys];
  const C z = make_float2(0.f, 0.f);
  const int R_ = COMP == 1 ? nK - 1 : n2 - 1;  // rows k (Ey) or j (Ez) = 1..R_
  const int M = n1 - 1;                         // march i = 1..M
  const int NC = (M + VW - 1) / VW;
  const int U = nl * NC;  // conveyor positions
  const int rr = threadIdx.x;
  const bool rowok = rr < R_;
  const int r = FWD ? 1 + rr : R_ - rr;
  // the row's axis (Z for Ey, Y for Ez) is fixed; the line's axis (Y for Ey, Z for Ez)
  // moves with the conveyor
  const Ax<F32> Rw = rowok ? (COMP == 1 ? axis<F32>(g.d3, g.d3s, g.r3, g.r3s, r) : axis<F32>(g.d2, g.d2s, g.r2, g.r2s, r))
                           : Ax<F32>{};
  const float gn = Rw.r * (FWD ? Rw.rsm : Rw.rs);
  // the rows the loads read (element i is row[i]) and the line's spacings
  C* own = nullptr;
  const C *nxt = nullptr, *xa = nullptr, *xb = nullptr, *ya = nullptr, *yb = nullptr, *yc = nullptr, *yd = nullptr;
  const C* bb = nullptr;
  const float* sg0 = nullptr;
  float lrs = 0.f, ld = 0.f;  // the line axis' rs (the coefficient of the line-axis differences) and d
  auto set_line = [&](int line) {
    const int k = COMP == 1 ? r : line;
    const int j = COMP == 1 ? line : r;
    const Ax<F32> LA = COMP == 1 ? axis_at<F32>(g.d2, g.d2s, g.r2, g.r2s, j) : axis_at<F32>(g.d3, g.d3s, g.r3, g.r3s, k);
    lrs = LA.rs;
    ld = LA.d;
    if (COMP == 1) {
      own = V.row(1, k, j);
      nxt = V.row(1, k - 1, j);
      xa = V.row(0, k, j + 1);
      xb = V.row(0, k, j);
      ya = V.row(2, k, j + 1);
      yb = V.row(2, k, j);
      yc = V.row(2, k - 1, j + 1);
      yd = V.row(2, k - 1, j);
      sg0 = g.s22 + ix2(n1, n2, k, j, 0);
    } else {
      own = V.row(2, k, j);
      nxt = V.row(2, k, j - 1);
      xa = V.row(0, k + 1, j);
      xb = V.row(0, k, j);
      ya = V.row(1, k + 1, j);
      yb = V.row(1, k, j);
      yc = V.row(1, k + 1, j - 1);
      yd = V.row(1, k, j - 1);
      sg0 = g.s33 + ix3(n1, n2, k, j, 0);
    }
    bb = V.brow(COMP, k, j);
  };
  if (rowok) set_line(line0);
  C* own_st = own;  // the row the stores go to (the loads run one position ahead)
  RawEyz<VW> raw;
  Lin32 lin[VW];
  auto load = [&](int c) {
#pragma unroll
    for (int q = 0; q < VW; q++) {
      const int m = c * VW + q;
      if (m < M) {
        const int i = FWD ? 1 + m : M - m;
        raw.X[q] = axis<F32>(g.d1, g.d1s, g.r1, g.r1s, i);
        raw.b[q] = bb ? ro(bb + i) : z;
        raw.sg[q] = ro(sg0 + i);
        raw.xA[q] = ro(xa + i);
        raw.xB[q] = ro(xb + i);
        raw.xC[q] = ro(xa + i - 1);
        raw.xD[q] = ro(xb + i - 1);
        if (COMP == 2 || !FWD) {
          raw.yA[q] = ro(ya + i);
          raw.yB[q] = ro(yb + i);
          raw.yC[q] = ro(yc + i);
          raw.yD[q] = ro(yd + i);
        }
        if (!FWD) {
          raw.own2[q] = own[i - 1];
          raw.rowold[q] = nxt[i];
        }
      }
    }
  };
  auto make = [&](int c) {
#pragma unroll
    for (int q = 0; q < VW; q++) {
      if (c * VW + q >= M) continue;
      const Ax<F32>& X = raw.X[q];
      const float gg = (X.rs + X.rsm) * X.r + (Rw.rs + Rw.rsm) * Rw.r;  // geo(Z, X) / geo(X, Y)
      const C dx = sub32(sub32(raw.xA[q], raw.xB[q]), sub32(raw.xC[q], raw.xD[q]));
      // Ey: Y.rs (Z.r dEz + X.r dEx); Ez: Z.rs (X.r dEx + Y.r dEy)
      C acc = scl32(X.r, dx);
      if (COMP == 2 || !FWD) {
        const C dy = sub32(sub32(raw.yA[q], raw.yB[q]), sub32(raw.yC[q], raw.yD[q]));
        acc = make_float2(acc.x + Rw.r * dy.x, acc.y + Rw.r * dy.y);
      }
      C kc = scl32(-lrs, acc);
      if (!FWD) {
        const C known = make_float2(X.r * X.rsm * raw.own2[q].x + Rw.r * Rw.rsm * raw.rowold[q].x,
                                    X.r * X.rsm * raw.own2[q].y + Rw.r * Rw.rsm * raw.rowold[q].y);
        kc = make_float2(kc.x + known.x, kc.y + known.y);
      }
      const float yd = COMP == 1 ? ld : Rw.d, zd = COMP == 1 ? Rw.d : ld;  // Y.d and Z.d
      lin[q] = lin_make(sc, g.fvm, gg, raw.sg[q], X.ds * yd * zd, raw.b[q], kc, X.r * (FWD ? X.rsm : X.rs), gn);
    }
  };
  C res[VW];
#pragma unroll
  for (int q = 0; q < VW; q++) res[q] = z;
  if (rowok && rr == 0 && U > 0) {
    load(0);
    make(0);
  }
  for (int T = 0; T < U + R_ - 1; T++) {
    const int u = T - rr;
    const bool act = rowok && u >= 0 && u < U;
    const bool nx = rowok && u + 1 >= 0 && u + 1 < U;
    int cn = 0;
    if (nx) {
      cn = (u + 1) % NC;
      if (cn == 0 && u + 1 > 0) set_line(line0 + (u + 1) / NC);  // the loads move to the next line
      load(cn);
    }
    C nb[VW];
    hand.get(res, nb, T);
    if (act) {
      const int c = u % NC;
      C prev = c > 0 ? res[VW - 1] : z;  // own row at the previous march position
#pragma unroll
      for (int q = 0; q < VW; q++) {
        const int m = c * VW + q;
        if (m >= M) {
          res[q] = z;
          continue;
        }
        const C v = lin_apply(lin[q], prev, nb[q]);
        own_st[FWD ? 1 + m : M - m] = v;
        res[q] = v;
        prev = v;
      }
      if (c == NC - 1) own_st = own;  // the stores follow the loads onto the next line
    } else {
#pragma unroll
      for (int q = 0; q < VW; q++) res[q] = z;
    }
    hand.put(res, T);
    if (nx) make(cn);
  }
  hand.finish(U + R_ - 1);
}

bool sweep_pipelined_fits(int comp, int n1, int n2, int nK)
{
  const int rows = comp == 2 ? n2 - 1 : nK - 1;
  return rows >= 1 && rows <= MAXROWS && n1 >= 2 && n2 >= 2;
}

template <class P, int VW, int MAXR>
static void launch_vw(const SweepP<P>& s, int comp, bool fwd, int nslot, cudaStream_t st, int lpc)
{
  const int n1 = s.g.n1, n2 = s.g.n2, nK = s.nK;
  const int rows = comp == 2 ? n2 - 1 : nK - 1;
  const int threads = (rows + 31) / 32 * 32;
  if constexpr (!P::exact) {  // complex64: the linear-form sweeps, lpc lines per CTA
    if (comp == 0) {
      dim3 grd(((n1 + VW - 1) / VW + lpc - 1) / lpc, nslot);
      if (fwd) count_launch(), k_sweep_ex32<true, VW, MAXR><<<grd, threads, 0, st>>>(s, lpc);
      else count_launch(), k_sweep_ex32<false, VW, MAXR><<<grd, threads, 0, st>>>(s, lpc);
    } else if (comp == 1) {
      dim3 grd((n2 + lpc - 1) / lpc, nslot);
      if (fwd) count_launch(), k_sweep_eyz32<1, true, VW, MAXR><<<grd, threads, 0, st>>>(s, lpc);
      else count_launch(), k_sweep_eyz32<1, false, VW, MAXR><<<grd, threads, 0, st>>>(s, lpc);
    } else {
      dim3 grd((nK + lpc - 1) / lpc, nslot);
      if (fwd) count_launch(), k_sweep_eyz32<2, true, VW, MAXR><<<grd, threads, 0, st>>>(s, lpc);
      else count_launch(), k_sweep_eyz32<2, false, VW, MAXR><<<grd, threads, 0, st>>>(s, lpc);
    }
  } else {  // complex128: the reference's operation order, one line per CTA
    if (comp == 0) {
      dim3 grd((n1 + VW - 1) / VW, nslot);
      if (fwd) count_launch(), k_sweep_ex<P, true, VW, MAXR><<<grd, threads, 0, st>>>(s);
      else count_launch(), k_sweep_ex<P, false, VW, MAXR><<<grd, threads, 0, st>>>(s);
    } else if (comp == 1) {
      dim3 grd(n2, nslot);
      if (fwd) count_launch(), k_sweep_eyz<P, 1, true, VW, MAXR><<<grd, threads, 0, st>>>(s);
      else count_launch(), k_sweep_eyz<P, 1, false, VW, MAXR><<<grd, threads, 0, st>>>(s);
    } else {
      dim3 grd(nK, nslot);
      if (fwd) count_launch(), k_sweep_eyz<P, 2, true, VW, MAXR><<<grd, threads, 0, st>>>(s);
      else count_launch(), k_sweep_eyz<P, 2, false, VW, MAXR><<<grd, threads, 0, st>>>(s);
    }
  }
}

// vw: points per thread and step (1, 2 or 4; other values select the default, the
// fastest measured on a 200x140x140 grid: 2 for complex64, 1 for complex128). Sweeps of
// more than 256 rows run 1 or 2 points per thread in CTAs of up to 512 threads.
// lines_per_cta: lines one CTA carries as a conveyor (complex64; >= 1).
template <class P>
void launch_sweep_pipelined(const SweepP<P>& s, int comp, bool fwd, int nslot, cudaStream_t st, int vw,
                            int lines_per_cta)
{
  if (vw != 1 && vw != 2 && vw != 4) vw = P::exact ? 1 : 2;
  const int lpc = lines_per_cta > 1 ? lines_per_cta : 1;
  const int rows = comp == 2 ? s.g.n2 - 1 : s.nK - 1;
  if (rows > NB_ROWS) {
    if (vw == 1) launch_vw<P, 1, MAXROWS>(s, comp, fwd, nslot, st, lpc);
    else launch_vw<P, 2, MAXROWS>(s, comp, fwd, nslot, st, lpc);
    return;
  }
  if (vw == 1) launch_vw<P, 1, NB_ROWS>(s, comp, fwd, nslot, st, lpc);
  else if (vw == 2) launch_vw<P, 2, NB_ROWS>(s, comp, fwd, nslot, st, lpc);
  else launch_vw<P, 4, NB_ROWS>(s, comp, fwd, nslot, st, lpc);
}

template void launch_sweep_pipelined<F64>(const SweepP<F64>&, int, bool, int, cudaStream_t, int, int);
template void launch_sweep_pipelined<F32>(const SweepP<F32>&, int, bool, int, cudaStream_t, int, int);

}  // namespace csem
