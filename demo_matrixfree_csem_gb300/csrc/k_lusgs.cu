// LU-SGS (fdfd.c:287-510) and A-phi (fdfd.c:513-821) preconditioner sweeps.
//
// Each component sweep of the reference is a lexicographic Gauss-Seidel pass in which
// the updated component couples to itself in only two directions; the third axis is
// independent:
//   Ex: couples in (j,k), independent i      Ey: couples in (i,k), independent j
//   Ez: couples in (i,j), independent k
// Every point of an anti-diagonal t = a + b of the coupled plane depends only on points
// of diagonal t-1 (forward) or t+1 (backward), so updating one diagonal at a time,
// all independent-axis lines and all systems of a batch at once, reproduces the
// lexicographic order exactly. The A-phi node potential couples in all three axes and
// is swept over i+j+k = s hyperplanes.
//
// Values a lexicographic sweep has not reached yet are zero in the reference (the
// output starts from zero); the forward kernels use those zeros directly instead of
// loading them.
#include "csem_cuda.cuh"
#include "engine.h"

namespace csem {

template <class P> struct SweepView {
  typedef typename P::C C;
  int n1, n2, vshift;
  C *Y[3];
  C *CAP[3];
  const C *X[3];
  __device__ __forceinline__ static long idx(int c, int n1, int n2, int k, int j, int i)
  {
    return c == 0 ? ix1(n1, n2, k, j, i) : (c == 1 ? ix2(n1, n2, k, j, i) : ix3(n1, n2, k, j, i));
  }
  __device__ __forceinline__ C ld(int c, int k, int j, int i) const
  {
    return k >= vshift ? Y[c][idx(c, n1, n2, k - vshift, j, i)] : CAP[c][idx(c, n1, n2, k, j, i)];
  }
  __device__ __forceinline__ void st(int c, int k, int j, int i, C v) const
  {
    if (k >= vshift) Y[c][idx(c, n1, n2, k - vshift, j, i)] = v;
    else CAP[c][idx(c, n1, n2, k, j, i)] = v;
  }
  __device__ __forceinline__ C ldb(int c, int k, int j, int i) const
  {
    return k >= vshift ? X[c][idx(c, n1, n2, k - vshift, j, i)] : P::mk(0, 0);
  }
};

template <class P>
__device__ __forceinline__ SweepView<P> make_view(const SweepP<P>& s, int slot, int sys)
{
  SweepView<P> v;
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

// node potential index (fdfd.c:19), same map as Ez
__device__ __forceinline__ long ixv(int n1, int n2, int k, int j, int i) { return ix3(n1, n2, k, j, i); }

// geometric part of the diagonal: (1/a0 + 1/a1)/A + (1/b0 + 1/b1)/B
template <class P>
__device__ __forceinline__ typename P::R geo2(typename P::R a0, typename P::R a1, typename P::R A, typename P::R b0,
                                              typename P::R b1, typename P::R B)
{
  typedef typename P::R R;
  const R one = 1;
  return P::add(P::div(P::add(P::div(one, a0), P::div(one, a1)), A),
                P::div(P::add(P::div(one, b0), P::div(one, b1)), B));
}

template <class P>
__device__ __forceinline__ typename P::C finish(typename P::C b, typename P::C aij, typename P::R geo,
                                                typename P::R sg, typename P::R vol, const SysScal<P>& sc, int fvm)
{
  typedef typename P::C C;
  C aii = rmul<P>(geo, sc.iwmu);
  aii.x = P::sub(aii.x, sg);
  if (fvm) {
    C f = rmul<P>(vol, sc.iom);
    aij = cmul<P>(aij, f);
    aii = cmul<P>(aii, f);
  }
  return cdiv<P>(csub<P>(b, aij), aii);
}

// Ex row (fdfd.c:357-369; A-phi fdfd.c:586-598)
template <class P, bool FWD, bool APHI>
__device__ __forceinline__ void row_ex(const SweepP<P>& s, const SweepView<P>& V, const typename P::C* vphi,
                                       const SysScal<P>& sc, int k, int j, int i)
{
  typedef typename P::C C;
  const GridP<P>& g = s.g;
  const C z = czero<P>();
  const C own = z;
  C eyA = FWD ? z : V.ld(1, k, j, i + 1), eyB = FWD ? z : V.ld(1, k, j, i);
  C eyC = FWD ? z : V.ld(1, k, j - 1, i + 1), eyD = FWD ? z : V.ld(1, k, j - 1, i);
  C exjp = FWD ? z : V.ld(0, k, j + 1, i), exjm = V.ld(0, k, j - 1, i);
  C exkp = FWD ? z : V.ld(0, k + 1, j, i), exkm = V.ld(0, k - 1, j, i);
  C ezA = FWD ? z : V.ld(2, k, j, i + 1), ezB = FWD ? z : V.ld(2, k, j, i);
  C ezC = FWD ? z : V.ld(2, k - 1, j, i + 1), ezD = FWD ? z : V.ld(2, k - 1, j, i);
  C t1 = csub<P>(cdivs<P>(csub<P>(eyA, eyB), g.d1s[i], g.r1s[i]), cdivs<P>(csub<P>(exjp, own), g.d2s[j], g.r2s[j]));
  C t2 = csub<P>(cdivs<P>(csub<P>(eyC, eyD), g.d1s[i], g.r1s[i]), cdivs<P>(csub<P>(own, exjm), g.d2s[j - 1], g.r2s[j - 1]));
  C t3 = csub<P>(cdivs<P>(csub<P>(exkp, own), g.d3s[k], g.r3s[k]), cdivs<P>(csub<P>(ezA, ezB), g.d1s[i], g.r1s[i]));
  C t4 = csub<P>(cdivs<P>(csub<P>(own, exkm), g.d3s[k - 1], g.r3s[k - 1]), cdivs<P>(csub<P>(ezC, ezD), g.d1s[i], g.r1s[i]));
  const typename P::R sg = g.s11[ix1(g.n1, g.n2, k, j, i)];
  C ownv = own;
  if (APHI && !FWD)
    ownv = cadd<P>(own, cdivs<P>(csub<P>(vphi[ixv(g.n1, g.n2, k, j, i + 1)], vphi[ixv(g.n1, g.n2, k, j, i)]), g.d1s[i], g.r1s[i]));
  C aij = csub<P>(cmul<P>(csub<P>(cdivs<P>(csub<P>(t1, t2), g.d2[j], g.r2[j]), cdivs<P>(csub<P>(t3, t4), g.d3[k], g.r3[k])), sc.iwmu),
                  rmul<P>(sg, ownv));
  typename P::R geo = geo2<P>(g.d2s[j], g.d2s[j - 1], g.d2[j], g.d3s[k], g.d3s[k - 1], g.d3[k]);
  typename P::R vol = g.fvm ? P::mul(P::mul(g.d1s[i], g.d2[j]), g.d3[k]) : 0;
  V.st(0, k, j, i, finish<P>(V.ldb(0, k, j, i), aij, geo, sg, vol, sc, g.fvm));
}

// Ey row (fdfd.c:383-395; A-phi fdfd.c:612-624)
template <class P, bool FWD, bool APHI>
__device__ __forceinline__ void row_ey(const SweepP<P>& s, const SweepView<P>& V, const typename P::C* vphi,
                                       const SysScal<P>& sc, int k, int j, int i)
{
  typedef typename P::C C;
  const GridP<P>& g = s.g;
  const C z = czero<P>();
  const C own = z;
  C ezA = FWD ? z : V.ld(2, k, j + 1, i), ezB = FWD ? z : V.ld(2, k, j, i);
  C ezC = FWD ? z : V.ld(2, k - 1, j + 1, i), ezD = FWD ? z : V.ld(2, k - 1, j, i);
  C eykp = FWD ? z : V.ld(1, k + 1, j, i), eykm = V.ld(1, k - 1, j, i);
  C eyip = FWD ? z : V.ld(1, k, j, i + 1), eyim = V.ld(1, k, j, i - 1);
  C exA = V.ld(0, k, j + 1, i), exB = V.ld(0, k, j, i);
  C exC = V.ld(0, k, j + 1, i - 1), exD = V.ld(0, k, j, i - 1);
  C t1 = csub<P>(cdivs<P>(csub<P>(ezA, ezB), g.d2s[j], g.r2s[j]), cdivs<P>(csub<P>(eykp, own), g.d3s[k], g.r3s[k]));
  C t2 = csub<P>(cdivs<P>(csub<P>(ezC, ezD), g.d2s[j], g.r2s[j]), cdivs<P>(csub<P>(own, eykm), g.d3s[k - 1], g.r3s[k - 1]));
  C t3 = csub<P>(cdivs<P>(csub<P>(eyip, own), g.d1s[i], g.r1s[i]), cdivs<P>(csub<P>(exA, exB), g.d2s[j], g.r2s[j]));
  C t4 = csub<P>(cdivs<P>(csub<P>(own, eyim), g.d1s[i - 1], g.r1s[i - 1]), cdivs<P>(csub<P>(exC, exD), g.d2s[j], g.r2s[j]));
  const typename P::R sg = g.s22[ix2(g.n1, g.n2, k, j, i)];
  C ownv = own;
  if (APHI && !FWD)
    ownv = cadd<P>(own, cdivs<P>(csub<P>(vphi[ixv(g.n1, g.n2, k, j + 1, i)], vphi[ixv(g.n1, g.n2, k, j, i)]), g.d2s[j], g.r2s[j]));
  C aij = csub<P>(cmul<P>(csub<P>(cdivs<P>(csub<P>(t1, t2), g.d3[k], g.r3[k]), cdivs<P>(csub<P>(t3, t4), g.d1[i], g.r1[i])), sc.iwmu),
                  rmul<P>(sg, ownv));
  typename P::R geo = geo2<P>(g.d3s[k], g.d3s[k - 1], g.d3[k], g.d1s[i], g.d1s[i - 1], g.d1[i]);
  // the reference uses Ex's cell volume here (fdfd.c:391)
  typename P::R vol = g.fvm ? P::mul(P::mul(g.d1s[i], g.d2[j]), g.d3[k]) : 0;
  V.st(1, k, j, i, finish<P>(V.ldb(1, k, j, i), aij, geo, sg, vol, sc, g.fvm));
}

// Ez row (fdfd.c:409-421; A-phi fdfd.c:638-650)
template <class P, bool FWD, bool APHI>
__device__ __forceinline__ void row_ez(const SweepP<P>& s, const SweepView<P>& V, const typename P::C* vphi,
                                       const SysScal<P>& sc, int k, int j, int i)
{
  typedef typename P::C C;
  const GridP<P>& g = s.g;
  const C z = czero<P>();
  const C own = z;
  C exA = V.ld(0, k + 1, j, i), exB = V.ld(0, k, j, i);
  C exC = V.ld(0, k + 1, j, i - 1), exD = V.ld(0, k, j, i - 1);
  C ezip = FWD ? z : V.ld(2, k, j, i + 1), ezim = V.ld(2, k, j, i - 1);
  C ezjp = FWD ? z : V.ld(2, k, j + 1, i), ezjm = V.ld(2, k, j - 1, i);
  C eyA = V.ld(1, k + 1, j, i), eyB = V.ld(1, k, j, i);
  C eyC = V.ld(1, k + 1, j - 1, i), eyD = V.ld(1, k, j - 1, i);
  C t1 = csub<P>(cdivs<P>(csub<P>(exA, exB), g.d3s[k], g.r3s[k]), cdivs<P>(csub<P>(ezip, own), g.d1s[i], g.r1s[i]));
  C t2 = csub<P>(cdivs<P>(csub<P>(exC, exD), g.d3s[k], g.r3s[k]), cdivs<P>(csub<P>(own, ezim), g.d1s[i - 1], g.r1s[i - 1]));
  C t3 = csub<P>(cdivs<P>(csub<P>(ezjp, own), g.d2s[j], g.r2s[j]), cdivs<P>(csub<P>(eyA, eyB), g.d3s[k], g.r3s[k]));
  C t4 = csub<P>(cdivs<P>(csub<P>(own, ezjm), g.d2s[j - 1], g.r2s[j - 1]), cdivs<P>(csub<P>(eyC, eyD), g.d3s[k], g.r3s[k]));
  const typename P::R sg = g.s33[ix3(g.n1, g.n2, k, j, i)];
  C ownv = own;
  if (APHI && !FWD)
    ownv = cadd<P>(own, cdivs<P>(csub<P>(vphi[ixv(g.n1, g.n2, k + 1, j, i)], vphi[ixv(g.n1, g.n2, k, j, i)]), g.d3s[k], g.r3s[k]));
  C aij = csub<P>(cmul<P>(csub<P>(cdivs<P>(csub<P>(t1, t2), g.d1[i], g.r1[i]), cdivs<P>(csub<P>(t3, t4), g.d2[j], g.r2[j])), sc.iwmu),
                  rmul<P>(sg, ownv));
  typename P::R geo = geo2<P>(g.d1s[i], g.d1s[i - 1], g.d1[i], g.d2s[j], g.d2s[j - 1], g.d2[j]);
  typename P::R vol = g.fvm ? P::mul(P::mul(g.d1s[i], g.d2[j]), g.d3[k]) : 0;
  V.st(2, k, j, i, finish<P>(V.ldb(2, k, j, i), aij, geo, sg, vol, sc, g.fvm));
}

// one anti-diagonal t of one component sweep
template <class P, int COMP, bool FWD, bool APHI>
__global__ void k_sweep(SweepP<P> s, int t)
{
  const int slot = blockIdx.z;
  const int sys = s.sys_list ? s.sys_list[slot] : slot;
  const int n1 = s.g.n1, n2 = s.g.n2, nK = s.nK;
  // coupled plane (a,b) and independent axis c per component
  const int Am = COMP == 0 ? n2 - 1 : n1 - 1;           // a in [1, Am]
  const int Bm = COMP == 2 ? n2 - 1 : nK - 1;           // b in [1, Bm]
  const int cN = COMP == 0 ? n1 : (COMP == 1 ? n2 : nK);
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int bmin = max(1, t - Am), bmax = min(Bm, t - 1);
  const int b = bmin + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  if (c >= cN || b > bmax) return;
  const int a = t - b;
  const SweepView<P> V = make_view<P>(s, slot, sys);
  const SysScal<P> sc = s.scal[sys];
  const typename P::C* vphi = APHI ? s.V + (size_t)slot * s.lv : nullptr;
  if (COMP == 0) row_ex<P, FWD, APHI>(s, V, vphi, sc, /*k*/ b, /*j*/ a, /*i*/ c);
  else if (COMP == 1) row_ey<P, FWD, APHI>(s, V, vphi, sc, /*k*/ b, /*j*/ c, /*i*/ a);
  else row_ez<P, FWD, APHI>(s, V, vphi, sc, /*k*/ c, /*j*/ b, /*i*/ a);
}

int sweep_diagonals(int comp, int n1, int n2, int nK)
{
  int Am = comp == 0 ? n2 - 1 : n1 - 1;
  int Bm = comp == 2 ? n2 - 1 : nK - 1;
  return Am + Bm - 1;  // t = 2 .. Am+Bm
}

template <class P>
void launch_sweep(const SweepP<P>& s, int comp, bool fwd, bool aphi, int t, int nslot, cudaStream_t st)
{
  const int n1 = s.g.n1, n2 = s.g.n2, nK = s.nK;
  const int Am = comp == 0 ? n2 - 1 : n1 - 1;
  const int Bm = comp == 2 ? n2 - 1 : nK - 1;
  const int cN = comp == 0 ? n1 : (comp == 1 ? n2 : nK);
  const int len = min(Bm, t - 1) - max(1, t - Am) + 1;
  if (len <= 0) return;
  dim3 blk(32, 4);
  dim3 grd((cN + 31) / 32, (len + 3) / 4, nslot);
#define CSEM_SW(C, F, A) count_launch(), k_sweep<P, C, F, A><<<grd, blk, 0, st>>>(s, t)
  if (!aphi) {
    if (comp == 0) { if (fwd) CSEM_SW(0, true, false); else CSEM_SW(0, false, false); }
    else if (comp == 1) { if (fwd) CSEM_SW(1, true, false); else CSEM_SW(1, false, false); }
    else { if (fwd) CSEM_SW(2, true, false); else CSEM_SW(2, false, false); }
  } else {
    if (comp == 0) { if (fwd) CSEM_SW(0, true, true); else CSEM_SW(0, false, true); }
    else if (comp == 1) { if (fwd) CSEM_SW(1, true, true); else CSEM_SW(1, false, true); }
    else { if (fwd) CSEM_SW(2, true, true); else CSEM_SW(2, false, true); }
  }
#undef CSEM_SW
}

// ---------------------------------------------------------------- A-phi extras
// bv = -div x on interior nodes (fdfd.c:553-566); zero elsewhere
template <class P>
__global__ void k_aphi_div(SweepP<P> s, typename P::C* __restrict__ BV)
{
  typedef typename P::C C;
  const int slot = blockIdx.z;
  const int sys = s.sys_list ? s.sys_list[slot] : slot;
  const GridP<P>& g = s.g;
  const int n1 = g.n1, n2 = g.n2, n3 = g.n3;
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= s.lv) return;
  const int i = (int)(q % (n1 + 1));
  const int j = (int)((q / (n1 + 1)) % (n2 + 1));
  const int k = (int)(q / ((long)(n1 + 1) * (n2 + 1)));
  C r = czero<P>();
  if (i >= 1 && i < n1 && j >= 1 && j < n2 && k >= 1 && k < n3) {
    const C* bx = s.X + (size_t)sys * g.lE;
    const C* by = bx + g.lEx;
    const C* bz = by + g.lEy;
    r = cadd<P>(r, cdivs<P>(cneg<P>(csub<P>(bx[ix1(n1, n2, k, j, i)], bx[ix1(n1, n2, k, j, i - 1)])), g.d1[i], g.r1[i]));
    r = cadd<P>(r, cdivs<P>(cneg<P>(csub<P>(by[ix2(n1, n2, k, j, i)], by[ix2(n1, n2, k, j - 1, i)])), g.d2[j], g.r2[j]));
    r = cadd<P>(r, cdivs<P>(cneg<P>(csub<P>(bz[ix3(n1, n2, k, j, i)], bz[ix3(n1, n2, k - 1, j, i)])), g.d3[k], g.r3[k]));
  }
  BV[(size_t)slot * s.lv + q] = r;
}

// one hyperplane i+j+k = t of the node-potential sweep (fdfd.c:654-710)
template <class P, bool FWD>
__global__ void k_aphi_phi(SweepP<P> s, typename P::C* __restrict__ VV, int t)
{
  typedef typename P::C C;
  typedef typename P::R R;
  const int slot = blockIdx.z;
  const int sys = s.sys_list ? s.sys_list[slot] : slot;
  const GridP<P>& g = s.g;
  const int n1 = g.n1, n2 = g.n2, n3 = g.n3;
  const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int j = 1 + blockIdx.y * blockDim.y + threadIdx.y;
  const int k = t - i - j;
  if (i >= n1 || j >= n2 || k < 1 || k >= n3) return;
  C* v = VV + (size_t)slot * s.lv;
  const C* bv = s.BV + (size_t)slot * s.lv;
  const C* ax = s.Y + (size_t)sys * g.lE;
  const C* ay = ax + g.lEx;
  const C* az = ay + g.lEy;
  const SysScal<P> sc = s.scal[sys];
  const C z = czero<P>();
  const C vp = z;  // v(k,j,i) is zeroed before its own update
  const C vip = FWD ? z : v[ixv(n1, n2, k, j, i + 1)], vim = v[ixv(n1, n2, k, j, i - 1)];
  const C vjp = FWD ? z : v[ixv(n1, n2, k, j + 1, i)], vjm = v[ixv(n1, n2, k, j - 1, i)];
  const C vkp = FWD ? z : v[ixv(n1, n2, k + 1, j, i)], vkm = v[ixv(n1, n2, k - 1, j, i)];
  const int kf = k + g.kstart;
  // the conductivities of the six faces around node (k,j,i): the reference reads the
  // lower faces unshifted (Q2, fdfd.c:666,668,670,695,697,699); with aphi_fix all six
  // come from the shifted operator-grid arrays
  const R s1p = g.s11[ix1(n1, n2, k, j, i)], s2p = g.s22[ix2(n1, n2, k, j, i)], s3p = g.s33[ix3(n1, n2, k, j, i)];
  const R s1m = s.aphi_fix ? g.s11[ix1(n1, n2, k, j, i - 1)] : s.s11u[ix1(n1, n2, k, j, i - 1)];
  const R s2m = s.aphi_fix ? g.s22[ix2(n1, n2, k, j - 1, i)] : s.s22u[ix2(n1, n2, k, j - 1, i)];
  const R s3m = s.aphi_fix ? g.s33[ix3(n1, n2, k - 1, j, i)] : s.s33u[ix3(n1, n2, k - 1, j, i)];
  C t1 = rmul<P>(s1p, cadd<P>(ax[ix1(n1, n2, k, j, i)], cdivs<P>(csub<P>(vip, vp), g.d1s[i], g.r1s[i])));
  C t2 = rmul<P>(s1m, cadd<P>(ax[ix1(n1, n2, k, j, i - 1)], cdivs<P>(csub<P>(vp, vim), g.d1s[i - 1], g.r1s[i - 1])));
  C t3 = rmul<P>(s2p, cadd<P>(ay[ix2(n1, n2, k, j, i)], cdivs<P>(csub<P>(vjp, vp), g.d2s[j], g.r2s[j])));
  C t4 = rmul<P>(s2m, cadd<P>(ay[ix2(n1, n2, k, j - 1, i)], cdivs<P>(csub<P>(vp, vjm), g.d2s[j - 1], g.r2s[j - 1])));
  C t5 = rmul<P>(s3p, cadd<P>(az[ix3(n1, n2, k, j, i)], cdivs<P>(csub<P>(vkp, vp), g.d3s[k], g.r3s[k])));
  C t6 = rmul<P>(s3m, cadd<P>(az[ix3(n1, n2, k - 1, j, i)], cdivs<P>(csub<P>(vp, vkm), g.d3s[k - 1], g.r3s[k - 1])));
  C aij = cadd<P>(cadd<P>(cdivs<P>(csub<P>(t1, t2), g.d1[i], g.r1[i]), cdivs<P>(csub<P>(t3, t4), g.d2[j], g.r2[j])),
                  cdivs<P>(csub<P>(t5, t6), g.d3[k], g.r3[k]));
  const R one = 1;
  // the reference's diagonal is the plain Laplacian's (Q3, fdfd.c:672,701) although the
  // couplings carry the face conductivities; with aphi_fix the diagonal carries them too,
  // the diagonal of div(sigma grad v), so the node sweep is a Gauss-Seidel sweep of
  // that operator
  const R w1p = s.aphi_fix ? s1p : one, w1m = s.aphi_fix ? s1m : one;
  const R w2p = s.aphi_fix ? s2p : one, w2m = s.aphi_fix ? s2m : one;
  const R w3p = s.aphi_fix ? s3p : one, w3m = s.aphi_fix ? s3m : one;
  R geo = P::add(P::add(P::div(P::add(P::div(w1p, g.d1s[i]), P::div(w1m, g.d1s[i - 1])), g.d1[i]),
                        P::div(P::add(P::div(w2p, g.d2s[j]), P::div(w2m, g.d2s[j - 1])), g.d2[j])),
                 P::div(P::add(P::div(w3p, g.d3s[k]), P::div(w3m, g.d3s[k - 1])), g.d3[k]));
  C aii = P::mk(-geo, 0);
  if (g.fvm) {
    C f = rmul<P>(P::mul(P::mul(g.d1s[i], g.d2[j]), g.d3[k]), sc.iom);
    aij = cmul<P>(aij, f);
    aii = cmul<P>(aii, f);
  }
  v[ixv(n1, n2, k, j, i)] = cdiv<P>(csub<P>(bv[ixv(n1, n2, k, j, i)], aij), aii);
  (void)kf;
}

// E = A + grad v (fdfd.c:796-819), in place on Y
template <class P>
__global__ void k_aphi_grad(SweepP<P> s, const typename P::C* __restrict__ VV)
{
  typedef typename P::C C;
  const int slot = blockIdx.z;
  const int sys = s.sys_list ? s.sys_list[slot] : slot;
  const GridP<P>& g = s.g;
  const int n1 = g.n1, n2 = g.n2, n3 = g.n3;
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= g.lE) return;
  const C* v = VV + (size_t)slot * s.lv;
  C* y = s.Y + (size_t)sys * g.lE;
  if (q < g.lEx) {
    int i = (int)(q % n1), j = (int)((q / n1) % (n2 + 1)), k = (int)(q / ((long)n1 * (n2 + 1)));
    if (k >= 1 && k < n3 && j >= 1 && j < n2)
      y[q] = cadd<P>(y[q], cdivs<P>(csub<P>(v[ixv(n1, n2, k, j, i + 1)], v[ixv(n1, n2, k, j, i)]), g.d1s[i], g.r1s[i]));
  } else if (q < g.lEx + g.lEy) {
    long r = q - g.lEx;
    int i = (int)(r % (n1 + 1)), j = (int)((r / (n1 + 1)) % n2), k = (int)(r / ((long)(n1 + 1) * n2));
    if (k >= 1 && k < n3 && i >= 1 && i < n1)
      y[q] = cadd<P>(y[q], cdivs<P>(csub<P>(v[ixv(n1, n2, k, j + 1, i)], v[ixv(n1, n2, k, j, i)]), g.d2s[j], g.r2s[j]));
  } else {
    long r = q - g.lEx - g.lEy;
    int i = (int)(r % (n1 + 1)), j = (int)((r / (n1 + 1)) % (n2 + 1)), k = (int)(r / ((long)(n1 + 1) * (n2 + 1)));
    if (k < n3 && j >= 1 && j < n2 && i >= 1 && i < n1)
      y[q] = cadd<P>(y[q], cdivs<P>(csub<P>(v[ixv(n1, n2, k + 1, j, i)], v[ixv(n1, n2, k, j, i)]), g.d3s[k], g.r3s[k]));
  }
}

int phi_diagonals(int n1, int n2, int n3) { return (n1 - 1) + (n2 - 1) + (n3 - 1) - 2; }  // t = 3 ..

template <class P>
void launch_aphi_div(const SweepP<P>& s, typename P::C* BV, int nslot, cudaStream_t st)
{
  dim3 grd((unsigned)((s.lv + 255) / 256), 1, nslot);
  count_launch(), k_aphi_div<P><<<grd, 256, 0, st>>>(s, BV);
}

template <class P>
void launch_aphi_phi(const SweepP<P>& s, typename P::C* V, int t, int nslot, cudaStream_t st)
{
  // t > 0: forward hyperplane t; t < 0: backward hyperplane -t
  dim3 blk(32, 4);
  dim3 grd((s.g.n1 - 1 + 31) / 32, (s.g.n2 - 1 + 3) / 4, nslot);
  if (t > 0) count_launch(), k_aphi_phi<P, true><<<grd, blk, 0, st>>>(s, V, t);
  else count_launch(), k_aphi_phi<P, false><<<grd, blk, 0, st>>>(s, V, -t);
}

template <class P>
void launch_aphi_grad(const SweepP<P>& s, const typename P::C* V, int nslot, cudaStream_t st)
{
  dim3 grd((unsigned)((s.g.lE + 255) / 256), 1, nslot);
  count_launch(), k_aphi_grad<P><<<grd, 256, 0, st>>>(s, V);
}

#define CSEM_INST(P)                                                                              \
  template void launch_sweep<P>(const SweepP<P>&, int, bool, bool, int, int, cudaStream_t);       \
  template void launch_aphi_div<P>(const SweepP<P>&, P::C*, int, cudaStream_t);                   \
  template void launch_aphi_phi<P>(const SweepP<P>&, P::C*, int, int, cudaStream_t);              \
  template void launch_aphi_grad<P>(const SweepP<P>&, const P::C*, int, cudaStream_t);
CSEM_INST(F64)
CSEM_INST(F32)
#undef CSEM_INST

}  // namespace csem
