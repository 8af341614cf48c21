// y = A x: the staggered-grid curl-curl operator of fdfd_apply (fdfd.c:86-205).
//
// One CTA owns a 31 x BY tile of (i,j) columns plus a one-column and one-row halo on the
// low sides (the halo threads only compute H) and marches a chunk of z-planes. At each
// plane it computes H = curl E / (i omega mu0) for its columns (fdfd.c:125-149), trades
// the neighbouring values by warp shuffles and shared memory, and produces
// y = curl H - sigma E for the tile (fdfd.c:176-203). H is never written to HBM, so one
// pass reads x and sigma and writes y.
//
// With the airwave boundary (airbc=1) the k=0 rows of bx/by use the ghost fields
// Hx(z=-dz/2), Hy(z=-dz/2) that the airwave pipeline derives from Hz(z=0)
// (fdfd.c:151-172); k_hz0 provides that Hz plane.
#include "csem_cuda.cuh"
#include "engine.h"
#include "k_dot_common.cuh"

namespace csem {

template <class P>
__device__ __forceinline__ void h_at(const GridP<P>& g, const typename P::C* __restrict__ Ex,
                                     const typename P::C* __restrict__ Ey, const typename P::C* __restrict__ Ez,
                                     typename P::C iwmu, int k, int j, int i, typename P::C& hx,
                                     typename P::C& hy, typename P::C& hz)
{
  typedef typename P::C C;
  const int n1 = g.n1, n2 = g.n2, n3 = g.n3, kf = k + g.kstart;
  hx = hy = hz = czero<P>();
  if (i < 0 || j < 0 || i > n1 || j > n2) return;
  if (j < n2 && k < n3) {  // Hx = (dEz/dy - dEy/dz) / (i w mu0)
    C t1 = cdivs<P>(csub<P>(Ez[ix3(n1, n2, k, j + 1, i)], Ez[ix3(n1, n2, k, j, i)]), g.d2s[j], g.r2s[j]);
    C t2 = cdivs<P>(csub<P>(Ey[ix2(n1, n2, k + 1, j, i)], Ey[ix2(n1, n2, k, j, i)]), g.d3s[kf], g.r3s[kf]);
    hx = cmul<P>(csub<P>(t1, t2), iwmu);
  }
  if (i < n1 && k < n3) {  // Hy = (dEx/dz - dEz/dx) / (i w mu0)
    C t1 = cdivs<P>(csub<P>(Ex[ix1(n1, n2, k + 1, j, i)], Ex[ix1(n1, n2, k, j, i)]), g.d3s[kf], g.r3s[kf]);
    C t2 = cdivs<P>(csub<P>(Ez[ix3(n1, n2, k, j, i + 1)], Ez[ix3(n1, n2, k, j, i)]), g.d1s[i], g.r1s[i]);
    hy = cmul<P>(csub<P>(t1, t2), iwmu);
  }
  if (i < n1 && j < n2) {  // Hz = (dEy/dx - dEx/dy) / (i w mu0)
    C t1 = cdivs<P>(csub<P>(Ey[ix2(n1, n2, k, j, i + 1)], Ey[ix2(n1, n2, k, j, i)]), g.d1s[i], g.r1s[i]);
    C t2 = cdivs<P>(csub<P>(Ex[ix1(n1, n2, k, j + 1, i)], Ex[ix1(n1, n2, k, j, i)]), g.d2s[j], g.r2s[j]);
    hz = cmul<P>(csub<P>(t1, t2), iwmu);
  }
}

// One warp per j row and one lane per i column: lanes cover i = 31*bx - 1 .. 31*bx + 30
// (lane 0 is the i-1 halo), warps cover j = BY*by - 1 .. BY*by + BY - 1 (warp 0 is the
// j-1 halo). Each thread keeps Ex and Ey of the next plane in registers for the plane
// after, gets the i+1 neighbours of Ey and Ez from the next lane, the i-1 neighbours of
// Hy and Hz from the previous lane, and the j-1 neighbours of Hx and Hz from the
// previous warp through shared memory (double-buffered by plane parity, one barrier per
// plane). Its column's spacings stay in registers and its element offsets advance by one
// plane stride per plane; the plane's spacings are uniform loads. H is evaluated exactly
// as in h_at, so complex128 results keep their bits.
// resident CTAs per SM the complex64 stencil's register budget is sized for (a build may
// set CSEM_FDFD_MINB to try others); 544-thread CTAs (BY = 16) get one, i.e. no cap below
// the 255 registers a thread may hold, as three of them would leave 32 per thread
#ifndef CSEM_FDFD_MINB
#define CSEM_FDFD_MINB 3
#endif
//
// EPI > 0 (complex64) folds the Krylov dot products of the result into the pass: EPI 1
// sums y conj(e) (BiCGStab's v.r0 after v = A p), EPI 2 sums e conj(y) and y conj(y) (s.t
// and t.t after t = A s), e read at the outputs' own indices. Each thread accumulates as
// the dot-product kernels do (compensated float pairs), the CTA sums its threads in a
// fixed tree and order, and writes part[slot][cta] (EPI 2: and part[nslot + slot][cta]),
// which launch_dot_finish adds up in a fixed order: deterministic, but a different
// partition of the sum than launch_dot's.
template <class P, int BY, int EPI>
__global__ void __launch_bounds__(32 * (BY + 1), sizeof(typename P::R) == 8 || BY >= 16 ? 1 : CSEM_FDFD_MINB)
k_fdfd(GridP<P> g, const SysScal<P>* __restrict__ scal, const typename P::C* __restrict__ X,
       typename P::C* __restrict__ Y, const typename P::C* __restrict__ GHX,
       const typename P::C* __restrict__ GHY, int kchunk, int nkc, const int* __restrict__ sys_list,
       const typename P::C* __restrict__ E, double2* __restrict__ part)
{
  typedef typename P::C C;
  typedef typename P::R R;
  __shared__ C sHx[2][BY + 1][32], sHz[2][BY + 1][32];
  const int lane = threadIdx.x, w = threadIdx.y;
  const int i = blockIdx.x * 31 + lane - 1;
  const int j = blockIdx.y * BY + w - 1;
  const int slot = blockIdx.z / nkc, kc = blockIdx.z % nkc;
  const int sys = sys_list ? sys_list[slot] : slot;
  const int n1 = g.n1, n2 = g.n2, n3 = g.n3, ks = g.kstart;
  const C* Ex = X + (size_t)sys * g.lE;
  const C* Ey = Ex + g.lEx;
  const C* Ez = Ey + g.lEy;
  C* bx = Y + (size_t)sys * g.lE;
  C* by = bx + g.lEx;
  C* bz = by + g.lEy;
  const C* epx = EPI ? E + (size_t)sys * g.lE : nullptr;  // the dot products' other vector
  const C* epy = EPI ? epx + g.lEx : nullptr;
  const C* epz = EPI ? epy + g.lEy : nullptr;
  DotAcc<P> dacc1, dacc2;
  auto dot = [&](C y, const C* e, long o) {
    if constexpr (EPI == 1) {
      dacc1.add(y, e[o]);
    } else if constexpr (EPI == 2) {
      dacc1.add(e[o], y);
      dacc2.add(y, y);
    }
  };
  const C iwmu = scal[sys].iwmu, iom = scal[sys].iom;
  const C* ghx = GHX ? GHX + (size_t)slot * (n1 + 1) * n2 : nullptr;  // ghosts are per slot
  const C* ghy = GHY ? GHY + (size_t)slot * n1 * (n2 + 1) : nullptr;
  const int kb = kc * kchunk;
  const int ke = min(n3 + 1, kb + kchunk);
  const bool inside = i >= 0 && j >= 0 && i <= n1 && j <= n2;  // H is zero outside
  const bool interior = lane >= 1 && w >= 1 && inside;        // this thread writes y
  const C z = czero<P>();
  const bool hasEx = inside && i < n1, hasEy = inside && j < n2;
  const bool hasExj = hasEx && j < n2;  // Ex(k, j+1, i) exists
  // the column's spacings
  const int ic = inside ? i : 0, jc = inside ? j : 0;
  const R d1s = g.d1s[ic], r1s = g.r1s[ic], d1 = g.d1[ic], r1 = g.r1[ic];
  const R d2s = g.d2s[jc], r2s = g.r2s[jc], d2 = g.d2[jc], r2 = g.r2[jc];
  // which outputs this column has, apart from the plane condition
  const bool outX = interior && i < n1, outY = interior && j < n2, outZ = interior;
  const bool inX = j >= 1 && j <= n2 - 1, inY = i >= 1 && i <= n1 - 1, inZ = inX && inY;
  // element offsets at plane k (the same for x, y and, plane-shifted, for sigma)
  const long sEx = (long)n1 * (n2 + 1), sEy = (long)(n1 + 1) * n2, sEz = (long)(n1 + 1) * (n2 + 1);
  long oEx = inside ? ix1(n1, n2, kb, j, i) : 0;
  long oEy = inside ? ix2(n1, n2, kb, j, i) : 0;
  long oEz = inside ? ix3(n1, n2, kb, j, i) : 0;
  const R* s11 = g.s11 + ks * sEx;
  const R* s22 = g.s22 + ks * sEy;
  const R* s33 = g.s33 + ks * sEz;

  C pHx = z, pHy = z, hx, hy, hz;
  if (kb > 0) {
    h_at<P>(g, Ex, Ey, Ez, iwmu, kb - 1, j, i, hx, hy, hz);
    pHx = hx;
    pHy = hy;
  }
  C exk = hasEx && kb <= n3 ? Ex[oEx] : z;
  C eyk = hasEy && kb <= n3 ? Ey[oEy] : z;
  // the loads of one plane: Ez, the j+1 neighbours, Ex and Ey of the plane above, and
  // sigma; issued one plane ahead of their use
  struct PlaneIn {
    C ez, ezj, exj, ex1, ey1;
    R s1, s2, s3;
  };
  auto load_plane = [&](int k, long oX, long oY, long oZ) {
    PlaneIn p;
    const bool kin = k < n3;
    p.ez = inside && kin ? Ez[oZ] : z;
    p.ezj = hasEy && kin ? Ez[oZ + (n1 + 1)] : z;
    p.exj = hasExj ? Ex[oX + n1] : z;
    p.ex1 = hasEx && kin ? Ex[oX + sEx] : z;
    p.ey1 = hasEy && kin ? Ey[oY + sEy] : z;
    p.s1 = outX ? s11[oX] : R(0);
    p.s2 = outY ? s22[oY] : R(0);
    p.s3 = outZ && kin ? s33[oZ] : R(0);
    return p;
  };
  PlaneIn nxt = load_plane(kb, oEx, oEy, oEz);
  for (int k = kb; k < ke; k++, oEx += sEx, oEy += sEy, oEz += sEz) {
    const int kf = k + ks;
    const int pb = k & 1;
    const bool kin = k < n3;
    const PlaneIn cur = nxt;
    if (k + 1 < ke) nxt = load_plane(k + 1, oEx + sEx, oEy + sEy, oEz + sEz);
    const R d3s = g.d3s[kf], r3s = g.r3s[kf], d3 = g.d3[kf], r3 = g.r3[kf];
    const C ez = cur.ez, ezj = cur.ezj, exj = cur.exj, ex1 = cur.ex1, ey1 = cur.ey1;
    C ezi, eyi;  // Ez(k, j, i+1), Ey(k, j, i+1): the next lane's, loaded by the last lane
    ezi.x = __shfl_down_sync(0xffffffffu, ez.x, 1);
    ezi.y = __shfl_down_sync(0xffffffffu, ez.y, 1);
    eyi.x = __shfl_down_sync(0xffffffffu, eyk.x, 1);
    eyi.y = __shfl_down_sync(0xffffffffu, eyk.y, 1);
    if (lane == 31) {
      ezi = hasEx && kin ? Ez[oEz + 1] : z;
      eyi = hasExj ? Ey[oEy + 1] : z;
    }
    // H at (k, j, i), the operations of h_at
    hx = hy = hz = z;
    if (hasEy && kin) {
      C t1 = cdivs<P>(csub<P>(ezj, ez), d2s, r2s);
      C t2 = cdivs<P>(csub<P>(ey1, eyk), d3s, r3s);
      hx = cmul<P>(csub<P>(t1, t2), iwmu);
    }
    if (hasEx && kin) {
      C t1 = cdivs<P>(csub<P>(ex1, exk), d3s, r3s);
      C t2 = cdivs<P>(csub<P>(ezi, ez), d1s, r1s);
      hy = cmul<P>(csub<P>(t1, t2), iwmu);
    }
    if (hasExj) {
      C t1 = cdivs<P>(csub<P>(eyi, eyk), d1s, r1s);
      C t2 = cdivs<P>(csub<P>(exj, exk), d2s, r2s);
      hz = cmul<P>(csub<P>(t1, t2), iwmu);
    }
    sHx[pb][w][lane] = hx;
    sHz[pb][w][lane] = hz;
    C hyl, hzl;  // Hy(k, j, i-1), Hz(k, j, i-1) from the previous lane
    hyl.x = __shfl_up_sync(0xffffffffu, hy.x, 1);
    hyl.y = __shfl_up_sync(0xffffffffu, hy.y, 1);
    hzl.x = __shfl_up_sync(0xffffffffu, hz.x, 1);
    hzl.y = __shfl_up_sync(0xffffffffu, hz.y, 1);
    __syncthreads();
    if (interior) {
      const C hxd = sHx[pb][w - 1][lane], hzd = sHz[pb][w - 1][lane];  // at j-1
      const bool kxy = (k >= 1 && k <= n3 - 1) || (k == 0 && g.airbc);
      if (outX) {  // bx
        C r = z;
        if (inX && kxy) {
          C hyb = k >= 1 ? pHy : ghy[i + (long)n1 * j];
          C t1 = cdivs<P>(csub<P>(hz, hzd), d2, r2);
          C t2 = cdivs<P>(csub<P>(hy, hyb), d3, r3);
          r = csub<P>(csub<P>(t1, t2), rmul<P>(cur.s1, exk));
          if (g.fvm) r = cmul<P>(r, rmul<P>(P::mul(P::mul(d1s, d2), d3), iom));
        }
        bx[oEx] = r;
        if (EPI) dot(r, epx, oEx);
      }
      if (outY) {  // by
        C r = z;
        if (inY && kxy) {
          C hxb = k >= 1 ? pHx : ghx[i + (long)(n1 + 1) * j];
          C t1 = cdivs<P>(csub<P>(hx, hxb), d3, r3);
          C t2 = cdivs<P>(csub<P>(hz, hzl), d1, r1);
          r = csub<P>(csub<P>(t1, t2), rmul<P>(cur.s2, eyk));
          if (g.fvm) r = cmul<P>(r, rmul<P>(P::mul(P::mul(d1, d2s), d3), iom));
        }
        by[oEy] = r;
        if (EPI) dot(r, epy, oEy);
      }
      if (outZ && kin) {  // bz
        C r = z;
        if (inZ) {
          C t1 = cdivs<P>(csub<P>(hy, hyl), d1, r1);
          C t2 = cdivs<P>(csub<P>(hx, hxd), d2, r2);
          r = csub<P>(csub<P>(t1, t2), rmul<P>(cur.s3, ez));
          if (g.fvm) r = cmul<P>(r, rmul<P>(P::mul(P::mul(d1, d2), d3s), iom));
        }
        bz[oEz] = r;
        if (EPI) dot(r, epz, oEz);
      }
    }
    pHx = hx;
    pHy = hy;
    exk = ex1;
    eyk = ey1;
  }
  if constexpr (EPI > 0) {
    __shared__ double2 red[2][BY + 1];
    const double2 v1 = warp_sum(dacc1.value());
    const double2 v2 = EPI == 2 ? warp_sum(dacc2.value()) : make_double2(0, 0);
    if (lane == 0) {
      red[0][w] = v1;
      red[1][w] = v2;
    }
    __syncthreads();
    if (w == 0 && lane == 0) {
      double2 a1 = make_double2(0, 0), a2 = make_double2(0, 0);
      for (int q = 0; q <= BY; q++) {
        a1.x = __dadd_rn(a1.x, red[0][q].x);
        a1.y = __dadd_rn(a1.y, red[0][q].y);
        a2.x = __dadd_rn(a2.x, red[1][q].x);
        a2.y = __dadd_rn(a2.y, red[1][q].y);
      }
      const int npart = gridDim.x * gridDim.y * nkc, nslot = gridDim.z / nkc;
      const int cta = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * kc);
      part[(size_t)slot * npart + cta] = a1;
      if (EPI == 2) part[(size_t)(nslot + slot) * npart + cta] = a2;
    }
  }
}

// Hz on the plane k=0 (operator grid) for the airwave: out[sys][j][i], i<n1, j<n2
template <class P>
__global__ void k_hz0(GridP<P> g, const SysScal<P>* __restrict__ scal, const typename P::C* __restrict__ X,
                      typename P::C* __restrict__ out, const int* __restrict__ sys_list)
{
  const int slot = blockIdx.z;
  const int sys = sys_list ? sys_list[slot] : slot;
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= g.n1 || j >= g.n2) return;
  const typename P::C* Ex = X + (size_t)sys * g.lE;
  const typename P::C* Ey = Ex + g.lEx;
  const typename P::C* Ez = Ey + g.lEy;
  typename P::C hx, hy, hz;
  h_at<P>(g, Ex, Ey, Ez, scal[sys].iwmu, 0, j, i, hx, hy, hz);
  out[(size_t)slot * g.n1 * g.n2 + i + (long)g.n1 * j] = hz;
}

int sm_count()
{
  static int sms[64] = {};  // per device, queried once
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  if (!sms[dev] && cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    (void)cudaGetLastError();
    sms[dev] = 152;
  }
  return sms[dev];
}

// by: output rows per CTA (4, 8 or 16; other values: 8); ctas_per_sm: how many CTAs per
// SM the grid aims for when it splits the planes into chunks (other than 1..16: 4), which
// sets the z-block depth. Neither changes any result: every output takes the same
// operands in the same operations.
struct FdfdShape {
  int gx, gy, nkc, kchunk;
};
static FdfdShape fdfd_shape(int n1, int n2, int n3, int nsys, int by, int ctas_per_sm)
{
  if (by != 4 && by != 16) by = 8;
  if (ctas_per_sm < 1 || ctas_per_sm > 16) ctas_per_sm = 4;
  FdfdShape f;
  f.gx = (n1 + 1 + 30) / 31;
  f.gy = (n2 + 1 + by - 1) / by;
  const long base = (long)f.gx * f.gy * nsys;
  // split the planes into chunks until about ctas_per_sm CTAs per SM are in the grid
  int nkc = (int)(((long)ctas_per_sm * sm_count() + base - 1) / base);
  const int maxc = (n3 + 1) / 8 > 0 ? (n3 + 1) / 8 : 1;  // chunks of at least 8 planes
  if (nkc > maxc) nkc = maxc;
  if (nkc < 1) nkc = 1;
  f.kchunk = (n3 + 1 + nkc - 1) / nkc;
  f.nkc = (n3 + 1 + f.kchunk - 1) / f.kchunk;
  return f;
}

int fdfd_partials(int n1, int n2, int n3, int nsys, int by, int ctas_per_sm)
{
  const FdfdShape f = fdfd_shape(n1, n2, n3, nsys, by, ctas_per_sm);
  return f.gx * f.gy * f.nkc;
}

template <class P, int BY, int EPI>
static void launch_fdfd_by(const GridP<P>& g, const SysScal<P>* scal, const typename P::C* X, typename P::C* Y,
                           const typename P::C* ghx, const typename P::C* ghy, int nsys, const int* sys_list,
                           cudaStream_t st, int ctas_per_sm, const typename P::C* E, double2* part)
{
  const FdfdShape f = fdfd_shape(g.n1, g.n2, g.n3, nsys, BY, ctas_per_sm);
  dim3 blk(32, BY + 1);
  dim3 grd(f.gx, f.gy, nsys * f.nkc);
  count_launch(), k_fdfd<P, BY, EPI><<<grd, blk, 0, st>>>(g, scal, X, Y, ghx, ghy, f.kchunk, f.nkc, sys_list, E, part);
}

template <class P, int EPI>
static void launch_fdfd_epi(const GridP<P>& g, const SysScal<P>* scal, const typename P::C* X, typename P::C* Y,
                            const typename P::C* ghx, const typename P::C* ghy, int nsys, const int* sys_list,
                            cudaStream_t st, int by, int ctas_per_sm, const typename P::C* E, double2* part)
{
  if (by == 4) launch_fdfd_by<P, 4, EPI>(g, scal, X, Y, ghx, ghy, nsys, sys_list, st, ctas_per_sm, E, part);
  else if (by == 16) launch_fdfd_by<P, 16, EPI>(g, scal, X, Y, ghx, ghy, nsys, sys_list, st, ctas_per_sm, E, part);
  else launch_fdfd_by<P, 8, EPI>(g, scal, X, Y, ghx, ghy, nsys, sys_list, st, ctas_per_sm, E, part);
}

template <class P>
void launch_fdfd(const GridP<P>& g, const SysScal<P>* scal, const typename P::C* X, typename P::C* Y,
                 const typename P::C* ghx, const typename P::C* ghy, int nsys, const int* sys_list,
                 cudaStream_t st, int by, int ctas_per_sm)
{
  launch_fdfd_epi<P, 0>(g, scal, X, Y, ghx, ghy, nsys, sys_list, st, by, ctas_per_sm, nullptr, nullptr);
}

void launch_fdfd_dot(const GridP<F32>& g, const SysScal<F32>* scal, const float2* X, float2* Y, const float2* ghx,
                     const float2* ghy, int nsys, const int* sys_list, cudaStream_t st, int by, int ctas_per_sm,
                     int kind, const float2* E, double2* part)
{
  if (kind == 2) launch_fdfd_epi<F32, 2>(g, scal, X, Y, ghx, ghy, nsys, sys_list, st, by, ctas_per_sm, E, part);
  else launch_fdfd_epi<F32, 1>(g, scal, X, Y, ghx, ghy, nsys, sys_list, st, by, ctas_per_sm, E, part);
}

template <class P>
void launch_hz0(const GridP<P>& g, const SysScal<P>* scal, const typename P::C* X, typename P::C* out,
                int nsys, const int* sys_list, cudaStream_t st)
{
  dim3 blk(32, 8);
  dim3 grd((g.n1 + 31) / 32, (g.n2 + 7) / 8, nsys);
  count_launch(), k_hz0<P><<<grd, blk, 0, st>>>(g, scal, X, out, sys_list);
}

template void launch_fdfd<F64>(const GridP<F64>&, const SysScal<F64>*, const double2*, double2*,
                               const double2*, const double2*, int, const int*, cudaStream_t, int, int);
template void launch_fdfd<F32>(const GridP<F32>&, const SysScal<F32>*, const float2*, float2*,
                               const float2*, const float2*, int, const int*, cudaStream_t, int, int);
template void launch_fdfd<F64Q>(const GridP<F64Q>&, const SysScal<F64Q>*, const double2*, double2*,
                                const double2*, const double2*, int, const int*, cudaStream_t, int, int);
template void launch_hz0<F64>(const GridP<F64>&, const SysScal<F64>*, const double2*, double2*, int,
                              const int*, cudaStream_t);
template void launch_hz0<F32>(const GridP<F32>&, const SysScal<F32>*, const float2*, float2*, int,
                              const int*, cudaStream_t);

}  // namespace csem
