// LU-SGS complex64 component sweeps that carry a group of systems at one frequency per CTA.
//
// The lockstep row pipelines of k_lusgs2.cu (one CTA per independent line, a thread per
// row, rows skewed by one march step, hand-over by warp shuffle and pairwise named
// barriers; fdfd.c:347-503 for the update), with NS systems per CTA. The systems of a
// group share the frequency, so everything a point's update takes from the grid and the
// frequency is loaded and computed once for the NS systems: the spacings, the
// conductivity and the shared part of the linear form (Coef32: 1/aii, w = iwmu/aii). Per
// system only b, the neighbour values and B = b/aii + w kc remain, and every warp carries
// NS independent chains where a single-system CTA has one. Each point is evaluated with
// the operations of k_sweep_ex32 / k_sweep_eyz32, so a system gets the values it gets in a
// single-system CTA up to the compiler's multiply-add contraction.
//
// Groups: groups[g * NS + q] is the slot of member q of group g, -1 when the group has
// fewer members (member 0 is always present); the host builds them from the systems'
// frequencies, so all members of a group have the same iom. A member's vectors are reached
// from member 0's row pointers by one element offset per plane: (its system - member 0's)
// lE in the vectors, (its slot - member 0's) capE in the air cap scratch.
#include "csem_cuda.cuh"
#include "engine.h"
#include "k_sweep_common.cuh"

namespace csem {

using namespace sweep;

namespace {

template <int NS> struct Members {
  bool ok[NS];
  long dY[NS], dC[NS];
};

template <int NS>
__device__ __forceinline__ void members_of(const SweepP<F32>& s, const int* gs, int& slot0, int& sys0, Members<NS>& mb)
{
  slot0 = gs[0];
  sys0 = s.sys_list ? s.sys_list[slot0] : slot0;
#pragma unroll
  for (int q = 0; q < NS; q++) {
    const int sl = q == 0 ? slot0 : gs[q];
    mb.ok[q] = sl >= 0;
    const int slq = sl >= 0 ? sl : slot0;
    const int syq = s.sys_list ? s.sys_list[slq] : slq;
    mb.dY[q] = (long)(syq - sys0) * s.g.lE;
    mb.dC[q] = (long)(slq - slot0) * s.capE;
  }
}

// member q's element offset, relative to member 0, for sweep plane k
template <int NS>
__device__ __forceinline__ long moff(const Members<NS>& mb, int q, int k, int vshift)
{
  return k >= vshift ? mb.dY[q] : mb.dC[q];
}

// resident CTAs per SM the register budget is sized for (CTAs of up to 256 threads)
template <int W> struct GroupMinBlocks {
  static constexpr int value = W >= 4 ? 1 : 2;
};

template <int VW, int NS> struct RawExG {
  float2 b[NS][VW], exjm[NS][VW], exkm[NS][VW], eyA[NS][VW], eyB[NS][VW], eyC[NS][VW], eyD[NS][VW], ezA[NS][VW],
      ezB[NS][VW], ezC[NS][VW], ezD[NS][VW];
  float sg[VW];
  Ax<F32> Y;
};

template <int VW, int NS> struct RawEyzG {
  float2 b[NS][VW], xA[NS][VW], xB[NS][VW], xC[NS][VW], xD[NS][VW], yA[NS][VW], yB[NS][VW], yC[NS][VW], yD[NS][VW],
      own2[NS][VW], rowold[NS][VW];
  float sg[VW];
  Ax<F32> X[VW];
};

}  // namespace

// Ex: rows k, march j, VW consecutive i per thread. grid (i groups, system groups)
template <bool FWD, int VW, int NS>
__global__ void __launch_bounds__(NB_ROWS, GroupMinBlocks<VW * NS>::value)
    k_sweep_ex32g(SweepP<F32> s, const int* groups)
{
  typedef float2 C;
  __shared__ HandOff<VW * NS, C, true> hand;
  int slot0, sys0;
  Members<NS> mb;
  members_of<NS>(s, groups + (size_t)blockIdx.y * NS, slot0, sys0, mb);
  const GridP<F32>& g = s.g;
  const int n1 = g.n1, n2 = g.n2, nK = s.nK;
  const View<F32> V = view_of<F32>(s, slot0, sys0);
  const SysScal<F32> sc = s.scal[sys0];
  const C z = make_float2(0.f, 0.f);
  const int R_ = nK - 1, M = n2 - 1;  // rows k = 1..R_, march j = 1..M
  const int rr = threadIdx.x;
  const bool rowok = rr < R_;
  const int k = FWD ? 1 + rr : R_ - rr;
  const int i0 = blockIdx.x * VW;
  const Ax<F32> Z = rowok ? axis<F32>(g.d3, g.d3s, g.r3, g.r3s, k) : Ax<F32>{};
  // member 0's rows at the line's first i, and each member's offsets for planes k, k-1
  C* ex0 = nullptr;
  const C *ex1 = nullptr, *ey0 = nullptr, *ez0 = nullptr, *ez1 = nullptr, *bb = nullptr;
  const float* sg0 = nullptr;
  long o0[NS], o1[NS];
#pragma unroll
  for (int q = 0; q < NS; q++) o0[q] = o1[q] = 0;
  if (rowok) {
    ex0 = V.row(0, k, 0) + i0;
    ex1 = V.row(0, k - 1, 0) + i0;
    ey0 = V.row(1, k, 0) + i0;
    ez0 = V.row(2, k, 0) + i0;
    ez1 = V.row(2, k - 1, 0) + i0;
    bb = V.brow(0, k, 0);
    if (bb) bb += i0;
    sg0 = g.s11 + ix1(n1, n2, k, 0, 0) + i0;
#pragma unroll
    for (int q = 0; q < NS; q++) {
      o0[q] = moff(mb, q, k, s.vshift);
      o1[q] = moff(mb, q, k - 1, s.vshift);
    }
  }
  const int L1 = n1 + 1;
  const float gn = Z.r * (FWD ? Z.rsm : Z.rs);
  Ax<F32> X[VW];
#pragma unroll
  for (int v = 0; v < VW; v++) X[v] = i0 + v < n1 ? axis_at<F32>(g.d1, g.d1s, g.r1, g.r1s, i0 + v) : Ax<F32>{};
  RawExG<VW, NS> raw;
  C B[NS][VW], w[VW];
  float gp = 0.f;
  auto load = [&](int c) {
    const int j = FWD ? 1 + c : M - c;
    raw.Y = axis<F32>(g.d2, g.d2s, g.r2, g.r2s, j);
    const int ox = j * n1, oy = j * L1;
#pragma unroll
    for (int v = 0; v < VW; v++) {
      if (i0 + v >= n1) continue;
      raw.sg[v] = ro(sg0 + ox + v);
#pragma unroll
      for (int q = 0; q < NS; q++) {
        if (!mb.ok[q]) continue;
        raw.b[q][v] = bb ? ro(bb + o0[q] + ox + v) : z;
        if (!FWD) {
          raw.exjm[q][v] = ex0[o0[q] + ox - n1 + v];
          raw.exkm[q][v] = ex1[o1[q] + ox + v];
          raw.eyA[q][v] = ro(ey0 + o0[q] + oy + v + 1);
          raw.eyB[q][v] = ro(ey0 + o0[q] + oy + v);
          raw.eyC[q][v] = ro(ey0 + o0[q] + oy - L1 + v + 1);
          raw.eyD[q][v] = ro(ey0 + o0[q] + oy - L1 + v);
          raw.ezA[q][v] = ro(ez0 + o0[q] + oy + v + 1);
          raw.ezB[q][v] = ro(ez0 + o0[q] + oy + v);
          raw.ezC[q][v] = ro(ez1 + o1[q] + oy + v + 1);
          raw.ezD[q][v] = ro(ez1 + o1[q] + oy + v);
        }
      }
    }
  };
  auto make = [&]() {
    const Ax<F32>& Y = raw.Y;
    const float gg = (Y.rs + Y.rsm) * Y.r + (Z.rs + Z.rsm) * Z.r;  // geo(Y, Z)
    gp = Y.r * (FWD ? Y.rsm : Y.rs);
#pragma unroll
    for (int v = 0; v < VW; v++) {
      if (i0 + v >= n1) continue;
      const Coef32 cf = lin_coef(sc, g.fvm, gg, raw.sg[v], X[v].ds * Y.d * Z.d);
      w[v] = cf.w;
#pragma unroll
      for (int q = 0; q < NS; q++) {
        if (!mb.ok[q]) continue;
        C kc = z;
        if (!FWD) {
          const C dy = sub32(sub32(raw.eyA[q][v], raw.eyB[q][v]), sub32(raw.eyC[q][v], raw.eyD[q][v]));
          const C dz = sub32(sub32(raw.ezA[q][v], raw.ezB[q][v]), sub32(raw.ezC[q][v], raw.ezD[q][v]));
          const C cross = scl32(X[v].rs, make_float2(Y.r * dy.x + Z.r * dz.x, Y.r * dy.y + Z.r * dz.y));
          const C known = make_float2(Y.r * Y.rsm * raw.exjm[q][v].x + Z.r * Z.rsm * raw.exkm[q][v].x,
                                      Y.r * Y.rsm * raw.exjm[q][v].y + Z.r * Z.rsm * raw.exkm[q][v].y);
          kc = sub32(known, cross);
        }
        B[q][v] = lin_B(cf, g.fvm, raw.b[q][v], kc);
      }
    }
  };
  C res[NS * VW];
#pragma unroll
  for (int e = 0; e < NS * VW; e++) res[e] = z;
  if (rowok && rr == 0 && M > 0) {
    load(0);
    make();
  }
  for (int T = 0; T < M + R_ - 1; T++) {
    const int c = T - rr;
    const bool act = rowok && c >= 0 && c < M;
    const bool nxt = rowok && c + 1 >= 0 && c + 1 < M;
    if (nxt) load(c + 1);
    C nb[NS * VW];
    hand.get(res, nb, T);
    if (act) {
      const int ox = (FWD ? 1 + c : M - c) * n1;
#pragma unroll
      for (int q = 0; q < NS; q++) {
#pragma unroll
        for (int v = 0; v < VW; v++) {
          const int e = q * VW + v;
          if (!mb.ok[q] || i0 + v >= n1) {
            res[e] = z;
            continue;
          }
          Lin32 L;
          L.B = B[q][v];
          L.w = w[v];
          L.gp = gp;
          L.gn = gn;
          const C val = lin_apply(L, c > 0 ? res[e] : z, nb[e]);  // prev: own row, previous j
          ex0[o0[q] + ox + v] = val;
          res[e] = val;
        }
      }
    } else {
#pragma unroll
      for (int e = 0; e < NS * VW; e++) res[e] = z;
    }
    hand.put(res, T);
    if (nxt) make();
  }
  hand.finish(M + R_ - 1);
}

// Ey (COMP 1: line j, rows k) / Ez (COMP 2: line k, rows j): march i in chunks of VW.
// grid (lines, system groups)
template <int COMP, bool FWD, int VW, int NS>
__global__ void __launch_bounds__(NB_ROWS, GroupMinBlocks<VW * NS>::value)
    k_sweep_eyz32g(SweepP<F32> s, const int* groups)
{
  typedef float2 C;
  __shared__ HandOff<VW * NS, C, true> hand;
  int slot0, sys0;
  Members<NS> mb;
  members_of<NS>(s, groups + (size_t)blockIdx.y * NS, slot0, sys0, mb);
  const GridP<F32>& g = s.g;
  const int n1 = g.n1, n2 = g.n2, nK = s.nK;
  const View<F32> V = view_of<F32>(s, slot0, sys0);
  const SysScal<F32> sc = s.scal[sys0];
  const C z = make_float2(0.f, 0.f);
  const int line = blockIdx.x;
  const int R_ = COMP == 1 ? nK - 1 : n2 - 1;  // rows k (Ey) or j (Ez) = 1..R_
  const int M = n1 - 1;                         // march i = 1..M
  const int NC = (M + VW - 1) / VW;
  const int rr = threadIdx.x;
  const bool rowok = rr < R_;
  const int r = FWD ? 1 + rr : R_ - rr;
  const int k = COMP == 1 ? r : line;
  const int j = COMP == 1 ? line : r;
  const Ax<F32> Rw = rowok ? (COMP == 1 ? axis<F32>(g.d3, g.d3s, g.r3, g.r3s, r) : axis<F32>(g.d2, g.d2s, g.r2, g.r2s, r))
                           : Ax<F32>{};
  const Ax<F32> LA = COMP == 1 ? axis_at<F32>(g.d2, g.d2s, g.r2, g.r2s, j) : axis_at<F32>(g.d3, g.d3s, g.r3, g.r3s, k);
  const float gn = Rw.r * (FWD ? Rw.rsm : Rw.rs);
  const float lrs = LA.rs, ld = LA.d;  // the line axis' rs and d
  // member 0's rows; the members' offsets for plane k (oA) and for the other plane the
  // update reads (oB: k - 1 for Ey, k + 1 for Ez)
  C* own = nullptr;
  const C *nxt = nullptr, *xa = nullptr, *xb = nullptr, *ya = nullptr, *yb = nullptr, *yc = nullptr, *yd = nullptr;
  const C* bb = nullptr;
  const float* sg0 = nullptr;
  long oA[NS], oB[NS];
#pragma unroll
  for (int q = 0; q < NS; q++) oA[q] = oB[q] = 0;
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
#pragma unroll
    for (int q = 0; q < NS; q++) {
      oA[q] = moff(mb, q, k, s.vshift);
      oB[q] = moff(mb, q, COMP == 1 ? k - 1 : k + 1, s.vshift);
    }
  }
  RawEyzG<VW, NS> raw;
  C B[NS][VW], w[VW];
  float gp[VW];
  auto load = [&](int c) {
#pragma unroll
    for (int v = 0; v < VW; v++) {
      const int m = c * VW + v;
      if (m >= M) continue;
      const int i = FWD ? 1 + m : M - m;
      raw.X[v] = axis<F32>(g.d1, g.d1s, g.r1, g.r1s, i);
      raw.sg[v] = ro(sg0 + i);
#pragma unroll
      for (int q = 0; q < NS; q++) {
        if (!mb.ok[q]) continue;
        const long a = oA[q], b2 = oB[q];
        const long oxa = COMP == 1 ? a : b2, oya = COMP == 1 ? a : b2, oyd = COMP == 1 ? b2 : a,
                   onx = COMP == 1 ? b2 : a;
        raw.b[q][v] = bb ? ro(bb + a + i) : z;
        raw.xA[q][v] = ro(xa + oxa + i);
        raw.xB[q][v] = ro(xb + a + i);
        raw.xC[q][v] = ro(xa + oxa + i - 1);
        raw.xD[q][v] = ro(xb + a + i - 1);
        if (COMP == 2 || !FWD) {
          raw.yA[q][v] = ro(ya + oya + i);
          raw.yB[q][v] = ro(yb + a + i);
          raw.yC[q][v] = ro(yc + b2 + i);
          raw.yD[q][v] = ro(yd + oyd + i);
        }
        if (!FWD) {
          raw.own2[q][v] = own[a + i - 1];
          raw.rowold[q][v] = nxt[onx + i];
        }
      }
    }
  };
  auto make = [&](int c) {
#pragma unroll
    for (int v = 0; v < VW; v++) {
      if (c * VW + v >= M) continue;
      const Ax<F32>& X = raw.X[v];
      const float gg = (X.rs + X.rsm) * X.r + (Rw.rs + Rw.rsm) * Rw.r;  // geo(Z, X) / geo(X, Y)
      const float ydd = COMP == 1 ? ld : Rw.d, zdd = COMP == 1 ? Rw.d : ld;  // Y.d and Z.d
      const Coef32 cf = lin_coef(sc, g.fvm, gg, raw.sg[v], X.ds * ydd * zdd);
      w[v] = cf.w;
      gp[v] = X.r * (FWD ? X.rsm : X.rs);
#pragma unroll
      for (int q = 0; q < NS; q++) {
        if (!mb.ok[q]) continue;
        const C dx = sub32(sub32(raw.xA[q][v], raw.xB[q][v]), sub32(raw.xC[q][v], raw.xD[q][v]));
        // Ey: Y.rs (Z.r dEz + X.r dEx); Ez: Z.rs (X.r dEx + Y.r dEy)
        C acc = scl32(X.r, dx);
        if (COMP == 2 || !FWD) {
          const C dy = sub32(sub32(raw.yA[q][v], raw.yB[q][v]), sub32(raw.yC[q][v], raw.yD[q][v]));
          acc = make_float2(acc.x + Rw.r * dy.x, acc.y + Rw.r * dy.y);
        }
        C kc = scl32(-lrs, acc);
        if (!FWD) {
          const C known = make_float2(X.r * X.rsm * raw.own2[q][v].x + Rw.r * Rw.rsm * raw.rowold[q][v].x,
                                      X.r * X.rsm * raw.own2[q][v].y + Rw.r * Rw.rsm * raw.rowold[q][v].y);
          kc = make_float2(kc.x + known.x, kc.y + known.y);
        }
        B[q][v] = lin_B(cf, g.fvm, raw.b[q][v], kc);
      }
    }
  };
  C res[NS * VW];
#pragma unroll
  for (int e = 0; e < NS * VW; e++) res[e] = z;
  if (rowok && rr == 0 && NC > 0) {
    load(0);
    make(0);
  }
  for (int T = 0; T < NC + R_ - 1; T++) {
    const int c = T - rr;
    const bool act = rowok && c >= 0 && c < NC;
    const bool nx = rowok && c + 1 >= 0 && c + 1 < NC;
    if (nx) load(c + 1);
    C nb[NS * VW];
    hand.get(res, nb, T);
    if (act) {
#pragma unroll
      for (int q = 0; q < NS; q++) {
        C prev = c > 0 ? res[q * VW + VW - 1] : z;  // own row at the previous march position
#pragma unroll
        for (int v = 0; v < VW; v++) {
          const int e = q * VW + v;
          const int m = c * VW + v;
          if (!mb.ok[q] || m >= M) {
            res[e] = z;
            continue;
          }
          Lin32 L;
          L.B = B[q][v];
          L.w = w[v];
          L.gp = gp[v];
          L.gn = gn;
          const C val = lin_apply(L, prev, nb[e]);
          own[oA[q] + (FWD ? 1 + m : M - m)] = val;
          res[e] = val;
          prev = val;
        }
      }
    } else {
#pragma unroll
      for (int e = 0; e < NS * VW; e++) res[e] = z;
    }
    hand.put(res, T);
    if (nx) make(c + 1);
  }
  hand.finish(NC + R_ - 1);
}

bool sweep_grouped_fits(int comp, int n1, int n2, int nK)
{
  const int rows = comp == 2 ? n2 - 1 : nK - 1;
  return rows >= 1 && rows <= NB_ROWS && n1 >= 2 && n2 >= 2;
}

template <int VW, int NS>
static void launch_grouped(const SweepP<F32>& s, int comp, bool fwd, const int* groups, int ngroups, cudaStream_t st)
{
  const int n1 = s.g.n1, n2 = s.g.n2, nK = s.nK;
  const int rows = comp == 2 ? n2 - 1 : nK - 1;
  const int threads = (rows + 31) / 32 * 32;
  if (comp == 0) {
    dim3 grd((n1 + VW - 1) / VW, ngroups);
    if (fwd) count_launch(), k_sweep_ex32g<true, VW, NS><<<grd, threads, 0, st>>>(s, groups);
    else count_launch(), k_sweep_ex32g<false, VW, NS><<<grd, threads, 0, st>>>(s, groups);
  } else if (comp == 1) {
    dim3 grd(n2, ngroups);
    if (fwd) count_launch(), k_sweep_eyz32g<1, true, VW, NS><<<grd, threads, 0, st>>>(s, groups);
    else count_launch(), k_sweep_eyz32g<1, false, VW, NS><<<grd, threads, 0, st>>>(s, groups);
  } else {
    dim3 grd(nK, ngroups);
    if (fwd) count_launch(), k_sweep_eyz32g<2, true, VW, NS><<<grd, threads, 0, st>>>(s, groups);
    else count_launch(), k_sweep_eyz32g<2, false, VW, NS><<<grd, threads, 0, st>>>(s, groups);
  }
}

// ns systems per CTA (2 or 4), vw points per thread and step (1 or 2; 4 systems take 1)
void launch_sweep_grouped(const SweepP<F32>& s, int comp, bool fwd, const int* groups, int ngroups, int ns, int vw,
                          cudaStream_t st)
{
  if (ns == 4) launch_grouped<1, 4>(s, comp, fwd, groups, ngroups, st);
  else if (vw == 2) launch_grouped<2, 2>(s, comp, fwd, groups, ngroups, st);
  else launch_grouped<1, 2>(s, comp, fwd, groups, ngroups, st);
}

}  // namespace csem
