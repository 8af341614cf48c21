// LU-SGS complex64 component sweeps split into a coalesced pass and a light sweep.
//
// In the linear form of the complex64 sweeps (k_sweep_common.cuh), a point's value is
// v = B + w (gp prev + gn nb): prev and nb are the only values written during the sweep
// before the point is reached (the own row's previous march position and the previous
// row at the same position, fdfd.c:347-503), and everything else B and w take - b, the
// conductivity, the spacings, the other two components and the own component's
// neighbours the sweep has not reached yet - holds the same value from the start of the
// sweep to the moment the point is evaluated. So:
//   * k_lusgs_prep computes B and w of every point of the sweep in one pass with a
//     thread per point along i, i.e. coalesced loads of all those operands, and stores
//     (B, w) as one 16-byte value per point and system (scratch SB, the component's
//     layout on the sweep grid, one block of sbs values per slot);
//   * the sweep (k_sweep_ex32s / k_sweep_eyz32s: the lockstep row pipelines of
//     k_lusgs2.cu, a thread per row) then reads one 16-byte value per point and the
//     spacings of the march axis, runs the chain and stores v.
// In the pipelined sweeps every operand load is a warp access with one lane per row, so
// each touches about as many 32-byte sectors as the warp has rows; moving them into the
// coalesced pass leaves the sweep one such access per point instead of up to twelve.
// B and w are the expressions of k_sweep_ex32 / k_sweep_eyz32's make(), so the values
// are those sweeps' up to the compiler's multiply-add contraction.
//
// The pass takes groups of slots at one frequency (a thread forms the point's 1/aii and w
// once for the group); the pipeline is instantiated per warp count so that its pairwise
// barrier ids are immediates (2 NW - 1 hardware barriers per CTA instead of 16), and may
// run a capped grid whose CTAs take lines in turn. Engine side (Ops::apply_lusgs): batches
// of 8 or more systems run as two halves on two streams.
#include "csem_cuda.cuh"
#include "engine.h"
#include "k_sweep_common.cuh"

namespace csem {

using namespace sweep;

namespace {

constexpr int PREP_THREADS = 128;

__device__ __forceinline__ float4 pack(float2 B, float2 w) { return make_float4(B.x, B.y, w.x, w.y); }

}  // namespace

// (B, w) of every point the sweep of component COMP in direction FWD updates.
// grid (i chunks x groups, j, k); the sweep's points: Ex k 1..nK-1, j 1..n2-1, i 0..n1-1;
// Ey k 1..nK-1, j 0..n2-1, i 1..n1-1; Ez k 0..nK-1, j 1..n2-1, i 1..n1-1.
// NS = 1: a group is one slot (blockIdx.x / nch); NS > 1: groups[g * NS + q] is the slot
// of member q of group g (-1: absent), all members at one frequency, so a thread loads
// the point's conductivity and spacings and forms 1/aii and w once for its group.
template <int COMP, bool FWD, int NS>
__global__ void __launch_bounds__(PREP_THREADS)
    k_lusgs_prep(SweepP<F32> s, float4* SB, long sbs, int nch, const int* groups)
{
  typedef float2 C;
  const int grp = blockIdx.x / nch;
  const int i = (blockIdx.x - grp * nch) * PREP_THREADS + threadIdx.x;
  const int j = blockIdx.y, k = blockIdx.z;
  const GridP<F32>& g = s.g;
  const int n1 = g.n1, n2 = g.n2, nK = s.nK;
  if (COMP == 0) {
    if (i >= n1 || j < 1 || j > n2 - 1 || k < 1 || k > nK - 1) return;
  } else if (COMP == 1) {
    if (i < 1 || i > n1 - 1 || j > n2 - 1 || k < 1 || k > nK - 1) return;
  } else {
    if (i < 1 || i > n1 - 1 || j < 1 || j > n2 - 1 || k > nK - 1) return;
  }
  const int* gs = NS > 1 ? groups + (size_t)grp * NS : nullptr;
  const int slot0 = NS > 1 ? gs[0] : grp;
  const SysScal<F32> sc = s.scal[s.sys_list ? s.sys_list[slot0] : slot0];
  const C z = make_float2(0.f, 0.f);
  if (COMP == 0) {
    const Ax<F32> X = axis_at<F32>(g.d1, g.d1s, g.r1, g.r1s, i);
    const Ax<F32> Y = axis<F32>(g.d2, g.d2s, g.r2, g.r2s, j);
    const Ax<F32> Z = axis<F32>(g.d3, g.d3s, g.r3, g.r3s, k);
    const float gg = (Y.rs + Y.rsm) * Y.r + (Z.rs + Z.rsm) * Z.r;  // geo(Y, Z)
    const long o = ix1(n1, n2, k, j, i);
    const Coef32 cf = lin_coef(sc, g.fvm, gg, ro(g.s11 + o), X.ds * Y.d * Z.d);
#pragma unroll 1
    for (int q = 0; q < NS; q++) {
      const int slot = NS > 1 ? gs[q] : slot0;
      if (slot < 0) continue;
      const View<F32> V = view_of<F32>(s, slot, s.sys_list ? s.sys_list[slot] : slot);
      const C* bb = V.brow(0, k, j);
      const C b = bb ? ro(bb + i) : z;
      C kc = z;
      if (!FWD) {
        const C* ey0 = V.row(1, k, j);
        const C* ey1 = V.row(1, k, j - 1);
        const C* ez0 = V.row(2, k, j);
        const C* ez1 = V.row(2, k - 1, j);
        const C dy = sub32(sub32(ro(ey0 + i + 1), ro(ey0 + i)), sub32(ro(ey1 + i + 1), ro(ey1 + i)));
        const C dz = sub32(sub32(ro(ez0 + i + 1), ro(ez0 + i)), sub32(ro(ez1 + i + 1), ro(ez1 + i)));
        const C cross = scl32(X.rs, make_float2(Y.r * dy.x + Z.r * dz.x, Y.r * dy.y + Z.r * dz.y));
        const C exjm = ro(V.row(0, k, j - 1) + i), exkm = ro(V.row(0, k - 1, j) + i);
        const C known = make_float2(Y.r * Y.rsm * exjm.x + Z.r * Z.rsm * exkm.x,
                                    Y.r * Y.rsm * exjm.y + Z.r * Z.rsm * exkm.y);
        kc = sub32(known, cross);
      }
      SB[(size_t)slot * sbs + o] = pack(lin_B(cf, g.fvm, b, kc), cf.w);
    }
  } else {
    // Ey: row axis Z (k), line axis Y (j); Ez: row axis Y (j), line axis Z (k)
    const Ax<F32> Rw = COMP == 1 ? axis<F32>(g.d3, g.d3s, g.r3, g.r3s, k) : axis<F32>(g.d2, g.d2s, g.r2, g.r2s, j);
    const Ax<F32> LA = COMP == 1 ? axis_at<F32>(g.d2, g.d2s, g.r2, g.r2s, j) : axis_at<F32>(g.d3, g.d3s, g.r3, g.r3s, k);
    const Ax<F32> X = axis<F32>(g.d1, g.d1s, g.r1, g.r1s, i);
    const long o = (COMP == 1 ? ix2(n1, n2, k, j, 0) : ix3(n1, n2, k, j, 0)) + i;
    const float gg = (X.rs + X.rsm) * X.r + (Rw.rs + Rw.rsm) * Rw.r;  // geo(Z, X) / geo(X, Y)
    const float ydd = COMP == 1 ? LA.d : Rw.d, zdd = COMP == 1 ? Rw.d : LA.d;  // Y.d and Z.d
    const Coef32 cf = lin_coef(sc, g.fvm, gg, ro((COMP == 1 ? g.s22 : g.s33) + o), X.ds * ydd * zdd);
#pragma unroll 1
    for (int q = 0; q < NS; q++) {
      const int slot = NS > 1 ? gs[q] : slot0;
      if (slot < 0) continue;
      const View<F32> V = view_of<F32>(s, slot, s.sys_list ? s.sys_list[slot] : slot);
      const C *own, *nxt, *xa, *xb, *ya, *yb, *yc, *yd;
      if (COMP == 1) {
        own = V.row(1, k, j);
        nxt = V.row(1, k - 1, j);
        xa = V.row(0, k, j + 1);
        xb = V.row(0, k, j);
        ya = V.row(2, k, j + 1);
        yb = V.row(2, k, j);
        yc = V.row(2, k - 1, j + 1);
        yd = V.row(2, k - 1, j);
      } else {
        own = V.row(2, k, j);
        nxt = V.row(2, k, j - 1);
        xa = V.row(0, k + 1, j);
        xb = V.row(0, k, j);
        ya = V.row(1, k + 1, j);
        yb = V.row(1, k, j);
        yc = V.row(1, k + 1, j - 1);
        yd = V.row(1, k, j - 1);
      }
      const C* bb = V.brow(COMP, k, j);
      const C b = bb ? ro(bb + i) : z;
      const C dx = sub32(sub32(ro(xa + i), ro(xb + i)), sub32(ro(xa + i - 1), ro(xb + i - 1)));
      // Ey: Y.rs (Z.r dEz + X.r dEx); Ez: Z.rs (X.r dEx + Y.r dEy)
      C acc = scl32(X.r, dx);
      if (COMP == 2 || !FWD) {
        const C dy = sub32(sub32(ro(ya + i), ro(yb + i)), sub32(ro(yc + i), ro(yd + i)));
        acc = make_float2(acc.x + Rw.r * dy.x, acc.y + Rw.r * dy.y);
      }
      C kc = scl32(-LA.rs, acc);
      if (!FWD) {
        const C own2 = ro(own + i - 1), rowold = ro(nxt + i);
        const C known = make_float2(X.r * X.rsm * own2.x + Rw.r * Rw.rsm * rowold.x,
                                    X.r * X.rsm * own2.y + Rw.r * Rw.rsm * rowold.y);
        kc = make_float2(kc.x + known.x, kc.y + known.y);
      }
      SB[(size_t)slot * sbs + o] = pack(lin_B(cf, g.fvm, b, kc), cf.w);
    }
  }
}

namespace {

// The hand-over of a CTA of NW warps (1..8: pairwise named barriers with immediate ids,
// so the CTA holds 2 NW - 1 hardware barriers), or, NW = 0, of up to 16 warps (two-slot
// buffer and a CTA barrier per step)
template <int VW, int NW> struct HandSel {
  typedef HandOffN<VW, float2, NW> type;
};
template <int VW> struct HandSel<VW, 0> {
  typedef HandOff<VW, float2, false> type;
};

// register budget: about 64 per thread (96 at 4 points per step), i.e. the CTAs per SM
// that this allows for NW warps; the barriers allow 64 / (2 NW - 1)
template <int VW, int NW> struct SplitBounds {
  static constexpr int threads = NW ? NW * 32 : MAXROWS;
  static constexpr int regs = VW >= 4 ? 96 : 64;
  static constexpr int raw = NW ? 65536 / (threads * regs) : 1;
  static constexpr int blocks = raw < 1 ? 1 : (raw > 16 ? 16 : raw);
};
#define CSEM_SWEEP_BOUNDS_S(VW, NW) __launch_bounds__(SplitBounds<VW, NW>::threads, SplitBounds<VW, NW>::blocks)

}  // namespace

// Ex: rows k, march j, VW consecutive i per thread; a line is an i group of one slot
template <bool FWD, int VW, int NW>
__global__ void CSEM_SWEEP_BOUNDS_S(VW, NW) k_sweep_ex32s(SweepP<F32> s, const float4* SB, long sbs, int nslot)
{
  typedef float2 C;
  __shared__ typename HandSel<VW, NW>::type hand;
  // a CTA takes lines (i group, slot) in turn: one per CTA when the grid covers them all,
  // several when the grid is capped (each line's hand-over generations balance, so the
  // next line starts on the same barriers)
  const int nlines = (s.g.n1 + VW - 1) / VW;
  for (long item = blockIdx.x; item < (long)nlines * nslot; item += gridDim.x) {
  const int slot = (int)(item / nlines);
  const int sys = s.sys_list ? s.sys_list[slot] : slot;
  const GridP<F32>& g = s.g;
  const int n1 = g.n1, n2 = g.n2, nK = s.nK;
  const View<F32> V = view_of<F32>(s, slot, sys);
  const C z = make_float2(0.f, 0.f);
  const int R_ = nK - 1, M = n2 - 1;  // rows k = 1..R_, march j = 1..M
  const int rr = threadIdx.x;
  const bool rowok = rr < R_;
  const int k = FWD ? 1 + rr : R_ - rr;
  const int i0 = (int)(item % nlines) * VW;
  float gn = 0.f;
  C* ex0 = nullptr;
  const float4* sb = nullptr;
  if (rowok) {
    const Ax<F32> Z = axis<F32>(g.d3, g.d3s, g.r3, g.r3s, k);
    gn = Z.r * (FWD ? Z.rsm : Z.rs);
    ex0 = V.row(0, k, 0) + i0;
    sb = SB + (size_t)slot * sbs + ix1(n1, n2, k, 0, i0);
  }
  float4 e[VW];
  float gpn = 0.f;
  auto load = [&](int c) {  // march position c of this row
    const int j = FWD ? 1 + c : M - c;
    gpn = ro(g.r2 + j) * ro(g.r2s + (FWD ? j - 1 : j));
#pragma unroll
    for (int v = 0; v < VW; v++)
      if (i0 + v < n1) e[v] = ro(sb + (long)j * n1 + v);
  };
  Lin32 lin[VW];
  auto make = [&]() {
#pragma unroll
    for (int v = 0; v < VW; v++) {
      lin[v].B = make_float2(e[v].x, e[v].y);
      lin[v].w = make_float2(e[v].z, e[v].w);
      lin[v].gp = gpn;
      lin[v].gn = gn;
    }
  };
  C res[VW];
#pragma unroll
  for (int v = 0; v < VW; v++) res[v] = z;
  if (rowok && rr == 0 && M > 0) {
    load(0);
    make();
  }
  for (int T = 0; T < M + R_ - 1; T++) {
    const int c = T - rr;
    const bool act = rowok && c >= 0 && c < M;
    const bool nxt = rowok && c + 1 >= 0 && c + 1 < M;
    if (nxt) load(c + 1);
    C nb[VW];
    hand.get(res, nb, T);
    if (act) {
      const int ox = (FWD ? 1 + c : M - c) * n1;
#pragma unroll
      for (int v = 0; v < VW; v++) {
        if (i0 + v >= n1) {
          res[v] = z;
          continue;
        }
        const C val = lin_apply(lin[v], c > 0 ? res[v] : z, nb[v]);  // prev: own row, previous j
        ex0[ox + v] = val;
        res[v] = val;
      }
    } else {
#pragma unroll
      for (int v = 0; v < VW; v++) res[v] = z;
    }
    hand.put(res, T);
    if (nxt) make();
  }
  hand.finish(M + R_ - 1);
  // every warp has closed this line's barrier generations before any starts the next:
  // a producer's first put of the next line does not wait on "empty", and a second
  // arrival on "full" before its consumer's last sync would complete that generation
  // without the consumer (checked by simulating the protocol over 1-8 warps, 1-6 steps
  // and 1-4 lines per CTA under random interleavings: it deadlocks without this barrier)
  __syncthreads();
  }
}

// Ey (COMP 1: line j, rows k) / Ez (COMP 2: line k, rows j): march i in chunks of VW
template <int COMP, bool FWD, int VW, int NW>
__global__ void CSEM_SWEEP_BOUNDS_S(VW, NW) k_sweep_eyz32s(SweepP<F32> s, const float4* SB, long sbs, int nslot)
{
  typedef float2 C;
  __shared__ typename HandSel<VW, NW>::type hand;
  const int nlines = COMP == 1 ? s.g.n2 : s.nK;  // lines (j for Ey, k for Ez) x slots, in turn as in k_sweep_ex32s
  for (long item = blockIdx.x; item < (long)nlines * nslot; item += gridDim.x) {
  const int slot = (int)(item / nlines);
  const int sys = s.sys_list ? s.sys_list[slot] : slot;
  const GridP<F32>& g = s.g;
  const int n1 = g.n1, n2 = g.n2, nK = s.nK;
  const View<F32> V = view_of<F32>(s, slot, sys);
  const C z = make_float2(0.f, 0.f);
  const int line = (int)(item % nlines);
  const int R_ = COMP == 1 ? nK - 1 : n2 - 1;  // rows k (Ey) or j (Ez) = 1..R_
  const int M = n1 - 1;                         // march i = 1..M
  const int NC = (M + VW - 1) / VW;
  const int rr = threadIdx.x;
  const bool rowok = rr < R_;
  const int r = FWD ? 1 + rr : R_ - rr;
  const int k = COMP == 1 ? r : line;
  const int j = COMP == 1 ? line : r;
  float gn = 0.f;
  C* own = nullptr;
  const float4* sb = nullptr;
  if (rowok) {
    const Ax<F32> Rw =
        COMP == 1 ? axis<F32>(g.d3, g.d3s, g.r3, g.r3s, r) : axis<F32>(g.d2, g.d2s, g.r2, g.r2s, r);
    gn = Rw.r * (FWD ? Rw.rsm : Rw.rs);
    own = V.row(COMP, k, j);
    sb = SB + (size_t)slot * sbs + (COMP == 1 ? ix2(n1, n2, k, j, 0) : ix3(n1, n2, k, j, 0));
  }
  float4 e[VW];
  float gpn[VW];
  auto load = [&](int c) {  // chunk c of this row
#pragma unroll
    for (int v = 0; v < VW; v++) {
      const int m = c * VW + v;
      if (m >= M) continue;
      const int i = FWD ? 1 + m : M - m;
      gpn[v] = ro(g.r1 + i) * ro(g.r1s + (FWD ? i - 1 : i));
      e[v] = ro(sb + i);
    }
  };
  Lin32 lin[VW];
  auto make = [&](int c) {
#pragma unroll
    for (int v = 0; v < VW; v++) {
      if (c * VW + v >= M) continue;
      lin[v].B = make_float2(e[v].x, e[v].y);
      lin[v].w = make_float2(e[v].z, e[v].w);
      lin[v].gp = gpn[v];
      lin[v].gn = gn;
    }
  };
  C res[VW];
#pragma unroll
  for (int v = 0; v < VW; v++) res[v] = z;
  if (rowok && rr == 0 && NC > 0) {
    load(0);
    make(0);
  }
  for (int T = 0; T < NC + R_ - 1; T++) {
    const int c = T - rr;
    const bool act = rowok && c >= 0 && c < NC;
    const bool nx = rowok && c + 1 >= 0 && c + 1 < NC;
    if (nx) load(c + 1);
    C nb[VW];
    hand.get(res, nb, T);
    if (act) {
      C prev = c > 0 ? res[VW - 1] : z;  // own row at the previous march position
#pragma unroll
      for (int v = 0; v < VW; v++) {
        const int m = c * VW + v;
        if (m >= M) {
          res[v] = z;
          continue;
        }
        const C val = lin_apply(lin[v], prev, nb[v]);
        own[FWD ? 1 + m : M - m] = val;
        res[v] = val;
        prev = val;
      }
    } else {
#pragma unroll
      for (int v = 0; v < VW; v++) res[v] = z;
    }
    hand.put(res, T);
    if (nx) make(c + 1);
  }
  hand.finish(NC + R_ - 1);
  __syncthreads();  // close this line's barrier generations first (see k_sweep_ex32s)
  }
}

long sweep_split_scratch(int n1, int n2, int nK)
{
  const long a = (long)n1 * (n2 + 1) * (nK + 1), b = (long)(n1 + 1) * n2 * (nK + 1),
             c = (long)(n1 + 1) * (n2 + 1) * nK;
  return a > b ? (a > c ? a : c) : (b > c ? b : c);
}

template <int VW, int NW>
static void launch_split_nw(const SweepP<F32>& s, int comp, bool fwd, int nslot, const float4* SB, long sbs,
                            int max_ctas, cudaStream_t st)
{
  const int n1 = s.g.n1, n2 = s.g.n2, nK = s.nK;
  const int rows = comp == 2 ? n2 - 1 : nK - 1;
  const int threads = NW ? NW * 32 : (rows + 31) / 32 * 32;
  const long nlines = comp == 0 ? (n1 + VW - 1) / VW : (comp == 1 ? n2 : nK);
  long items = nlines * nslot;
  const unsigned grd = (unsigned)(max_ctas > 0 && items > max_ctas ? max_ctas : items);
  if (comp == 0) {
    if (fwd) count_launch(), k_sweep_ex32s<true, VW, NW><<<grd, threads, 0, st>>>(s, SB, sbs, nslot);
    else count_launch(), k_sweep_ex32s<false, VW, NW><<<grd, threads, 0, st>>>(s, SB, sbs, nslot);
  } else if (comp == 1) {
    if (fwd) count_launch(), k_sweep_eyz32s<1, true, VW, NW><<<grd, threads, 0, st>>>(s, SB, sbs, nslot);
    else count_launch(), k_sweep_eyz32s<1, false, VW, NW><<<grd, threads, 0, st>>>(s, SB, sbs, nslot);
  } else {
    if (fwd) count_launch(), k_sweep_eyz32s<2, true, VW, NW><<<grd, threads, 0, st>>>(s, SB, sbs, nslot);
    else count_launch(), k_sweep_eyz32s<2, false, VW, NW><<<grd, threads, 0, st>>>(s, SB, sbs, nslot);
  }
}

template <int VW>
static void launch_split_vw(const SweepP<F32>& s, int comp, bool fwd, int nslot, const float4* SB, long sbs,
                            int max_ctas, cudaStream_t st)
{
  const int rows = comp == 2 ? s.g.n2 - 1 : s.nK - 1;
  switch ((rows + 31) / 32) {  // warps of the CTA: one row per thread
    case 1: launch_split_nw<VW, 1>(s, comp, fwd, nslot, SB, sbs, max_ctas, st); break;
    case 2: launch_split_nw<VW, 2>(s, comp, fwd, nslot, SB, sbs, max_ctas, st); break;
    case 3: launch_split_nw<VW, 3>(s, comp, fwd, nslot, SB, sbs, max_ctas, st); break;
    case 4: launch_split_nw<VW, 4>(s, comp, fwd, nslot, SB, sbs, max_ctas, st); break;
    case 5: launch_split_nw<VW, 5>(s, comp, fwd, nslot, SB, sbs, max_ctas, st); break;
    case 6: launch_split_nw<VW, 6>(s, comp, fwd, nslot, SB, sbs, max_ctas, st); break;
    case 7: launch_split_nw<VW, 7>(s, comp, fwd, nslot, SB, sbs, max_ctas, st); break;
    case 8: launch_split_nw<VW, 8>(s, comp, fwd, nslot, SB, sbs, max_ctas, st); break;
    default: launch_split_nw<VW < 4 ? VW : 2, 0>(s, comp, fwd, nslot, SB, sbs, max_ctas, st); break;  // 257..512 rows
  }
}

template <int COMP, bool FWD>
static void launch_prep(const SweepP<F32>& s, int nslot, float4* SB, long sbs, const int* groups, int ngroups, int ns,
                        cudaStream_t st)
{
  // a thread per point along i, every (j, k) plane row, every slot or group of slots
  const int nch = (s.g.n1 + PREP_THREADS - 1) / PREP_THREADS;
  if (groups && ns == SPLIT_GROUP) {
    dim3 pg((unsigned)(nch * ngroups), (unsigned)s.g.n2, (unsigned)s.nK);
    count_launch(), k_lusgs_prep<COMP, FWD, SPLIT_GROUP><<<pg, PREP_THREADS, 0, st>>>(s, SB, sbs, nch, groups);
  } else {
    dim3 pg((unsigned)(nch * nslot), (unsigned)s.g.n2, (unsigned)s.nK);
    count_launch(), k_lusgs_prep<COMP, FWD, 1><<<pg, PREP_THREADS, 0, st>>>(s, SB, sbs, nch, nullptr);
  }
}

void launch_split_prep(const SweepP<F32>& s, int comp, bool fwd, int nslot, float4* SB, long sbs, const int* groups,
                       int ngroups, int ns, cudaStream_t st)
{
  if (comp == 0) {
    if (fwd) launch_prep<0, true>(s, nslot, SB, sbs, groups, ngroups, ns, st);
    else launch_prep<0, false>(s, nslot, SB, sbs, groups, ngroups, ns, st);
  } else if (comp == 1) {
    if (fwd) launch_prep<1, true>(s, nslot, SB, sbs, groups, ngroups, ns, st);
    else launch_prep<1, false>(s, nslot, SB, sbs, groups, ngroups, ns, st);
  } else {
    if (fwd) launch_prep<2, true>(s, nslot, SB, sbs, groups, ngroups, ns, st);
    else launch_prep<2, false>(s, nslot, SB, sbs, groups, ngroups, ns, st);
  }
}

void launch_split_sweep(const SweepP<F32>& s, int comp, bool fwd, int nslot, const float4* SB, long sbs, int vw,
                        int max_ctas, cudaStream_t st)
{
  if (vw == 1) launch_split_vw<1>(s, comp, fwd, nslot, SB, sbs, max_ctas, st);
  else if (vw == 4) launch_split_vw<4>(s, comp, fwd, nslot, SB, sbs, max_ctas, st);
  else launch_split_vw<2>(s, comp, fwd, nslot, SB, sbs, max_ctas, st);
}

void launch_sweep_split(const SweepP<F32>& s, int comp, bool fwd, int nslot, float4* SB, long sbs, int vw,
                        const int* groups, int ngroups, int ns, cudaStream_t st)
{
  launch_split_prep(s, comp, fwd, nslot, SB, sbs, groups, ngroups, ns, st);
  launch_split_sweep(s, comp, fwd, nslot, SB, sbs, vw, 0, st);  // one CTA per line
}

}  // namespace csem
