// LU-SGS component sweeps in complex64, line-tiled (one launch per component sweep).
#include "csem_cuda.cuh"
#include "engine.h"
#include <algorithm>
#include <type_traits>
#include "k_sweep_common.cuh"

namespace csem {

using namespace sweep;

// ---------------------------------------------------------------------------------------
// complex64 sweeps, line-tiled: lanes along the independent axis, rows in warp blocks.
//
// A CTA owns 32 consecutive independent lines of one system (one lane each: i for Ex,
// so its loads and stores are coalesced; j for Ey; k for Ez) and every row of the sweep.
// The rows, in sweep order, are cut into contiguous blocks of B, one per warp. All
// warps advance together, one march chunk of VW positions per step, skewed by one chunk
// per warp: at step T warp w works on chunk T - w of each of its rows, row after row.
// A row's chunk needs the previous row's values at the same march positions and its own
// value at the previous position: inside a warp's block the previous row was computed
// just before (registers), the block's first row reads the last row of the warp before,
// which that warp produced one step earlier (shared memory, double-buffered by step
// parity), and a row's own previous value stays in a register from the step before. One
// CTA barrier per step.
//
// Per point the update is the linear form of the complex64 pipelined sweeps above
// (lin_make / lin_apply with the same operands and expressions), so this schedule and
// the pipelined one compute the same values.

// largest CTA of a variant (its register budget follows): blocks of 16 rows up to 512
// threads, of 8 up to 768, of 4 up to 1024
template <int BMAX> struct TileThreads {
  static constexpr int value = BMAX >= 16 ? 512 : (BMAX >= 8 ? 768 : 1024);
};

// Ex: lanes along i (coalesced), rows k in warp blocks of at most BMAX, march j (one
// position per step). Each step runs in two passes over the warp's rows: first the
// loads and every part of the update that does not depend on the chain (lin_make: the
// right-hand side, the conductivity, the cross-coupling and not-yet-swept neighbours,
// all fixed before the chain reaches them), with the loads of all rows in flight
// together; then the chain itself (lin_apply) row after row from registers. A row's own
// previous value stays in a register between steps.
template <bool FWD, int BMAX>
__global__ void __launch_bounds__(TileThreads<BMAX>::value, 1) k_sweep_tile_ex32(SweepP<F32> s, int B)
{
  typedef float2 C;
  extern __shared__ float2 tile_hand[];  // [2][NW][32]: the last row of each warp's block
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, NW = blockDim.x >> 5;
  const int slot = blockIdx.y;
  const int sys = s.sys_list ? s.sys_list[slot] : slot;
  const GridP<F32>& g = s.g;
  const int n1 = g.n1, n2 = g.n2;
  const int R = s.nK - 1, M = n2 - 1;  // rows k = 1..R, march j = 1..M
  const int line = blockIdx.x * 32 + lane;
  const bool lineok = line < n1;
  const int i = lineok ? line : n1 - 1;  // clamped: loads stay in bounds
  const View<F32> V = view_of<F32>(s, slot, sys);
  const SysScal<F32> sc = s.scal[sys];
  const C z = make_float2(0.f, 0.f);
  const int r0 = w * B;
  const int bend = min(B, R - r0);
  const Ax<F32> X = axis_at<F32>(g.d1, g.d1s, g.r1, g.r1s, i);
  C prev[BMAX];
#pragma unroll
  for (int b = 0; b < BMAX; b++) prev[b] = z;
  for (int T = 0; T < M + NW - 1; T++) {
    const int c = T - w;
    if (c >= 0 && c < M) {
      const int j = FWD ? 1 + c : M - c;
      const Ax<F32> Y = axis<F32>(g.d2, g.d2s, g.r2, g.r2s, j);
      const float gp = Y.r * (FWD ? Y.rsm : Y.rs);
      float2 lB[BMAX], lw[BMAX];  // B and w of each row's linear form
#pragma unroll
      for (int b = 0; b < BMAX; b++) {  // pass 1: independent of the chain
        if (b < bend) {
          const int ri = r0 + b;
          const int k = FWD ? 1 + ri : R - ri;
          const Ax<F32> Z = axis<F32>(g.d3, g.d3s, g.r3, g.r3s, k);
          const C* bb = V.brow(0, k, j);
          const C bv = bb ? ro(bb + i) : z;
          const float sg = ro(g.s11 + ix1(n1, n2, k, j, i));
          C kc = z;
          if (!FWD) {  // the other components (swept before), own-component values not yet swept
            const C* ey0 = V.row(1, k, j);
            const C* ey1 = V.row(1, k, j - 1);
            const C* ez0 = V.row(2, k, j);
            const C* ez1 = V.row(2, k - 1, j);
            const C exjm = *V.at(0, k, j - 1, i);
            const C exkm = *V.at(0, k - 1, j, i);
            const C dy = sub32(sub32(ro(ey0 + i + 1), ro(ey0 + i)), sub32(ro(ey1 + i + 1), ro(ey1 + i)));
            const C dz = sub32(sub32(ro(ez0 + i + 1), ro(ez0 + i)), sub32(ro(ez1 + i + 1), ro(ez1 + i)));
            const C cross = scl32(X.rs, make_float2(Y.r * dy.x + Z.r * dz.x, Y.r * dy.y + Z.r * dz.y));
            const C known = make_float2(Y.r * Y.rsm * exjm.x + Z.r * Z.rsm * exkm.x,
                                        Y.r * Y.rsm * exjm.y + Z.r * Z.rsm * exkm.y);
            kc = sub32(known, cross);
          }
          const float gg = (Y.rs + Y.rsm) * Y.r + (Z.rs + Z.rsm) * Z.r;
          const Lin32 L = lin_make(sc, g.fvm, gg, sg, X.ds * Y.d * Z.d, bv, kc, gp, 0.f);
          lB[b] = L.B;
          lw[b] = L.w;
        }
      }
      C nb = w > 0 ? tile_hand[(((T - 1) & 1) * NW + (w - 1)) * 32 + lane] : z;
#pragma unroll
      for (int b = 0; b < BMAX; b++) {  // pass 2: the chain
        if (b < bend) {
          const int ri = r0 + b;
          const int k = FWD ? 1 + ri : R - ri;
          Lin32 L;
          L.B = lB[b];
          L.w = lw[b];
          L.gp = gp;
          L.gn = ro(g.r3 + k) * (FWD ? ro(g.r3s + k - 1) : ro(g.r3s + k));  // Z.r * (Z.rsm or Z.rs)
          const C v = lin_apply(L, prev[b], nb);
          if (lineok) *V.at(0, k, j, i) = v;
          prev[b] = v;
          nb = v;
        }
      }
      if (w + 1 < NW) tile_hand[((T & 1) * NW + w) * 32 + lane] = nb;
    }
    __syncthreads();
  }
}

// Ey (COMP 1: line j, rows k) / Ez (COMP 2: line k, rows j): march i, VW positions per
// step, the same two passes (the VW positions of a row form a chain of their own in
// pass 2). A row's own previous value stays in a register between steps.
template <int COMP, bool FWD, int VW, int BMAX>
__global__ void __launch_bounds__(TileThreads<BMAX>::value, 1) k_sweep_tile_eyz32(SweepP<F32> s, int B)
{
  typedef float2 C;
  // hand-over [2][NW][VW][32], then each warp's linear forms [NW][BMAX][VW][32] (B, w)
  extern __shared__ float2 tile_sh[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, NW = blockDim.x >> 5;
  float2* hand = tile_sh;
  float4* lsh = reinterpret_cast<float4*>(tile_sh + 2 * NW * VW * 32) + (size_t)w * BMAX * VW * 32 + lane;
  const int slot = blockIdx.y;
  const int sys = s.sys_list ? s.sys_list[slot] : slot;
  const GridP<F32>& g = s.g;
  const int n1 = g.n1, n2 = g.n2, nK = s.nK;
  const int R = COMP == 1 ? nK - 1 : n2 - 1;  // rows k (Ey) or j (Ez) = 1..R
  const int M = n1 - 1;                        // march i = 1..M
  const int L = COMP == 1 ? n2 : nK;
  const int line = blockIdx.x * 32 + lane;
  const bool lineok = line < L;
  const int ln = lineok ? line : L - 1;
  const View<F32> V = view_of<F32>(s, slot, sys);
  const SysScal<F32> sc = s.scal[sys];
  const C z = make_float2(0.f, 0.f);
  const int NC = (M + VW - 1) / VW;
  const int r0 = w * B;
  const int bend = min(B, R - r0);
  // the line's spacings: Y (Ey) or Z (Ez)
  const Ax<F32> LA = COMP == 1 ? axis_at<F32>(g.d2, g.d2s, g.r2, g.r2s, ln) : axis_at<F32>(g.d3, g.d3s, g.r3, g.r3s, ln);
  const float lrs = LA.rs;
  C prev[BMAX];
#pragma unroll
  for (int b = 0; b < BMAX; b++) prev[b] = z;
  for (int T = 0; T < NC + NW - 1; T++) {
    const int c = T - w;
    if (c >= 0 && c < NC) {
#pragma unroll 2
      for (int b = 0; b < bend; b++) {  // pass 1: independent of the chain, into shared memory
        {
          const int r = FWD ? 1 + r0 + b : R - r0 - b;
          const int k = COMP == 1 ? r : ln;
          const int j = COMP == 1 ? ln : r;
          const Ax<F32> Rw = COMP == 1 ? axis<F32>(g.d3, g.d3s, g.r3, g.r3s, k) : axis<F32>(g.d2, g.d2s, g.r2, g.r2s, j);
          const float grow = (Rw.rs + Rw.rsm) * Rw.r;
          const float dyz = LA.d * Rw.d;  // Y.d * Z.d
          const C* own = V.row(COMP, k, j);
          const C* nxt = COMP == 1 ? V.row(1, k - 1, j) : V.row(2, k, j - 1);
          const C* xa = COMP == 1 ? V.row(0, k, j + 1) : V.row(0, k + 1, j);
          const C* xb = V.row(0, k, j);
          const C* ya = COMP == 1 ? V.row(2, k, j + 1) : V.row(1, k + 1, j);
          const C* yb = COMP == 1 ? V.row(2, k, j) : V.row(1, k, j);
          const C* yc = COMP == 1 ? V.row(2, k - 1, j + 1) : V.row(1, k + 1, j - 1);
          const C* yd = COMP == 1 ? V.row(2, k - 1, j) : V.row(1, k, j - 1);
          const C* bb = V.brow(COMP, k, j);
          const float* sg0 = COMP == 1 ? g.s22 + ix2(n1, n2, k, j, 0) : g.s33 + ix3(n1, n2, k, j, 0);
#pragma unroll
          for (int q = 0; q < VW; q++) {
            const int m = min(c * VW + q, M - 1);  // clamped: positions past the end are not stored
            const int i = FWD ? 1 + m : M - m;
            const Ax<F32> X = axis<F32>(g.d1, g.d1s, g.r1, g.r1s, i);
            const C bv = bb ? ro(bb + i) : z;
            const float sg = ro(sg0 + i);
            const float gg = (X.rs + X.rsm) * X.r + grow;
            const C dx = sub32(sub32(ro(xa + i), ro(xb + i)), sub32(ro(xa + i - 1), ro(xb + i - 1)));
            C acc = scl32(X.r, dx);
            if (COMP == 2 || !FWD) {
              const C dy = sub32(sub32(ro(ya + i), ro(yb + i)), sub32(ro(yc + i), ro(yd + i)));
              acc = make_float2(acc.x + Rw.r * dy.x, acc.y + Rw.r * dy.y);
            }
            C kc = scl32(-lrs, acc);
            if (!FWD) {  // this row at the next position and the next row: not yet swept
              const C own2 = own[i - 1], rowold = nxt[i];
              const C known = make_float2(X.r * X.rsm * own2.x + Rw.r * Rw.rsm * rowold.x,
                                          X.r * X.rsm * own2.y + Rw.r * Rw.rsm * rowold.y);
              kc = make_float2(kc.x + known.x, kc.y + known.y);
            }
            const Lin32 L = lin_make(sc, g.fvm, gg, sg, X.ds * dyz, bv, kc, 0.f, 0.f);
            lsh[(b * VW + q) * 32] = make_float4(L.B.x, L.B.y, L.w.x, L.w.y);  // only this lane reads it
          }
        }
      }
      C nb[VW];
#pragma unroll
      for (int q = 0; q < VW; q++) nb[q] = w > 0 ? hand[(((T - 1) & 1) * NW + (w - 1)) * VW * 32 + q * 32 + lane] : z;
#pragma unroll
      for (int b = 0; b < BMAX; b++) {  // pass 2: the chain
        if (b < bend) {
          const int r = FWD ? 1 + r0 + b : R - r0 - b;
          const int k = COMP == 1 ? r : ln;
          const int j = COMP == 1 ? ln : r;
          C* own = V.row(COMP, k, j);
          // the row neighbour's coefficient: Rw.r * (Rw.rsm or Rw.rs) of the row's axis
          const float* rr = COMP == 1 ? g.r3 : g.r2;
          const float* rrs = COMP == 1 ? g.r3s : g.r2s;
          const float gn = ro(rr + r) * (FWD ? ro(rrs + r - 1) : ro(rrs + r));
          C pv = prev[b];
#pragma unroll
          for (int q = 0; q < VW; q++) {
            const int m = c * VW + q;
            if (m < M) {
              const int i = FWD ? 1 + m : M - m;
              const float4 t = lsh[(b * VW + q) * 32];
              Lin32 L;
              L.B = make_float2(t.x, t.y);
              L.w = make_float2(t.z, t.w);
              L.gp = ro(g.r1 + i) * (FWD ? ro(g.r1s + i - 1) : ro(g.r1s + i));  // X.r * (X.rsm or X.rs)
              L.gn = gn;
              const C v = lin_apply(L, pv, nb[q]);
              if (lineok) own[i] = v;
              pv = v;
              nb[q] = v;
            }
          }
          prev[b] = pv;
        }
      }
      if (w + 1 < NW) {
#pragma unroll
        for (int q = 0; q < VW; q++) hand[((T & 1) * NW + w) * VW * 32 + q * 32 + lane] = nb[q];
      }
    }
    __syncthreads();
  }
}

namespace {

// one instantiation per (component, direction, points per step, rows per warp)
template <int COMP, bool FWD, int VW, int BMAX>
void launch_tile(const SweepP<F32>& s, int nslot, cudaStream_t st, int B, int NW, int lines)
{
  const dim3 grd((unsigned)((lines + 31) / 32), (unsigned)nslot);
  size_t shm;
  void (*kern)(SweepP<F32>, int);
  if constexpr (COMP == 0) {
    shm = sizeof(float2) * 2 * (size_t)NW * 32;
    kern = k_sweep_tile_ex32<FWD, BMAX>;
  } else {
    shm = sizeof(float2) * (size_t)2 * NW * VW * 32 + sizeof(float4) * (size_t)NW * BMAX * VW * 32;
    kern = k_sweep_tile_eyz32<COMP, FWD, VW, BMAX>;
  }
  // the larger dynamic shared memory limit, once per instantiation and device (the first
  // launch of a batch runs outside any stream capture)
  static bool attr[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (shm > 48 * 1024 && dev >= 0 && dev < 64 && !attr[dev]) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
    attr[dev] = true;
  }
  count_launch(), kern<<<grd, NW * 32, shm, st>>>(s, B);
}

template <int COMP, bool FWD, int BMAX>
void launch_tile_vw(const SweepP<F32>& s, int nslot, cudaStream_t st, int B, int NW, int lines, int vw)
{
  if constexpr (COMP == 0) {
    launch_tile<0, FWD, 1, BMAX>(s, nslot, st, B, NW, lines);
  } else {
    if (vw == 1 || BMAX > 8) launch_tile<COMP, FWD, 1, BMAX>(s, nslot, st, B, NW, lines);
    else if (vw == 2 || BMAX > 4) launch_tile<COMP, FWD, 2, BMAX>(s, nslot, st, B, NW, lines);
    else launch_tile<COMP, FWD, 4, BMAX>(s, nslot, st, B, NW, lines);
  }
}

}  // namespace

namespace {

// Shape of one tiled sweep: rows per warp block (bmax), march positions per step (vw),
// warps and dynamic shared memory. At most 16 linear forms per thread (bmax * vw).
struct TileShape {
  int bmax, vw, nw, b;
  size_t shm;
};

TileShape tile_shape(int comp, int R, int rows_per_warp, int vw)
{
  TileShape t;
  t.vw = comp == 0 ? 1 : (vw == 1 || vw == 2 ? vw : 4);
  t.bmax = rows_per_warp == 4 || rows_per_warp == 16 ? rows_per_warp : 8;
  if (comp != 0) t.bmax = std::min(t.bmax, 16 / t.vw);
  t.nw = (R + t.bmax - 1) / t.bmax;
  t.b = (R + t.nw - 1) / t.nw;
  t.shm = comp == 0 ? sizeof(float2) * 2 * (size_t)t.nw * 32
                    : sizeof(float2) * 2 * (size_t)t.nw * t.vw * 32 + sizeof(float4) * (size_t)t.nw * t.bmax * t.vw * 32;
  return t;
}

constexpr size_t kTileMaxShm = 220 * 1024;

}  // namespace

bool sweep_tiled_fits(int comp, int n1, int n2, int nK, int rows_per_warp, int vw)
{
  const int R = comp == 2 ? n2 - 1 : nK - 1;
  if (R < 1 || n1 < 2 || n2 < 2) return false;
  const TileShape t = tile_shape(comp, R, rows_per_warp, vw);
  const int maxw = (t.bmax == 4 ? TileThreads<4>::value : (t.bmax == 8 ? TileThreads<8>::value : TileThreads<16>::value)) / 32;
  return t.nw <= maxw && t.shm <= kTileMaxShm;
}

// rows_per_warp: 4, 8 or 16 (other values: 8); vw: march positions per step of the Ey
// and Ez sweeps, 1, 2 or 4 (other values: 4), with at most 16 rows x positions per
// thread; the Ex sweep takes one position per step. Callers check sweep_tiled_fits.
void launch_sweep_tiled(const SweepP<F32>& s, int comp, bool fwd, int nslot, cudaStream_t st, int rows_per_warp,
                        int vw)
{
  const int R = comp == 2 ? s.g.n2 - 1 : s.nK - 1;
  const TileShape t = tile_shape(comp, R, rows_per_warp, vw);
  const int L = comp == 0 ? s.g.n1 : (comp == 1 ? s.g.n2 : s.nK);
  auto go = [&](auto comp_c, auto fwd_c) {
    constexpr int C_ = decltype(comp_c)::value;
    constexpr bool F_ = decltype(fwd_c)::value;
    if (t.bmax == 4) launch_tile_vw<C_, F_, 4>(s, nslot, st, t.b, t.nw, L, t.vw);
    else if (t.bmax == 8) launch_tile_vw<C_, F_, 8>(s, nslot, st, t.b, t.nw, L, t.vw);
    else launch_tile_vw<C_, F_, 16>(s, nslot, st, t.b, t.nw, L, t.vw);
  };
  using I0 = std::integral_constant<int, 0>;
  using I1 = std::integral_constant<int, 1>;
  using I2 = std::integral_constant<int, 2>;
  using T_ = std::true_type;
  using F_ = std::false_type;
  if (comp == 0) fwd ? go(I0{}, T_{}) : go(I0{}, F_{});
  else if (comp == 1) fwd ? go(I1{}, T_{}) : go(I1{}, F_{});
  else fwd ? go(I2{}, T_{}) : go(I2{}, F_{});
}

}  // namespace csem
