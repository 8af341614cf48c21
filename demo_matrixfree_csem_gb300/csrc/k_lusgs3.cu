// LU-SGS component sweeps in complex64, line-tiled (one launch per component sweep).
#include "csem_cuda.cuh"
#include "engine.h"
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
// position per step). A row's own previous value stays in a register.
template <bool FWD, int BMAX>
__global__ void __launch_bounds__(TileThreads<BMAX>::value) k_sweep_tile_ex32(SweepP<F32> s, int B)
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
  const Ax<F32> X = axis_at<F32>(g.d1, g.d1s, g.r1, g.r1s, i);
  C prev[BMAX];
#pragma unroll
  for (int b = 0; b < BMAX; b++) prev[b] = z;
  for (int T = 0; T < M + NW - 1; T++) {
    const int c = T - w;
    if (c >= 0 && c < M) {
      const int j = FWD ? 1 + c : M - c;
      const Ax<F32> Y = axis<F32>(g.d2, g.d2s, g.r2, g.r2s, j);
      C nb = w > 0 ? tile_hand[(((T - 1) & 1) * NW + (w - 1)) * 32 + lane] : z;
#pragma unroll
      for (int b = 0; b < BMAX; b++) {
        const int ri = r0 + b;
        if (b < B && ri < R) {
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
          const Lin32 lin = lin_make(sc, g.fvm, gg, sg, X.ds * Y.d * Z.d, bv, kc, Y.r * (FWD ? Y.rsm : Y.rs),
                                     Z.r * (FWD ? Z.rsm : Z.rs));
          const C v = lin_apply(lin, prev[b], nb);
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
// step. A row's own previous value is kept in shared memory between steps.
template <int COMP, bool FWD, int VW, int BMAX>
__global__ void __launch_bounds__(TileThreads<BMAX>::value) k_sweep_tile_eyz32(SweepP<F32> s, int B)
{
  typedef float2 C;
  extern __shared__ float2 tile_sh[];  // hand-over [2][NW][VW][32], then own values [NW][BMAX][32]
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, NW = blockDim.x >> 5;
  float2* hand = tile_sh;
  float2* prevs = tile_sh + 2 * NW * VW * 32 + (size_t)w * BMAX * 32 + lane;
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
  // the line's spacings: Y (Ey) or Z (Ez)
  const Ax<F32> LA = COMP == 1 ? axis_at<F32>(g.d2, g.d2s, g.r2, g.r2s, ln) : axis_at<F32>(g.d3, g.d3s, g.r3, g.r3s, ln);
  const float lrs = LA.rs;
  for (int b = 0; b < B; b++) prevs[b * 32] = z;
  for (int T = 0; T < NC + NW - 1; T++) {
    const int c = T - w;
    if (c >= 0 && c < NC) {
      C nb[VW];
#pragma unroll
      for (int q = 0; q < VW; q++) nb[q] = w > 0 ? hand[(((T - 1) & 1) * NW + (w - 1)) * VW * 32 + q * 32 + lane] : z;
      const int bend = min(B, R - r0);
#pragma unroll 1
      for (int b = 0; b < bend; b++) {
        const int r = FWD ? 1 + r0 + b : R - r0 - b;
        const int k = COMP == 1 ? r : ln;
        const int j = COMP == 1 ? ln : r;
        const Ax<F32> Rw = COMP == 1 ? axis<F32>(g.d3, g.d3s, g.r3, g.r3s, k) : axis<F32>(g.d2, g.d2s, g.r2, g.r2s, j);
        const float gn = Rw.r * (FWD ? Rw.rsm : Rw.rs);
        const float grow = (Rw.rs + Rw.rsm) * Rw.r;
        const float dyz = COMP == 1 ? LA.d * Rw.d : Rw.d * LA.d;  // Y.d * Z.d
        C* own = V.row(COMP, k, j);
        const C* nxt = COMP == 1 ? V.row(1, k - 1, j) : V.row(2, k, j - 1);
        const C* xa = COMP == 1 ? V.row(0, k, j + 1) : V.row(0, k + 1, j);
        const C* xb = V.row(0, k, j);
        const C* ya = COMP == 1 ? V.row(2, k, j + 1) : V.row(1, k + 1, j);
        const C* yb = COMP == 1 ? V.row(2, k, j) : V.row(1, k, j);
        const C* yc = COMP == 1 ? V.row(2, k - 1, j + 1) : V.row(1, k + 1, j - 1);
        const C* yd = COMP == 1 ? V.row(2, k - 1, j) : V.row(1, k, j - 1);
        const C* bb = V.brow(COMP, k, j);
        const float* sg0 = COMP == 1 ? g.s22 + ix2(n1, n2, k, j, 0) : g.s33 + ix3(n1, n2, k, j, 0);
        C pv = prevs[b * 32];
#pragma unroll
        for (int q = 0; q < VW; q++) {
          const int m = c * VW + q;
          if (m < M) {
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
            const Lin32 lin = lin_make(sc, g.fvm, gg, sg, X.ds * dyz, bv, kc, X.r * (FWD ? X.rsm : X.rs), gn);
            const C v = lin_apply(lin, pv, nb[q]);
            if (lineok) own[i] = v;
            pv = v;
            nb[q] = v;
          }
        }
        prevs[b * 32] = pv;
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
    shm = sizeof(float2) * ((size_t)2 * NW * VW * 32 + (size_t)NW * BMAX * 32);
    kern = k_sweep_tile_eyz32<COMP, FWD, VW, BMAX>;
  }
  static bool attr = false;  // the larger dynamic shared memory limit, once per instantiation
  if (shm > 48 * 1024 && !attr) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
    attr = true;
  }
  count_launch(), kern<<<grd, NW * 32, shm, st>>>(s, B);
}

template <int COMP, bool FWD, int BMAX>
void launch_tile_vw(const SweepP<F32>& s, int nslot, cudaStream_t st, int B, int NW, int lines, int vw)
{
  if constexpr (COMP == 0) {
    launch_tile<0, FWD, 1, BMAX>(s, nslot, st, B, NW, lines);
  } else {
    if (vw == 1) launch_tile<COMP, FWD, 1, BMAX>(s, nslot, st, B, NW, lines);
    else if (vw == 2) launch_tile<COMP, FWD, 2, BMAX>(s, nslot, st, B, NW, lines);
    else launch_tile<COMP, FWD, 4, BMAX>(s, nslot, st, B, NW, lines);
  }
}

template <int COMP, bool FWD>
void launch_tile_b(const SweepP<F32>& s, int nslot, cudaStream_t st, int bmax, int vw)
{
  int R, M, L;
  const int n1 = s.g.n1, n2 = s.g.n2, nK = s.nK;
  if (COMP == 0) { R = nK - 1; M = n2 - 1; L = n1; }
  else if (COMP == 1) { R = nK - 1; M = n1 - 1; L = n2; }
  else { R = n2 - 1; M = n1 - 1; L = nK; }
  (void)M;
  // the fewest warps whose blocks of at most bmax rows cover the rows, then balanced blocks
  const int NW = (R + bmax - 1) / bmax;
  const int B = (R + NW - 1) / NW;
  if (bmax <= 4) launch_tile_vw<COMP, FWD, 4>(s, nslot, st, B, NW, L, vw);
  else if (bmax <= 8) launch_tile_vw<COMP, FWD, 8>(s, nslot, st, B, NW, L, vw);
  else launch_tile_vw<COMP, FWD, 16>(s, nslot, st, B, NW, L, vw);
}

}  // namespace

bool sweep_tiled_fits(int comp, int n1, int n2, int nK, int rows_per_warp)
{
  const int R = comp == 2 ? n2 - 1 : nK - 1;
  const int b = rows_per_warp <= 4 ? 4 : (rows_per_warp <= 8 ? 8 : 16);
  const int maxw = (b == 4 ? TileThreads<4>::value : (b == 8 ? TileThreads<8>::value : TileThreads<16>::value)) / 32;
  return R >= 1 && (R + b - 1) / b <= maxw && n1 >= 2 && n2 >= 2;
}

// rows_per_warp: 4, 8 or 16 (other values: 8); vw: march positions per step of the Ey
// and Ez sweeps, 1, 2 or 4 (other values: 4); the Ex sweep takes one per step.
void launch_sweep_tiled(const SweepP<F32>& s, int comp, bool fwd, int nslot, cudaStream_t st, int rows_per_warp,
                        int vw)
{
  const int bmax = rows_per_warp == 4 || rows_per_warp == 16 ? rows_per_warp : 8;
  if (vw != 1 && vw != 2) vw = 4;
  if (comp == 0) {
    if (fwd) launch_tile_b<0, true>(s, nslot, st, bmax, vw);
    else launch_tile_b<0, false>(s, nslot, st, bmax, vw);
  } else if (comp == 1) {
    if (fwd) launch_tile_b<1, true>(s, nslot, st, bmax, vw);
    else launch_tile_b<1, false>(s, nslot, st, bmax, vw);
  } else {
    if (fwd) launch_tile_b<2, true>(s, nslot, st, bmax, vw);
    else launch_tile_b<2, false>(s, nslot, st, bmax, vw);
  }
}

}  // namespace csem
