// Vector kernels of the Krylov loops (solver.c) and the complex dot product
// s = sum a_i conj(b_i) (cdotprod.c:13-19).
//
// Dot products are deterministic: a fixed partition of the vector into `nblk` blocks
// (a function of the length only), a fixed per-thread order, a fixed shuffle tree and
// a fixed-order sum of block partials. Complex128 inputs accumulate in FP64. For
// complex64 inputs each product term is split exactly (p = a*b, e = fma(a,b,-p)) and
// summed per thread with a compensated (TwoSum) float pair, so the per-thread partials
// carry ~48 significant bits; partials are combined in FP64.
#include "csem_cuda.cuh"
#include "engine.h"
#include "solver_state.h"
#include "k_dot_common.cuh"

namespace csem {

static constexpr int DOT_THREADS = 256;

int dot_blocks(long n)
{
  long b = (n + DOT_THREADS * 8 - 1) / (DOT_THREADS * 8);
  if (b < 1) b = 1;
  if (b > 1024) b = 1024;
  return (int)b;
}

// a per-system double2 scalar in the vector's precision
template <class P> __device__ __forceinline__ typename P::C cast_c(double2 v);
template <> __device__ __forceinline__ double2 cast_c<F64>(double2 v) { return v; }
template <> __device__ __forceinline__ float2 cast_c<F32>(double2 v) { return make_float2((float)v.x, (float)v.y); }

__device__ __forceinline__ double2 block_sum(double2 v)
{
  __shared__ double2 red[DOT_THREADS / 32];
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = l < DOT_THREADS / 32 ? red[l] : make_double2(0, 0);
    v = warp_sum(v);
  }
  __syncthreads();
  return v;
}

// partial[slot][blk] = sum over the block's chunk of a*conj(b)
template <class P>
__global__ void __launch_bounds__(DOT_THREADS)
k_dot_partial(const typename P::C* __restrict__ A, const typename P::C* __restrict__ B, long n, long stride,
              const int* __restrict__ sys_list, double2* __restrict__ partial, int nblk)
{
  const int slot = blockIdx.y;
  const int sys = sys_list ? sys_list[slot] : slot;
  const typename P::C* a = A + (size_t)sys * stride;
  const typename P::C* b = B + (size_t)sys * stride;
  const long chunk = (n + nblk - 1) / nblk;
  const long beg = (long)blockIdx.x * chunk, end = min(n, beg + chunk);
  DotAcc<P> d;
  for (long q = beg + threadIdx.x; q < end; q += DOT_THREADS) d.add(a[q], b[q]);
  const double2 acc = block_sum(d.value());
  if (threadIdx.x == 0) partial[(size_t)slot * nblk + blockIdx.x] = acc;
}

// Two dot products a1*conj(b1) and a2*conj(b2) in one pass, with the partition, per-thread
// order and tree of k_dot_partial, so each equals its single-dot result bit for bit.
// Vectors the two share (s.t and t.t, r.r and r.r0) are read from DRAM once.
// partial[slot][blk] and partial[nslot + slot][blk].
template <class P>
__global__ void __launch_bounds__(DOT_THREADS)
k_dot2_partial(const typename P::C* __restrict__ A1, const typename P::C* __restrict__ B1,
               const typename P::C* __restrict__ A2, const typename P::C* __restrict__ B2, long n, long stride,
               const int* __restrict__ sys_list, double2* __restrict__ partial, int nblk)
{
  const int slot = blockIdx.y;
  const int sys = sys_list ? sys_list[slot] : slot;
  const size_t so = (size_t)sys * stride;
  const long chunk = (n + nblk - 1) / nblk;
  const long beg = (long)blockIdx.x * chunk, end = min(n, beg + chunk);
  DotAcc<P> d1, d2;
  for (long q = beg + threadIdx.x; q < end; q += DOT_THREADS) {
    d1.add(A1[so + q], B1[so + q]);
    d2.add(A2[so + q], B2[so + q]);
  }
  const double2 acc1 = block_sum(d1.value());
  const double2 acc2 = block_sum(d2.value());
  if (threadIdx.x == 0) {
    partial[(size_t)slot * nblk + blockIdx.x] = acc1;
    partial[(size_t)(gridDim.y + slot) * nblk + blockIdx.x] = acc2;
  }
}

__global__ void k_dot_final(const double2* __restrict__ partial, int nblk, double2* __restrict__ out)
{
  const int slot = blockIdx.x;
  double2 acc = make_double2(0, 0);
  for (int q = threadIdx.x; q < nblk; q += DOT_THREADS) {
    double2 v = partial[(size_t)slot * nblk + q];
    acc.x = __dadd_rn(acc.x, v.x);
    acc.y = __dadd_rn(acc.y, v.y);
  }
  acc = block_sum(acc);
  if (threadIdx.x == 0) out[slot] = acc;
}

// out1[slot], out2[slot] from the two partial sets of k_dot2_partial (k_dot_final's order)
__global__ void k_dot2_final(const double2* __restrict__ partial, int nblk, double2* __restrict__ out1,
                             double2* __restrict__ out2)
{
  const int slot = blockIdx.x;
  for (int h = 0; h < 2; h++) {
    const double2* pp = partial + (size_t)(h * gridDim.x + slot) * nblk;
    double2 acc = make_double2(0, 0);
    for (int q = threadIdx.x; q < nblk; q += DOT_THREADS) {
      double2 v = pp[q];
      acc.x = __dadd_rn(acc.x, v.x);
      acc.y = __dadd_rn(acc.y, v.y);
    }
    acc = block_sum(acc);
    if (threadIdx.x == 0) (h ? out2 : out1)[slot] = acc;
  }
}

// complex128 <a, b> in the reference's order (cdotprod.c:13-19): s += a_i conj(b_i) from
// i = 0 to n-1, each product and each addition rounded once, so the result is the
// reference's bit for bit. The sum is one dependent chain per component: thread 0 adds
// a chunk of products from shared memory while the other threads form the next chunk's
// products (coalesced loads), one CTA per call.
static constexpr int SEQ_CHUNK = 1024;  // 2 x 16 KB of products

__global__ void __launch_bounds__(DOT_THREADS)
k_dot_seq(const double2* __restrict__ a, const double2* __restrict__ b, long n, double2* __restrict__ out)
{
  __shared__ double2 prod[2][SEQ_CHUNK];
  const long nch = (n + SEQ_CHUNK - 1) / SEQ_CHUNK;
  auto fill = [&](long c, int first, int step) {
    double2* pb = prod[c & 1];
    for (int t = first; t < SEQ_CHUNK; t += step) {
      const long q = c * SEQ_CHUNK + t;
      if (q < n) pb[t] = cmul<F64>(a[q], make_double2(b[q].x, -b[q].y));
    }
  };
  if (nch > 0) fill(0, threadIdx.x, DOT_THREADS);
  __syncthreads();
  double sr = 0.0, si = 0.0;
  for (long c = 0; c < nch; c++) {
    if (threadIdx.x == 0) {
      const double2* pb = prod[c & 1];
      const int m = (int)min((long)SEQ_CHUNK, n - c * SEQ_CHUNK);
      for (int t = 0; t < m; t++) {
        const double2 v = pb[t];
        sr = __dadd_rn(sr, v.x);
        si = __dadd_rn(si, v.y);
      }
    } else if (c + 1 < nch) {
      fill(c + 1, threadIdx.x - 1, DOT_THREADS - 1);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = make_double2(sr, si);
}

void launch_dot_seq(const double2* a, const double2* b, long n, double2* out, cudaStream_t st)
{
  count_launch(), k_dot_seq<<<1, DOT_THREADS, 0, st>>>(a, b, n, out);
}

// The flexible BiCGStab update with its two dot products in one pass (solver.c:153-156,
// 157-160): x += alpha pp + omega ss, r = s - omega t (ss in a buffer of its own), then
// r.conj(r) and r.conj(r0). The pass walks the dot products' partition in their
// per-thread order, so both values equal those of k_dot2_partial on the updated r bit for
// bit; systems no longer running keep x and r and still get their dot products.
template <class P>
__global__ void __launch_bounds__(DOT_THREADS)
k_xr_dot2(long n, const int* __restrict__ sys_list, const KrylovScalars* __restrict__ ks,
          typename P::C* __restrict__ x, const typename P::C* __restrict__ pp, const typename P::C* __restrict__ ss,
          typename P::C* __restrict__ r, const typename P::C* __restrict__ s, const typename P::C* __restrict__ t,
          const typename P::C* __restrict__ r0, double2* __restrict__ partial, int nblk)
{
  typedef typename P::C C;
  const int slot = blockIdx.y;
  const int sys = sys_list ? sys_list[slot] : slot;
  const size_t so = (size_t)sys * n;
  const long chunk = (n + nblk - 1) / nblk;
  const long beg = (long)blockIdx.x * chunk, end = min(n, beg + chunk);
  const bool run = ks[sys].status == ST_RUNNING;
  const C alpha = cast_c<P>(ks[sys].alpha), omega = cast_c<P>(ks[sys].omega);
  DotAcc<P> d1, d2;
  for (long q = beg + threadIdx.x; q < end; q += DOT_THREADS) {
    C rv;
    if (run) {
      x[so + q] = cadd<P>(x[so + q], cadd<P>(cmul<P>(alpha, pp[so + q]), cmul<P>(omega, ss[so + q])));
      rv = csub<P>(s[so + q], cmul<P>(omega, t[so + q]));
      r[so + q] = rv;
    } else {
      rv = r[so + q];
    }
    d1.add(rv, rv);
    d2.add(rv, r0[so + q]);
  }
  const double2 acc1 = block_sum(d1.value());
  const double2 acc2 = block_sum(d2.value());
  if (threadIdx.x == 0) {
    partial[(size_t)slot * nblk + blockIdx.x] = acc1;
    partial[(size_t)(gridDim.y + slot) * nblk + blockIdx.x] = acc2;
  }
}

template <class P>
void launch_xr_dot2(long n, int nslot, const int* sys_list, const KrylovScalars* ks, typename P::C* x,
                    const typename P::C* pp, const typename P::C* ss, typename P::C* r, const typename P::C* s,
                    const typename P::C* t, const typename P::C* r0, double2* partial, int nblk, double2* out_rr,
                    double2* out_rr0, cudaStream_t st)
{
  dim3 grd(nblk, nslot);
  count_launch(), k_xr_dot2<P><<<grd, DOT_THREADS, 0, st>>>(n, sys_list, ks, x, pp, ss, r, s, t, r0, partial, nblk);
  count_launch(), k_dot2_final<<<nslot, DOT_THREADS, 0, st>>>(partial, nblk, out_rr, out_rr0);
}

template <class P>
void launch_dot(const typename P::C* a, const typename P::C* b, long n, long stride, int nslot,
                const int* sys_list, double2* partial, int nblk, double2* out, cudaStream_t st)
{
  dim3 grd(nblk, nslot);
  count_launch(), k_dot_partial<P><<<grd, DOT_THREADS, 0, st>>>(a, b, n, stride, sys_list, partial, nblk);
  count_launch(), k_dot_final<<<nslot, DOT_THREADS, 0, st>>>(partial, nblk, out);
}

template <class P>
void launch_dot2(const typename P::C* a1, const typename P::C* b1, const typename P::C* a2,
                 const typename P::C* b2, long n, long stride, int nslot, const int* sys_list, double2* partial,
                 int nblk, double2* out1, double2* out2, cudaStream_t st)
{
  dim3 grd(nblk, nslot);
  count_launch(), k_dot2_partial<P><<<grd, DOT_THREADS, 0, st>>>(a1, b1, a2, b2, n, stride, sys_list, partial, nblk);
  count_launch(), k_dot2_final<<<nslot, DOT_THREADS, 0, st>>>(partial, nblk, out1, out2);
}

void launch_dot_finish(const double2* partial, int nblk, int nslot, double2* out1, double2* out2, cudaStream_t st)
{
  if (out2) count_launch(), k_dot2_final<<<nslot, DOT_THREADS, 0, st>>>(partial, nblk, out1, out2);
  else count_launch(), k_dot_final<<<nslot, DOT_THREADS, 0, st>>>(partial, nblk, out1);
}

template void launch_dot<F64>(const double2*, const double2*, long, long, int, const int*, double2*, int,
                              double2*, cudaStream_t);
template void launch_dot<F32>(const float2*, const float2*, long, long, int, const int*, double2*, int,
                              double2*, cudaStream_t);
template void launch_dot2<F32>(const float2*, const float2*, const float2*, const float2*, long, long, int,
                               const int*, double2*, int, double2*, double2*, cudaStream_t);
template void launch_xr_dot2<F32>(long, int, const int*, const KrylovScalars*, float2*, const float2*,
                                  const float2*, float2*, const float2*, const float2*, const float2*, double2*, int,
                                  double2*, double2*, cudaStream_t);

// ------------------------------------------------------------------ vector updates

#define CSEM_VEC_PROLOGUE                                                  \
  const int slot = blockIdx.y;                                             \
  const int sys = sys_list ? sys_list[slot] : slot;                        \
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;              \
  if (q >= n) return;                                                      \
  const size_t o = (size_t)sys * n + q;

// r = b - v; p = r; r0 = r   (solver.c:108-112)
template <class P>
__global__ void k_vec_init(long n, const int* __restrict__ sys_list, const typename P::C* __restrict__ b,
                           const typename P::C* __restrict__ v, typename P::C* __restrict__ r,
                           typename P::C* __restrict__ p, typename P::C* __restrict__ r0)
{
  CSEM_VEC_PROLOGUE
  typename P::C x = csub<P>(b[o], v[o]);
  r[o] = x;
  p[o] = x;
  r0[o] = x;
}

// r = b - w   (solver.c:198,423)
template <class P>
__global__ void k_vec_sub(long n, const int* __restrict__ sys_list, const typename P::C* __restrict__ b,
                          const typename P::C* __restrict__ w, typename P::C* __restrict__ r)
{
  CSEM_VEC_PROLOGUE
  r[o] = csub<P>(b[o], w[o]);
}

// s = r - alpha v   (solver.c:147)
template <class P>
__global__ void k_vec_s(long n, const int* __restrict__ sys_list, const KrylovScalars* __restrict__ ks,
                        const typename P::C* __restrict__ r, const typename P::C* __restrict__ v,
                        typename P::C* __restrict__ s)
{
  CSEM_VEC_PROLOGUE
  if (ks[sys].status != ST_RUNNING) return;  // finished systems keep their vectors
  const typename P::C alpha = cast_c<P>(ks[sys].alpha);
  s[o] = csub<P>(r[o], cmul<P>(alpha, v[o]));
}

// x += alpha pp + omega ss; r = s - omega t   (solver.c:153-156, flexible: ss lives in r;
// solver.c:63-66, plain: pp = p and ss = s)
template <class P, bool SS_IS_S>
__global__ void k_vec_xr(long n, const int* __restrict__ sys_list, const KrylovScalars* __restrict__ ks,
                         typename P::C* __restrict__ x, const typename P::C* __restrict__ pp,
                         typename P::C* __restrict__ r, const typename P::C* __restrict__ s,
                         const typename P::C* __restrict__ t)
{
  CSEM_VEC_PROLOGUE
  if (ks[sys].status != ST_RUNNING) return;
  const typename P::C alpha = cast_c<P>(ks[sys].alpha), omega = cast_c<P>(ks[sys].omega);
  const typename P::C ss = SS_IS_S ? s[o] : r[o];
  x[o] = cadd<P>(x[o], cadd<P>(cmul<P>(alpha, pp[o]), cmul<P>(omega, ss)));
  r[o] = csub<P>(s[o], cmul<P>(omega, t[o]));
}

// p = r + beta (p - omega v)   (solver.c:166)
template <class P>
__global__ void k_vec_p(long n, const int* __restrict__ sys_list, const KrylovScalars* __restrict__ ks,
                        const typename P::C* __restrict__ r, typename P::C* __restrict__ p,
                        const typename P::C* __restrict__ v)
{
  CSEM_VEC_PROLOGUE
  if (ks[sys].status != ST_RUNNING) return;
  const typename P::C beta = cast_c<P>(ks[sys].beta), omega = cast_c<P>(ks[sys].omega);
  p[o] = cadd<P>(r[o], cmul<P>(beta, csub<P>(p[o], cmul<P>(omega, v[o]))));
}

// y = a*x + y with a per-system scalar taken from a double2 array (GMRES updates)
template <class P>
__global__ void k_vec_axpy(long n, const int* __restrict__ sys_list, const double2* __restrict__ coef,
                           int coef_stride, int neg, const typename P::C* __restrict__ x,
                           typename P::C* __restrict__ y)
{
  CSEM_VEC_PROLOGUE
  const typename P::C a = cast_c<P>(coef[(size_t)slot * coef_stride]);
  if (neg) y[o] = csub<P>(y[o], cmul<P>(a, x[o]));   // w -= h*v   (solver.c:221)
  else y[o] = cadd<P>(y[o], cmul<P>(a, x[o]));       // x += y*v   (solver.c:272)
}

// y = x / d with a per-system complex divisor (GMRES v_{j+1} = w / h, beta scaling)
template <class P>
__global__ void k_vec_cdiv(long n, const int* __restrict__ sys_list, const double2* __restrict__ d, int dstride,
                           int real_only, const typename P::C* __restrict__ x, typename P::C* __restrict__ y)
{
  CSEM_VEC_PROLOGUE
  const typename P::C dv = cast_c<P>(d[(size_t)slot * dstride]);
  if (real_only) y[o] = cdivr<P>(x[o], dv.x);
  else y[o] = cdiv<P>(x[o], dv);
}

template <class P>
void launch_vec(int op, long n, int nslot, const int* sys_list, const KrylovScalars* ks, typename P::C* a,
                typename P::C* b, typename P::C* c, typename P::C* d, typename P::C* e, cudaStream_t st)
{
  dim3 grd((unsigned)((n + 255) / 256), nslot);
  switch (op) {
  case VEC_INIT: count_launch(), k_vec_init<P><<<grd, 256, 0, st>>>(n, sys_list, a, b, c, d, e); break;
  case VEC_S: count_launch(), k_vec_s<P><<<grd, 256, 0, st>>>(n, sys_list, ks, a, b, c); break;
  case VEC_XR: count_launch(), k_vec_xr<P, false><<<grd, 256, 0, st>>>(n, sys_list, ks, a, b, c, d, e); break;
  case VEC_SUB: count_launch(), k_vec_sub<P><<<grd, 256, 0, st>>>(n, sys_list, a, b, c); break;
  case VEC_XR_PLAIN: count_launch(), k_vec_xr<P, true><<<grd, 256, 0, st>>>(n, sys_list, ks, a, b, c, d, e); break;
  case VEC_P: count_launch(), k_vec_p<P><<<grd, 256, 0, st>>>(n, sys_list, ks, a, b, c); break;
  }
}

template <class P>
void launch_axpy(long n, int nslot, const int* sys_list, const double2* coef, int coef_stride, int neg,
                 const typename P::C* x, typename P::C* y, cudaStream_t st)
{
  dim3 grd((unsigned)((n + 255) / 256), nslot);
  count_launch(), k_vec_axpy<P><<<grd, 256, 0, st>>>(n, sys_list, coef, coef_stride, neg, x, y);
}

template <class P>
void launch_cdivv(long n, int nslot, const int* sys_list, const double2* d, int dstride, int real_only,
                  const typename P::C* x, typename P::C* y, cudaStream_t st)
{
  dim3 grd((unsigned)((n + 255) / 256), nslot);
  count_launch(), k_vec_cdiv<P><<<grd, 256, 0, st>>>(n, sys_list, d, dstride, real_only, x, y);
}

#define CSEM_INST(P)                                                                                        \
  template void launch_vec<P>(int, long, int, const int*, const KrylovScalars*, P::C*, P::C*, P::C*, P::C*, \
                              P::C*, cudaStream_t);                                                         \
  template void launch_axpy<P>(long, int, const int*, const double2*, int, int, const P::C*, P::C*,         \
                               cudaStream_t);                                                               \
  template void launch_cdivv<P>(long, int, const int*, const double2*, int, int, const P::C*, P::C*,        \
                                cudaStream_t);
CSEM_INST(F64)
CSEM_INST(F32)
#undef CSEM_INST

}  // namespace csem
