// The assembled operator as a comparison point for the matrix-free one (the reference's
// Acsr_init / Acsr_apply, Acsr.c:704-716, airbc=0 only there as here).
//
// A is assembled on the device by probing the matrix-free operator: every row of the
// curl-curl operator couples to 13 columns, all within one index step in each direction
// (an Ex row: Ex at (k, j+-1, i), (k+-1, j, i), (k, j, i); Ey at (k, j, i), (k, j, i+1),
// (k, j-1, i), (k, j-1, i+1); Ez at (k, j, i), (k, j, i+1), (k-1, j, i), (k-1, j, i+1);
// the Ey and Ez rows alike), so the columns of one component whose (i, j, k) agree
// modulo 3 never share a row. Applying the stencil to the 81 indicator vectors of
// (component, i mod 3, j mod 3, k mod 3) therefore yields every entry exactly once:
// entry (r, col) is row r of the response to col's class. Rows are stored with 13 slots
// (32-bit column indices; slots outside the grid hold a zero on the diagonal), then
// cuSPARSE's SpMV and the stencil are timed on the same random vector and compared.
#include <cusparse.h>
#include <cmath>
#include <vector>
#include "engine_model.h"

namespace csem {

namespace {

constexpr int SLOTS = 13;

struct Layout {
  int n1, n2, n3;
  long lEx, lEy;
  __device__ __forceinline__ long idx(int c, int k, int j, int i) const
  {
    if (c == 0) return i + (long)n1 * (j + (long)(n2 + 1) * k);
    if (c == 1) return lEx + i + (long)(n1 + 1) * (j + (long)n2 * k);
    return lEx + lEy + i + (long)(n1 + 1) * (j + (long)(n2 + 1) * k);
  }
  // extents of component c: i < ni, j < nj, k < nk
  __device__ __forceinline__ void ext(int c, int& ni, int& nj, int& nk) const
  {
    ni = c == 0 ? n1 : n1 + 1;
    nj = c == 1 ? n2 : n2 + 1;
    nk = c == 2 ? n3 : n3 + 1;
  }
  __device__ __forceinline__ void decode(long q, int& c, int& k, int& j, int& i) const
  {
    c = q < lEx ? 0 : (q < lEx + lEy ? 1 : 2);
    const long o = c == 0 ? q : (c == 1 ? q - lEx : q - lEx - lEy);
    int ni, nj, nk;
    ext(c, ni, nj, nk);
    i = (int)(o % ni);
    j = (int)((o / ni) % nj);
    k = (int)(o / ((long)ni * nj));
  }
};

// the 13 coupled columns of a row of component c, as (component, dk, dj, di), in
// increasing column order
struct Tap {
  signed char c, dk, dj, di;
};
__constant__ Tap c_taps[3][SLOTS] = {
    {{0, -1, 0, 0}, {0, 0, -1, 0}, {0, 0, 0, 0}, {0, 0, 1, 0}, {0, 1, 0, 0},
     {1, 0, -1, 0}, {1, 0, -1, 1}, {1, 0, 0, 0}, {1, 0, 0, 1},
     {2, -1, 0, 0}, {2, -1, 0, 1}, {2, 0, 0, 0}, {2, 0, 0, 1}},
    {{0, 0, 0, -1}, {0, 0, 0, 0}, {0, 0, 1, -1}, {0, 0, 1, 0},
     {1, -1, 0, 0}, {1, 0, 0, -1}, {1, 0, 0, 0}, {1, 0, 0, 1}, {1, 1, 0, 0},
     {2, -1, 0, 0}, {2, -1, 1, 0}, {2, 0, 0, 0}, {2, 0, 1, 0}},
    {{0, 0, 0, -1}, {0, 0, 0, 0}, {0, 1, 0, -1}, {0, 1, 0, 0},
     {1, 0, -1, 0}, {1, 0, 0, 0}, {1, 1, -1, 0}, {1, 1, 0, 0},
     {2, 0, -1, 0}, {2, 0, 0, -1}, {2, 0, 0, 0}, {2, 0, 0, 1}, {2, 0, 1, 0}}};

__device__ __forceinline__ int class_of(int c, int k, int j, int i) { return c * 27 + (i % 3) * 9 + (j % 3) * 3 + k % 3; }

// columns and probe classes of every slot; slots outside the grid: the diagonal, class 255
__global__ void k_pattern(Layout L, long n, int* __restrict__ col, unsigned char* __restrict__ cls)
{
  const long r = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  int c, k, j, i;
  L.decode(r, c, k, j, i);
  for (int s = 0; s < SLOTS; s++) {
    const Tap t = c_taps[c][s];
    const int kk = k + t.dk, jj = j + t.dj, ii = i + t.di;
    int ni, nj, nk;
    L.ext(t.c, ni, nj, nk);
    const bool in = kk >= 0 && jj >= 0 && ii >= 0 && kk < nk && jj < nj && ii < ni;
    col[r * SLOTS + s] = in ? (int)L.idx(t.c, kk, jj, ii) : (int)r;
    cls[r * SLOTS + s] = in ? (unsigned char)class_of(t.c, kk, jj, ii) : 255;
  }
}

template <class C>
__global__ void k_indicator(Layout L, long n, int probe, C* __restrict__ x)
{
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  int c, k, j, i;
  L.decode(q, c, k, j, i);
  x[q].x = class_of(c, k, j, i) == probe ? 1 : 0;
  x[q].y = 0;
}

template <class C>
__global__ void k_scatter(long n, int probe, const unsigned char* __restrict__ cls, const C* __restrict__ y,
                          C* __restrict__ val)
{
  const long e = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n * SLOTS) return;
  if (cls[e] == probe) val[e] = y[e / SLOTS];
  else if (cls[e] == 255) val[e].x = val[e].y = 0;
}

__global__ void k_row_ptr(long n, int* __restrict__ rp)
{
  const long r = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r <= n) rp[r] = (int)(r * SLOTS);
}

// a fixed pseudo-random vector (SplitMix64 of the index) in [-1, 1)
template <class C>
__global__ void k_random(long n, C* __restrict__ x)
{
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  unsigned long long z = (unsigned long long)q * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  x[q].x = (double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
  x[q].y = (double)((z * 0x9E3779B97F4A7C15ull) >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

#define CSEM_SPARSE_TRY(x)                                                                      \
  do {                                                                                          \
    cusparseStatus_t s_ = (x);                                                                  \
    if (s_ != CUSPARSE_STATUS_SUCCESS) throw CudaError(cudaErrorUnknown, #x, __FILE__, __LINE__); \
  } while (0)

template <class P>
void compare(Model* m, cudaStream_t st, double iom_re, double iom_im, int nrep, double* out)
{
  typedef typename P::C C;
  const long n = m->lE;
  const Layout L{m->n1, m->n2, m->n3, m->lEx, m->lEy};
  Ops<P> ops(m, 1, st);
  DevBuf sc, col, cls, val, rp, x, y, yr, work;
  const SysScal<F64> s64 = sys_scal64(iom_re, iom_im);
  sc.alloc(sizeof(SysScal<P>));
  if constexpr (P::exact) {
    CSEM_CUDA_TRY(cudaMemcpyAsync(sc.p, &s64, sizeof(s64), cudaMemcpyHostToDevice, st));
  } else {
    const SysScal<F32> s32 = sys_scal32(s64);
    CSEM_CUDA_TRY(cudaMemcpyAsync(sc.p, &s32, sizeof(s32), cudaMemcpyHostToDevice, st));
  }
  col.alloc(sizeof(int) * n * SLOTS);
  cls.alloc(n * SLOTS);
  val.alloc(sizeof(C) * n * SLOTS);
  rp.alloc(sizeof(int) * (n + 1));
  x.alloc(sizeof(C) * n);
  y.alloc(sizeof(C) * n);
  yr.alloc(sizeof(C) * n);
  const unsigned nb = (unsigned)((n + 255) / 256), nbe = (unsigned)((n * SLOTS + 255) / 256);
  count_launch(), k_pattern<<<nb, 256, 0, st>>>(L, n, col.as<int>(), cls.as<unsigned char>());
  count_launch(), k_row_ptr<<<(unsigned)((n + 256) / 256), 256, 0, st>>>(n, rp.as<int>());
  const SysScal<P>* scp = sc.as<SysScal<P>>();
  for (int probe = 0; probe < 81; probe++) {
    count_launch(), k_indicator<C><<<nb, 256, 0, st>>>(L, n, probe, x.as<C>());
    ops.apply_A(x.as<C>(), y.as<C>(), 1, nullptr, scp);
    count_launch(), k_scatter<C><<<nbe, 256, 0, st>>>(n, probe, cls.as<unsigned char>(), y.as<C>(), val.as<C>());
  }
  CSEM_CUDA_TRY(cudaGetLastError());
  count_launch(), k_random<C><<<nb, 256, 0, st>>>(n, x.as<C>());

  // cuSPARSE objects and events, released on every exit (errors throw)
  struct Res {
    cusparseHandle_t h = nullptr;
    cusparseSpMatDescr_t A = nullptr;
    cusparseDnVecDescr_t X = nullptr, Y = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    ~Res()
    {
      if (X) cusparseDestroyDnVec(X);
      if (Y) cusparseDestroyDnVec(Y);
      if (A) cusparseDestroySpMat(A);
      if (h) cusparseDestroy(h);
      if (e0) cudaEventDestroy(e0);
      if (e1) cudaEventDestroy(e1);
    }
  } res;
  cusparseHandle_t& h = res.h;
  cusparseSpMatDescr_t& A = res.A;
  cusparseDnVecDescr_t &X = res.X, &Y = res.Y;
  cudaEvent_t &e0 = res.e0, &e1 = res.e1;
  CSEM_SPARSE_TRY(cusparseCreate(&h));
  const cudaDataType dt = P::exact ? CUDA_C_64F : CUDA_C_32F;
  CSEM_SPARSE_TRY(cusparseSetStream(h, st));
  CSEM_SPARSE_TRY(cusparseCreateCsr(&A, n, n, n * SLOTS, rp.p, col.p, val.p, CUSPARSE_INDEX_32I, CUSPARSE_INDEX_32I,
                                    CUSPARSE_INDEX_BASE_ZERO, dt));
  CSEM_SPARSE_TRY(cusparseCreateDnVec(&X, n, x.p, dt));
  CSEM_SPARSE_TRY(cusparseCreateDnVec(&Y, n, yr.p, dt));
  C one, zero;
  one.x = 1;
  one.y = 0;
  zero.x = 0;
  zero.y = 0;
  size_t wb = 0;
  CSEM_SPARSE_TRY(cusparseSpMV_bufferSize(h, CUSPARSE_OPERATION_NON_TRANSPOSE, &one, A, X, &zero, Y, dt,
                                          CUSPARSE_SPMV_ALG_DEFAULT, &wb));
  work.alloc(wb > 0 ? wb : 16);
  CSEM_CUDA_TRY(cudaEventCreate(&e0));
  CSEM_CUDA_TRY(cudaEventCreate(&e1));
  auto spmv = [&]() {
    CSEM_SPARSE_TRY(cusparseSpMV(h, CUSPARSE_OPERATION_NON_TRANSPOSE, &one, A, X, &zero, Y, dt,
                                 CUSPARSE_SPMV_ALG_DEFAULT, work.p));
  };
  auto stencil = [&]() { ops.apply_A(x.as<C>(), y.as<C>(), 1, nullptr, scp); };
  float ms_csr = 0, ms_st = 0;
  spmv();
  stencil();
  CSEM_CUDA_TRY(cudaEventRecord(e0, st));
  for (int q = 0; q < nrep; q++) spmv();
  CSEM_CUDA_TRY(cudaEventRecord(e1, st));
  CSEM_CUDA_TRY(cudaEventSynchronize(e1));
  CSEM_CUDA_TRY(cudaEventElapsedTime(&ms_csr, e0, e1));
  CSEM_CUDA_TRY(cudaEventRecord(e0, st));
  for (int q = 0; q < nrep; q++) stencil();
  CSEM_CUDA_TRY(cudaEventRecord(e1, st));
  CSEM_CUDA_TRY(cudaEventSynchronize(e1));
  CSEM_CUDA_TRY(cudaEventElapsedTime(&ms_st, e0, e1));
  std::vector<C> a(n), b(n);
  CSEM_CUDA_TRY(cudaMemcpyAsync(a.data(), yr.p, sizeof(C) * n, cudaMemcpyDeviceToHost, st));
  CSEM_CUDA_TRY(cudaMemcpyAsync(b.data(), y.p, sizeof(C) * n, cudaMemcpyDeviceToHost, st));
  CSEM_CUDA_TRY(cudaStreamSynchronize(st));
  double dmax = 0, ymax = 0;
  for (long q = 0; q < n; q++) {
    const double dx = (double)a[q].x - (double)b[q].x, dy = (double)a[q].y - (double)b[q].y;
    const double d = dx * dx + dy * dy, yy = (double)b[q].x * b[q].x + (double)b[q].y * b[q].y;
    if (d > dmax) dmax = d;
    if (yy > ymax) ymax = yy;
  }
  out[0] = ms_csr / nrep;
  out[1] = ms_st / nrep;
  out[2] = ymax > 0 ? std::sqrt(dmax / ymax) : 0.0;
  out[3] = (double)n * SLOTS;
  // bytes one SpMV must move: values, column indices, row pointers, x and y
  out[4] = (double)n * SLOTS * (sizeof(C) + sizeof(int)) + sizeof(int) * (n + 1.0) + 2.0 * sizeof(C) * n;
}

}  // namespace

void csr_compare(Model* m, cudaStream_t st, int prec, double iom_re, double iom_im, int nrep, double* out)
{
  if (prec == 64) compare<F64>(m, st, iom_re, iom_im, nrep, out);
  else compare<F32>(m, st, iom_re, iom_im, nrep, out);
}

}  // namespace csem
