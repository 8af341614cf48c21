// Source injection (inject_source, inject_extract.c:24-120) and receiver extraction
// (extract_emf, inject_extract.c:123-213) on the device, in FP64 with the reference's
// operation order. One thread handles one (system, channel) source or one
// (system, channel, receiver) triple; positions are found with the reference's
// bisection (find_index.c:9-30).
//
// Reference behaviours kept on purpose: with airbc the source's conductivity lookup is
// made after shifting k by -nb (so it reads nb rows higher in the air-included array,
// inject_extract.c:55-63), while the Ez receiver uses the unshifted row
// (inject_extract.c:194-206). AcqGrid::fix_src_sigma = 1 (the context option "fix_quirks")
// looks the source's conductivity up at its own row of the air-included array instead.
#include "csem_cuda.cuh"
#include "engine_acq.h"

namespace csem {

__device__ __forceinline__ int find_index_d(int n, const double* x, double val)
{
  int low = 0, high = n - 1;
  while (low < high) {
    int i = (low + high) / 2;
    if (x[i] <= val) low = i;
    if (x[i] > val) high = i;
    if (low == high || low == high - 1) break;
  }
  return low;
}

struct Corner { int i, j, k; double w1, w2, w3; };

// locate a point on the staggered grid of channel ch (0 Ex, 1 Ey, 2 Ez)
__device__ __forceinline__ Corner locate(const AcqGrid& g, int ch, double px, double py, double pz, double* vol)
{
  Corner c;
  const double* X1 = ch == 0 ? g.x1s : g.x1;
  const double* X2 = ch == 1 ? g.x2s : g.x2;
  const double* X3 = ch == 2 ? g.x3s : g.x3;
  c.i = find_index_d(ch == 0 ? g.n1 : g.n1 + 1, X1, px);
  c.j = find_index_d(ch == 1 ? g.n2 : g.n2 + 1, X2, py);
  c.k = find_index_d(ch == 2 ? g.n3f : g.n3f + 1, X3, pz);
  c.w1 = __ddiv_rn(__dsub_rn(px, X1[c.i]), __dsub_rn(X1[c.i + 1], X1[c.i]));
  c.w2 = __ddiv_rn(__dsub_rn(py, X2[c.j]), __dsub_rn(X2[c.j + 1], X2[c.j]));
  c.w3 = __ddiv_rn(__dsub_rn(pz, X3[c.k]), __dsub_rn(X3[c.k + 1], X3[c.k]));
  if (vol)
    *vol = __dmul_rn(__dmul_rn(__dsub_rn(X1[c.i + 1], X1[c.i]), __dsub_rn(X2[c.j + 1], X2[c.j])),
                     __dsub_rn(X3[c.k + 1], X3[c.k]));
  return c;
}

__device__ __forceinline__ long eidx(const AcqGrid& g, int ch, int k, int j, int i)
{
  const int n1 = g.n1, n2 = g.n2;
  return ch == 0 ? ix1(n1, n2, k, j, i) : (ch == 1 ? g.lEx + ix2(n1, n2, k, j, i) : g.lEx + g.lEy + ix3(n1, n2, k, j, i));
}

// b[sys] += unit dipole of source sys (b must be zero beforehand)
__global__ void k_inject(AcqGrid g, int nslot, const float* __restrict__ src, const double2* __restrict__ iom,
                         const int* __restrict__ ch, int nch, double2* __restrict__ B)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nslot) return;
  double2* b = B + (size_t)t * g.lE;
  const double px = src[3 * t], py = src[3 * t + 1], pz = src[3 * t + 2];
  for (int ic = 0; ic < nch; ic++) {
    const int c = ch[ic];
    if (c < 0 || c > 2) continue;
    double vol;
    Corner q = locate(g, c, px, py, pz, &vol);
    double2 sv = make_double2(__ddiv_rn(1., vol), 0.);
    if (g.fvm) sv = iom[t];
    if (c < 2) sv = cdivr<F64>(sv, (double)g.rho_water);
    int k = q.k - (g.airbc ? g.nb : 0);
    if (k < 0) continue;  // above the operator grid (the host rejects such positions first)
    const int ksig = g.fix_src_sigma ? q.k : k;  // row of the conductivity lookup
    for (int m = 0; m < 8; m++) {
      const int di = m & 1, dj = (m >> 1) & 1, dk = m >> 2;
      const double a1 = di ? q.w1 : __dsub_rn(1., q.w1), a2 = dj ? q.w2 : __dsub_rn(1., q.w2),
                   a3 = dk ? q.w3 : __dsub_rn(1., q.w3);
      const int kk = k + dk, jj = q.j + dj, ii = q.i + di;
      double2 v;
      if (c == 0) v = cdivr<F64>(sv, g.s11[ix1(g.n1, g.n2, ksig + dk, jj, ii)]);
      else if (c == 1) v = cdivr<F64>(sv, g.s22[ix2(g.n1, g.n2, ksig + dk, jj, ii)]);
      else v = sv;
      v = rmul<F64>(a3, rmul<F64>(a2, rmul<F64>(a1, v)));
      const long p = eidx(g, c, kk, jj, ii);
      b[p] = cadd<F64>(b[p], v);
    }
  }
}

// out[slot][ic][r] = trilinear gather of channel ch[ic] at receiver r
template <class C>
__global__ void k_extract(AcqGrid g, int nslot, int nch, const int* __restrict__ ch, int nrec,
                          const float* __restrict__ rec, const C* __restrict__ X, long xstride,
                          const int* __restrict__ sys_list, double2* __restrict__ out)
{
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)nslot * nch * nrec) return;
  const int r = (int)(t % nrec), ic = (int)((t / nrec) % nch), slot = (int)(t / ((long)nrec * nch));
  const int sys = sys_list ? sys_list[slot] : slot;
  const C* x = X + (size_t)sys * xstride;
  const int c = ch[ic];
  double2 s = make_double2(0., 0.);
  if (c >= 0 && c <= 2) {
    const double px = rec[5 * r], py = rec[5 * r + 1], pz = rec[5 * r + 2];
    Corner q = locate(g, c, px, py, pz, nullptr);
    const int kk0 = q.k;
    const int k = q.k - (g.airbc ? g.nb : 0);
    for (int m = 0; m < 8 && k >= 0; m++) {
      const int di = m & 1, dj = (m >> 1) & 1, dk = m >> 2;
      const double a1 = di ? q.w1 : __dsub_rn(1., q.w1), a2 = dj ? q.w2 : __dsub_rn(1., q.w2),
                   a3 = dk ? q.w3 : __dsub_rn(1., q.w3);
      const C e = x[eidx(g, c, k + dk, q.j + dj, q.i + di)];
      double2 v = make_double2((double)e.x, (double)e.y);
      if (c == 2) v = rmul<F64>(g.s33[ix3(g.n1, g.n2, kk0 + dk, q.j + dj, q.i + di)], v);
      s = cadd<F64>(s, rmul<F64>(a3, rmul<F64>(a2, rmul<F64>(a1, v))));
    }
    if (c == 2) s = rmul<F64>((double)g.rho_water, s);
  }
  out[t] = s;
}

void launch_inject(const AcqGrid& g, int nslot, const float* src, const double2* iom, const int* ch, int nch,
                   double2* B, cudaStream_t st)
{
  count_launch(), k_inject<<<(nslot + 31) / 32, 32, 0, st>>>(g, nslot, src, iom, ch, nch, B);
}

template <class C>
void launch_extract(const AcqGrid& g, int nslot, int nch, const int* ch, int nrec, const float* rec, const C* X,
                    long xstride, const int* sys_list, double2* out, cudaStream_t st)
{
  long n = (long)nslot * nch * nrec;
  if (n == 0) return;
  count_launch(), k_extract<C><<<(unsigned)((n + 127) / 128), 128, 0, st>>>(g, nslot, nch, ch, nrec, rec, X, xstride, sys_list, out);
}
template void launch_extract<double2>(const AcqGrid&, int, int, const int*, int, const float*, const double2*, long,
                                      const int*, double2*, cudaStream_t);
template void launch_extract<float2>(const AcqGrid&, int, int, const int*, int, const float*, const float2*, long,
                                     const int*, double2*, cudaStream_t);

}  // namespace csem
