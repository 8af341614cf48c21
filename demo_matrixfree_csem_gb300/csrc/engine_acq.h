// Device view used by source injection and receiver extraction.
#pragma once
#include <cuda_runtime.h>

namespace csem {

struct AcqGrid {
  int n1, n2, n3f, nb, airbc, fvm;  // full padded grid
  long lEx, lEy, lE;                // operator-grid vector layout
  const double *x1, *x2, *x3, *x1s, *x2s, *x3s;
  const double *s11, *s22, *s33;    // full-grid conductivities
  float rho_water;
  int fix_src_sigma;  // 1: the source's conductivity at its own row (not the reference's -nb shift)
};

void launch_inject(const AcqGrid& g, int nslot, const float* src, const double2* iom, const int* ch, int nch,
                   double2* B, cudaStream_t st);
template <class C>
void launch_extract(const AcqGrid& g, int nslot, int nch, const int* ch, int nrec, const float* rec, const C* X,
                    long xstride, const int* sys_list, double2* out, cudaStream_t st);

}  // namespace csem
