// Optional per-operator device timing: CUDA events recorded on the operator's own
// stream around each application, summed on demand. Off unless csem_profile(1).
#pragma once
#include <cuda_runtime.h>

namespace csem {

enum ProfCat {
  PROF_A64 = 0, PROF_A32 = 1, PROF_LUSGS64 = 2, PROF_LUSGS32 = 3, PROF_APHI64 = 4, PROF_APHI32 = 5,
  PROF_AIR64 = 6, PROF_AIR32 = 7, PROF_STENCIL64 = 8, PROF_STENCIL32 = 9, PROF_NCAT = 16
};

// count of this library's kernel launches (cuFFT's own kernels excluded)
void count_launch(int n = 1);

bool prof_on();
int prof_begin(int cat, cudaStream_t st, int units);   // returns a token (-1 when off)
void prof_end(int token, cudaStream_t st);

// `units` = systems processed by this application (for bytes-per-application figures)
struct ProfScope {
  int tok;
  cudaStream_t st;
  ProfScope(int cat, cudaStream_t s, int units) : tok(prof_on() ? prof_begin(cat, s, units) : -1), st(s) {}
  ~ProfScope() { if (tok >= 0) prof_end(tok, st); }
};

}  // namespace csem
