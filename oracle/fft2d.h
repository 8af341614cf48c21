/* Self-written unnormalised 2-D DFT used by the CPU oracle (test infrastructure). */
#ifndef CSEM_ORACLE_FFT2D_H
#define CSEM_ORACLE_FFT2D_H
#ifdef __cplusplus
extern "C" {
#endif
/* In-place DFT of a row-major complex array data[n0][n1] (interleaved re/im doubles,
 * n1 fastest). sign = -1: forward, +1: backward. No normalisation. */
void csem_fft2d(int n0, int n1, double *data, int sign);
#ifdef __cplusplus
}
#endif
#endif
