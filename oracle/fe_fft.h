/* fe_fft.h -- the oracle's own complex FFT (test infrastructure only). */
#ifndef FE_FFT_H
#define FE_FFT_H
#ifdef __cplusplus
extern "C" {
#endif
/* In-place unnormalised DFT of n complex values spaced `stride` complex
 * elements apart: X[k] = sum_j x[j] exp(sign*2*pi*i*j*k/n). */
void fe_fft1d(double *data, int n, long stride, int sign);
/* In-place 3-D DFT of a row-major n0 x n1 x n2 complex grid. */
void fe_fft3d(double *data, int n0, int n1, int n2, int sign);
#ifdef __cplusplus
}
#endif
#endif
