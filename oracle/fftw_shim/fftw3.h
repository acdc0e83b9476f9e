/*
 * fftw3.h -- project-written stand-in for the five FFTW3 entry points the
 * reference's SPME code calls (pme_setup.c:47-48,67-68,78-79,
 * pme_calc.c:50,113,314,377, allocate.c:499).  FFTW3 is not installed on
 * either build machine, so the reference is linked against this shim when it
 * is compiled as an oracle.  It is test infrastructure only.
 *
 * Conventions follow FFTW3's published definition of the unnormalised
 * complex DFT:  out[k] = sum_j in[j] * exp(sign * 2*pi*i * j.k / n),
 * FFTW_FORWARD = -1, FFTW_BACKWARD = +1, row-major (last index fastest).
 */
#ifndef FE_FFTW_SHIM_H
#define FE_FFTW_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef struct fe_fftw_plan_s *fftw_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_PATIENT (1U << 5)
#define FFTW_EXHAUSTIVE (1U << 3)

fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex *in,
                           fftw_complex *out, int sign, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);
void *fftw_malloc(size_t n);
void fftw_free(void *p);

#ifdef __cplusplus
}
#endif
#endif
