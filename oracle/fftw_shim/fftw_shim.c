/*
 * fftw_shim.c -- implements the five FFTW3 symbols the reference's SPME code
 * uses, on top of the oracle's own FFT (fe_fft.c).  Linked only into the
 * oracle build of the reference; never into the product.
 */
#include <stdlib.h>

#include "fftw3.h"
#include "../fe_fft.h"

struct fe_fftw_plan_s {
  int n0, n1, n2, sign;
  fftw_complex *in, *out;
};

fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex *in,
                           fftw_complex *out, int sign, unsigned flags) {
  (void)flags;
  fftw_plan p = (fftw_plan)calloc(1, sizeof(*p));
  p->n0 = n0; p->n1 = n1; p->n2 = n2; p->sign = sign;
  p->in = in; p->out = out;
  return p;
}

void fftw_execute(const fftw_plan p) {
  long n = (long)p->n0 * p->n1 * p->n2;
  if (p->in != p->out)
    for (long i = 0; i < n; i++) {
      p->out[i][0] = p->in[i][0];
      p->out[i][1] = p->in[i][1];
    }
  fe_fft3d(&p->out[0][0], p->n0, p->n1, p->n2, p->sign);
}

void fftw_destroy_plan(fftw_plan p) { free(p); }
void *fftw_malloc(size_t n) { return malloc(n); }
void fftw_free(void *p) { free(p); }
