/*
 * fe_fft.c -- a small mixed-radix complex FFT written for the oracle.
 *
 * Test infrastructure only: it backs (1) the FFTW3 shim that the reference's
 * SPME code is linked against when the reference is built as an oracle
 * (pme_calc.c:50,113 call fftw_execute on a 3-D in-place plan) and (2) the
 * oracle's own restatement of pme_calc.  The product path uses cuFFT.
 *
 * Algorithm: recursive decimation-in-time Cooley-Tukey over the prime
 * factors of n (any n; a radix-p step costs O(p^2) per group, so primes are
 * handled by the same code as 2/3/5).  Twiddles exp(sign*2*pi*i*j/N) are
 * tabulated once per axis length from cos/sin of the exact angle.
 * Definition (FFTW3's): X[k] = sum_j x[j] exp(sign*2*pi*i*j*k/n), unnormalised.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "fe_fft.h"

static int smallest_factor(int n) {
  if (n % 2 == 0) return 2;
  for (int p = 3; p * p <= n; p += 2)
    if (n % p == 0) return p;
  return n;
}

/* in: complex samples at in[0], in[stride], ... (n of them)
 * out: n contiguous complex results.  tw: table of N twiddles. */
static void fft_rec(const double *in, long stride, double *out, int n,
                    const double *tw, int N, double *scratch) {
  if (n == 1) {
    out[0] = in[0];
    out[1] = in[1];
    return;
  }
  int p = smallest_factor(n);
  int m = n / p;
  for (int r = 0; r < p; r++)
    fft_rec(in + 2 * r * stride, stride * p, out + 2 * r * m, m, tw, N,
            scratch);
  /* combine: X[k + q m] = sum_r Y_r[k] * W_n^{r (k + q m)} */
  int step = N / n; /* W_n^j = tw[(j*step) % N] */
  double *acc = scratch; /* 2*p doubles */
  for (int k = 0; k < m; k++) {
    for (int q = 0; q < p; q++) {
      double sr = 0.0, si = 0.0;
      int kk = k + q * m;
      for (int r = 0; r < p; r++) {
        long j = ((long)r * kk) % n;
        const double *w = tw + 2 * ((j * step) % N);
        const double *y = out + 2 * (r * m + k);
        sr += y[0] * w[0] - y[1] * w[1];
        si += y[0] * w[1] + y[1] * w[0];
      }
      acc[2 * q] = sr;
      acc[2 * q + 1] = si;
    }
    for (int q = 0; q < p; q++) {
      out[2 * (k + q * m)] = acc[2 * q];
      out[2 * (k + q * m) + 1] = acc[2 * q + 1];
    }
  }
}

static double *make_twiddles(int n, int sign) {
  double *tw = (double *)malloc(sizeof(double) * 2 * (size_t)n);
  const double two_pi = 6.283185307179586476925286766559;
  for (int j = 0; j < n; j++) {
    double a = two_pi * (double)j / (double)n;
    tw[2 * j] = cos(a);
    tw[2 * j + 1] = (double)sign * sin(a);
  }
  return tw;
}

void fe_fft1d(double *data, int n, long stride, int sign) {
  double *tw = make_twiddles(n, sign);
  double *line = (double *)malloc(sizeof(double) * 2 * (size_t)n);
  double *scratch = (double *)malloc(sizeof(double) * 2 * (size_t)n);
  fft_rec(data, stride, line, n, tw, n, scratch);
  for (int i = 0; i < n; i++) {
    data[2 * i * stride] = line[2 * i];
    data[2 * i * stride + 1] = line[2 * i + 1];
  }
  free(scratch);
  free(line);
  free(tw);
}

void fe_fft3d(double *data, int n0, int n1, int n2, int sign) {
  int dims[3] = {n0, n1, n2};
  long strides[3] = {(long)n1 * n2, n2, 1};
  int nmax = n0 > n1 ? (n0 > n2 ? n0 : n2) : (n1 > n2 ? n1 : n2);
  double *line = (double *)malloc(sizeof(double) * 2 * (size_t)nmax);
  double *scratch = (double *)malloc(sizeof(double) * 2 * (size_t)nmax);
  for (int ax = 0; ax < 3; ax++) {
    int n = dims[ax];
    if (n == 1) continue;
    double *tw = make_twiddles(n, sign);
    long st = strides[ax];
    /* iterate over all lines along axis ax */
    int o1 = (ax == 0) ? n1 : n0, o2 = (ax == 2) ? n1 : n2;
    for (int a = 0; a < o1; a++) {
      for (int b = 0; b < o2; b++) {
        long base;
        if (ax == 0) base = (long)a * n2 + b;
        else if (ax == 1) base = (long)a * n1 * n2 + b;
        else base = (long)a * n1 * n2 + (long)b * n2;
        double *d = data + 2 * base;
        fft_rec(d, st, line, n, tw, n, scratch);
        for (int i = 0; i < n; i++) {
          d[2 * i * st] = line[2 * i];
          d[2 * i * st + 1] = line[2 * i + 1];
        }
      }
    }
    free(tw);
  }
  free(scratch);
  free(line);
}
