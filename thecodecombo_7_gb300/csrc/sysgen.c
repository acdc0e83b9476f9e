/*
 * sysgen.c -- host helper for the synthetic workloads (not part of the
 * force engine): random sequential placement of molecule centres in a
 * periodic cube with a minimum centre distance, over a candidate stream the
 * caller draws (so the result depends only on the seed).
 *
 * Candidates are taken in order; each is accepted iff it lies at least dmin
 * (minimum image) from every earlier acceptance.  A cell grid of edge >= dmin
 * with up to 8 centres per cell keeps each test O(1).
 * Returns the number of candidates consumed, or -1 when the candidates ran
 * out first, or -2 when a cell overflowed.
 */
#include <math.h>
#include <stdlib.h>

long fe_sysgen_place(const double *cand, long ncand, double L, double dmin, long n_mol,
                     double *out, long *n_done) {
  int m = (int)(L / dmin);
  if (m < 1) m = 1;
  double cell = L / m;
  const int slots = 8;
  long ncell = (long)m * m * m;
  int *cnt = (int *)calloc((size_t)ncell, sizeof(int));
  double *occ = (double *)malloc(sizeof(double) * 3 * (size_t)ncell * slots);
  double d2 = dmin * dmin;
  long count = *n_done;
  /* re-insert centres already placed (resumption across candidate chunks) */
  for (long k = 0; k < count; k++) {
    int cx = ((int)((out[3 * k] + L / 2) / cell)) % m;
    int cy = ((int)((out[3 * k + 1] + L / 2) / cell)) % m;
    int cz = ((int)((out[3 * k + 2] + L / 2) / cell)) % m;
    long c = ((long)cx * m + cy) * m + cz;
    int s = cnt[c]++;
    for (int d = 0; d < 3; d++) occ[(c * slots + s) * 3 + d] = out[3 * k + d];
  }
  long used = -1;
  for (long t = 0; t < ncand && count < n_mol; t++) {
    const double *p = cand + 3 * t;
    int ci[3];
    for (int d = 0; d < 3; d++) ci[d] = ((int)((p[d] + L / 2) / cell)) % m;
    int ok = 1;
    for (int ox = -1; ox <= 1 && ok; ox++)
      for (int oy = -1; oy <= 1 && ok; oy++)
        for (int oz = -1; oz <= 1 && ok; oz++) {
          int x = (ci[0] + ox + m) % m, y = (ci[1] + oy + m) % m, z = (ci[2] + oz + m) % m;
          long c = ((long)x * m + y) * m + z;
          for (int s = 0; s < cnt[c]; s++) {
            double r2 = 0.0;
            for (int d = 0; d < 3; d++) {
              double dd = occ[(c * slots + s) * 3 + d] - p[d];
              dd -= L * rint(dd / L);
              r2 += dd * dd;
            }
            if (r2 < d2) {
              ok = 0;
              break;
            }
          }
        }
    if (!ok) continue;
    long c = ((long)ci[0] * m + ci[1]) * m + ci[2];
    if (cnt[c] >= slots) {
      free(cnt);
      free(occ);
      return -2;
    }
    int s = cnt[c]++;
    for (int d = 0; d < 3; d++) {
      occ[(c * slots + s) * 3 + d] = p[d];
      out[3 * count + d] = p[d];
    }
    count++;
    if (count == n_mol) used = t + 1;
  }
  free(cnt);
  free(occ);
  *n_done = count;
  return used;
}
