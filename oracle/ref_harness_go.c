/*
 * ref_harness_go.c -- TEST INFRASTRUCTURE ONLY.  Drives the reference's own
 * Go-model routines (cgolik.c, compiled with -DGOLIK -DNLIST from the
 * unmodified sources) on one chain, as forces() does in a GOLIK build:
 * cbb_golik (bonds), cba_golik (bends), cda_golik (torsions) and
 * cnbnd_golik (native and non-native pairs), each into a zeroed ff[0].
 *
 * The parameters are set the way read_golik.c:14-205 / set_go_params
 * (read_golik.c:210-360, with GOBT) would from a native structure: every
 * pair a < b gets eps = golik eps and sigma = 2^(-1/6) r0 for a native
 * contact (distance r0), 2^(-1/6) d_repulsive otherwise; bonded pairs
 * eps = sigma = 0 and no contact (read_golik.c:99-110); bond lengths and
 * bend angles of the native structure; torsion phases zero (GOBT).  The pair
 * list holds every pair b > a (cnbnd_golik applies its own cutoffs).
 *
 * Input (binary, little endian): int32 N; double L, eps [kJ/mol],
 * d_repulsive, rc; double pos[3N]; double bond_r0[N-1]; double
 * bend_t0[N-2]; int32 nnat; nnat x (int32 a, int32 b, double r0) with a < b.
 * Output: tagged doubles f_bond, f_bend, f_tors, f_nb (3N each) and en
 * (ebond, ebend, etors, cnbnd_golik's energy[0..4]).
 *
 * Usage: ref_harness_go <system.bin> <out.bin>
 */
#define MAIN
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "defines.h"

double cbb_golik(int);
double cba_golik(int);
double cda_golik(int);
void cnbnd_golik(int, double *);

static FILE *g_out;

static void die(const char *m) {
  fprintf(stderr, "ref_harness_go: %s\n", m);
  exit(2);
}

static void rd(void *p, size_t sz, size_t n, FILE *f) {
  if (fread(p, sz, n, f) != n) die("short read");
}

static void dump_d(const char *tag, const double *p, int64_t n) {
  char t[16];
  memset(t, 0, sizeof t);
  strncpy(t, tag, 15);
  int64_t nb = n * 8;
  if (fwrite(t, 1, 16, g_out) != 16 || fwrite(&nb, 8, 1, g_out) != 1 ||
      fwrite(p, 8, (size_t)n, g_out) != (size_t)n)
    die("short write");
}

static void dump_ff(const char *tag, int N) {
  double *b = malloc(sizeof(double) * 3 * (size_t)N);
  for (int i = 0; i < N; i++) {
    b[3 * i] = ff[0][i].x;
    b[3 * i + 1] = ff[0][i].y;
    b[3 * i + 2] = ff[0][i].z;
  }
  dump_d(tag, b, 3 * (int64_t)N);
  free(b);
}

static void zero_ff(int N) {
  for (int i = 0; i < N; i++) ff[0][i].x = ff[0][i].y = ff[0][i].z = 0.0;
}

int main(int argc, char **argv) {
  if (argc < 3) die("usage: ref_harness_go <system.bin> <out.bin>");
  FILE *f = fopen(argv[1], "rb");
  if (!f) die("cannot open input");
  int32_t N;
  rd(&N, 4, 1, f);
  double hd[4];
  rd(hd, 8, 4, f);
  const double L = hd[0], eps = hd[1], d_rep = hd[2], rc = hd[3];
  const double factor = pow(2.0, -(1.0 / 6.0));  /* read_golik.c:38 */

  sim.NB = 1;
  sim.rc = rc;
  box[0].boxns = N;
  box[0].lx = box[0].ly = box[0].lz = L;
  box[0].hx = box[0].hy = box[0].hz = 0.5 * L;
  box[0].rc2 = rc * rc;
  box[0].rc4 = box[0].rc2 * box[0].rc2;

  atom = calloc(1, sizeof(struct atoms *));
  atom[0] = calloc(N, sizeof(struct atoms));
  ff = calloc(1, sizeof(struct veloc *));
  ff[0] = calloc(N, sizeof(struct veloc));
  double *pos = malloc(sizeof(double) * 3 * (size_t)N);
  rd(pos, 8, 3 * (size_t)N, f);
  for (int i = 0; i < N; i++) {
    atom[0][i].x = pos[3 * i];
    atom[0][i].y = pos[3 * i + 1];
    atom[0][i].z = pos[3 * i + 2];
  }

  /* bonds, bends, torsions along the chain */
  bondN[0] = N - 1;
  bond = calloc(1, sizeof(struct bonds *));
  bond[0] = calloc(N, sizeof(struct bonds));
  for (int i = 0; i < N - 1; i++) {
    bond[0][i].a = i;
    bond[0][i].b = i + 1;
    rd(&bond[0][i].req, 8, 1, f);
  }
  bendN[0] = N - 2;
  bend = calloc(1, sizeof(struct bends *));
  bend[0] = calloc(N, sizeof(struct bends));
  for (int i = 0; i < N - 2; i++) {
    bend[0][i].a = i;
    bend[0][i].b = i + 1;
    bend[0][i].c = i + 2;
    rd(&bend[0][i].angeq, 8, 1, f);
  }
  torsN[0] = N - 3 > 0 ? N - 3 : 0;
  tors = calloc(1, sizeof(struct torsions *));
  tors[0] = calloc(N, sizeof(struct torsions));
  for (int i = 0; i < N - 3; i++) {
    tors[0][i].a = i;
    tors[0][i].b = i + 1;
    tors[0][i].c = i + 2;
    tors[0][i].d = i + 3;
  }

  /* golik and the pair table (set_go_params, read_golik.c:99-110) */
  golik = calloc(1, sizeof(struct golik_struct));
  golik[0].eps = eps;
  golik[0].d_repulsive = d_rep;
  golik[0].Psite = N;
  golik[0].contact = calloc(N, sizeof(int *));
  ljset = calloc(1, sizeof(struct interb));
  ljset[0].pot = calloc(N, sizeof(struct inter *));
  for (int a = 0; a < N; a++) {
    golik[0].contact[a] = calloc(N, sizeof(int));
    ljset[0].pot[a] = calloc(N, sizeof(struct inter));
    for (int b = a + 1; b < N; b++) {
      ljset[0].pot[a][b].eps = eps;
      ljset[0].pot[a][b].sig = factor * d_rep;
    }
  }
  int32_t nnat;
  rd(&nnat, 4, 1, f);
  for (int q = 0; q < nnat; q++) {
    int32_t ab[2];
    double r0;
    rd(ab, 4, 2, f);
    rd(&r0, 8, 1, f);
    if (ab[0] < 0 || ab[1] >= N || ab[0] >= ab[1]) die("bad native pair");
    golik[0].contact[ab[0]][ab[1]] = 1;
    ljset[0].pot[ab[0]][ab[1]].sig = factor * r0;
  }
  fclose(f);
  for (int a = 0; a + 1 < N; a++) {
    ljset[0].pot[a][a + 1].eps = 0.0;
    ljset[0].pot[a][a + 1].sig = 0.0;
    golik[0].contact[a][a + 1] = 0;
  }
  gosol.lambda = 0.0;

  /* every pair b > a in the list */
  nlist = calloc(1, sizeof(struct nlist_def));
  nlist[0].count = calloc(N, sizeof(int));
  nlist[0].list = calloc(N, sizeof(int *));
  for (int a = 0; a < N; a++) {
    nlist[0].list[a] = calloc(N, sizeof(int));
    for (int b = a + 1; b < N; b++) nlist[0].list[a][nlist[0].count[a]++] = b;
  }

  g_out = fopen(argv[2], "wb");
  if (!g_out) die("cannot open output");
  double en[8];
  zero_ff(N);
  en[0] = cbb_golik(0);
  dump_ff("f_bond", N);
  zero_ff(N);
  en[1] = cba_golik(0);
  dump_ff("f_bend", N);
  zero_ff(N);
  en[2] = cda_golik(0);
  dump_ff("f_tors", N);
  zero_ff(N);
  cnbnd_golik(0, en + 3);
  dump_ff("f_nb", N);
  dump_d("en", en, 8);
  fclose(g_out);
  return 0;
}
