/*
 * ref_harness.c -- drives the REFERENCE's own hot-path C routines (compiled
 * from the unmodified sources with oracle/build_ref.sh) on a system described
 * in a project binary file, and dumps their outputs for golden fixtures.
 *
 * Test infrastructure only.  It plays the part of the reference's main.c
 * initialisation (main.c:298-496): it defines the globals (MAIN), fills the
 * fields the hot path reads -- sim (read_sim.c), box (read_config.c:317-331),
 * atom/atnopbc/pott (read_topology.c), bond/bend/xint (read_topology.c),
 * epstmp/sigtmp/atom_type (read_atom.c), the nlist arrays (allocate.c:312-360)
 * and the SPME arrays (allocate.c:446-505) -- then calls the reference's own
 * setlj(), ewald_setup(), nblist(), forces(), pme_calc(), integrate_vverlet(),
 * integrate_nhc() and kinet() exactly as its step loops do
 * (nve_md.c:359-393, nvt_md.c:529-531).
 *
 * Build flags: -DNLIST -DEWALD -DSPME -DSTYPE (exclusions through the STYPE
 * hash, nblist.c:156-174; cnonbond_nblist.c:202-266).
 *
 * Usage:  ref_harness <mode> <system.bin> <out.bin> [nsteps]
 *   mode nblist : counts + rows of nlist and nlist_ew (+ xflags)
 *   mode forces : force/energy breakdown at the input configuration
 *   mode nve    : nsteps of NVE velocity Verlet (list rebuilt every nlist)
 *   mode nhc    : nsteps of NHC-VV (integrate_nhc / integrate_vverlet / integrate_nhc)
 *   mode drift  : drift() (drift.c:21) on the input velocities
 *   mode mtsnhc : as mts with integrate_mts_nhc.c:37 (nvt_md.c:552) and
 *                 sim.xRESPA = argv[6] (0: thermostat per long step, 1:
 *                 per short step)
 *   mode mts    : nsteps long steps of RESPA (integrate_mts.c:37) with
 *                 nshort short steps each (argv[5]; init.c:314 sets
 *                 dtlong = dt * nshort); force_short / force_long /
 *                 forces / kinet before the loop as nve_md.c:298-304 does
 *   mode nlcheck (the -DDLIST build, ref_harness_dlist): nblist, then per
 *                 case of <cases.bin> (the 4th argument) the snapshot
 *                 positions plus the case's displacements, pbc_all, and
 *                 nl_check(lb, ub) (nblist.c:607-647); dumps the flags and
 *                 the checked positions
 *   mode mc      (the -DMC classic-Ewald build, ref_harness_mc, feature flags
 *                 -DNLIST -DEWALD -DMC -DSTYPE without SPME): <moves.bin>
 *                 (4th argument) gives kmax, max_k_square and trial moves
 *                 (site range and new positions); ewald_setup, nblist, then
 *                 enbnd_mc(lb, ub) -- its ewald_kspace_mc and ewald_rspace_mc
 *                 (ewald_mc.c:42-641) included -- on the configuration before
 *                 and after each move (the move undone after), as
 *                 forces_mc(lb, ub, 0|1) does around a trial move
 *                 (forces_mc.c:90-573, mcmove_displ.c:70,117)
 */
#define MAIN
#include "defines.h"

#include <stdint.h>

void setlj(void);
void ewald_setup(int);
void nblist(int);
#ifdef MC
void enbnd_mc(int, int, int, double *);
#else
void forces(int);
void charge_grid(int);
void pme_calc(int, double *);
void cnonbondnl(int, double *);
void integrate_vverlet(int, double);
void integrate_mts(int, double);
void integrate_mts_nhc(int, double);
void force_short(int);
void force_long(int);
void integrate_nhc(double, int);
void kinet(int);
void pbc_all(int);
#endif
#ifdef DLIST
void nl_check(int, int, int);
#endif
#ifndef MC
void drift(int);
#endif
#ifndef MC
double cbond(int);
double cbend(int);
double curey(int);
double ctorsion(int);
double cimproper(int);
#endif

static FILE *g_out;

static void die(const char *m) {
  fprintf(stderr, "ref_harness: %s\n", m);
  exit(2);
}

static void rd(void *p, size_t sz, size_t n, FILE *f) {
  if (fread(p, sz, n, f) != n) die("short read");
}

static void wr(const void *p, size_t sz, size_t n) {
  if (fwrite(p, sz, n, g_out) != n) die("short write");
}

static void wr_tag(const char *tag, int64_t nbytes) {
  char t[16];
  memset(t, 0, sizeof t);
  strncpy(t, tag, 15);
  wr(t, 1, 16);
  wr(&nbytes, sizeof nbytes, 1);
}

static void dump_d(const char *tag, const double *p, int64_t n) {
  wr_tag(tag, n * 8);
  wr(p, 8, (size_t)n);
}

static void dump_i(const char *tag, const int *p, int64_t n) {
  wr_tag(tag, n * 4);
  wr(p, 4, (size_t)n);
}

/* ---- system file (written by oracle/sysfile.py) ---- */
static int N, NT, NBD, NBN, NX, NHC_M;
static double *vel0;

static void load_system(const char *path) {
  FILE *f = fopen(path, "rb");
  if (!f) die("cannot open system file");
  char magic[8];
  rd(magic, 1, 8, f);
  if (memcmp(magic, "FESYS01", 7) != 0) die("bad magic");
  int32_t hi[12];
  rd(hi, 4, 12, f);
  N = hi[0]; NT = hi[1]; NBD = hi[2]; NBN = hi[3]; NX = hi[4];
  sim.grid[0] = hi[5]; sim.grid[1] = hi[6]; sim.grid[2] = hi[7];
  sim.order = hi[8];
  NHC_M = hi[9];
  sim.nlist = (unsigned long)hi[10];
  double hd[12];
  rd(hd, 8, 12, f);
  int k = 0;
  sim.NB = 1;
  box[k].lx = hd[0]; box[k].ly = hd[1]; box[k].lz = hd[2];
  sim.rc = hd[3]; sim.rclist = hd[4]; sim.rclist_ew = hd[5]; sim.rc_ew = hd[6];
  sim.kappa[k] = hd[7]; sim.epsRF[k] = hd[8]; sim.dt = hd[9]; sim.T[k] = hd[10];
  nhc[k].Q = hd[11];

  /* read_config.c:317-331 */
  box[k].hx = box[k].lx / 2.0; box[k].hy = box[k].ly / 2.0; box[k].hz = box[k].lz / 2.0;
  box[k].vol = box[k].lx * box[k].ly * box[k].lz;
  box[k].rc2 = sim.rc * sim.rc;
  box[k].least_boxh = (box[k].lx < box[k].ly ? (box[k].lx < box[k].lz ? box[k].lx : box[k].lz)
                                             : (box[k].ly < box[k].lz ? box[k].ly : box[k].lz)) /
                      2.0;
  box[k].rc4 = box[k].rc2 * box[k].rc2;
  box[k].boxns = N;
  box[k].nfree = 3.0 * N - 3.0;

  /* atom types (read_atom.c): CHARMM eps (kcal/mol, <= 0) and Rmin/2 */
  NUM_ATOM = NT;
  atom_type = calloc(NT, sizeof(struct atomtype));
  for (int t = 0; t < NT; t++) {
    double e, s;
    rd(&e, 8, 1, f);
    rd(&s, 8, 1, f);
    atom_type[t].atomid = t;
    epstmp[0][t] = e; sigtmp[0][t] = s;
    epstmp[1][t] = e; sigtmp[1][t] = s;
  }
  NUM_NBFIX = 0;

  atom = calloc(1, sizeof(struct atoms *));
  atnopbc = calloc(1, sizeof(struct atoms *));
  pott = calloc(1, sizeof(struct inter *));
  atom[k] = calloc(N, sizeof(struct atoms));
  atnopbc[k] = calloc(N, sizeof(struct atoms));
  pott[k] = calloc(N, sizeof(struct inter));
  vel0 = calloc(3 * (size_t)N, sizeof(double));
  for (int i = 0; i < N; i++) {
    double r[5];
    int32_t t;
    rd(r, 8, 5, f);
    rd(&t, 4, 1, f);
    atom[k][i].x = r[0]; atom[k][i].y = r[1]; atom[k][i].z = r[2];
    atom[k][i].q = r[3];
    atom[k][i].atomid = t;
    atnopbc[k][i] = atom[k][i];
    pott[k][i].qq = r[3];
    pott[k][i].mas = r[4];
    pott[k][i].id = t;
  }
  rd(vel0, 8, 3 * (size_t)N, f);

  bond = calloc(1, sizeof(struct bonds *));
  bond[k] = calloc(NBD + 1, sizeof(struct bonds));
  bondN[k] = NBD;
  for (int i = 0; i < NBD; i++) {
    int32_t ab[2];
    double p[2];
    rd(ab, 4, 2, f);
    rd(p, 8, 2, f);
    bond[k][i].a = ab[0]; bond[k][i].b = ab[1];
    bond[k][i].req = p[0]; bond[k][i].krbond = p[1];
  }
  bend = calloc(1, sizeof(struct bends *));
  bend[k] = calloc(NBN + 1, sizeof(struct bends));
  bendN[k] = NBN;
  for (int i = 0; i < NBN; i++) {
    int32_t abc[3];
    double p[2];
    rd(abc, 4, 3, f);
    rd(p, 8, 2, f);
    bend[k][i].a = abc[0]; bend[k][i].b = abc[1]; bend[k][i].c = abc[2];
    bend[k][i].angeq = p[0]; bend[k][i].krbend = p[1];
  }
  xint = calloc(1, sizeof(struct excinter *));
  xint[k] = calloc(NX + 1, sizeof(struct excinter));
  xintN[k] = NX;
  for (int i = 0; i < NX; i++) {
    int32_t e[3];
    rd(e, 4, 3, f);
    xint[k][i].a = e[0]; xint[k][i].b = e[1]; xint[k][i].xflag = e[2];
  }
  /* optional trailer "FEXT": Urey-Bradley, torsion and improper records
   * (read_topology.c fills urey[k], tors[k], impr[k]) */
  int32_t next[3] = {0, 0, 0};
  char tag[4];
  if (fread(tag, 1, 4, f) == 4) {
    if (memcmp(tag, "FEXT", 4) != 0) die("bad trailer");
    rd(next, 4, 3, f);
  }
  urey = calloc(1, sizeof(struct ureys *));
  urey[k] = calloc(next[0] + 1, sizeof(struct ureys));
  ureyN[k] = next[0];
  for (int i = 0; i < next[0]; i++) {
    int32_t ab[2];
    double p[2];
    rd(ab, 4, 2, f);
    rd(p, 8, 2, f);
    urey[k][i].a = ab[0]; urey[k][i].b = ab[1];
    urey[k][i].Seq = p[0]; urey[k][i].k = p[1];
  }
  tors = calloc(1, sizeof(struct torsions *));
  tors[k] = calloc(next[1] + 1, sizeof(struct torsions));
  torsN[k] = next[1];
  for (int i = 0; i < next[1]; i++) {
    int32_t abcd[4];
    double p[18];
    rd(abcd, 4, 4, f);
    rd(p, 8, 18, f);
    tors[k][i].a = abcd[0]; tors[k][i].b = abcd[1];
    tors[k][i].c = abcd[2]; tors[k][i].d = abcd[3];
    for (int t = 0; t < 6; t++) {
      tors[k][i].kphi[t] = p[t];
      tors[k][i].nphi[t] = p[6 + t];
      tors[k][i].delphi[t] = p[12 + t];
    }
    tors[k][i].phitag = 1; /* every angle lands in .phi (ctorsion.c:172) */
  }
  impr = calloc(1, sizeof(struct impropers *));
  impr[k] = calloc(next[2] + 1, sizeof(struct impropers));
  imprN[k] = next[2];
  for (int i = 0; i < next[2]; i++) {
    int32_t abcd[4];
    double p[2];
    rd(abcd, 4, 4, f);
    rd(p, 8, 2, f);
    impr[k][i].a = abcd[0]; impr[k][i].b = abcd[1];
    impr[k][i].c = abcd[2]; impr[k][i].d = abcd[3];
    impr[k][i].kimpr = p[0]; impr[k][i].angeq = p[1];
  }
  fclose(f);

  /* STYPE ljset: NUM_ATOM x NUM_ATOM (read_topology allocates it) */
  ljset = calloc(NT, sizeof(struct inter *));
  for (int t = 0; t < NT; t++) ljset[t] = calloc(NT, sizeof(struct inter));
  table = calloc(1, sizeof(struct hashlist *));
}

static void alloc_state(void) {
  int k = 0;
  ff = calloc(1, sizeof(struct veloc *));
  vv = calloc(1, sizeof(struct veloc *));
  uu = calloc(1, sizeof(struct veloc *));
  ff[k] = calloc(N, sizeof(struct veloc));
  ff_short = calloc(1, sizeof(struct veloc *));
  ff_long = calloc(1, sizeof(struct veloc *));
  ff_short[k] = calloc(N, sizeof(struct veloc));
  ff_long[k] = calloc(N, sizeof(struct veloc));
  vv[k] = calloc(N, sizeof(struct veloc));
  uu[k] = calloc(N, sizeof(struct veloc));
  for (int i = 0; i < N; i++) {
    vv[k][i].x = vel0[3 * i];
    vv[k][i].y = vel0[3 * i + 1];
    vv[k][i].z = vel0[3 * i + 2];
    uu[k][i] = vv[k][i];
  }
  /* allocate.c:312-360; every row sized N so no capacity exit can fire */
  max_num_neighbors = N;
  nlist = calloc(1, sizeof(struct nlist_def));
  nlist_ew = calloc(1, sizeof(struct nlist_def));
  struct nlist_def *ls[2] = {&nlist[k], &nlist_ew[k]};
  for (int l = 0; l < 2; l++) {
    ls[l]->count = calloc(N, sizeof(int));
    ls[l]->list = calloc(N, sizeof(int *));
    ls[l]->xflag = calloc(N, sizeof(int *));
    for (int i = 0; i < N; i++) {
      ls[l]->list[i] = calloc(N, sizeof(int));
      ls[l]->xflag[i] = calloc(N, sizeof(int));
    }
  }
#ifdef SPME
  /* allocate.c:446-505 */
  int ORDER = sim.order;
  int GX = sim.grid[0], GY = sim.grid[1], GZ = sim.grid[2];
  ss = calloc(N + 1, sizeof(struct pmedat));
  mm = calloc(N + 1, sizeof(struct pmedat *));
  dm = calloc(N + 1, sizeof(struct pmedat *));
  for (int i = 0; i < N + 1; i++) {
    mm[i] = calloc(ORDER + 1, sizeof(struct pmedat));
    dm[i] = calloc(ORDER + 1, sizeof(struct pmedat));
  }
  mn = calloc(ORDER + 2, sizeof(double));
  dmn = calloc(ORDER + 2, sizeof(double));
  bsp_modx = calloc(GX + 5, sizeof(double));
  bsp_mody = calloc(GY + 5, sizeof(double));
  bsp_modz = calloc(GZ + 5, sizeof(double));
  gridmx = greater(GX, greater(GY, GZ)) + 5;
  bsp_arr = calloc(gridmx, sizeof(double));
  long ngrid = (long)(GX + 5) * (GY + 5) * (GZ + 5);
  qgrida = fftw_malloc(sizeof(fftw_complex) * ngrid);
  memset(qgrida, 0, sizeof(fftw_complex) * ngrid);
#endif

  nhc[k].M = NHC_M > 0 ? NHC_M : 1;
  nhc[k].Nc = 1;
  nhc[k].Nys = 1;
  nhc[k].w = calloc(1, sizeof(double));
  nhc[k].zeta = calloc(nhc[k].M, sizeof(struct NH_therm));
  /* read_config.c:358-383 */
  double kT = KB * sim.T[k] * 1E-4;
  double Q = nhc[k].Q;
  for (int i = 0; i < nhc[k].M - 1; i++)
    nhc[k].zeta[i + 1].G = (Q * nhc[k].zeta[i].v * nhc[k].zeta[i].v - kT) / Q;
  nhc[k].w[0] = 1;
}

static void dump_xyz(const char *tag, struct veloc *v) {
  double *b = malloc(sizeof(double) * 3 * (size_t)N);
  for (int i = 0; i < N; i++) {
    b[3 * i] = v[i].x; b[3 * i + 1] = v[i].y; b[3 * i + 2] = v[i].z;
  }
  dump_d(tag, b, 3 * (int64_t)N);
  free(b);
}

static void dump_pos(const char *tag, struct atoms *a) {
  double *b = malloc(sizeof(double) * 3 * (size_t)N);
  for (int i = 0; i < N; i++) {
    b[3 * i] = a[i].x; b[3 * i + 1] = a[i].y; b[3 * i + 2] = a[i].z;
  }
  dump_d(tag, b, 3 * (int64_t)N);
  free(b);
}

static void dump_list(const char *tag, struct nlist_def *l) {
  char t[16];
  int64_t tot = 0;
  for (int i = 0; i < N; i++) tot += l->count[i];
  int *rows = malloc(sizeof(int) * (size_t)(tot + 1));
  int *fl = malloc(sizeof(int) * (size_t)(tot + 1));
  int64_t p = 0;
  for (int i = 0; i < N; i++)
    for (int j = 0; j < l->count[i]; j++) {
      rows[p] = l->list[i][j];
      fl[p] = l->xflag[i][j];
      p++;
    }
  snprintf(t, sizeof t, "%s_cnt", tag);
  dump_i(t, l->count, N);
  snprintf(t, sizeof t, "%s_idx", tag);
  dump_i(t, rows, tot);
  snprintf(t, sizeof t, "%s_flg", tag);
  dump_i(t, fl, tot);
  free(rows);
  free(fl);
}

static void en_record(double *r) {
  /* order: kinet, bond, bend, nbond, nbonds, coulomb, rewald, rewalds,
   *        kewald, sewald, iewald, tewald */
  int k = 0;
  r[0] = en[k].kinet; r[1] = en[k].bond; r[2] = en[k].bend;
  r[3] = en[k].nbond; r[4] = en[k].nbonds; r[5] = en[k].coulomb;
  r[6] = en[k].rewald; r[7] = en[k].rewalds; r[8] = en[k].kewald;
  r[9] = en[k].sewald; r[10] = en[k].iewald; r[11] = en[k].tewald;
}

#ifdef MC
/* The classic-Ewald MC energies (enbnd_mc with ewald_kspace_mc and
 * ewald_rspace_mc) before and after each trial move of <moves.bin>:
 * int32 kmax, max_k_square, nmoves; per move int32 lb, ub, then (ub - lb)
 * x 3 doubles of new positions. */
static void run_mc(const char *moves_path) {
  int k = 0;
  FILE *mf = fopen(moves_path, "rb");
  if (!mf) die("cannot open moves file");
  int32_t h[3];
  rd(h, 4, 3, mf);
  sim.kmax[k][0] = sim.kmax[k][1] = sim.kmax[k][2] = h[0];
  sim.max_k_square[k] = h[1];
  /* allocate.c:207-230 (MC force accumulators), 506-516 (k-vectors) */
  ffox = calloc(1, sizeof(double *));
  ffoy = calloc(1, sizeof(double *));
  ffoz = calloc(1, sizeof(double *));
  ffox[k] = calloc(N, sizeof(double));
  ffoy[k] = calloc(N, sizeof(double));
  ffoz[k] = calloc(N, sizeof(double));
  kvec = calloc(1, sizeof(double *));
  kvec[k] = calloc((size_t)(h[0] + 1) * (2 * h[0] + 1) * (2 * h[0] + 1), sizeof(double));
  total_k_vectors = calloc(1, sizeof(int));
  setlj();
  ewald_setup(k);
  nblist(k);
  int nm = h[2];
  double *e = malloc(sizeof(double) * 16 * (size_t)(nm + 1));
  int32_t *rng = malloc(sizeof(int32_t) * 2 * (size_t)(nm + 1));
  enbnd_mc(0, N, k, e); /* the whole configuration */
  rng[0] = 0;
  rng[1] = N;
  double tk = total_k_vectors[k];
  for (int m = 0; m < nm; m++) {
    int32_t r[2];
    rd(r, 4, 2, mf);
    int lb = r[0], ub = r[1];
    if (lb < 0 || ub > N || ub <= lb || ub - lb > 64) die("bad move range");
    double old[64][3], nw[64][3];
    rd(nw, 8, 3 * (size_t)(ub - lb), mf);
    enbnd_mc(lb, ub, k, e + 16 * (m + 1)); /* forces_mc(lb, ub, 0, k) */
    for (int i = lb; i < ub; i++) {
      old[i - lb][0] = atom[k][i].x; old[i - lb][1] = atom[k][i].y; old[i - lb][2] = atom[k][i].z;
      atom[k][i].x = nw[i - lb][0]; atom[k][i].y = nw[i - lb][1]; atom[k][i].z = nw[i - lb][2];
    }
    enbnd_mc(lb, ub, k, e + 16 * (m + 1) + 8); /* forces_mc(lb, ub, 1, k) */
    for (int i = lb; i < ub; i++) {
      atom[k][i].x = old[i - lb][0]; atom[k][i].y = old[i - lb][1]; atom[k][i].z = old[i - lb][2];
    }
    rng[2 * (m + 1)] = lb;
    rng[2 * (m + 1) + 1] = ub;
  }
  fclose(mf);
  /* e[0..7]: enbnd_mc energy[] of the whole box; per move 8 before, 8 after */
  dump_d("mc_energy", e, 16 * (int64_t)(nm + 1));
  dump_i("mc_rng_idx", rng, 2 * (int64_t)(nm + 1));
  dump_d("mc_nk", &tk, 1);
  free(e);
  free(rng);
}
#endif

int main(int argc, char **argv) {
  if (argc < 4) die("usage: ref_harness <mode> <system.bin> <out.bin> [nsteps]");
  const char *mode = argv[1];
  load_system(argv[2]);
  alloc_state();
  g_out = fopen(argv[3], "wb");
  if (!g_out) die("cannot open output");
  int k = 0;
#ifdef MC
  if (strcmp(mode, "mc") != 0 || argc < 5) die("the MC build runs: mc <system> <out> <moves>");
  run_mc(argv[4]);
  fclose(g_out);
  return 0;
#endif
  setlj();
  ewald_setup(k);

#ifndef MC
  if (strcmp(mode, "nblist") == 0) {
    nblist(k);
    dump_list("nl", &nlist[k]);
    dump_list("nlew", &nlist_ew[k]);
  } else if (strcmp(mode, "forces") == 0) {
    nblist(k);
    /* SPME charge grid after spreading (pme_qgrid.c:13-121) */
    charge_grid(k);
    {
      int ng = sim.grid[0] * sim.grid[1] * sim.grid[2];
      double *g = malloc(sizeof(double) * (size_t)ng);
      for (int i = 0; i < ng; i++) g[i] = qgrida[i][0];
      dump_d("qgrid", g, ng);
      free(g);
    }
    /* reciprocal part alone (pme_calc.c:18-119) */
    double epme[3];
    memset(ff[k], 0, sizeof(struct veloc) * N);
    pme_calc(k, epme);
    dump_xyz("f_pme", ff[k]);
    dump_d("e_pme", epme, 3);
    /* non-bonded incl. reciprocal (cnonbond_nblist.c:51-622) */
    double enb[8];
    memset(ff[k], 0, sizeof(struct veloc) * N);
    cnonbondnl(k, enb);
    dump_xyz("f_nonbond", ff[k]);
    dump_d("e_nonbond", enb, 8);
    /* bonded alone */
    memset(ff[k], 0, sizeof(struct veloc) * N);
    double eb[2];
    eb[0] = cbond(k);
    eb[1] = cbend(k);
    dump_xyz("f_bonded", ff[k]);
    dump_d("e_bonded", eb, 2);
    /* Urey-Bradley, torsions and impropers alone (forces.c:183-188) */
    double e3[3];
    memset(ff[k], 0, sizeof(struct veloc) * N);
    e3[0] = curey(k);
    dump_xyz("f_urey", ff[k]);
    memset(ff[k], 0, sizeof(struct veloc) * N);
    e3[1] = ctorsion(k);
    dump_xyz("f_tors", ff[k]);
    memset(ff[k], 0, sizeof(struct veloc) * N);
    e3[2] = cimproper(k);
    dump_xyz("f_impr", ff[k]);
    dump_d("e_ext", e3, 3);
    {
      double *tau = malloc(sizeof(double) * (size_t)(torsN[k] + 1));
      for (int i = 0; i < torsN[k]; i++) tau[i] = tors[k][i].phi;
      dump_d("tau", tau, torsN[k]);
      free(tau);
    }
    /* full forces() (forces.c:118-446) */
    forces(k);
    dump_xyz("f_total", ff[k]);
    double r[12];
    kinet(k);
    en_record(r);
    dump_d("en", r, 12);
    double rx[3] = {en[k].urey, en[k].tors, en[k].impr};
    dump_d("en_ext", rx, 3);
  } else if (strcmp(mode, "drift") == 0) {
    /* drift.c:21: net-momentum removal from the input velocities */
    drift(k);
    dump_xyz("vel", vv[k]);
    dump_xyz("vel_uu", uu[k]);
  } else if (strcmp(mode, "nve") == 0 || strcmp(mode, "nhc") == 0) {
    int nsteps = argc > 4 ? atoi(argv[4]) : 10;
    int use_nhc = strcmp(mode, "nhc") == 0;
    /* main.c:475-496: list, forces, kinetic energy before the loop */
    nblist(k);
    forces(k);
    kinet(k);
    double *rec = malloc(sizeof(double) * 12 * (size_t)(nsteps + 1));
    en_record(rec);
    for (int i = 1; i <= nsteps; i++) {
      if (i % sim.nlist == 0) nblist(k); /* nve_md.c:366 */
      if (use_nhc) {                     /* nvt_md.c:529-531 */
        integrate_nhc(sim.dt, k);
        integrate_vverlet(k, 1.0);
        integrate_nhc(sim.dt, k);
      } else {
        integrate_vverlet(k, 1.0); /* nve_md.c:393 */
      }
      kinet(k); /* nve_md.c:418 */
      en_record(rec + 12 * i);
    }
    dump_d("en_steps", rec, 12 * (int64_t)(nsteps + 1));
    dump_pos("pos", atom[k]);
    dump_pos("pos_nopbc", atnopbc[k]);
    dump_xyz("vel", vv[k]);
    dump_xyz("force", ff[k]);
    if (use_nhc) {
      double z[3 * 16];
      int M = nhc[k].M < 16 ? nhc[k].M : 16;
      for (int j = 0; j < M; j++) {
        z[3 * j] = nhc[k].zeta[j].r;
        z[3 * j + 1] = nhc[k].zeta[j].v;
        z[3 * j + 2] = nhc[k].zeta[j].G;
      }
      dump_d("zeta", z, 3 * (int64_t)M);
    }
    free(rec);
  } else if (strcmp(mode, "mts") == 0 || strcmp(mode, "mtsnhc") == 0) {
    int nsteps = argc > 4 ? atoi(argv[4]) : 6;
    int use_nhc = strcmp(mode, "mtsnhc") == 0;
    sim.nsteps = argc > 5 ? atoi(argv[5]) : 4;
    sim.xRESPA[k] = argc > 6 ? atoi(argv[6]) : 0;
    sim.dtlong = sim.dt * sim.nsteps; /* init.c:314 */
    nblist(k);
    force_short(k); /* nve_md.c:298-304 */
    force_long(k);
    forces(k);
    kinet(k);
    double *rec = malloc(sizeof(double) * 15 * (size_t)(nsteps + 1));
    en_record(rec);
    rec[12] = en[k].urey; rec[13] = en[k].tors; rec[14] = en[k].impr;
    for (int i = 1; i <= nsteps; i++) {
      if (i % sim.nlist == 0) nblist(k);
      if (use_nhc) integrate_mts_nhc(k, 1.0); /* nvt_md.c:552 */
      else integrate_mts(k, 1.0);             /* nve_md.c:412 */
      kinet(k);
      en_record(rec + 15 * i);
      rec[15 * i + 12] = en[k].urey; rec[15 * i + 13] = en[k].tors;
      rec[15 * i + 14] = en[k].impr;
    }
    dump_d("en_steps", rec, 15 * (int64_t)(nsteps + 1));
    dump_pos("pos", atom[k]);
    dump_pos("pos_nopbc", atnopbc[k]);
    dump_xyz("vel", vv[k]);
    dump_xyz("vel_uu", uu[k]);
    dump_xyz("force", ff[k]);
    dump_xyz("f_short", ff_short[k]);
    dump_xyz("f_long", ff_long[k]);
    if (use_nhc) {
      double z[3 * 16];
      int M = nhc[k].M < 16 ? nhc[k].M : 16;
      for (int j = 0; j < M; j++) {
        z[3 * j] = nhc[k].zeta[j].r;
        z[3 * j + 1] = nhc[k].zeta[j].v;
        z[3 * j + 2] = nhc[k].zeta[j].G;
      }
      dump_d("zeta", z, 3 * (int64_t)M);
    }
    free(rec);
#ifdef DLIST
  } else if (strcmp(mode, "nlcheck") == 0) {
    /* allocate.c:51-74 */
    rx0 = calloc(1, sizeof(double *));
    ry0 = calloc(1, sizeof(double *));
    rz0 = calloc(1, sizeof(double *));
    rx0[k] = calloc(N, sizeof(double));
    ry0[k] = calloc(N, sizeof(double));
    rz0[k] = calloc(N, sizeof(double));
    nl_flag = calloc(1, sizeof(int));
    nblist(k); /* takes the snapshot, nblist.c:583-591 */
    if (argc < 5) die("nlcheck needs a cases file");
    FILE *cf = fopen(argv[4], "rb");
    if (!cf) die("cannot open cases file");
    int32_t ncase;
    rd(&ncase, 4, 1, cf);
    int *flags = malloc(sizeof(int) * (size_t)ncase);
    double *pos = malloc(sizeof(double) * 3 * (size_t)N * (size_t)ncase);
    for (int c = 0; c < ncase; c++) {
      int32_t hdr[3];
      rd(hdr, 4, 3, cf);
      for (int i = 0; i < N; i++) {
        atom[k][i].x = rx0[k][i];
        atom[k][i].y = ry0[k][i];
        atom[k][i].z = rz0[k][i];
      }
      for (int m = 0; m < hdr[2]; m++) {
        int32_t idx;
        double d[3];
        rd(&idx, 4, 1, cf);
        rd(d, 8, 3, cf);
        if (idx < 0 || idx >= N) die("case index out of range");
        atom[k][idx].x += d[0];
        atom[k][idx].y += d[1];
        atom[k][idx].z += d[2];
      }
      pbc_all(k);
      nl_flag[k] = 0;
      nl_check(hdr[0], hdr[1], k);
      flags[c] = nl_flag[k];
      for (int i = 0; i < N; i++) {
        pos[3 * ((size_t)c * N + i)] = atom[k][i].x;
        pos[3 * ((size_t)c * N + i) + 1] = atom[k][i].y;
        pos[3 * ((size_t)c * N + i) + 2] = atom[k][i].z;
      }
    }
    fclose(cf);
    double *p0 = malloc(sizeof(double) * 3 * (size_t)N);
    for (int i = 0; i < N; i++) {
      p0[3 * i] = rx0[k][i];
      p0[3 * i + 1] = ry0[k][i];
      p0[3 * i + 2] = rz0[k][i];
    }
    dump_d("pos0", p0, 3 * (int64_t)N);
    dump_d("pos_cases", pos, 3 * (int64_t)N * ncase);
    dump_i("nl_flg", flags, ncase);
    free(p0);
    free(pos);
    free(flags);
#endif
  } else {
    die("unknown mode");
  }
#endif
  fclose(g_out);
  return 0;
}
