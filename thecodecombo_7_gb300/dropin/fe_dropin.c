/*
 * fe_dropin.c -- the reference's own hot-path symbols on top of libfe.so.
 *
 * Compiled INSIDE the reference's build, against its defines.h, in one of two
 * forms chosen by the reference's own feature flags:
 *
 *   MD form (-DNLIST -DEWALD -DSPME -DSTYPE): replaces nblist.c,
 *     cnonbond_nblist.c, pme_qgrid.c, pme_calc.c, pme_setup.c, pme_spline.c,
 *     integrate_vverlet.c, integrate_nhc.c, pbc_all.c, kinet.c, forces.c,
 *     drift.c, isokin.c, swap_box.c and, for RESPA (FP64 engine),
 *     integrate_mts.c, integrate_mts_nhc.c, force_short.c and force_long.c.
 *   MC form (-DNLIST -DEWALD -DMC -DSTYPE, classic Ewald, no SPME): replaces
 *     forces_mc.c, enbnd_mc.c, ewald_mc.c, nblist_pivot.c, drift.c.
 *
 * Each symbol keeps the prototype its callers declare and the semantics of
 * the routine it replaces: it brings the device up to date with the host
 * state that routine reads, runs the engine, and writes back the host state
 * that routine writes, so host code between calls (output, MC restores,
 * checkpoints) keeps working on the reference's own arrays.
 *
 * Uploads (MD form).  By default every call uploads the host arrays it reads.
 * With FE_DROPIN_TRUST=1 in the environment a box's arrays are uploaded only
 * when the device copy may differ from the host's: on the first call, and
 * after the shim's own host-side changes (swap_box, isokin); the shim's
 * downloads leave host and device equal.  That holds for the step loops whose
 * every routine is here (nve_md.c and nvt_md.c with velocity Verlet and
 * Nose-Hoover); host code that edits atom/vv/uu/ff between calls in other
 * ways (leap-frog integrate, Andersen collisions) needs the default.
 * FE_HOST_NLIST=1 makes nblist() also fill the host nlist[k] / nlist_ew[k]
 * rows for host readers (the device list is the engine's).
 *
 * MC form.  The engine keeps the configuration and the structure factor on
 * the device and evaluates a trial move's energy change incrementally.
 * forces_mc(lb, ub, 0, k) first brings the device up to date: if the host
 * still holds the previous trial positions the move was accepted and is
 * committed (fe_mc_accept); if it holds anything else the host was changed
 * (a restore after a rejected move needs nothing; swaps or edits elsewhere
 * re-upload and recompute S(k)).  Energies of the pairs touching [lb, ub)
 * and the whole reciprocal energy come from fe_mc_site_energy; the bonded
 * terms from the reference's own ebond_mc/ebend_mc/etors_mc/eimpr_mc.
 * forces_mc(lb, ub, 1, k) adds the change from fe_mc_delta_terms, so that
 * enmc[k].n_* - enmc[k].o_* and the update of en[k] are the reference's
 * (forces_mc.c:511-534).  The reference's MC forces (ffox ..) are not
 * produced: the moves use energies only.
 *
 * Bonded terms: bonds and bends come with the box; Urey-Bradley (urey[k]),
 * torsion (tors[k]) and improper (impr[k]) records are uploaded once with it
 * (fe_set_ureys / fe_set_torsions / fe_set_impropers), forces() fills
 * en[k].urey, .tors and .impr, and each torsion's angle goes back to
 * tors[k][i].phi / psi / theta when the system tags any (ctorsion.c:172-175).
 *
 * A -DBGO build of the reference gets the engine's BGO pair form (its
 * 12-10-6 LJ term, cnonbond_nblist.c:294-307) on every box.
 *
 * Errors print the engine's message and exit() with the reference's codes
 * (5: neighbour list over capacity, nblist.c:185-197; 20: non-neutral box,
 * ewald.c:185-194; 1 otherwise).  FE_PRECISION=mixed in the environment
 * selects the mixed-precision engine (MD form).
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>

#include "defines.h"
#include "fe.h"

#if defined(SPME)
#define FE_DROPIN_MD 1
#elif defined(MC)
#define FE_DROPIN_MC 1
#endif
#if !defined(NLIST) || !defined(EWALD) || !defined(STYPE) || \
    !(defined(FE_DROPIN_MD) || defined(FE_DROPIN_MC))
#error "fe_dropin.c replaces the NLIST + EWALD + STYPE build with SPME (MD) or MC (classic Ewald)"
#endif

static fe_box *g_fe[NBOXES];

static void fe_die(int rc, const char *where) {
  fprintf(stdout, "GPU engine error in %s: %s\n", where, fe_last_error());
  exit(rc == FE_ERR_OVERFLOW ? 5 : rc == FE_ERR_CHARGE ? 20 : 1);
}

#define FE_OR_DIE(call, where)   \
  do {                           \
    int rc_ = (call);            \
    if (rc_ != FE_OK) fe_die(rc_, where); \
  } while (0)

static int env_on(const char *name) {
  const char *v = getenv(name);
  return v && v[0] == '1';
}

/* Urey-Bradley (urey[k]), torsion (tors[k]) and improper (impr[k]) records
 * of read_topology.c, uploaded once with the box. */
static void set_ext_bonded(fe_box *b, int k) {
#ifndef NEUTRAL
  int nu = ureyN[k];
  if (nu > 0) {
    int *ab = malloc(sizeof(int) * 2 * nu);
    double *seq = malloc(sizeof(double) * nu), *kk = malloc(sizeof(double) * nu);
    for (int i = 0; i < nu; i++) {
      ab[2 * i] = urey[k][i].a;
      ab[2 * i + 1] = urey[k][i].b;
      seq[i] = urey[k][i].Seq;
      kk[i] = urey[k][i].k;
    }
    FE_OR_DIE(fe_set_ureys(b, nu, ab, seq, kk), "setup (ureys)");
    free(ab); free(seq); free(kk);
  }
#endif
  int nt = torsN[k];
  if (nt > 0) {
    int *abcd = malloc(sizeof(int) * 4 * nt);
    double *kp = malloc(sizeof(double) * 6 * nt), *np = malloc(sizeof(double) * 6 * nt);
    double *dp = malloc(sizeof(double) * 6 * nt);
    for (int i = 0; i < nt; i++) {
      abcd[4 * i] = tors[k][i].a;
      abcd[4 * i + 1] = tors[k][i].b;
      abcd[4 * i + 2] = tors[k][i].c;
      abcd[4 * i + 3] = tors[k][i].d;
      for (int t = 0; t < 6; t++) {
        kp[6 * i + t] = tors[k][i].kphi[t];
        np[6 * i + t] = tors[k][i].nphi[t];
        dp[6 * i + t] = tors[k][i].delphi[t];
      }
    }
    FE_OR_DIE(fe_set_torsions(b, nt, abcd, kp, np, dp), "setup (torsions)");
    free(abcd); free(kp); free(np); free(dp);
  }
  int ni = imprN[k];
  if (ni > 0) {
    int *abcd = malloc(sizeof(int) * 4 * ni);
    double *kk = malloc(sizeof(double) * ni), *eq = malloc(sizeof(double) * ni);
    for (int i = 0; i < ni; i++) {
      abcd[4 * i] = impr[k][i].a;
      abcd[4 * i + 1] = impr[k][i].b;
      abcd[4 * i + 2] = impr[k][i].c;
      abcd[4 * i + 3] = impr[k][i].d;
      kk[i] = impr[k][i].kimpr;
      eq[i] = impr[k][i].angeq;
    }
    FE_OR_DIE(fe_set_impropers(b, ni, abcd, kk, eq), "setup (impropers)");
    free(abcd); free(kk); free(eq);
  }
}

/* ctorsion.c:172-175: each torsion's angle into phi / psi / theta by its tag */
static void put_torsion_angles(fe_box *b, int k) {
  int nt = torsN[k], tagged = 0;
  for (int i = 0; i < nt && !tagged; i++)
    tagged = tors[k][i].phitag == 1 || tors[k][i].psitag == 1 || tors[k][i].thetag == 1;
  if (!tagged) return;
  double *tau = malloc(sizeof(double) * nt);
  FE_OR_DIE(fe_get_torsion_angles(b, tau), "torsion angles");
  for (int i = 0; i < nt; i++) {
    if (tors[k][i].phitag == 1) tors[k][i].phi = tau[i];
    else if (tors[k][i].psitag == 1) tors[k][i].psi = tau[i];
    else if (tors[k][i].thetag == 1) tors[k][i].theta = tau[i];
  }
  free(tau);
}

/* Builds the engine's box k from the reference's globals (sim, box[k],
 * pott[k], atom[k], ljset, bond[k], bend[k], xint[k], nhc[k]). */
static fe_box *fe_of(int k) {
  if (g_fe[k]) return g_fe[k];
  int n = box[k].boxns;
  double *q = malloc(sizeof(double) * n), *mass = malloc(sizeof(double) * n);
  int *type = malloc(sizeof(int) * n);
  for (int i = 0; i < n; i++) {
    q[i] = pott[k][i].qq;
    mass[i] = pott[k][i].mas;
    type[i] = atom[k][i].atomid;
  }
  int nt = NUM_ATOM;
  double *eps = malloc(sizeof(double) * nt * nt), *sig = malloc(sizeof(double) * nt * nt);
  for (int a = 0; a < nt; a++)
    for (int b = 0; b < nt; b++) {
      eps[a * nt + b] = ljset[a][b].eps;
      sig[a * nt + b] = ljset[a][b].sig;
    }
  int nb = bondN[k], na = bendN[k], nx = xintN[k];
  int *bab = malloc(sizeof(int) * 2 * (nb + 1)), *aabc = malloc(sizeof(int) * 3 * (na + 1));
  double *breq = malloc(sizeof(double) * (nb + 1)), *bk = malloc(sizeof(double) * (nb + 1));
  double *at0 = malloc(sizeof(double) * (na + 1)), *ak = malloc(sizeof(double) * (na + 1));
  int *xab = malloc(sizeof(int) * 2 * (nx + 1)), *xfl = malloc(sizeof(int) * (nx + 1));
  for (int i = 0; i < nb; i++) {
    bab[2 * i] = bond[k][i].a;
    bab[2 * i + 1] = bond[k][i].b;
    breq[i] = bond[k][i].req;
    bk[i] = bond[k][i].krbond;
  }
  for (int i = 0; i < na; i++) {
    aabc[3 * i] = bend[k][i].a;
    aabc[3 * i + 1] = bend[k][i].b;
    aabc[3 * i + 2] = bend[k][i].c;
    at0[i] = bend[k][i].angeq;
    ak[i] = bend[k][i].krbend;
  }
  for (int i = 0; i < nx; i++) {
    xab[2 * i] = xint[k][i].a;
    xab[2 * i + 1] = xint[k][i].b;
    xfl[i] = xint[k][i].xflag;
  }
  fe_box_params p;
  memset(&p, 0, sizeof p);
  p.n = n;
  p.ntypes = nt;
  p.L[0] = box[k].lx;
  p.L[1] = box[k].ly;
  p.L[2] = box[k].lz;
  p.rc = sim.rc;
  p.rclist = sim.rclist;
  p.rclist_ew = sim.rclist_ew;
  p.kappa = sim.kappa[k];
  p.epsRF = sim.epsRF[k];
  p.dt = sim.dt;
  p.T = sim.T[k];
#ifdef FE_DROPIN_MD
  p.grid[0] = sim.grid[0];
  p.grid[1] = sim.grid[1];
  p.grid[2] = sim.grid[2];
  p.order = sim.order;
  const char *prec = getenv("FE_PRECISION");
  p.precision = (prec && strcmp(prec, "mixed") == 0) ? FE_PREC_MIXED : FE_PREC_FP64;
#else
  /* classic Ewald: the box's SPME arrays are not used; keep them small */
  p.grid[0] = p.grid[1] = p.grid[2] = 8;
  p.order = 4;
  p.precision = FE_PREC_FP64;
#endif
  p.max_neighbors = max_num_neighbors;
  p.device = 0;
  p.q = q;
  p.mass = mass;
  p.type = type;
  p.lj_eps = eps;
  p.lj_sig = sig;
  p.nbond = nb;
  p.bond_ab = bab;
  p.bond_req = breq;
  p.bond_k = bk;
  p.nbend = na;
  p.bend_abc = aabc;
  p.bend_theta0 = at0;
  p.bend_k = ak;
  p.nexcl = nx;
  p.excl_ab = xab;
  p.excl_flag = xfl;
  p.nhc_M = nhc[k].M;
  p.nhc_Q = nhc[k].Q;
  p.nfree = box[k].nfree;
  FE_OR_DIE(fe_box_create(&g_fe[k], &p), "setup");
  free(q); free(mass); free(type); free(eps); free(sig); free(bab); free(aabc); free(breq);
  free(bk); free(at0); free(ak); free(xab); free(xfl);
  if (nhc[k].zeta) FE_OR_DIE(fe_set_nhc_state(g_fe[k], &nhc[k].zeta[0].r), "setup");
  set_ext_bonded(g_fe[k], k);
#ifdef BGO
  /* the build's pair form, cnonbond_nblist.c:294-307 */
  FE_OR_DIE(fe_box_set_lj_form(g_fe[k], 2), "setup");
#endif
  return g_fe[k];
}

/* drift.c:21 (velocities only, as the original) */
void drift(int ibox) {
  fe_box *b = fe_of(ibox);
  FE_OR_DIE(fe_set_velocities(b, &vv[ibox][0].x, &uu[ibox][0].x), "drift");
  FE_OR_DIE(fe_drift(b), "drift");
  FE_OR_DIE(fe_get_velocities(b, &vv[ibox][0].x, NULL), "drift");
}

#ifdef FE_DROPIN_MD
/* ------------------------------------------------------------------------ */
/* MD form                                                                  */

/* device copy equal to the host's (used under FE_DROPIN_TRUST=1) */
static struct {
  int pos, nopbc, vel, ff;
} g_ok[NBOXES];

static int trust(void) {
  static int t = -1;
  if (t < 0) t = env_on("FE_DROPIN_TRUST");
  return t;
}

static void put_atoms(fe_box *b, int k, int nopbc) {
  if (!trust() || !g_ok[k].pos)
    FE_OR_DIE(fe_set_positions(b, atom[k], sizeof(struct atoms), offsetof(struct atoms, x), 0),
              "upload");
  g_ok[k].pos = 1;
  if (nopbc && (!trust() || !g_ok[k].nopbc)) {
    FE_OR_DIE(fe_set_positions_nopbc(b, atnopbc[k], sizeof(struct atoms),
                                     offsetof(struct atoms, x)), "upload");
    g_ok[k].nopbc = 1;
  }
}

static void put_vel(fe_box *b, int k) {
  if (!trust() || !g_ok[k].vel)
    FE_OR_DIE(fe_set_velocities(b, &vv[k][0].x, &uu[k][0].x), "upload");
  g_ok[k].vel = 1;
}

static void put_ff(fe_box *b, int k) {
  if (!trust() || !g_ok[k].ff) FE_OR_DIE(fe_set_forces(b, &ff[k][0].x), "upload");
  g_ok[k].ff = 1;
}

static void get_atoms(fe_box *b, int k, int nopbc) {
  FE_OR_DIE(fe_get_positions(b, atom[k], sizeof(struct atoms), offsetof(struct atoms, x)),
            "download");
  g_ok[k].pos = 1;
  if (nopbc) {
    FE_OR_DIE(fe_get_positions_nopbc(b, atnopbc[k], sizeof(struct atoms),
                                     offsetof(struct atoms, x)), "download");
    g_ok[k].nopbc = 1;
  }
}

/* forces.c:204-219 */
static void put_energies(int k, const double *e) {
  en[k].bond = e[FE_EN_BOND];
  en[k].bend = e[FE_EN_BEND];
#ifndef NEUTRAL
  en[k].urey = e[FE_EN_UREY];
#endif
  en[k].tors = e[FE_EN_TORS];
  en[k].impr = e[FE_EN_IMPR];
  put_torsion_angles(g_fe[k], k);
  en[k].nbond = e[FE_EN_NBOND];
  en[k].nbonds = e[FE_EN_NBONDS];
  en[k].coulomb = e[FE_EN_COULOMB];
  en[k].tewald = e[FE_EN_TEWALD];
  en[k].rewald = e[FE_EN_REWALD];
  en[k].rewalds = e[FE_EN_REWALDS];
  en[k].kewald = e[FE_EN_KEWALD];
  en[k].sewald = e[FE_EN_SEWALD];
  en[k].iewald = e[FE_EN_IEWALD];
}

/* The device list as the host's nlist[k] / nlist_ew[k] rows (allocate.c:
 * 312-360 layout, ascending b, xflags); the engine lists dr2 < min(rclist^2,
 * rclist_ew^2), which is each list when the two radii are equal. */
static void fill_host_lists(fe_box *b, int k) {
  int n = box[k].boxns;
  int64_t tot = 0;
  int *cnt = malloc(sizeof(int) * n);
  FE_OR_DIE(fe_nblist_download(b, cnt, NULL, NULL, 0, &tot), "nblist");
  int *idx = malloc(sizeof(int) * (tot + 1)), *flg = malloc(sizeof(int) * (tot + 1));
  FE_OR_DIE(fe_nblist_download(b, cnt, idx, flg, tot + 1, &tot), "nblist");
  int64_t off = 0;
  for (int a = 0; a < n; a++) {
    if (cnt[a] > max_num_neighbors) fe_die(FE_ERR_OVERFLOW, "nblist (host rows)");
    nlist[k].count[a] = cnt[a];
    nlist_ew[k].count[a] = cnt[a];
    for (int j = 0; j < cnt[a]; j++) {
      nlist[k].list[a][j] = nlist_ew[k].list[a][j] = idx[off + j];
      nlist[k].xflag[a][j] = nlist_ew[k].xflag[a][j] = flg[off + j];
    }
    off += cnt[a];
  }
  free(cnt);
  free(idx);
  free(flg);
}

/* nblist.c:32 (under DLIST it also takes the snapshot nl_check compares
 * against and clears nl_flag, nblist.c:583-591) */
void nblist(int ibox) {
  fe_box *b = fe_of(ibox);
  put_atoms(b, ibox, 0);
  FE_OR_DIE(fe_nblist(b), "nblist");
  if (env_on("FE_HOST_NLIST")) fill_host_lists(b, ibox);
#ifdef DLIST
  nl_flag[ibox] = 0;
#endif
}

#ifdef DLIST
/* nblist.c:607 */
void nl_check(int lb, int ub, int k) {
  fe_box *b = fe_of(k);
  int f = 0;
  put_atoms(b, k, 0);
  FE_OR_DIE(fe_nl_check(b, lb, ub, &f), "nl_check");
  if (f) nl_flag[k] = 1;
}
#endif

/* forces.c:118 */
void forces(int ibox) {
  fe_box *b = fe_of(ibox);
  double e[FE_EN_COUNT];
  put_atoms(b, ibox, 0);
  FE_OR_DIE(fe_forces(b, e), "forces");
  FE_OR_DIE(fe_get_forces(b, &ff[ibox][0].x), "forces");
  g_ok[ibox].ff = 1;
  put_energies(ibox, e);
}

/* cnonbond_nblist.c:51 (accumulates into ff like the original) */
void cnonbondnl(int ibox, double *energy) {
  fe_box *b = fe_of(ibox);
  put_atoms(b, ibox, 0);
  put_ff(b, ibox);
  FE_OR_DIE(fe_cnonbondnl(b, energy), "cnonbondnl");
  FE_OR_DIE(fe_get_forces(b, &ff[ibox][0].x), "cnonbondnl");
}

/* pme_calc.c:18 (accumulates into ff like the original) */
void pme_calc(int k, double *energy) {
  fe_box *b = fe_of(k);
  put_atoms(b, k, 0);
  put_ff(b, k);
  FE_OR_DIE(fe_pme_calc(b, energy), "pme_calc");
  FE_OR_DIE(fe_get_forces(b, &ff[k][0].x), "pme_calc");
}

/* pme_calc.c:122 (accumulates into ff like the original, from the grid of
 * the last pme_calc) */
void pme_force(int k) {
  fe_box *b = fe_of(k);
  put_ff(b, k);
  FE_OR_DIE(fe_pme_force(b), "pme_force");
  FE_OR_DIE(fe_get_forces(b, &ff[k][0].x), "pme_force");
}

/* pme_qgrid.c:13: fills qgrida (real part, imaginary zero) */
void charge_grid(int k) {
  fe_box *b = fe_of(k);
  int ng = sim.grid[0] * sim.grid[1] * sim.grid[2];
  double *g = malloc(sizeof(double) * ng);
  put_atoms(b, k, 0);
  FE_OR_DIE(fe_charge_grid(b), "charge_grid");
  FE_OR_DIE(fe_get_charge_grid(b, g), "charge_grid");
  for (int i = 0; i < ng; i++) {
    qgrida[i][0] = g[i];
    qgrida[i][1] = 0.0;
  }
  free(g);
}

/* pme_setup.c:59: the engine sets up SPME (B-spline moduli, grids, FFT
 * plans) when it creates the box */
void pme_init(int k) { (void)fe_of(k); }

/* pme_setup.c:75: frees every box of the engine */
void pme_clean(void) {
  for (int k = 0; k < NBOXES; k++)
    if (g_fe[k]) {
      fe_box_destroy(g_fe[k]);
      g_fe[k] = NULL;
      memset(&g_ok[k], 0, sizeof g_ok[k]);
    }
}

/* pme_spline.c:10 (B-spline weights and derivatives of order sim.order) */
void fillspline(double w, double *array, double *darray) {
  FE_OR_DIE(fe_bspline(sim.order, w, array, darray), "fillspline");
}

/* integrate_vverlet.c:36 (pbc_all and forces inside, as the original) */
void integrate_vverlet(int ibox, double vscal) {
  fe_box *b = fe_of(ibox);
  double e[FE_EN_COUNT];
  put_atoms(b, ibox, 1);
  put_vel(b, ibox);
  put_ff(b, ibox);
  FE_OR_DIE(fe_integrate_vverlet(b, vscal, e), "integrate_vverlet");
  get_atoms(b, ibox, 1);
  FE_OR_DIE(fe_get_velocities(b, &vv[ibox][0].x, &uu[ibox][0].x), "integrate_vverlet");
  FE_OR_DIE(fe_get_forces(b, &ff[ibox][0].x), "integrate_vverlet");
  put_energies(ibox, e);
}

/* force_short.c:46: bonds, bends, Urey-Bradley into ff and ff_short;
 * en[k].bond / bend / urey */
void force_short(int ibox) {
  fe_box *b = fe_of(ibox);
  double e[FE_EN_COUNT];
  put_atoms(b, ibox, 0);
  FE_OR_DIE(fe_force_short(b, e), "force_short");
  FE_OR_DIE(fe_get_forces(b, &ff[ibox][0].x), "force_short");
  FE_OR_DIE(fe_get_forces_mts(b, &ff_short[ibox][0].x, NULL), "force_short");
  g_ok[ibox].ff = 1;
  en[ibox].bond = e[FE_EN_BOND];
  en[ibox].bend = e[FE_EN_BEND];
#ifndef NEUTRAL
  en[ibox].urey = e[FE_EN_UREY];
#endif
}

/* force_long.c:46: torsions, impropers and cnonbondnl into ff and ff_long;
 * the other en[k] terms as force_long.c:94-116 sets them */
void force_long(int ibox) {
  fe_box *b = fe_of(ibox);
  double e[FE_EN_COUNT];
  put_atoms(b, ibox, 0);
  FE_OR_DIE(fe_force_long(b, e), "force_long");
  FE_OR_DIE(fe_get_forces(b, &ff[ibox][0].x), "force_long");
  FE_OR_DIE(fe_get_forces_mts(b, NULL, &ff_long[ibox][0].x), "force_long");
  g_ok[ibox].ff = 1;
  double bond = en[ibox].bond, bend = en[ibox].bend;
#ifndef NEUTRAL
  double ur = en[ibox].urey;
#endif
  put_energies(ibox, e);
  en[ibox].bond = bond;
  en[ibox].bend = bend;
#ifndef NEUTRAL
  en[ibox].urey = ur;
#endif
}

/* integrate_mts.c:37: one RESPA long step of sim.nsteps short steps
 * (dtlong = dt * nsteps, init.c:314); reads atom, atnopbc, vv, ff_short and
 * ff_long, writes them back with uu, ff and the energies of both classes */
void integrate_mts(int ibox, double vscal) {
  fe_box *b = fe_of(ibox);
  double e[FE_EN_COUNT];
  put_atoms(b, ibox, 1);
  put_vel(b, ibox);
  FE_OR_DIE(fe_set_forces_mts(b, &ff_short[ibox][0].x, &ff_long[ibox][0].x), "integrate_mts");
  FE_OR_DIE(fe_integrate_mts(b, vscal, sim.nsteps, e), "integrate_mts");
  get_atoms(b, ibox, 1);
  FE_OR_DIE(fe_get_velocities(b, &vv[ibox][0].x, &uu[ibox][0].x), "integrate_mts");
  FE_OR_DIE(fe_get_forces(b, &ff[ibox][0].x), "integrate_mts");
  FE_OR_DIE(fe_get_forces_mts(b, &ff_short[ibox][0].x, &ff_long[ibox][0].x), "integrate_mts");
  g_ok[ibox].ff = 1;
  put_energies(ibox, e);
}

/* integrate_mts_nhc.c:37 (nvt_md.c:552): RESPA with the chain of
 * integrate_nhc placed by sim.xRESPA[k]; nhc[k].zeta goes both ways */
void integrate_mts_nhc(int ibox, double vscal) {
  fe_box *b = fe_of(ibox);
  double e[FE_EN_COUNT];
  (void)vscal;  /* integrate_mts_nhc.c does not apply it */
  put_atoms(b, ibox, 1);
  put_vel(b, ibox);
  FE_OR_DIE(fe_set_forces_mts(b, &ff_short[ibox][0].x, &ff_long[ibox][0].x), "integrate_mts_nhc");
  FE_OR_DIE(fe_set_nhc_state(b, &nhc[ibox].zeta[0].r), "integrate_mts_nhc");
  FE_OR_DIE(fe_integrate_mts_nhc(b, sim.nsteps, sim.xRESPA[ibox], e), "integrate_mts_nhc");
  get_atoms(b, ibox, 1);
  FE_OR_DIE(fe_get_velocities(b, &vv[ibox][0].x, &uu[ibox][0].x), "integrate_mts_nhc");
  FE_OR_DIE(fe_get_forces(b, &ff[ibox][0].x), "integrate_mts_nhc");
  FE_OR_DIE(fe_get_forces_mts(b, &ff_short[ibox][0].x, &ff_long[ibox][0].x), "integrate_mts_nhc");
  FE_OR_DIE(fe_get_nhc_state(b, &nhc[ibox].zeta[0].r), "integrate_mts_nhc");
  g_ok[ibox].ff = 1;
  put_energies(ibox, e);
}

/* kinet.c:18 */
void kinet(int ibox) {
  fe_box *b = fe_of(ibox);
  double ken[6], kin;
  put_vel(b, ibox);
  FE_OR_DIE(fe_kinet(b, ken, &kin), "kinet");
  for (int i = 0; i < 6; i++) en[ibox].ken[i] = ken[i];
  en[ibox].kinet = kin;
}

/* integrate_nhc.c:40 (its kinet() call leaves en[k].ken/kinet of the
 * velocities before scaling, as here) */
void integrate_nhc(double time_step, int ibox) {
  fe_box *b = fe_of(ibox);
  kinet(ibox);
  FE_OR_DIE(fe_set_nhc_state(b, &nhc[ibox].zeta[0].r), "integrate_nhc");
  FE_OR_DIE(fe_integrate_nhc(b, time_step), "integrate_nhc");
  FE_OR_DIE(fe_get_velocities(b, &vv[ibox][0].x, &uu[ibox][0].x), "integrate_nhc");
  FE_OR_DIE(fe_get_nhc_state(b, &nhc[ibox].zeta[0].r), "integrate_nhc");
}

/* pbc_all.c:23 */
void pbc_all(int ibox) {
  fe_box *b = fe_of(ibox);
  put_atoms(b, ibox, 0);
  FE_OR_DIE(fe_pbc_all(b), "pbc_all");
  get_atoms(b, ibox, 0);
}

/* isokin.c:22: the reference's velocity scaling on the host; the device
 * copy of the velocities is refreshed at the next call that reads them */
void isokin(int ibox) {
  int k = ibox;
  double scale = sqrt(sim.T[k] / box[k].temp);
  for (int i = 0; i < box[k].boxns; i++) {
    vv[k][i].x *= scale;
    vv[k][i].y *= scale;
    vv[k][i].z *= scale;
    uu[k][i].x *= scale;
    uu[k][i].y *= scale;
    uu[k][i].z *= scale;
  }
  g_ok[k].vel = 0;
}

/* swap_box.c:5: the reference's acceptance test (same draw of ran2) and the
 * same exchange of the host arrays and en[]; on the device the two boxes'
 * engine states are exchanged (positions, forces, lists move with their
 * configurations) and each keeps its own temperature, so only the rescaled
 * velocities are uploaded.  Boxes of different sizes or shapes fall back to
 * uploading everything. */
double ran2(void);
int swap_box(int ibox) {
  int k = ibox;
  double delta_beta = 1.0 / sim.kT[k] - 1.0 / sim.kT[k + 1];
  double delta_energy = en[k].potens - en[k + 1].potens;
  double accep_crit = exp(delta_beta * delta_energy);
  if (!(accep_crit > ran2())) return 0;
  int n = box[k].boxns;
  for (int i = 0; i < n; i++) {
    struct atoms a = atom[k][i], an = atnopbc[k][i];
    atom[k][i] = atom[k + 1][i];
    atnopbc[k][i] = atnopbc[k + 1][i];
    atom[k + 1][i] = a;
    atnopbc[k + 1][i] = an;
    struct veloc f = ff[k][i], v = vv[k][i];
    ff[k][i] = ff[k + 1][i];
    ff[k + 1][i] = f;
    vv[k][i] = vv[k + 1][i];
    vv[k + 1][i] = v;
  }
  double v_scale_1 = sqrt(sim.T[k] / sim.T[k + 1]);
  for (int i = 0; i < n; i++) {
    vv[k][i].x *= v_scale_1;
    vv[k][i].y *= v_scale_1;
    vv[k][i].z *= v_scale_1;
    vv[k + 1][i].x /= v_scale_1;
    vv[k + 1][i].y /= v_scale_1;
    vv[k + 1][i].z /= v_scale_1;
    uu[k][i] = vv[k][i];
    uu[k + 1][i] = vv[k + 1][i];
  }
  struct energy e = en[k];
  en[k] = en[k + 1];
  en[k + 1] = e;
  if (g_fe[k] && g_fe[k + 1] && box[k].boxns == box[k + 1].boxns && box[k].lx == box[k + 1].lx &&
      box[k].ly == box[k + 1].ly && box[k].lz == box[k + 1].lz) {
    fe_box *t = g_fe[k];
    g_fe[k] = g_fe[k + 1];
    g_fe[k + 1] = t;
    FE_OR_DIE(fe_box_set_temperature(g_fe[k], sim.T[k]), "swap_box");
    FE_OR_DIE(fe_box_set_temperature(g_fe[k + 1], sim.T[k + 1]), "swap_box");
    FE_OR_DIE(fe_set_velocities(g_fe[k], &vv[k][0].x, &uu[k][0].x), "swap_box");
    FE_OR_DIE(fe_set_velocities(g_fe[k + 1], &vv[k + 1][0].x, &uu[k + 1][0].x), "swap_box");
    g_ok[k].vel = g_ok[k + 1].vel = 1;
  } else {
    memset(&g_ok[k], 0, sizeof g_ok[k]);
    memset(&g_ok[k + 1], 0, sizeof g_ok[k + 1]);
  }
  nblist(k); /* swap_box.c: the lists of both boxes are rebuilt */
  nblist(k + 1);
  return 1;
}
#endif /* FE_DROPIN_MD */

#ifdef FE_DROPIN_MC
/* ------------------------------------------------------------------------ */
/* MC form (classic Ewald)                                                  */

double ebond_mc(int);
double ebend_mc(int);
double etors_mc(int);
double eimpr_mc(int);
#ifndef NEUTRAL
double eurey_mc(int);
#endif

/* per box: the positions the device holds, and the last trial move */
static struct {
  double *dev;      /* 3 n */
  int lb, ub;       /* pending trial [lb, ub), ub == 0: none */
  double trial[64][3];
  double t_old[6];  /* fe_mc_site_energy of the last forces_mc(.., 0, ..) */
} g_mc[NBOXES];

static void upload_all(fe_box *b, int k) {
  int n = box[k].boxns;
  FE_OR_DIE(fe_set_positions(b, atom[k], sizeof(struct atoms), offsetof(struct atoms, x), 1),
            "upload");
  for (int i = 0; i < n; i++) {
    g_mc[k].dev[3 * i] = atom[k][i].x;
    g_mc[k].dev[3 * i + 1] = atom[k][i].y;
    g_mc[k].dev[3 * i + 2] = atom[k][i].z;
  }
  if (sim.kmax[k][0] != sim.kmax[k][1] || sim.kmax[k][0] != sim.kmax[k][2]) {
    fprintf(stdout, "GPU engine: the MC path needs the same kmax along x, y and z\n");
    exit(1);
  }
  FE_OR_DIE(fe_mc_setup(b, sim.kmax[k][0], sim.max_k_square[k], sim.rc_ew), "mc setup");
  g_mc[k].ub = 0;
}

/* brings the device to the host's configuration (see the header) */
static fe_box *mc_sync(int k) {
  fe_box *b = fe_of(k);
  int n = box[k].boxns;
  if (!g_mc[k].dev) {
    g_mc[k].dev = malloc(sizeof(double) * 3 * n);
    upload_all(b, k);
    return b;
  }
  if (g_mc[k].ub > 0) {
    int same = 1;
    for (int i = g_mc[k].lb; i < g_mc[k].ub && same; i++) {
      const double *t = g_mc[k].trial[i - g_mc[k].lb];
      same = atom[k][i].x == t[0] && atom[k][i].y == t[1] && atom[k][i].z == t[2];
    }
    if (same) { /* the move was kept: commit it on the device */
      FE_OR_DIE(fe_mc_accept(b), "mc accept");
      for (int i = g_mc[k].lb; i < g_mc[k].ub; i++)
        memcpy(&g_mc[k].dev[3 * i], g_mc[k].trial[i - g_mc[k].lb], sizeof(double) * 3);
    }
    g_mc[k].ub = 0;
  }
  for (int i = 0; i < n; i++)
    if (atom[k][i].x != g_mc[k].dev[3 * i] || atom[k][i].y != g_mc[k].dev[3 * i + 1] ||
        atom[k][i].z != g_mc[k].dev[3 * i + 2]) {
      upload_all(b, k);
      break;
    }
  return b;
}

/* enbnd_mc energy[8] (enbnd_mc.c:459-467) from the six terms
 * {reciprocal, LJ, LJ shift, real, real shift, intra} */
static void energy8(int k, const double *t, double *e) {
  double sew = en[k].sewald;
  e[0] = t[1] + t[3] - t[5] + (t[0] - sew);
  e[1] = e[0] - t[2];
  e[2] = t[3] + (t[0] - sew) - t[5];
  e[3] = t[4];
  e[4] = t[0];
  e[5] = sew;
  e[6] = t[5];
  e[7] = t[3];
}

/* enbnd_mc.c:26: energies of the pairs touching [lb, ub) plus the whole
 * reciprocal energy (the reference's ewald_rspace_mc also counts the other
 * pairs of rows below ub; they cancel in every difference forces_mc takes) */
void enbnd_mc(int lb, int ub, int ibox, double *energy) {
  fe_box *b = mc_sync(ibox);
  double t[6];
  FE_OR_DIE(fe_mc_site_energy(b, lb, ub, t), "enbnd_mc");
  energy8(ibox, t, energy);
}

/* ewald_mc.c:42 */
void ewald_kspace_mc(int ibox, double *enkewald) {
  fe_box *b = mc_sync(ibox);
  FE_OR_DIE(fe_mc_kspace_energy(b, &enkewald[0]), "ewald_kspace_mc");
  enkewald[1] = en[ibox].sewald;
  enkewald[2] = enkewald[0] - enkewald[1];
}

/* ewald_mc.c:328 (the correct minimum image; see the header of k_mc.cu) */
void ewald_rspace_mc(int lb, int ub, int ibox, double *energy) {
  fe_box *b = mc_sync(ibox);
  double t[6];
  FE_OR_DIE(fe_mc_site_energy(b, lb, ub, t), "ewald_rspace_mc");
  energy[0] = t[3];
  energy[1] = t[3] - t[4];
  energy[2] = t[5];
}

/* nblist_pivot.c:26: the engine finds each move's partners itself, so the
 * list rows need no update for it; host rows keep their last build */
void nblist_pivot(int ibox, int ub) {
  (void)ibox;
  (void)ub;
}

static void set_mc_energies(int k, int tag, const double *t) {
  double e[8];
  energy8(k, t, e);
  double bond = ebond_mc(k), bend = ebend_mc(k), tors = etors_mc(k), impr = eimpr_mc(k);
#ifndef NEUTRAL
  double urey = eurey_mc(k);
#endif
#define SETMC(f, v) (tag ? (enmc[k].n_##f = (v)) : (enmc[k].o_##f = (v)))
  SETMC(bond, bond);
  SETMC(bend, bend);
  SETMC(tors, tors);
  SETMC(impr, impr);
#ifndef NEUTRAL
  SETMC(urey, urey);
#endif
  SETMC(nbond, e[0]);
  SETMC(nbonds, e[1]);
  SETMC(coulomb, e[2]);
  SETMC(tewald, e[2]);
  SETMC(rewald, e[7]);
  SETMC(rewalds, e[3]);
  SETMC(kewald, e[4]);
  SETMC(sewald, e[5]);
  SETMC(iewald, e[6]);
  double poten = bond + bend + tors + e[0] + impr, potens = bond + bend + tors + e[1] + impr;
#ifndef NEUTRAL
  poten += urey;
  potens += urey;
#endif
  SETMC(poten, poten);
  SETMC(potens, potens);
#undef SETMC
}

/* forces_mc.c:90 */
void forces_mc(int lb, int ub, int tag, int ibox) {
  int k = ibox;
  if (ub - lb > 64 || ub <= lb) {
    fprintf(stdout, "GPU engine: forces_mc moves at most 64 sites (got %d)\n", ub - lb);
    exit(1);
  }
  if (tag == 0) {
    fe_box *b = mc_sync(k);
    FE_OR_DIE(fe_mc_site_energy(b, lb, ub, g_mc[k].t_old), "forces_mc");
    set_mc_energies(k, 0, g_mc[k].t_old);
    return;
  }
  fe_box *b = fe_of(k);
  double d[6], t[6];
  for (int i = lb; i < ub; i++) {
    g_mc[k].trial[i - lb][0] = atom[k][i].x;
    g_mc[k].trial[i - lb][1] = atom[k][i].y;
    g_mc[k].trial[i - lb][2] = atom[k][i].z;
  }
  FE_OR_DIE(fe_mc_delta_terms(b, lb, ub, &g_mc[k].trial[0][0], d), "forces_mc");
  g_mc[k].lb = lb;
  g_mc[k].ub = ub;
  for (int q = 0; q < 6; q++) t[q] = g_mc[k].t_old[q] + d[q];
  set_mc_energies(k, 1, t);
  /* forces_mc.c:511-534 */
  en[k].bond += enmc[k].n_bond - enmc[k].o_bond;
  en[k].bend += enmc[k].n_bend - enmc[k].o_bend;
  en[k].tors += enmc[k].n_tors - enmc[k].o_tors;
  en[k].impr += enmc[k].n_impr - enmc[k].o_impr;
  en[k].nbond += enmc[k].n_nbond - enmc[k].o_nbond;
  en[k].nbonds += enmc[k].n_nbonds - enmc[k].o_nbonds;
#ifndef NEUTRAL
  en[k].urey += enmc[k].n_urey - enmc[k].o_urey;
#endif
  en[k].coulomb += enmc[k].n_coulomb - enmc[k].o_coulomb;
  en[k].tewald += enmc[k].n_tewald - enmc[k].o_tewald;
  en[k].rewald += enmc[k].n_rewald - enmc[k].o_rewald;
  en[k].rewalds += enmc[k].n_rewalds - enmc[k].o_rewalds;
  en[k].kewald += enmc[k].n_kewald - enmc[k].o_kewald;
  en[k].sewald += enmc[k].n_sewald - enmc[k].o_sewald;
  en[k].iewald += enmc[k].n_iewald - enmc[k].o_iewald;
}
#endif /* FE_DROPIN_MC */
