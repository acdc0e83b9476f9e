/*
 * fe_dropin.c -- the reference's own hot-path symbols on top of libfe.so.
 *
 * Compiled INSIDE the reference's build (against its defines.h, with its
 * feature flags -DNLIST -DEWALD -DSPME -DSTYPE), in place of nblist.c,
 * cnonbond_nblist.c, pme_qgrid.c, pme_calc.c, integrate_vverlet.c,
 * integrate_nhc.c, pbc_all.c, kinet.c and forces.c.  Each symbol keeps the
 * prototype its callers declare and the semantics of the routine it replaces:
 * it uploads the host state that routine reads, runs the engine, and writes
 * back the host state that routine writes, so host code between calls
 * (output, MC restore, swaps, checkpoints) is unaffected.
 *
 * Errors print the engine's message and exit() with the reference's codes
 * (5: neighbour list over capacity, nblist.c:185-197; 20: non-neutral box,
 * ewald.c:185-194; 1 otherwise).  FE_PRECISION=mixed in the environment
 * selects the mixed-precision engine.
 */
#include <stddef.h>
#include <stdint.h>

#include "defines.h"
#include "fe.h"

#if !defined(NLIST) || !defined(EWALD) || !defined(SPME) || !defined(STYPE)
#error "fe_dropin.c replaces the NLIST + EWALD + SPME + STYPE build of the hot path"
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

/* Builds the engine's box k from the reference's globals (sim, box[k],
 * pott[k], atom[k], ljset, bond[k], bend[k], xint[k], nhc[k]). */
static fe_box *fe_of(int k) {
  if (g_fe[k]) return g_fe[k];
  int n = box[k].boxns;
  if (torsN[k] > 0 || imprN[k] > 0
#ifndef NEUTRAL
      || ureyN[k] > 0
#endif
  ) {
    fprintf(stdout, "GPU engine: torsions, impropers and Urey-Bradley terms are not on the "
                    "device path; use the CPU build for this system\n");
    exit(1);
  }
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
  p.grid[0] = sim.grid[0];
  p.grid[1] = sim.grid[1];
  p.grid[2] = sim.grid[2];
  p.order = sim.order;
  const char *prec = getenv("FE_PRECISION");
  p.precision = (prec && strcmp(prec, "mixed") == 0) ? FE_PREC_MIXED : FE_PREC_FP64;
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
  return g_fe[k];
}

static void put_atoms(fe_box *b, int k, int nopbc) {
  FE_OR_DIE(fe_set_positions(b, atom[k], sizeof(struct atoms), offsetof(struct atoms, x), 0),
            "upload");
  if (nopbc)
    FE_OR_DIE(fe_set_positions_nopbc(b, atnopbc[k], sizeof(struct atoms),
                                     offsetof(struct atoms, x)), "upload");
}

static void get_atoms(fe_box *b, int k, int nopbc) {
  FE_OR_DIE(fe_get_positions(b, atom[k], sizeof(struct atoms), offsetof(struct atoms, x)),
            "download");
  if (nopbc)
    FE_OR_DIE(fe_get_positions_nopbc(b, atnopbc[k], sizeof(struct atoms),
                                     offsetof(struct atoms, x)), "download");
}

/* forces.c:204-219 */
static void put_energies(int k, const double *e) {
  en[k].bond = e[FE_EN_BOND];
  en[k].bend = e[FE_EN_BEND];
#ifndef NEUTRAL
  en[k].urey = 0.0;
#endif
  en[k].tors = 0.0;
  en[k].impr = 0.0;
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

/* nblist.c:32 (under DLIST it also takes the snapshot nl_check compares
 * against and clears nl_flag, nblist.c:583-591) */
void nblist(int ibox) {
  fe_box *b = fe_of(ibox);
  put_atoms(b, ibox, 0);
  FE_OR_DIE(fe_nblist(b), "nblist");
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
  put_energies(ibox, e);
}

/* cnonbond_nblist.c:51 (accumulates into ff like the original) */
void cnonbondnl(int ibox, double *energy) {
  fe_box *b = fe_of(ibox);
  put_atoms(b, ibox, 0);
  FE_OR_DIE(fe_set_forces(b, &ff[ibox][0].x), "cnonbondnl");
  FE_OR_DIE(fe_cnonbondnl(b, energy), "cnonbondnl");
  FE_OR_DIE(fe_get_forces(b, &ff[ibox][0].x), "cnonbondnl");
}

/* pme_calc.c:18 (accumulates into ff like the original) */
void pme_calc(int k, double *energy) {
  fe_box *b = fe_of(k);
  put_atoms(b, k, 0);
  FE_OR_DIE(fe_set_forces(b, &ff[k][0].x), "pme_calc");
  FE_OR_DIE(fe_pme_calc(b, energy), "pme_calc");
  FE_OR_DIE(fe_get_forces(b, &ff[k][0].x), "pme_calc");
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

/* integrate_vverlet.c:36 (pbc_all and forces inside, as the original) */
void integrate_vverlet(int ibox, double vscal) {
  fe_box *b = fe_of(ibox);
  double e[FE_EN_COUNT];
  put_atoms(b, ibox, 1);
  FE_OR_DIE(fe_set_velocities(b, &vv[ibox][0].x, &uu[ibox][0].x), "integrate_vverlet");
  FE_OR_DIE(fe_set_forces(b, &ff[ibox][0].x), "integrate_vverlet");
  FE_OR_DIE(fe_integrate_vverlet(b, vscal, e), "integrate_vverlet");
  get_atoms(b, ibox, 1);
  FE_OR_DIE(fe_get_velocities(b, &vv[ibox][0].x, &uu[ibox][0].x), "integrate_vverlet");
  FE_OR_DIE(fe_get_forces(b, &ff[ibox][0].x), "integrate_vverlet");
  put_energies(ibox, e);
}

/* kinet.c:18 */
void kinet(int ibox) {
  fe_box *b = fe_of(ibox);
  double ken[6], kin;
  FE_OR_DIE(fe_set_velocities(b, &vv[ibox][0].x, &uu[ibox][0].x), "kinet");
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
