/*
 * fe_oracle.h -- CPU restatement of the reference's force-engine hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load it, and only as the
 * checker or as the timed CPU baseline -- never as the product path.
 *
 * Every routine restates one reference routine in the same floating-point
 * operation order (each cites file:line), so that, compiled without FMA
 * contraction and without fast-math, it reproduces the reference bit for bit
 * on the same inputs.  Arrays are plain: positions/forces/velocities are
 * interleaved xyz doubles, lists are CSR.
 */
#ifndef FE_ORACLE_H
#define FE_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int n;           /* atoms (box[k].boxns) */
  int ntypes;      /* site types (NUM_ATOM) */
  double L[3];     /* box lengths (box[k].lx/ly/lz) */
  double rc;       /* sim.rc */
  double rclist;   /* sim.rclist */
  double rclist_ew;/* sim.rclist_ew */
  double kappa;    /* sim.kappa[k] */
  double epsRF;    /* sim.epsRF[k] */
  double dt;       /* sim.dt [ps] */
  double T;        /* sim.T[k] [K] */
  int grid[3];     /* sim.grid */
  int order;       /* sim.order */
  /* optional CHARMM LJ switch between r_on and rc (0 = off = reference) */
  double r_switch;
  const double *q;     /* n, charges (pott[k][i].qq) */
  const double *mass;  /* n, amu (pott[k][i].mas) */
  const int *type;     /* n, site type (atom[k][i].atomid) */
  const double *lj_eps;/* ntypes*ntypes mixed eps [kJ/mol] (ljset[ta][tb].eps) */
  const double *lj_sig;/* ntypes*ntypes mixed R_min [A]  (ljset[ta][tb].sig) */
  int nbond;
  const int *bond_ab;      /* 2*nbond */
  const double *bond_req;  /* nbond */
  const double *bond_k;    /* nbond, kJ/mol/A^2, E = k (r-r0)^2 */
  int nbend;
  const int *bend_abc;     /* 3*nbend */
  const double *bend_theta0; /* nbend, rad */
  const double *bend_k;    /* nbend, kJ/mol/rad^2, E = k (th-th0)^2 */
  int nexcl;
  const int *excl_ab;      /* 2*nexcl (xint[k][i].a/b) */
  const int *excl_flag;    /* nexcl (xint[k][i].xflag: 1 bond 2 bend 3 exNB 4 1-4) */
  int lj_form;             /* 0 CHARMM eps[(R/r)^12 - 2(R/r)^6]; 2 the BGO build's
                              eps[13(R/r)^12 - 18(R/r)^10 + 4(R/r)^6] (cnonbond_nblist.c:294-307) */
} or_system;

/* Energy record in the reference's en[k] vocabulary (forces.c:204-219). */
typedef struct {
  double bond, bend;
  double nbond, nbonds;          /* interen[0], interen[1] */
  double coulomb;                /* interen[2] (= tewald) */
  double rewald, rewalds;        /* interen[7], interen[3] */
  double kewald, sewald, iewald; /* interen[4], [5], [6] */
  double tewald;
} or_energy;

/* mixing of per-type CHARMM parameters exactly as setlj.c:181-191 (STYPE):
 * eps_kcal are the (negative) CHARMM eps, rmin_half the R_min/2 values. */
void or_setlj(int ntypes, const double *eps_kcal, const double *rmin_half,
              double *lj_eps, double *lj_sig);

/* nblist.c:91-325 (O(N^2) path, EWALD + STYPE): half list b > a with
 * dr2 < rclist_ew^2 (nlist_ew) and additionally dr2 < rclist^2 (nlist).
 * CSR out: cnt[n], idx/flag[<= cap].  Returns total nlist entries, or -1
 * when cap is exceeded.  Either list may be NULL to skip it. */
int64_t or_nblist(const or_system *s, const double *pos, int *cnt, int *idx,
                  int *flag, int64_t cap, int *cnt_ew, int *idx_ew,
                  int *flag_ew, int64_t cap_ew);

/* cnonbond_nblist.c:51-622 without the trailing pme_calc: accumulates into
 * ff and returns e5 = {enonbond, enonbonds, eewald_real, eewald_reals,
 * eewald_intra}. */
void or_cnonbond_pairs(const or_system *s, const double *pos, const int *cnt,
                       const int *idx, const int *flag, double *ff,
                       double e5[5]);

/* pme_setup.c:59-130: B-spline moduli (arrays of grid+1, 1-based). */
void or_pme_bspline(const or_system *s, double *bx, double *by, double *bz);

/* pme_qgrid.c:13-121: real part of the spread grid (grid0*grid1*grid2). */
void or_charge_grid(const or_system *s, const double *pos, double *grid);

/* pme_calc.c:18-279 (charge_grid, BACKWARD FFT, reciprocal loop, FORWARD FFT,
 * pme_force incl. mean-force removal).  Accumulates into ff;
 * e3 = {E_rec, E_self, E_rec - E_self}. */
void or_pme_calc(const or_system *s, const double *pos, double sewald,
                 double *ff, double e3[3]);

/* ewald.c:172-178 self energy (en[k].sewald). */
double or_ewald_self(const or_system *s);

/* cbond.c:27-180 and cbend.c:24-218 (accumulate into ff, return energy). */
double or_cbond(const or_system *s, const double *pos, double *ff);
double or_cbend(const or_system *s, const double *pos, double *ff);
/* Urey-Bradley 1-3 terms (curey.c:37-106), proper torsions (ctorsion.c:63-246;
 * tau_out, may be NULL, gets each torsion's angle) and improper torsions
 * (cimproper.c:55-221); each adds its forces to ff and returns its energy. */
double or_curey(const or_system *s, const double *pos, int nurey, const int *ab,
                const double *seq, const double *k, double *ff);
double or_ctorsion(const or_system *s, const double *pos, int ntors, const int *abcd,
                   const double *kphi, const double *nphi, const double *delphi, double *ff,
                   double *tau_out);
double or_cimproper(const or_system *s, const double *pos, int nimpr, const int *abcd,
                    const double *kimpr, const double *angeq, double *ff);

/* forces.c:118-446: zero ff, bonded, cnonbondnl (+ pme_calc), energies. */
void or_forces(const or_system *s, const double *pos, const int *cnt,
               const int *idx, const int *flag, double sewald, double *ff,
               or_energy *en);

/* pbc_all.c:23-88 */
void or_pbc_all(const or_system *s, double *pos);

/* kinet.c:18-68: returns en[k].kinet, fills ken[6] if not NULL. */
double or_kinet(const or_system *s, const double *vv, const double *uu,
                double *ken);

/* integrate_vverlet.c:36-103 (calls or_pbc_all and or_forces). */
void or_integrate_vverlet(const or_system *s, double vscal, double *pos,
                          double *pos_nopbc, double *vv, double *uu,
                          double *ff, const int *cnt, const int *idx,
                          const int *flag, double sewald, or_energy *en);

/* integrate_nhc.c:40-161 with Nc = Nys = 1, w[0] = 1 (read_sim.c:544-545).
 * zeta: 3*M doubles {r, v, G} per thermostat; nfree = box[k].nfree. */
void or_integrate_nhc(const or_system *s, double time_step, int M, double Q,
                      double nfree, double *zeta, double *vv, double *uu);

/* Full NVE / NHC trajectory in the reference's step order (nve_md.c:359-418,
 * nvt_md.c:529-531, main.c:475-496).  rec gets 12 doubles per step
 * (0..nsteps) in the order kinet, bond, bend, nbond, nbonds, coulomb, rewald,
 * rewalds, kewald, sewald, iewald, tewald.  Returns 0, or -1 on list
 * overflow. */
int or_run_md(const or_system *s, int nsteps, int nlist_freq, int use_nhc,
              int nhc_M, double nhc_Q, double *pos, double *pos_nopbc,
              double *vv, double *ff, double *zeta, double *rec);
/* or_run_md with tstamp[i] = CLOCK_MONOTONIC seconds at the end of step i
 * (tstamp[0] after the initial list and forces); for timing the CPU path. */
int or_run_md_timed(const or_system *s, int nsteps, int nlist_freq, int use_nhc,
                    int nhc_M, double nhc_Q, double *pos, double *pos_nopbc,
                    double *vv, double *ff, double *zeta, double *rec, double *tstamp);

/* pme_spline.c:10-49 B-spline weights / derivatives, array[0..order] */
void or_fillspline(int order, double w, double *array, double *darray);
/* drift.c:21-66 momentum removal on vv (n x 3) */
void or_drift(const or_system *s, double *vv);

/* ---- classic-Ewald MC energy path (ewald.c:46-118, ewald_mc.c) ---- */

/* number of k-vectors of ewald_setup's enumeration (ewald.c:104-118) */
int or_ewald_nk(int kmax_x, int kmax_y, int kmax_z, int max_k_square);

/* ewald_kspace_mc energy (ewald_mc.c:42-324) with kvec from ewald.c:104-118;
 * returns enkewald[0] (k-space energy, kJ/mol). */
double or_ewald_kspace_energy(const or_system *s, const double *pos, int kmax,
                              int max_k_square);

/* Real-space Ewald + LJ energy of every list pair with a < ub
 * (ewald_mc.c:328-641 / enbnd_mc.c:26-501 restated with the correct minimum
 * image, i.e. what the reference computes for pairs that do not cross the
 * periodic boundary).  e4 = {lj, real, real_shift, intra}. */
void or_mc_pair_energy(const or_system *s, const double *pos, const int *cnt,
                       const int *idx, const int *flag, double rc_ew, int lb,
                       int ub, double e4[4]);

/* Exact Ewald energy change of moving atoms [lb,ub) from pos to pos_new:
 * reciprocal (incremental structure-factor update, same k set as
 * ewald_setup) + real space + LJ over all pairs touching [lb,ub) with
 * minimum image.  Returns dE = E(new) - E(old) in kJ/mol; parts (may be NULL)
 * = {dE_recip, dE_real, dE_lj}. */
double or_mc_delta_energy(const or_system *s, const double *pos,
                          const double *pos_new, int lb, int ub, int kmax,
                          int max_k_square, double rc_ew, double parts[3]);

/* ---- counter-based random numbers and replica exchange ---- */

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11). */
void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* Uniform [0,1) from words 0,1 of the draw at counter (lane, event lo, event
 * hi, tag) under key (seed lo, seed hi): 53 bits. */
double or_uniform(uint64_t seed, uint32_t tag, uint64_t event, uint32_t lane);
/* One exchange attempt (swap_box.c:5-86) on temperature slots: pairs
 * (s, s+1) with s = attempt & 1, 2 + (attempt & 1), ... (repexch.c:273-301);
 * accept when exp((1/kT_s - 1/kT_s+1)(U_box(s) - U_box(s+1))) > u.  Updates
 * slot_box; vmode[b] = 1 (multiply by vfac) / 2 (divide) / 0 for each box.
 * Returns the number of accepted swaps. */
int or_rex_attempt(int R, const double *T_slot, const double *potens_box, int *slot_box,
                   uint64_t attempt, uint64_t seed, int *vmode, double *vfac);

/* ---- Go-model chains (the batched replica-exchange workload) ---- */

typedef struct {
  double eps;        /* kJ/mol */
  double sigma_rep;  /* non-native repulsion sigma [A] */
  double rc_rep;     /* its cutoff [A] (energy shifted to zero there) */
  double k_bond;     /* E = k (r - r_bond)^2 [kJ/mol/A^2] */
  double r_bond;
  double mass;       /* amu */
  double gamma;      /* 1/ps */
  double dt;         /* ps */
  int min_sep;       /* non-bonded pairs need |i - j| >= min_sep */
} or_go_params;

/* Forces (f, 3N, overwritten) and potential energy of one chain whose beads
 * have global indices gbase..gbase+N-1; natives as CSR over global indices. */
double or_go_forces(int N, const double *pos, int gbase, const int *nat_start, const int *nat_j,
                    const double *nat_r0, const or_go_params *p, double *f);
/* nsteps BAOAB Langevin steps at temperature T with the draws of step
 * step0.. (Philox4x32-10, tag "GOL1", Box-Muller); returns the final
 * potential energy. */
double or_go_baoab(int N, double *pos, double *vel, int gbase, const int *nat_start,
                   const int *nat_j, const double *nat_r0, const or_go_params *p, double T,
                   uint64_t seed, uint64_t step0, int nsteps);

/* The reference's own Go model (cgolik.c, GOLIK build, protein sites only,
 * no periodic images): bonds E = eps dr^2 + 100 eps dr^4 (cbb_golik,
 * cgolik.c:25-174), bends E = 10 eps (theta - theta0)^2 (cba_golik,
 * :176-367), torsions E = 0.2 eps (1 + cos 3 tau) (cda_golik, :369-641, GOBT
 * phases zero), natives 4 eps [(s/r)^12 - (s/r)^6] with s = 2^(-1/6) r0
 * shifted at rc, non-natives the same with s = 2^(-1/6) d_rep cut at d_rep
 * and lifted by eps (cnbnd_golik, :644-948); bonded pairs excluded.
 * term: 0 bonds, 1 bends, 2 torsions, 3 pairs (then e2 = {energy[0],
 * energy[1]} of cnbnd_golik: unshifted and shifted).  Forces into f (3N,
 * overwritten); returns the term's energy (shifted for pairs). */
typedef struct {
  double eps;    /* kJ/mol */
  double d_rep;  /* non-native cut [A] */
  double rc;     /* native cutoff [A] */
} or_go_hc_params;
double or_go_hc_term(int N, const double *pos, int gbase, const int *nat_start, const int *nat_j,
                     const double *nat_r0, const or_go_hc_params *p, const double *bond_r0,
                     const double *bend_t0, int term, double *f, double *e2);
/* or_go_baoab with the forces of the reference's Go model (the sum of the
 * four terms above; the potential energy returned is that sum, pairs
 * shifted). */
double or_go_baoab_hc(int N, double *pos, double *vel, int gbase, const int *nat_start,
                      const int *nat_j, const double *nat_r0, const or_go_params *p,
                      const or_go_hc_params *hc, const double *bond_r0, const double *bend_t0,
                      double T, uint64_t seed, uint64_t step0, int nsteps);

#ifdef __cplusplus
}
#endif
#endif
