/*
 * fe.h -- C ABI of the GB300 force engine (libfe.so).
 *
 * One fe_box holds one simulation box of the reference (its `ibox`) resident
 * in GPU memory: positions, velocities, forces, the Verlet list, the SPME
 * grids and plans.  Every entry point below replaces one routine of the
 * reference's hot path (file:line of the routine it replaces is on each);
 * arguments are plain pointers and sizes, arrays on the host side use the
 * reference's own layouts:
 *   - `struct atoms` records (defines.h:307-317): x, y, z doubles at a byte
 *     offset inside a record of `stride` bytes (64 / 16 with gcc LP64);
 *   - `struct veloc` records (defines.h:508-512): 3 doubles, stride 24, which
 *     is also a plain interleaved xyz array;
 *   - energies as the reference's en[k] fields (FE_EN_* indices).
 * Units are the reference's (A, ps, amu, e, kJ/mol).
 *
 * Errors: every call returns FE_OK (0) or an FE_ERR_* code; fe_last_error()
 * gives the message.  Nothing falls back to the CPU: without a usable CUDA
 * device fe_box_create fails with FE_ERR_CUDA.
 *
 * Threading: a box is used by one host thread at a time (the reference is
 * single-threaded and loops boxes sequentially).  Work is issued on the box's
 * stream (fe_box_set_stream); calls that return host data synchronise it.
 */
#ifndef FE_H
#define FE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FE_ABI_VERSION 2  /* 2: en[k] records carry urey, tors, impr */

enum {
  FE_OK = 0,
  FE_ERR_CUDA = 1,     /* CUDA / cuFFT failure or no device */
  FE_ERR_ARG = 2,      /* invalid argument */
  FE_ERR_OVERFLOW = 5, /* neighbour-list row over capacity (nblist.c:185-197 exit 5) */
  FE_ERR_CHARGE = 20,  /* non-neutral box (ewald.c:185-194 exit 20) */
  FE_ERR_STATE = 30,   /* call order (e.g. forces before a list exists) */
  FE_ERR_DEVICE = 31,  /* a kernel reported an error status (bounded loop ran out, bad index) */
  FE_ERR_SIZE = 32     /* request beyond a fixed maximum */
};

/* arithmetic of the pair / SPME kernels */
enum {
  FE_PREC_FP64 = 0, /* plain FP64: the drop-in (same arithmetic as the reference) */
  FE_PREC_MIXED = 1 /* FP32 pair/PME math, 64-bit fixed-point force sums, FP64 integration */
};

/* en[k] fields, in this order, for every energy record */
enum {
  FE_EN_KINET = 0, FE_EN_BOND, FE_EN_BEND, FE_EN_NBOND, FE_EN_NBONDS,
  FE_EN_COULOMB, FE_EN_REWALD, FE_EN_REWALDS, FE_EN_KEWALD, FE_EN_SEWALD,
  FE_EN_IEWALD, FE_EN_TEWALD, FE_EN_UREY, FE_EN_TORS, FE_EN_IMPR, FE_EN_COUNT
};

typedef struct fe_box fe_box;

/* Box description: what read_sim.c / read_config.c / read_topology.c /
 * setlj.c leave in sim, box[k], pott[k], ljset, bond[k], bend[k], xint[k]. */
typedef struct {
  int n;              /* box[k].boxns */
  int ntypes;         /* NUM_ATOM (site types) */
  double L[3];        /* box[k].lx, ly, lz */
  double rc;          /* sim.rc */
  double rclist;      /* sim.rclist */
  double rclist_ew;   /* sim.rclist_ew */
  double kappa;       /* sim.kappa[k] */
  double epsRF;       /* sim.epsRF[k] */
  double dt;          /* sim.dt [ps] */
  double T;           /* sim.T[k] [K] */
  int grid[3];        /* sim.grid */
  int order;          /* sim.order (B-spline order, 3..8) */
  double r_switch;    /* LJ switch start (CHARMM switch r_switch..rc); 0 = off (reference) */
  int precision;      /* FE_PREC_* */
  int max_neighbors;  /* capacity per list row; 0 = the reference's rule (allocate.c:321-322) */
  int device;         /* CUDA device ordinal */
  /* sites */
  const double *q;    /* n  pott[k][i].qq */
  const double *mass; /* n  pott[k][i].mas */
  const int *type;    /* n  atom[k][i].atomid */
  const double *lj_eps; /* ntypes*ntypes, ljset[ta][tb].eps [kJ/mol] */
  const double *lj_sig; /* ntypes*ntypes, ljset[ta][tb].sig (R_min) [A] */
  /* bonded terms of forces() (cbond.c, cbend.c) */
  int nbond;
  const int *bond_ab;        /* 2*nbond */
  const double *bond_req;    /* nbond */
  const double *bond_k;      /* nbond, E = k (r - req)^2 */
  int nbend;
  const int *bend_abc;       /* 3*nbend (apex in the middle) */
  const double *bend_theta0; /* nbend [rad] */
  const double *bend_k;      /* nbend, E = k (theta - theta0)^2 */
  /* excluded / modified pairs (xint[k]): flag 1 bond, 2 bend, 3 exNB, 4 1-4 */
  int nexcl;
  const int *excl_ab;   /* 2*nexcl */
  const int *excl_flag; /* nexcl */
  /* Nose-Hoover chain (nhc[k], read_sim.c:537-561) */
  int nhc_M;
  double nhc_Q;
  double nfree;       /* box[k].nfree; <= 0 means 3n - 3 (read_config.c:340-342) */
} fe_box_params;

/* ---- lifetime ---------------------------------------------------------- */

/* Allocates the box on the device (the reference's allocate.c:312-505 and
 * ewald_setup(), ewald.c:46-197: SPME setup, B-spline moduli, self energy,
 * neutrality check).  Returns FE_ERR_CHARGE for a non-neutral box. */
int fe_box_create(fe_box **out, const fe_box_params *p);
/* Frees everything (pme_clean, pme_setup.c:249-257, and mem_free.c). */
void fe_box_destroy(fe_box *box);
/* Issue all work of this box on `stream` (a cudaStream_t); NULL = the box's own. */
int fe_box_set_stream(fe_box *box, void *stream);
const char *fe_last_error(void);
int fe_abi_version(void);

/* ---- state transfer (host <-> device) ----------------------------------- */

/* Positions from `struct atoms`-like records: x at `off_x`, y, z following,
 * `stride` bytes apart (atom[k]: stride 64, off_x 16).  Also sets the
 * unwrapped copy (atnopbc) when `nopbc` is nonzero. */
int fe_set_positions(fe_box *box, const void *atoms, size_t stride, size_t off_x, int nopbc);
int fe_get_positions(fe_box *box, void *atoms, size_t stride, size_t off_x);
int fe_set_positions_nopbc(fe_box *box, const void *atoms, size_t stride, size_t off_x);
int fe_get_positions_nopbc(fe_box *box, void *atoms, size_t stride, size_t off_x);
/* `struct veloc` arrays (vv[k], uu[k], ff[k]): n x 3 doubles */
int fe_set_velocities(fe_box *box, const double *vv, const double *uu);
int fe_get_velocities(fe_box *box, double *vv, double *uu);
int fe_get_forces(fe_box *box, double *ff);
/* ff[k] before routines that accumulate into it (cnonbondnl, pme_calc) or
 * read it (the first half-kick of integrate_vverlet). */
int fe_set_forces(fe_box *box, const double *ff);
/* NHC state nhc[k].zeta[j].{r,v,G}: 3*M doubles */
int fe_set_nhc_state(fe_box *box, const double *zeta);
int fe_get_nhc_state(fe_box *box, double *zeta);

/* ---- hot path ------------------------------------------------------------ */

/* nblist(ibox), nblist.c:32-592: half Verlet list b > a with the reference's
 * distance test (components against rclist, dr2 < rclist^2 and
 * dr2 < rclist_ew^2), built from a cell grid on the device.  Rows keep the
 * reference's order (ascending b) and carry the xint flag. */
int fe_nblist(fe_box *box);
/* Copies the list to the host as CSR (count[n], idx/flag[<= cap]); returns
 * FE_ERR_SIZE when cap is too small.  *total gets the number of entries. */
int fe_nblist_download(fe_box *box, int *count, int *idx, int *flag, int64_t cap, int64_t *total);

/* forces(ibox), forces.c:118-446: zero ff, cbond, cbend, cnonbondnl (pair
 * loop + pme_calc).  `en` (may be NULL) gets FE_EN_COUNT values with
 * FE_EN_KINET left as the last kinet() result. */
int fe_forces(fe_box *box, double *en);
/* cnonbondnl(ibox, energy), cnonbond_nblist.c:51-622: accumulates the pair
 * and SPME forces into ff; energy[8] as the reference assembles it. */
int fe_cnonbondnl(fe_box *box, double *energy8);
/* pme_calc(k, energy), pme_calc.c:18-279 (charge_grid, FFTs, reciprocal
 * sum, pme_force with mean-force removal): accumulates into ff. */
int fe_pme_calc(fe_box *box, double *energy3);
/* The LJ form of the pair loop, as the reference's build chooses it: 0 its
 * default eps[(R/r)^12 - 2(R/r)^6]; 2 its BGO build (cnonbond_nblist.c:
 * 294-307), eps[13(R/r)^12 - 18(R/r)^10 + 4(R/r)^6] with the shifted energy
 * at rc likewise.  FP64 boxes without the LJ switch (FE_ERR_STATE
 * otherwise). */
int fe_box_set_lj_form(fe_box *box, int form);
/* pme_force(k), pme_calc.c:122-279: the reciprocal forces from the grid as
 * the last fe_pme_calc left it (convolved, back in real space) and the
 * splines of the last charge_grid, mean force removed, accumulated into ff
 * (pme_calc calls it at its end; the drop-in exports it for callers of its
 * own). */
int fe_pme_force(fe_box *box);
/* fillspline(w, array, darray), pme_spline.c:10-49: B-spline weights
 * array[1..order] and derivatives darray[1..order] at fraction w (host
 * arithmetic, the reference's recursion; arrays of order + 1 doubles). */
int fe_bspline(int order, double w, double *array, double *darray);
/* charge_grid(k), pme_qgrid.c:13-121: spread charges; fe_get_charge_grid
 * copies the real grid (grid[0]*grid[1]*grid[2] doubles, x slowest). */
int fe_charge_grid(fe_box *box);
int fe_get_charge_grid(fe_box *box, double *grid);
/* cbond + cbend energies into en2 (forces accumulated into ff). */
int fe_bonded(fe_box *box, double *en2);

/* ---- bonded terms beyond bonds and bends (read_topology.c fills urey[k],
 * tors[k], impr[k]); each call replaces the box's set of that kind and
 * forces() includes them from then on (FE_EN_UREY, FE_EN_TORS, FE_EN_IMPR). */
/* Urey-Bradley 1-3 terms, curey.c:37-106: E = k (r_ab - seq)^2.
 * ab: 2*n site indices; seq [A]; k [kJ/mol/A^2]. */
int fe_set_ureys(fe_box *box, int n, const int *ab, const double *seq, const double *k);
/* Proper torsions, ctorsion.c:63-246: E = sum_t kphi[t] (1 + cos(nphi[t] tau
 * - delphi[t])) over t < 6, the series ending at the first kphi[t] == 0 (as the
 * reference's loop); tau is the dihedral a-b-c-d.  abcd: 4*n; kphi, nphi,
 * delphi: 6*n each (struct torsions' arrays) [kJ/mol, 1, rad]. */
int fe_set_torsions(fe_box *box, int n, const int *abcd, const double *kphi,
                    const double *nphi, const double *delphi);
/* Improper torsions, cimproper.c:55-221: E = kimpr (tau - angeq)^2.
 * abcd: 4*n; kimpr [kJ/mol/rad^2]; angeq [rad]. */
int fe_set_impropers(fe_box *box, int n, const int *abcd, const double *kimpr,
                     const double *angeq);
/* The dihedral tau of every torsion at the last force evaluation
 * (ctorsion.c:172-175 stores it in tors[k][i].phi / psi / theta by tag). */
int fe_get_torsion_angles(fe_box *box, double *tau);
/* curey + ctorsion + cimproper energies into en3 (forces accumulated into ff). */
int fe_bonded_ext(fe_box *box, double *en3);
/* zero ff (forces.c:126-130) */
int fe_zero_forces(fe_box *box);

/* pbc_all(ibox), pbc_all.c:23-88 */
int fe_pbc_all(fe_box *box);
/* kinet(ibox), kinet.c:18-68: ken[6] tensor and the scalar (may be NULL) */
int fe_kinet(fe_box *box, double *ken6, double *kinet);
/* integrate_vverlet(ibox, vscal), integrate_vverlet.c:36-103 (includes
 * pbc_all and forces); `en` as for fe_forces, may be NULL. */
int fe_integrate_vverlet(fe_box *box, double vscal, double *en);
/* Host arrays of one integrate_vverlet call as the drop-in makes it: the
 * wrapped positions (struct atoms records by stride/offset, as
 * fe_set_positions), the unwrapped ones (atnopbc), vv, uu and ff (3n
 * doubles each); all are read before the step and written after it. */
typedef struct fe_md_io {
  void *atoms;
  size_t atoms_stride, atoms_off;
  void *nopbc;
  size_t nopbc_stride, nopbc_off;
  double *vv, *uu, *ff;
} fe_md_io;
/* integrate_vverlet with its host state in one call: the uploads of atom,
 * atnopbc, vv and ff (uu is only written, integrate_vverlet.c:95-97), the
 * step, the downloads of all five and `en`.  With every array in pinned host
 * memory and 24-byte strides the copies are queued around the step (the
 * positions' download on a second stream while the forces are evaluated)
 * and the call synchronises once (copies and kernels are captured as one
 * graph on the first call with a given set of arrays and vscal, and
 * replayed while they stay the same); otherwise it makes the separate calls
 * (fe_set_positions .. fe_get_forces) with their own synchronisations.
 * Same results either way. */
int fe_integrate_vverlet_host(fe_box *box, double vscal, const fe_md_io *io, double *en);
/* integrate_nhc(time_step, ibox), integrate_nhc.c:40-161 (Nc = Nys = 1) */
int fe_integrate_nhc(fe_box *box, double time_step);
/* RESPA multiple time stepping (FP64 boxes; FE_ERR_STATE for mixed):
 * force_short(ibox), force_short.c:46-137: cbond + cbend + curey into
 * ff_short (ff holds them after the call, en's bond/bend/urey updated). */
int fe_force_short(fe_box *box, double *en);
/* force_long(ibox), force_long.c:46-145: ctorsion + cimproper + cnonbondnl
 * (with SPME) into ff and ff_long; en's other terms updated. */
int fe_force_long(fe_box *box, double *en);
/* integrate_mts(ibox, vscal), integrate_mts.c:37-140: one long step of
 * nshort short steps (sim.nsteps; the long step dt * nshort, init.c:314),
 * pbc_all and both force classes inside; uu = vv after; `en` may be NULL.
 * ff_short and ff_long start at zero as the reference's arrays do: call
 * fe_force_short and fe_force_long first (nve_md.c:298-304). */
int fe_integrate_mts(fe_box *box, double vscal, int nshort, double *en);
/* integrate_mts_nhc(ibox, vscal), integrate_mts_nhc.c:37-162: RESPA with
 * the Nose-Hoover chain of fe_integrate_nhc applied over half a long step at
 * both ends of the long step (xrespa = sim.xRESPA = 0) or over half a short
 * step at both ends of every short step (xrespa = 1); the kicks carry no
 * vscal, as there. */
int fe_integrate_mts_nhc(fe_box *box, int nshort, int xrespa, double *en);
/* The ff_short / ff_long arrays (either pointer may be NULL). */
int fe_get_forces_mts(fe_box *box, double *ff_short, double *ff_long);
int fe_set_forces_mts(fe_box *box, const double *ff_short, const double *ff_long);
/* drift(ibox), drift.c:21-66: removes the net momentum from the velocities
 * (v_i -= (sum_j m_j v_j / n) / m_i); uu is left as it is. */
int fe_drift(fe_box *box);
/* The thermostat temperature sim.T[k] of the box (integrate_nhc reads it):
 * replica swaps that move a configuration to another box keep the box's
 * temperature (swap_box.c:5-86). */
int fe_box_set_temperature(fe_box *box, double T);

/* The production step loop of nve_md.c:359-418 (use_nhc = 0) or nvt_md.c
 * with ID2 == 4 (use_nhc = 1): for i = 1..nsteps { if i % nlist_freq == 0
 * nblist; [nhc]; integrate_vverlet(1.0); [nhc]; kinet }, captured in a CUDA
 * graph and replayed.  `rec` (may be NULL) gets FE_EN_COUNT doubles per step
 * (nsteps records). `first_step` is the value of i for the first step. */
int fe_run_md(fe_box *box, int nsteps, int nlist_freq, int use_nhc, long first_step, double *rec);

/* ---- classic-Ewald Monte Carlo energy path (ewald_mc.c, enbnd_mc.c) --------- */

/* Set up the k-vector table of ewald_setup (ewald.c:95-118) for kmax in
 * each direction and max_k_square, and the structure factor S(k) of the
 * current positions.  rc_ew is sim.rc_ew. */
int fe_mc_setup(fe_box *box, int kmax, int max_k_square, double rc_ew);
/* Energy change of moving sites [lb, ub) to new_pos (n_moved x 3 doubles):
 * exact reciprocal part from the incremental structure-factor update plus
 * real-space Ewald and shifted LJ over all pairs touching the moved sites
 * (minimum image).  parts3 (may be NULL) = {dE_recip, dE_real, dE_lj}.
 * Replaces forces_mc(lb,ub,0|1,k) old/new differencing (forces_mc.c:90-573). */
int fe_mc_delta(fe_box *box, int lb, int ub, const double *new_pos, double *dE, double *parts3);
/* The same move with the change split into the reference's energy terms
 * (ewald_mc.c / enbnd_mc.c): terms6 = {reciprocal (ewald_kspace_mc
 * enkewald[0]), LJ (enonbond), LJ shift constant (enonbonds; 0 under the
 * switch), real space (eewald_real), its shift constant (eewald_reals),
 * intramolecular correction (eewald_intra)}, each new minus old. */
int fe_mc_delta_terms(fe_box *box, int lb, int ub, const double *new_pos, double *terms6);
/* The current energy of the pairs touching sites [lb, ub) in the same six
 * terms, the first being the whole reciprocal energy: enbnd_mc(lb, ub) of
 * enbnd_mc.c:26-501 (whose ewald_rspace_mc also counts the pairs of rows
 * below lb that do not touch the range; they cancel in every difference). */
int fe_mc_site_energy(fe_box *box, int lb, int ub, double *terms6);
/* Commit the last fe_mc_delta move (positions and S(k) update) -- the
 * accepted branch of mcmove_trans.c:177; a rejected move needs no call
 * (mcmove_rstr restores nothing on the device). */
int fe_mc_accept(fe_box *box);
/* Current k-space energy from the maintained S(k) (ewald_kspace_mc enkewald[0]). */
int fe_mc_kspace_energy(fe_box *box, double *e);

/* ---- allocation-free entry (no counterpart in the reference) ---------------
 *
 * For callers that may not allocate device memory themselves -- a plug-in
 * inside a host program whose device memory all comes from that program's own
 * allocator (a caching allocator or a pool reserved once under a fixed
 * budget).  Computes the classic-Ewald reciprocal energy of ewald_kspace_mc
 * (ewald_mc.c:186-287 with the k-vectors of ewald.c:104-118, in kJ/mol) of
 * n sites given as device memory xyzq[4*i+0..3] = x, y, z, q, into the device
 * double *energy, on `stream` (a cudaStream_t, NULL = the legacy default
 * stream).  L is a host array of the 3 box lengths.  Allocates nothing: its
 * only temporary is a fixed 64 KB array in device memory that each GPU using
 * the library keeps until the process exits.  Limit: (kmax+1)*(2*kmax+1)^2 <=
 * 8192 candidate k-vectors (kmax <= 12), else FE_ERR_SIZE.  The first call on
 * a device looks up that array's device address, so make the first call on
 * each device before any stream capture (outside a capture every call looks
 * it up again, so a device reset between calls is fine).  All calls share the
 * array; calls whose kernels overlap on the GPU race and must be serialised.
 * xyzq and energy must be device or managed memory: a host pointer is refused
 * with FE_ERR_ARG before anything is launched. */
int fe_ewald_kspace_energy_noalloc(const double *xyzq, int n, const double *L, double kappa,
                                   int kmax, int max_k_square, double *energy, void *stream);

/* ---- Monte Carlo chains resident on the device ------------------------- */

/* nchains independent Metropolis chains of rigid-molecule moves on copies of
 * the box's current configuration, one CTA per chain, thousands of moves per
 * launch.  Replaces the move loop of nvt_mc.c:70-422 with its energy calls
 * (forces_mc.c:90-573, ewald_kspace_mc ewald_mc.c:42-324, ewald_rspace_mc
 * ewald_mc.c:328-641 with the correct minimum image) and its acceptance rule
 * (mcmove_displ.c:130-137).  A move picks a molecule (mol_first[m] ..
 * mol_first[m+1]-1, at most 8 sites) uniformly; with probability p_rot it
 * rotates it about its centre of mass by an angle uniform in
 * [-rot_max, rot_max] [rad] around a uniform random axis, otherwise it
 * translates it by (u - 0.5) * delta per axis (mcmove_displ.c:92-94).  dE is
 * the shifted LJ within rc, real-space Ewald within rc_ew and the
 * classic-Ewald reciprocal sum over the k-vectors of ewald_setup with
 * |n|^2 <= max_k_square (ewald.c:104-118, kappa of the box), in kJ/mol; T
 * sets beta = 1/(RG T / 1000).  Coordinates are kept as 32-bit fixed-point
 * fractions of the box and pair/phase arithmetic is FP32 with FP64 sums
 * (|dE error| ~1e-3 kJ/mol).  Limits: n <= 10240 sites, <= 8 site types,
 * <= 1024 k-vectors; excluded pairs must lie inside molecules.  Draws are
 * Philox4x32-10 keyed by seed with counter (chain, move).  The first log_cap
 * moves of chain 0 are logged. */
int fe_mc_chains_setup(fe_box *box, int nchains, const int *mol_first, int nmol, int kmax,
                       int max_k_square, double rc_ew, double T, double delta, double rot_max,
                       double p_rot, uint64_t seed, int log_cap);
/* nmoves further moves of every chain. */
int fe_mc_chains_run(fe_box *box, int64_t nmoves);
/* Chain state: xyz (n x 3, wrapped to [-L/2, L/2)), moves made, moves accepted. */
int fe_mc_chains_state(fe_box *box, int chain, double *xyz, int64_t *moves, int64_t *accepted);
/* Reciprocal energy sum_k c_k |S_k|^2 of a chain from its running S(k) [kJ/mol]. */
int fe_mc_chains_kspace_energy(fe_box *box, int chain, double *e);
/* Logged moves of chain 0: rec[12] per move = {2 lb + is_rotation, sites,
 * accepted, dE, dE_k (both NaN when not evaluated), dE_real, u1, dE1 (stage-1
 * energy; dE in exact mode), u2, stage-1 accepted, dE_k evaluated, surrogate
 * g(after) - g(before)}; fx[24] per move = trial fixed-point coordinates
 * (x, y, z per site; position = (u / 2^32 - 0.5) L). */
int fe_mc_chains_log(fe_box *box, double *rec, uint32_t *fx, int64_t cap, int64_t *count);

/* ---- Monte Carlo surrogate network (no counterpart in the reference) ---- */

/* g(x) = w3 . silu(W2 silu(W1 (x - mean) * istd + b1) + b2) + b3, 64 inputs,
 * hidden 128 + 128, trained and evaluated with BF16-in / FP32-accumulate
 * tensor-core kernels (tcgen05).  A sample is 128 floats (descriptors of a
 * trial move before | after) and a target y; the model's prediction is
 * g(after) - g(before).  Parameters are packed W1[128][64], b1[128],
 * W2[128][128], b2[128], w3[128], b3 (fe_mlp_param_count() floats). */
typedef struct fe_mlp fe_mlp;
int fe_mlp_create(fe_mlp **out, int device, uint64_t seed);
void fe_mlp_destroy(fe_mlp *mlp);
int fe_mlp_param_count(void);
int fe_mlp_set_params(fe_mlp *mlp, const float *params, const float *mean, const float *istd);
int fe_mlp_get_params(fe_mlp *mlp, float *params, float *mean, float *istd);
/* Loss (mean squared error) and gradient at the current parameters for B
 * samples (B % 64 == 0); out2B (may be NULL) gets g of the 2B rows
 * (before rows first). */
int fe_mlp_grad(fe_mlp *mlp, const float *data, const float *y, int B, float *grad, float *loss,
                float *out2B);
/* Adam on shuffled batches; normalisation set from the samples first;
 * loss_hist[e] = mean batch loss of epoch e. */
int fe_mlp_train(fe_mlp *mlp, const float *data, const float *y, int64_t n, int epochs, int batch,
                 float lr, uint64_t seed, float *loss_hist);
/* Delayed acceptance for the MC chains (Christen & Fox 2005).  Stage 1
 * accepts with min(1, exp(-beta dE1)), dE1 = exact real-space + LJ dE plus
 * the surrogate's g(after) - g(before) for the reciprocal part; only then is
 * the exact reciprocal dE_k computed and stage 2 accepts with
 * min(1, exp(-beta (dE - dE1))).  The surrogate's difference form is
 * antisymmetric under reversing a move, so the chain keeps exact detailed
 * balance for the full Ewald energy.  Descriptors (64 per configuration):
 * for each moved site and partner within 9 A, the partner charge spread
 * over 16 tent functions of r centred at 1.0, 1.5, .., 8.5 A, in 4 channels
 * (site charge sign x partner charge sign). */
/* Store (descriptors before, after, exact dE_k) of up to per_chain moves of
 * every chain (0 = stop collecting); under delayed acceptance the last value
 * is the surrogate's estimate instead of dE_k. */
int fe_mc_chains_collect(fe_box *box, int64_t per_chain);
/* Collected samples, 129 floats each, chain after chain (out may be NULL). */
int fe_mc_chains_samples(fe_box *box, float *out, int64_t cap, int64_t *count);
/* Trains the network on the collected samples without leaving the device. */
int fe_mc_chains_train_surrogate(fe_box *box, fe_mlp *mlp, int epochs, int batch, float lr,
                                 uint64_t seed, float *loss_hist);
/* Copies the network into the chains (bf16 weights, FP32 arithmetic in the kernel). */
int fe_mc_chains_set_surrogate(fe_box *box, fe_mlp *mlp);
/* 0: exact dE in one stage; 1: delayed acceptance (after set_surrogate);
 * 2 and 3: the same two with the reciprocal change recomputed from every site
 * at every evaluation (S(k) before and after the move summed over all sites,
 * float-pair sums) -- the cost of the reference's ewald_kspace_mc evaluation
 * (ewald_mc.c:109-156, called before and after each trial by forces_mc), kept
 * as the denominator of its delayed-acceptance comparison. */
int fe_mc_chains_set_mode(fe_box *box, int mode);
/* {moves, accepted, stage-1 accepted, exact reciprocal evaluations} of a chain. */
int fe_mc_chains_stats(fe_box *box, int chain, int64_t *out4);

/* The tensor-core GEMM alone: D (M x N fp32) = A (M x K) B (N x K)^T + bias,
 * A and B as bf16 bit patterns; M % 128 == 0, N in 32..256 step 32,
 * K % 64 == 0. */
int fe_tc_gemm_bf16(const uint16_t *A, const uint16_t *B, const float *bias, float *D, int M,
                    int N, int K);

/* ---- replicas stepped together, exchange on the device ----------------- */

/* A batch steps several boxes (any sizes, same device, same Nose-Hoover
 * chain length) in one CUDA graph per step, each box on its own stream, and
 * attempts replica exchanges on the device.  Replaces the box loop and the
 * swap schedule of repexch.c:139-214,268-305 and swap_box (swap_box.c:5-86).
 * Temperature slot s initially belongs to box s at that box's params.T.  An
 * accepted swap exchanges the slots (temperature and chain state) of two
 * boxes instead of their coordinates and rescales their velocities as
 * swap_box does.  The batch does not own the boxes. */
typedef struct fe_batch fe_batch;
int fe_batch_create(fe_batch **out, fe_box *const *boxes, int nbox, uint64_t seed);
void fe_batch_destroy(fe_batch *batch);
/* Steps first_step .. first_step+nsteps-1 of every box: a list rebuild before
 * step i when i % nlist_freq == 0, an exchange attempt after step i when
 * swap_freq > 0 and i % swap_freq == 0 (repexch.c counts steps from 1).
 * use_nhc: integrate_nhc around integrate_vverlet (nvt_md.c:529-531). */
int fe_batch_run(fe_batch *batch, int nsteps, int nlist_freq, int swap_freq, long first_step,
                 int use_nhc);
/* Any pointer may be NULL.  slot_box[s]: box holding slot s; T_box[b]:
 * current temperature of box b; accepted/attempted[s]: swaps of the slot
 * pair (s, s+1); attempts: exchange attempts made. */
int fe_batch_state(fe_batch *batch, int *slot_box, double *T_box, int64_t *accepted,
                   int64_t *attempted, uint64_t *attempts);
/* The stream the step graphs are launched on (for events around fe_batch_run). */
int fe_batch_get_stream(fe_batch *batch, void **stream);
/* Own kernel launches in one step graph: [plain, list, exchange, list+exchange];
 * -1 for a variant not captured yet. */
int fe_batch_step_launches(fe_batch *batch, int *launches4);
/* Fused stepping (the default when every box is mixed precision with
 * molecules as contiguous runs of sites): each kernel of the step runs once
 * for all boxes, box r owning a contiguous range of its blocks, and the
 * charge grids of boxes of equal shape are transformed by one batched FFT;
 * list rebuilds stay per box.  on = 0 steps every box on its own stream
 * (one graph branch per box).  Results are the same either way (fixed-point
 * sums).  FE_ERR_ARG when on = 1 and a box does not allow it. */
int fe_batch_set_fused(fe_batch *batch, int on);

/* ---- batched replica exchange of Go-model chains ------------------------ */

/* nrep C-alpha chains (one per replica, 2..1024 beads each) stepped with
 * BAOAB Langevin dynamics (Leimkuhler & Matthews 2013) in one persistent
 * launch per exchange segment, one CTA per replica; replaces the replica loop
 * of repexch.c:139-305 with cnbnd_golik (cgolik.c:644-948) as its pair loop
 * and swap_box (swap_box.c:5-86) as its exchange.  Energy function: bonds
 * k_bond (r - r_bond)^2; native pairs eps [5 (r0/r)^12 - 6 (r0/r)^10] (r0 =
 * native distance, no cutoff); other pairs with |i - j| >= min_sep
 * eps (sigma_rep/r)^12 shifted to zero at rc_rep.  Forces FP32, positions,
 * velocities and the thermostat FP64.  Exchanges swap temperatures between
 * replicas (slots as in swap_box) and rescale velocities by sqrt(T_s/T_s+1). */
typedef struct {
  double eps;        /* native / repulsive energy scale [kJ/mol] */
  double sigma_rep;  /* non-native repulsion sigma [A] */
  double rc_rep;     /* non-native repulsion cutoff [A] */
  double k_bond;     /* [kJ/mol/A^2], E = k (r - r_bond)^2 */
  double r_bond;     /* [A] */
  double mass;       /* bead mass [amu] */
  double gamma;      /* Langevin friction [1/ps] */
  double dt;         /* [ps] */
  int min_sep;       /* non-bonded pairs need |i - j| >= min_sep */
  int device;
} fe_go_params;
typedef struct fe_go fe_go;
/* nbeads[r] beads per replica, concatenated pos/vel (3 doubles per bead),
 * natives as CSR over the global bead index (both directions, partners in
 * the same chain) with native distances nat_r0; T[r] the starting
 * temperature (slot r). */
int fe_go_create(fe_go **out, int nrep, const int *nbeads, const double *pos, const double *vel,
                 const int *nat_start, const int *nat_j, const double *nat_r0, const double *T,
                 const fe_go_params *p, uint64_t seed);
void fe_go_destroy(fe_go *go);
/* nsteps steps; an exchange attempt after every swap_freq steps (0 = none). */
int fe_go_run(fe_go *go, int64_t nsteps, int swap_freq);
/* Forces (FP32, returned as doubles) and potential energy per replica at the
 * current positions. */
int fe_go_forces(fe_go *go, double *f, double *epot);
/* Any pointer may be NULL; accepted/attempted per slot pair (s, s+1). */
int fe_go_state(fe_go *go, double *pos, double *vel, double *T, double *epot, int *slot_rep,
                int64_t *accepted, int64_t *attempted, uint64_t *steps);
int fe_go_get_stream(fe_go *go, void **stream);
/* Switches the batch to the reference's own Go model (cgolik.c): bonds
 * eps dr^2 + 100 eps dr^4 with bond_r0[i] the length of bond (i, i+1)
 * (global bead index; the last bead of a chain unused), bends
 * 10 eps (theta - theta0)^2 with bend_t0[i] the angle centred at bead i,
 * torsions 0.2 eps (1 + cos 3 tau), natives 4 eps [(s/r)^12 - (s/r)^6] with
 * s = 2^(-1/6) r0 within rc (energy shifted to zero there), non-natives the
 * same with s = 2^(-1/6) d_rep within d_rep, lifted by eps; only bonded
 * pairs excluded. */
int fe_go_set_reference_form(fe_go *go, const double *bond_r0, const double *bend_t0,
                             double d_rep, double rc);
/* The launch's load-balance plan: *ncta CTAs (clusters of four), *slots the
 * CTAs the GPU holds at once, parts[r] (nrep ints, may be NULL) the CTAs
 * that share replica r's chain (1 to 4). */
int fe_go_layout(fe_go *go, int *ncta, int *slots, int *parts);

/* ---- launch-shape autotuning (no counterpart in the reference) --------- */

/* Times the mixed-precision pair kernel over the box's current list for
 * warps per block in {4, 8, 16}, register budgets of 40 and 64 per thread
 * and several grid sizes, and keeps the fastest for this box (results do not
 * depend on the shape: forces are fixed-point sums).  choice3 = {warps per
 * block, registers per thread, blocks}, *us = its time per launch.
 * Recomputes the forces afterwards; a no-op for FP64 boxes. */
int fe_autotune(fe_box *box, int *choice3, double *us);

/* ---- instrumentation (no counterpart in the reference) ----------------- */

enum { FE_KERNEL_PAIR = 0, FE_KERNEL_SPREAD = 1, FE_KERNEL_LIST = 2 };
/* Re-launches one kernel of the force step on the current state `reps` times
 * between CUDA events on the box's stream; *us = mean device time per launch.
 * Scratch sums are overwritten; call fe_forces again before reading forces. */
int fe_time_kernel(fe_box *box, int which, int reps, double *us);
/* Measured arithmetic peak of a device, the denominator of pipe fractions:
 * which = 0 FP32 FMA, 1 FP64 FMA (TFLOP/s, an FMA counted as two), 2 the
 * special-function unit's ex2.approx (Tera-ops/s). */
int fe_pipe_peak(int device, int which, double *tera_per_s);
/* Number of this library's own kernel launches in one fe_run_md step without
 * and with a list rebuild (cuFFT's kernels not included). */
int fe_step_launches(fe_box *box, int use_nhc, int *plain, int *with_list);
/* Entries of the current pair list (half list in FP64 mode, full list in
 * mixed mode) and the longest row. */
int fe_list_stats(fe_box *box, int64_t *entries, int *max_row);
/* FP64 boxes: {half-list entries, pairs within rc that the pair loop
 * evaluates, those with an LJ term, excluded pairs within rc} of the current
 * list -- the units of the pair loop's algorithmic FLOP count. */
int fe_pair_counts(fe_box *box, int64_t *counts4);
/* nl_check(lb, ub, k), nblist.c:607-647 (DLIST): *nl_flag = 1 if any site
 * of [lb, ub) has moved more than (rclist - rc)/4 since the last fe_nblist
 * (along one axis or in distance, with the reference's image rule), else 0.
 * The reference keeps its nl_flag set until the next nblist; a caller that
 * mirrors it ORs the result in. */
int fe_nl_check(fe_box *box, int lb, int ub, int *nl_flag);
/* Mixed mode: entries and longest row of the inner list (rc + 0.8 A) the
 * pair kernel walks between prunes, and how many pair-kernel launches have
 * pruned it from the outer list so far (after every list rebuild, and when a
 * site has moved 0.4 A since the last prune).  FE_ERR_STATE in FP64 mode or
 * when the inner list is off (rc + 0.8 A >= rclist). */
int fe_inner_list_stats(fe_box *box, int64_t *entries, int *max_row, int64_t *prunes);

#ifdef __cplusplus
}
#endif
#endif
