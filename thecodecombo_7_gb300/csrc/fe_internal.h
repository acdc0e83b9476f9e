// fe_internal.h -- device-resident state of one box and the launch wrappers
// shared by the translation units of libfe.so.
#pragma once

#include <cuda_runtime.h>
#include <cufft.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/fe.h"

namespace fe {

struct Mixed;
struct McChains;
struct Mlp;

// Physical constants of the reference (defines.h:62-75).
constexpr double kPI = 3.141592653589793238462643383;
constexpr double kKB = 1.380662E-23;
constexpr double kNA = 6.022045E23;
constexpr double kAU = 1.6605655E-27;
constexpr double kELEC = 8.987551789e19;
constexpr double kELEQ = 1.602176462e-19;
constexpr double kE14FAC = 0.4;

// device status word bits (box->status): set by kernels, checked on the host
enum : int {
  ST_LIST_OVERFLOW = 1,   // a list row exceeded its capacity
  ST_CELL_OVERFLOW = 2,   // a cell bin exceeded its capacity
  ST_PBC_LOOP = 4,        // pbc wrap did not converge (non-finite or runaway position)
  ST_GRID_OVERFLOW = 8,   // an SPME grid bin exceeded its capacity
  ST_BAD_INDEX = 16,      // an index outside its array was met and skipped
};

// Slots of the device scalar block (box->scal).  Energies FE_EN_* first.
enum : int {
  SC_EN = 0,                       // FE_EN_COUNT energies
  SC_LJ = FE_EN_COUNT,             // enonbond
  SC_LJS,                          // enonbonds
  SC_REAL,                         // eewald_real
  SC_REALS,                        // eewald_reals
  SC_INTRA,                        // eewald_intra
  SC_BOND, SC_BEND,                // cbond, cbend
  SC_UREY, SC_TORS, SC_IMPR,       // curey, ctorsion, cimproper
  SC_ENREC,                        // sum eterm * |S|^2 (before the fan factor)
  SC_FMEAN,                        // 3 slots: sum of the reciprocal forces
  SC_KEN = SC_FMEAN + 3,           // 6 slots: kinetic-energy tensor
  SC_NHC_SCALE = SC_KEN + 6,       // last NHC velocity scale
  SC_ENERGY8,                      // 8 slots: cnonbondnl energy[]
  SC_ENERGY3 = SC_ENERGY8 + 8,     // 3 slots: pme_calc energy[]
  SC_MX_PAIR = SC_ENERGY3 + 3,     // 4 slots: mixed pair sums (lj, ljs, real, sum qq)
  SC_MX_EXCL = SC_MX_PAIR + 4,     // 5 slots: mixed exclusion sums (.., intra)
  SC_TEMP = SC_MX_EXCL + 5,        // thermostat temperature [K] (sim.T[k]); exchanges rewrite it
  SC_MX_INTRA,                     // 7 slots: fused intramolecular sums (5 exclusion, bond, bend)
  SC_EXT_TMP = SC_MX_INTRA + 7,    // 3 slots: curey/ctorsion/cimproper sums of a subset of the kinds
  SC_COUNT = SC_EXT_TMP + 3
};

// Largest number of blocks a partial-sum kernel may use.
constexpr int kMaxPartialBlocks = 4096;
constexpr int kPartialTerms = 8;
constexpr int kFaccSlots = 16;

struct Box {
  fe_box_params p;  // scalars (pointers inside are not kept)
  int n = 0, nt = 0;
  int dev = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  // fe_integrate_vverlet_host: a copy stream for the positions' download,
  // which overlaps the force evaluation (created on first use)
  cudaStream_t s_io = nullptr;
  cudaEvent_t ev_io_pos = nullptr, ev_io_done = nullptr;
  // graph of the host-buffer step, captured for one set of host arrays and
  // one velocity scale; dropped with the step graphs when the box changes
  cudaGraphExec_t g_io = nullptr;
  const void *io_key[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  double io_vscal = 0.0;
  int prec = FE_PREC_FP64;
  int lj_form = 0;  // the pair loop's LJ form: 0 CHARMM, 2 the reference's BGO build

  // sites
  double4 *pos_q = nullptr;   // x, y, z (wrapped), q
  double *pos_nopbc = nullptr;  // 3n
  double4 *pos_list0 = nullptr; // n: wrapped positions at the last list build (nl_check)
  int *nl_dev = nullptr;        // 1: nl_check's flag
  double *vv = nullptr, *uu = nullptr, *ff = nullptr;  // 3n, struct veloc layout
  double *ff_short = nullptr, *ff_long = nullptr;      // 3n each, RESPA's fast and slow forces
  double *mass = nullptr;
  double *imass100 = nullptr;  // 100 / mass (integrate_vverlet.c:56), one division at setup
  int *type = nullptr;
  double *lj_eps = nullptr, *lj_sig = nullptr;  // nt*nt
  // exclusions, per atom, both directions, in xint order
  int *x_start = nullptr, *x_partner = nullptr, *x_flag = nullptr;
  int nexcl = 0;
  // bonded
  int nbond = 0, nbend = 0;
  int *bond_ab = nullptr, *bend_abc = nullptr;
  double *bond_req = nullptr, *bond_k = nullptr, *bend_t0 = nullptr, *bend_k = nullptr;
  // Urey-Bradley, proper and improper torsions (fe_set_ureys / _torsions / _impropers)
  int nurey = 0, ntors = 0, nimpr = 0;
  int *urey_ab = nullptr, *tors_abcd = nullptr, *impr_abcd = nullptr;
  double *urey_seq = nullptr, *urey_k = nullptr;
  double *tors_par = nullptr;  // 18 per torsion: kphi[6], nphi[6], delphi[6]
  double *tors_tau = nullptr;  // the angle of each torsion at the last evaluation
  double *impr_k = nullptr, *impr_eq = nullptr;

  // cell grid for the list build
  int nc[3] = {1, 1, 1};
  int ncells = 1;
  int *cell_count = nullptr, *cell_start = nullptr, *cell_fill = nullptr, *cell_atoms = nullptr;
  int *cell_of = nullptr;  // n

  // Verlet list: padded rows (the reference's list[i][max_num_neighbors])
  int max_nb = 0;          // row capacity
  int *nl_count = nullptr; // n
  int *nl_ent = nullptr;   // n * max_nb, entry = b * 8 + xflag
  bool have_list = false;
  // set by step_body around a mixed NVE force evaluation: the force
  // finalisation and the energy assembly run inside the second half kick
  bool fold_tail = false;

  // SPME
  int G[3] = {0, 0, 0};
  int order = 4;
  long K = 0, Kh = 0;          // real grid points, half-spectrum points
  double *eterm = nullptr;     // Kh, exp(-pi^2 m^2/kappa^2)/(pi V m^2 B(m)); index 0 -> 1
  double *kweight = nullptr;   // Kh, 1 or 2 (half-spectrum multiplicity), 0 at m = 0
  double *grid = nullptr;      // K real grid (spread / convolved)
  cufftDoubleComplex *grid_k = nullptr;  // Kh
  cufftHandle plan_r2c = 0, plan_c2r = 0;
  bool plans = false;
  int *spl_floor = nullptr;    // 3n floor grid index (int)(ss)
  double *spl_m = nullptr;     // n * order * 3, weights mm[1..order] per axis
  double *spl_d = nullptr;     // n * order * 3, derivatives dm[1..order]
  double *fp = nullptr;        // 3n reciprocal forces before mean removal
  int gcap = 16;               // atoms per SPME bin
  int *gbin_count = nullptr;   // K
  int *gbin_atoms = nullptr;   // K * gcap
  double sewald = 0.0;

  // reductions and scalars
  double *partials = nullptr;  // kMaxPartialBlocks * kPartialTerms
  double *scal = nullptr;      // SC_COUNT
  int *status = nullptr;       // device status word
  unsigned *ticket = nullptr;  // last-block counter of the fused reductions (0 between kernels)
  unsigned long long *facc = nullptr;  // kFaccSlots fixed-point sums of block_fix_final (0 between kernels)
  double *host_scal = nullptr; // pinned SC_COUNT

  // NHC
  int nhc_M = 1;
  double nhc_Q = 1.0;
  double nfree = 0.0;
  double *zeta = nullptr;      // 3*M

  // run_md recording
  double *rec = nullptr;       // device records
  long rec_cap = 0;
  int *rec_counter = nullptr;
  cudaGraphExec_t g_step = nullptr, g_step_list = nullptr;
  int g_key = -1;              // graph capture key (use_nhc)
  int launches_plain = 0, launches_list = 0;  // own kernels per step
  double *stage = nullptr;     // pinned host staging, 4n doubles
  double *xyz_dev = nullptr;   // device staging, 3n doubles (packed x, y, z)

  // MC (classic Ewald)
  int mc_nk = 0, mc_kmax = 0, mc_mks = 0;
  double mc_rc_ew = 0.0;
  double *mc_kvec = nullptr;   // nk: 2*pi*exp(-b k^2)/k^2/V times multiplicity
  int *mc_kidx = nullptr;      // 3*nk
  double2 *mc_S = nullptr;     // nk structure factor
  double2 *mc_dS = nullptr;    // nk pending update
  double *mc_newpos = nullptr; // staged move
  int mc_lb = 0, mc_ub = 0, mc_pending = 0;
  double *mc_part = nullptr;   // partial sums
  int mc_nmax = 0;             // capacity of a staged move

  // mixed-precision path (k_mixed.cu); null in FP64 mode
  Mixed *mx = nullptr;
  McChains *mcc = nullptr;     // device-resident Monte Carlo chains (k_mcrun.cu)
};

// Per-box arguments of the batched integrator kernels (k_integrate.cu): a
// replica batch keeps one per box in device memory.
struct BIntArgs {
  int n, nhc_M;
  double dt, dt_h, nhc_Q, nfree;
  double3 L, H;
  const double *mass, *imass100;
  double *ff, *vv, *uu, *nopbc;
  double4 *pos;
  double *zeta, *scal;
  unsigned long long *facc;
  unsigned *ticket;
  int *status;
  double *rec;
  long rec_cap;
  int *rec_counter;
  // energy assembly of forces()
  double fan, sewald, erfc_rc_over_rc;
  int mixed, mixed_fused;
};

// ---- error plumbing ----
void set_error(const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);
int cufft_fail(cufftResult r, const char *what);
int check_status(Box *b);  // reads the device status word (synchronises)

#define FE_CUDA(call)                                         \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return ::fe::cuda_fail(e_, #call); \
  } while (0)

// counts this library's kernel launches (one per FE_LAUNCH_CHECK)
extern thread_local long g_launches;

#define FE_LAUNCH_CHECK(what)                                 \
  do {                                                        \
    ++::fe::g_launches;                                       \
    cudaError_t e_ = cudaGetLastError();                      \
    if (e_ != cudaSuccess) return ::fe::cuda_fail(e_, what);  \
  } while (0)

// ---- launch wrappers (each returns FE_OK or an error code) ----
// k_nblist.cu
int nblist_setup(Box *b);
int launch_nblist(Box *b);
int launch_nl_check(Box *b, int lb, int ub, int *dflag);  // nblist.c:607-647
// k_pair64.cu
int launch_pair64(Box *b);
int pair_counts64(Box *b, long long *out4);  // instrumentation: half-list counts
int launch_bonded64(Box *b);
// Urey-Bradley, torsions, impropers: into ff (FP64 atomics) or the mixed
// path's fixed-point sums (to_fixed); energies to SC_UREY..SC_IMPR
int launch_bonded_ext(Box *b, bool to_fixed, int kinds = 7);  // kinds: 1 urey, 2 torsion, 4 improper
// k_respa.cu (FP64 drop-in): force_short.c, force_long.c, integrate_mts.c
int respa_alloc(Box *b);
int respa_force_short(Box *b);
int respa_force_long(Box *b);
int respa_step(Box *b, double vscal, int nshort, int xrespa);  // xrespa < 0: no thermostat
// k_spme.cu
int spme_setup(Box *b);
int launch_charge_grid64(Box *b);
int launch_pme64(Box *b);  // spread .. gather; fp and SC_FMEAN, SC_ENREC
int launch_pme_gather64(Box *b);  // the gather alone from the convolved grid
// k_integrate.cu
int launch_reduce(Box *b, const double *partials, int nblocks, int nterms, int slot, double scale);
int launch_zero_forces(Box *b);
int launch_apply_pme(Box *b);        // ff += fp - mean
int launch_assemble_energies(Box *b, int with_bonded);
int launch_vv1(Box *b, double vscal);  // half kick, drift, pbc_all
int launch_vv2(Box *b, double vscal);  // half kick, uu = vv
int launch_pbc(Box *b);
int launch_kinet(Box *b);
int launch_vv2_kinet(Box *b, double vscal);  // vv2 with the kinetic tensor folded in
int launch_nhc(Box *b, double time_step);
int launch_record(Box *b);
// batched step, integrator side (every box of a batch per launch)
BIntArgs make_bint_args(Box *b);
void mixed_bint_fields(Box *b, BIntArgs *a);  // k_mixed.cu
unsigned long long *mixed_force_sums(Box *b);  // k_mixed.cu: the fixed-point force sums
// mixed NVE: force finalisation, energy assembly, second half kick, kinet, record
int launch_vv2_mx_tail(Box *b);
int launch_vv1_mx(Box *b, double vscal);  // k_integrate_mx.cu (mixed boxes)
int launch_b_kinet_nhc(const BIntArgs *A, const int *off, int nbox, int blocks, cudaStream_t s);
int launch_b_vv1(const BIntArgs *A, const int *off, int nbox, int blocks, int nhc,
                 cudaStream_t s);
int launch_b_vv2(const BIntArgs *A, const int *off, int nbox, int blocks, int nhc,
                 cudaStream_t s);
int launch_b_scale_kinet(const BIntArgs *A, const int *off, int nbox, int blocks,
                         int chain_next, cudaStream_t s);
// one MD step of the box on its stream (nve_md.c:359-418 / nvt_md.c:529-531)
int step_body(Box *b, bool with_list, bool use_nhc);
// packed xyz (3n doubles) <-> the double4 positions, on the box's stream
int launch_xyz_scatter(Box *b, const double *xyz, bool to_pos, bool to_nopbc);
int launch_xyz_gather(Box *b, double *xyz);
// instrumentation: relaunch one kernel (FE_KERNEL_*) on the current state
int relaunch_kernel(Box *b, int which);
// k_mc.cu
int mc_setup(Box *b, int kmax, int mks, double rc_ew);
int mc_delta(Box *b, int lb, int ub, const double *new_pos_host, double *dE, double *parts);
int mc_terms(Box *b, int lb, int ub, const double *new_pos_host, double *terms6);
int launch_drift(Box *b);
int mc_accept(Box *b);
int mc_kspace_energy(Box *b, double *e);
void mc_free(Box *b);
// k_mcrun.cu
void mcc_free(Box *b);
// k_mlp.cu: train the surrogate on device-resident samples
int mlp_train_device(Mlp *m, const float *data, const float *y, long long n, int epochs, int B,
                     float lr, uint64_t seed, float *loss_hist);
Mlp *mlp_from_handle(fe_mlp *h);

}  // namespace fe

struct fe_box {
  fe::Box b;
};
