// fe_mixed.h -- device state of the mixed-precision path (k_mixed.cu).
#pragma once

#include <cuda_runtime.h>
#include <cufft.h>

#include "fe_df.cuh"

namespace fe {

struct Box;

// Device state of the pair kernel: need (set by a list rebuild), the largest
// squared displacement since the last prune (float bits), a prune count and
// the next row to hand out (zero between launches).
constexpr int kIntraMaxSites = 8;

struct MxPruneState {
  int need;
  unsigned dmax2;
  unsigned long long prunes;
  int next_row;
  int pad;
};

// The topology of a box whose molecules are all alike (same size, terms and
// site types at the same positions, consecutive from site 0): the fused
// intramolecular kernel then reads it from the launch parameters instead of
// following per-molecule index lists.
constexpr int kTplTerms = 16;
struct IntraTpl {
  int ns, nx, nb, na;
  int xa[kTplTerms], xb[kTplTerms], xf[kTplTerms];
  int ba[kTplTerms], bb[kTplTerms];
  float breq[kTplTerms], breq_lo[kTplTerms], bk[kTplTerms];  // r0 as hi + lo floats
  int aa[kTplTerms], ab[kTplTerms], ac[kTplTerms];
  float at0[kTplTerms], at0_lo[kTplTerms], ak[kTplTerms];       // theta0 as hi + lo floats
  int type[kIntraMaxSites];
};

struct Mixed {
  bool uniform = false;  // all molecules alike: tpl holds their topology
  IntraTpl tpl;
  // cell grid (edge >= rlist / 3) used to sort sites and enumerate candidates
  int nc[3] = {1, 1, 1};
  double h[3] = {0, 0, 0};
  int ncells = 1;
  int *cell_count = nullptr, *cell_start = nullptr, *cell_fill = nullptr, *cell_of = nullptr;
  int *perm = nullptr;            // sorted slot -> original site
  int *iperm = nullptr;           // original site -> sorted slot
  int *cell_s = nullptr;          // cell of each sorted slot at the last rebuild
  int *type_s = nullptr;          // site type per sorted slot
  int4 *posfx = nullptr;          // sorted x, y, z as 32-bit fractions of L; w = bits of (float)q
  // outer list (rlist, rebuilt every nlist steps) and inner list (rc + skin,
  // rewritten by the pair kernel when it prunes); rows hold LJ pairs at the
  // front and the rest at the back, entries are sorted-slot indices
  int cap = 0;
  int *cnt_lj = nullptr, *cnt_nl = nullptr, *ent = nullptr;
  int *icnt_lj = nullptr, *icnt_nl = nullptr, *ient = nullptr;
  double skin = 0.8;              // inner list radius = rc + skin
  bool inner_on = false;          // rc + skin < rlist: the inner list is used
  int4 *snap = nullptr;           // posfx at the last prune
  MxPruneState *ps = nullptr;
  unsigned long long *fix = nullptr;  // 3n fixed-point forces (2^32 per kJ/mol/A)
  // the reciprocal-space branch runs on its own stream beside the pair
  // kernel, with its own last-block reduction slots
  cudaStream_t s2 = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  unsigned long long *facc2 = nullptr;
  unsigned *ticket2 = nullptr;
  float *lj_tab = nullptr;        // nt*nt x (eps, sig^2, shift constant)
  unsigned char *lj_on = nullptr; // nt*nt: pair type has an LJ term
  unsigned *lj_row = nullptr;     // nt <= 32: bit t of lj_row[t'] = lj_on[t][t']
  int nexcl = 0;
  int *excl_ab = nullptr, *excl_flag = nullptr;
  float *eterm32 = nullptr, *kw32 = nullptr;
  float *grid32 = nullptr;
  cufftComplex *grid32k = nullptr;
  cufftHandle plan_r2c = 0, plan_c2r = 0;
  bool plans = false;
  int *floor3 = nullptr;
  unsigned long long *gfix = nullptr;  // K fixed-point grid sums (2^40 per unit), kept zeroed
  float *sm = nullptr, *sd = nullptr;
  double erfc_rc_over_rc = 0.0;
  // pair kernel launch shape (mixed_autotune): warps per block, grid (0: one warp per row)
  int tune_nw = 8;
  int tune_rw = 48;     // resident warps per SM the register budget is sized for
  int tune_blocks = 0;
  int nsm = 152;                  // SMs of the box's device
  // Molecules for the fused intramolecular kernel: every bonded and excluded
  // pair lies inside a contiguous run of at most kIntraMaxSites sites.
  // nmol == 0: the topology does not allow it (separate kernels are used).
  int nmol = 0;
  int intra_maxs = kIntraMaxSites;  // sites of the largest molecule
  int *mol_first = nullptr;                    // nmol + 1
  int *mol_x = nullptr, *mol_xi = nullptr;     // CSR: exclusion indices per molecule
  int *mol_b = nullptr, *mol_bi = nullptr;     // bond indices
  int *mol_a = nullptr, *mol_ai = nullptr;     // bend indices
  // double-float intramolecular correction energy: exp(k/64) table, constants
  float2 *exptab = nullptr;
  DfIntra dfi{};
};


int mixed_setup(Box *b);
void mixed_free(Box *b);
int launch_mixed_list(Box *b);      // sort + outer list
int forces_mixed(Box *b);
int launch_mixed_assemble(Box *b);
// the pair kernel alone (inner list unless a rebuild or a displacement asks
// for a prune)
int launch_mx_pair_only(Box *b);
int launch_mx_spread_only(Box *b);  // the spreading kernel alone (timing)
int mixed_autotune(Box *b, int *nw, int *rw, int *blocks, double *us);
void mixed_counts(Box *b, const int **lj, const int **rest);  // device row counts (outer)
void mixed_inner_counts(Box *b, const int **lj, const int **rest, bool *on);
MxPruneState *mixed_prune_state(Box *b);
void k_cell_scan_ext(const int *count, int ncells, int *start, int *fill, cudaStream_t s);
// replica batches: the force evaluation of every box in one launch per kernel
struct BMxPlan;
int mixed_batch_plan(Box *const *boxes, int nbox, BMxPlan **out);
int mixed_batch_forces(BMxPlan *plan, cudaStream_t s);
int mixed_batch_list(BMxPlan *plan, cudaStream_t s);
void mixed_batch_free(BMxPlan *plan);

}  // namespace fe
