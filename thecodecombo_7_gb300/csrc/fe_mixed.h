// fe_mixed.h -- device state of the mixed-precision path (k_mixed.cu).
#pragma once

#include <cuda_runtime.h>
#include <cufft.h>

namespace fe {

struct Box;

struct Mixed {
  int nc[3] = {1, 1, 1};
  double h[3] = {0, 0, 0};
  int ncells = 1;
  int *cell_count = nullptr, *cell_start = nullptr, *cell_fill = nullptr, *cell_of = nullptr;
  int *perm = nullptr;    // sorted slot -> original site
  int *iperm = nullptr;   // original site -> sorted slot
  int *cell_s = nullptr;  // cell assigned to each sorted slot at the last rebuild
  int *type_s = nullptr;  // site type per sorted slot
  float4 *pos32 = nullptr;
  int cap = 0;            // full-list row capacity
  int *count = nullptr, *ent = nullptr;
  unsigned long long *fix = nullptr;  // 3n fixed-point forces (2^32 per kJ/mol/A)
  float *shift_tab = nullptr;         // 343 x (hi xyz, lo xyz)
  float *lj_tab = nullptr;            // nt*nt x (eps, sig^2, shift constant)
  int nexcl = 0;
  int *excl_ab = nullptr, *excl_flag = nullptr;
  float *eterm32 = nullptr, *kw32 = nullptr;
  float *grid32 = nullptr;
  cufftComplex *grid32k = nullptr;
  cufftHandle plan_r2c = 0, plan_c2r = 0;
  bool plans = false;
  int *floor3 = nullptr;
  float *sm = nullptr, *sd = nullptr;
  double erfc_rc_over_rc = 0.0;
};

int mixed_setup(Box *b);
void mixed_free(Box *b);
int launch_mixed_list(Box *b);
int forces_mixed(Box *b);
int launch_mixed_assemble(Box *b);
int launch_mx_pair_only(Box *b);
const int *mixed_counts(Box *b);    // device row counts of the full list    // the pair kernel alone (timing)
int launch_mx_spread_only(Box *b);  // the spreading kernel alone (timing)
void k_cell_scan_ext(const int *count, int ncells, int *start, int *fill, cudaStream_t s);

}  // namespace fe
