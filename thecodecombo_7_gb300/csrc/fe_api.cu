// fe_api.cu -- the C ABI of libfe.so (include/fe.h): box lifetime, host <->
// device transfers in the reference's layouts, and the drivers that chain the
// kernels in the order of the reference's routines.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "fe_internal.h"
#include "fe_mixed.h"

namespace fe {

static thread_local std::string g_err;
thread_local long g_launches = 0;

void set_error(const std::string &msg) { g_err = msg; }

int cuda_fail(cudaError_t e, const char *what) {
  set_error(std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e));
  return FE_ERR_CUDA;
}

int cufft_fail(cufftResult r, const char *what) {
  set_error(std::string("cuFFT error ") + std::to_string((int)r) + " in " + what);
  return FE_ERR_CUDA;
}

// the error behind a device status word st (zero: none); clears the word
static int status_error(Box *b, int st) {
  if (st == 0) return FE_OK;
  FE_CUDA(cudaMemsetAsync(b->status, 0, sizeof(int), b->stream));
  std::string m = "device status:";
  if (st & ST_LIST_OVERFLOW)
    m += " neighbour-list row over capacity (increase max_neighbors or check the density);";
  if (st & ST_CELL_OVERFLOW) m += " cell bin over capacity;";
  if (st & ST_PBC_LOOP) m += " periodic wrap did not converge (non-finite or runaway position);";
  if (st & ST_GRID_OVERFLOW) m += " SPME bin over capacity;";
  if (st & ST_BAD_INDEX) m += " index out of range skipped;";
  set_error(m);
  if (st & ST_LIST_OVERFLOW) return FE_ERR_OVERFLOW;
  return FE_ERR_DEVICE;
}

int check_status(Box *b) {
  int st = 0;
  FE_CUDA(cudaMemcpyAsync(&st, b->status, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  FE_CUDA(cudaStreamSynchronize(b->stream));
  return status_error(b, st);
}

template <class T>
static int upload(T **dst, const T *src, size_t count) {
  FE_CUDA(cudaMalloc(dst, sizeof(T) * (count ? count : 1)));
  if (count) FE_CUDA(cudaMemcpy(*dst, src, sizeof(T) * count, cudaMemcpyHostToDevice));
  return FE_OK;
}

// scalars and the status word to the host with one synchronisation
static int sync_scal(Box *b) {
  int st = 0;
  FE_CUDA(cudaMemcpyAsync(b->host_scal, b->scal, sizeof(double) * SC_COUNT, cudaMemcpyDeviceToHost,
                          b->stream));
  FE_CUDA(cudaMemcpyAsync(&st, b->status, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  FE_CUDA(cudaStreamSynchronize(b->stream));
  return status_error(b, st);
}

// the list, then the snapshot nl_check compares against (nblist.c:583-591)
static int launch_list(Box *b) {
  int rc = b->mx ? launch_mixed_list(b) : launch_nblist(b);
  if (rc) return rc;
  FE_CUDA(cudaMemcpyAsync(b->pos_list0, b->pos_q, sizeof(double4) * b->n,
                          cudaMemcpyDeviceToDevice, b->stream));
  return FE_OK;
}

// forces() on the device, forces.c:118-219
static int forces_device(Box *b) {
  if (!b->have_list) {
    set_error("forces requested before a neighbour list was built (call nblist first)");
    return FE_ERR_STATE;
  }
  if (b->mx) return forces_mixed(b);
  int rc;
  if ((rc = launch_zero_forces(b))) return rc;
  if ((rc = launch_bonded64(b))) return rc;
  if ((rc = launch_bonded_ext(b, false))) return rc;
  if ((rc = launch_pair64(b))) return rc;
  if ((rc = launch_pme64(b))) return rc;
  if ((rc = launch_apply_pme(b))) return rc;
  return launch_assemble_energies(b, 1);
}

static void free_box(Box *b) {
  void *ptrs[] = {b->pos_q, b->pos_nopbc, b->pos_list0, b->nl_dev, b->vv, b->uu, b->ff, b->mass, b->imass100, b->type, b->lj_eps,
                  b->lj_sig, b->x_start, b->x_partner, b->x_flag, b->bond_ab, b->bend_abc,
                  b->bond_req, b->bond_k, b->bend_t0, b->bend_k, b->cell_count, b->cell_start,
                  b->cell_fill, b->cell_atoms, b->cell_of, b->nl_count, b->nl_ent, b->eterm,
                  b->kweight, b->grid, b->grid_k, b->spl_floor, b->spl_m, b->spl_d, b->fp,
                  b->gbin_count, b->gbin_atoms, b->partials, b->scal, b->status, b->ticket, b->facc, b->xyz_dev, b->zeta, b->rec,
                  b->rec_counter, b->urey_ab, b->urey_seq, b->urey_k, b->tors_abcd, b->tors_par,
                  b->tors_tau, b->impr_abcd, b->impr_k, b->impr_eq, b->ff_short, b->ff_long};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  mc_free(b);
  mcc_free(b);
  mixed_free(b);
  if (b->host_scal) cudaFreeHost(b->host_scal);
  if (b->stage) cudaFreeHost(b->stage);
  if (b->plans) {
    cufftDestroy(b->plan_r2c);
    cufftDestroy(b->plan_c2r);
  }
  if (b->g_step) cudaGraphExecDestroy(b->g_step);
  if (b->g_step_list) cudaGraphExecDestroy(b->g_step_list);
  if (b->own_stream && b->stream) cudaStreamDestroy(b->stream);
  if (b->g_io) cudaGraphExecDestroy(b->g_io);
  if (b->s_io) cudaStreamDestroy(b->s_io);
  if (b->ev_io_pos) cudaEventDestroy(b->ev_io_pos);
  if (b->ev_io_done) cudaEventDestroy(b->ev_io_done);
}

static int create(Box *b, const fe_box_params *p) {
  b->p = *p;
  b->n = p->n;
  b->nt = p->ntypes;
  b->dev = p->device;
  b->prec = p->precision;
  if (p->n < 2 || p->ntypes < 1 || !p->q || !p->mass || !p->type || !p->lj_eps || !p->lj_sig) {
    set_error("fe_box_create: n >= 2, ntypes >= 1 and q/mass/type/lj tables are required");
    return FE_ERR_ARG;
  }
  if (p->order < 3 || p->order > 8) {
    set_error("fe_box_create: SPME order must be in 3..8");
    return FE_ERR_ARG;
  }
  for (int d = 0; d < 3; d++)
    if (p->grid[d] < p->order || p->L[d] <= 0.0) {
      set_error("fe_box_create: grid must be >= order and box lengths positive");
      return FE_ERR_ARG;
    }
  if (p->rc <= 0.0 || p->rclist < p->rc || p->kappa <= 0.0 || p->epsRF == 0.0) {
    set_error("fe_box_create: need rc > 0, rclist >= rc, kappa > 0, epsRF != 0");
    return FE_ERR_ARG;
  }
  if (p->precision != FE_PREC_FP64 && p->precision != FE_PREC_MIXED) {
    set_error("fe_box_create: unknown precision");
    return FE_ERR_ARG;
  }
  for (int i = 0; i < p->n; i++)
    if (p->type[i] < 0 || p->type[i] >= p->ntypes) {
      set_error("fe_box_create: site type out of range");
      return FE_ERR_ARG;
    }
  // ewald.c:185-194 neutrality (summed in site order)
  double charge = 0.0;
  for (int i = 0; i < p->n; i++) charge += p->q[i];
  if (fabs(charge) > 0.000005) {
    char m[160];
    snprintf(m, sizeof m,
             "The charge of the system is %f; Ewald summation needs a neutral system", charge);
    set_error(m);
    return FE_ERR_CHARGE;
  }
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    set_error(std::string("no CUDA device available: ") +
              (e != cudaSuccess ? cudaGetErrorString(e) : "0 devices"));
    return FE_ERR_CUDA;
  }
  FE_CUDA(cudaSetDevice(p->device));
  FE_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  b->own_stream = true;
  int n = p->n;
  std::vector<double4> pq(n);
  for (int i = 0; i < n; i++) pq[i] = make_double4(0.0, 0.0, 0.0, p->q[i]);
  int rc;
  if ((rc = upload(&b->pos_q, pq.data(), n))) return rc;
  FE_CUDA(cudaMalloc(&b->pos_nopbc, sizeof(double) * 3 * n));
  FE_CUDA(cudaMalloc(&b->pos_list0, sizeof(double4) * n));
  FE_CUDA(cudaMalloc(&b->nl_dev, sizeof(int)));
  FE_CUDA(cudaMalloc(&b->vv, sizeof(double) * 3 * n));
  FE_CUDA(cudaMalloc(&b->uu, sizeof(double) * 3 * n));
  FE_CUDA(cudaMalloc(&b->ff, sizeof(double) * 3 * n));
  FE_CUDA(cudaMemset(b->pos_nopbc, 0, sizeof(double) * 3 * n));
  FE_CUDA(cudaMemset(b->vv, 0, sizeof(double) * 3 * n));
  FE_CUDA(cudaMemset(b->uu, 0, sizeof(double) * 3 * n));
  FE_CUDA(cudaMemset(b->ff, 0, sizeof(double) * 3 * n));
  if ((rc = upload(&b->mass, p->mass, n))) return rc;
  {
    std::vector<double> im(n);
    for (int i = 0; i < n; i++) im[i] = 100.0 / p->mass[i];
    if ((rc = upload(&b->imass100, im.data(), n))) return rc;
  }
  if ((rc = upload(&b->type, p->type, n))) return rc;
  size_t nt2 = (size_t)p->ntypes * p->ntypes;
  if ((rc = upload(&b->lj_eps, p->lj_eps, nt2))) return rc;
  if ((rc = upload(&b->lj_sig, p->lj_sig, nt2))) return rc;
  // exclusions: per site, both directions, xint order kept
  b->nexcl = p->nexcl;
  std::vector<int> xs(n + 1, 0), xp(2 * (size_t)p->nexcl + 1), xf(2 * (size_t)p->nexcl + 1);
  for (int i = 0; i < p->nexcl; i++) {
    int a = p->excl_ab[2 * i], c = p->excl_ab[2 * i + 1];
    if (a < 0 || a >= n || c < 0 || c >= n) {
      set_error("fe_box_create: exclusion index out of range");
      return FE_ERR_ARG;
    }
    xs[a + 1]++;
    xs[c + 1]++;
  }
  for (int i = 0; i < n; i++) xs[i + 1] += xs[i];
  std::vector<int> fill(n, 0);
  for (int i = 0; i < p->nexcl; i++) {
    int a = p->excl_ab[2 * i], c = p->excl_ab[2 * i + 1];
    int pa = xs[a] + fill[a]++;
    xp[pa] = c;
    xf[pa] = p->excl_flag[i];
    int pc = xs[c] + fill[c]++;
    xp[pc] = a;
    xf[pc] = p->excl_flag[i];
  }
  if ((rc = upload(&b->x_start, xs.data(), xs.size()))) return rc;
  if ((rc = upload(&b->x_partner, xp.data(), xp.size()))) return rc;
  if ((rc = upload(&b->x_flag, xf.data(), xf.size()))) return rc;
  // bonded
  b->nbond = p->nbond;
  b->nbend = p->nbend;
  for (int i = 0; i < 2 * p->nbond; i++)
    if (p->bond_ab[i] < 0 || p->bond_ab[i] >= n) {
      set_error("fe_box_create: bond index out of range");
      return FE_ERR_ARG;
    }
  for (int i = 0; i < 3 * p->nbend; i++)
    if (p->bend_abc[i] < 0 || p->bend_abc[i] >= n) {
      set_error("fe_box_create: bend index out of range");
      return FE_ERR_ARG;
    }
  if ((rc = upload(&b->bond_ab, p->bond_ab, 2 * (size_t)p->nbond))) return rc;
  if ((rc = upload(&b->bond_req, p->bond_req, (size_t)p->nbond))) return rc;
  if ((rc = upload(&b->bond_k, p->bond_k, (size_t)p->nbond))) return rc;
  if ((rc = upload(&b->bend_abc, p->bend_abc, 3 * (size_t)p->nbend))) return rc;
  if ((rc = upload(&b->bend_t0, p->bend_theta0, (size_t)p->nbend))) return rc;
  if ((rc = upload(&b->bend_k, p->bend_k, (size_t)p->nbend))) return rc;
  // scalars, status
  FE_CUDA(cudaMalloc(&b->partials, sizeof(double) * kMaxPartialBlocks * kPartialTerms));
  FE_CUDA(cudaMalloc(&b->scal, sizeof(double) * SC_COUNT));
  FE_CUDA(cudaMemset(b->scal, 0, sizeof(double) * SC_COUNT));
  FE_CUDA(cudaMemcpy(b->scal + SC_TEMP, &p->T, sizeof(double), cudaMemcpyHostToDevice));
  FE_CUDA(cudaMalloc(&b->status, sizeof(int)));
  FE_CUDA(cudaMemset(b->status, 0, sizeof(int)));
  FE_CUDA(cudaMalloc(&b->facc, sizeof(unsigned long long) * kFaccSlots));
  FE_CUDA(cudaMemset(b->facc, 0, sizeof(unsigned long long) * kFaccSlots));
  FE_CUDA(cudaMalloc(&b->ticket, sizeof(unsigned)));
  FE_CUDA(cudaMemset(b->ticket, 0, sizeof(unsigned)));
  FE_CUDA(cudaMallocHost(&b->host_scal, sizeof(double) * SC_COUNT));
  FE_CUDA(cudaMallocHost(&b->stage, sizeof(double) * 4 * (size_t)n));
  FE_CUDA(cudaMalloc(&b->xyz_dev, sizeof(double) * 3 * (size_t)n));
  FE_CUDA(cudaMalloc(&b->rec_counter, sizeof(int)));
  // self energy, ewald.c:61,172-178
  double fconv = (kELEC * kELEQ * kELEQ * kNA * 0.001) / p->epsRF;
  double vs = 0.0;
  for (int i = 0; i < n; i++) vs += p->q[i] * p->q[i];
  vs *= p->kappa / sqrt(kPI);
  b->sewald = vs * fconv;
  // NHC state, read_config.c:358-370
  b->nhc_M = p->nhc_M > 0 ? p->nhc_M : 1;
  b->nhc_Q = p->nhc_Q != 0.0 ? p->nhc_Q : 1.0e-18;
  b->nfree = p->nfree > 0.0 ? p->nfree : 3.0 * n - 3.0;
  std::vector<double> z(3 * b->nhc_M, 0.0);
  double kT = kKB * p->T * 1E-4;
  for (int i = 0; i < b->nhc_M - 1; i++)
    z[3 * (i + 1) + 2] = (b->nhc_Q * z[3 * i + 1] * z[3 * i + 1] - kT) / b->nhc_Q;
  if ((rc = upload(&b->zeta, z.data(), z.size()))) return rc;
  if ((rc = nblist_setup(b))) return rc;
  if ((rc = spme_setup(b))) return rc;
  if (p->precision == FE_PREC_MIXED) {
    b->mx = new Mixed();
    double kr = p->kappa * p->rc, z = fabs(kr), t = 1.0 / (1.0 + 0.5 * z);
    double v = t * exp(-z * z + -1.26551223 +
                       t * (1.00002368 + t * (0.37409196 + t * (0.09678418 +
                       t * (-0.18628806 + t * (0.27886807 + t * (-1.13520398 +
                       t * (1.48851587 + t * (-0.82215223 + t * 0.17087277)))))))));
    b->mx->erfc_rc_over_rc = v / p->rc;  // ewald.c:817-836 at kappa*rc
    if ((rc = mixed_setup(b))) return rc;
  }
  FE_CUDA(cudaDeviceSynchronize());
  return FE_OK;
}

// Host <-> device transfer of x, y, z from `struct atoms`-like records.  A
// contiguous xyz array (stride 24, offset 0) in page-locked memory is copied
// by DMA as it is; anything else is packed through the box's pinned staging
// buffer.  One linear copy either way; the double4 layout is handled by a
// kernel on the device.
static bool pinned_host(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

static int xyz_to_device(Box *b, const void *atoms, size_t stride, size_t off, double *dst) {
  if (!atoms || stride < 24) {
    set_error("positions: null pointer or stride < 24");
    return FE_ERR_ARG;
  }
  size_t bytes = sizeof(double) * 3 * (size_t)b->n;
  const char *base = (const char *)atoms + off;
  const void *src = base;
  if (!(stride == 24 && pinned_host(base))) {
    double *st = b->stage;
    if (stride == 24) memcpy(st, base, bytes);
    else
      for (int i = 0; i < b->n; i++) memcpy(st + 3 * (size_t)i, base + (size_t)i * stride, 24);
    src = st;
  }
  FE_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, b->stream));
  return FE_OK;
}

static int xyz_to_host(Box *b, const double *src, void *atoms, size_t stride, size_t off) {
  if (!atoms || stride < 24) {
    set_error("positions: null pointer or stride < 24");
    return FE_ERR_ARG;
  }
  size_t bytes = sizeof(double) * 3 * (size_t)b->n;
  char *base = (char *)atoms + off;
  bool direct = stride == 24 && pinned_host(base);
  FE_CUDA(cudaMemcpyAsync(direct ? (void *)base : (void *)b->stage, src, bytes,
                          cudaMemcpyDeviceToHost, b->stream));
  FE_CUDA(cudaStreamSynchronize(b->stream));
  if (!direct) {
    const double *st = b->stage;
    if (stride == 24) memcpy(base, st, bytes);
    else
      for (int i = 0; i < b->n; i++) memcpy(base + (size_t)i * stride, st + 3 * (size_t)i, 24);
  }
  return FE_OK;
}

// one step of the production loop (graph body)
int step_body(Box *b, bool with_list, bool use_nhc) {
  int rc;
  if (with_list && (rc = launch_list(b))) return rc;
  if (use_nhc && (rc = launch_nhc(b, b->p.dt))) return rc;
  if ((rc = launch_vv1(b, 1.0))) return rc;
  // mixed NVE: the force finalisation, the energy assembly, the second half
  // kick, kinet and the record in one launch
  const bool tail = b->mx != nullptr && !use_nhc;
  b->fold_tail = tail;
  rc = forces_device(b);
  b->fold_tail = false;
  if (rc) return rc;
  if (tail) return launch_vv2_mx_tail(b);
  if (use_nhc) {
    if ((rc = launch_vv2(b, 1.0))) return rc;
    if ((rc = launch_nhc(b, b->p.dt))) return rc;
    if ((rc = launch_kinet(b))) return rc;
  } else {
    // kinet of the fresh velocities folded into the second half kick
    if ((rc = launch_vv2_kinet(b, 1.0))) return rc;
  }
  return launch_record(b);
}

int relaunch_kernel(Box *b, int which) {
  if (b->mx) {
    if (which == FE_KERNEL_PAIR) return launch_mx_pair_only(b);
    if (which == FE_KERNEL_SPREAD) return launch_mx_spread_only(b);
    if (which == FE_KERNEL_LIST) return launch_mixed_list(b);
  } else {
    if (which == FE_KERNEL_PAIR) return launch_pair64(b);
    if (which == FE_KERNEL_SPREAD) return launch_charge_grid64(b);
    if (which == FE_KERNEL_LIST) return launch_nblist(b);
  }
  set_error("fe_time_kernel: unknown kernel id");
  return FE_ERR_ARG;
}

static void drop_io_graph(Box *b) {
  if (b->g_io) cudaGraphExecDestroy(b->g_io);
  b->g_io = nullptr;
}

static int capture(Box *b, bool with_list, bool use_nhc, cudaGraphExec_t *out) {
  cudaGraph_t g;
  FE_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  long l0 = g_launches;
  int rc = step_body(b, with_list, use_nhc);
  int nl = (int)(g_launches - l0);
  if (with_list) b->launches_list = nl;
  else b->launches_plain = nl;
  cudaError_t e = cudaStreamEndCapture(b->stream, &g);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
  return FE_OK;
}

}  // namespace fe

using namespace fe;

extern "C" {

int fe_abi_version(void) { return FE_ABI_VERSION; }

const char *fe_last_error(void) { return g_err.c_str(); }

int fe_box_create(fe_box **out, const fe_box_params *p) {
  if (!out || !p) {
    set_error("fe_box_create: null argument");
    return FE_ERR_ARG;
  }
  *out = nullptr;
  fe_box *fb = new fe_box();
  int rc = create(&fb->b, p);
  if (rc) {
    free_box(&fb->b);
    delete fb;
    return rc;
  }
  *out = fb;
  return FE_OK;
}

void fe_box_destroy(fe_box *box) {
  if (!box) return;
  cudaSetDevice(box->b.dev);
  cudaStreamSynchronize(box->b.stream);
  free_box(&box->b);
  delete box;
}

int fe_box_set_stream(fe_box *box, void *stream) {
  if (!box) return FE_ERR_ARG;
  Box *b = &box->b;
  FE_CUDA(cudaStreamSynchronize(b->stream));
  if (b->own_stream) cudaStreamDestroy(b->stream);
  if (stream) {
    b->stream = (cudaStream_t)stream;
    b->own_stream = false;
  } else {
    FE_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    b->own_stream = true;
  }
  if (b->g_step) cudaGraphExecDestroy(b->g_step);
  if (b->g_step_list) cudaGraphExecDestroy(b->g_step_list);
  b->g_step = b->g_step_list = nullptr;
  b->g_key = -1;
  drop_io_graph(b);
  return FE_OK;
}

int fe_set_positions(fe_box *box, const void *atoms, size_t stride, size_t off_x, int nopbc) {
  if (!box) return FE_ERR_ARG;
  Box *b = &box->b;
  int rc = xyz_to_device(b, atoms, stride, off_x, b->xyz_dev);
  if (rc) return rc;
  if ((rc = launch_xyz_scatter(b, b->xyz_dev, true, nopbc != 0))) return rc;
  FE_CUDA(cudaStreamSynchronize(b->stream));
  return FE_OK;
}

int fe_get_positions(fe_box *box, void *atoms, size_t stride, size_t off_x) {
  if (!box) return FE_ERR_ARG;
  Box *b = &box->b;
  int rc = launch_xyz_gather(b, b->xyz_dev);
  if (rc) return rc;
  return xyz_to_host(b, b->xyz_dev, atoms, stride, off_x);
}

int fe_set_positions_nopbc(fe_box *box, const void *atoms, size_t stride, size_t off_x) {
  if (!box) return FE_ERR_ARG;
  Box *b = &box->b;
  int rc = xyz_to_device(b, atoms, stride, off_x, b->pos_nopbc);
  if (rc) return rc;
  FE_CUDA(cudaStreamSynchronize(b->stream));
  return FE_OK;
}

int fe_get_positions_nopbc(fe_box *box, void *atoms, size_t stride, size_t off_x) {
  if (!box) return FE_ERR_ARG;
  return xyz_to_host(&box->b, box->b.pos_nopbc, atoms, stride, off_x);
}

int fe_set_velocities(fe_box *box, const double *vv, const double *uu) {
  if (!box || !vv) return FE_ERR_ARG;
  Box *b = &box->b;
  size_t bytes = sizeof(double) * 3 * b->n;
  FE_CUDA(cudaMemcpyAsync(b->vv, vv, bytes, cudaMemcpyHostToDevice, b->stream));
  FE_CUDA(cudaMemcpyAsync(b->uu, uu ? uu : vv, bytes, cudaMemcpyHostToDevice, b->stream));
  FE_CUDA(cudaStreamSynchronize(b->stream));
  return FE_OK;
}

int fe_get_velocities(fe_box *box, double *vv, double *uu) {
  if (!box) return FE_ERR_ARG;
  Box *b = &box->b;
  size_t bytes = sizeof(double) * 3 * b->n;
  if (vv) FE_CUDA(cudaMemcpyAsync(vv, b->vv, bytes, cudaMemcpyDeviceToHost, b->stream));
  if (uu) FE_CUDA(cudaMemcpyAsync(uu, b->uu, bytes, cudaMemcpyDeviceToHost, b->stream));
  FE_CUDA(cudaStreamSynchronize(b->stream));
  return FE_OK;
}

int fe_get_forces(fe_box *box, double *ff) {
  if (!box || !ff) return FE_ERR_ARG;
  Box *b = &box->b;
  FE_CUDA(cudaMemcpyAsync(ff, b->ff, sizeof(double) * 3 * b->n, cudaMemcpyDeviceToHost, b->stream));
  FE_CUDA(cudaStreamSynchronize(b->stream));
  return FE_OK;
}

int fe_set_forces(fe_box *box, const double *ff) {
  if (!box || !ff) return FE_ERR_ARG;
  Box *b = &box->b;
  FE_CUDA(cudaMemcpyAsync(b->ff, ff, sizeof(double) * 3 * b->n, cudaMemcpyHostToDevice, b->stream));
  FE_CUDA(cudaStreamSynchronize(b->stream));
  return FE_OK;
}

int fe_set_nhc_state(fe_box *box, const double *zeta) {
  if (!box || !zeta) return FE_ERR_ARG;
  Box *b = &box->b;
  FE_CUDA(cudaMemcpyAsync(b->zeta, zeta, sizeof(double) * 3 * b->nhc_M, cudaMemcpyHostToDevice,
                          b->stream));
  FE_CUDA(cudaStreamSynchronize(b->stream));
  return FE_OK;
}

int fe_get_nhc_state(fe_box *box, double *zeta) {
  if (!box || !zeta) return FE_ERR_ARG;
  Box *b = &box->b;
  FE_CUDA(cudaMemcpyAsync(zeta, b->zeta, sizeof(double) * 3 * b->nhc_M, cudaMemcpyDeviceToHost,
                          b->stream));
  FE_CUDA(cudaStreamSynchronize(b->stream));
  return FE_OK;
}

int fe_nblist(fe_box *box) {
  if (!box) return FE_ERR_ARG;
  int rc = launch_list(&box->b);
  if (rc) return rc;
  return check_status(&box->b);
}

int fe_nblist_download(fe_box *box, int *count, int *idx, int *flag, int64_t cap, int64_t *total) {
  if (!box || !count) return FE_ERR_ARG;
  Box *b = &box->b;
  if (!b->have_list || b->mx) {
    set_error(b->mx ? "list download is available for the FP64 drop-in list only"
                    : "no neighbour list built yet");
    return FE_ERR_STATE;
  }
  std::vector<int> ent((size_t)b->n * b->max_nb);
  FE_CUDA(cudaMemcpyAsync(count, b->nl_count, sizeof(int) * b->n, cudaMemcpyDeviceToHost, b->stream));
  FE_CUDA(cudaMemcpyAsync(ent.data(), b->nl_ent, sizeof(int) * ent.size(), cudaMemcpyDeviceToHost,
                          b->stream));
  FE_CUDA(cudaStreamSynchronize(b->stream));
  int64_t tot = 0;
  for (int i = 0; i < b->n; i++) tot += count[i];
  if (total) *total = tot;
  if (tot > cap || !idx) {
    set_error("fe_nblist_download: capacity too small");
    return idx ? FE_ERR_SIZE : FE_OK;
  }
  int64_t p = 0;
  for (int i = 0; i < b->n; i++)
    for (int j = 0; j < count[i]; j++) {
      int e = ent[(size_t)i * b->max_nb + j];
      idx[p] = e >> 3;
      if (flag) flag[p] = e & 7;
      p++;
    }
  return FE_OK;
}

int fe_zero_forces(fe_box *box) {
  if (!box) return FE_ERR_ARG;
  int rc = launch_zero_forces(&box->b);
  if (rc) return rc;
  FE_CUDA(cudaStreamSynchronize(box->b.stream));
  return FE_OK;
}

int fe_forces(fe_box *box, double *en) {
  if (!box) return FE_ERR_ARG;
  Box *b = &box->b;
  int rc = forces_device(b);
  if (rc) return rc;
  if ((rc = sync_scal(b))) return rc;
  if (en)
    for (int i = 0; i < FE_EN_COUNT; i++) en[i] = b->host_scal[i];
  return FE_OK;
}

int fe_cnonbondnl(fe_box *box, double *energy8) {
  if (!box) return FE_ERR_ARG;
  Box *b = &box->b;
  if (!b->have_list) {
    set_error("cnonbondnl requested before a neighbour list was built");
    return FE_ERR_STATE;
  }
  if (b->mx) {
    set_error("fe_cnonbondnl is the FP64 drop-in entry; the mixed path evaluates fe_forces");
    return FE_ERR_STATE;
  }
  int rc;
  if ((rc = launch_pair64(b))) return rc;
  if ((rc = launch_pme64(b))) return rc;
  if ((rc = launch_apply_pme(b))) return rc;
  if ((rc = launch_assemble_energies(b, 0))) return rc;
  if ((rc = sync_scal(b))) return rc;
  if (energy8)
    for (int i = 0; i < 8; i++) energy8[i] = b->host_scal[SC_ENERGY8 + i];
  return FE_OK;
}

int fe_pme_calc(fe_box *box, double *energy3) {
  if (!box) return FE_ERR_ARG;
  Box *b = &box->b;
  if (b->mx) {
    set_error("fe_pme_calc is the FP64 drop-in entry; the mixed path evaluates fe_forces");
    return FE_ERR_STATE;
  }
  int rc;
  if ((rc = launch_pme64(b))) return rc;
  if ((rc = launch_apply_pme(b))) return rc;
  if ((rc = launch_assemble_energies(b, 0))) return rc;
  if ((rc = sync_scal(b))) return rc;
  if (energy3)
    for (int i = 0; i < 3; i++) energy3[i] = b->host_scal[SC_ENERGY3 + i];
  return FE_OK;
}

int fe_box_set_lj_form(fe_box *box, int form) {
  if (!box || (form != 0 && form != 2)) {
    set_error("fe_box_set_lj_form: form is 0 (CHARMM) or 2 (BGO)");
    return FE_ERR_ARG;
  }
  Box *b = &box->b;
  if (form == 2 && (b->mx || b->p.r_switch > 0.0)) {
    set_error("fe_box_set_lj_form: the BGO form is the FP64 drop-in's, without the LJ switch");
    return FE_ERR_STATE;
  }
  b->lj_form = form;
  b->g_key = -1;  // step graphs are recaptured
  drop_io_graph(b);
  return FE_OK;
}

int fe_pme_force(fe_box *box) {
  if (!box) return FE_ERR_ARG;
  Box *b = &box->b;
  if (b->mx) {
    set_error("fe_pme_force is the FP64 drop-in entry; the mixed path evaluates fe_forces");
    return FE_ERR_STATE;
  }
  int rc;
  if ((rc = launch_pme_gather64(b))) return rc;
  if ((rc = launch_apply_pme(b))) return rc;
  return check_status(b);
}

int fe_charge_grid(fe_box *box) {
  if (!box) return FE_ERR_ARG;
  int rc = launch_charge_grid64(&box->b);
  if (rc) return rc;
  return check_status(&box->b);
}

int fe_get_charge_grid(fe_box *box, double *grid) {
  if (!box || !grid) return FE_ERR_ARG;
  Box *b = &box->b;
  FE_CUDA(cudaMemcpyAsync(grid, b->grid, sizeof(double) * b->K, cudaMemcpyDeviceToHost, b->stream));
  FE_CUDA(cudaStreamSynchronize(b->stream));
  return FE_OK;
}

int fe_bonded(fe_box *box, double *en2) {
  if (!box) return FE_ERR_ARG;
  Box *b = &box->b;
  int rc = launch_bonded64(b);
  if (rc) return rc;
  if ((rc = sync_scal(b))) return rc;
  if (en2) {
    en2[0] = b->host_scal[SC_BOND];
    en2[1] = b->host_scal[SC_BEND];
  }
  return FE_OK;
}

// the step graphs were captured without the changed terms: recapture
static void drop_step_graphs(Box *b) {
  if (b->g_step) cudaGraphExecDestroy(b->g_step);
  if (b->g_step_list) cudaGraphExecDestroy(b->g_step_list);
  b->g_step = b->g_step_list = nullptr;
  b->g_key = -1;
  drop_io_graph(b);
}

static bool sites_in_range(const int *idx, size_t count, int n) {
  for (size_t i = 0; i < count; i++)
    if (idx[i] < 0 || idx[i] >= n) return false;
  return true;
}

static int replace_bytes(Box *b, void **dst, const void *src, size_t bytes) {
  if (*dst) {
    FE_CUDA(cudaStreamSynchronize(b->stream));
    cudaFree(*dst);
    *dst = nullptr;
  }
  if (bytes == 0) return FE_OK;
  FE_CUDA(cudaMalloc(dst, bytes));
  FE_CUDA(cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice));
  return FE_OK;
}
#define replace_array(b, dst, src, count) \
  replace_bytes((b), (void **)(dst), (const void *)(src), sizeof(**(dst)) * (count))

int fe_set_ureys(fe_box *box, int n, const int *ab, const double *seq, const double *k) {
  if (!box || n < 0 || (n > 0 && (!ab || !seq || !k))) return FE_ERR_ARG;
  Box *b = &box->b;
  if (!sites_in_range(ab, 2 * (size_t)n, b->n)) {
    set_error("fe_set_ureys: site index outside the box");
    return FE_ERR_ARG;
  }
  int rc;
  if ((rc = replace_array(b, &b->urey_ab, ab, 2 * (size_t)n))) return rc;
  if ((rc = replace_array(b, &b->urey_seq, seq, (size_t)n))) return rc;
  if ((rc = replace_array(b, &b->urey_k, k, (size_t)n))) return rc;
  b->nurey = n;
  drop_step_graphs(b);
  return FE_OK;
}

int fe_set_torsions(fe_box *box, int n, const int *abcd, const double *kphi,
                    const double *nphi, const double *delphi) {
  if (!box || n < 0 || (n > 0 && (!abcd || !kphi || !nphi || !delphi))) return FE_ERR_ARG;
  Box *b = &box->b;
  if (!sites_in_range(abcd, 4 * (size_t)n, b->n)) {
    set_error("fe_set_torsions: site index outside the box");
    return FE_ERR_ARG;
  }
  std::vector<double> par(18 * (size_t)n);
  for (int i = 0; i < n; i++)
    for (int t = 0; t < 6; t++) {
      par[18 * (size_t)i + t] = kphi[6 * (size_t)i + t];
      par[18 * (size_t)i + 6 + t] = nphi[6 * (size_t)i + t];
      par[18 * (size_t)i + 12 + t] = delphi[6 * (size_t)i + t];
    }
  int rc;
  if ((rc = replace_array(b, &b->tors_abcd, abcd, 4 * (size_t)n))) return rc;
  if ((rc = replace_array(b, &b->tors_par, (const double *)par.data(), par.size()))) return rc;
  std::vector<double> zero((size_t)n, 0.0);
  if ((rc = replace_array(b, &b->tors_tau, (const double *)zero.data(), zero.size()))) return rc;
  b->ntors = n;
  drop_step_graphs(b);
  return FE_OK;
}

int fe_set_impropers(fe_box *box, int n, const int *abcd, const double *kimpr,
                     const double *angeq) {
  if (!box || n < 0 || (n > 0 && (!abcd || !kimpr || !angeq))) return FE_ERR_ARG;
  Box *b = &box->b;
  if (!sites_in_range(abcd, 4 * (size_t)n, b->n)) {
    set_error("fe_set_impropers: site index outside the box");
    return FE_ERR_ARG;
  }
  int rc;
  if ((rc = replace_array(b, &b->impr_abcd, abcd, 4 * (size_t)n))) return rc;
  if ((rc = replace_array(b, &b->impr_k, kimpr, (size_t)n))) return rc;
  if ((rc = replace_array(b, &b->impr_eq, angeq, (size_t)n))) return rc;
  b->nimpr = n;
  drop_step_graphs(b);
  return FE_OK;
}

int fe_get_torsion_angles(fe_box *box, double *tau) {
  if (!box || (!tau && box->b.ntors > 0)) return FE_ERR_ARG;
  Box *b = &box->b;
  if (b->ntors == 0) return FE_OK;
  FE_CUDA(cudaMemcpyAsync(tau, b->tors_tau, sizeof(double) * b->ntors, cudaMemcpyDeviceToHost,
                          b->stream));
  FE_CUDA(cudaStreamSynchronize(b->stream));
  return FE_OK;
}

int fe_bonded_ext(fe_box *box, double *en3) {
  if (!box) return FE_ERR_ARG;
  Box *b = &box->b;
  int rc = launch_bonded_ext(b, false);
  if (rc) return rc;
  if ((rc = sync_scal(b))) return rc;
  if (en3)
    for (int t = 0; t < 3; t++) en3[t] = b->nurey + b->ntors + b->nimpr ? b->host_scal[SC_UREY + t] : 0.0;
  return FE_OK;
}

int fe_pbc_all(fe_box *box) {
  if (!box) return FE_ERR_ARG;
  int rc = launch_pbc(&box->b);
  if (rc) return rc;
  return check_status(&box->b);
}

int fe_kinet(fe_box *box, double *ken6, double *kinet) {
  if (!box) return FE_ERR_ARG;
  Box *b = &box->b;
  int rc = launch_kinet(b);
  if (rc) return rc;
  if ((rc = sync_scal(b))) return rc;
  if (ken6)
    for (int i = 0; i < 6; i++) ken6[i] = b->host_scal[SC_KEN + i];
  if (kinet) *kinet = b->host_scal[FE_EN_KINET];
  return FE_OK;
}

int fe_integrate_vverlet(fe_box *box, double vscal, double *en) {
  if (!box) return FE_ERR_ARG;
  Box *b = &box->b;
  int rc;
  if ((rc = launch_vv1(b, vscal))) return rc;
  if ((rc = forces_device(b))) return rc;
  if ((rc = launch_vv2(b, vscal))) return rc;
  if ((rc = sync_scal(b))) return rc;
  if (en)
    for (int i = 0; i < FE_EN_COUNT; i++) en[i] = b->host_scal[i];
  return FE_OK;
}

// RESPA runs on the FP64 drop-in: the mixed path folds the bonded terms and
// the exclusion corrections into one fixed-point pass
static int respa_check(Box *b, const char *what) {
  if (b->mx) {
    set_error(std::string(what) + ": RESPA runs on the FP64 engine (FE_PREC_FP64)");
    return FE_ERR_STATE;
  }
  if (!b->have_list) {
    set_error(std::string(what) + " requested before a neighbour list was built");
    return FE_ERR_STATE;
  }
  return FE_OK;
}

static void copy_en(const Box *b, double *en) {
  if (en)
    for (int i = 0; i < FE_EN_COUNT; i++) en[i] = b->host_scal[i];
}

int fe_force_short(fe_box *box, double *en) {
  if (!box) return FE_ERR_ARG;
  Box *b = &box->b;
  int rc;
  if ((rc = respa_check(b, "fe_force_short"))) return rc;
  if ((rc = respa_force_short(b))) return rc;
  // force_short.c leaves ff holding the fast forces
  FE_CUDA(cudaMemcpyAsync(b->ff, b->ff_short, sizeof(double) * 3 * (size_t)b->n,
                          cudaMemcpyDeviceToDevice, b->stream));
  if ((rc = launch_assemble_energies(b, 1))) return rc;
  if ((rc = sync_scal(b))) return rc;
  copy_en(b, en);
  return FE_OK;
}

int fe_force_long(fe_box *box, double *en) {
  if (!box) return FE_ERR_ARG;
  Box *b = &box->b;
  int rc;
  if ((rc = respa_check(b, "fe_force_long"))) return rc;
  if ((rc = respa_force_long(b))) return rc;
  if ((rc = launch_assemble_energies(b, 1))) return rc;
  if ((rc = sync_scal(b))) return rc;
  copy_en(b, en);
  return FE_OK;
}

int fe_integrate_mts(fe_box *box, double vscal, int nshort, double *en) {
  if (!box || nshort < 1) return FE_ERR_ARG;
  Box *b = &box->b;
  int rc;
  if ((rc = respa_check(b, "fe_integrate_mts"))) return rc;
  if ((rc = respa_step(b, vscal, nshort, -1))) return rc;
  if ((rc = sync_scal(b))) return rc;
  copy_en(b, en);
  return FE_OK;
}

int fe_integrate_mts_nhc(fe_box *box, int nshort, int xrespa, double *en) {
  if (!box || nshort < 1 || (xrespa != 0 && xrespa != 1)) return FE_ERR_ARG;
  Box *b = &box->b;
  int rc;
  if ((rc = respa_check(b, "fe_integrate_mts_nhc"))) return rc;
  if ((rc = respa_step(b, 1.0, nshort, xrespa))) return rc;
  if ((rc = sync_scal(b))) return rc;
  copy_en(b, en);
  return FE_OK;
}

int fe_get_forces_mts(fe_box *box, double *ff_short, double *ff_long) {
  if (!box) return FE_ERR_ARG;
  Box *b = &box->b;
  int rc = respa_alloc(b);
  if (rc) return rc;
  const size_t bytes = sizeof(double) * 3 * (size_t)b->n;
  if (ff_short) FE_CUDA(cudaMemcpyAsync(ff_short, b->ff_short, bytes, cudaMemcpyDeviceToHost, b->stream));
  if (ff_long) FE_CUDA(cudaMemcpyAsync(ff_long, b->ff_long, bytes, cudaMemcpyDeviceToHost, b->stream));
  FE_CUDA(cudaStreamSynchronize(b->stream));
  return FE_OK;
}

int fe_set_forces_mts(fe_box *box, const double *ff_short, const double *ff_long) {
  if (!box) return FE_ERR_ARG;
  Box *b = &box->b;
  int rc = respa_alloc(b);
  if (rc) return rc;
  const size_t bytes = sizeof(double) * 3 * (size_t)b->n;
  if (ff_short) FE_CUDA(cudaMemcpyAsync(b->ff_short, ff_short, bytes, cudaMemcpyHostToDevice, b->stream));
  if (ff_long) FE_CUDA(cudaMemcpyAsync(b->ff_long, ff_long, bytes, cudaMemcpyHostToDevice, b->stream));
  FE_CUDA(cudaStreamSynchronize(b->stream));
  return FE_OK;
}

// the gather of the wrapped positions into xyz_dev on stream `s`
static int k_xyz_gather_on(Box *b, cudaStream_t s) {
  cudaStream_t keep = b->stream;
  b->stream = s;
  int rc = launch_xyz_gather(b, b->xyz_dev);
  b->stream = keep;
  return rc;
}

// The host-buffer step's copies and kernels: uploads of the step's inputs,
// the first half kick and drift, the positions' download on the copy
// stream beside the force evaluation, the second half kick and the
// downloads of velocities and forces; joined back into b->stream.
static int io_step_body(Box *b, double vscal, const fe_md_io *io, char *ap, char *np) {
  int rc;
  const size_t bytes = sizeof(double) * 3 * (size_t)b->n;
  // uu is written by the step, not read (integrate_vverlet.c:95-97)
  FE_CUDA(cudaMemcpyAsync(b->xyz_dev, ap, bytes, cudaMemcpyHostToDevice, b->stream));
  if ((rc = launch_xyz_scatter(b, b->xyz_dev, true, false))) return rc;
  FE_CUDA(cudaMemcpyAsync(b->pos_nopbc, np, bytes, cudaMemcpyHostToDevice, b->stream));
  FE_CUDA(cudaMemcpyAsync(b->vv, io->vv, bytes, cudaMemcpyHostToDevice, b->stream));
  FE_CUDA(cudaMemcpyAsync(b->ff, io->ff, bytes, cudaMemcpyHostToDevice, b->stream));
  if ((rc = launch_vv1(b, vscal))) return rc;
  // the positions are final after the drift: their download runs on the
  // copy stream while the forces are evaluated
  FE_CUDA(cudaEventRecord(b->ev_io_pos, b->stream));
  FE_CUDA(cudaStreamWaitEvent(b->s_io, b->ev_io_pos, 0));
  if ((rc = k_xyz_gather_on(b, b->s_io))) return rc;
  FE_CUDA(cudaMemcpyAsync(ap, b->xyz_dev, bytes, cudaMemcpyDeviceToHost, b->s_io));
  FE_CUDA(cudaMemcpyAsync(np, b->pos_nopbc, bytes, cudaMemcpyDeviceToHost, b->s_io));
  FE_CUDA(cudaEventRecord(b->ev_io_done, b->s_io));
  if ((rc = forces_device(b))) return rc;
  if ((rc = launch_vv2(b, vscal))) return rc;
  FE_CUDA(cudaMemcpyAsync(io->vv, b->vv, bytes, cudaMemcpyDeviceToHost, b->stream));
  FE_CUDA(cudaMemcpyAsync(io->uu, b->uu, bytes, cudaMemcpyDeviceToHost, b->stream));
  FE_CUDA(cudaMemcpyAsync(io->ff, b->ff, bytes, cudaMemcpyDeviceToHost, b->stream));
  FE_CUDA(cudaStreamWaitEvent(b->stream, b->ev_io_done, 0));
  return FE_OK;
}

int fe_integrate_vverlet_host(fe_box *box, double vscal, const fe_md_io *io, double *en) {
  if (!box || !io || !io->atoms || !io->nopbc || !io->vv || !io->uu || !io->ff) {
    set_error("fe_integrate_vverlet_host: null argument");
    return FE_ERR_ARG;
  }
  Box *b = &box->b;
  char *ap = (char *)io->atoms + io->atoms_off, *np = (char *)io->nopbc + io->nopbc_off;
  const bool queued = io->atoms_stride == 24 && io->nopbc_stride == 24 && pinned_host(ap) &&
                      pinned_host(np) && pinned_host(io->vv) && pinned_host(io->uu) &&
                      pinned_host(io->ff);
  int rc;
  if (!queued) {
    if ((rc = fe_set_positions(box, io->atoms, io->atoms_stride, io->atoms_off, 0))) return rc;
    if ((rc = fe_set_positions_nopbc(box, io->nopbc, io->nopbc_stride, io->nopbc_off))) return rc;
    if ((rc = fe_set_velocities(box, io->vv, io->uu))) return rc;
    if ((rc = fe_set_forces(box, io->ff))) return rc;
    if ((rc = fe_integrate_vverlet(box, vscal, en))) return rc;
    if ((rc = fe_get_positions(box, io->atoms, io->atoms_stride, io->atoms_off))) return rc;
    if ((rc = fe_get_positions_nopbc(box, io->nopbc, io->nopbc_stride, io->nopbc_off))) return rc;
    if ((rc = fe_get_velocities(box, io->vv, io->uu))) return rc;
    return fe_get_forces(box, io->ff);
  }
  if (!b->s_io) {
    FE_CUDA(cudaStreamCreateWithFlags(&b->s_io, cudaStreamNonBlocking));
    FE_CUDA(cudaEventCreateWithFlags(&b->ev_io_pos, cudaEventDisableTiming));
    FE_CUDA(cudaEventCreateWithFlags(&b->ev_io_done, cudaEventDisableTiming));
  }
  // one graph per set of host arrays and velocity scale: a caller that
  // keeps its arrays (the reference's atom, atnopbc, vv, uu, ff) replays it
  const void *key[5] = {ap, np, io->vv, io->uu, io->ff};
  if (!b->g_io || b->io_vscal != vscal || memcmp(key, b->io_key, sizeof key) != 0) {
    drop_io_graph(b);
    cudaGraph_t g;
    FE_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    rc = io_step_body(b, vscal, io, ap, np);
    cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (rc) {
      if (e == cudaSuccess) cudaGraphDestroy(g);
      return rc;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture (host-buffer step)");
    e = cudaGraphInstantiate(&b->g_io, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      b->g_io = nullptr;
      return cuda_fail(e, "cudaGraphInstantiate (host-buffer step)");
    }
    memcpy(b->io_key, key, sizeof key);
    b->io_vscal = vscal;
  }
  FE_CUDA(cudaGraphLaunch(b->g_io, b->stream));
  if ((rc = sync_scal(b))) return rc;
  copy_en(b, en);
  return FE_OK;
}

int fe_integrate_nhc(fe_box *box, double time_step) {
  if (!box) return FE_ERR_ARG;
  Box *b = &box->b;
  int rc = launch_nhc(b, time_step);
  if (rc) return rc;
  return check_status(b);
}

int fe_run_md(fe_box *box, int nsteps, int nlist_freq, int use_nhc, long first_step, double *rec) {
  if (!box || nsteps < 0 || nlist_freq <= 0) return FE_ERR_ARG;
  Box *b = &box->b;
  if (!b->have_list) {
    set_error("run_md requested before a neighbour list was built");
    return FE_ERR_STATE;
  }
  if (nsteps == 0) return FE_OK;
  // records go to the host only when asked; without `rec` the graphs keep
  // whatever record buffer they were captured with (the kernel stops at its end)
  if (rec && b->rec_cap < nsteps) {
    if (b->rec) cudaFree(b->rec);
    b->rec = nullptr;
    FE_CUDA(cudaMalloc(&b->rec, sizeof(double) * FE_EN_COUNT * (size_t)nsteps));
    b->rec_cap = nsteps;
    // the record kernel's capacity is baked into the graphs: recapture
    if (b->g_step) cudaGraphExecDestroy(b->g_step);
    if (b->g_step_list) cudaGraphExecDestroy(b->g_step_list);
    b->g_step = b->g_step_list = nullptr;
    b->g_key = -1;
  }
  FE_CUDA(cudaMemsetAsync(b->rec_counter, 0, sizeof(int), b->stream));
  int key = use_nhc ? 1 : 0;
  int rc;
  if (b->g_key != key) {
    if (b->g_step) cudaGraphExecDestroy(b->g_step);
    if (b->g_step_list) cudaGraphExecDestroy(b->g_step_list);
    b->g_step = b->g_step_list = nullptr;
    if ((rc = capture(b, false, use_nhc != 0, &b->g_step))) return rc;
    if ((rc = capture(b, true, use_nhc != 0, &b->g_step_list))) return rc;
    b->g_key = key;
  }
  for (long i = first_step; i < first_step + nsteps; i++) {
    cudaGraphExec_t g = b->g_step;
    if (i % nlist_freq == 0) g = b->g_step_list;
    FE_CUDA(cudaGraphLaunch(g, b->stream));
  }
  if (rec)
    FE_CUDA(cudaMemcpyAsync(rec, b->rec, sizeof(double) * FE_EN_COUNT * (size_t)nsteps,
                            cudaMemcpyDeviceToHost, b->stream));
  if ((rc = sync_scal(b))) return rc;
  return FE_OK;
}

int fe_autotune(fe_box *box, int *choice3, double *us) {
  if (!box) return FE_ERR_ARG;
  Box *b = &box->b;
  if (!b->mx) return FE_OK;  // the FP64 drop-in keeps the reference's one-row-per-warp shape
  if (!b->have_list) {
    set_error("fe_autotune needs a neighbour list");
    return FE_ERR_STATE;
  }
  int nw = 0, rw = 0, blocks = 0;
  int rc = mixed_autotune(b, &nw, &rw, &blocks, us);
  if (rc) return rc;
  if (choice3) {
    choice3[0] = nw;
    choice3[1] = (65536 / (rw * 32)) & ~7;  // the per-thread register cap it compiles to
    choice3[2] = blocks;
  }
  b->g_key = -1;  // step graphs are recaptured with the new shape
  drop_io_graph(b);
  return forces_device(b);
}

int fe_time_kernel(fe_box *box, int which, int reps, double *us) {
  if (!box || reps < 1 || !us) return FE_ERR_ARG;
  Box *b = &box->b;
  if (!b->have_list) {
    set_error("fe_time_kernel needs a built list");
    return FE_ERR_STATE;
  }
  cudaEvent_t e0, e1;
  FE_CUDA(cudaEventCreate(&e0));
  FE_CUDA(cudaEventCreate(&e1));
  int rc = relaunch_kernel(b, which);  // warm
  if (rc) return rc;
  FE_CUDA(cudaEventRecord(e0, b->stream));
  for (int r = 0; r < reps; r++)
    if ((rc = relaunch_kernel(b, which))) return rc;
  FE_CUDA(cudaEventRecord(e1, b->stream));
  FE_CUDA(cudaEventSynchronize(e1));
  float ms = 0.f;
  FE_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *us = 1000.0 * ms / reps;
  return check_status(b);
}

int fe_step_launches(fe_box *box, int use_nhc, int *plain, int *with_list) {
  if (!box) return FE_ERR_ARG;
  Box *b = &box->b;
  int key = use_nhc ? 1 : 0;
  if (b->g_key != key) {
    set_error("fe_step_launches: run fe_run_md with the same use_nhc first");
    return FE_ERR_STATE;
  }
  if (plain) *plain = b->launches_plain;
  if (with_list) *with_list = b->launches_list;
  return FE_OK;
}

int fe_pair_counts(fe_box *box, int64_t *counts4) {
  if (!box || !counts4) return FE_ERR_ARG;
  Box *b = &box->b;
  if (b->mx || !b->have_list) {
    set_error("fe_pair_counts needs an FP64 box with a list");
    return FE_ERR_STATE;
  }
  long long c[4];
  int rc = pair_counts64(b, c);
  if (rc) return rc;
  for (int t = 0; t < 4; t++) counts4[t] = c[t];
  return FE_OK;
}

int fe_list_stats(fe_box *box, int64_t *entries, int *max_row) {
  if (!box) return FE_ERR_ARG;
  Box *b = &box->b;
  if (!b->have_list) {
    set_error("no list built yet");
    return FE_ERR_STATE;
  }
  std::vector<int> c(b->n), c2(b->n, 0);
  if (b->mx) {
    const int *a = nullptr, *r = nullptr;
    mixed_counts(b, &a, &r);
    FE_CUDA(cudaMemcpyAsync(c.data(), a, sizeof(int) * b->n, cudaMemcpyDeviceToHost, b->stream));
    FE_CUDA(cudaMemcpyAsync(c2.data(), r, sizeof(int) * b->n, cudaMemcpyDeviceToHost, b->stream));
  } else {
    FE_CUDA(cudaMemcpyAsync(c.data(), b->nl_count, sizeof(int) * b->n, cudaMemcpyDeviceToHost,
                            b->stream));
  }
  FE_CUDA(cudaStreamSynchronize(b->stream));
  for (int i = 0; i < b->n; i++) c[i] += c2[i];
  int64_t e = 0;
  int m = 0;
  for (int v : c) {
    e += v;
    if (v > m) m = v;
  }
  if (entries) *entries = e;
  if (max_row) *max_row = m;
  return FE_OK;
}

int fe_nl_check(fe_box *box, int lb, int ub, int *nl_flag) {
  if (!box || !nl_flag || lb < 0 || ub < lb || ub > box->b.n) return FE_ERR_ARG;
  Box *b = &box->b;
  if (!b->have_list) {
    set_error("fe_nl_check needs a list built by fe_nblist");
    return FE_ERR_STATE;
  }
  FE_CUDA(cudaMemsetAsync(b->nl_dev, 0, sizeof(int), b->stream));
  int rc = launch_nl_check(b, lb, ub, b->nl_dev);
  if (rc) return rc;
  int f = 0;
  FE_CUDA(cudaMemcpyAsync(&f, b->nl_dev, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  FE_CUDA(cudaStreamSynchronize(b->stream));
  *nl_flag = f;
  return FE_OK;
}

int fe_inner_list_stats(fe_box *box, int64_t *entries, int *max_row, int64_t *prunes) {
  if (!box) return FE_ERR_ARG;
  Box *b = &box->b;
  const int *a = nullptr, *r = nullptr;
  bool on = false;
  if (b->mx) mixed_inner_counts(b, &a, &r, &on);
  if (!on) {
    set_error("fe_inner_list_stats: no inner list (FP64 mode, or rc + skin >= rclist)");
    return FE_ERR_STATE;
  }
  std::vector<int> c(b->n), c2(b->n);
  MxPruneState st;
  FE_CUDA(cudaMemcpyAsync(c.data(), a, sizeof(int) * b->n, cudaMemcpyDeviceToHost, b->stream));
  FE_CUDA(cudaMemcpyAsync(c2.data(), r, sizeof(int) * b->n, cudaMemcpyDeviceToHost, b->stream));
  FE_CUDA(cudaMemcpyAsync(&st, mixed_prune_state(b), sizeof(st), cudaMemcpyDeviceToHost,
                          b->stream));
  FE_CUDA(cudaStreamSynchronize(b->stream));
  int64_t e = 0;
  int m = 0;
  for (int i = 0; i < b->n; i++) {
    int v = c[i] + c2[i];
    e += v;
    if (v > m) m = v;
  }
  if (entries) *entries = e;
  if (max_row) *max_row = m;
  if (prunes) *prunes = (int64_t)st.prunes;
  return FE_OK;
}

int fe_mc_setup(fe_box *box, int kmax, int max_k_square, double rc_ew) {
  if (!box || kmax < 1 || max_k_square < 1 || rc_ew <= 0.0) return FE_ERR_ARG;
  return mc_setup(&box->b, kmax, max_k_square, rc_ew);
}

int fe_mc_delta(fe_box *box, int lb, int ub, const double *new_pos, double *dE, double *parts3) {
  if (!box || !new_pos || lb < 0 || ub <= lb || ub > box->b.n) return FE_ERR_ARG;
  return mc_delta(&box->b, lb, ub, new_pos, dE, parts3);
}

int fe_mc_delta_terms(fe_box *box, int lb, int ub, const double *new_pos, double *terms6) {
  if (!box || !new_pos || !terms6) return FE_ERR_ARG;
  return mc_terms(&box->b, lb, ub, new_pos, terms6);
}

int fe_mc_site_energy(fe_box *box, int lb, int ub, double *terms6) {
  if (!box || !terms6) return FE_ERR_ARG;
  return mc_terms(&box->b, lb, ub, nullptr, terms6);
}

// pme_spline.c:10-49: cardinal B-spline weights array[1..order] and their
// derivatives darray[1..order] at fraction w, by the same recursion (and
// operation order) as the reference; host arithmetic (the kernels have their
// own device copies of it).
int fe_bspline(int order, double w, double *array, double *darray) {
  if (order < 3 || order > 16 || !array || !darray) {
    set_error("fe_bspline: order in 3..16 and two arrays of order + 1 doubles");
    return FE_ERR_ARG;
  }
  for (int i = 3; i <= order; i++) array[i] = 0.0;
  array[2] = w;
  array[1] = 1.0 - w;
  array[0] = 0.0;
  for (int i = 3; i <= order - 1; i++) {
    double div = (double)(1.0 / (i - 1));
    array[i] = div * w * array[i - 1];
    double di = (double)(i);
    for (int j = 1; j <= (i - 2); j++) {
      double dj = (double)(j);
      array[i - j] = div * ((w + dj) * array[i - j - 1] + (di - dj - w) * array[i - j]);
    }
    array[1] *= div * (1.0 - w);
  }
  darray[0] = 0.0;
  darray[1] = -array[1];
  for (int i = 2; i <= order; i++) darray[i] = array[i - 1] - array[i];
  int kk = order;
  double div = (double)(1.0 / (kk - 1));
  array[kk] = div * w * array[kk - 1];
  double dkk = (double)(kk);
  for (int i = 1; i <= (kk - 2); i++) {
    double di = (double)(i);
    array[kk - i] = div * ((w + di) * array[kk - i - 1] + (dkk - di - w) * array[kk - i]);
  }
  array[1] *= div * (1.0 - w);
  return FE_OK;
}

int fe_drift(fe_box *box) {
  if (!box) return FE_ERR_ARG;
  return launch_drift(&box->b);
}

int fe_box_set_temperature(fe_box *box, double T) {
  if (!box || !(T > 0.0)) return FE_ERR_ARG;
  Box *b = &box->b;
  b->p.T = T;
  FE_CUDA(cudaMemcpyAsync(b->scal + SC_TEMP, &b->p.T, sizeof(double), cudaMemcpyHostToDevice,
                          b->stream));
  FE_CUDA(cudaStreamSynchronize(b->stream));
  return FE_OK;
}

int fe_mc_accept(fe_box *box) {
  if (!box) return FE_ERR_ARG;
  return mc_accept(&box->b);
}

int fe_mc_kspace_energy(fe_box *box, double *e) {
  if (!box || !e) return FE_ERR_ARG;
  return mc_kspace_energy(&box->b, e);
}

}  // extern "C"
