// k_replica.cu -- many boxes stepped together, with replica exchange on the
// device.
//
// The reference steps its boxes one after another (repexch.c:139-214) and,
// every cyc_swap steps, attempts swaps of neighbouring temperatures with
// swap_box (swap_box.c:5-86, schedule repexch.c:268-305): pairs (0,1),(2,3),..
// on one attempt, (1,2),(3,4),.. on the next; accept when
// exp((1/kT_k - 1/kT_k+1)(U_k - U_k+1)) > ran2(); on acceptance exchange the
// coordinates, forces and velocities of the two boxes and rescale the
// velocities by sqrt(T_k/T_k+1).
//
// Here one CUDA graph holds one step of every box, each box on its own stream
// (the branches run concurrently and fill the GPU even when single boxes are
// small), and the exchange is two kernels at the end of the graph.  Instead
// of moving coordinates, an accepted swap exchanges which temperature slot
// each box holds: slot s keeps its temperature and its Nose-Hoover chain
// state (as box k keeps nhc[k] in the reference), the boxes keep their atoms.
// For equal boxes this is the same Markov chain as swapping coordinates; it
// is also what makes boxes of different sizes exchangeable.  The velocity
// rescale keeps the reference's arithmetic: the box moving down a slot is
// multiplied by sqrt(T_s/T_s+1), the one moving up is divided by it, and
// uu = vv for both.  Uniform numbers come from Philox4x32-10 keyed by the
// batch seed and the attempt number, so the host can reproduce every
// decision.
#include <cmath>
#include <vector>

#include "fe_internal.h"
#include "fe_mixed.h"
#include "fe_rng.cuh"

namespace fe {

struct RexRep {
  double *scal;  // energies (FE_EN_*) and SC_TEMP
  double *vv, *uu;
  double *zeta;  // 3*M
  int n3, m3;
};

struct Batch {
  std::vector<Box *> boxes;
  int R = 0;
  int dev = 0;
  cudaStream_t main = nullptr;
  cudaEvent_t fork = nullptr, done = nullptr;
  std::vector<cudaEvent_t> join;
  RexRep *d_rep = nullptr;
  double *d_Tslot = nullptr;        // temperature of each slot
  int *d_slot_rep = nullptr;        // box holding each slot
  int *d_vmode = nullptr;           // per box: 0 none, 1 multiply, 2 divide
  double *d_vfac = nullptr;         // per box: sqrt(T_s / T_s+1)
  long long *d_acc = nullptr;       // per slot pair (s, s+1) at index s
  long long *d_att = nullptr;
  unsigned long long *d_attempt = nullptr;  // attempts made so far
  uint64_t seed = 0;
  int max_n3 = 0;
  // step graphs: bit 0 list, bit 1 exchange, bit 2 last step of a run (fused
  // Nose-Hoover: the last step leaves the next step's first chain update out)
  cudaGraphExec_t g[8] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  int launches[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int g_key = -1;
  // fused step: every box in one launch per kernel (mixed-precision boxes)
  bool fused = false;
  BMxPlan *mx = nullptr;
  BIntArgs *d_bint = nullptr;
  int *d_off_red = nullptr, *d_off_site = nullptr;  // block ranges: reductions, per site
  int tot_red = 0, tot_site = 0;
};

// Boltzmann energy in kJ/mol as read_sim.c:351 (sim.kT = RG * T * .001).
__device__ __forceinline__ double rex_kT(double T) { return ((kKB * kNA) * T) * .001; }

// The reference's en[k].potens for the water force field (calcvalue.c:43):
// bond + bend + nbonds (torsion, improper and Urey-Bradley terms are zero).
// en[k].potens of calcvalue.c:45-53 (no GOLIK, no SASA, not NEUTRAL)
__device__ __forceinline__ double rex_potens(const double *s) {
  return s[FE_EN_BOND] + s[FE_EN_BEND] + s[FE_EN_TORS] + s[FE_EN_NBONDS] + s[FE_EN_IMPR] +
         s[FE_EN_UREY];
}

__global__ void k_rex_decide(int R, const RexRep *__restrict__ rep, const double *__restrict__ Tslot,
                             int *__restrict__ slot_rep, int *__restrict__ vmode,
                             double *__restrict__ vfac, long long *__restrict__ acc,
                             long long *__restrict__ att, unsigned long long *__restrict__ attempt_ctr,
                             uint64_t seed) {
  __shared__ unsigned long long attempt;
  if (threadIdx.x == 0) attempt = *attempt_ctr;
  for (int r = threadIdx.x; r < R; r += blockDim.x) vmode[r] = 0;
  __syncthreads();
  int parity = (int)(attempt & 1ull);  // sim_hyb.flag alternation, repexch.c:273-301
  for (int t = threadIdx.x;; t += blockDim.x) {
    int s = parity + 2 * t;
    if (s + 1 >= R) break;
    int r1 = slot_rep[s], r2 = slot_rep[s + 1];
    double delta_beta = 1.0 / rex_kT(Tslot[s]) - 1.0 / rex_kT(Tslot[s + 1]);
    double delta_energy = rex_potens(rep[r1].scal) - rex_potens(rep[r2].scal);
    double accep_crit = exp(delta_beta * delta_energy);
    double u = fe_uniform(seed, kRngTagExchange, attempt, (uint32_t)s);
    att[s] += 1;
    if (accep_crit > u) {
      acc[s] += 1;
      slot_rep[s] = r2;
      slot_rep[s + 1] = r1;
      double v_scale_1 = sqrt(Tslot[s] / Tslot[s + 1]);
      vmode[r2] = 1;  // now in slot s:   vv *= v_scale_1
      vfac[r2] = v_scale_1;
      vmode[r1] = 2;  // now in slot s+1: vv /= v_scale_1
      vfac[r1] = v_scale_1;
      rep[r2].scal[SC_TEMP] = Tslot[s];
      rep[r1].scal[SC_TEMP] = Tslot[s + 1];
      // the chain state belongs to the slot
      double *z1 = rep[r1].zeta, *z2 = rep[r2].zeta;
      for (int j = 0; j < rep[r1].m3; j++) {
        double t1 = z1[j];
        z1[j] = z2[j];
        z2[j] = t1;
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) *attempt_ctr = attempt + 1ull;
}

__global__ void k_rex_apply(const RexRep *__restrict__ rep, const int *__restrict__ vmode,
                            const double *__restrict__ vfac) {
  int r = blockIdx.y;
  int mode = vmode[r];
  if (mode == 0) return;
  RexRep p = rep[r];
  double f = vfac[r];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < p.n3; i += gridDim.x * blockDim.x) {
    double v = p.vv[i];
    v = mode == 1 ? v * f : v / f;
    p.vv[i] = v;
    p.uu[i] = v;
  }
}

static int launch_exchange(Batch *B) {
  k_rex_decide<<<1, 256, 0, B->main>>>(B->R, B->d_rep, B->d_Tslot, B->d_slot_rep, B->d_vmode,
                                       B->d_vfac, B->d_acc, B->d_att, B->d_attempt, B->seed);
  FE_LAUNCH_CHECK("k_rex_decide");
  int bx = (B->max_n3 + 255) / 256;
  if (bx > 64) bx = 64;
  k_rex_apply<<<dim3(bx, B->R), 256, 0, B->main>>>(B->d_rep, B->d_vmode, B->d_vfac);
  FE_LAUNCH_CHECK("k_rex_apply");
  return FE_OK;
}

static void free_fused(Batch *B) {
  if (B->mx) mixed_batch_free(B->mx);
  B->mx = nullptr;
  cudaFree(B->d_bint);
  cudaFree(B->d_off_red);
  cudaFree(B->d_off_site);
  B->d_bint = nullptr;
  B->d_off_red = B->d_off_site = nullptr;
  B->fused = false;
}

// Sets up the fused step (all boxes per launch) when every box allows it.
static int setup_fused(Batch *B) {
  BMxPlan *plan = nullptr;
  int rc = mixed_batch_plan(B->boxes.data(), B->R, &plan);
  if (rc) return rc;
  B->mx = plan;
  std::vector<BIntArgs> args(B->R);
  std::vector<int> ored(B->R + 1, 0), osite(B->R + 1, 0);
  for (int r = 0; r < B->R; r++) {
    Box *b = B->boxes[r];
    args[r] = make_bint_args(b);
    args[r].rec = nullptr;  // batches keep no per-step records
    args[r].rec_cap = 0;
    int nred = (b->n + 255) / 256;
    ored[r + 1] = ored[r] + (nred > 512 ? 512 : nred);
    osite[r + 1] = osite[r] + (b->n + 255) / 256;
  }
  B->tot_red = ored[B->R];
  B->tot_site = osite[B->R];
  FE_CUDA(cudaMalloc(&B->d_bint, sizeof(BIntArgs) * B->R));
  FE_CUDA(cudaMalloc(&B->d_off_red, sizeof(int) * (B->R + 1)));
  FE_CUDA(cudaMalloc(&B->d_off_site, sizeof(int) * (B->R + 1)));
  FE_CUDA(cudaMemcpy(B->d_bint, args.data(), sizeof(BIntArgs) * B->R, cudaMemcpyHostToDevice));
  FE_CUDA(cudaMemcpy(B->d_off_red, ored.data(), sizeof(int) * (B->R + 1), cudaMemcpyHostToDevice));
  FE_CUDA(cudaMemcpy(B->d_off_site, osite.data(), sizeof(int) * (B->R + 1),
                     cudaMemcpyHostToDevice));
  B->fused = true;
  return FE_OK;
}

// One step of every box as the fused kernels, one launch per kernel for all
// boxes: [list rebuild,] [NHC scale,] half kick, forces, half kick [NHC],
// as step_body.  With Nose-Hoover the first chain update of a step needs the
// kinetic energy of the velocities the previous step ended with, which the
// previous step's last pass has just summed: that pass applies it
// (chain_next) unless an exchange follows (which rescales velocities and
// swaps temperatures: capture_batch recomputes it after the exchange) or the
// step ends a run (fe_batch_run starts every run with the update).
static int fused_step(Batch *B, bool with_list, bool use_nhc, bool chain_next) {
  int rc = FE_OK;
  cudaStream_t s = B->main;
  if (with_list && (rc = mixed_batch_list(B->mx, s))) return rc;
  const int nb = B->R, nhc = use_nhc ? 1 : 0;
  if ((rc = launch_b_vv1(B->d_bint, B->d_off_site, nb, B->tot_site, nhc, s))) return rc;
  if ((rc = mixed_batch_forces(B->mx, s))) return rc;
  if ((rc = launch_b_vv2(B->d_bint, B->d_off_red, nb, B->tot_red, nhc, s))) return rc;
  if (use_nhc && (rc = launch_b_scale_kinet(B->d_bint, B->d_off_red, nb, B->tot_red,
                                             chain_next ? 1 : 0, s)))
    return rc;
  return FE_OK;
}

static void free_batch(Batch *B) {
  free_fused(B);
  for (auto &g : B->g)
    if (g) cudaGraphExecDestroy(g);
  for (auto e : B->join)
    if (e) cudaEventDestroy(e);
  if (B->fork) cudaEventDestroy(B->fork);
  if (B->done) cudaEventDestroy(B->done);
  cudaFree(B->d_rep);
  cudaFree(B->d_Tslot);
  cudaFree(B->d_slot_rep);
  cudaFree(B->d_vmode);
  cudaFree(B->d_vfac);
  cudaFree(B->d_acc);
  cudaFree(B->d_att);
  cudaFree(B->d_attempt);
  if (B->main) cudaStreamDestroy(B->main);
}

static int capture_batch(Batch *B, bool with_list, bool exchange, bool last, bool use_nhc,
                         cudaGraphExec_t *out, int *nlaunch) {
  cudaGraph_t g = nullptr;
  FE_CUDA(cudaStreamBeginCapture(B->main, cudaStreamCaptureModeThreadLocal));
  long l0 = g_launches;
  int rc = FE_OK;
  cudaError_t e = cudaSuccess;
  if (B->fused) {
    rc = fused_step(B, with_list, use_nhc, use_nhc && !exchange && !last);
  } else {
    e = cudaEventRecord(B->fork, B->main);
    for (int r = 0; r < B->R && rc == FE_OK && e == cudaSuccess; r++) {
      Box *b = B->boxes[r];
      e = cudaStreamWaitEvent(b->stream, B->fork, 0);
      if (e != cudaSuccess) break;
      rc = step_body(b, with_list, use_nhc);
      if (rc) break;
      e = cudaEventRecord(B->join[r], b->stream);
      if (e != cudaSuccess) break;
      e = cudaStreamWaitEvent(B->main, B->join[r], 0);
    }
  }
  if (rc == FE_OK && e == cudaSuccess && exchange) rc = launch_exchange(B);
  // fused Nose-Hoover: the next step's first chain update, from the
  // velocities as the exchange left them
  if (rc == FE_OK && e == cudaSuccess && exchange && B->fused && use_nhc && !last)
    rc = launch_b_kinet_nhc(B->d_bint, B->d_off_red, B->R, B->tot_red, B->main);
  *nlaunch = (int)(g_launches - l0);
  cudaError_t ee = cudaStreamEndCapture(B->main, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return cuda_fail(e, "batch capture");
  }
  if (ee != cudaSuccess) return cuda_fail(ee, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
  return FE_OK;
}

}  // namespace fe

using namespace fe;

struct fe_batch {
  Batch B;
};

extern "C" {

int fe_batch_create(fe_batch **out, fe_box *const *boxes, int nrep, uint64_t seed) {
  if (!out || !boxes || nrep < 1 || nrep > 4096) {
    set_error("fe_batch_create: need 1..4096 boxes");
    return FE_ERR_ARG;
  }
  *out = nullptr;
  fe_batch *fb = new fe_batch();
  Batch *B = &fb->B;
  B->R = nrep;
  B->seed = seed;
  std::vector<RexRep> reps(nrep);
  std::vector<double> T(nrep);
  std::vector<int> slot(nrep);
  int rc = FE_OK;
  for (int r = 0; r < nrep; r++) {
    if (!boxes[r]) {
      set_error("fe_batch_create: null box");
      rc = FE_ERR_ARG;
      break;
    }
    Box *b = &boxes[r]->b;
    for (int q = 0; q < r; q++)
      if (B->boxes[q] == b) {
        set_error("fe_batch_create: a box is listed twice");
        rc = FE_ERR_ARG;
      }
    if (rc) break;
    if (r == 0) B->dev = b->dev;
    if (b->dev != B->dev) {
      set_error("fe_batch_create: boxes live on different devices");
      rc = FE_ERR_ARG;
      break;
    }
    if (r > 0 && b->nhc_M != B->boxes[0]->nhc_M) {
      set_error("fe_batch_create: boxes have Nose-Hoover chains of different lengths");
      rc = FE_ERR_ARG;
      break;
    }
    B->boxes.push_back(b);
    reps[r] = RexRep{b->scal, b->vv, b->uu, b->zeta, 3 * b->n, 3 * b->nhc_M};
    T[r] = b->p.T;
    slot[r] = r;
    if (3 * b->n > B->max_n3) B->max_n3 = 3 * b->n;
  }
  if (rc) {
    delete fb;
    return rc;
  }
  cudaSetDevice(B->dev);
  cudaError_t e = cudaSuccess;
#define BT(x)                                  \
  do {                                         \
    if (e == cudaSuccess) e = (x);             \
  } while (0)
  BT(cudaStreamCreateWithFlags(&B->main, cudaStreamNonBlocking));
  BT(cudaEventCreateWithFlags(&B->fork, cudaEventDisableTiming));
  BT(cudaEventCreateWithFlags(&B->done, cudaEventDisableTiming));
  B->join.assign(nrep, nullptr);
  for (int r = 0; r < nrep; r++) BT(cudaEventCreateWithFlags(&B->join[r], cudaEventDisableTiming));
  BT(cudaMalloc(&B->d_rep, sizeof(RexRep) * nrep));
  BT(cudaMalloc(&B->d_Tslot, sizeof(double) * nrep));
  BT(cudaMalloc(&B->d_slot_rep, sizeof(int) * nrep));
  BT(cudaMalloc(&B->d_vmode, sizeof(int) * nrep));
  BT(cudaMalloc(&B->d_vfac, sizeof(double) * nrep));
  BT(cudaMalloc(&B->d_acc, sizeof(long long) * nrep));
  BT(cudaMalloc(&B->d_att, sizeof(long long) * nrep));
  BT(cudaMalloc(&B->d_attempt, sizeof(unsigned long long)));
  BT(cudaMemcpy(B->d_rep, reps.data(), sizeof(RexRep) * nrep, cudaMemcpyHostToDevice));
  BT(cudaMemcpy(B->d_Tslot, T.data(), sizeof(double) * nrep, cudaMemcpyHostToDevice));
  BT(cudaMemcpy(B->d_slot_rep, slot.data(), sizeof(int) * nrep, cudaMemcpyHostToDevice));
  BT(cudaMemset(B->d_vmode, 0, sizeof(int) * nrep));
  BT(cudaMemset(B->d_vfac, 0, sizeof(double) * nrep));
  BT(cudaMemset(B->d_acc, 0, sizeof(long long) * nrep));
  BT(cudaMemset(B->d_att, 0, sizeof(long long) * nrep));
  BT(cudaMemset(B->d_attempt, 0, sizeof(unsigned long long)));
  // each box starts at its own temperature (slot r = box r)
  for (int r = 0; r < nrep; r++)
    BT(cudaMemcpy(B->boxes[r]->scal + SC_TEMP, &T[r], sizeof(double), cudaMemcpyHostToDevice));
#undef BT
  if (e != cudaSuccess) {
    rc = cuda_fail(e, "fe_batch_create");
    free_batch(B);
    delete fb;
    return rc;
  }
  // the fused step where every box allows it (mixed precision, contiguous
  // molecules); otherwise each box steps on its own stream
  if (setup_fused(B) != FE_OK) free_fused(B);
  *out = fb;
  return FE_OK;
}

int fe_batch_set_fused(fe_batch *batch, int on) {
  if (!batch) return FE_ERR_ARG;
  Batch *B = &batch->B;
  cudaStreamSynchronize(B->main);
  for (int k = 0; k < 8; k++)
    if (B->g[k]) {
      cudaGraphExecDestroy(B->g[k]);
      B->g[k] = nullptr;
      B->launches[k] = -1;
    }
  B->g_key = -1;
  free_fused(B);
  if (!on) return FE_OK;
  int rc = setup_fused(B);
  if (rc) free_fused(B);
  return rc;
}

void fe_batch_destroy(fe_batch *batch) {
  if (!batch) return;
  cudaStreamSynchronize(batch->B.main);
  free_batch(&batch->B);
  delete batch;
}

int fe_batch_run(fe_batch *batch, int nsteps, int nlist_freq, int swap_freq, long first_step,
                 int use_nhc) {
  if (!batch || nsteps < 0 || nlist_freq <= 0 || swap_freq < 0) return FE_ERR_ARG;
  Batch *B = &batch->B;
  for (Box *b : B->boxes)
    if (!b->have_list) {
      set_error("fe_batch_run requested before every box has a neighbour list");
      return FE_ERR_STATE;
    }
  if (nsteps == 0) return FE_OK;
  int key = use_nhc ? 1 : 0;
  int rc;
  if (B->g_key != key) {
    for (auto &g : B->g) {
      if (g) cudaGraphExecDestroy(g);
      g = nullptr;
    }
    B->g_key = -1;
  }
  // work queued on the boxes' own streams comes first
  for (Box *b : B->boxes) FE_CUDA(cudaStreamSynchronize(b->stream));
  // fused Nose-Hoover: the first step's first chain update, from the current
  // velocities (every run ends without it)
  if (B->fused && use_nhc &&
      (rc = launch_b_kinet_nhc(B->d_bint, B->d_off_red, B->R, B->tot_red, B->main)))
    return rc;
  const long end = first_step + nsteps;
  for (long i = first_step; i < end; i++) {
    int v = (i % nlist_freq == 0 ? 1 : 0) | (swap_freq > 0 && i % swap_freq == 0 ? 2 : 0) |
            (B->fused && use_nhc && i == end - 1 ? 4 : 0);
    if (!B->g[v]) {
      if ((rc = capture_batch(B, v & 1, v & 2, v & 4, use_nhc != 0, &B->g[v], &B->launches[v])))
        return rc;
      B->g_key = key;
    }
    FE_CUDA(cudaGraphLaunch(B->g[v], B->main));
  }
  FE_CUDA(cudaEventRecord(B->done, B->main));
  for (Box *b : B->boxes) {
    FE_CUDA(cudaStreamWaitEvent(b->stream, B->done, 0));
    if ((rc = check_status(b))) return rc;
  }
  return FE_OK;
}

int fe_batch_state(fe_batch *batch, int *slot_box, double *T_box, int64_t *accepted,
                   int64_t *attempted, uint64_t *attempts) {
  if (!batch) return FE_ERR_ARG;
  Batch *B = &batch->B;
  int R = B->R;
  FE_CUDA(cudaStreamSynchronize(B->main));
  if (slot_box)
    FE_CUDA(cudaMemcpy(slot_box, B->d_slot_rep, sizeof(int) * R, cudaMemcpyDeviceToHost));
  if (T_box)
    for (int r = 0; r < R; r++)
      FE_CUDA(cudaMemcpy(T_box + r, B->boxes[r]->scal + SC_TEMP, sizeof(double),
                         cudaMemcpyDeviceToHost));
  if (accepted)
    FE_CUDA(cudaMemcpy(accepted, B->d_acc, sizeof(long long) * R, cudaMemcpyDeviceToHost));
  if (attempted)
    FE_CUDA(cudaMemcpy(attempted, B->d_att, sizeof(long long) * R, cudaMemcpyDeviceToHost));
  if (attempts)
    FE_CUDA(cudaMemcpy(attempts, B->d_attempt, sizeof(unsigned long long), cudaMemcpyDeviceToHost));
  return FE_OK;
}

int fe_batch_get_stream(fe_batch *batch, void **stream) {
  if (!batch || !stream) return FE_ERR_ARG;
  *stream = (void *)batch->B.main;
  return FE_OK;
}

int fe_batch_step_launches(fe_batch *batch, int *launches4) {
  if (!batch || !launches4) return FE_ERR_ARG;
  for (int v = 0; v < 4; v++) launches4[v] = batch->B.g[v] ? batch->B.launches[v] : -1;
  return FE_OK;
}

}  // extern "C"
