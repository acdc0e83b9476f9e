// k_go.cu -- batched replica exchange of C-alpha Go-model chains: one
// persistent launch runs a whole exchange segment (thousands of Langevin
// steps) of every replica, one CTA per replica and one thread per bead.
//
// The reference's Go pair loop (cnbnd_golik, cgolik.c:644-948) walks the
// Verlet list with a dense N x N native-contact matrix (golik[k].contact)
// and a separate repulsive cut for non-native pairs; replicas are stepped
// one after another (repexch.c:139-214) and swapped by swap_box
// (swap_box.c:5-86).  Here:
//   - energy function of the chain workload: bonds k (r - r0)^2 (cbond.c
//     convention), native pairs eps [5 (r0/r)^12 - 6 (r0/r)^10] (12-10
//     attraction with its minimum -eps at the native distance r0, as in the
//     BGO branch's 12-10 form, cnonbond_nblist.c:294-307), non-native pairs
//     eps (sigma/r)^12 shifted to zero at rc (repulsion only), pairs closer
//     than min_sep along the chain excluded;
//   - the native contacts as a bitmask (N^2 bits per replica, in shared
//     memory) plus a CSR list of (partner, r0^2) for the attraction;
//   - forces in FP32, all pairs of the chain per bead (<= 1024 beads), split
//     over 1-8 adjacent threads per bead and summed by warp shuffles; no
//     atomics, fixed order;
//   - positions and velocities in FP64 registers of the owning thread for
//     the whole segment; BAOAB Langevin (Leimkuhler & Matthews 2013) with the
//     O step v = c1 v + c2 sqrt(kT/m) xi in FP64, xi Gaussian by Box-Muller
//     from Philox4x32-10 draws keyed by (bead, step);
//   - after the segment, one exchange kernel: adjacent temperature slots as
//     swap_box does (pairs alternate between attempts), acceptance
//     exp((1/kT_s - 1/kT_s+1)(U_s - U_s+1)) > u, velocity rescale by
//     sqrt(T_s/T_s+1); it also advances the device step counter, so the
//     pair (segment, exchange) is captured once as a CUDA graph and replayed.
#include <cmath>
#include <vector>

#include "fe_internal.h"
#include "fe_rng.cuh"

namespace fe {

constexpr int kGoMaxBeads = 1024;
constexpr uint32_t kRngTagGo = 0x474F4C31u;  // "GOL1"

struct GoK {
  float eps, sig2, rc2, e_shift, kb, r0b;
  double acc_fac;   // 100 / m: kJ/mol/A per amu -> A/ps^2
  double dt, c1, c2;
  double vscale;    // sqrt(100 / m): sqrt(kT [kJ/mol]) -> A/ps
  int min_sep;
  int nrep;
  int tpb;          // threads per bead (power of two)
  uint64_t seed;
};

struct GoD {
  const int *start;      // nrep + 1: first bead of each replica
  const int *maskoff;    // nrep: first mask word of each replica
  const unsigned *mask;  // native bitmask rows (N words of ceil(N/32) per replica)
  const int *nat_start;  // total + 1 (CSR over global bead index)
  const int *nat_j;      // global partner index
  const float *nat_r02;  // native distance squared
  double *x, *v;         // 3 * total
  float *f;              // 3 * total (fe_go_forces)
  double *T;             // nrep: current temperature of each replica
  double *epot;          // nrep: potential energy after the last step
  unsigned long long *step;  // steps done (drives the draws)
  // exchange
  double *Tslot;
  int *slot_rep;
  long long *acc, *att;
  unsigned long long *attempt;
};

// Force on bead i of a chain of N (positions in shared memory) from the
// partners j = sub, sub + T, sub + 2T, ... (T threads per bead, sub its
// index); natives and bonds are added by sub 0 only.  Returns this thread's
// share of the potential energy (pairs and bonds split in half).
__device__ __forceinline__ float go_force(const GoK &K, const GoD &D, const float4 *__restrict__ p,
                                          const unsigned *__restrict__ mrow, int N, int i, int sub,
                                          int T, int gbase, float &fx, float &fy, float &fz) {
  float4 pi = p[i];
  float e = 0.f;
  fx = fy = fz = 0.f;
  for (int j = sub; j < N; j += T) {
    int sep = i > j ? i - j : j - i;
    if (sep < K.min_sep) continue;
    if ((mrow[j >> 5] >> (j & 31)) & 1u) continue;  // native: below
    float4 pj = p[j];
    float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
    float r2 = dx * dx + dy * dy + dz * dz;
    if (r2 >= K.rc2) continue;
    float ri2 = __fdividef(1.f, r2);
    float s2 = K.sig2 * ri2;
    float s6 = s2 * s2 * s2;
    float s12 = s6 * s6;
    e += 0.5f * (K.eps * s12 - K.e_shift);
    float fs = 12.f * K.eps * s12 * ri2;
    fx = fmaf(fs, dx, fx);
    fy = fmaf(fs, dy, fy);
    fz = fmaf(fs, dz, fz);
  }
  if (sub != 0) return e;
  int g = gbase + i;
  for (int q = D.nat_start[g]; q < D.nat_start[g + 1]; q++) {
    int j = D.nat_j[q] - gbase;
    float4 pj = p[j];
    float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
    float r2 = dx * dx + dy * dy + dz * dz;
    float ri2 = __fdividef(1.f, r2);
    float s2 = D.nat_r02[q] * ri2;
    float s10 = s2 * s2 * s2 * s2 * s2;
    float s12 = s10 * s2;
    e += 0.5f * K.eps * (5.f * s12 - 6.f * s10);
    float fs = 60.f * K.eps * (s12 - s10) * ri2;
    fx = fmaf(fs, dx, fx);
    fy = fmaf(fs, dy, fy);
    fz = fmaf(fs, dz, fz);
  }
  for (int nb = -1; nb <= 1; nb += 2) {
    int j = i + nb;
    if (j < 0 || j >= N) continue;
    float4 pj = p[j];
    float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
    float r = sqrtf(dx * dx + dy * dy + dz * dz);
    float dr = r - K.r0b;
    e += 0.5f * K.kb * dr * dr;
    float fs = -2.f * K.kb * dr / r;
    fx = fmaf(fs, dx, fx);
    fy = fmaf(fs, dy, fy);
    fz = fmaf(fs, dz, fz);
  }
  return e;
}

// sum over the T adjacent lanes of one bead (T a power of two <= 32)
__device__ __forceinline__ float go_lane_sum(float v, int T) {
  for (int o = T >> 1; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// three standard normals for (bead, step): Box-Muller on one Philox draw
__device__ __forceinline__ void go_normals(uint64_t seed, uint32_t bead, unsigned long long step,
                                           float &z0, float &z1, float &z2) {
  Philox4 c;
  c.v[0] = bead;
  c.v[1] = (uint32_t)step;
  c.v[2] = (uint32_t)(step >> 32);
  c.v[3] = kRngTagGo;
  Philox4 r = philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  float u1 = (float)((r.v[0] >> 8) + 1u) * 0x1p-24f;  // (0, 1]
  float u2 = (float)(r.v[1] >> 8) * 0x1p-24f;
  float u3 = (float)((r.v[2] >> 8) + 1u) * 0x1p-24f;
  float u4 = (float)(r.v[3] >> 8) * 0x1p-24f;
  float ra = sqrtf(-2.f * logf(u1)), rb = sqrtf(-2.f * logf(u3));
  float s, cth;
  sincospif(2.f * u2, &s, &cth);
  z0 = ra * cth;
  z1 = ra * s;
  sincospif(2.f * u4, &s, &cth);
  z2 = rb * cth;
}

__device__ __forceinline__ double go_block_sum(double v, double *red) {
  const int tid = threadIdx.x;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((tid & 31) == 0) red[tid >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (tid == 0) {
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w];
    red[32] = s;
  }
  __syncthreads();
  return red[32];
}

// One segment of nsteps BAOAB steps of every replica (mode 0), or a single
// force evaluation into D.f (mode 1).
__global__ void __launch_bounds__(kGoMaxBeads, 1) k_go_segment(GoK K, GoD D, int nsteps, int mode) {
  extern __shared__ float4 go_pos[];
  const int r = blockIdx.x, T = K.tpb;
  const int i = threadIdx.x / T, sub = threadIdx.x % T;
  const int gbase = D.start[r], N = D.start[r + 1] - gbase;
  const int W = (N + 31) >> 5;
  unsigned *mask = (unsigned *)(go_pos + N);
  __shared__ double red[33];
  for (int t = threadIdx.x; t < N * W; t += blockDim.x) mask[t] = D.mask[D.maskoff[r] + t];
  const bool bead = i < N;          // this thread works on a bead
  const bool own = bead && sub == 0;  // ... and owns its coordinates
  double x0 = 0, x1 = 0, x2 = 0, v0 = 0, v1 = 0, v2 = 0;
  if (own) {
    const double *xp = D.x + 3 * (size_t)(gbase + i), *vp = D.v + 3 * (size_t)(gbase + i);
    x0 = xp[0];
    x1 = xp[1];
    x2 = xp[2];
    v0 = vp[0];
    v1 = vp[1];
    v2 = vp[2];
    go_pos[i] = make_float4((float)x0, (float)x1, (float)x2, 0.f);
  }
  __syncthreads();
  const unsigned *mrow = mask + (bead ? i : 0) * W;
  float fx = 0.f, fy = 0.f, fz = 0.f, e = 0.f;
  if (bead) e = go_force(K, D, go_pos, mrow, N, i, sub, T, gbase, fx, fy, fz);
  fx = go_lane_sum(fx, T);
  fy = go_lane_sum(fy, T);
  fz = go_lane_sum(fz, T);
  if (mode == 1) {
    if (own) {
      float *fp = D.f + 3 * (size_t)(gbase + i);
      fp[0] = fx;
      fp[1] = fy;
      fp[2] = fz;
    }
    double et = go_block_sum(bead ? (double)e : 0.0, red);
    if (threadIdx.x == 0) D.epot[r] = et;
    return;
  }
  const unsigned long long step0 = *D.step;
  const double kT = ((kKB * kNA) * D.T[r]) * .001;  // read_sim.c:351, kJ/mol
  const double sv = K.vscale * sqrt(kT) * K.c2;
  const double hdt = 0.5 * K.dt, ha = 0.5 * K.dt * K.acc_fac;
  for (int s = 0; s < nsteps; s++) {
    if (own) {
      // B, A, O, A
      v0 += ha * fx;
      v1 += ha * fy;
      v2 += ha * fz;
      x0 += hdt * v0;
      x1 += hdt * v1;
      x2 += hdt * v2;
      float z0, z1, z2;
      go_normals(K.seed, (uint32_t)(gbase + i), step0 + s, z0, z1, z2);
      v0 = K.c1 * v0 + sv * z0;
      v1 = K.c1 * v1 + sv * z1;
      v2 = K.c1 * v2 + sv * z2;
      x0 += hdt * v0;
      x1 += hdt * v1;
      x2 += hdt * v2;
    }
    __syncthreads();  // everyone is done reading the old positions
    if (own) go_pos[i] = make_float4((float)x0, (float)x1, (float)x2, 0.f);
    __syncthreads();
    if (bead) e = go_force(K, D, go_pos, mrow, N, i, sub, T, gbase, fx, fy, fz);
    fx = go_lane_sum(fx, T);
    fy = go_lane_sum(fy, T);
    fz = go_lane_sum(fz, T);
    if (own) {
      v0 += ha * fx;  // B
      v1 += ha * fy;
      v2 += ha * fz;
    }
  }
  if (own) {
    double *xp = D.x + 3 * (size_t)(gbase + i), *vp = D.v + 3 * (size_t)(gbase + i);
    xp[0] = x0;
    xp[1] = x1;
    xp[2] = x2;
    vp[0] = v0;
    vp[1] = v1;
    vp[2] = v2;
  }
  double et = go_block_sum(bead ? (double)e : 0.0, red);
  if (threadIdx.x == 0) D.epot[r] = et;
}

// Advances the step counter by nsteps; when `exchange`, one swap_box attempt
// over the temperature slots and the velocity rescale of swapped replicas.
__global__ void k_go_exchange(GoD D, int nrep, int nsteps, int exchange, uint64_t seed) {
  __shared__ int vmode[kGoMaxBeads];
  __shared__ double vfac[kGoMaxBeads];
  __shared__ unsigned long long attempt;
  const int tid = threadIdx.x;
  if (tid == 0) {
    *D.step += (unsigned long long)nsteps;
    attempt = *D.attempt;
  }
  for (int q = tid; q < nrep; q += blockDim.x) vmode[q] = 0;
  __syncthreads();
  if (!exchange) return;
  int parity = (int)(attempt & 1ull);
  for (int t = tid;; t += blockDim.x) {
    int s = parity + 2 * t;
    if (s + 1 >= nrep) break;
    int r1 = D.slot_rep[s], r2 = D.slot_rep[s + 1];
    double kT1 = ((kKB * kNA) * D.Tslot[s]) * .001, kT2 = ((kKB * kNA) * D.Tslot[s + 1]) * .001;
    double crit = exp((1.0 / kT1 - 1.0 / kT2) * (D.epot[r1] - D.epot[r2]));
    D.att[s] += 1;
    if (crit > fe_uniform(seed, kRngTagExchange, attempt, (uint32_t)s)) {
      D.acc[s] += 1;
      D.slot_rep[s] = r2;
      D.slot_rep[s + 1] = r1;
      double f = sqrt(D.Tslot[s] / D.Tslot[s + 1]);
      vmode[r2] = 1;
      vfac[r2] = f;
      vmode[r1] = 2;
      vfac[r1] = f;
      D.T[r2] = D.Tslot[s];
      D.T[r1] = D.Tslot[s + 1];
    }
  }
  __syncthreads();
  if (tid == 0) *D.attempt = attempt + 1ull;
  for (int q = 0; q < nrep; q++) {
    if (!vmode[q]) continue;
    int a = D.start[q], b = D.start[q + 1];
    for (int t = 3 * a + tid; t < 3 * b; t += blockDim.x)
      D.v[t] = vmode[q] == 1 ? D.v[t] * vfac[q] : D.v[t] / vfac[q];
  }
}

struct GoBatch {
  int nrep = 0, total = 0, maxN = 0, dev = 0;
  GoK K{};
  GoD D{};
  size_t smem = 0;
  cudaStream_t st = nullptr;
  cudaGraphExec_t g = nullptr;
  int g_len = -1;
  uint64_t seed = 0;
  std::vector<void *> allocs;
};

static void go_free(GoBatch *G) {
  if (G->g) cudaGraphExecDestroy(G->g);
  for (void *p : G->allocs) cudaFree(p);
  if (G->st) cudaStreamDestroy(G->st);
}

template <typename T>
static int go_upload(GoBatch *G, T **dst, const T *src, size_t n) {
  FE_CUDA(cudaMalloc((void **)dst, sizeof(T) * (n ? n : 1)));
  G->allocs.push_back((void *)*dst);
  if (src && n) FE_CUDA(cudaMemcpy((void *)*dst, src, sizeof(T) * n, cudaMemcpyHostToDevice));
  return FE_OK;
}

// threads per bead: as many as fit the longest chain into 1024 threads (a
// power of two, at most 8); the block is rounded up to whole warps
static int go_tpb(int maxN) {
  int t = 1;
  while (t < 8 && 2 * t * maxN <= kGoMaxBeads) t *= 2;
  return t;
}
static int go_threads(const GoBatch *G) { return ((G->maxN * G->K.tpb + 31) / 32) * 32; }

static int go_launch_segment(GoBatch *G, int nsteps, int exchange) {
  k_go_segment<<<G->nrep, go_threads(G), G->smem, G->st>>>(G->K, G->D, nsteps, 0);
  FE_LAUNCH_CHECK("k_go_segment");
  k_go_exchange<<<1, 256, 0, G->st>>>(G->D, G->nrep, nsteps, exchange, G->seed);
  FE_LAUNCH_CHECK("k_go_exchange");
  return FE_OK;
}

}  // namespace fe

using namespace fe;

struct fe_go {
  GoBatch G;
};

extern "C" {

int fe_go_create(fe_go **out, int nrep, const int *nbeads, const double *pos, const double *vel,
                 const int *nat_start, const int *nat_j, const double *nat_r0, const double *T,
                 const fe_go_params *p, uint64_t seed) {
  if (!out || nrep < 1 || nrep > kGoMaxBeads || !nbeads || !pos || !vel || !nat_start ||
      !nat_j || !nat_r0 || !T || !p) {
    set_error("fe_go_create: invalid argument");
    return FE_ERR_ARG;
  }
  *out = nullptr;
  std::vector<int> start(nrep + 1, 0), maskoff(nrep, 0);
  int maxN = 0;
  for (int r = 0; r < nrep; r++) {
    if (nbeads[r] < 2 || nbeads[r] > kGoMaxBeads) {
      set_error("fe_go_create: chains need 2..1024 beads");
      return FE_ERR_SIZE;
    }
    start[r + 1] = start[r] + nbeads[r];
    if (nbeads[r] > maxN) maxN = nbeads[r];
  }
  int total = start[nrep];
  // native bitmask rows, checking that natives stay inside their chain
  std::vector<unsigned> mask;
  std::vector<float> r02(nat_start[total]);
  for (int r = 0; r < nrep; r++) {
    int N = nbeads[r], W = (N + 31) / 32;
    maskoff[r] = (int)mask.size();
    mask.resize(mask.size() + (size_t)N * W, 0u);
    for (int i = 0; i < N; i++) {
      int gi = start[r] + i;
      for (int q = nat_start[gi]; q < nat_start[gi + 1]; q++) {
        int j = nat_j[q] - start[r];
        if (j < 0 || j >= N || j == i) {
          set_error("fe_go_create: a native partner lies outside its chain");
          return FE_ERR_ARG;
        }
        mask[maskoff[r] + (size_t)i * W + (j >> 5)] |= 1u << (j & 31);
        r02[q] = (float)(nat_r0[q] * nat_r0[q]);
      }
    }
  }
  fe_go *h = new fe_go();
  GoBatch *G = &h->G;
  G->nrep = nrep;
  G->total = total;
  G->maxN = maxN;
  G->dev = p->device;
  G->seed = seed;
  GoK &K = G->K;
  K.eps = (float)p->eps;
  K.sig2 = (float)(p->sigma_rep * p->sigma_rep);
  K.rc2 = (float)(p->rc_rep * p->rc_rep);
  double sr = p->sigma_rep / p->rc_rep, sr6 = sr * sr * sr * sr * sr * sr;
  K.e_shift = (float)(p->eps * sr6 * sr6);
  K.kb = (float)p->k_bond;
  K.r0b = (float)p->r_bond;
  K.acc_fac = 100.0 / p->mass;
  K.vscale = sqrt(100.0 / p->mass);
  K.dt = p->dt;
  K.c1 = exp(-p->gamma * p->dt);
  K.c2 = sqrt(1.0 - K.c1 * K.c1);
  K.min_sep = p->min_sep < 1 ? 1 : p->min_sep;
  K.nrep = nrep;
  K.tpb = go_tpb(maxN);
  K.seed = seed;
  int rc = FE_OK;
  std::vector<int> slot(nrep);
  for (int r = 0; r < nrep; r++) slot[r] = r;
  do {
    if (cudaSetDevice(G->dev) != cudaSuccess) {
      rc = cuda_fail(cudaGetLastError(), "cudaSetDevice");
      break;
    }
    if (cudaStreamCreateWithFlags(&G->st, cudaStreamNonBlocking) != cudaSuccess) {
      rc = cuda_fail(cudaGetLastError(), "cudaStreamCreate");
      break;
    }
    GoD &D = G->D;
    if ((rc = go_upload(G, (int **)&D.start, start.data(), start.size()))) break;
    if ((rc = go_upload(G, (int **)&D.maskoff, maskoff.data(), maskoff.size()))) break;
    if ((rc = go_upload(G, (unsigned **)&D.mask, mask.data(), mask.size()))) break;
    if ((rc = go_upload(G, (int **)&D.nat_start, nat_start, (size_t)total + 1))) break;
    if ((rc = go_upload(G, (int **)&D.nat_j, nat_j, (size_t)nat_start[total]))) break;
    if ((rc = go_upload(G, (float **)&D.nat_r02, r02.data(), r02.size()))) break;
    if ((rc = go_upload(G, &D.x, pos, 3 * (size_t)total))) break;
    if ((rc = go_upload(G, &D.v, vel, 3 * (size_t)total))) break;
    if ((rc = go_upload(G, &D.f, (const float *)nullptr, 3 * (size_t)total))) break;
    if ((rc = go_upload(G, &D.T, T, (size_t)nrep))) break;
    if ((rc = go_upload(G, &D.Tslot, T, (size_t)nrep))) break;
    if ((rc = go_upload(G, &D.epot, (const double *)nullptr, (size_t)nrep))) break;
    if ((rc = go_upload(G, &D.slot_rep, slot.data(), (size_t)nrep))) break;
    std::vector<long long> z(nrep, 0);
    if ((rc = go_upload(G, &D.acc, z.data(), (size_t)nrep))) break;
    if ((rc = go_upload(G, &D.att, z.data(), (size_t)nrep))) break;
    unsigned long long zero = 0;
    if ((rc = go_upload(G, &D.step, &zero, 1))) break;
    if ((rc = go_upload(G, &D.attempt, &zero, 1))) break;
    G->smem = sizeof(float4) * (size_t)maxN + sizeof(unsigned) * (size_t)maxN * ((maxN + 31) / 32);
    if (cudaFuncSetAttribute(k_go_segment, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)G->smem) != cudaSuccess) {
      rc = cuda_fail(cudaGetLastError(), "cudaFuncSetAttribute");
      break;
    }
  } while (0);
  if (rc) {
    go_free(G);
    delete h;
    return rc;
  }
  *out = h;
  return FE_OK;
}

void fe_go_destroy(fe_go *h) {
  if (!h) return;
  if (h->G.st) cudaStreamSynchronize(h->G.st);
  go_free(&h->G);
  delete h;
}

int fe_go_run(fe_go *h, int64_t nsteps, int swap_freq) {
  if (!h || nsteps < 0 || swap_freq < 0) return FE_ERR_ARG;
  GoBatch *G = &h->G;
  int rc;
  if (swap_freq > 0) {
    if (G->g_len != swap_freq) {
      if (G->g) cudaGraphExecDestroy(G->g);
      G->g = nullptr;
      cudaGraph_t gr;
      FE_CUDA(cudaStreamBeginCapture(G->st, cudaStreamCaptureModeThreadLocal));
      rc = go_launch_segment(G, swap_freq, 1);
      cudaError_t e = cudaStreamEndCapture(G->st, &gr);
      if (rc) return rc;
      if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
      e = cudaGraphInstantiate(&G->g, gr, 0);
      cudaGraphDestroy(gr);
      if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
      G->g_len = swap_freq;
    }
    int64_t full = nsteps / swap_freq;
    for (int64_t s = 0; s < full; s++) FE_CUDA(cudaGraphLaunch(G->g, G->st));
    int rest = (int)(nsteps - full * swap_freq);
    if (rest && (rc = go_launch_segment(G, rest, 0))) return rc;
  } else if (nsteps > 0) {
    if ((rc = go_launch_segment(G, (int)nsteps, 0))) return rc;
  }
  FE_CUDA(cudaStreamSynchronize(G->st));
  return FE_OK;
}

int fe_go_forces(fe_go *h, double *f, double *epot) {
  if (!h) return FE_ERR_ARG;
  GoBatch *G = &h->G;
  k_go_segment<<<G->nrep, go_threads(G), G->smem, G->st>>>(G->K, G->D, 0, 1);
  FE_LAUNCH_CHECK("k_go_segment");
  FE_CUDA(cudaStreamSynchronize(G->st));
  if (f) {
    std::vector<float> t(3 * (size_t)G->total);
    FE_CUDA(cudaMemcpy(t.data(), G->D.f, sizeof(float) * t.size(), cudaMemcpyDeviceToHost));
    for (size_t q = 0; q < t.size(); q++) f[q] = t[q];
  }
  if (epot) FE_CUDA(cudaMemcpy(epot, G->D.epot, sizeof(double) * G->nrep, cudaMemcpyDeviceToHost));
  return FE_OK;
}

int fe_go_state(fe_go *h, double *pos, double *vel, double *T, double *epot, int *slot_rep,
                int64_t *accepted, int64_t *attempted, uint64_t *steps) {
  if (!h) return FE_ERR_ARG;
  GoBatch *G = &h->G;
  FE_CUDA(cudaStreamSynchronize(G->st));
  size_t n3 = 3 * (size_t)G->total;
  if (pos) FE_CUDA(cudaMemcpy(pos, G->D.x, sizeof(double) * n3, cudaMemcpyDeviceToHost));
  if (vel) FE_CUDA(cudaMemcpy(vel, G->D.v, sizeof(double) * n3, cudaMemcpyDeviceToHost));
  if (T) FE_CUDA(cudaMemcpy(T, G->D.T, sizeof(double) * G->nrep, cudaMemcpyDeviceToHost));
  if (epot) FE_CUDA(cudaMemcpy(epot, G->D.epot, sizeof(double) * G->nrep, cudaMemcpyDeviceToHost));
  if (slot_rep)
    FE_CUDA(cudaMemcpy(slot_rep, G->D.slot_rep, sizeof(int) * G->nrep, cudaMemcpyDeviceToHost));
  if (accepted)
    FE_CUDA(cudaMemcpy(accepted, G->D.acc, sizeof(long long) * G->nrep, cudaMemcpyDeviceToHost));
  if (attempted)
    FE_CUDA(cudaMemcpy(attempted, G->D.att, sizeof(long long) * G->nrep, cudaMemcpyDeviceToHost));
  if (steps) FE_CUDA(cudaMemcpy(steps, G->D.step, sizeof(unsigned long long), cudaMemcpyDeviceToHost));
  return FE_OK;
}

int fe_go_get_stream(fe_go *h, void **stream) {
  if (!h || !stream) return FE_ERR_ARG;
  *stream = (void *)h->G.st;
  return FE_OK;
}

}  // extern "C"
