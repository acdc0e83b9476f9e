// k_mcrun.cu -- Monte Carlo chains resident on the GPU: rigid-molecule
// translation and rotation moves with the exact classic-Ewald energy change,
// many moves per launch, one CTA per chain.
//
// The reference's MC (nvt_mc.c:70-422, mcmove_displ.c:33-139,
// mcmove_trans.c:46-182) picks a move on the host, recomputes energies with
// forces_mc / ewald_kspace_mc (ewald_mc.c:42-324) and applies the Metropolis
// rule "arg = (U_i - U_f) beta; accept if arg > 0 or exp(arg) > ran2()".
// Here each chain is one CTA that keeps its whole state in shared memory
// and registers for a launch of thousands of sequential moves:
//   - site coordinates as 32-bit fixed-point fractions of the box (int4:
//     x, y, z, charge bits), so a wrapped integer difference is the exact
//     minimum image and a move never needs a periodic wrap;
//   - the structure factor S(k) of the k-vectors of ewald_setup
//     (ewald.c:104-118, |n|^2 <= max_k_square), one k-vector per thread, kept
//     in registers for the whole launch as a float pair (hi + lo);
//   - k.r phases as exact 32-bit integers (k_x u_x + k_y u_y + k_z u_z mod
//     2^32 is the phase in units of 2 pi / 2^32), reduced to a quarter turn
//     before one FP32 sincospi;
//   - pair energies (shifted LJ within rc, unshifted erfc real-space Ewald
//     within rc_ew, the reference's erfc fit, ewald.c:817) in FP32, summed
//     per thread and reduced in a fixed order (deterministic).
// A move: thread 0 draws it (Philox4x32-10, counter = chain and move
// number), all threads evaluate dE_real over every other site and dE_k over
// their k-vector, a block reduction gives dE, thread 0 applies the
// Metropolis rule, and an accepted move updates S and the coordinates.
// Intramolecular pairs do not change under rigid moves and are skipped; the
// setup checks that every excluded pair lies inside one molecule.
#include <cmath>
#include <cstring>
#include <vector>

#include "fe_internal.h"
#include "fe_rng.cuh"

namespace fe {

constexpr int kMccThreads = 1024;
constexpr int kMccMaxSites = 8;   // sites per molecule
constexpr int kMccMaxTypes = 8;
constexpr int kMccMaxK = kMccThreads;  // one k-vector per thread
constexpr int kMccMaxN = 10240;   // sites per chain (shared-memory state)
constexpr int kMccLogD = 12;      // doubles per logged move
constexpr int kMlpInputs = 64, kMlpHidden = 128;  // surrogate network (k_mlp.cu)
// b1, b2, w3, b3, input mean, input 1/std
constexpr int kMlpFb = 3 * kMlpHidden + 1 + 2 * kMlpInputs;
constexpr long long kMccChunk = 16384;  // moves per launch

struct MccParams {
  int n, nmol, nk, nt;
  float sLf[3];      // L / 2^32 per axis
  double sLd[3];
  float rc2, rce2, kappa, fconv;
  float ron2, inv_sw_den;  // LJ switch (ron2 = 0: the reference's shift, lj[2])
  double beta;       // 1 / kT [mol/kJ], kT = RG T / 1000 (read_sim.c:351)
  double delta;      // translation (u - 0.5) * delta per axis (mcmove_displ.c:92-94)
  double rot_max;    // rotation angle in [-rot_max, rot_max] about the centre of mass
  double p_rot;      // probability that a move is a rotation
  uint64_t seed;
  int log_cap;
  int mode;          // 0: exact dE; 1: delayed acceptance with the surrogate
  int full;          // 1: the reciprocal change recomputed from every site (the reference's cost)
  int desc;          // descriptors computed (mode 1 or sample collection)
  int collect;       // store (descriptors, exact dE_k) samples in mode 0
  long long sample_cap;  // samples per chain
};

struct MccDev {
  int4 *posfx;              // nchains * n
  double2 *S;               // nchains * nk
  const int4 *kv;           // nk: kx, ky, kz
  const double *ck;         // nk: multiplicity * kvec * fconv
  const int *mol_first;     // nmol + 1
  const unsigned char *type;  // n
  const float *mass;        // n
  const float *lj;          // nt * nt * 3: eps, sig^2, energy at rc
  long long *moves, *accepted;  // nchains
  double *log;              // log_cap * kMccLogD (chain 0)
  unsigned *log_fx;         // log_cap * kMccMaxSites * 3
  long long *stats;         // nchains * 2: stage-1 accepts, exact k-space evaluations
  float *samples;           // nchains * sample_cap * 129
  long long *nsamples;      // nchains
  const unsigned short *w1t;  // surrogate, bf16: W1 (input-normalised) transposed [64][128]
  const unsigned short *w2t;  // W2 transposed [128][128]
  const float *fb;          // b1, b2, w3, b3, input mean, input 1/std
};

struct McChains {
  int nchains = 0;
  MccParams P{};
  MccDev D{};
  int kmax = 0, mks = 0;
  double rc_ew = 0.0;
  std::vector<int> mol_first;
};

// the reference's erfc fit (ewald.c:817-836) in FP32, with exp(-z^2) given
__device__ __forceinline__ float mcc_erfc(float z, float ex) {
  float t = __fdividef(1.0f, 1.0f + 0.5f * z);
  float p = fmaf(t, 0.17087277f, -0.82215223f);
  p = fmaf(t, p, 1.48851587f);
  p = fmaf(t, p, -1.13520398f);
  p = fmaf(t, p, 0.27886807f);
  p = fmaf(t, p, -0.18628806f);
  p = fmaf(t, p, 0.09678418f);
  p = fmaf(t, p, 0.37409196f);
  p = fmaf(t, p, 1.00002368f);
  p = fmaf(t, p, -1.26551223f);
  return t * ex * __expf(p);
}

// exp(i 2 pi ph / 2^32): nearest quarter turn exactly, the rest by sincospi
__device__ __forceinline__ void phase_sincos(uint32_t ph, float &s, float &c) {
  uint32_t q = (ph + 0x20000000u) >> 30;
  int32_t r = (int32_t)(ph - (q << 30));  // in [-2^29, 2^29)
  float sr, cr;
  sincospif((float)r * 0x1p-31f, &sr, &cr);
  switch (q & 3u) {
    case 0: s = sr; c = cr; break;
    case 1: s = cr; c = -sr; break;
    case 2: s = -sr; c = -cr; break;
    default: s = -cr; c = sr; break;
  }
}

// energy of one pair at squared distance r2 (shifted or switched LJ +
// real-space Ewald)
__device__ __forceinline__ float mcc_pair(const MccParams &P, float r2, float qq,
                                          const float *lj) {
  float e = 0.f;
  if (r2 <= P.rce2 && qq != 0.f) {
    float r = sqrtf(r2);
    float kr = P.kappa * r;
    e = qq * mcc_erfc(kr, __expf(-kr * kr)) / r;
  }
  if (r2 <= P.rc2 && lj[0] != 0.f) {
    float sr2 = lj[1] / r2;
    float sr6 = sr2 * sr2 * sr2;
    float elj = lj[0] * (sr6 * sr6 - 2.f * sr6) - lj[2];
    if (r2 > P.ron2 && P.ron2 > 0.f) {
      float c = P.rc2 - r2;
      elj *= c * c * (P.rc2 + 2.f * r2 - 3.f * P.ron2) * P.inv_sw_den;
    }
    e += elj;
  }
  return e;
}

__device__ __forceinline__ float u32_uniform_f(uint32_t w) { return (float)(w >> 8) * 0x1p-24f; }

// error-free sum of two floats (Knuth TwoSum): s + e == a + b exactly
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// S(k) as an unevaluated float pair hi + lo (about 48 bits): adds a float
__device__ __forceinline__ void ff_add(float &hi, float &lo, float x) {
  float s, e;
  two_sum(hi, x, s, e);
  e += lo;
  hi = s + e;
  lo = e - (hi - s);
}

__device__ __forceinline__ float bf16_to_f(unsigned short h) {
  return __uint_as_float((uint32_t)h << 16);
}

__device__ __forceinline__ float silu_f(float z) { return z / (1.f + __expf(-z)); }

// Block-wide sums of two floats in a fixed order; every thread gets both.
__device__ __forceinline__ void block_sum2(float &a, float &b, float *ra, float *rb) {
  const int tid = threadIdx.x;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  if ((tid & 31) == 0) {
    ra[tid >> 5] = a;
    rb[tid >> 5] = b;
  }
  __syncthreads();
  if (tid < 32) {
    a = tid < (int)(blockDim.x >> 5) ? ra[tid] : 0.f;
    b = tid < (int)(blockDim.x >> 5) ? rb[tid] : 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if (tid == 0) {
      ra[32] = a;
      rb[32] = b;
    }
  }
  __syncthreads();
  a = ra[32];
  b = rb[32];
}

// Descriptor bin of a pair at distance r: tent functions centred at
// kDescR0 + k * kDescDr (k = 0..15), weighted by the partner's charge.
constexpr float kDescR0 = 1.0f, kDescDr = 0.5f, kDescRmax = 9.0f, kDescScale = 65536.f;

// All per-move arithmetic is FP32 (GB300's FP64 rate is a small fraction of
// its FP32 rate): pair energies, phases, the block reductions, the proposal
// and the Metropolis tests.  S(k) is carried as a float pair so that
// thousands of accepted increments do not drift.
__global__ void __launch_bounds__(kMccThreads, 1)
k_mcc_run(MccParams P, MccDev D, long long nmoves) {
  extern __shared__ int4 sm_pos[];  // n
  unsigned char *sm_typ = (unsigned char *)(sm_pos + P.n);
  float *sm_lj = (float *)(sm_typ + ((P.n + 15) & ~15));
  int *sm_cand = (int *)(sm_lj + ((P.nt * P.nt * 3 + 3) & ~3));  // 32 * chunk
  const int chunk = ((P.n + 31) / 32 + 31) & ~31;                   // sites per warp
  int *sm_hist = sm_cand + 32 * chunk;                               // 32 x 128 (descriptors)
  unsigned short *sm_w1t = (unsigned short *)(sm_hist + (P.desc ? 32 * 2 * kMlpInputs : 0));
  unsigned short *sm_w2t = sm_w1t + kMlpInputs * kMlpHidden;
  float *sm_fb = (float *)(sm_w2t + kMlpHidden * kMlpHidden);       // kMlpFb floats
  __shared__ unsigned mv_old[kMccMaxSites][3], mv_new[kMccMaxSites][3];
  __shared__ float mv_q[kMccMaxSites];
  __shared__ int mv_t[kMccMaxSites];
  __shared__ int mv_lb, mv_m, mv_rot, decision, stage1;
  __shared__ float mv_u, mv_u2, mv_scr2;
  __shared__ float red_a[33], red_b[33];
  __shared__ int cand_cnt[32], cand_off[33];
  __shared__ float sm_desc[2][kMlpInputs];
  __shared__ float sm_h1[2][kMlpHidden];

  const int chain = blockIdx.x;
  const int tid = threadIdx.x;
  int4 *gpos = D.posfx + (size_t)chain * P.n;
  for (int i = tid; i < P.n; i += blockDim.x) {
    sm_pos[i] = gpos[i];
    sm_typ[i] = D.type[i];
  }
  for (int i = tid; i < P.nt * P.nt * 3; i += blockDim.x) sm_lj[i] = D.lj[i];
  if (P.desc)
    for (int i = tid; i < 32 * 2 * kMlpInputs; i += blockDim.x) sm_hist[i] = 0;
  if (P.mode == 1) {
    for (int i = tid; i < kMlpInputs * kMlpHidden; i += blockDim.x) sm_w1t[i] = D.w1t[i];
    for (int i = tid; i < kMlpHidden * kMlpHidden; i += blockDim.x) sm_w2t[i] = D.w2t[i];
    for (int i = tid; i < kMlpFb; i += blockDim.x) sm_fb[i] = D.fb[i];
  }
  int kx = 0, ky = 0, kz = 0;
  float ck = 0.f, Sxh = 0.f, Sxl = 0.f, Syh = 0.f, Syl = 0.f;
  if (tid < P.nk) {
    int4 k = D.kv[tid];
    kx = k.x;
    ky = k.y;
    kz = k.z;
    ck = (float)D.ck[tid];
    double2 S = D.S[(size_t)chain * P.nk + tid];
    Sxh = (float)S.x;
    Sxl = (float)(S.x - (double)Sxh);
    Syh = (float)S.y;
    Syl = (float)(S.y - (double)Syh);
  }
  const float invx = 1.0f / P.sLf[0], invy = 1.0f / P.sLf[1], invz = 1.0f / P.sLf[2];
  const float beta = (float)P.beta;
  long long move0 = D.moves[chain];
  long long nacc = 0, n_s1 = 0, n_k = 0;
  long long nsamp = P.collect ? D.nsamples[chain] : 0;
  __syncthreads();

  for (long long it = 0; it < nmoves; ++it) {
    long long mv = move0 + it;
    // ---- propose (thread 0) ----
    if (tid == 0) {
      Philox4 c0, c1;
      c0.v[0] = c1.v[0] = (uint32_t)chain;
      c0.v[1] = c1.v[1] = (uint32_t)mv;
      c0.v[2] = c1.v[2] = (uint32_t)((unsigned long long)mv >> 32);
      c0.v[3] = kRngTagMC;
      c1.v[3] = kRngTagMC + 1u;
      Philox4 r0 = philox4x32_10(c0, (uint32_t)P.seed, (uint32_t)(P.seed >> 32));
      Philox4 r1 = philox4x32_10(c1, (uint32_t)P.seed, (uint32_t)(P.seed >> 32));
      int mol = (int)(((unsigned long long)r0.v[0] * (unsigned)P.nmol) >> 32);
      int lb = D.mol_first[mol], m = D.mol_first[mol + 1] - lb;
      int rot = (m > 1 && u32_uniform_f(r0.v[1]) < (float)P.p_rot) ? 1 : 0;
      int4 p0 = sm_pos[lb];
      unsigned u0x = (unsigned)p0.x, u0y = (unsigned)p0.y, u0z = (unsigned)p0.z;
      for (int i = 0; i < m; i++) {
        int4 p = sm_pos[lb + i];
        mv_old[i][0] = (unsigned)p.x;
        mv_old[i][1] = (unsigned)p.y;
        mv_old[i][2] = (unsigned)p.z;
        mv_q[i] = __int_as_float(p.w);
        mv_t[i] = sm_typ[lb + i];
      }
      if (rot) {
        // site offsets from site 0 (exact minimum image), centre of mass
        float rel[kMccMaxSites][3];
        float cx = 0.f, cy = 0.f, cz = 0.f, msum = 0.f;
        for (int i = 0; i < m; i++) {
          rel[i][0] = (float)(int)(mv_old[i][0] - u0x) * P.sLf[0];
          rel[i][1] = (float)(int)(mv_old[i][1] - u0y) * P.sLf[1];
          rel[i][2] = (float)(int)(mv_old[i][2] - u0z) * P.sLf[2];
          float w = D.mass[lb + i];
          cx = fmaf(w, rel[i][0], cx);
          cy = fmaf(w, rel[i][1], cy);
          cz = fmaf(w, rel[i][2], cz);
          msum += w;
        }
        cx /= msum;
        cy /= msum;
        cz /= msum;
        // uniform axis (cos theta uniform, phi uniform), angle uniform in [-max, max]
        float cth = 2.f * u32_uniform_f(r0.v[2]) - 1.f;
        float sph, cph;
        sincospif(2.f * u32_uniform_f(r0.v[3]), &sph, &cph);
        float sth = sqrtf(fmaxf(0.f, 1.f - cth * cth));
        float ax = sth * cph, ay = sth * sph, az = cth;
        float ang = (2.f * u32_uniform_f(r1.v[2]) - 1.f) * (float)P.rot_max;
        float sa, ca;
        sincosf(ang, &sa, &ca);
        float t = 1.f - ca;
        float R00 = t * ax * ax + ca, R01 = t * ax * ay - sa * az, R02 = t * ax * az + sa * ay;
        float R10 = t * ax * ay + sa * az, R11 = t * ay * ay + ca, R12 = t * ay * az - sa * ax;
        float R20 = t * ax * az - sa * ay, R21 = t * ay * az + sa * ax, R22 = t * az * az + ca;
        for (int i = 0; i < m; i++) {
          float dx = rel[i][0] - cx, dy = rel[i][1] - cy, dz = rel[i][2] - cz;
          float nx = cx + R00 * dx + R01 * dy + R02 * dz;
          float ny = cy + R10 * dx + R11 * dy + R12 * dz;
          float nz = cz + R20 * dx + R21 * dy + R22 * dz;
          mv_new[i][0] = u0x + (unsigned)__float2int_rn(nx * invx);
          mv_new[i][1] = u0y + (unsigned)__float2int_rn(ny * invy);
          mv_new[i][2] = u0z + (unsigned)__float2int_rn(nz * invz);
        }
      } else {
        // one integer shift for every site: the molecule stays exactly rigid
        float dlt = (float)P.delta;
        unsigned sx = (unsigned)__float2int_rn((u32_uniform_f(r0.v[2]) - 0.5f) * dlt * invx);
        unsigned sy = (unsigned)__float2int_rn((u32_uniform_f(r0.v[3]) - 0.5f) * dlt * invy);
        unsigned sz = (unsigned)__float2int_rn((u32_uniform_f(r1.v[2]) - 0.5f) * dlt * invz);
        for (int i = 0; i < m; i++) {
          mv_new[i][0] = mv_old[i][0] + sx;
          mv_new[i][1] = mv_old[i][1] + sy;
          mv_new[i][2] = mv_old[i][2] + sz;
        }
      }
      // candidates: sites within max(rc, rc_ew) + the molecule's extent of site 0
      float ext2 = 0.f;
      for (int i = 1; i < m; i++) {
        float ex = (float)(int)(mv_old[i][0] - u0x) * P.sLf[0];
        float ey = (float)(int)(mv_old[i][1] - u0y) * P.sLf[1];
        float ez = (float)(int)(mv_old[i][2] - u0z) * P.sLf[2];
        ext2 = fmaxf(ext2, ex * ex + ey * ey + ez * ez);
      }
      float rs = sqrtf(fmaxf(P.rc2, P.rce2)) + sqrtf(ext2) + 0.01f;
      mv_scr2 = rs * rs;
      mv_lb = lb;
      mv_m = m;
      mv_rot = rot;
      mv_u = u32_uniform_f(r1.v[0]);
      mv_u2 = u32_uniform_f(r1.v[1]);
    }
    __syncthreads();
    const int lb = mv_lb, m = mv_m;
    // ---- real space, pass 1: sites near the molecule (old or new place) ----
    // Each warp scans a fixed chunk of sites and appends candidates to its
    // own segment in scan order, so the candidate order never depends on
    // timing and the sums below stay deterministic.
    {
      const int w = tid >> 5, l = tid & 31;
      const int j0 = w * chunk;
      int cnt = 0;
      for (int jj = 0; jj < chunk; jj += 32) {
        int j = j0 + jj + l;
        bool c = false;
        if (j < P.n && (j < lb || j >= lb + m)) {
          int4 pj = sm_pos[j];
          float dx = (float)(int)(mv_old[0][0] - (unsigned)pj.x) * P.sLf[0];
          float dy = (float)(int)(mv_old[0][1] - (unsigned)pj.y) * P.sLf[1];
          float dz = (float)(int)(mv_old[0][2] - (unsigned)pj.z) * P.sLf[2];
          float r2o = dx * dx + dy * dy + dz * dz;
          dx = (float)(int)(mv_new[0][0] - (unsigned)pj.x) * P.sLf[0];
          dy = (float)(int)(mv_new[0][1] - (unsigned)pj.y) * P.sLf[1];
          dz = (float)(int)(mv_new[0][2] - (unsigned)pj.z) * P.sLf[2];
          float r2n = dx * dx + dy * dy + dz * dz;
          c = r2o <= mv_scr2 || r2n <= mv_scr2;
        }
        unsigned bal = __ballot_sync(0xffffffffu, c);
        if (c) sm_cand[j0 + cnt + __popc(bal & ((1u << l) - 1u))] = j;
        cnt += __popc(bal);
      }
      if (l == 0) cand_cnt[w] = cnt;
    }
    __syncthreads();
    if (tid < 32) {
      int c = cand_cnt[tid], x = c;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (tid >= o) x += y;
      }
      cand_off[tid] = x - c;
      if (tid == 31) cand_off[32] = x;
    }
    __syncthreads();
    // ---- real space, pass 2: (candidate, site, old/new) items over all threads ----
    float de = 0.f;
    {
      int *hist = sm_hist + (tid >> 5) * 2 * kMlpInputs;
      const int per = 2 * m, items = cand_off[32] * per;
      for (int t = tid; t < items; t += blockDim.x) {
        int ci = t / per, rest = t - ci * per;
        int i = rest >> 1, isnew = rest & 1;
        int w = 0;
#pragma unroll
        for (int step = 16; step > 0; step >>= 1)
          if (w + step < 32 && cand_off[w + step] <= ci) w += step;
        int j = sm_cand[w * chunk + (ci - cand_off[w])];
        int4 pj = sm_pos[j];
        float qj = __int_as_float(pj.w);
        const float *lj = sm_lj + (mv_t[i] * P.nt + sm_typ[j]) * 3;
        float qq = mv_q[i] * qj * P.fconv;
        const unsigned *u = isnew ? mv_new[i] : mv_old[i];
        float dx = (float)(int)(u[0] - (unsigned)pj.x) * P.sLf[0];
        float dy = (float)(int)(u[1] - (unsigned)pj.y) * P.sLf[1];
        float dz = (float)(int)(u[2] - (unsigned)pj.z) * P.sLf[2];
        float r2 = dx * dx + dy * dy + dz * dz;
        if (r2 <= P.rce2 || r2 <= P.rc2) {
          float e = mcc_pair(P, r2, qq, lj);
          de += isnew ? e : -e;
        }
        if (P.desc && r2 < kDescRmax * kDescRmax) {
          // 4 channels (site charge sign x partner charge sign) x 16 tents
          float x = (sqrtf(r2) - kDescR0) * (1.f / kDescDr);
          int k0 = x < 0.f ? 0 : (int)x;
          float f = x < 0.f ? 0.f : x - (float)k0;
          int base = isnew * kMlpInputs + ((mv_q[i] < 0.f ? 0 : 2) + (qj < 0.f ? 0 : 1)) * 16;
          if (k0 < 16) atomicAdd(&hist[base + k0], __float2int_rn((1.f - f) * qj * kDescScale));
          if (k0 + 1 < 16) atomicAdd(&hist[base + k0 + 1], __float2int_rn(f * qj * kDescScale));
        }
      }
    }
    float g_part = 0.f;
    if (P.desc) {
      __syncthreads();
      if (tid < 2 * kMlpInputs) {
        int s = 0;
        for (int w = 0; w < 32; w++) {
          s += sm_hist[w * 2 * kMlpInputs + tid];
          sm_hist[w * 2 * kMlpInputs + tid] = 0;
        }
        sm_desc[tid / kMlpInputs][tid % kMlpInputs] = (float)s * (1.f / kDescScale);
      }
      __syncthreads();
      if (P.mode == 1) {
        // surrogate: rows 0 (before) and 1 (after), one hidden unit per thread
        if (tid < 2 * kMlpHidden) {
          int r = tid / kMlpHidden, u = tid % kMlpHidden;
          const float *mean = sm_fb + 3 * kMlpHidden + 1, *istd = mean + kMlpInputs;
          float h = sm_fb[u];
#pragma unroll 8
          for (int i = 0; i < kMlpInputs; i++)
            h = fmaf(bf16_to_f(sm_w1t[i * kMlpHidden + u]), (sm_desc[r][i] - mean[i]) * istd[i], h);
          sm_h1[r][u] = silu_f(h);
        }
        __syncthreads();
        if (tid < 2 * kMlpHidden) {
          int r = tid / kMlpHidden, u = tid % kMlpHidden;
          float h = sm_fb[kMlpHidden + u];
#pragma unroll 8
          for (int v = 0; v < kMlpHidden; v++)
            h = fmaf(bf16_to_f(sm_w2t[v * kMlpHidden + u]), sm_h1[r][v], h);
          float o = sm_fb[2 * kMlpHidden + u] * silu_f(h);
          g_part = r ? o : -o;  // g(after) - g(before); b3 cancels
        }
      }
    }
    // ---- stage 1 (delayed acceptance) or the single exact stage ----
    float dk = 0.f, dSx = 0.f, dSy = 0.f, ghat = 0.f, dE1 = 0.f;
    if (P.mode == 1) {
      float a = de, b = g_part;
      block_sum2(a, b, red_a, red_b);
      de = a;
      ghat = b;
      dE1 = de + ghat;
      if (tid == 0) {
        float arg = -dE1 * beta;
        stage1 = (arg > 0.f) ? 1 : (__expf(arg) > mv_u ? 1 : 0);
      }
      __syncthreads();
    } else {
      if (tid == 0) stage1 = 1;
    }
    const bool need_k = (P.mode == 0) || stage1;
    if (need_k) {
      if (tid < P.nk && P.full) {
        // the reference's evaluation (ewald_mc.c:109-156 before and after the
        // move, forces_mc.c:90-573): S(k) of the old and of the new
        // configuration summed over every site (float-pair sums)
        float soxh = 0.f, soxl = 0.f, soyh = 0.f, soyl = 0.f;
        float snxh = 0.f, snxl = 0.f, snyh = 0.f, snyl = 0.f;
        for (int j = 0; j < P.n; j++) {
          int4 pj = sm_pos[j];
          float q = __int_as_float(pj.w);
          float so, co;
          phase_sincos((uint32_t)kx * (unsigned)pj.x + (uint32_t)ky * (unsigned)pj.y +
                           (uint32_t)kz * (unsigned)pj.z,
                       so, co);
          ff_add(soxh, soxl, q * co);
          ff_add(soyh, soyl, q * so);
          if (j >= lb && j < lb + m) {
            const unsigned *u = mv_new[j - lb];
            phase_sincos((uint32_t)kx * u[0] + (uint32_t)ky * u[1] + (uint32_t)kz * u[2], so, co);
          }
          ff_add(snxh, snxl, q * co);
          ff_add(snyh, snyl, q * so);
        }
        double sox = (double)soxh + soxl, soy = (double)soyh + soyl;
        double snx = (double)snxh + snxl, sny = (double)snyh + snyl;
        dSx = (float)(snx - sox);
        dSy = (float)(sny - soy);
        dk = (float)((double)ck * ((snx * snx + sny * sny) - (sox * sox + soy * soy)));
      } else if (tid < P.nk) {
        for (int i = 0; i < m; i++) {
          uint32_t po = (uint32_t)kx * mv_old[i][0] + (uint32_t)ky * mv_old[i][1] +
                        (uint32_t)kz * mv_old[i][2];
          uint32_t pn = (uint32_t)kx * mv_new[i][0] + (uint32_t)ky * mv_new[i][1] +
                        (uint32_t)kz * mv_new[i][2];
          float so, co, sn, cn;
          phase_sincos(po, so, co);
          phase_sincos(pn, sn, cn);
          dSx = fmaf(mv_q[i], cn - co, dSx);
          dSy = fmaf(mv_q[i], sn - so, dSy);
        }
        // |S + dS|^2 - |S|^2 = 2 Re(conj(S) dS) + |dS|^2
        dk = ck * (2.f * (Sxh * dSx + Syh * dSy) + dSx * dSx + dSy * dSy);
      }
      float a = (P.mode == 0) ? de : 0.f, b = dk;
      block_sum2(a, b, red_a, red_b);
      if (P.mode == 0) de = a;
      dk = b;
    }
    if (tid == 0) {
      int acc;
      float dE = de + dk;
      if (P.mode == 0) {
        float arg = -dE * beta;  // (U_initial - U_final) * beta, mcmove_displ.c:130-137
        acc = (arg > 0.f) ? 1 : (__expf(arg) > mv_u ? 1 : 0);
        dE1 = dE;
      } else if (stage1) {
        // second stage: min(1, exp(-beta (dE - dE1))) with the exact dE
        float arg = -(dk - ghat) * beta;
        acc = (arg > 0.f) ? 1 : (__expf(arg) > mv_u2 ? 1 : 0);
      } else {
        acc = 0;
      }
      decision = acc;
      if (chain == 0 && it < (long long)P.log_cap && D.log) {
        double *L = D.log + (size_t)it * kMccLogD;
        double nan = __longlong_as_double(0x7ff8000000000000ll);
        L[0] = (double)((mv_lb << 1) | mv_rot);
        L[1] = (double)m;
        L[2] = (double)acc;
        L[3] = need_k ? (double)dE : nan;
        L[4] = need_k ? (double)dk : nan;
        L[5] = (double)de;
        L[6] = (double)mv_u;
        L[7] = (double)dE1;
        L[8] = (double)mv_u2;
        L[9] = (double)stage1;
        L[10] = (double)(need_k ? 1 : 0);
        L[11] = (double)ghat;
        unsigned *F = D.log_fx + (size_t)it * kMccMaxSites * 3;
        for (int i = 0; i < m; i++)
          for (int c = 0; c < 3; c++) F[i * 3 + c] = mv_new[i][c];
      }
    }
    // samples: descriptors before / after and the exact dE_k (exact mode) or
    // the surrogate's estimate (delayed acceptance)
    if (P.collect && nsamp < P.sample_cap) {
      float *smp = D.samples + ((size_t)chain * P.sample_cap + nsamp) * (2 * kMlpInputs + 1);
      if (tid < 2 * kMlpInputs) smp[tid] = sm_desc[tid / kMlpInputs][tid % kMlpInputs];
      if (tid == 2 * kMlpInputs) smp[tid] = P.mode == 0 ? dk : ghat;
      nsamp++;
    }
    __syncthreads();
    if (stage1) n_s1++;
    if (need_k) n_k++;
    if (decision) {
      if (tid < P.nk) {
        ff_add(Sxh, Sxl, dSx);
        ff_add(Syh, Syl, dSy);
      }
      if (tid < m) {
        int4 p = sm_pos[lb + tid];
        p.x = (int)mv_new[tid][0];
        p.y = (int)mv_new[tid][1];
        p.z = (int)mv_new[tid][2];
        sm_pos[lb + tid] = p;
      }
      nacc++;
    }
    __syncthreads();
  }
  for (int i = tid; i < P.n; i += blockDim.x) gpos[i] = sm_pos[i];
  if (tid < P.nk)
    D.S[(size_t)chain * P.nk + tid] =
        make_double2((double)Sxh + (double)Sxl, (double)Syh + (double)Syl);
  if (tid == 0) {
    D.moves[chain] = move0 + nmoves;
    D.accepted[chain] += nacc;
    D.stats[2 * chain] += n_s1;
    D.stats[2 * chain + 1] += n_k;
    if (P.collect) D.nsamples[chain] = nsamp;
  }
}

// host: exp(i 2 pi ph / 2^32) in FP64
static void host_phase(uint32_t ph, double &s, double &c) {
  double ang = 2.0 * kPI * ((double)ph * 0x1p-32);
  s = sin(ang);
  c = cos(ang);
}

void mcc_free(Box *b) {
  McChains *M = b->mcc;
  if (!M) return;
  void *ptrs[] = {M->D.posfx, M->D.S, (void *)M->D.kv, (void *)M->D.ck, (void *)M->D.mol_first,
                  (void *)M->D.type, (void *)M->D.mass, (void *)M->D.lj, M->D.moves,
                  M->D.accepted, M->D.log, M->D.log_fx, M->D.stats, M->D.samples,
                  M->D.nsamples, (void *)M->D.w1t, (void *)M->D.w2t, (void *)M->D.fb};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  delete M;
  b->mcc = nullptr;
}

static int mcc_setup(Box *b, int nchains, const int *mol_first, int nmol, int kmax, int mks,
                     double rc_ew, double T, double delta, double rot_max, double p_rot,
                     uint64_t seed, int log_cap) {
  int n = b->n, nt = b->nt;
  if (nchains < 1 || nchains > 4096 || nmol < 1 || !mol_first || kmax < 1 || mks < 1 ||
      rc_ew <= 0.0 || T <= 0.0 || delta < 0.0 || rot_max < 0.0 || p_rot < 0.0 || p_rot > 1.0 ||
      log_cap < 0) {
    set_error("fe_mc_chains_setup: invalid argument");
    return FE_ERR_ARG;
  }
  if (n > kMccMaxN || nt > kMccMaxTypes) {
    set_error("fe_mc_chains_setup: at most 10240 sites and 8 site types per chain");
    return FE_ERR_SIZE;
  }
  if (mol_first[0] != 0 || mol_first[nmol] != n) {
    set_error("fe_mc_chains_setup: molecules must cover sites 0..n-1 in order");
    return FE_ERR_ARG;
  }
  std::vector<int> mol_of(n, -1);
  for (int m = 0; m < nmol; m++) {
    int sz = mol_first[m + 1] - mol_first[m];
    if (sz < 1 || sz > kMccMaxSites) {
      set_error("fe_mc_chains_setup: molecules need 1..8 sites");
      return FE_ERR_SIZE;
    }
    for (int i = mol_first[m]; i < mol_first[m + 1]; i++) mol_of[i] = m;
  }
  // every excluded pair must lie inside one molecule (rigid moves leave them unchanged)
  std::vector<int> xs(n + 1), xp(b->nexcl > 0 ? 2 * b->nexcl : 1);
  FE_CUDA(cudaMemcpy(xs.data(), b->x_start, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost));
  if (xs[n] > 0)
    FE_CUDA(cudaMemcpy(xp.data(), b->x_partner, sizeof(int) * xs[n], cudaMemcpyDeviceToHost));
  for (int a = 0; a < n; a++)
    for (int p = xs[a]; p < xs[a + 1]; p++)
      if (mol_of[xp[p]] != mol_of[a]) {
        set_error("fe_mc_chains_setup: an excluded pair spans two molecules");
        return FE_ERR_ARG;
      }
  // k-vectors in ewald_setup's order (ewald.c:104-118)
  double lx = b->p.L[0], ly = b->p.L[1], lz = b->p.L[2];
  double two_pi = 2.0 * kPI, boxv = lx * ly * lz, bb = 0.25 / (b->p.kappa * b->p.kappa);
  double fconv = (kELEC * kELEQ * kELEQ * kNA * 0.001);
  std::vector<int4> kv;
  std::vector<double> ckv;
  for (int kx = 0; kx <= kmax; ++kx)
    for (int ky = -kmax; ky <= kmax; ++ky)
      for (int kz = -kmax; kz <= kmax; ++kz) {
        int ksq = kx * kx + ky * ky + kz * kz;
        if (ksq > mks || ksq == 0) continue;
        double rkx = two_pi * (double)kx / lx, rky = two_pi * (double)ky / ly,
               rkz = two_pi * (double)kz / lz;
        double rksq = rkx * rkx + rky * rky + rkz * rkz;
        double kvec = two_pi * exp(-bb * rksq) / rksq / boxv;
        ckv.push_back((kx == 0 ? 1.0 : 2.0) * kvec * fconv);
        kv.push_back(make_int4(kx, ky, kz, 0));
      }
  int nk = (int)kv.size();
  if (nk > kMccMaxK) {
    set_error("fe_mc_chains_setup: more than 1024 k-vectors");
    return FE_ERR_SIZE;
  }
  // state from the box's current positions
  std::vector<double4> pq(n);
  FE_CUDA(cudaMemcpy(pq.data(), b->pos_q, sizeof(double4) * n, cudaMemcpyDeviceToHost));
  std::vector<int4> fx(n);
  double L3[3] = {lx, ly, lz};
  for (int i = 0; i < n; i++) {
    double x[3] = {pq[i].x, pq[i].y, pq[i].z};
    unsigned u[3];
    for (int a = 0; a < 3; a++) {
      double f = x[a] / L3[a] + 0.5;
      f -= floor(f);
      u[a] = (unsigned)(long long)llrint(f * 4294967296.0);
    }
    float qf = (float)pq[i].w;
    int qb;
    memcpy(&qb, &qf, 4);
    fx[i] = make_int4((int)u[0], (int)u[1], (int)u[2], qb);
  }
  std::vector<double2> S(nk);
  for (int k = 0; k < nk; k++) {
    double sr = 0.0, si = 0.0;
    for (int i = 0; i < n; i++) {
      uint32_t ph = (uint32_t)kv[k].x * (uint32_t)fx[i].x + (uint32_t)kv[k].y * (uint32_t)fx[i].y +
                    (uint32_t)kv[k].z * (uint32_t)fx[i].z;
      double s, c;
      host_phase(ph, s, c);
      double q = (double)pq[i].w;
      sr += q * c;
      si += q * s;
    }
    S[k] = make_double2(sr, si);
  }
  std::vector<int> ty(n);
  std::vector<double> ms(n), eps(nt * nt), sig(nt * nt);
  FE_CUDA(cudaMemcpy(ty.data(), b->type, sizeof(int) * n, cudaMemcpyDeviceToHost));
  FE_CUDA(cudaMemcpy(ms.data(), b->mass, sizeof(double) * n, cudaMemcpyDeviceToHost));
  FE_CUDA(cudaMemcpy(eps.data(), b->lj_eps, sizeof(double) * nt * nt, cudaMemcpyDeviceToHost));
  FE_CUDA(cudaMemcpy(sig.data(), b->lj_sig, sizeof(double) * nt * nt, cudaMemcpyDeviceToHost));
  std::vector<unsigned char> ty8(n);
  std::vector<float> mf(n), lj(nt * nt * 3);
  for (int i = 0; i < n; i++) {
    ty8[i] = (unsigned char)ty[i];
    mf[i] = (float)ms[i];
  }
  double rc2 = b->p.rc * b->p.rc;
  for (int t = 0; t < nt * nt; t++) {
    double e = eps[t], s2 = sig[t] * sig[t];
    bool on = (e * sig[t]) != 0.0;
    double sr2s = s2 / rc2, sr6s = sr2s * sr2s * sr2s;
    lj[3 * t] = on ? (float)e : 0.f;
    lj[3 * t + 1] = (float)s2;
    lj[3 * t + 2] = on && !(b->p.r_switch > 0.0) ? (float)(e * (sr6s * sr6s - 2.0 * sr6s)) : 0.f;
  }
  mcc_free(b);
  McChains *M = new McChains();
  b->mcc = M;
  M->nchains = nchains;
  M->kmax = kmax;
  M->mks = mks;
  M->rc_ew = rc_ew;
  M->mol_first.assign(mol_first, mol_first + nmol + 1);
  MccParams &P = M->P;
  P.n = n;
  P.nmol = nmol;
  P.nk = nk;
  P.nt = nt;
  for (int a = 0; a < 3; a++) {
    P.sLd[a] = L3[a] * 0x1p-32;
    P.sLf[a] = (float)P.sLd[a];
  }
  P.rc2 = (float)rc2;
  P.rce2 = (float)(rc_ew * rc_ew);
  {
    double ron2 = b->p.r_switch > 0.0 ? b->p.r_switch * b->p.r_switch : 0.0;
    P.ron2 = (float)ron2;
    P.inv_sw_den = (float)(1.0 / ((rc2 - ron2) * (rc2 - ron2) * (rc2 - ron2)));
  }
  P.kappa = (float)b->p.kappa;
  P.fconv = (float)fconv;
  P.beta = 1.0 / (((kKB * kNA) * T) * .001);
  P.delta = delta;
  P.rot_max = rot_max;
  P.p_rot = p_rot;
  P.seed = seed;
  P.log_cap = log_cap;
  MccDev &D = M->D;
  FE_CUDA(cudaMalloc(&D.posfx, sizeof(int4) * (size_t)n * nchains));
  FE_CUDA(cudaMalloc(&D.S, sizeof(double2) * (size_t)nk * nchains));
  FE_CUDA(cudaMalloc((void **)&D.kv, sizeof(int4) * nk));
  FE_CUDA(cudaMalloc((void **)&D.ck, sizeof(double) * nk));
  FE_CUDA(cudaMalloc((void **)&D.mol_first, sizeof(int) * (nmol + 1)));
  FE_CUDA(cudaMalloc((void **)&D.type, n));
  FE_CUDA(cudaMalloc((void **)&D.mass, sizeof(float) * n));
  FE_CUDA(cudaMalloc((void **)&D.lj, sizeof(float) * nt * nt * 3));
  FE_CUDA(cudaMalloc(&D.moves, sizeof(long long) * nchains));
  FE_CUDA(cudaMalloc(&D.accepted, sizeof(long long) * nchains));
  if (log_cap > 0) {
    FE_CUDA(cudaMalloc(&D.log, sizeof(double) * kMccLogD * (size_t)log_cap));
    FE_CUDA(cudaMalloc(&D.log_fx, sizeof(unsigned) * kMccMaxSites * 3 * (size_t)log_cap));
  }
  for (int c = 0; c < nchains; c++) {
    FE_CUDA(cudaMemcpy(D.posfx + (size_t)c * n, fx.data(), sizeof(int4) * n, cudaMemcpyHostToDevice));
    FE_CUDA(cudaMemcpy(D.S + (size_t)c * nk, S.data(), sizeof(double2) * nk, cudaMemcpyHostToDevice));
  }
  FE_CUDA(cudaMemcpy((void *)D.kv, kv.data(), sizeof(int4) * nk, cudaMemcpyHostToDevice));
  FE_CUDA(cudaMemcpy((void *)D.ck, ckv.data(), sizeof(double) * nk, cudaMemcpyHostToDevice));
  FE_CUDA(cudaMemcpy((void *)D.mol_first, mol_first, sizeof(int) * (nmol + 1), cudaMemcpyHostToDevice));
  FE_CUDA(cudaMemcpy((void *)D.type, ty8.data(), n, cudaMemcpyHostToDevice));
  FE_CUDA(cudaMemcpy((void *)D.mass, mf.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
  FE_CUDA(cudaMemcpy((void *)D.lj, lj.data(), sizeof(float) * nt * nt * 3, cudaMemcpyHostToDevice));
  FE_CUDA(cudaMemset(D.moves, 0, sizeof(long long) * nchains));
  FE_CUDA(cudaMemset(D.accepted, 0, sizeof(long long) * nchains));
  FE_CUDA(cudaMalloc(&D.stats, sizeof(long long) * 2 * nchains));
  FE_CUDA(cudaMemset(D.stats, 0, sizeof(long long) * 2 * nchains));
  P.mode = 0;
  P.full = 0;
  P.desc = 0;
  P.collect = 0;
  P.sample_cap = 0;
  return FE_OK;
}

// dynamic shared memory of k_mcc_run for the current flags
static size_t mcc_smem(const MccParams &P) {
  int n = P.n, nt = P.nt;
  int chunk = ((n + 31) / 32 + 31) & ~31;
  size_t s = sizeof(int4) * (size_t)n + (size_t)((n + 15) & ~15) +
             sizeof(float) * (size_t)((nt * nt * 3 + 3) & ~3) + sizeof(int) * 32 * (size_t)chunk;
  if (P.desc) s += sizeof(int) * 32 * 2 * kMlpInputs;
  if (P.mode == 1)
    s += 2 * (size_t)(kMlpInputs * kMlpHidden + kMlpHidden * kMlpHidden) + sizeof(float) * kMlpFb;
  return s;
}

constexpr size_t kMccSmemMax = 227 * 1024 - 4096;  // dynamic part; static shared ~3 KB

static int mcc_check_smem(const MccParams &P) {
  if (mcc_smem(P) > kMccSmemMax) {
    set_error("fe_mc_chains: too many sites for this mode's shared-memory state");
    return FE_ERR_SIZE;
  }
  return FE_OK;
}

static int mcc_run(Box *b, long long nmoves) {
  McChains *M = b->mcc;
  if (!M) {
    set_error("fe_mc_chains_run before fe_mc_chains_setup");
    return FE_ERR_STATE;
  }
  if (nmoves < 0) return FE_ERR_ARG;
  // the log covers the first log_cap moves of chain 0 from setup on
  long long done = 0;
  while (done < nmoves) {
    long long c = nmoves - done < kMccChunk ? nmoves - done : kMccChunk;
    MccParams P = M->P;
    // log index = move number within this launch; shift the log window
    MccDev D = M->D;
    long long logged = 0;
    FE_CUDA(cudaMemcpyAsync(&logged, D.moves, sizeof(long long), cudaMemcpyDeviceToHost, b->stream));
    FE_CUDA(cudaStreamSynchronize(b->stream));
    if (D.log && logged < P.log_cap) {
      D.log += (size_t)logged * kMccLogD;
      D.log_fx += (size_t)logged * kMccMaxSites * 3;
      P.log_cap = (int)(P.log_cap - logged);
    } else {
      P.log_cap = 0;
    }
    size_t smem = mcc_smem(P);
    FE_CUDA(cudaFuncSetAttribute(k_mcc_run, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem));
    k_mcc_run<<<M->nchains, kMccThreads, smem, b->stream>>>(P, D, c);
    FE_LAUNCH_CHECK("k_mcc_run");
    done += c;
  }
  FE_CUDA(cudaStreamSynchronize(b->stream));
  return FE_OK;
}

}  // namespace fe

using namespace fe;

extern "C" {

int fe_mc_chains_setup(fe_box *box, int nchains, const int *mol_first, int nmol, int kmax,
                       int max_k_square, double rc_ew, double T, double delta, double rot_max,
                       double p_rot, uint64_t seed, int log_cap) {
  if (!box) return FE_ERR_ARG;
  return mcc_setup(&box->b, nchains, mol_first, nmol, kmax, max_k_square, rc_ew, T, delta, rot_max,
                   p_rot, seed, log_cap);
}

int fe_mc_chains_run(fe_box *box, int64_t nmoves) {
  if (!box) return FE_ERR_ARG;
  return mcc_run(&box->b, (long long)nmoves);
}

int fe_mc_chains_state(fe_box *box, int chain, double *xyz, int64_t *moves, int64_t *accepted) {
  if (!box || !box->b.mcc) return FE_ERR_STATE;
  Box *b = &box->b;
  McChains *M = b->mcc;
  if (chain < 0 || chain >= M->nchains) return FE_ERR_ARG;
  FE_CUDA(cudaStreamSynchronize(b->stream));
  int n = M->P.n;
  if (xyz) {
    std::vector<int4> fx(n);
    FE_CUDA(cudaMemcpy(fx.data(), M->D.posfx + (size_t)chain * n, sizeof(int4) * n,
                       cudaMemcpyDeviceToHost));
    for (int i = 0; i < n; i++) {
      unsigned u[3] = {(unsigned)fx[i].x, (unsigned)fx[i].y, (unsigned)fx[i].z};
      for (int a = 0; a < 3; a++)
        xyz[3 * i + a] = ((double)u[a] * 0x1p-32 - 0.5) * b->p.L[a];
    }
  }
  if (moves)
    FE_CUDA(cudaMemcpy(moves, M->D.moves + chain, sizeof(long long), cudaMemcpyDeviceToHost));
  if (accepted)
    FE_CUDA(cudaMemcpy(accepted, M->D.accepted + chain, sizeof(long long), cudaMemcpyDeviceToHost));
  return FE_OK;
}

int fe_mc_chains_kspace_energy(fe_box *box, int chain, double *e) {
  if (!box || !box->b.mcc || !e) return FE_ERR_STATE;
  McChains *M = box->b.mcc;
  if (chain < 0 || chain >= M->nchains) return FE_ERR_ARG;
  FE_CUDA(cudaStreamSynchronize(box->b.stream));
  int nk = M->P.nk;
  std::vector<double2> S(nk);
  std::vector<double> ck(nk);
  FE_CUDA(cudaMemcpy(S.data(), M->D.S + (size_t)chain * nk, sizeof(double2) * nk,
                     cudaMemcpyDeviceToHost));
  FE_CUDA(cudaMemcpy(ck.data(), M->D.ck, sizeof(double) * nk, cudaMemcpyDeviceToHost));
  double s = 0.0;
  for (int k = 0; k < nk; k++) s += ck[k] * (S[k].x * S[k].x + S[k].y * S[k].y);
  *e = s;
  return FE_OK;
}

int fe_mc_chains_collect(fe_box *box, int64_t per_chain) {
  if (!box || !box->b.mcc || per_chain < 0) return FE_ERR_ARG;
  McChains *M = box->b.mcc;
  if (M->D.samples) cudaFree(M->D.samples);
  if (M->D.nsamples) cudaFree(M->D.nsamples);
  M->D.samples = nullptr;
  M->D.nsamples = nullptr;
  M->P.collect = 0;
  M->P.sample_cap = 0;
  M->P.desc = M->P.mode == 1 ? 1 : 0;
  if (per_chain == 0) return FE_OK;
  MccParams P = M->P;
  P.desc = 1;
  int rc = mcc_check_smem(P);
  if (rc) return rc;
  FE_CUDA(cudaMalloc(&M->D.samples, sizeof(float) * (2 * kMlpInputs + 1) * (size_t)per_chain *
                                        M->nchains));
  FE_CUDA(cudaMalloc(&M->D.nsamples, sizeof(long long) * M->nchains));
  FE_CUDA(cudaMemset(M->D.nsamples, 0, sizeof(long long) * M->nchains));
  M->P.collect = 1;
  M->P.desc = 1;
  M->P.sample_cap = per_chain;
  return FE_OK;
}

// samples of every chain, chain after chain: out rows of 129 floats
// (64 descriptors before, 64 after, exact dE_k)
int fe_mc_chains_samples(fe_box *box, float *out, int64_t cap, int64_t *count) {
  if (!box || !box->b.mcc) return FE_ERR_STATE;
  McChains *M = box->b.mcc;
  FE_CUDA(cudaStreamSynchronize(box->b.stream));
  int64_t total = 0;
  if (M->D.nsamples) {
    std::vector<long long> ns(M->nchains);
    FE_CUDA(cudaMemcpy(ns.data(), M->D.nsamples, sizeof(long long) * M->nchains,
                       cudaMemcpyDeviceToHost));
    const size_t row = 2 * kMlpInputs + 1;
    for (int c = 0; c < M->nchains; c++) {
      long long k = ns[c];
      if (out && total + k > cap) k = cap - total;
      if (out && k > 0)
        FE_CUDA(cudaMemcpy(out + (size_t)total * row,
                           M->D.samples + (size_t)c * M->P.sample_cap * row,
                           sizeof(float) * row * (size_t)k, cudaMemcpyDeviceToHost));
      total += k > 0 ? k : 0;
    }
  }
  if (count) *count = total;
  return FE_OK;
}

__global__ void k_mcc_split(long long n, const float *__restrict__ rows, float *__restrict__ data,
                            float *__restrict__ y) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * 129) return;
  long long r = t / 129;
  int f = (int)(t % 129);
  if (f < 128) data[r * 128 + f] = rows[t];
  else y[r] = rows[t];
}

// Trains `mlp` on the collected samples of every chain (on the device).
int fe_mc_chains_train_surrogate(fe_box *box, fe_mlp *mlp, int epochs, int batch, float lr,
                                 uint64_t seed, float *loss_hist) {
  if (!box || !box->b.mcc || !mlp) return FE_ERR_ARG;
  McChains *M = box->b.mcc;
  if (!M->D.nsamples) {
    set_error("fe_mc_chains_train_surrogate: no samples collected");
    return FE_ERR_STATE;
  }
  FE_CUDA(cudaStreamSynchronize(box->b.stream));
  std::vector<long long> ns(M->nchains);
  FE_CUDA(cudaMemcpy(ns.data(), M->D.nsamples, sizeof(long long) * M->nchains,
                     cudaMemcpyDeviceToHost));
  long long total = 0;
  for (long long k : ns) total += k;
  if (total < batch) {
    set_error("fe_mc_chains_train_surrogate: fewer samples than one batch");
    return FE_ERR_STATE;
  }
  const size_t row = 2 * kMlpInputs + 1;
  float *rows = nullptr, *data = nullptr, *y = nullptr;
  int rc = FE_OK;
  cudaError_t e = cudaMalloc(&rows, sizeof(float) * row * (size_t)total);
  if (e == cudaSuccess) e = cudaMalloc(&data, sizeof(float) * 128 * (size_t)total);
  if (e == cudaSuccess) e = cudaMalloc(&y, sizeof(float) * (size_t)total);
  long long off = 0;
  for (int c = 0; c < M->nchains && e == cudaSuccess; c++) {
    if (ns[c] > 0)
      e = cudaMemcpy(rows + (size_t)off * row, M->D.samples + (size_t)c * M->P.sample_cap * row,
                     sizeof(float) * row * (size_t)ns[c], cudaMemcpyDeviceToDevice);
    off += ns[c];
  }
  if (e == cudaSuccess) {
    long long th = total * 129;
    k_mcc_split<<<(unsigned)((th + 255) / 256), 256>>>(total, rows, data, y);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess)
    rc = mlp_train_device(mlp_from_handle(mlp), data, y, total, epochs, batch, lr, seed,
                          loss_hist);
  cudaFree(rows);
  cudaFree(data);
  cudaFree(y);
  if (e != cudaSuccess) return cuda_fail(e, "fe_mc_chains_train_surrogate");
  return rc;
}

// Loads the surrogate for delayed acceptance: bf16 W1 and W2 transposed,
// fp32 biases, output weights and input normalisation.
int fe_mc_chains_set_surrogate(fe_box *box, fe_mlp *mlp) {
  if (!box || !box->b.mcc || !mlp) return FE_ERR_ARG;
  McChains *M = box->b.mcc;
  int np = fe_mlp_param_count();
  std::vector<float> Pm(np), mean(kMlpInputs), istd(kMlpInputs);
  int rc = fe_mlp_get_params(mlp, Pm.data(), mean.data(), istd.data());
  if (rc) return rc;
  const int H = kMlpHidden, I = kMlpInputs;
  const float *W1 = Pm.data(), *b1 = W1 + H * I, *W2 = b1 + H, *b2 = W2 + H * H, *w3 = b2 + H,
              *b3 = w3 + H;
  std::vector<unsigned short> w1t(I * H), w2t(H * H);
  std::vector<float> fb(kMlpFb);
  auto to_bf16 = [](float f) -> unsigned short {
    uint32_t u;
    memcpy(&u, &f, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);
    return (unsigned short)(u >> 16);
  };
  for (int u = 0; u < H; u++) {
    for (int i = 0; i < I; i++) w1t[i * H + u] = to_bf16(W1[u * I + i]);
    fb[u] = b1[u];
    fb[H + u] = b2[u];
    fb[2 * H + u] = w3[u];
    for (int v = 0; v < H; v++) w2t[v * H + u] = to_bf16(W2[u * H + v]);
  }
  fb[3 * H] = b3[0];
  for (int i = 0; i < I; i++) {
    fb[3 * H + 1 + i] = mean[i];
    fb[3 * H + 1 + I + i] = istd[i];
  }
  MccParams P = M->P;
  P.mode = 1;
  P.desc = 1;
  if ((rc = mcc_check_smem(P))) return rc;
  if (!M->D.w1t) {
    FE_CUDA(cudaMalloc((void **)&M->D.w1t, 2 * (size_t)I * H));
    FE_CUDA(cudaMalloc((void **)&M->D.w2t, 2 * (size_t)H * H));
    FE_CUDA(cudaMalloc((void **)&M->D.fb, sizeof(float) * kMlpFb));
  }
  FE_CUDA(cudaMemcpy((void *)M->D.w1t, w1t.data(), 2 * (size_t)I * H, cudaMemcpyHostToDevice));
  FE_CUDA(cudaMemcpy((void *)M->D.w2t, w2t.data(), 2 * (size_t)H * H, cudaMemcpyHostToDevice));
  FE_CUDA(cudaMemcpy((void *)M->D.fb, fb.data(), sizeof(float) * kMlpFb, cudaMemcpyHostToDevice));
  return FE_OK;
}

// 0: exact dE (one stage); 1: delayed acceptance (needs a surrogate)
int fe_mc_chains_set_mode(fe_box *box, int mode) {
  if (!box || !box->b.mcc || mode < 0 || mode > 3) return FE_ERR_ARG;
  McChains *M = box->b.mcc;
  if ((mode & 1) && !M->D.w1t) {
    set_error("fe_mc_chains_set_mode: delayed acceptance needs fe_mc_chains_set_surrogate first");
    return FE_ERR_STATE;
  }
  MccParams P = M->P;
  P.mode = mode & 1;
  P.full = mode >> 1;
  P.desc = (P.mode == 1 || P.collect) ? 1 : 0;
  int rc = mcc_check_smem(P);
  if (rc) return rc;
  M->P = P;
  return FE_OK;
}

int fe_mc_chains_stats(fe_box *box, int chain, int64_t *out4) {
  if (!box || !box->b.mcc || !out4) return FE_ERR_ARG;
  McChains *M = box->b.mcc;
  if (chain < 0 || chain >= M->nchains) return FE_ERR_ARG;
  FE_CUDA(cudaStreamSynchronize(box->b.stream));
  long long v[4];
  FE_CUDA(cudaMemcpy(&v[0], M->D.moves + chain, sizeof(long long), cudaMemcpyDeviceToHost));
  FE_CUDA(cudaMemcpy(&v[1], M->D.accepted + chain, sizeof(long long), cudaMemcpyDeviceToHost));
  FE_CUDA(cudaMemcpy(&v[2], M->D.stats + 2 * chain, 2 * sizeof(long long), cudaMemcpyDeviceToHost));
  for (int i = 0; i < 4; i++) out4[i] = v[i];
  return FE_OK;
}

int fe_mc_chains_log(fe_box *box, double *rec, uint32_t *fx, int64_t cap, int64_t *count) {
  if (!box || !box->b.mcc) return FE_ERR_STATE;
  McChains *M = box->b.mcc;
  FE_CUDA(cudaStreamSynchronize(box->b.stream));
  long long moved = 0;
  FE_CUDA(cudaMemcpy(&moved, M->D.moves, sizeof(long long), cudaMemcpyDeviceToHost));
  long long nlog = moved < M->P.log_cap ? moved : M->P.log_cap;
  if (nlog > cap) nlog = cap;
  if (count) *count = nlog;
  if (nlog > 0 && rec)
    FE_CUDA(cudaMemcpy(rec, M->D.log, sizeof(double) * kMccLogD * nlog, cudaMemcpyDeviceToHost));
  if (nlog > 0 && fx)
    FE_CUDA(cudaMemcpy(fx, M->D.log_fx, sizeof(unsigned) * kMccMaxSites * 3 * nlog,
                       cudaMemcpyDeviceToHost));
  return FE_OK;
}

}  // extern "C"
