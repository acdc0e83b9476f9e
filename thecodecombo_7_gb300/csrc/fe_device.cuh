// fe_device.cuh -- device helpers shared by the FP64 kernels.
//
// The FP64 translation units are compiled with -fmad=false so that every
// multiply and add rounds separately, as the reference's C does; the pair
// set of the neighbour list then matches the reference bit for bit.
#pragma once

#include <cuda_runtime.h>

#include "fe_internal.h"

namespace fe {

// A block's view of the grid it works in: its index and the block count of
// its box.  A launch over one box is the whole grid; a launch over many boxes
// (replica batches) gives each box a contiguous range of blocks and each
// block finds its box from the range table, so one kernel body serves both.
struct VBlk {
  int id, n;
};
__device__ __forceinline__ VBlk vblk_self() { return {(int)blockIdx.x, (int)gridDim.x}; }
// box r of this block in a many-box launch: off[r] <= blockIdx.x < off[r + 1]
__device__ __forceinline__ int vblk_box(const int *__restrict__ off, int nbox) {
  int lo = 0, hi = nbox, b = (int)blockIdx.x;
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (__ldg(off + mid) <= b) lo = mid;
    else hi = mid;
  }
  return lo;
}
__device__ __forceinline__ VBlk vblk_of(const int *__restrict__ off, int r) {
  int o = __ldg(off + r);
  return {(int)blockIdx.x - o, __ldg(off + r + 1) - o};
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Deterministic block sum of up to kPartialTerms values; thread 0 writes
// partials[blockIdx.x * kPartialTerms + t].  blockDim.x must be a multiple
// of 32 and at most 1024.
template <int NT>
__device__ __forceinline__ void block_partials(double (&v)[NT], double *partials,
                                               VBlk vb = vblk_self()) {
  __shared__ double sh[32][NT];
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int t = 0; t < NT; t++) {
    double s = warp_sum(v[t]);
    if (lane == 0) sh[wid][t] = s;
  }
  __syncthreads();
  if (wid == 0) {
    int nw = blockDim.x >> 5;
#pragma unroll
    for (int t = 0; t < NT; t++) {
      double s = lane < nw ? sh[lane][t] : 0.0;
      s = warp_sum(s);
      if (lane == 0) partials[vb.id * kPartialTerms + t] = s;
    }
  }
}

// Like block_partials, then the last block to finish sums every block's
// partials in a fixed order into out[0..NT) (deterministic, one launch; the
// threadfence/ticket pattern).  `ticket` is a device counter that is 0 on
// entry and left 0 on exit.  blockDim.x <= 256.
template <int NT>
__device__ __forceinline__ bool block_partials_final(double (&v)[NT], double *partials,
                                                     unsigned *ticket, double *out,
                                                     VBlk vb = vblk_self()) {
  block_partials<NT>(v, partials, vb);  // thread 0 writes this block's partials
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(ticket, 1u) == (unsigned)vb.n - 1;
  __syncthreads();
  if (!last) return false;
  __threadfence();
  __shared__ double red[256];
  for (int t = 0; t < NT; t++) {
    double s = 0.0;
    for (int b = threadIdx.x; b < vb.n; b += blockDim.x)
      s += ((volatile double *)partials)[b * kPartialTerms + t];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) red[i] = 0.0;
    __syncthreads();
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
      if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[t] = red[0];
    __syncthreads();
  }
  if (threadIdx.x == 0) *ticket = 0u;
  return true;
}

// Deterministic grid-wide sum of NT values per thread through 64-bit fixed
// point: FP32 values are first summed over the warp in a fixed butterfly
// order, FP64 and integer values are converted per lane; the (warp or lane)
// values are rounded to integer multiples of 2^-shift, and the integer sums
// across lanes, warps and blocks are exact and independent of order, so the
// hot kernels need no FP64 arithmetic for their reductions.  Each block adds its sums to
// acc[0..NT) (one atomic per value); the last block to finish writes
// out[t] = acc[t] * 2^-shift as doubles and leaves acc and ticket at zero.
// blockDim.x a multiple of 32, at most 1024; NT <= blockDim.x.  Per-thread
// (warp or lane) values must stay below 2^(63 - shift) in magnitude, and so
// must the total.
__device__ __forceinline__ long long to_fixed(float x, int shift) {
  return __float2ll_rn(x * __int_as_float((127 + shift) << 23));
}
__device__ __forceinline__ long long to_fixed(double x, int shift) {
  return __double2ll_rn(x * ldexp(1.0, shift));
}
__device__ __forceinline__ long long to_fixed(long long x, int) { return x; }

// The block's part of block_fix_final: its sums added to acc[0..NT).
template <int NT, typename T>
__device__ __forceinline__ void block_fix_add(const T (&v)[NT], int shift,
                                              unsigned long long *acc) {
  __shared__ long long shq[32][NT];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  long long q[NT];
#pragma unroll
  for (int t = 0; t < NT; t++) {
    if (sizeof(T) == sizeof(float)) {
      // FP32 lanes: a fixed butterfly in FP32, one conversion per warp
      T w = v[t];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
      q[t] = to_fixed(w, shift);
    } else {
      // FP64 or integer lanes: convert per lane, integer butterfly (FP64 adds
      // cost more than conversions on this GPU)
      q[t] = to_fixed(v[t], shift);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) q[t] += __shfl_xor_sync(0xffffffffu, q[t], o);
    }
    if (lane == 0) shq[wid][t] = q[t];
  }
  __syncthreads();
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int t = 0; t < NT; t++) {
      long long x = lane < nw ? shq[lane][t] : 0ll;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
      if (lane == 0) atomicAdd(&acc[t], (unsigned long long)x);
    }
  }
}

template <int NT, typename T>
__device__ __forceinline__ bool block_fix_final(const T (&v)[NT], int shift,
                                                unsigned long long *acc, unsigned *ticket,
                                                double *out, VBlk vb = vblk_self()) {
  __shared__ bool last_blk;
  block_fix_add<NT>(v, shift, acc);
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last_blk = atomicAdd(ticket, 1u) == (unsigned)vb.n - 1;
  __syncthreads();
  if (!last_blk) return false;
  __threadfence();
  if (threadIdx.x < NT) {
    unsigned long long a = atomicExch(&acc[threadIdx.x], 0ull);
    out[threadIdx.x] = (double)(long long)a * ldexp(1.0, -shift);
  }
  if (threadIdx.x == 0) *ticket = 0u;
  __syncthreads();  // out[] complete for the caller's last-block epilogue
  return true;
}

// The reference's erfc (ewald.c:817-836): the Chebyshev fit "erfcc" of
// Numerical Recipes (Press et al., 2nd ed., sec. 6.2), fractional error
// below 1.2e-7, same evaluation order.  The exponential is CUDA's exp.
__device__ __forceinline__ double ref_erfc(double x) {
  double z = fabs(x);
  double t = 1.0 / (1.0 + 0.5 * z);
  double v = t * exp(-z * z + -1.26551223 +
                     t * (1.00002368 +
                     t * (0.37409196 +
                     t * (0.09678418 +
                     t * (-0.18628806 +
                     t * (0.27886807 +
                     t * (-1.13520398 +
                     t * (1.48851587 +
                     t * (-0.82215223 + t * 0.17087277)))))))));
  if (x < 0) return 2.0 - v;
  return v;
}

// The mixed path's partial sums combined into the reference's slots (the
// pair, exclusion / intramolecular and bonded sums of k_mixed.cu).
__device__ __forceinline__ void mixed_slots_dev(double *__restrict__ s, double erfc_rc_over_rc,
                                                int fused) {
  if (fused) {
    for (int t = 0; t < 5; t++) s[SC_MX_EXCL + t] = s[SC_MX_INTRA + t];
    s[SC_BOND] = s[SC_MX_INTRA + 5];
    s[SC_BEND] = s[SC_MX_INTRA + 6];
  }
  s[SC_LJ] = s[SC_MX_PAIR + 0] + s[SC_MX_EXCL + 0];
  s[SC_LJS] = s[SC_MX_PAIR + 1] + s[SC_MX_EXCL + 1];
  s[SC_REAL] = s[SC_MX_PAIR + 2] + s[SC_MX_EXCL + 2];
  s[SC_REALS] = (s[SC_MX_PAIR + 3] + s[SC_MX_EXCL + 3]) * erfc_rc_over_rc;
  s[SC_INTRA] = s[SC_MX_EXCL + 4];
}

// energy[8] of cnonbondnl (cnonbond_nblist.c:613-620), pme_calc's energy[3]
// (pme_calc.c:99-101) and, with_bonded, en[k] of forces() (forces.c:172-219)
__device__ __forceinline__ void assemble_dev(double *__restrict__ s, double fan, double sewald,
                                             int with_bonded) {
  double ek0 = s[SC_ENREC] * fan;
  double ek1 = sewald;
  double ek2 = ek0 - ek1;
  s[SC_ENERGY3 + 0] = ek0;
  s[SC_ENERGY3 + 1] = ek1;
  s[SC_ENERGY3 + 2] = ek2;
  double er0 = s[SC_REAL], er1 = s[SC_REAL] - s[SC_REALS], er2 = s[SC_INTRA];
  double e[8];
  e[0] = s[SC_LJ] + er0 - er2 + ek2;
  e[1] = e[0] - s[SC_LJS];
  e[2] = er0 + ek2 - er2;
  e[3] = er0 - er1;
  e[4] = ek0;
  e[5] = ek1;
  e[6] = er2;
  e[7] = er0;
  for (int k = 0; k < 8; k++) s[SC_ENERGY8 + k] = e[k];
  if (with_bonded) {
    s[FE_EN_BOND] = s[SC_BOND];
    s[FE_EN_BEND] = s[SC_BEND];
    s[FE_EN_UREY] = s[SC_UREY];
    s[FE_EN_TORS] = s[SC_TORS];
    s[FE_EN_IMPR] = s[SC_IMPR];
    s[FE_EN_NBOND] = e[0];
    s[FE_EN_NBONDS] = e[1];
    s[FE_EN_COULOMB] = e[2];
    s[FE_EN_TEWALD] = e[2];
    s[FE_EN_REWALD] = e[7];
    s[FE_EN_REWALDS] = e[3];
    s[FE_EN_KEWALD] = e[4];
    s[FE_EN_SEWALD] = e[5];
    s[FE_EN_IEWALD] = e[6];
  }
}

// qa * qb * QFACTOR in the reference's evaluation order (QFACTOR is an
// unparenthesised macro, defines.h:71).
__device__ __forceinline__ double qfactor_mul(double x) {
  return ((((x * kELEC) * kELEQ) * kELEQ) * kNA) * 1.0E-3;
}

// pbc_all for one coordinate, bounded (the reference loops until inside)
__device__ __forceinline__ double pbc_wrap(double d, double h, double l, int *bad) {
  double pbc = 0.0;
  int it = 0;
  while (d < -h || d > h) {
    if (d < -h) pbc = +l;
    if (d > h) pbc = -l;
    d += pbc;
    if (++it > 64) {
      *bad = 1;
      break;
    }
  }
  return d;
}

__device__ __forceinline__ void kinet_scalars(double *__restrict__ s) {
  double f = (0.125) * (kNA * kAU * 10.0);  // kinet.c:50-65
  for (int i = 0; i < 6; i++) s[SC_KEN + i] *= f;
  s[FE_EN_KINET] = s[SC_KEN + 0] + s[SC_KEN + 2] + s[SC_KEN + 5];
}

__device__ __forceinline__ void record_dev(const double *__restrict__ s, double *__restrict__ rec,
                                           long cap, int *__restrict__ counter) {
  int c = *counter;
  if (c < cap)
    for (int t = 0; t < FE_EN_COUNT; t++) rec[(long)c * FE_EN_COUNT + t] = s[t];
  *counter = c + 1;
}

// integrate_nhc.c:57-147 (Nc = Nys = 1, w[0] = 1): the chain, one thread.
// The temperature is read from s[SC_TEMP] so that replica exchanges can
// change it on the device between graph replays.
__device__ __forceinline__ void nhc_chain_dev(int M, double Q, double nfree, double time_step,
                                              double *__restrict__ zeta, double *__restrict__ s) {
  double T = s[SC_TEMP];
#define ZR(j) zeta[3 * (j)]
#define ZV(j) zeta[3 * (j) + 1]
#define ZG(j) zeta[3 * (j) + 2]
  int M1 = M - 1, M2 = M - 2;
  double NkT = nfree * kKB * T * 1E-4;
  double kT = kKB * T * 1E-4;
  double akin = 2.0 * s[FE_EN_KINET] * 1000.0 * 1E-4 / kNA;
  double scale = 1.0;
  double dt = time_step * 1.0 / (double)1;
  double dt2 = dt / 2.0, dt4 = dt / 4.0, dt8 = dt / 8.0;
  double AA;
  ZG(0) = (akin - NkT) / Q;
  ZV(M1) += ZG(M1) * dt4;
  for (int j = 0; j < M1; j++) {
    AA = exp(-dt8 * ZV(M1 - j));
    ZV(M2 - j) = ZV(M2 - j) * AA * AA + dt4 * ZG(M2 - j) * AA;
  }
  AA = exp(-dt2 * ZV(0));
  scale = scale * AA;
  for (int j = 0; j < M; j++) ZR(j) += ZV(j) * dt2;
  ZG(0) = (scale * scale * akin - NkT) / Q;
  for (int j = 0; j < M - 1; j++) {
    AA = exp(-dt8 * ZV(j + 1));
    ZV(j) = ZV(j) * AA * AA + dt4 * ZG(j) * AA;
    ZG(j + 1) = (Q * ZV(j) * ZV(j) - kT) / Q;
  }
  ZV(M - 1) += ZG(M - 1) * dt4;
  s[SC_NHC_SCALE] = scale;
#undef ZR
#undef ZV
#undef ZG
}

// Exclusive prefix sum of one int per thread over a block of up to 1024
// threads (warp shuffles, then the warp totals); *total gets the block's sum.
__device__ __forceinline__ int block_exclusive_scan(int v, int *total) {
  __shared__ int wsum[32];
  __shared__ int wtot;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[w] = x;
  __syncthreads();
  if (w == 0) {
    int y = lane < nw ? wsum[lane] : 0, z = y;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int q = __shfl_up_sync(0xffffffffu, z, o);
      if (lane >= o) z += q;
    }
    wsum[lane] = z - y;
    if (lane == 31) wtot = z;  // the block total (nw <= 32)
  }
  __syncthreads();
  int base = wsum[w];
  *total = wtot;
  __syncthreads();
  return base + x - v;
}

}  // namespace fe
