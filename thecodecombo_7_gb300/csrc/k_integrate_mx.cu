// k_integrate_mx.cu -- the integrator kernels of the mixed-precision step,
// compiled with FMA contraction: the FP64 update of positions and velocities
// (integrate_vverlet.c:54-83) and, for NVE, the tail of the step in one
// launch.  The drop-in's kernels of the same steps (k_integrate.cu) round each
// multiply and add separately as the reference's C does; the mixed path keeps
// FP64 state but needs no such parity, and on this GPU the FP64 pipe is what
// bounds these kernels, so fused multiply-adds cut their time.
#include "fe_device.cuh"

namespace fe {

// integrate_vverlet.c:54-83: half kick, drift (atom and atnopbc), pbc_all
__global__ void k_vv1_mx(int n, double vscal, double dt, double dt_h, double3 L, double3 H,
                         const double *__restrict__ imass100, const double *__restrict__ ff,
                         double *__restrict__ vv, double4 *__restrict__ pos,
                         double *__restrict__ nopbc, int *__restrict__ status) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double c = dt_h * imass100[i];
  double v0 = vscal * (vv[3 * i] + c * ff[3 * i]);
  double v1 = vscal * (vv[3 * i + 1] + c * ff[3 * i + 1]);
  double v2 = vscal * (vv[3 * i + 2] + c * ff[3 * i + 2]);
  vv[3 * i] = v0;
  vv[3 * i + 1] = v1;
  vv[3 * i + 2] = v2;
  nopbc[3 * i] += dt * v0;
  nopbc[3 * i + 1] += dt * v1;
  nopbc[3 * i + 2] += dt * v2;
  double4 p = pos[i];
  p.x += dt * v0;
  p.y += dt * v1;
  p.z += dt * v2;
  int bad = 0;
  p.x = pbc_wrap(p.x, H.x, L.x, &bad);
  p.y = pbc_wrap(p.y, H.y, L.y, &bad);
  p.z = pbc_wrap(p.z, H.z, L.z, &bad);
  if (bad) atomicOr(status, ST_PBC_LOOP);
  pos[i] = p;
}

int launch_vv1_mx(Box *b, double vscal) {
  double3 L = make_double3(b->p.L[0], b->p.L[1], b->p.L[2]);
  double3 H = make_double3(b->p.L[0] / 2.0, b->p.L[1] / 2.0, b->p.L[2] / 2.0);
  double dt = b->p.dt, dt_h = 0.5 * b->p.dt;
  k_vv1_mx<<<(b->n + 255) / 256, 256, 0, b->stream>>>(b->n, vscal, dt, dt_h, L, H, b->imass100,
                                                      b->ff, b->vv, b->pos_q, b->pos_nopbc,
                                                      b->status);
  FE_LAUNCH_CHECK("k_vv1_mx");
  return FE_OK;
}

// Mixed precision, NVE: the tail of a step in one launch -- the FP64 forces
// from the fixed-point sums minus the mean reciprocal force (k_mx_finalize),
// the energy assembly in block 0 (k_mx_slots, k_assemble), the second half
// kick with uu = vv and the kinetic tensor (k_vv2_kinet); the last block
// finishes kinet and writes the step's record (k_record).
constexpr double kMxForceFix = 4294967296.0;  // 2^32 per kJ/mol/A

__global__ void k_vv2_mx_tail(BIntArgs a, const unsigned long long *__restrict__ fix) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    mixed_slots_dev(a.scal, a.erfc_rc_over_rc, a.mixed_fused);
    assemble_dev(a.scal, a.fan, a.sewald, 1);
  }
  __shared__ double mean[3];
  if (threadIdx.x < 3) mean[threadIdx.x] = a.scal[SC_FMEAN + threadIdx.x] / kMxForceFix / (double)a.n;
  __syncthreads();
  double k[6] = {0, 0, 0, 0, 0, 0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) {
    double imass = a.imass100[i];
    double v[3];
    for (int c = 0; c < 3; c++) {
      double f = (double)(long long)fix[3 * i + c] * (1.0 / kMxForceFix) - mean[c];
      a.ff[3 * i + c] = f;
      v[c] = (a.vv[3 * i + c] + 1.0 * a.dt_h * imass * f);
      a.vv[3 * i + c] = v[c];
      a.uu[3 * i + c] = v[c];
    }
    double fac = a.mass[i];
    double sx = v[0] + v[0], sy = v[1] + v[1], sz = v[2] + v[2];
    k[0] += fac * sx * sx;
    k[1] += fac * sy * sx;
    k[2] += fac * sy * sy;
    k[3] += fac * sz * sx;
    k[4] += fac * sz * sy;
    k[5] += fac * sz * sz;
  }
  if (block_fix_final<6>(k, 20, a.facc, a.ticket, a.scal + SC_KEN) && threadIdx.x == 0) {
    kinet_scalars(a.scal);
    record_dev(a.scal, a.rec, a.rec_cap, a.rec_counter);
  }
}

int launch_vv2_mx_tail(Box *b) {
  BIntArgs a = make_bint_args(b);
  int blocks = (b->n + 255) / 256;
  if (blocks > 512) blocks = 512;
  k_vv2_mx_tail<<<blocks, 256, 0, b->stream>>>(a, mixed_force_sums(b));
  FE_LAUNCH_CHECK("k_vv2_mx_tail");
  return FE_OK;
}

// ---------------------------------------------------------------------------
// Integrator kernels of a batched step: every box of a replica batch in one
// launch per kernel (blocks of box r: off[r] .. off[r+1]-1).  The arithmetic
// is that of the single-box kernels above, site for site; the Nose-Hoover
// velocity scale is applied inside the next per-site pass instead of in a
// launch of its own, and the energy assembly rides on the second half kick.


// kinet (fixed point, as k_kinet_fix) and the first Nose-Hoover chain update
__global__ void k_b_kinet_nhc(const BIntArgs *__restrict__ A, const int *__restrict__ off,
                              int nbox) {
  const int r = vblk_box(off, nbox);
  const BIntArgs &a = A[r];
  const VBlk vb = vblk_of(off, r);
  double k[6] = {0, 0, 0, 0, 0, 0};
  for (int i = vb.id * blockDim.x + threadIdx.x; i < a.n; i += vb.n * blockDim.x) {
    double fac = a.mass[i];
    double sx = a.vv[3 * i] + a.uu[3 * i];
    double sy = a.vv[3 * i + 1] + a.uu[3 * i + 1];
    double sz = a.vv[3 * i + 2] + a.uu[3 * i + 2];
    k[0] += fac * sx * sx;
    k[1] += fac * sy * sx;
    k[2] += fac * sy * sy;
    k[3] += fac * sz * sx;
    k[4] += fac * sz * sy;
    k[5] += fac * sz * sz;
  }
  if (block_fix_final<6>(k, 20, a.facc, a.ticket, a.scal + SC_KEN, vb) && threadIdx.x == 0) {
    kinet_scalars(a.scal);
    nhc_chain_dev(a.nhc_M, a.nhc_Q, a.nfree, a.dt, a.zeta, a.scal);
  }
}

// [Nose-Hoover velocity scale, integrate_nhc.c:152-159] then the first half
// kick, drift and pbc_all (integrate_vverlet.c:54-83, vscal = 1)
__global__ void k_b_vv1(const BIntArgs *__restrict__ A, const int *__restrict__ off, int nbox,
                        int nhc) {
  const int r = vblk_box(off, nbox);
  const BIntArgs &a = A[r];
  const VBlk vb = vblk_of(off, r);
  int i = vb.id * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  double v[3];
  for (int c = 0; c < 3; c++) v[c] = a.vv[3 * i + c];
  if (nhc) {
    double scale = a.scal[SC_NHC_SCALE];
    for (int c = 0; c < 3; c++) {
      v[c] = v[c] * scale;
      a.uu[3 * i + c] = a.uu[3 * i + c] * scale;
    }
  }
  double imass = a.imass100[i];
  for (int c = 0; c < 3; c++) {
    v[c] = 1.0 * (v[c] + a.dt_h * imass * a.ff[3 * i + c]);
    a.vv[3 * i + c] = v[c];
  }
  double ddx = a.dt * v[0], ddy = a.dt * v[1], ddz = a.dt * v[2];
  a.nopbc[3 * i] += ddx;
  a.nopbc[3 * i + 1] += ddy;
  a.nopbc[3 * i + 2] += ddz;
  double4 p = a.pos[i];
  p.x += ddx;
  p.y += ddy;
  p.z += ddz;
  int bad = 0;
  p.x = pbc_wrap(p.x, a.H.x, a.L.x, &bad);
  p.y = pbc_wrap(p.y, a.H.y, a.L.y, &bad);
  p.z = pbc_wrap(p.z, a.H.z, a.L.z, &bad);
  if (bad) atomicOr(a.status, ST_PBC_LOOP);
  a.pos[i] = p;
}

// the energy assembly of forces() (block 0), the second half kick with uu =
// vv and the kinetic tensor; then either the record (NVE) or the second
// chain update (NHC)
__global__ void k_b_vv2(const BIntArgs *__restrict__ A, const int *__restrict__ off, int nbox,
                        int nhc) {
  const int r = vblk_box(off, nbox);
  const BIntArgs &a = A[r];
  const VBlk vb = vblk_of(off, r);
  if (vb.id == 0 && threadIdx.x == 0) {
    if (a.mixed) mixed_slots_dev(a.scal, a.erfc_rc_over_rc, a.mixed_fused);
    assemble_dev(a.scal, a.fan, a.sewald, 1);
  }
  double k[6] = {0, 0, 0, 0, 0, 0};
  for (int i = vb.id * blockDim.x + threadIdx.x; i < a.n; i += vb.n * blockDim.x) {
    double imass = a.imass100[i];
    double v[3];
    for (int c = 0; c < 3; c++) {
      v[c] = (a.vv[3 * i + c] + 1.0 * a.dt_h * imass * a.ff[3 * i + c]);
      a.vv[3 * i + c] = v[c];
      a.uu[3 * i + c] = v[c];
    }
    double fac = a.mass[i];
    double sx = v[0] + v[0], sy = v[1] + v[1], sz = v[2] + v[2];
    k[0] += fac * sx * sx;
    k[1] += fac * sy * sx;
    k[2] += fac * sy * sy;
    k[3] += fac * sz * sx;
    k[4] += fac * sz * sy;
    k[5] += fac * sz * sz;
  }
  if (block_fix_final<6>(k, 20, a.facc, a.ticket, a.scal + SC_KEN, vb) && threadIdx.x == 0) {
    kinet_scalars(a.scal);
    if (nhc) nhc_chain_dev(a.nhc_M, a.nhc_Q, a.nfree, a.dt, a.zeta, a.scal);
    else record_dev(a.scal, a.rec, a.rec_cap, a.rec_counter);
  }
}

// NHC: the second velocity scale, kinet of the scaled velocities and the record
__global__ void k_b_scale_kinet(const BIntArgs *__restrict__ A, const int *__restrict__ off,
                                int nbox, int chain_next) {
  const int r = vblk_box(off, nbox);
  const BIntArgs &a = A[r];
  const VBlk vb = vblk_of(off, r);
  double scale = a.scal[SC_NHC_SCALE];
  double k[6] = {0, 0, 0, 0, 0, 0};
  for (int i = vb.id * blockDim.x + threadIdx.x; i < a.n; i += vb.n * blockDim.x) {
    double v[3], u[3];
    for (int c = 0; c < 3; c++) {
      v[c] = a.vv[3 * i + c] * scale;
      u[c] = a.uu[3 * i + c] * scale;
      a.vv[3 * i + c] = v[c];
      a.uu[3 * i + c] = u[c];
    }
    double fac = a.mass[i];
    double sx = v[0] + u[0], sy = v[1] + u[1], sz = v[2] + u[2];
    k[0] += fac * sx * sx;
    k[1] += fac * sy * sx;
    k[2] += fac * sy * sy;
    k[3] += fac * sz * sx;
    k[4] += fac * sz * sy;
    k[5] += fac * sz * sz;
  }
  if (block_fix_final<6>(k, 20, a.facc, a.ticket, a.scal + SC_KEN, vb) && threadIdx.x == 0) {
    kinet_scalars(a.scal);
    record_dev(a.scal, a.rec, a.rec_cap, a.rec_counter);
    // the next step's first chain update needs the kinetic energy of exactly
    // these velocities (k_b_kinet_nhc would recompute the same sums)
    if (chain_next) nhc_chain_dev(a.nhc_M, a.nhc_Q, a.nfree, a.dt, a.zeta, a.scal);
  }
}

int launch_b_kinet_nhc(const BIntArgs *A, const int *off, int nbox, int blocks, cudaStream_t s) {
  k_b_kinet_nhc<<<blocks, 256, 0, s>>>(A, off, nbox);
  FE_LAUNCH_CHECK("k_b_kinet_nhc");
  return FE_OK;
}
int launch_b_vv1(const BIntArgs *A, const int *off, int nbox, int blocks, int nhc,
                 cudaStream_t s) {
  k_b_vv1<<<blocks, 256, 0, s>>>(A, off, nbox, nhc);
  FE_LAUNCH_CHECK("k_b_vv1");
  return FE_OK;
}
int launch_b_vv2(const BIntArgs *A, const int *off, int nbox, int blocks, int nhc,
                 cudaStream_t s) {
  k_b_vv2<<<blocks, 256, 0, s>>>(A, off, nbox, nhc);
  FE_LAUNCH_CHECK("k_b_vv2");
  return FE_OK;
}
int launch_b_scale_kinet(const BIntArgs *A, const int *off, int nbox, int blocks,
                         int chain_next, cudaStream_t s) {
  k_b_scale_kinet<<<blocks, 256, 0, s>>>(A, off, nbox, chain_next);
  FE_LAUNCH_CHECK("k_b_scale_kinet");
  return FE_OK;
}

}  // namespace fe
