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

}  // namespace fe
