// k_integrate.cu -- FP64 per-site update kernels and the scalar bookkeeping of
// forces(): deterministic partial-sum reduction, reciprocal-force mean
// removal (pme_calc.c:268-277), energy assembly (cnonbond_nblist.c:613-620,
// forces.c:204-219), velocity Verlet (integrate_vverlet.c:36-103) with
// pbc_all (pbc_all.c:23-88), kinet (kinet.c:18-68) and the Nose-Hoover chain
// (integrate_nhc.c:40-161).  Compiled with -fmad=false.
#include <cstring>

#include "fe_device.cuh"

namespace fe {

// one block; sums partials[b * kPartialTerms + t] over b in a fixed order
__global__ void k_reduce(const double *__restrict__ partials, int nblocks, int nterms,
                         double *__restrict__ out, double scale) {
  __shared__ double sh[256];
  for (int t = 0; t < nterms; t++) {
    double s = 0.0;
    for (int bidx = threadIdx.x; bidx < nblocks; bidx += blockDim.x)
      s += partials[bidx * kPartialTerms + t];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
      if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[t] = sh[0] * scale;
    __syncthreads();
  }
}

int launch_reduce(Box *b, const double *partials, int nblocks, int nterms, int slot, double scale) {
  k_reduce<<<1, 256, 0, b->stream>>>(partials, nblocks, nterms, b->scal + slot, scale);
  FE_LAUNCH_CHECK("k_reduce");
  return FE_OK;
}

int launch_zero_forces(Box *b) {
  FE_CUDA(cudaMemsetAsync(b->ff, 0, sizeof(double) * 3 * b->n, b->stream));
  return FE_OK;
}

// ff += fp, then ff -= sum(fp)/n (pme_calc.c:198-200 and 268-277)
__global__ void k_apply_pme(int n, const double *__restrict__ fp, const double *__restrict__ scal,
                            double *__restrict__ ff) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * n) return;
  int c = i % 3;
  double mean = scal[SC_FMEAN + c] / (double)(n);
  double v = ff[i] + fp[i];
  ff[i] = v - mean;
}

int launch_apply_pme(Box *b) {
  k_apply_pme<<<(3 * b->n + 255) / 256, 256, 0, b->stream>>>(b->n, b->fp, b->scal, b->ff);
  FE_LAUNCH_CHECK("k_apply_pme");
  return FE_OK;
}

// energy[8] of cnonbondnl and en[k] of forces()
__global__ void k_assemble(double *__restrict__ s, double fan, double sewald, int with_bonded) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  assemble_dev(s, fan, sewald, with_bonded);
}

int launch_assemble_energies(Box *b, int with_bonded) {
  double fan = 0.5 * kELEC * kELEQ * kELEQ * kNA * 1.0E-3 / b->p.epsRF;
  k_assemble<<<1, 32, 0, b->stream>>>(b->scal, fan, b->sewald, with_bonded);
  FE_LAUNCH_CHECK("k_assemble");
  return FE_OK;
}

// integrate_vverlet.c:54-83: half kick, drift (atom and atnopbc), pbc_all
__global__ void k_vv1(int n, double vscal, double dt, double dt_h, double3 L, double3 H,
                      const double *__restrict__ imass100, const double *__restrict__ ff,
                      double *__restrict__ vv, double4 *__restrict__ pos,
                      double *__restrict__ nopbc, int *__restrict__ status) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double imass = imass100[i];
  double v0 = vscal * (vv[3 * i] + dt_h * imass * ff[3 * i]);
  double v1 = vscal * (vv[3 * i + 1] + dt_h * imass * ff[3 * i + 1]);
  double v2 = vscal * (vv[3 * i + 2] + dt_h * imass * ff[3 * i + 2]);
  vv[3 * i] = v0;
  vv[3 * i + 1] = v1;
  vv[3 * i + 2] = v2;
  double ddx = dt * v0, ddy = dt * v1, ddz = dt * v2;
  nopbc[3 * i] += ddx;
  nopbc[3 * i + 1] += ddy;
  nopbc[3 * i + 2] += ddz;
  double4 p = pos[i];
  p.x += ddx;
  p.y += ddy;
  p.z += ddz;
  int bad = 0;
  p.x = pbc_wrap(p.x, H.x, L.x, &bad);
  p.y = pbc_wrap(p.y, H.y, L.y, &bad);
  p.z = pbc_wrap(p.z, H.z, L.z, &bad);
  if (bad) atomicOr(status, ST_PBC_LOOP);
  pos[i] = p;
}

int launch_vv1(Box *b, double vscal) {
  if (b->mx) return launch_vv1_mx(b, vscal);
  double3 L = make_double3(b->p.L[0], b->p.L[1], b->p.L[2]);
  double3 H = make_double3(b->p.L[0] / 2.0, b->p.L[1] / 2.0, b->p.L[2] / 2.0);  // pbc_all.c hx
  double dt = b->p.dt, dt_h = 0.5 * b->p.dt;
  k_vv1<<<(b->n + 255) / 256, 256, 0, b->stream>>>(b->n, vscal, dt, dt_h, L, H, b->imass100, b->ff,
                                                   b->vv, b->pos_q, b->pos_nopbc, b->status);
  FE_LAUNCH_CHECK("k_vv1");
  return FE_OK;
}

__global__ void k_pbc(int n, double3 L, double4 *__restrict__ pos, int *__restrict__ status) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double4 p = pos[i];
  int bad = 0;
  p.x = pbc_wrap(p.x, L.x / 2.0, L.x, &bad);
  p.y = pbc_wrap(p.y, L.y / 2.0, L.y, &bad);
  p.z = pbc_wrap(p.z, L.z / 2.0, L.z, &bad);
  if (bad) atomicOr(status, ST_PBC_LOOP);
  pos[i] = p;
}

int launch_pbc(Box *b) {
  double3 L = make_double3(b->p.L[0], b->p.L[1], b->p.L[2]);
  k_pbc<<<(b->n + 255) / 256, 256, 0, b->stream>>>(b->n, L, b->pos_q, b->status);
  FE_LAUNCH_CHECK("k_pbc");
  return FE_OK;
}

// integrate_vverlet.c:93-102: second half kick and uu = vv
__global__ void k_vv2(int n, double vscal, double dt_h, const double *__restrict__ imass100,
                      const double *__restrict__ ff, double *__restrict__ vv,
                      double *__restrict__ uu) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double imass = imass100[i];
  for (int c = 0; c < 3; c++) {
    double v = (vv[3 * i + c] + vscal * dt_h * imass * ff[3 * i + c]);
    vv[3 * i + c] = v;
    uu[3 * i + c] = v;
  }
}

int launch_vv2(Box *b, double vscal) {
  double dt_h = 0.5 * b->p.dt;
  k_vv2<<<(b->n + 255) / 256, 256, 0, b->stream>>>(b->n, vscal, dt_h, b->imass100, b->ff, b->vv,
                                                   b->uu);
  FE_LAUNCH_CHECK("k_vv2");
  return FE_OK;
}

// integrate_vverlet.c:93-102 and kinet.c:31-65 in one pass: second half
// kick, uu = vv, and the kinetic tensor of the new velocities
__global__ void k_vv2_kinet(int n, double vscal, double dt_h, const double *__restrict__ mass,
                            const double *__restrict__ imass100,
                            const double *__restrict__ ff, double *__restrict__ vv,
                            double *__restrict__ uu, unsigned long long *__restrict__ facc,
                            unsigned *__restrict__ ticket, double *__restrict__ s) {
  double k[6] = {0, 0, 0, 0, 0, 0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double imass = imass100[i];
    double v[3];
    for (int c = 0; c < 3; c++) {
      v[c] = (vv[3 * i + c] + vscal * dt_h * imass * ff[3 * i + c]);
      vv[3 * i + c] = v[c];
      uu[3 * i + c] = v[c];
    }
    double fac = mass[i];
    double sx = v[0] + v[0], sy = v[1] + v[1], sz = v[2] + v[2];
    k[0] += fac * sx * sx;
    k[1] += fac * sy * sx;
    k[2] += fac * sy * sy;
    k[3] += fac * sz * sx;
    k[4] += fac * sz * sy;
    k[5] += fac * sz * sz;
  }
  // exact fixed-point sums (2^-20 amu A^2/ps^2 resolution): no FP64 tree
  if (block_fix_final<6>(k, 20, facc, ticket, s + SC_KEN) && threadIdx.x == 0) {
    double f = (0.125) * (kNA * kAU * 10.0);  // kinet.c:50-65
    for (int i = 0; i < 6; i++) s[SC_KEN + i] *= f;
    s[FE_EN_KINET] = s[SC_KEN + 0] + s[SC_KEN + 2] + s[SC_KEN + 5];
  }
}

int launch_vv2_kinet(Box *b, double vscal) {
  double dt_h = 0.5 * b->p.dt;
  int blocks = (b->n + 255) / 256;
  if (blocks > 512) blocks = 512;
  k_vv2_kinet<<<blocks, 256, 0, b->stream>>>(b->n, vscal, dt_h, b->mass, b->imass100, b->ff, b->vv, b->uu,
                                             b->facc, b->ticket, b->scal);
  FE_LAUNCH_CHECK("k_vv2_kinet");
  return FE_OK;
}

// kinet.c:31-43 partial sums of the kinetic tensor
__global__ void k_kinet(int n, const double *__restrict__ mass, const double *__restrict__ vv,
                        const double *__restrict__ uu, double *__restrict__ partials) {
  double k[6] = {0, 0, 0, 0, 0, 0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double fac = mass[i];
    double sx = vv[3 * i] + uu[3 * i];
    double sy = vv[3 * i + 1] + uu[3 * i + 1];
    double sz = vv[3 * i + 2] + uu[3 * i + 2];
    k[0] += fac * sx * sx;
    k[1] += fac * sy * sx;
    k[2] += fac * sy * sy;
    k[3] += fac * sz * sx;
    k[4] += fac * sz * sy;
    k[5] += fac * sz * sz;
  }
  block_partials<6>(k, partials);
}

// kinet.c:50-65 unit conversion and the scalar
__global__ void k_kinet_final(double *__restrict__ s) {
  if (threadIdx.x != 0) return;
  double f = (0.125) * (kNA * kAU * 10.0);
  for (int i = 0; i < 6; i++) s[SC_KEN + i] *= f;
  s[FE_EN_KINET] = s[SC_KEN + 0] + s[SC_KEN + 2] + s[SC_KEN + 5];
}

// kinet for the mixed-precision path: the same tensor in one launch, summed
// in exact fixed point (2^-20 amu A^2/ps^2) like the fused second half kick
__global__ void k_kinet_fix(int n, const double *__restrict__ mass, const double *__restrict__ vv,
                            const double *__restrict__ uu, unsigned long long *__restrict__ facc,
                            unsigned *__restrict__ ticket, double *__restrict__ s) {
  double k[6] = {0, 0, 0, 0, 0, 0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double fac = mass[i];
    double sx = vv[3 * i] + uu[3 * i];
    double sy = vv[3 * i + 1] + uu[3 * i + 1];
    double sz = vv[3 * i + 2] + uu[3 * i + 2];
    k[0] += fac * sx * sx;
    k[1] += fac * sy * sx;
    k[2] += fac * sy * sy;
    k[3] += fac * sz * sx;
    k[4] += fac * sz * sy;
    k[5] += fac * sz * sz;
  }
  if (block_fix_final<6>(k, 20, facc, ticket, s + SC_KEN) && threadIdx.x == 0) {
    double f = (0.125) * (kNA * kAU * 10.0);  // kinet.c:50-65
    for (int i = 0; i < 6; i++) s[SC_KEN + i] *= f;
    s[FE_EN_KINET] = s[SC_KEN + 0] + s[SC_KEN + 2] + s[SC_KEN + 5];
  }
}

// drift(ibox), drift.c:21-66: the net momentum P = sum m v divided by the
// number of sites, then v_i -= (P / n) / m_i (velocities only, uu kept).
__global__ void k_momentum(int n, const double *__restrict__ mass, const double *__restrict__ vv,
                           double *__restrict__ partials) {
  double v[3] = {0.0, 0.0, 0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double m = mass[i];
    v[0] += m * vv[3 * i];
    v[1] += m * vv[3 * i + 1];
    v[2] += m * vv[3 * i + 2];
  }
  block_partials<3>(v, partials);
}

__global__ void k_drift_remove(int n, const double *__restrict__ mass, const double *__restrict__ p,
                               double *__restrict__ vv) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double ns = 1.0 * n;
  double imass = 1.0 / mass[i];
  vv[3 * i] -= (p[0] / ns) * imass;
  vv[3 * i + 1] -= (p[1] / ns) * imass;
  vv[3 * i + 2] -= (p[2] / ns) * imass;
}

int launch_drift(Box *b) {
  int blocks = (b->n + 255) / 256;
  if (blocks > 1024) blocks = 1024;
  k_momentum<<<blocks, 256, 0, b->stream>>>(b->n, b->mass, b->vv, b->partials);
  FE_LAUNCH_CHECK("k_momentum");
  int rc = launch_reduce(b, b->partials, blocks, 3, SC_ENERGY3, 1.0);  // scratch slots
  if (rc) return rc;
  k_drift_remove<<<(b->n + 255) / 256, 256, 0, b->stream>>>(b->n, b->mass, b->scal + SC_ENERGY3,
                                                           b->vv);
  FE_LAUNCH_CHECK("k_drift_remove");
  return FE_OK;
}

int launch_kinet(Box *b) {
  int blocks = (b->n + 255) / 256;
  if (blocks > 512) blocks = 512;
  if (b->mx) {
    k_kinet_fix<<<blocks, 256, 0, b->stream>>>(b->n, b->mass, b->vv, b->uu, b->facc, b->ticket,
                                               b->scal);
    FE_LAUNCH_CHECK("k_kinet_fix");
    return FE_OK;
  }
  k_kinet<<<blocks, 256, 0, b->stream>>>(b->n, b->mass, b->vv, b->uu, b->partials);
  FE_LAUNCH_CHECK("k_kinet");
  int rc = launch_reduce(b, b->partials, blocks, 6, SC_KEN, 1.0);
  if (rc) return rc;
  k_kinet_final<<<1, 32, 0, b->stream>>>(b->scal);
  FE_LAUNCH_CHECK("k_kinet_final");
  return FE_OK;
}


__global__ void k_nhc_chain(int M, double Q, double nfree, double time_step,
                            double *__restrict__ zeta, double *__restrict__ s) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  nhc_chain_dev(M, Q, nfree, time_step, zeta, s);
}

// integrate_nhc.c:152-159
__global__ void k_nhc_scale(int n3, const double *__restrict__ s, double *__restrict__ vv,
                            double *__restrict__ uu) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n3) return;
  double scale = s[SC_NHC_SCALE];
  vv[i] = vv[i] * scale;
  uu[i] = uu[i] * scale;
}

int launch_nhc(Box *b, double time_step) {
  int rc = launch_kinet(b);  // integrate_nhc.c:68
  if (rc) return rc;
  k_nhc_chain<<<1, 32, 0, b->stream>>>(b->nhc_M, b->nhc_Q, b->nfree, time_step, b->zeta,
                                       b->scal);
  FE_LAUNCH_CHECK("k_nhc_chain");
  k_nhc_scale<<<(3 * b->n + 255) / 256, 256, 0, b->stream>>>(3 * b->n, b->scal, b->vv, b->uu);
  FE_LAUNCH_CHECK("k_nhc_scale");
  return FE_OK;
}

__global__ void k_record(const double *__restrict__ s, double *__restrict__ rec, long cap,
                         int *__restrict__ counter) {
  int c = *counter;
  if (threadIdx.x < FE_EN_COUNT && c < cap) rec[(long)c * FE_EN_COUNT + threadIdx.x] = s[threadIdx.x];
  __syncthreads();
  if (threadIdx.x == 0) *counter = c + 1;
}

__global__ void k_xyz_scatter(int n, const double *__restrict__ xyz, double4 *__restrict__ pos,
                              double *__restrict__ nopbc) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
  if (pos) {
    double4 p = pos[i];
    p.x = x;
    p.y = y;
    p.z = z;
    pos[i] = p;
  }
  if (nopbc) {
    nopbc[3 * i] = x;
    nopbc[3 * i + 1] = y;
    nopbc[3 * i + 2] = z;
  }
}

__global__ void k_xyz_gather(int n, const double4 *__restrict__ pos, double *__restrict__ xyz) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double4 p = pos[i];
  xyz[3 * i] = p.x;
  xyz[3 * i + 1] = p.y;
  xyz[3 * i + 2] = p.z;
}

int launch_xyz_scatter(Box *b, const double *xyz, bool to_pos, bool to_nopbc) {
  k_xyz_scatter<<<(b->n + 255) / 256, 256, 0, b->stream>>>(b->n, xyz, to_pos ? b->pos_q : nullptr,
                                                           to_nopbc ? b->pos_nopbc : nullptr);
  FE_LAUNCH_CHECK("k_xyz_scatter");
  return FE_OK;
}

int launch_xyz_gather(Box *b, double *xyz) {
  k_xyz_gather<<<(b->n + 255) / 256, 256, 0, b->stream>>>(b->n, b->pos_q, xyz);
  FE_LAUNCH_CHECK("k_xyz_gather");
  return FE_OK;
}

BIntArgs make_bint_args(Box *b) {
  BIntArgs a;
  memset(&a, 0, sizeof a);
  a.n = b->n;
  a.nhc_M = b->nhc_M;
  a.dt = b->p.dt;
  a.dt_h = 0.5 * b->p.dt;
  a.nhc_Q = b->nhc_Q;
  a.nfree = b->nfree;
  a.L = make_double3(b->p.L[0], b->p.L[1], b->p.L[2]);
  a.H = make_double3(b->p.L[0] / 2.0, b->p.L[1] / 2.0, b->p.L[2] / 2.0);
  a.mass = b->mass;
  a.imass100 = b->imass100;
  a.ff = b->ff;
  a.vv = b->vv;
  a.uu = b->uu;
  a.nopbc = b->pos_nopbc;
  a.pos = b->pos_q;
  a.zeta = b->zeta;
  a.scal = b->scal;
  a.facc = b->facc;
  a.ticket = b->ticket;
  a.status = b->status;
  a.rec = b->rec;
  a.rec_cap = b->rec_cap;
  a.rec_counter = b->rec_counter;
  a.fan = 0.5 * kELEC * kELEQ * kELEQ * kNA * 1.0E-3 / b->p.epsRF;
  a.sewald = b->sewald;
  a.mixed = b->mx != nullptr;
  mixed_bint_fields(b, &a);
  return a;
}

int launch_record(Box *b) {
  k_record<<<1, 32, 0, b->stream>>>(b->scal, b->rec, b->rec_cap, b->rec_counter);
  FE_LAUNCH_CHECK("k_record");
  return FE_OK;
}

}  // namespace fe
