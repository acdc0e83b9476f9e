// k_respa.cu -- reversible multiple time stepping (RESPA, Tuckerman et al.,
// J. Chem. Phys. 97, 1990 (1992)) on the FP64 drop-in, as the reference's
// integrate_mts.c:37-140 does it:
//   - fast forces (force_short.c:46-137): cbond, cbend, curey into ff_short;
//   - slow forces (force_long.c:46-145): ctorsion, cimproper and cnonbondnl
//     (the pair loop with SPME) into ff_long;
//   - one long step: a half kick with the slow forces, nsteps short steps
//     (half kick with the fast forces, drift of atom and atnopbc, pbc_all,
//     fast forces, half kick), the slow forces, a half kick with them, and
//     uu = vv;
//   - the Nose-Hoover form (integrate_mts_nhc.c:37-162): integrate_nhc over
//     half a long step at both ends of the long step (sim.xRESPA = 0) or over
//     half a short step at both ends of every short step (sim.xRESPA = 1);
//     its kicks carry no vscal.
// Compiled with -fmad=false; every kick keeps the reference's operation
// order (left to right: dt * imass * f, vscal applied where it applies it).
// Kernels fuse what runs site by site in a row: the opening slow kick with
// the first short step's kick and drift, the closing kick of one short step
// with the opening kick of the next, and the last closing fast kick with the
// slow one after the slow forces (neither kick reads what the forces write).
#include "fe_device.cuh"
#include "fe_internal.h"

namespace fe {

// integrate_mts.c:58-66 (when `lead`), nkick fast half kicks (:76-81,
// :111-115), the drift of atom and atnopbc (:86-97) and pbc_all
// (pbc_all.c:23-88)
__global__ void k_mts_drift(int n, int lead, int nkick, double vscal, double dt_longh,
                            double vs_dt_shorth, double dt, double3 L, double3 H,
                            const double *__restrict__ imass100,
                            const double *__restrict__ f_long, const double *__restrict__ f_short,
                            double *__restrict__ vv, double4 *__restrict__ pos,
                            double *__restrict__ nopbc, int *__restrict__ status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double imass = imass100[i];
  double d[3];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    double w = vv[3 * i + c];
    if (lead) w = vscal * (w + dt_longh * imass * f_long[3 * i + c]);
    for (int k = 0; k < nkick; k++) w = w + vs_dt_shorth * imass * f_short[3 * i + c];
    vv[3 * i + c] = w;
    d[c] = dt * w;
    nopbc[3 * i + c] += d[c];
  }
  double4 p = pos[i];
  p.x += d[0];
  p.y += d[1];
  p.z += d[2];
  int bad = 0;
  p.x = pbc_wrap(p.x, H.x, L.x, &bad);
  p.y = pbc_wrap(p.y, H.y, L.y, &bad);
  p.z = pbc_wrap(p.z, H.z, L.z, &bad);
  if (bad) atomicOr(status, ST_PBC_LOOP);
  pos[i] = p;
}

// a closing fast half kick (integrate_mts.c:111-115); on the last short
// step (`last`) also the slow one (:128-132) and uu = vv (:133-135)
__global__ void k_mts_close(int n, int last, double vs_dt_shorth, double vs_dt_longh,
                            const double *__restrict__ imass100,
                            const double *__restrict__ f_short, const double *__restrict__ f_long,
                            double *__restrict__ vv, double *__restrict__ uu) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * n) return;
  const double imass = imass100[i / 3];
  double w = vv[i];
  w = w + vs_dt_shorth * imass * f_short[i];
  if (last) {
    w = w + vs_dt_longh * imass * f_long[i];
    uu[i] = w;
  }
  vv[i] = w;
}

// ff_short and ff_long on first use, zeroed as the reference's allocation
int respa_alloc(Box *b) {
  const size_t bytes = sizeof(double) * 3 * (size_t)b->n;
  for (double **p : {&b->ff_short, &b->ff_long}) {
    if (*p) continue;
    FE_CUDA(cudaMalloc(p, bytes));
    FE_CUDA(cudaMemsetAsync(*p, 0, bytes, b->stream));
  }
  return FE_OK;
}

// force_short.c:46-137: the fast forces straight into ff_short
int respa_force_short(Box *b) {
  int rc = respa_alloc(b);
  if (rc) return rc;
  double *keep = b->ff;
  b->ff = b->ff_short;
  if (!(rc = launch_zero_forces(b)) && !(rc = launch_bonded64(b)))
    rc = launch_bonded_ext(b, false, 1);
  b->ff = keep;
  return rc;
}

// force_long.c:46-145: the slow forces into ff, then ff_long = ff
int respa_force_long(Box *b) {
  int rc = respa_alloc(b);
  if (rc) return rc;
  if ((rc = launch_zero_forces(b))) return rc;
  if ((rc = launch_bonded_ext(b, false, 6))) return rc;
  if ((rc = launch_pair64(b))) return rc;
  if ((rc = launch_pme64(b))) return rc;
  if ((rc = launch_apply_pme(b))) return rc;
  FE_CUDA(cudaMemcpyAsync(b->ff_long, b->ff, sizeof(double) * 3 * (size_t)b->n,
                          cudaMemcpyDeviceToDevice, b->stream));
  return FE_OK;
}

// integrate_mts.c:37-140 (xrespa < 0) or integrate_mts_nhc.c:37-162 with
// sim.xRESPA = xrespa (0 or 1): one long step of nshort short steps
int respa_step(Box *b, double vscal, int nshort, int xrespa) {
  int rc = respa_alloc(b);
  if (rc) return rc;
  if (xrespa >= 0) vscal = 1.0;  // integrate_mts_nhc.c kicks without it
  const double dt = b->p.dt;
  const double dtlong = dt * nshort;  // init.c:314, sim.dtlong = sim.dt * sim.nsteps
  const double dt_shorth = 0.5 * dt, dt_longh = 0.5 * dtlong;
  const double3 L = make_double3(b->p.L[0], b->p.L[1], b->p.L[2]);
  const double3 H = make_double3(b->p.L[0] / 2.0, b->p.L[1] / 2.0, b->p.L[2] / 2.0);
  const int blocks = (b->n + 255) / 256, blocks3 = (3 * b->n + 255) / 256;
  if (xrespa == 0 && (rc = launch_nhc(b, dt_longh))) return rc;
  for (int j = 0; j < nshort; j++) {
    if (xrespa == 1 && (rc = launch_nhc(b, dt_shorth))) return rc;
    // the closing kick of the previous short step joins this one's opening
    // kick unless a thermostat pass runs between them
    const int nkick = (j > 0 && xrespa != 1) ? 2 : 1;
    k_mts_drift<<<blocks, 256, 0, b->stream>>>(b->n, j == 0, nkick, vscal, dt_longh,
                                               vscal * dt_shorth, dt, L, H, b->imass100,
                                               b->ff_long, b->ff_short, b->vv, b->pos_q,
                                               b->pos_nopbc, b->status);
    FE_LAUNCH_CHECK("k_mts_drift");
    if ((rc = respa_force_short(b))) return rc;
    const bool last = j == nshort - 1;
    if (last && (rc = respa_force_long(b))) return rc;
    if (last || xrespa == 1) {
      k_mts_close<<<blocks3, 256, 0, b->stream>>>(b->n, last, vscal * dt_shorth,
                                                  vscal * dt_longh, b->imass100, b->ff_short,
                                                  b->ff_long, b->vv, b->uu);
      FE_LAUNCH_CHECK("k_mts_close");
    }
    if (xrespa == 1 && (rc = launch_nhc(b, dt_shorth))) return rc;
  }
  if (xrespa == 0 && (rc = launch_nhc(b, dt_longh))) return rc;
  return launch_assemble_energies(b, 1);
}

}  // namespace fe
