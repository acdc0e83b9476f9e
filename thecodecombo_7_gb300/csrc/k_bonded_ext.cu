// k_bonded_ext.cu -- the bonded terms of forces() beyond bonds and bends:
// Urey-Bradley 1-3 terms (curey.c:37-106), proper torsions (ctorsion.c:63-246)
// and improper torsions (cimproper.c:55-221), in FP64 for both precisions.
//
// One thread per term.  The torsion and improper geometry is the reference's
// (unit bond vectors, the two cross products with the central bond, the sign
// from their cross product along it, tau = sign * acos of the clamped
// cosine) and its force transformation onto the four sites; only the order of
// the final per-site sums differs (atomics).  The drop-in precision adds the
// forces to ff through FP64 atomics; the mixed precision adds them to the
// 64-bit fixed-point force sums (2^32 per kJ/mol/A, exact and order-free).
// Energies are summed exactly in 64-bit fixed point (2^-32 kJ/mol) and land in
// the slots SC_UREY, SC_TORS, SC_IMPR.  These terms are few (a few per
// molecule) and run once per force evaluation, so FP64 costs little here and
// keeps acos well conditioned near 0 and pi.
#include "fe_device.cuh"
#include "fe_mixed.h"

namespace fe {

constexpr double kExtFix = 4294967296.0;  // 2^32: the mixed force sums' scale

__device__ __forceinline__ void min_image3(double3 L, double3 H, double *d) {
  double l[3] = {L.x, L.y, L.z}, h[3] = {H.x, H.y, H.z};
#pragma unroll
  for (int c = 0; c < 3; c++) {
    if (d[c] > h[c]) d[c] -= l[c];
    else if (d[c] < -h[c]) d[c] += l[c];
  }
}

template <bool FIXED>
__device__ __forceinline__ void add_force(double *ff, unsigned long long *fix, int i, int c,
                                          double v) {
  if (FIXED)
    atomicAdd(&fix[3 * i + c], (unsigned long long)__double2ll_rn(v * kExtFix));
  else
    atomicAdd(&ff[3 * i + c], v);
}

struct ExtArgs {
  double3 L, H;
  int nurey, ntors, nimpr;
  const int *urey_ab;
  const double *urey_seq, *urey_k;
  const int *tors_abcd;
  const double *tors_par;  // 18 per torsion: kphi[6], nphi[6], delphi[6]
  double *tors_tau;
  const int *impr_abcd;
  const double *impr_k, *impr_eq;
  // the terms evaluated: [t0, t1) of urey, then torsion, then improper
  // order; `kinds` (bit 0 urey, 1 torsion, 2 improper) are the energies
  // written to fin[0..2] when not all three are evaluated
  int t0, t1, kinds;
  double *fin;
};

// the dihedral (a, b, c, d) and its generalised force fr = -dE/dtau applied
// to the four sites (ctorsion.c:80-246, cimproper.c:71-221)
struct Dihedral {
  double u[3], w[3];  // eab x ebc, ecd x ebc
  double rab, rbc, rcd, irab, irbc, ircd, cosb, cosc, isinb2, isinc2;
  double tau;
};

__device__ __forceinline__ void dihedral_geom(const double4 *__restrict__ pos, double3 L,
                                              double3 H, int ia, int ib, int ic, int id,
                                              Dihedral &D) {
  double4 A = pos[ia], B = pos[ib], Cc = pos[ic], Dd = pos[id];
  double dab[3] = {B.x - A.x, B.y - A.y, B.z - A.z};
  double dbc[3] = {Cc.x - B.x, Cc.y - B.y, Cc.z - B.z};
  double dcd[3] = {Dd.x - Cc.x, Dd.y - Cc.y, Dd.z - Cc.z};
  min_image3(L, H, dab);
  min_image3(L, H, dbc);
  min_image3(L, H, dcd);
  D.rab = sqrt(dab[0] * dab[0] + dab[1] * dab[1] + dab[2] * dab[2]);
  D.irab = 1.0 / D.rab;
  D.rbc = sqrt(dbc[0] * dbc[0] + dbc[1] * dbc[1] + dbc[2] * dbc[2]);
  D.irbc = 1.0 / D.rbc;
  D.rcd = sqrt(dcd[0] * dcd[0] + dcd[1] * dcd[1] + dcd[2] * dcd[2]);
  D.ircd = 1.0 / D.rcd;
  double eab[3], ebc[3], ecd[3];
#pragma unroll
  for (int c = 0; c < 3; c++) {
    eab[c] = dab[c] * D.irab;
    ebc[c] = dbc[c] * D.irbc;
    ecd[c] = dcd[c] * D.ircd;
  }
  D.u[0] = eab[1] * ebc[2] - eab[2] * ebc[1];
  D.u[1] = eab[2] * ebc[0] - eab[0] * ebc[2];
  D.u[2] = eab[0] * ebc[1] - eab[1] * ebc[0];
  D.cosb = -(eab[0] * ebc[0] + eab[1] * ebc[1] + eab[2] * ebc[2]);
  D.isinb2 = 1.0 / (1.0 - D.cosb * D.cosb);
  D.w[0] = ecd[1] * ebc[2] - ecd[2] * ebc[1];
  D.w[1] = ecd[2] * ebc[0] - ecd[0] * ebc[2];
  D.w[2] = ecd[0] * ebc[1] - ecd[1] * ebc[0];
  D.cosc = -(ecd[0] * ebc[0] + ecd[1] * ebc[1] + ecd[2] * ebc[2]);
  D.isinc2 = 1.0 / (1.0 - D.cosc * D.cosc);
  double x0 = -(D.u[1] * D.w[2] - D.u[2] * D.w[1]);
  double x1 = -(D.u[2] * D.w[0] - D.u[0] * D.w[2]);
  double x2 = -(D.u[0] * D.w[1] - D.u[1] * D.w[0]);
  double num = x0 * ebc[0] + x1 * ebc[1] + x2 * ebc[2];
  double costau = -(D.u[0] * D.w[0] + D.u[1] * D.w[1] + D.u[2] * D.w[2]) * sqrt(D.isinb2) *
                  sqrt(D.isinc2);
  costau = fmin(1.0, fmax(-1.0, costau));
  D.tau = (num >= 0.0 ? 1.0 : -1.0) * acos(costau);
}

template <bool FIXED>
__device__ __forceinline__ void dihedral_force(const Dihedral &D, double fr, int ia, int ib,
                                               int ic, int id, double *ff,
                                               unsigned long long *fix) {
  double fa = -fr * D.irab * D.isinb2;
  double fb1 = fr * (D.rbc - D.rab * D.cosb) * D.irab * D.irbc * D.isinb2;
  double fb2 = fr * D.cosc * D.irbc * D.isinc2;
  double fc1 = fr * (D.rbc - D.rcd * D.cosc) * D.ircd * D.irbc * D.isinc2;
  double fc2 = fr * D.cosb * D.irbc * D.isinb2;
  double fd = -fr * D.ircd * D.isinc2;
#pragma unroll
  for (int c = 0; c < 3; c++) {
    add_force<FIXED>(ff, fix, ia, c, fa * D.u[c]);
    add_force<FIXED>(ff, fix, ib, c, fb1 * D.u[c] + fb2 * D.w[c]);
    add_force<FIXED>(ff, fix, ic, c, fc1 * D.w[c] + fc2 * D.u[c]);
    add_force<FIXED>(ff, fix, id, c, fd * D.w[c]);
  }
}

template <bool FIXED>
__global__ void __launch_bounds__(256)
k_bonded_ext(ExtArgs a, const double4 *__restrict__ pos, double *__restrict__ ff,
             unsigned long long *__restrict__ fix, unsigned long long *__restrict__ facc,
             unsigned *__restrict__ ticket, double *__restrict__ out) {
  double e[3] = {0.0, 0.0, 0.0};  // urey, torsion, improper
  for (int t = a.t0 + blockIdx.x * blockDim.x + threadIdx.x; t < a.t1;
       t += gridDim.x * blockDim.x) {
    if (t < a.nurey) {
      int ia = a.urey_ab[2 * t], ib = a.urey_ab[2 * t + 1];
      double4 A = pos[ia], B = pos[ib];
      double d[3] = {B.x - A.x, B.y - A.y, B.z - A.z};
      min_image3(a.L, a.H, d);
      double dr = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      double dri = 1.0 / dr;
      double rr = dr - a.urey_seq[t];
      double fr = -a.urey_k[t] * rr * 2.0;
      e[0] += -(fr * rr * 0.5);
#pragma unroll
      for (int c = 0; c < 3; c++) {
        double f = fr * dri * d[c];
        add_force<FIXED>(ff, fix, ia, c, -f);
        add_force<FIXED>(ff, fix, ib, c, f);
      }
    } else if (t < a.nurey + a.ntors) {
      int u = t - a.nurey;
      const int *q = a.tors_abcd + 4 * u;
      Dihedral D;
      dihedral_geom(pos, a.L, a.H, q[0], q[1], q[2], q[3], D);
      a.tors_tau[u] = D.tau;
      const double *kp = a.tors_par + 18 * u;
      double fr = 0.0, et = 0.0;
      for (int s = 0; s < 6; s++) {  // the series ends at the first zero kphi
        if (kp[s] == 0.0) break;
        double arg = kp[6 + s] * D.tau - kp[12 + s];
        fr += kp[s] * kp[6 + s] * sin(arg);
        et += kp[s] * (1.0 + cos(arg));
      }
      e[1] += et;
      dihedral_force<FIXED>(D, fr, q[0], q[1], q[2], q[3], ff, fix);
    } else {
      int u = t - a.nurey - a.ntors;
      const int *q = a.impr_abcd + 4 * u;
      Dihedral D;
      dihedral_geom(pos, a.L, a.H, q[0], q[1], q[2], q[3], D);
      double rr = D.tau - a.impr_eq[u];
      double fr = -2.0 * a.impr_k[u] * rr;
      e[2] += -fr * rr * 0.5;
      dihedral_force<FIXED>(D, fr, q[0], q[1], q[2], q[3], ff, fix);
    }
  }
  const bool last = block_fix_final<3>(e, 32, facc, ticket, out);
  // a subset of the kinds: only their energies leave the scratch slots
  if (last && a.kinds != 7 && threadIdx.x < 3 && ((a.kinds >> threadIdx.x) & 1))
    a.fin[threadIdx.x] = out[threadIdx.x];
}

int launch_bonded_ext(Box *b, bool to_fixed, int kinds) {
  const int tot = b->nurey + b->ntors + b->nimpr;
  ExtArgs a;
  a.t0 = (kinds & 1) ? 0 : (kinds & 2) ? b->nurey : b->nurey + b->ntors;
  a.t1 = (kinds & 4) ? tot : (kinds & 2) ? b->nurey + b->ntors : b->nurey;
  a.kinds = kinds;
  a.fin = b->scal + SC_UREY;
  if (tot == 0) return FE_OK;
  if (a.t1 <= a.t0) {  // none of these kinds: their energies are zero
    for (int k = 0; k < 3; k++)
      if ((kinds >> k) & 1) FE_CUDA(cudaMemsetAsync(b->scal + SC_UREY + k, 0, sizeof(double), b->stream));
    return FE_OK;
  }
  a.L = make_double3(b->p.L[0], b->p.L[1], b->p.L[2]);
  a.H = make_double3(b->p.L[0] / 2.0, b->p.L[1] / 2.0, b->p.L[2] / 2.0);
  a.nurey = b->nurey;
  a.ntors = b->ntors;
  a.nimpr = b->nimpr;
  a.urey_ab = b->urey_ab;
  a.urey_seq = b->urey_seq;
  a.urey_k = b->urey_k;
  a.tors_abcd = b->tors_abcd;
  a.tors_par = b->tors_par;
  a.tors_tau = b->tors_tau;
  a.impr_abcd = b->impr_abcd;
  a.impr_k = b->impr_k;
  a.impr_eq = b->impr_eq;
  int blocks = (a.t1 - a.t0 + 255) / 256;
  if (blocks > 1024) blocks = 1024;
  if (to_fixed) {
    if (!b->mx) {
      set_error("fixed-point bonded terms need a mixed-precision box");
      return FE_ERR_STATE;
    }
    k_bonded_ext<true><<<blocks, 256, 0, b->stream>>>(a, b->pos_q, nullptr, b->mx->fix, b->facc,
                                                      b->ticket, b->scal + SC_UREY);
  } else {
    k_bonded_ext<false><<<blocks, 256, 0, b->stream>>>(
        a, b->pos_q, b->ff, nullptr, b->facc, b->ticket,
        b->scal + (kinds == 7 ? SC_UREY : SC_EXT_TMP));
  }
  FE_LAUNCH_CHECK("k_bonded_ext");
  return FE_OK;
}

}  // namespace fe
