// k_pair64.cu -- FP64 drop-in kernels of forces(): the non-bonded pair loop
// of cnonbondnl (cnonbond_nblist.c:134-523, SPME + STYPE branch) and the
// bonded terms cbond (cbond.c:27-180) and cbend (cbend.c:24-218).
//
// Compiled with -fmad=false: each expression is evaluated with the
// reference's roundings, so per-pair forces and energies equal the
// reference's up to CUDA's exp (<= 1 ulp from glibc's).  Only the order of
// the final force sums differs (Newton-3 scatter through FP64 atomics).
#include "fe_device.cuh"

namespace fe {

struct PairParams {
  double3 L, H;
  double rc, rc2, kappa, kpi, epsRF, erfc_rc;
  double ron2, sw_den;  // optional CHARMM switch (ron2 = 0: off)
  int lj_form;          // 0 CHARMM (the reference's default build); 2 its BGO build
  int n, nt, max_nb;
};

// One warp per row a of the half list; lanes walk the row's entries.
__global__ void __launch_bounds__(128)
k_pair64(PairParams P, const double4 *__restrict__ pos, const int *__restrict__ type,
         const double *__restrict__ lj_eps, const double *__restrict__ lj_sig,
         const int *__restrict__ count, const int *__restrict__ ent, double *__restrict__ ff,
         double *__restrict__ partials) {
  int lane = threadIdx.x & 31;
  int wpb = blockDim.x >> 5;
  double e_lj = 0.0, e_ljs = 0.0, e_real = 0.0, e_reals = 0.0, e_intra = 0.0;
  for (int a = blockIdx.x * wpb + (threadIdx.x >> 5); a < P.n - 1; a += gridDim.x * wpb) {
    double4 pa = pos[a];
    int ta = type[a];
    int cnt = count[a];
    const int *row = ent + (size_t)a * P.max_nb;
    double fxa = 0.0, fya = 0.0, fza = 0.0;
    for (int bb = lane; bb < cnt; bb += 32) {
      int e = row[bb];
      int b = e >> 3, xflag = e & 7;
      double4 pb = pos[b];
      double dx = pa.x - pb.x;
      double dy = pa.y - pb.y;
      double dz = pa.z - pb.z;
      if (dx > P.H.x) dx -= P.L.x;
      else if (dx < -P.H.x) dx += P.L.x;
      if (dy > P.H.y) dy -= P.L.y;
      else if (dy < -P.H.y) dy += P.L.y;
      if (dz > P.H.z) dz -= P.L.z;
      else if (dz < -P.H.z) dz += P.L.z;
      double dr2 = dx * dx + dy * dy + dz * dz;
      if (dr2 > P.rc2) continue;
      int tb = type[b];
      double sig = lj_sig[ta * P.nt + tb];
      double eps = lj_eps[ta * P.nt + tb];
      double qq = qfactor_mul(pa.w * pb.w);
      double qqab = qq;
      if (xflag) {
        if (xflag != 4) {
          sig = 0.0;
          eps = 0.0;
          qq = 0.0;
        } else {
          qq *= kE14FAC;
        }
      }
      double force = 0.0;
      if ((eps * sig) != 0.0) {
        double sr2 = (sig * sig) / dr2;
        double sr6 = sr2 * sr2 * sr2;
        double sr12 = sr6 * sr6;
        double flj = (12.0 * eps / dr2) * (sr12 - sr6);
        double elj = eps * (sr12 - 2.0 * sr6);
        if (P.lj_form == 2) {
          // the BGO build (cnonbond_nblist.c:294-307): eps [13 (R/r)^12 -
          // 18 (R/r)^10 + 4 (R/r)^6], shifted sum at rc as the default form
          double sr10 = sr6 * sr2 * sr2;
          double sr2s = (sig * sig) / P.rc2;
          double sr6s = sr2s * sr2s * sr2s;
          double sr12s = sr6s * sr6s;
          double sr10s = sr6s * sr2s * sr2s;
          force = eps / dr2 * (156.0 * sr12 - 180.0 * sr10 + 24.0 * sr6);
          e_lj += eps * (13.0 * sr12 - 18.0 * sr10 + 4.0 * sr6);
          e_ljs += eps * (13.0 * sr12s - 18.0 * sr10s + 4.0 * sr6s);
        } else if (P.ron2 > 0.0) {
          if (dr2 > P.ron2) {
            double c = P.rc2 - dr2;
            double sw = c * c * (P.rc2 + 2.0 * dr2 - 3.0 * P.ron2) / P.sw_den;
            double dsw = 12.0 * c * (dr2 - P.ron2) / P.sw_den;
            flj = flj * sw + elj * dsw;
            elj = elj * sw;
          }
          force = flj;
          e_lj += elj;
        } else {
          double sr2s = (sig * sig) / P.rc2;
          double sr6s = sr2s * sr2s * sr2s;
          double sr12s = sr6s * sr6s;
          force = flj;
          e_lj += elj;
          e_ljs += eps * (sr12s - 2.0 * sr6s);
        }
      }
      double dr = sqrt(dr2);
      double dri = 1.0 / dr;
      double kr = P.kappa * dr;
      double erfckr = ref_erfc(kr);
      double kpidrexpkr2 = 2.0 * P.kpi * dr * exp(-kr * kr);
      qq /= P.epsRF;
      if (qq != 0.0) {
        e_real += qq * erfckr * dri;
        e_reals += qq * P.erfc_rc / P.rc;
        force += (qq * dri / dr2) * (erfckr + kpidrexpkr2);
      }
      if (xflag) {
        if (xflag == 4) qqab *= (1.0 - kE14FAC);
        e_intra += qqab * (1.0 - erfckr) * dri;
        force -= (qqab * dri / dr2) * ((1.0 - erfckr) - kpidrexpkr2);
      }
      if (force != 0.0) {
        double fx = force * dx, fy = force * dy, fz = force * dz;
        fxa += fx;
        fya += fy;
        fza += fz;
        atomicAdd(&ff[3 * b], -fx);
        atomicAdd(&ff[3 * b + 1], -fy);
        atomicAdd(&ff[3 * b + 2], -fz);
      }
    }
    fxa = warp_sum(fxa);
    fya = warp_sum(fya);
    fza = warp_sum(fza);
    if (lane == 0) {
      atomicAdd(&ff[3 * a], fxa);
      atomicAdd(&ff[3 * a + 1], fya);
      atomicAdd(&ff[3 * a + 2], fza);
    }
  }
  double v[5] = {e_lj, e_ljs, e_real, e_reals, e_intra};
  block_partials<5>(v, partials);
}

__global__ void __launch_bounds__(256)
k_bonded64(int nbond, int nbend, double3 L, const double4 *__restrict__ pos,
           const int *__restrict__ bond_ab, const double *__restrict__ bond_req,
           const double *__restrict__ bond_k, const int *__restrict__ bend_abc,
           const double *__restrict__ bend_t0, const double *__restrict__ bend_k,
           double *__restrict__ ff, double *__restrict__ partials) {
  double eb = 0.0, ea = 0.0;
  const double hx = L.x / 2.0, hy = L.y / 2.0, hz = L.z / 2.0;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nbond + nbend;
       t += gridDim.x * blockDim.x) {
    if (t < nbond) {
      int ia = bond_ab[2 * t], ib = bond_ab[2 * t + 1];
      double4 A = pos[ia], B = pos[ib];
      double dx = B.x - A.x, dy = B.y - A.y, dz = B.z - A.z;
      if (dx > hx) dx -= L.x;
      else if (dx < -hx) dx += L.x;
      if (dy > hy) dy -= L.y;
      else if (dy < -hy) dy += L.y;
      if (dz > hz) dz -= L.z;
      else if (dz < -hz) dz += L.z;
      double drr = dx * dx + dy * dy + dz * dz;
      double dr = sqrt(drr);
      double dri = 1.0 / dr;
      double rr = dr - bond_req[t];
      double fr = -bond_k[t] * rr * 2.0;
      eb += -(fr * rr * 0.5);
      double fx = fr * dri * dx, fy = fr * dri * dy, fz = fr * dri * dz;
      atomicAdd(&ff[3 * ia], -fx);
      atomicAdd(&ff[3 * ia + 1], -fy);
      atomicAdd(&ff[3 * ia + 2], -fz);
      atomicAdd(&ff[3 * ib], fx);
      atomicAdd(&ff[3 * ib + 1], fy);
      atomicAdd(&ff[3 * ib + 2], fz);
    } else {
      int u = t - nbond;
      int ia = bend_abc[3 * u], ib = bend_abc[3 * u + 1], ic = bend_abc[3 * u + 2];
      double4 A = pos[ia], B = pos[ib], Cc = pos[ic];
      double dax = A.x - B.x, day = A.y - B.y, daz = A.z - B.z;
      double dcx = Cc.x - B.x, dcy = Cc.y - B.y, dcz = Cc.z - B.z;
      if (dax > hx) dax -= L.x;
      else if (dax < -hx) dax += L.x;
      if (day > hy) day -= L.y;
      else if (day < -hy) day += L.y;
      if (daz > hz) daz -= L.z;
      else if (daz < -hz) daz += L.z;
      if (dcx > hx) dcx -= L.x;
      else if (dcx < -hx) dcx += L.x;
      if (dcy > hy) dcy -= L.y;
      else if (dcy < -hy) dcy += L.y;
      if (dcz > hz) dcz -= L.z;
      else if (dcz < -hz) dcz += L.z;
      double drai = 1.0 / sqrt(dax * dax + day * day + daz * daz);
      double erax = dax * drai, eray = day * drai, eraz = daz * drai;
      double drci = 1.0 / sqrt(dcx * dcx + dcy * dcy + dcz * dcz);
      double ercx = dcx * drci, ercy = dcy * drci, ercz = dcz * drci;
      double cosphi = erax * ercx + eray * ercy + eraz * ercz;
      double phi = acos(cosphi);
      double isinphi = 1.0 / sqrt(1.0 - cosphi * cosphi);
      double rr = phi - bend_t0[u];
      double fr = -bend_k[u] * rr * 2.0;
      ea += -fr * rr * 0.5;
      double irasin = drai * isinphi * fr;
      double ircsin = drci * isinphi * fr;
      double fxa = (erax * cosphi - ercx) * irasin;
      double fya = (eray * cosphi - ercy) * irasin;
      double fza = (eraz * cosphi - ercz) * irasin;
      double fxc = (ercx * cosphi - erax) * ircsin;
      double fyc = (ercy * cosphi - eray) * ircsin;
      double fzc = (ercz * cosphi - eraz) * ircsin;
      atomicAdd(&ff[3 * ia], fxa);
      atomicAdd(&ff[3 * ia + 1], fya);
      atomicAdd(&ff[3 * ia + 2], fza);
      atomicAdd(&ff[3 * ib], -(fxa + fxc));
      atomicAdd(&ff[3 * ib + 1], -(fya + fyc));
      atomicAdd(&ff[3 * ib + 2], -(fza + fzc));
      atomicAdd(&ff[3 * ic], fxc);
      atomicAdd(&ff[3 * ic + 1], fyc);
      atomicAdd(&ff[3 * ic + 2], fzc);
    }
  }
  double v[2] = {eb, ea};
  block_partials<2>(v, partials);
}

// Counts of the half list (instrumentation): entries, pairs within rc that
// the pair loop evaluates (not excluded), and those with an LJ term -- the
// units of the pair loop's algorithmic FLOP count.
__global__ void k_pair_counts(PairParams P, const double4 *__restrict__ pos,
                              const int *__restrict__ type, const double *__restrict__ lj_eps,
                              const double *__restrict__ lj_sig, const int *__restrict__ count,
                              const int *__restrict__ ent, unsigned long long *__restrict__ out) {
  unsigned long long c[4] = {0, 0, 0, 0};
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < P.n - 1; a += gridDim.x * blockDim.x) {
    double4 pa = pos[a];
    const int *row = ent + (size_t)a * P.max_nb;
    int cnt = count[a];
    c[0] += cnt;
    for (int bb = 0; bb < cnt; bb++) {
      int e = row[bb];
      int b = e >> 3, xflag = e & 7;
      double4 pb = pos[b];
      double dx = pa.x - pb.x, dy = pa.y - pb.y, dz = pa.z - pb.z;
      dx -= P.L.x * rint(dx / P.L.x);
      dy -= P.L.y * rint(dy / P.L.y);
      dz -= P.L.z * rint(dz / P.L.z);
      if (dx * dx + dy * dy + dz * dz > P.rc2) continue;
      if (xflag != 0 && xflag != 4) {
        c[3]++;
        continue;
      }
      c[1]++;
      int k = type[a] * P.nt + type[b];
      if (lj_eps[k] * lj_sig[k] != 0.0) c[2]++;
    }
  }
  for (int t = 0; t < 4; t++) atomicAdd(&out[t], c[t]);
}

int pair_counts64(Box *b, long long *out4) {
  PairParams P;
  P.L = make_double3(b->p.L[0], b->p.L[1], b->p.L[2]);
  P.rc2 = b->p.rc * b->p.rc;
  P.n = b->n;
  P.nt = b->nt;
  P.max_nb = b->max_nb;
  unsigned long long *d = nullptr;
  FE_CUDA(cudaMalloc(&d, 4 * sizeof(unsigned long long)));
  cudaMemsetAsync(d, 0, 4 * sizeof(unsigned long long), b->stream);
  int blocks = (b->n + 255) / 256;
  k_pair_counts<<<blocks, 256, 0, b->stream>>>(P, b->pos_q, b->type, b->lj_eps, b->lj_sig,
                                               b->nl_count, b->nl_ent, d);
  cudaError_t e = cudaGetLastError();
  unsigned long long h[4] = {0, 0, 0, 0};
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_fail(e, "k_pair_counts");
  for (int t = 0; t < 4; t++) out4[t] = (long long)h[t];
  return FE_OK;
}

static double host_ref_erfc(double x) {
  // same function as ref_erfc (ewald.c:817-836), evaluated on the host once
  double z = fabs(x);
  double t = 1.0 / (1.0 + 0.5 * z);
  double v = t * exp(-z * z + -1.26551223 +
                     t * (1.00002368 + t * (0.37409196 + t * (0.09678418 +
                     t * (-0.18628806 + t * (0.27886807 + t * (-1.13520398 +
                     t * (1.48851587 + t * (-0.82215223 + t * 0.17087277)))))))));
  return x < 0 ? 2.0 - v : v;
}

int launch_pair64(Box *b) {
  PairParams P;
  P.L = make_double3(b->p.L[0], b->p.L[1], b->p.L[2]);
  P.H = make_double3(b->p.L[0] / 2.0, b->p.L[1] / 2.0, b->p.L[2] / 2.0);
  P.rc = b->p.rc;
  P.rc2 = b->p.rc * b->p.rc;
  P.kappa = b->p.kappa;
  P.kpi = 1.0 * b->p.kappa / sqrt(kPI);
  P.epsRF = b->p.epsRF;
  P.erfc_rc = host_ref_erfc(b->p.kappa * b->p.rc);
  P.ron2 = b->p.r_switch > 0.0 ? b->p.r_switch * b->p.r_switch : 0.0;
  P.sw_den = P.ron2 > 0.0 ? (P.rc2 - P.ron2) * (P.rc2 - P.ron2) * (P.rc2 - P.ron2) : 0.0;
  P.lj_form = b->lj_form;
  P.n = b->n;
  P.nt = b->nt;
  P.max_nb = b->max_nb;
  int rows = b->n - 1;
  int blocks = (rows + 3) / 4;
  if (blocks > 2048) blocks = 2048;
  if (blocks < 1) blocks = 1;
  k_pair64<<<blocks, 128, 0, b->stream>>>(P, b->pos_q, b->type, b->lj_eps, b->lj_sig, b->nl_count,
                                          b->nl_ent, b->ff, b->partials);
  FE_LAUNCH_CHECK("k_pair64");
  return launch_reduce(b, b->partials, blocks, 5, SC_LJ, 1.0);
}

int launch_bonded64(Box *b) {
  int tot = b->nbond + b->nbend;
  int blocks = (tot + 255) / 256;
  if (blocks > 1024) blocks = 1024;
  if (blocks < 1) blocks = 1;
  double3 L = make_double3(b->p.L[0], b->p.L[1], b->p.L[2]);
  k_bonded64<<<blocks, 256, 0, b->stream>>>(b->nbond, b->nbend, L, b->pos_q, b->bond_ab,
                                            b->bond_req, b->bond_k, b->bend_abc, b->bend_t0,
                                            b->bend_k, b->ff, b->partials);
  FE_LAUNCH_CHECK("k_bonded64");
  return launch_reduce(b, b->partials, blocks, 2, SC_BOND, 1.0);
}

}  // namespace fe
