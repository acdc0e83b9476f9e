// k_mc.cu -- exact Ewald energy change of a Monte Carlo trial move.
//
// The reference evaluates a move by recomputing the whole classic-Ewald
// energy before and after it (forces_mc.c:90-573 calling ewald_kspace_mc,
// ewald_mc.c:42-324, O(N * n_k), and ewald_rspace_mc / enbnd_mc over the
// list).  Here the structure factor S(k) = sum_i q_i exp(i k.r_i) of the
// k-vectors of ewald_setup (ewald.c:95-118) stays resident and a move of
// sites [lb, ub) costs O(m * n_k) for the reciprocal part,
//   dE_k = fconv * sum_k c_k (|S_k + dS_k|^2 - |S_k|^2),
//   dS_k = sum_{i moved} q_i (exp(i k.r_i') - exp(i k.r_i)),
// with c_k = kvec_k (kx = 0) or 2 kvec_k (kx > 0), plus O(m * N) for the
// real-space Ewald term (erfc as the reference's, ewald.c:817) and the
// shifted LJ term over every pair touching the moved sites, minimum image.
// Accepting a move adds dS to S; rejecting needs nothing.
#include <cmath>
#include <vector>

#include "fe_device.cuh"

namespace fe {

constexpr int kMcMaxMoved = 64;  // sites per trial move

__global__ void k_mc_structure(int n, int nk, double3 tp, const double4 *__restrict__ pos,
                               const int *__restrict__ kidx, double2 *__restrict__ S) {
  // one block per k-vector; fixed-order block sum (deterministic)
  int k = blockIdx.x;
  if (k >= nk) return;
  double kx = tp.x * kidx[3 * k], ky = tp.y * kidx[3 * k + 1], kz = tp.z * kidx[3 * k + 2];
  double sr = 0.0, si = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double4 p = pos[i];
    double s, c;
    sincos(kx * p.x + ky * p.y + kz * p.z, &s, &c);
    sr += p.w * c;
    si += p.w * s;
  }
  __shared__ double shr[256], shi[256];
  shr[threadIdx.x] = sr;
  shi[threadIdx.x] = si;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      shr[threadIdx.x] += shr[threadIdx.x + w];
      shi[threadIdx.x] += shi[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) S[k] = make_double2(shr[0], shi[0]);
}

// reciprocal part: one thread per k-vector
__global__ void k_mc_recip(int nk, int lb, int m, double3 tp, const double4 *__restrict__ pos,
                           const double *__restrict__ newpos, const int *__restrict__ kidx,
                           const double *__restrict__ ck, const double2 *__restrict__ S,
                           double2 *__restrict__ dS, double *__restrict__ partials) {
  double e = 0.0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nk; k += gridDim.x * blockDim.x) {
    double kx = tp.x * kidx[3 * k], ky = tp.y * kidx[3 * k + 1], kz = tp.z * kidx[3 * k + 2];
    double dr = 0.0, di = 0.0;
    for (int j = 0; j < m; j++) {
      double4 p = pos[lb + j];
      double s0, c0, s1, c1;
      sincos(kx * p.x + ky * p.y + kz * p.z, &s0, &c0);
      sincos(kx * newpos[3 * j] + ky * newpos[3 * j + 1] + kz * newpos[3 * j + 2], &s1, &c1);
      dr += p.w * (c1 - c0);
      di += p.w * (s1 - s0);
    }
    double2 s = S[k];
    dS[k] = make_double2(dr, di);
    // |S + dS|^2 - |S|^2 = 2 Re(conj(S) dS) + |dS|^2
    e += ck[k] * (2.0 * (s.x * dr + s.y * di) + dr * dr + di * di);
  }
  double v[1] = {e};
  block_partials<1>(v, partials);
}

struct McPair {
  double3 L, H;
  double rc2, rce2, kappa, fconv, lj_shift_rc2;
  double ron2, sw_den;  // LJ switch (ron2 = 0: the reference's shift)
  double erfc_rce;      // erfc(kappa rc_ew) / rc_ew
  int n, nt, lb, ub;
};

__device__ __forceinline__ int mc_xflag(const int *__restrict__ xs, const int *__restrict__ xp,
                                        const int *__restrict__ xf, int a, int b) {
  int f = 0;
  for (int p = xs[a]; p < xs[a + 1]; p++)
    if (xp[p] == b) f = xf[p];
  return f;
}

// one pair's MC energy terms, as ewald_mc.c:390-606 / enbnd_mc.c with the
// minimum image of cnonbond_nblist.c:167-172, added to t[5]:
//   t[0] LJ within rc (switched when r_switch > 0), t[1] its shift constant
//   eps (sr12s - 2 sr6s) (enonbonds; 0 under the switch), t[2] real-space
//   Ewald qq erfc(kr)/r within rc_ew, t[3] its shift constant
//   qq erfc(k rc_ew)/rc_ew (eewald_reals), t[4] the excluded-pair correction
//   qq12 (1 - erfc(kr))/r (eewald_intra)
__device__ __forceinline__ void mc_pair_terms(const McPair &P, double3 pa, double qa, int ta,
                                              double3 pb, double qb, int tb, int xflag,
                                              const double *__restrict__ lj_eps,
                                              const double *__restrict__ lj_sig, double *t) {
  double dx = pa.x - pb.x, dy = pa.y - pb.y, dz = pa.z - pb.z;
  if (dx > P.H.x) dx -= P.L.x;
  else if (dx < -P.H.x) dx += P.L.x;
  if (dy > P.H.y) dy -= P.L.y;
  else if (dy < -P.H.y) dy += P.L.y;
  if (dz > P.H.z) dz -= P.L.z;
  else if (dz < -P.H.z) dz += P.L.z;
  double dr2 = dx * dx + dy * dy + dz * dz;
  if (dr2 <= P.rc2) {
    double sig = lj_sig[ta * P.nt + tb], eps = lj_eps[ta * P.nt + tb];
    if (xflag && xflag != 4) {
      sig = 0.0;
      eps = 0.0;
    }
    if ((eps * sig) != 0.0) {
      double sr2 = (sig * sig) / dr2;
      double sr6 = sr2 * sr2 * sr2;
      double sr12 = sr6 * sr6;
      if (P.ron2 > 0.0) {  // optional CHARMM switch (no shift), as the pair kernel
        double e = eps * (sr12 - 2.0 * sr6);
        if (dr2 > P.ron2) {
          double c = P.rc2 - dr2;
          e *= c * c * (P.rc2 + 2.0 * dr2 - 3.0 * P.ron2) / P.sw_den;
        }
        t[0] += e;
      } else {
        double sr2s = (sig * sig) / P.rc2;
        double sr6s = sr2s * sr2s * sr2s;
        double sr12s = sr6s * sr6s;
        t[0] += eps * (sr12 - 2.0 * sr6);
        t[1] += eps * (sr12s - 2.0 * sr6s);
      }
    }
  }
  if (dr2 > P.rce2) return;
  double qqab = qa * qb * P.fconv;
  double qq = qqab;
  if (xflag) qq = (xflag == 4) ? kE14FAC * qqab : 0.0;
  double dr = sqrt(dr2);
  double dri = 1.0 / dr;
  double erfckr = ref_erfc(P.kappa * dr);
  if (qq != 0.0) {
    t[2] += qq * erfckr * dri;
    t[3] += qq * P.erfc_rce;
  }
  if (xflag) {
    double qq12 = qqab;
    if (xflag == 4) qq12 *= (1.0 - kE14FAC);
    t[4] += qq12 * (1.0 - erfckr) * dri;
  }
}

// grid-stride over (moved site j, partner b): the pair terms of
// mc_pair_terms, new minus old (DELTA) or of the current configuration
// (the energy of the pairs touching sites [lb, ub))
template <bool DELTA>
__global__ void k_mc_pairs(McPair P, const double4 *__restrict__ pos, const int *__restrict__ type,
                           const double *__restrict__ newpos, const double *__restrict__ lj_eps,
                           const double *__restrict__ lj_sig, const int *__restrict__ xs,
                           const int *__restrict__ xp, const int *__restrict__ xf,
                           double *__restrict__ partials) {
  int m = P.ub - P.lb;
  double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  long total = (long)m * P.n;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long)gridDim.x * blockDim.x) {
    int j = (int)(t / P.n);
    int b = (int)(t % P.n);
    int a = P.lb + j;
    if (b == a) continue;
    bool bmoved = (b >= P.lb && b < P.ub);
    if (bmoved && b < a) continue;  // a moved pair counted once
    double4 A = pos[a], B = pos[b];
    int xflag = mc_xflag(xs, xp, xf, a, b);
    double3 ao = make_double3(A.x, A.y, A.z);
    double3 bo = make_double3(B.x, B.y, B.z);
    double to[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    mc_pair_terms(P, ao, A.w, type[a], bo, B.w, type[b], xflag, lj_eps, lj_sig, to);
    if (DELTA) {
      double3 an = make_double3(newpos[3 * j], newpos[3 * j + 1], newpos[3 * j + 2]);
      double3 bn = bmoved ? make_double3(newpos[3 * (b - P.lb)], newpos[3 * (b - P.lb) + 1],
                                         newpos[3 * (b - P.lb) + 2])
                          : bo;
      double tn[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
      mc_pair_terms(P, an, A.w, type[a], bn, B.w, type[b], xflag, lj_eps, lj_sig, tn);
#pragma unroll
      for (int q = 0; q < 5; q++) acc[q] += tn[q] - to[q];
    } else {
#pragma unroll
      for (int q = 0; q < 5; q++) acc[q] += to[q];
    }
  }
  block_partials<5>(acc, partials);
}

__global__ void k_mc_commit(int nk, int lb, int m, const double *__restrict__ newpos,
                            const double2 *__restrict__ dS, double2 *__restrict__ S,
                            double4 *__restrict__ pos) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nk) {
    double2 s = S[t], d = dS[t];
    S[t] = make_double2(s.x + d.x, s.y + d.y);
  }
  if (t < m) {
    double4 p = pos[lb + t];
    p.x = newpos[3 * t];
    p.y = newpos[3 * t + 1];
    p.z = newpos[3 * t + 2];
    pos[lb + t] = p;
  }
}

__global__ void k_mc_kenergy(int nk, const double *__restrict__ ck, const double2 *__restrict__ S,
                             double *__restrict__ partials) {
  double e = 0.0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nk; k += gridDim.x * blockDim.x) {
    double2 s = S[k];
    e += ck[k] * (s.x * s.x + s.y * s.y);
  }
  double v[1] = {e};
  block_partials<1>(v, partials);
}

int mc_setup(Box *b, int kmax, int mks, double rc_ew) {
  mc_free(b);
  double kappa = b->p.kappa;
  double two_pi = 2.0 * kPI;
  double lx = b->p.L[0], ly = b->p.L[1], lz = b->p.L[2];
  double boxv = lx * ly * lz;
  double bb = 0.25 / (kappa * kappa);
  double fconv = (kELEC * kELEQ * kELEQ * kNA * 0.001);
  std::vector<double> ck;
  std::vector<int> kid;
  for (int kx = 0; kx <= kmax; ++kx) {  // ewald.c:104-118 order
    double rkx = two_pi * (double)kx / lx;
    for (int ky = -kmax; ky <= kmax; ++ky) {
      double rky = two_pi * (double)ky / ly;
      for (int kz = -kmax; kz <= kmax; ++kz) {
        double rkz = two_pi * (double)kz / lz;
        int ksq = kx * kx + ky * ky + kz * kz;
        if (ksq <= mks && ksq != 0) {
          double rksq = rkx * rkx + rky * rky + rkz * rkz;
          double kvec = two_pi * exp(-bb * rksq) / rksq / boxv;
          ck.push_back((kx == 0 ? 1.0 : 2.0) * kvec * fconv);
          kid.push_back(kx);
          kid.push_back(ky);
          kid.push_back(kz);
        }
      }
    }
  }
  b->mc_nk = (int)ck.size();
  b->mc_kmax = kmax;
  b->mc_mks = mks;
  b->mc_rc_ew = rc_ew;
  b->mc_nmax = kMcMaxMoved;
  FE_CUDA(cudaMalloc(&b->mc_kvec, sizeof(double) * b->mc_nk));
  FE_CUDA(cudaMalloc(&b->mc_kidx, sizeof(int) * 3 * b->mc_nk));
  FE_CUDA(cudaMalloc(&b->mc_S, sizeof(double2) * b->mc_nk));
  FE_CUDA(cudaMalloc(&b->mc_dS, sizeof(double2) * b->mc_nk));
  FE_CUDA(cudaMalloc(&b->mc_newpos, sizeof(double) * 3 * kMcMaxMoved));
  FE_CUDA(cudaMalloc(&b->mc_part, sizeof(double) * kMaxPartialBlocks * kPartialTerms));
  FE_CUDA(cudaMemcpyAsync(b->mc_kvec, ck.data(), sizeof(double) * b->mc_nk, cudaMemcpyHostToDevice,
                          b->stream));
  FE_CUDA(cudaMemcpyAsync(b->mc_kidx, kid.data(), sizeof(int) * kid.size(), cudaMemcpyHostToDevice,
                          b->stream));
  double3 tp = make_double3(two_pi * (1.0 / lx), two_pi * (1.0 / ly), two_pi * (1.0 / lz));
  k_mc_structure<<<b->mc_nk, 256, 0, b->stream>>>(b->n, b->mc_nk, tp, b->pos_q, b->mc_kidx, b->mc_S);
  FE_LAUNCH_CHECK("k_mc_structure");
  FE_CUDA(cudaStreamSynchronize(b->stream));
  b->mc_pending = 0;
  return FE_OK;
}

static double host_erfc_nr(double x) {
  // the reference's erfc fit (ewald.c:817-836), evaluated once on the host
  double z = fabs(x);
  double t = 1.0 / (1.0 + 0.5 * z);
  double v = t * exp(-z * z + -1.26551223 +
                     t * (1.00002368 + t * (0.37409196 + t * (0.09678418 +
                     t * (-0.18628806 + t * (0.27886807 + t * (-1.13520398 +
                     t * (1.48851587 + t * (-0.82215223 + t * 0.17087277)))))))));
  return x < 0 ? 2.0 - v : v;
}

// Energy terms of the pairs touching sites [lb, ub): with new_pos_host, the
// change when those sites move there (and the reciprocal change, dS kept for
// fe_mc_accept); without, the current energies (and the whole reciprocal
// energy).  terms[6] = {reciprocal, LJ, LJ shift constant, real space, its
// shift constant, intramolecular correction} (see mc_pair_terms).
int mc_terms(Box *b, int lb, int ub, const double *new_pos_host, double *terms) {
  if (!b->mc_S) {
    set_error("fe_mc_delta / fe_mc_site_energy before fe_mc_setup");
    return FE_ERR_STATE;
  }
  int m = ub - lb;
  if (lb < 0 || ub > b->n || m < 1) {
    set_error("fe_mc: site range outside the box");
    return FE_ERR_ARG;
  }
  const bool delta = new_pos_host != nullptr;
  if (delta && m > kMcMaxMoved) {
    set_error("fe_mc_delta: at most 64 sites per move");
    return FE_ERR_SIZE;
  }
  double h[6];
  if (delta) {
    FE_CUDA(cudaMemcpyAsync(b->mc_newpos, new_pos_host, sizeof(double) * 3 * m,
                            cudaMemcpyHostToDevice, b->stream));
    double two_pi = 2.0 * kPI;
    double3 tp = make_double3(two_pi * (1.0 / b->p.L[0]), two_pi * (1.0 / b->p.L[1]),
                              two_pi * (1.0 / b->p.L[2]));
    int kb = (b->mc_nk + 127) / 128;
    k_mc_recip<<<kb, 128, 0, b->stream>>>(b->mc_nk, lb, m, tp, b->pos_q, b->mc_newpos,
                                          b->mc_kidx, b->mc_kvec, b->mc_S, b->mc_dS, b->mc_part);
    FE_LAUNCH_CHECK("k_mc_recip");
    int rc = launch_reduce(b, b->mc_part, kb, 1, SC_ENERGY3, 1.0);  // scratch slot
    if (rc) return rc;
    FE_CUDA(cudaMemcpyAsync(h, b->scal + SC_ENERGY3, sizeof(double), cudaMemcpyDeviceToHost,
                            b->stream));
  } else {
    int rc = mc_kspace_energy(b, h);
    if (rc) return rc;
  }
  McPair P;
  P.L = make_double3(b->p.L[0], b->p.L[1], b->p.L[2]);
  P.H = make_double3(b->p.L[0] / 2.0, b->p.L[1] / 2.0, b->p.L[2] / 2.0);
  P.rc2 = b->p.rc * b->p.rc;
  P.ron2 = b->p.r_switch > 0.0 ? b->p.r_switch * b->p.r_switch : 0.0;
  P.sw_den = (P.rc2 - P.ron2) * (P.rc2 - P.ron2) * (P.rc2 - P.ron2);
  P.rce2 = b->mc_rc_ew * b->mc_rc_ew;
  P.kappa = b->p.kappa;
  P.erfc_rce = host_erfc_nr(b->p.kappa * b->mc_rc_ew) / b->mc_rc_ew;
  P.fconv = (kELEC * kELEQ * kELEQ * kNA * 0.001);
  P.n = b->n;
  P.nt = b->nt;
  P.lb = lb;
  P.ub = ub;
  long total = (long)m * b->n;
  int pb = (int)((total + 255) / 256);
  if (pb > 2048) pb = 2048;  // partial slots: kMaxPartialBlocks / 2
  double *part = b->mc_part + kMaxPartialBlocks * kPartialTerms / 2;
  if (delta)
    k_mc_pairs<true><<<pb, 256, 0, b->stream>>>(P, b->pos_q, b->type, b->mc_newpos, b->lj_eps,
                                                b->lj_sig, b->x_start, b->x_partner, b->x_flag,
                                                part);
  else
    k_mc_pairs<false><<<pb, 256, 0, b->stream>>>(P, b->pos_q, b->type, b->mc_newpos, b->lj_eps,
                                                 b->lj_sig, b->x_start, b->x_partner, b->x_flag,
                                                 part);
  FE_LAUNCH_CHECK("k_mc_pairs");
  int rc = launch_reduce(b, part, pb, 5, SC_ENERGY8, 1.0);  // scratch slots
  if (rc) return rc;
  FE_CUDA(cudaMemcpyAsync(h + 1, b->scal + SC_ENERGY8, sizeof(double) * 5, cudaMemcpyDeviceToHost,
                          b->stream));
  FE_CUDA(cudaStreamSynchronize(b->stream));
  for (int q = 0; q < 6; q++) terms[q] = h[q];
  if (delta) {
    b->mc_lb = lb;
    b->mc_ub = ub;
    b->mc_pending = 1;
  }
  return FE_OK;
}

int mc_delta(Box *b, int lb, int ub, const double *new_pos_host, double *dE, double *parts) {
  double t[6];
  int rc = mc_terms(b, lb, ub, new_pos_host, t);
  if (rc) return rc;
  double dk = t[0], dlj = t[1] - t[2], dreal = t[3] - t[5];
  if (dE) *dE = dk + dreal + dlj;
  if (parts) {
    parts[0] = dk;
    parts[1] = dreal;
    parts[2] = dlj;
  }
  return FE_OK;
}

int mc_accept(Box *b) {
  if (!b->mc_pending) {
    set_error("fe_mc_accept without a pending fe_mc_delta");
    return FE_ERR_STATE;
  }
  int m = b->mc_ub - b->mc_lb;
  int t = b->mc_nk > m ? b->mc_nk : m;
  k_mc_commit<<<(t + 255) / 256, 256, 0, b->stream>>>(b->mc_nk, b->mc_lb, m, b->mc_newpos, b->mc_dS,
                                                      b->mc_S, b->pos_q);
  FE_LAUNCH_CHECK("k_mc_commit");
  FE_CUDA(cudaStreamSynchronize(b->stream));
  b->mc_pending = 0;
  return FE_OK;
}

int mc_kspace_energy(Box *b, double *e) {
  if (!b->mc_S) {
    set_error("fe_mc_kspace_energy before fe_mc_setup");
    return FE_ERR_STATE;
  }
  int kb = (b->mc_nk + 127) / 128;
  k_mc_kenergy<<<kb, 128, 0, b->stream>>>(b->mc_nk, b->mc_kvec, b->mc_S, b->mc_part);
  FE_LAUNCH_CHECK("k_mc_kenergy");
  int rc = launch_reduce(b, b->mc_part, kb, 1, SC_ENERGY3, 1.0);
  if (rc) return rc;
  FE_CUDA(cudaMemcpyAsync(e, b->scal + SC_ENERGY3, sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  FE_CUDA(cudaStreamSynchronize(b->stream));
  return FE_OK;
}

void mc_free(Box *b) {
  void *ptrs[] = {b->mc_kvec, b->mc_kidx, b->mc_S, b->mc_dS, b->mc_newpos, b->mc_part};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  b->mc_kvec = nullptr;
  b->mc_kidx = nullptr;
  b->mc_S = nullptr;
  b->mc_dS = nullptr;
  b->mc_newpos = nullptr;
  b->mc_part = nullptr;
  b->mc_nk = 0;
}

}  // namespace fe
