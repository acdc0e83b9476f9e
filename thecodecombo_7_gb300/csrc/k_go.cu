// k_go.cu -- batched replica exchange of C-alpha Go-model chains: one
// persistent launch runs a whole exchange segment (thousands of Langevin
// steps) of every replica, one to four CTAs per replica and one to sixteen
// threads per bead.
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
//     over 1-16 adjacent threads per bead and summed by warp shuffles; no
//     atomics, fixed order;
//   - load balance over the SMs: the launch runs clusters of four CTAs, and a
//     long chain is split over 2 to 4 CTAs of one cluster (each owns a
//     contiguous slice of beads and computes their forces from all beads of
//     the chain).  Every CTA holds the whole chain's FP32 positions in two
//     shared-memory buffers; after each update a CTA stores its slice into
//     the next buffer of every CTA of its chain (distributed shared memory)
//     and one cluster barrier per step orders the stores before the reads.
//     Shorter chains take one CTA each; the split of each chain is planned
//     on the host to level the partners each thread walks per step over the
//     CTAs the GPU holds at once;
//   - the FP64 state update by one thread per bead, apart from the force
//     layout, so that each warp's FP64 instructions carry 32 beads; the
//     pair energies are summed only in the last force evaluation of a
//     segment (the exchange needs no other);
//   - positions and velocities in FP64 registers of the owning thread for
//     the whole segment; BAOAB Langevin (Leimkuhler & Matthews 2013) with the
//     O step v = c1 v + c2 sqrt(kT/m) xi in FP64 (the noise term itself
//     formed in FP32), xi Gaussian by Box-Muller from Philox4x32-10 draws
//     keyed by (bead, step); the closing B of one step and the opening B of
//     the next are one kick of 2 (dt/2) f / m;
//   - a second energy function, the reference's own Go model (cgolik.c,
//     fe_go_set_reference_form): bonds eps dr^2 + 100 eps dr^4, bends
//     10 eps (theta - theta0)^2, three-fold torsions, natives 12-6 cut and
//     shifted at rc, non-natives WCA within d_rep; each bead computes the
//     bends and torsions that move it (the kernel is a template on the form);
//   - after the segment, one exchange kernel: adjacent temperature slots as
//     swap_box does (pairs alternate between attempts), acceptance
//     exp((1/kT_s - 1/kT_s+1)(U_s - U_s+1)) > u, velocity rescale by
//     sqrt(T_s/T_s+1); it also advances the device step counter, so the
//     pair (segment, exchange) is captured once as a CUDA graph and replayed.
#include <algorithm>
#include <cmath>
#include <vector>

#include "fe_internal.h"
#include "fe_rng.cuh"

namespace fe {

constexpr int kGoMaxBeads = 1024;
constexpr int kGoBlock = 1024;   // threads per CTA
constexpr int kGoCluster = 4;    // CTAs per cluster; a chain takes 1 to 4 of them
constexpr int kGoMaxTpb = 16;    // threads per bead at most
constexpr uint32_t kRngTagGo = 0x474F4C31u;  // "GOL1"

// What one CTA of the launch does: beads [lo, lo + nb) of replica `rep`
// with `tpb` threads per bead; its chain is shared by the cluster ranks
// [peer0, peer0 + npeer).  rep < 0: a padding CTA that only joins the
// cluster barriers.
struct GoCta {
  int rep, lo, nb, tpb, peer0, npeer;
};

struct GoK {
  float eps, sig2, rc2, e_shift, kb, r0b;
  // the non-native pair within rc2: E = c12/r^12 - c6/r^6 + e0, force
  // (f12/r^12 - f6/r^6)/r^2 along the separation
  float c12, f12, c6, f6, e0;
  // form 1, the reference's own model (cgolik.c): natives 12-6 with
  // sigma^2 = 2^(-1/3) r0^2 cut and shifted at rc2n; bonds with a quartic
  // term kq (r - r0)^4 and per-bond r0; bends kth (theta - theta0)^2;
  // torsions kph (1 + cos 3 tau)
  int form;
  float rc2n, kq, kth, kph;
  double acc_fac;   // 100 / m: kJ/mol/A per amu -> A/ps^2
  double dt, c1, c2;
  double vscale;    // sqrt(100 / m): sqrt(kT [kJ/mol]) -> A/ps
  int min_sep;
  int nrep;
  int maxN;         // longest chain: the stride of the two position buffers
  uint64_t seed;
};

struct GoD {
  const GoCta *cta;      // one per CTA of the launch
  const int *start;      // nrep + 1: first bead of each replica
  const int *maskoff;    // nrep: first mask word of each replica
  const unsigned *mask;  // native bitmask rows (N words of ceil(N/32) per replica)
  const int *nat_start;  // total + 1 (CSR over global bead index)
  const int *nat_j;      // global partner index
  const float *nat_r02;  // native distance squared
  const float *bond_r0;  // form 1: length of bond (i, i+1) per global bead i
  const float *bend_t0;  // form 1: angle centred at global bead i
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

// The bend (c - 1, c, c + 1) of the reference's Go model (cba_golik,
// cgolik.c:204-296: E = kth (theta - theta0)^2): the force on its site
// `which` (0, 1, 2) added to f, the energy returned.
__device__ __forceinline__ float go_bend(const float4 *__restrict__ p, int c, float t0, float kth,
                                         int which, float &fx, float &fy, float &fz) {
  const float4 A = p[c - 1], B = p[c], C = p[c + 1];
  const float dax = A.x - B.x, day = A.y - B.y, daz = A.z - B.z;
  const float dcx = C.x - B.x, dcy = C.y - B.y, dcz = C.z - B.z;
  const float drai = rsqrtf(dax * dax + day * day + daz * daz);
  const float erax = dax * drai, eray = day * drai, eraz = daz * drai;
  const float drci = rsqrtf(dcx * dcx + dcy * dcy + dcz * dcz);
  const float ercx = dcx * drci, ercy = dcy * drci, ercz = dcz * drci;
  float cosphi = erax * ercx + eray * ercy + eraz * ercz;
  cosphi = fminf(fmaxf(cosphi, -1.f), 1.f);
  // sin from the cross product of the unit vectors: accurate in FP32 also
  // where the three sites are nearly collinear (1 - cos^2 is not)
  const float qx = eray * ercz - eraz * ercy, qy = eraz * ercx - erax * ercz,
              qz = erax * ercy - eray * ercx;
  const float sin2 = fmaxf(qx * qx + qy * qy + qz * qz, 1e-20f);
  const float rr = atan2f(sqrtf(sin2), cosphi) - t0;
  const float isinphi = rsqrtf(sin2);
  const float fr = -2.f * kth * rr;
  const float irasin = drai * isinphi * fr, ircsin = drci * isinphi * fr;
  const float fxa = (erax * cosphi - ercx) * irasin, fya = (eray * cosphi - ercy) * irasin,
              fza = (eraz * cosphi - ercz) * irasin;
  const float fxc = (ercx * cosphi - erax) * ircsin, fyc = (ercy * cosphi - eray) * ircsin,
              fzc = (ercz * cosphi - eraz) * ircsin;
  if (which == 0) {
    fx += fxa; fy += fya; fz += fza;
  } else if (which == 2) {
    fx += fxc; fy += fyc; fz += fzc;
  } else {
    fx -= fxa + fxc; fy -= fya + fyc; fz -= fza + fzc;
  }
  return kth * rr * rr;
}

// The torsion (a, a + 1, a + 2, a + 3) of the reference's Go model
// (cda_golik, cgolik.c:399-610, three-fold, phase zero: E = kph (1 +
// cos 3 tau)): the force on its site `which` (0..3) added, the energy
// returned.
__device__ __forceinline__ float go_tors(const float4 *__restrict__ p, int a, float kph,
                                         int which, float &fx, float &fy, float &fz) {
  const float4 A = p[a], B = p[a + 1], C = p[a + 2], Dd = p[a + 3];
  const float dabx = B.x - A.x, daby = B.y - A.y, dabz = B.z - A.z;
  const float dbcx = C.x - B.x, dbcy = C.y - B.y, dbcz = C.z - B.z;
  const float dcdx = Dd.x - C.x, dcdy = Dd.y - C.y, dcdz = Dd.z - C.z;
  const float rab = sqrtf(dabx * dabx + daby * daby + dabz * dabz), irab = 1.f / rab;
  const float erabx = dabx * irab, eraby = daby * irab, erabz = dabz * irab;
  const float rbc = sqrtf(dbcx * dbcx + dbcy * dbcy + dbcz * dbcz), irbc = 1.f / rbc;
  const float erbcx = dbcx * irbc, erbcy = dbcy * irbc, erbcz = dbcz * irbc;
  const float rcd = sqrtf(dcdx * dcdx + dcdy * dcdy + dcdz * dcdz), ircd = 1.f / rcd;
  const float ercdx = dcdx * ircd, ercdy = dcdy * ircd, ercdz = dcdz * ircd;
  const float abbcx = eraby * erbcz - erabz * erbcy, abbcy = erabz * erbcx - erabx * erbcz,
              abbcz = erabx * erbcy - eraby * erbcx;
  const float cosb = -(erabx * erbcx + eraby * erbcy + erabz * erbcz);
  // 1 / sin^2 of the two bends from the cross products (1 - cos^2 loses its
  // digits in FP32 where a bend is nearly straight)
  const float isinb2 = 1.f / fmaxf(abbcx * abbcx + abbcy * abbcy + abbcz * abbcz, 1e-20f),
              isinb = sqrtf(isinb2);
  const float dccbx = ercdy * erbcz - ercdz * erbcy, dccby = ercdz * erbcx - ercdx * erbcz,
              dccbz = ercdx * erbcy - ercdy * erbcx;
  const float cosc = -(ercdx * erbcx + ercdy * erbcy + ercdz * erbcz);
  const float isinc2 = 1.f / fmaxf(dccbx * dccbx + dccby * dccby + dccbz * dccbz, 1e-20f),
              isinc = sqrtf(isinc2);
  const float abcdx = -(abbcy * dccbz - abbcz * dccby), abcdy = -(abbcz * dccbx - abbcx * dccbz),
              abcdz = -(abbcx * dccby - abbcy * dccbx);
  // tau as the reference defines it (sign of num, angle between the two
  // plane normals) but from atan2 of the normals' cross and dot products,
  // accurate near 0 and pi where acos is not
  const float num = abcdx * erbcx + abcdy * erbcy + abcdz * erbcz;
  const float ctau = -(abbcx * dccbx + abbcy * dccby + abbcz * dccbz);
  const float tau = atan2f(num, ctau);
  float s3, c3;
  sincosf(3.f * tau, &s3, &c3);
  const float fr = 3.f * kph * s3;
  if (which == 0) {
    const float fa = -fr * irab * isinb2;
    fx += fa * abbcx; fy += fa * abbcy; fz += fa * abbcz;
  } else if (which == 1) {
    const float fb1 = fr * (rbc - rab * cosb) * irab * irbc * isinb2;
    const float fb2 = fr * cosc * irbc * isinc2;
    fx += fb1 * abbcx + fb2 * dccbx; fy += fb1 * abbcy + fb2 * dccby; fz += fb1 * abbcz + fb2 * dccbz;
  } else if (which == 2) {
    const float fc1 = fr * (rbc - rcd * cosc) * ircd * irbc * isinc2;
    const float fc2 = fr * cosb * irbc * isinb2;
    fx += fc1 * dccbx + fc2 * abbcx; fy += fc1 * dccby + fc2 * abbcy; fz += fc1 * dccbz + fc2 * abbcz;
  } else {
    const float fd = -fr * ircd * isinc2;
    fx += fd * dccbx; fy += fd * dccby; fz += fd * dccbz;
  }
  return kph * (1.f + c3);
}

// Force on bead i of a chain of N (positions in shared memory) from the
// partners j = sub, sub + T, sub + 2T, ... (T threads per bead, sub its
// index); natives likewise over the bead's CSR row, bonds by sub 0 only.
// The partners of one 32-bead word are taken in groups of up to four whose
// positions are loaded together.  Returns this thread's share of the
// potential energy (pairs and bonds split in half).
template <int T, bool WITH_E, int FORM>
__device__ __forceinline__ float go_force_t(const GoK &K, const GoD &D, const float4 *__restrict__ p,
                                            const unsigned *__restrict__ mrow, int N, int i,
                                            int sub, int gbase, float &fx, float &fy, float &fz) {
  constexpr int PER = 32 / T;           // this thread's partners per word
  constexpr int G = PER < 4 ? PER : 4;  // loads in flight
  const float4 pi = p[i];
  float e = 0.f;
  fx = fy = fz = 0.f;
  // the row's bits mark the pairs the repulsion skips: natives (below) and
  // |i - j| < min_sep, the bead itself included
  const int nw = (N + 31) >> 5;
  for (int w = 0; w < nw; w++) {
    const unsigned skip = mrow[w];
    const int base = w << 5;
#pragma unroll
    for (int k0 = 0; k0 < PER; k0 += G) {
      float4 pj[G];
#pragma unroll
      for (int k = 0; k < G; k++) pj[k] = p[min(base + sub + (k0 + k) * T, N - 1)];
#pragma unroll
      for (int k = 0; k < G; k++) {
        const int b = sub + (k0 + k) * T;
        const float dx = pi.x - pj[k].x, dy = pi.y - pj[k].y, dz = pi.z - pj[k].z;
        const float r2 = dx * dx + dy * dy + dz * dz;
        if (base + b < N && !((skip >> b) & 1u) && r2 < K.rc2) {
          const float ri2 = __fdividef(1.f, r2);
          const float ri6 = ri2 * ri2 * ri2;
          const float ri12 = ri6 * ri6;
          if (WITH_E)
            e += 0.5f * (FORM == 0 ? fmaf(K.c12, ri12, K.e0) : fmaf(K.c12, ri12, -K.c6 * ri6) + K.e0);
          const float fs = (FORM == 0 ? K.f12 * ri12 : fmaf(K.f12, ri12, -K.f6 * ri6)) * ri2;
          fx = fmaf(fs, dx, fx);
          fy = fmaf(fs, dy, fy);
          fz = fmaf(fs, dz, fz);
        }
      }
    }
  }
  const int g = gbase + i;
  for (int q = D.nat_start[g] + sub; q < D.nat_start[g + 1]; q += T) {
    int j = D.nat_j[q] - gbase;
    float4 pj = p[j];
    float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
    float r2 = dx * dx + dy * dy + dz * dz;
    float ri2 = __fdividef(1.f, r2);
    float fs;
    if (FORM == 0) {
      float s2 = D.nat_r02[q] * ri2;
      float s10 = s2 * s2 * s2 * s2 * s2;
      float s12 = s10 * s2;
      if (WITH_E) e += 0.5f * K.eps * (5.f * s12 - 6.f * s10);
      fs = 60.f * K.eps * (s12 - s10) * ri2;
    } else {
      if (r2 > K.rc2n) continue;
      const float sg2 = 0.79370052598409973738f * D.nat_r02[q];  // (2^(-1/6) r0)^2
      float s2 = sg2 * ri2, s6 = s2 * s2 * s2, s12 = s6 * s6;
      if (WITH_E) {
        float c2 = sg2 / K.rc2n, c6 = c2 * c2 * c2;
        e += 0.5f * 4.f * K.eps * ((s12 - s6) - (c6 * c6 - c6));
      }
      fs = 48.f * K.eps * ri2 * (s12 - 0.5f * s6);
    }
    fx = fmaf(fs, dx, fx);
    fy = fmaf(fs, dy, fy);
    fz = fmaf(fs, dz, fz);
  }
  if (sub != 0) return e;
  for (int nb = -1; nb <= 1; nb += 2) {
    int j = i + nb;
    if (j < 0 || j >= N) continue;
    float4 pj = p[j];
    float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
    float r = sqrtf(dx * dx + dy * dy + dz * dz);
    float dr = r - (FORM == 0 ? K.r0b : D.bond_r0[g + min(nb, 0)]);
    float fs;
    if (FORM == 0) {
      if (WITH_E) e += 0.5f * K.kb * dr * dr;
      fs = -2.f * K.kb * dr / r;
    } else {
      if (WITH_E) e += 0.5f * dr * dr * fmaf(K.kq, dr * dr, K.kb);
      fs = -dr * fmaf(4.f * K.kq, dr * dr, 2.f * K.kb) / r;
    }
    fx = fmaf(fs, dx, fx);
    fy = fmaf(fs, dy, fy);
    fz = fmaf(fs, dz, fz);
  }
  if (FORM == 1) {
    // the bends and torsions that move this bead: each computed whole, this
    // bead's share of the force kept, its energy split over its beads
#pragma unroll
    for (int c = i - 1; c <= i + 1; c++)
      if (c >= 1 && c + 1 < N) {
        const float eb = go_bend(p, c, D.bend_t0[gbase + c], K.kth, i - (c - 1), fx, fy, fz);
        if (WITH_E) e += eb * (1.f / 3.f);
      }
#pragma unroll
    for (int a = i - 3; a <= i; a++)
      if (a >= 0 && a + 3 < N) {
        const float et = go_tors(p, a, K.kph, i - a, fx, fy, fz);
        if (WITH_E) e += 0.25f * et;
      }
  }
  return e;
}

template <bool WITH_E, int FORM>
__device__ __forceinline__ float go_force(const GoK &K, const GoD &D, const float4 *__restrict__ p,
                                          const unsigned *__restrict__ mrow, int N, int i, int sub,
                                          int T, int gbase, float &fx, float &fy, float &fz) {
  switch (T) {
    case 1: return go_force_t<1, WITH_E, FORM>(K, D, p, mrow, N, i, sub, gbase, fx, fy, fz);
    case 2: return go_force_t<2, WITH_E, FORM>(K, D, p, mrow, N, i, sub, gbase, fx, fy, fz);
    case 4: return go_force_t<4, WITH_E, FORM>(K, D, p, mrow, N, i, sub, gbase, fx, fy, fz);
    case 8: return go_force_t<8, WITH_E, FORM>(K, D, p, mrow, N, i, sub, gbase, fx, fy, fz);
    default: return go_force_t<16, WITH_E, FORM>(K, D, p, mrow, N, i, sub, gbase, fx, fy, fz);
  }
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

// Distributed shared memory and the cluster barrier (PTX ISA: mapa,
// st.shared::cluster, barrier.cluster).
__device__ __forceinline__ uint32_t go_cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t go_peer_addr(const void *p, uint32_t rank) {
  uint32_t a = (uint32_t)__cvta_generic_to_shared(p), d;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(rank));
  return d;
}
__device__ __forceinline__ void go_st_peer(uint32_t a, float4 v) {
  asm volatile("st.shared::cluster.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(a), "f"(v.x), "f"(v.y),
               "f"(v.z), "f"(v.w)
               : "memory");
}
__device__ __forceinline__ void go_st_peer(uint32_t a, double v) {
  asm volatile("st.shared::cluster.f64 [%0], %1;" ::"r"(a), "d"(v) : "memory");
}
// every thread of the cluster: stores before it are seen by loads after it
__device__ __forceinline__ void go_cluster_sync() {
  asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}

// bead i's FP32 position into buffer slot i of every CTA of the chain
__device__ __forceinline__ void go_publish(const GoCta &c, float4 *buf, int i, double x0, double x1,
                                           double x2) {
  const float4 p = make_float4((float)x0, (float)x1, (float)x2, 0.f);
  for (int q = 0; q < c.npeer; q++) go_st_peer(go_peer_addr(buf + i, (uint32_t)(c.peer0 + q)), p);
}

// One segment of nsteps BAOAB steps of every replica (mode 0), or a single
// force evaluation into D.f (mode 1).  Launched in clusters of kGoCluster
// CTAs; every thread of every CTA runs the same barriers.  Forces use T
// threads per bead; the FP64 state update uses one thread per bead (thread
// t integrates bead lo + t), so each warp's FP64 instructions carry 32
// beads — the FP64 pipe is narrow on this part.  The forces pass between
// the two layouts through shared memory.
template <int FORM>
__global__ void __launch_bounds__(kGoBlock, 1) k_go_segment(GoK K, GoD D, int nsteps, int mode) {
  extern __shared__ float4 go_pos[];  // two buffers of K.maxN, then the skip rows
  __shared__ double red[33];
  __shared__ double epart[kGoCluster];
  __shared__ float4 fsh[kGoBlock];    // the lane-summed force of each bead of the slice
  const GoCta c = D.cta[blockIdx.x];
  const bool live = c.rep >= 0;
  const int T = live ? c.tpb : 1;
  const int il = threadIdx.x / T, sub = threadIdx.x % T;
  const int gbase = live ? D.start[c.rep] : 0;
  const int N = live ? D.start[c.rep + 1] - gbase : 0;
  const int W = (N + 31) >> 5;
  unsigned *rows = (unsigned *)(go_pos + 2 * K.maxN);
  const bool bead = live && il < c.nb;  // this thread computes forces on bead lo + il
  const int i = c.lo + il;
  const bool integ = live && (int)threadIdx.x < c.nb;  // ... integrates bead lo + tid
  const int ib = c.lo + (int)threadIdx.x;
  if (live) {
    const unsigned *src = D.mask + D.maskoff[c.rep] + (size_t)c.lo * W;
    for (int t = threadIdx.x; t < c.nb * W; t += blockDim.x) rows[t] = src[t];
  }
  __syncthreads();
  const unsigned *mrow = rows + (bead ? il : 0) * W;
  if (bead && sub == 0) {
    unsigned *row = rows + il * W;
    for (int j = max(0, i - K.min_sep + 1); j <= min(N - 1, i + K.min_sep - 1); j++)
      row[j >> 5] |= 1u << (j & 31);
  }
  double x0 = 0, x1 = 0, x2 = 0, v0 = 0, v1 = 0, v2 = 0;
  if (integ) {
    const double *xp = D.x + 3 * (size_t)(gbase + ib), *vp = D.v + 3 * (size_t)(gbase + ib);
    x0 = xp[0];
    x1 = xp[1];
    x2 = xp[2];
    v0 = vp[0];
    v1 = vp[1];
    v2 = vp[2];
  }
  go_cluster_sync();  // every CTA of the cluster runs: its shared memory may be written
  if (integ) go_publish(c, go_pos, ib, x0, x1, x2);
  go_cluster_sync();
  float fx = 0.f, fy = 0.f, fz = 0.f, e = 0.f;
  if (bead) {
    if (mode == 1 || nsteps == 0) e = go_force<true, FORM>(K, D, go_pos, mrow, N, i, sub, T, gbase, fx, fy, fz);
    else go_force<false, FORM>(K, D, go_pos, mrow, N, i, sub, T, gbase, fx, fy, fz);
  }
  fx = go_lane_sum(fx, T);
  fy = go_lane_sum(fy, T);
  fz = go_lane_sum(fz, T);
  if (bead && sub == 0) fsh[il] = make_float4(fx, fy, fz, 0.f);
  __syncthreads();
  if (mode == 1) {
    if (integ) {
      const float4 f = fsh[threadIdx.x];
      float *fp = D.f + 3 * (size_t)(gbase + ib);
      fp[0] = f.x;
      fp[1] = f.y;
      fp[2] = f.z;
    }
    nsteps = 0;
  }
  const unsigned long long step0 = *D.step;
  const double kT = live ? ((kKB * kNA) * D.T[c.rep]) * .001 : 0.0;  // read_sim.c:351, kJ/mol
  const float svf = (float)(K.vscale * sqrt(kT) * K.c2);  // the noise amplitude
  const double hdt = 0.5 * K.dt, ha = 0.5 * K.dt * K.acc_fac;
  for (int s = 0; s < nsteps; s++) {
    float4 *nxt = go_pos + ((s + 1) & 1) * K.maxN;
    if (integ) {
      const float4 f = fsh[threadIdx.x];
      // the closing B of step s - 1 (s > 0) and the B of step s, then A, O, A
      const double k = s > 0 ? 2.0 * ha : ha;
      v0 += k * f.x;
      v1 += k * f.y;
      v2 += k * f.z;
      x0 += hdt * v0;
      x1 += hdt * v1;
      x2 += hdt * v2;
      float z0, z1, z2;
      go_normals(K.seed, (uint32_t)(gbase + ib), step0 + s, z0, z1, z2);
      v0 = K.c1 * v0 + (double)(svf * z0);
      v1 = K.c1 * v1 + (double)(svf * z1);
      v2 = K.c1 * v2 + (double)(svf * z2);
      x0 += hdt * v0;
      x1 += hdt * v1;
      x2 += hdt * v2;
      // every CTA of the chain read this buffer last in step s - 1, before
      // the barrier that ended that step
      go_publish(c, nxt, ib, x0, x1, x2);
    }
    go_cluster_sync();  // also: fsh was read above before it is written below
    if (bead) {  // the energy of the last step only
      if (s == nsteps - 1) e = go_force<true, FORM>(K, D, nxt, mrow, N, i, sub, T, gbase, fx, fy, fz);
      else go_force<false, FORM>(K, D, nxt, mrow, N, i, sub, T, gbase, fx, fy, fz);
    }
    fx = go_lane_sum(fx, T);
    fy = go_lane_sum(fy, T);
    fz = go_lane_sum(fz, T);
    if (bead && sub == 0) fsh[il] = make_float4(fx, fy, fz, 0.f);
    __syncthreads();
  }
  if (integ && nsteps > 0) {
    const float4 f = fsh[threadIdx.x];
    v0 += ha * f.x;  // the closing B of the last step
    v1 += ha * f.y;
    v2 += ha * f.z;
    double *xp = D.x + 3 * (size_t)(gbase + ib), *vp = D.v + 3 * (size_t)(gbase + ib);
    xp[0] = x0;
    xp[1] = x1;
    xp[2] = x2;
    vp[0] = v0;
    vp[1] = v1;
    vp[2] = v2;
  }
  // the chain's potential energy: each CTA's block sum into the slot of its
  // part in the first CTA of the chain, summed there in part order
  const double et = go_block_sum(bead ? (double)e : 0.0, red);
  const int part = (int)go_cluster_rank() - c.peer0;
  if (threadIdx.x == 0 && live) go_st_peer(go_peer_addr(&epart[part], (uint32_t)c.peer0), et);
  go_cluster_sync();
  if (threadIdx.x == 0 && live && part == 0) {
    double sum = 0.0;
    for (int q = 0; q < c.npeer; q++) sum += epart[q];
    D.epot[c.rep] = sum;
  }
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
  int ncta = 0;     // CTAs of the launch (a multiple of kGoCluster)
  int slots = 0;    // CTAs resident at once, as planned for
  std::vector<int> parts;  // CTAs per replica
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

// threads per bead for a slice of nb beads: as many as fit the CTA (a
// power of two, at most kGoMaxTpb)
static int go_tpb(int nb) {
  int t = 1;
  while (t < kGoMaxTpb && 2 * t * nb <= kGoBlock) t *= 2;
  return t;
}

// The cost of one CTA holding a slice of nb beads of a chain of N: the
// partners each of its threads walks per step.
static int go_cost(int N, int parts) {
  const int nb = (N + parts - 1) / parts;
  return (N + go_tpb(nb) - 1) / go_tpb(nb);
}

// Clusters that chains split into `parts` CTAs pack into: a 4-way chain
// fills one, a 3-way chain takes one with room for a single-CTA chain, 2-way
// chains pair up or share with single-CTA chains.
static int go_clusters(const std::vector<int> &parts) {
  int n[5] = {0, 0, 0, 0, 0};
  for (int p : parts) n[p]++;
  const int ones = std::max(0, n[1] - n[3]);
  return n[4] + n[3] + (2 * n[2] + ones + kGoCluster - 1) / kGoCluster;
}

// Splits each chain over 1 to 4 CTAs of one cluster: starting from one each,
// the chain whose CTA has the highest cost takes the fewest more CTAs that
// lower it, while the clusters needed fit the `slots` CTAs the GPU holds at
// once; then packs the chains into clusters (no chain crosses a cluster)
// and pads the last one.
static std::vector<GoCta> go_plan(const std::vector<int> &nb, int slots) {
  const int n = (int)nb.size();
  std::vector<int> parts(n, 1);
  for (;;) {
    int r = 0;
    for (int q = 1; q < n; q++)
      if (go_cost(nb[q], parts[q]) > go_cost(nb[r], parts[r])) r = q;
    int P = parts[r] + 1;
    while (P <= kGoCluster && go_cost(nb[r], P) >= go_cost(nb[r], parts[r])) P++;
    if (P > kGoCluster) break;
    std::vector<int> trial = parts;
    trial[r] = P;
    if (go_clusters(trial) * kGoCluster > slots) break;
    parts = trial;
  }
  std::vector<GoCta> t;
  auto add = [&](int r) {
    const int base = (int)t.size(), P = parts[r];
    for (int p = 0; p < P; p++) {
      int lo = (int)((long long)p * nb[r] / P), hi = (int)((long long)(p + 1) * nb[r] / P);
      t.push_back(GoCta{r, lo, hi - lo, go_tpb(hi - lo), base % kGoCluster, P});
    }
  };
  const GoCta pad{-1, 0, 0, 1, 0, 0};
  std::vector<int> ones;
  for (int r = 0; r < n; r++)
    if (parts[r] == 1) ones.push_back(r);
  size_t next1 = 0;
  for (int r = 0; r < n; r++)
    if (parts[r] == 4) add(r);
  for (int r = 0; r < n; r++)
    if (parts[r] == 3) {
      add(r);
      if (next1 < ones.size()) add(ones[next1++]);
      else t.push_back(pad);
    }
  for (int r = 0; r < n; r++)
    if (parts[r] == 2) add(r);
  for (; next1 < ones.size(); next1++) add(ones[next1]);
  while (t.size() % kGoCluster) t.push_back(pad);
  return t;
}

static int go_launch(GoBatch *G, int nsteps, int mode) {
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = kGoCluster;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3((unsigned)G->ncta);
  cfg.blockDim = dim3(kGoBlock);
  cfg.dynamicSmemBytes = G->smem;
  cfg.stream = G->st;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  cudaError_t e = G->K.form == 0
                      ? cudaLaunchKernelEx(&cfg, k_go_segment<0>, G->K, G->D, nsteps, mode)
                      : cudaLaunchKernelEx(&cfg, k_go_segment<1>, G->K, G->D, nsteps, mode);
  if (e != cudaSuccess) return cuda_fail(e, "k_go_segment");
  return FE_OK;
}

static int go_launch_segment(GoBatch *G, int nsteps, int exchange) {
  int rc = go_launch(G, nsteps, 0);
  if (rc) return rc;
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
  {
    double s2 = p->sigma_rep * p->sigma_rep, s12 = s2 * s2 * s2 * s2 * s2 * s2;
    K.c12 = (float)(p->eps * s12);
    K.f12 = (float)(12.0 * p->eps * s12);
  }
  K.c6 = K.f6 = 0.f;
  K.e0 = -K.e_shift;
  K.form = 0;
  K.kq = K.kth = K.kph = 0.f;
  K.rc2n = 0.f;
  K.kb = (float)p->k_bond;
  K.r0b = (float)p->r_bond;
  K.acc_fac = 100.0 / p->mass;
  K.vscale = sqrt(100.0 / p->mass);
  K.dt = p->dt;
  K.c1 = exp(-p->gamma * p->dt);
  K.c2 = sqrt(1.0 - K.c1 * K.c1);
  K.min_sep = p->min_sep < 1 ? 1 : p->min_sep;
  K.nrep = nrep;
  K.maxN = maxN;
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
    // two position buffers of the longest chain, and the skip rows of the
    // largest slice (sized for one CTA per chain, which bounds any split)
    size_t rowsz = 0;
    for (int r = 0; r < nrep; r++)
      rowsz = std::max(rowsz, (size_t)nbeads[r] * ((nbeads[r] + 31) / 32));
    G->smem = 2 * sizeof(float4) * (size_t)maxN + sizeof(unsigned) * rowsz;
    // the kernel's limit set once for the largest batch any handle can hold
    // (1,024 beads), so that handles of different sizes never lower it
    // under one another's launches
    const int smem_cap = (int)(2 * sizeof(float4) * kGoMaxBeads +
                               sizeof(unsigned) * kGoMaxBeads * (kGoMaxBeads / 32));
    if (cudaFuncSetAttribute(k_go_segment<0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem_cap) != cudaSuccess ||
        cudaFuncSetAttribute(k_go_segment<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem_cap) != cudaSuccess) {
      rc = cuda_fail(cudaGetLastError(), "cudaFuncSetAttribute");
      break;
    }
    // CTAs resident at once: whole clusters of this kernel's shape
    int nsm = 0, nclu = 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, G->dev) != cudaSuccess) {
      rc = cuda_fail(cudaGetLastError(), "cudaDeviceGetAttribute");
      break;
    }
    {
      cudaLaunchConfig_t cfg = {};
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = kGoCluster;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.gridDim = dim3((unsigned)(kGoCluster * ((nsm + kGoCluster - 1) / kGoCluster)));
      cfg.blockDim = dim3(kGoBlock);
      cfg.dynamicSmemBytes = G->smem;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      if (cudaOccupancyMaxActiveClusters(&nclu, k_go_segment<1>, &cfg) != cudaSuccess) {
        cudaGetLastError();
        nclu = nsm / kGoCluster;
      }
    }
    std::vector<int> nbv(nbeads, nbeads + nrep);
    G->slots = std::max(1, std::min(nclu, nsm / kGoCluster)) * kGoCluster;
    std::vector<GoCta> plan = go_plan(nbv, G->slots);
    G->ncta = (int)plan.size();
    G->parts.assign(nrep, 0);
    for (const GoCta &c : plan)
      if (c.rep >= 0 && c.lo == 0) G->parts[c.rep] = c.npeer;
    if ((rc = go_upload(G, (GoCta **)&D.cta, plan.data(), plan.size()))) break;
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
  int rc = go_launch(G, 0, 1);
  if (rc) return rc;
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

int fe_go_set_reference_form(fe_go *h, const double *bond_r0, const double *bend_t0,
                             double d_rep, double rc) {
  if (!h || !bond_r0 || !bend_t0 || !(d_rep > 0.0) || !(rc > d_rep)) {
    set_error("fe_go_set_reference_form: invalid argument");
    return FE_ERR_ARG;
  }
  GoBatch *G = &h->G;
  FE_CUDA(cudaStreamSynchronize(G->st));
  std::vector<float> br(G->total), bt(G->total);
  for (int i = 0; i < G->total; i++) {
    br[i] = (float)bond_r0[i];
    bt[i] = (float)bend_t0[i];
  }
  int rc_ = FE_OK;
  if (!G->D.bond_r0 && (rc_ = go_upload(G, (float **)&G->D.bond_r0, br.data(), br.size())))
    return rc_;
  if (!G->D.bend_t0 && (rc_ = go_upload(G, (float **)&G->D.bend_t0, bt.data(), bt.size())))
    return rc_;
  FE_CUDA(cudaMemcpy((void *)G->D.bond_r0, br.data(), sizeof(float) * br.size(),
                     cudaMemcpyHostToDevice));
  FE_CUDA(cudaMemcpy((void *)G->D.bend_t0, bt.data(), sizeof(float) * bt.size(),
                     cudaMemcpyHostToDevice));
  GoK &K = G->K;
  const double eps = K.eps;  // kJ/mol
  const double factor = pow(2.0, -1.0 / 6.0);  // read_golik.c:38
  const double sg = factor * d_rep, s6 = pow(sg, 6.0), s12 = s6 * s6;
  // non-natives: 4 eps [(s/r)^12 - (s/r)^6] + eps within d_rep (cgolik.c:780-800)
  K.rc2 = (float)(d_rep * d_rep);
  K.c12 = (float)(4.0 * eps * s12);
  K.c6 = (float)(4.0 * eps * s6);
  K.f12 = (float)(48.0 * eps * s12);
  K.f6 = (float)(24.0 * eps * s6);
  K.e0 = (float)eps;
  K.rc2n = (float)(rc * rc);
  K.kb = (float)eps;           // cbb_golik: -k1 = eps, -k2 = 100 eps
  K.kq = (float)(100.0 * eps);
  K.kth = (float)(10.0 * eps);  // cba_golik: k_theta = -10 eps
  K.kph = (float)(0.2 * eps);   // cda_golik: k_phi = 0.2 eps
  K.min_sep = 2;                // only bonded pairs are excluded (read_golik.c:99-110)
  K.form = 1;
  if (G->g) cudaGraphExecDestroy(G->g);  // recaptured with the new parameters
  G->g = nullptr;
  G->g_len = -1;
  return FE_OK;
}

int fe_go_layout(fe_go *h, int *ncta, int *slots, int *parts) {
  if (!h) return FE_ERR_ARG;
  const GoBatch *G = &h->G;
  if (ncta) *ncta = G->ncta;
  if (slots) *slots = G->slots;
  if (parts)
    for (int r = 0; r < G->nrep; r++) parts[r] = G->parts[r];
  return FE_OK;
}

int fe_go_get_stream(fe_go *h, void **stream) {
  if (!h || !stream) return FE_ERR_ARG;
  *stream = (void *)h->G.st;
  return FE_OK;
}

}  // extern "C"
