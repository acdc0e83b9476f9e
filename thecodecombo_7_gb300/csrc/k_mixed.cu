// k_mixed.cu -- the mixed-precision force engine: FP32 pair and SPME math,
// 64-bit fixed-point force sums (exact, so the result does not depend on
// summation order), FP64 integration and energy reductions.
//
// Layout (rebuilt with the list, every nlist steps):
//   * sites are sorted by a cell grid of edge h >= rlist/2; perm[s] is the
//     original index of sorted slot s, and each slot keeps the cell it was
//     assigned to until the next rebuild;
//   * every step, pos32[s] = (x - C_cell) wrapped to the nearest image, in
//     FP32 (|.| ~ h/2, so FP32 rounding is ~2e-7 A), and q;
//   * the list is FULL (both directions, no Newton-3 scatter, no atomics on
//     the j side): row s holds entries (j << 9) | code for every non-excluded
//     j within rlist, code = the integer image shift o in {-3..3}^3 such
//     that d = (r_i - r_j) + o * h exactly; o*h is a hi+lo float pair in
//     shared memory;
//   * excluded / 1-4 pairs (xint) are handled by a separate kernel over the
//     exclusion list (cnonbond_nblist.c:245-263, 416-437 semantics).
// One warp per i site walks its row with coalesced entry loads; each lane
// keeps an FP32 partial, converts it to fixed point (2^32 per kJ/mol/A) and
// the warp adds the integers -- exact and order independent.
#include <climits>
#include <cmath>
#include <vector>

#include "fe_device.cuh"
#include "fe_mixed.h"

namespace fe {

constexpr double kFixScale = 4294967296.0;  // 2^32
constexpr float kFixScaleF = 4294967296.0f;
constexpr int kMxWarps = 8;                 // warps per block in the pair kernel
constexpr int kMxMaxCellAtoms = 2048;       // sites per cell a sort block handles
constexpr int kCodes = 343;                 // 7^3 image shifts

__device__ __forceinline__ long long to_fix(float v) { return __float2ll_rn(v * kFixScaleF); }

__device__ __forceinline__ int shift_code(int ox, int oy, int oz) {
  return ((ox + 3) * 7 + (oy + 3)) * 7 + (oz + 3);
}

// ---------------------------------------------------------------------------
// list build

__global__ void k_mx_cell(int n, const double4 *__restrict__ pos, double3 L, double3 h, int3 nc,
                          int *__restrict__ cell_of, int *__restrict__ count) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double4 p = pos[i];
  int cx = (int)floor((p.x + 0.5 * L.x) / h.x);
  int cy = (int)floor((p.y + 0.5 * L.y) / h.y);
  int cz = (int)floor((p.z + 0.5 * L.z) / h.z);
  cx = min(max(cx, 0), nc.x - 1);
  cy = min(max(cy, 0), nc.y - 1);
  cz = min(max(cz, 0), nc.z - 1);
  int c = (cx * nc.y + cy) * nc.z + cz;
  cell_of[i] = c;
  atomicAdd(&count[c], 1);
}

__global__ void k_mx_fill(int n, const int *__restrict__ cell_of, const int *__restrict__ start,
                          int *__restrict__ fill, int *__restrict__ perm) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int c = cell_of[i];
  int s = atomicAdd(&fill[c], 1);
  perm[start[c] + s] = i;
}

// order each cell's sites by original index (deterministic layout)
__global__ void k_mx_cellsort(const int *__restrict__ start, int *__restrict__ perm,
                              int *__restrict__ iperm, int *__restrict__ cell_s,
                              int *__restrict__ status) {
  __shared__ int buf[kMxMaxCellAtoms];
  int c = blockIdx.x;
  int s0 = start[c], s1 = start[c + 1];
  int m = s1 - s0;
  if (m > kMxMaxCellAtoms) {
    if (threadIdx.x == 0) atomicOr(status, ST_CELL_OVERFLOW);
    m = kMxMaxCellAtoms;
  }
  int P = 1;
  while (P < m) P <<= 1;
  for (int i = threadIdx.x; i < P; i += blockDim.x) buf[i] = i < m ? perm[s0 + i] : INT_MAX;
  __syncthreads();
  for (int k = 2; k <= P; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < P; i += blockDim.x) {
        int ixj = i ^ j;
        if (ixj > i) {
          int a = buf[i], b = buf[ixj];
          bool up = (i & k) == 0;
          if ((a > b) == up) {
            buf[i] = b;
            buf[ixj] = a;
          }
        }
      }
      __syncthreads();
    }
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    int o = buf[i];
    perm[s0 + i] = o;
    iperm[o] = s0 + i;
    cell_s[s0 + i] = c;
  }
}

// per step: sorted FP32 cell-relative coordinates and charge
__global__ void k_mx_convert(int n, const double4 *__restrict__ pos, const int *__restrict__ perm,
                             const int *__restrict__ cell_s, double3 L, double3 h, int3 nc,
                             float4 *__restrict__ pos32) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  int i = perm[s];
  int c = cell_s[s];
  int cz = c % nc.z, cy = (c / nc.z) % nc.y, cx = c / (nc.z * nc.y);
  double4 p = pos[i];
  double rx = p.x - ((cx + 0.5) * h.x - 0.5 * L.x);
  double ry = p.y - ((cy + 0.5) * h.y - 0.5 * L.y);
  double rz = p.z - ((cz + 0.5) * h.z - 0.5 * L.z);
  rx -= L.x * rint(rx / L.x);
  ry -= L.y * rint(ry / L.y);
  rz -= L.z * rint(rz / L.z);
  pos32[s] = make_float4((float)rx, (float)ry, (float)rz, (float)p.w);
}

__device__ __forceinline__ int mx_is_excluded(const int *__restrict__ xs, const int *__restrict__ xp,
                                              int a, int b) {
  for (int p = xs[a]; p < xs[a + 1]; p++)
    if (xp[p] == b) return 1;
  return 0;
}

// one warp per sorted site: all non-excluded j != i within rlist, in a fixed
// (cell, slot) order -- no sort needed for a deterministic row
__global__ void __launch_bounds__(kMxWarps * 32)
k_mx_list(int n, const float4 *__restrict__ pos32, const int *__restrict__ perm,
          const int *__restrict__ cell_s, const int *__restrict__ cstart, int3 nc, float3 hf,
          float3 Lf, float rlist2, const int *__restrict__ xs, const int *__restrict__ xp,
          int cap, int *__restrict__ count, int *__restrict__ ent, int *__restrict__ status) {
  int lane = threadIdx.x & 31;
  int nx = nc.x >= 5 ? 5 : nc.x, ny = nc.y >= 5 ? 5 : nc.y, nz = nc.z >= 5 ? 5 : nc.z;
  for (int s = blockIdx.x * kMxWarps + (threadIdx.x >> 5); s < n; s += gridDim.x * kMxWarps) {
    float4 ri = pos32[s];
    int c = cell_s[s];
    int cz = c % nc.z, cy = (c / nc.z) % nc.y, cx = c / (nc.z * nc.y);
    int oi = perm[s];
    int cnt = 0;
    int *row = ent + (size_t)s * cap;
    for (int ix = 0; ix < nx; ix++) {
      int x = nc.x >= 5 ? (cx + ix - 2 + nc.x) % nc.x : ix;
      for (int iy = 0; iy < ny; iy++) {
        int y = nc.y >= 5 ? (cy + iy - 2 + nc.y) % nc.y : iy;
        for (int iz = 0; iz < nz; iz++) {
          int z = nc.z >= 5 ? (cz + iz - 2 + nc.z) % nc.z : iz;
          int cj = (x * nc.y + y) * nc.z + z;
          // raw cell offset and the image that brings the cell nearest
          int dcx = cx - x, dcy = cy - y, dcz = cz - z;
          int s0 = cstart[cj], s1 = cstart[cj + 1];
          for (int base = s0; base < s1; base += 32) {
            int j = base + lane;
            bool ok = false;
            int code = 0;
            if (j < s1 && j != s) {
              float4 rj = pos32[j];
              float rx = ri.x - rj.x, ry = ri.y - rj.y, rz = ri.z - rj.z;
              // d_raw = r_i - r_j + (c_i - c_j) h ; o = (c_i - c_j) - nc * k
              float ddx = rx + dcx * hf.x, ddy = ry + dcy * hf.y, ddz = rz + dcz * hf.z;
              int kx = (int)rintf(ddx / Lf.x), ky = (int)rintf(ddy / Lf.y), kz = (int)rintf(ddz / Lf.z);
              int ox = dcx - kx * nc.x, oy = dcy - ky * nc.y, oz = dcz - kz * nc.z;
              if (ox >= -3 && ox <= 3 && oy >= -3 && oy <= 3 && oz >= -3 && oz <= 3) {
                float dx = rx + ox * hf.x, dy = ry + oy * hf.y, dz = rz + oz * hf.z;
                float r2 = dx * dx + dy * dy + dz * dz;
                if (r2 < rlist2) {
                  ok = !mx_is_excluded(xs, xp, oi, perm[j]);
                  code = shift_code(ox, oy, oz);
                }
              }
            }
            unsigned m = __ballot_sync(0xffffffffu, ok);
            if (ok) {
              int p = cnt + __popc(m & ((1u << lane) - 1u));
              if (p < cap) row[p] = (j << 9) | code;
            }
            cnt += __popc(m);
          }
        }
      }
    }
    if (lane == 0) {
      count[s] = cnt < cap ? cnt : cap;
      if (cnt > cap) atomicOr(status, ST_LIST_OVERFLOW);
    }
  }
}

// ---------------------------------------------------------------------------
// pair kernel

struct MxPair {
  int n, nt, cap;
  float rc2, kappa, c2k, qfe;  // c2k = 2 kappa / sqrt(pi); qfe = QFACTOR / epsRF
  float ron2, sw_den;
};

// the reference's erfc (ewald.c:817-836, Numerical Recipes "erfcc") in FP32;
// ex = exp(-z^2) is shared with the force term
__device__ __forceinline__ float erfc_nr_f(float z, float ex) {
  float t = __frcp_rn(1.0f + 0.5f * z);
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

__global__ void __launch_bounds__(kMxWarps * 32)
k_mx_pair(MxPair P, const float4 *__restrict__ pos32, const int *__restrict__ type_s,
          const int *__restrict__ perm, const int *__restrict__ count, const int *__restrict__ ent,
          const float *__restrict__ shift_tab, const float *__restrict__ lj_tab,
          unsigned long long *__restrict__ fix, double *__restrict__ partials) {
  extern __shared__ float sh[];
  float *s_shift = sh;                 // kCodes * 6: hi xyz, lo xyz
  float *s_lj = sh + kCodes * 6;       // nt*nt*3: eps, sig^2, shift const
  for (int i = threadIdx.x; i < kCodes * 6; i += blockDim.x) s_shift[i] = shift_tab[i];
  for (int i = threadIdx.x; i < P.nt * P.nt * 3; i += blockDim.x) s_lj[i] = lj_tab[i];
  __syncthreads();
  int lane = threadIdx.x & 31;
  float e_lj = 0.f, e_ljs = 0.f, e_real = 0.f, qsum = 0.f;
  for (int s = blockIdx.x * kMxWarps + (threadIdx.x >> 5); s < P.n; s += gridDim.x * kMxWarps) {
    float4 ri = pos32[s];
    int ti = type_s[s];
    int cnt = count[s];
    const int *row = ent + (size_t)s * P.cap;
    float fx = 0.f, fy = 0.f, fz = 0.f;
    for (int bb = lane; bb < cnt; bb += 32) {
      int e = row[bb];
      int j = e >> 9;
      const float *o = s_shift + (e & 511) * 6;
      float4 rj = pos32[j];
      float dx = ((ri.x - rj.x) + o[0]) + o[3];
      float dy = ((ri.y - rj.y) + o[1]) + o[4];
      float dz = ((ri.z - rj.z) + o[2]) + o[5];
      float r2 = dx * dx + dy * dy + dz * dz;
      if (r2 > P.rc2) continue;
      float rinv = rsqrtf(r2);
      float r = r2 * rinv;
      float rinv2 = rinv * rinv;
      float qq = ri.w * rj.w * P.qfe;
      float kr = P.kappa * r;
      float ex = __expf(-kr * kr);
      float erfckr = erfc_nr_f(kr, ex);
      float F = qq * rinv * rinv2 * (erfckr + P.c2k * r * ex);
      e_real += qq * erfckr * rinv;
      qsum += qq;
      int tj = type_s[j];
      const float *lj = s_lj + (ti * P.nt + tj) * 3;
      float eps = lj[0];
      if (eps != 0.f) {
        float sr2 = lj[1] * rinv2;
        float sr6 = sr2 * sr2 * sr2;
        float sr12 = sr6 * sr6;
        float flj = 12.f * eps * rinv2 * (sr12 - sr6);
        float elj = eps * (sr12 - 2.f * sr6);
        if (P.ron2 > 0.f) {
          if (r2 > P.ron2) {
            float c = P.rc2 - r2;
            float sw = c * c * (P.rc2 + 2.f * r2 - 3.f * P.ron2) / P.sw_den;
            float dsw = 12.f * c * (r2 - P.ron2) / P.sw_den;
            flj = flj * sw + elj * dsw;
            elj = elj * sw;
          }
        } else {
          e_ljs += eps * lj[2];
        }
        F += flj;
        e_lj += elj;
      }
      fx += F * dx;
      fy += F * dy;
      fz += F * dz;
    }
    long long ix = to_fix(fx), iy = to_fix(fy), iz = to_fix(fz);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      ix += __shfl_xor_sync(0xffffffffu, ix, o);
      iy += __shfl_xor_sync(0xffffffffu, iy, o);
      iz += __shfl_xor_sync(0xffffffffu, iz, o);
    }
    if (lane == 0) {
      int oi = perm[s];
      atomicAdd(&fix[3 * oi], (unsigned long long)ix);
      atomicAdd(&fix[3 * oi + 1], (unsigned long long)iy);
      atomicAdd(&fix[3 * oi + 2], (unsigned long long)iz);
    }
  }
  // every pair was visited from both ends
  double v[4] = {0.5 * (double)e_lj, 0.5 * (double)e_ljs, 0.5 * (double)e_real, 0.5 * (double)qsum};
  block_partials<4>(v, partials);
}

// excluded and 1-4 pairs (xint), cnonbond_nblist.c:245-263 and 416-437:
// inside rc an excluded pair contributes no LJ and no real-space term but the
// intra correction -qq (1 - erfc(kr)) / r; a 1-4 pair gets LJ, real space
// scaled by E14FAC and the correction with (1 - E14FAC)
__global__ void k_mx_excl(int nexcl, const int *__restrict__ ab, const int *__restrict__ flag,
                          const double4 *__restrict__ pos, const int *__restrict__ type, double3 L,
                          int nt, const float *__restrict__ lj_tab, float rc2, float kappa,
                          float c2k, float qf, float epsRF, unsigned long long *__restrict__ fix,
                          double *__restrict__ partials) {
  float e_intra = 0.f, e_lj = 0.f, e_ljs = 0.f, e_real = 0.f, qsum = 0.f;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nexcl; t += gridDim.x * blockDim.x) {
    int a = ab[2 * t], b = ab[2 * t + 1], xf = flag[t];
    if (xf == 0) continue;
    double4 A = pos[a], B = pos[b];
    double ddx = A.x - B.x, ddy = A.y - B.y, ddz = A.z - B.z;
    ddx -= L.x * rint(ddx / L.x);
    ddy -= L.y * rint(ddy / L.y);
    ddz -= L.z * rint(ddz / L.z);
    float dx = (float)ddx, dy = (float)ddy, dz = (float)ddz;
    float r2 = dx * dx + dy * dy + dz * dz;
    if (r2 > rc2) continue;
    float rinv = rsqrtf(r2), r = r2 * rinv, rinv2 = rinv * rinv;
    float kr = kappa * r;
    float ex = __expf(-kr * kr);
    float erfckr = erfc_nr_f(kr, ex);
    float qqab = (float)A.w * (float)B.w * qf;
    float F = 0.f;
    float qcorr = qqab;
    if (xf == 4) {
      float qq = qqab * (float)kE14FAC / epsRF;
      F += qq * rinv * rinv2 * (erfckr + c2k * r * ex);
      e_real += qq * erfckr * rinv;
      qsum += qq;
      const float *lj = lj_tab + (type[a] * nt + type[b]) * 3;
      if (lj[0] != 0.f) {
        float sr2 = lj[1] * rinv2, sr6 = sr2 * sr2 * sr2, sr12 = sr6 * sr6;
        F += 12.f * lj[0] * rinv2 * (sr12 - sr6);
        e_lj += lj[0] * (sr12 - 2.f * sr6);
        e_ljs += lj[0] * lj[2];
      }
      qcorr *= (1.f - (float)kE14FAC);
    }
    float erfkr = 1.f - erfckr;
    e_intra += qcorr * erfkr * rinv;
    F -= qcorr * rinv * rinv2 * (erfkr - c2k * r * ex);
    long long fxq = to_fix(F * dx), fyq = to_fix(F * dy), fzq = to_fix(F * dz);
    atomicAdd(&fix[3 * a], (unsigned long long)fxq);
    atomicAdd(&fix[3 * a + 1], (unsigned long long)fyq);
    atomicAdd(&fix[3 * a + 2], (unsigned long long)fzq);
    atomicAdd(&fix[3 * b], (unsigned long long)(-fxq));
    atomicAdd(&fix[3 * b + 1], (unsigned long long)(-fyq));
    atomicAdd(&fix[3 * b + 2], (unsigned long long)(-fzq));
  }
  double v[5] = {(double)e_lj, (double)e_ljs, (double)e_real, (double)qsum, (double)e_intra};
  block_partials<5>(v, partials);
}

// bonded terms in FP32 from FP64 differences (cbond.c, cbend.c)
__global__ void k_mx_bonded(int nbond, int nbend, double3 L, const double4 *__restrict__ pos,
                            const int *__restrict__ bond_ab, const double *__restrict__ bond_req,
                            const double *__restrict__ bond_k, const int *__restrict__ bend_abc,
                            const double *__restrict__ bend_t0, const double *__restrict__ bend_k,
                            unsigned long long *__restrict__ fix, double *__restrict__ partials) {
  float eb = 0.f, ea = 0.f;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nbond + nbend;
       t += gridDim.x * blockDim.x) {
    if (t < nbond) {
      int ia = bond_ab[2 * t], ib = bond_ab[2 * t + 1];
      double4 A = pos[ia], B = pos[ib];
      double ddx = B.x - A.x, ddy = B.y - A.y, ddz = B.z - A.z;
      ddx -= L.x * rint(ddx / L.x);
      ddy -= L.y * rint(ddy / L.y);
      ddz -= L.z * rint(ddz / L.z);
      float dx = (float)ddx, dy = (float)ddy, dz = (float)ddz;
      float dr = sqrtf(dx * dx + dy * dy + dz * dz);
      float rr = dr - (float)bond_req[t];
      float fr = -(float)bond_k[t] * rr * 2.f;
      eb += -(fr * rr * 0.5f);
      float s = fr / dr;
      long long fxq = to_fix(s * dx), fyq = to_fix(s * dy), fzq = to_fix(s * dz);
      atomicAdd(&fix[3 * ia], (unsigned long long)(-fxq));
      atomicAdd(&fix[3 * ia + 1], (unsigned long long)(-fyq));
      atomicAdd(&fix[3 * ia + 2], (unsigned long long)(-fzq));
      atomicAdd(&fix[3 * ib], (unsigned long long)fxq);
      atomicAdd(&fix[3 * ib + 1], (unsigned long long)fyq);
      atomicAdd(&fix[3 * ib + 2], (unsigned long long)fzq);
    } else {
      int u = t - nbond;
      int ia = bend_abc[3 * u], ib = bend_abc[3 * u + 1], ic = bend_abc[3 * u + 2];
      double4 A = pos[ia], B = pos[ib], Cc = pos[ic];
      double d0 = A.x - B.x, d1 = A.y - B.y, d2 = A.z - B.z;
      double e0 = Cc.x - B.x, e1 = Cc.y - B.y, e2 = Cc.z - B.z;
      d0 -= L.x * rint(d0 / L.x);
      d1 -= L.y * rint(d1 / L.y);
      d2 -= L.z * rint(d2 / L.z);
      e0 -= L.x * rint(e0 / L.x);
      e1 -= L.y * rint(e1 / L.y);
      e2 -= L.z * rint(e2 / L.z);
      float dax = (float)d0, day = (float)d1, daz = (float)d2;
      float dcx = (float)e0, dcy = (float)e1, dcz = (float)e2;
      float drai = rsqrtf(dax * dax + day * day + daz * daz);
      float erax = dax * drai, eray = day * drai, eraz = daz * drai;
      float drci = rsqrtf(dcx * dcx + dcy * dcy + dcz * dcz);
      float ercx = dcx * drci, ercy = dcy * drci, ercz = dcz * drci;
      float cosphi = erax * ercx + eray * ercy + eraz * ercz;
      cosphi = fminf(fmaxf(cosphi, -1.f), 1.f);
      float phi = acosf(cosphi);
      float isinphi = rsqrtf(fmaxf(1.f - cosphi * cosphi, 1e-20f));
      float rr = phi - (float)bend_t0[u];
      float fr = -(float)bend_k[u] * rr * 2.f;
      ea += -fr * rr * 0.5f;
      float irasin = drai * isinphi * fr, ircsin = drci * isinphi * fr;
      float fxa = (erax * cosphi - ercx) * irasin, fya = (eray * cosphi - ercy) * irasin,
            fza = (eraz * cosphi - ercz) * irasin;
      float fxc = (ercx * cosphi - erax) * ircsin, fyc = (ercy * cosphi - eray) * ircsin,
            fzc = (ercz * cosphi - eraz) * ircsin;
      long long ax = to_fix(fxa), ay = to_fix(fya), az = to_fix(fza);
      long long cx = to_fix(fxc), cy = to_fix(fyc), cz = to_fix(fzc);
      atomicAdd(&fix[3 * ia], (unsigned long long)ax);
      atomicAdd(&fix[3 * ia + 1], (unsigned long long)ay);
      atomicAdd(&fix[3 * ia + 2], (unsigned long long)az);
      atomicAdd(&fix[3 * ib], (unsigned long long)(-(ax + cx)));
      atomicAdd(&fix[3 * ib + 1], (unsigned long long)(-(ay + cy)));
      atomicAdd(&fix[3 * ib + 2], (unsigned long long)(-(az + cz)));
      atomicAdd(&fix[3 * ic], (unsigned long long)cx);
      atomicAdd(&fix[3 * ic + 1], (unsigned long long)cy);
      atomicAdd(&fix[3 * ic + 2], (unsigned long long)cz);
    }
  }
  double v[2] = {(double)eb, (double)ea};
  block_partials<2>(v, partials);
}

// ---------------------------------------------------------------------------
// SPME in FP32

__device__ __forceinline__ int wrapg32(int v, int g) {
  v %= g;
  return v < 0 ? v + g : v;
}

// B-spline weights of order p at fraction w (same recursion as
// pme_spline.c:10-49), FP32
__device__ __forceinline__ void fillspline_f(int order, float w, float *array, float *darray) {
  for (int i = 3; i <= order; i++) array[i] = 0.f;
  array[2] = w;
  array[1] = 1.f - w;
  array[0] = 0.f;
  for (int i = 3; i <= order - 1; i++) {
    float div = 1.f / (float)(i - 1);
    array[i] = div * w * array[i - 1];
    for (int j = 1; j <= (i - 2); j++)
      array[i - j] = div * ((w + j) * array[i - j - 1] + ((float)(i - j) - w) * array[i - j]);
    array[1] *= div * (1.f - w);
  }
  darray[0] = 0.f;
  darray[1] = -array[1];
  for (int i = 2; i <= order; i++) darray[i] = array[i - 1] - array[i];
  int kk = order;
  float div = 1.f / (float)(kk - 1);
  array[kk] = div * w * array[kk - 1];
  for (int i = 1; i <= (kk - 2); i++)
    array[kk - i] = div * ((w + i) * array[kk - i - 1] + ((float)(kk - i) - w) * array[kk - i]);
  array[1] *= div * (1.f - w);
}

// per sorted slot: origin cell (FP64 fraction), FP32 weights, binning
__global__ void k_mx_splines(int n, int order, int3 G, double3 L, const double4 *__restrict__ pos,
                             const int *__restrict__ perm, int *__restrict__ floor3,
                             float *__restrict__ sm, float *__restrict__ sd, int gcap,
                             int *__restrict__ bcount, int *__restrict__ batoms,
                             int *__restrict__ status) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  double4 p = pos[perm[s]];
  double ss[3] = {G.x * (p.x / L.x + 0.5), G.y * (p.y / L.y + 0.5), G.z * (p.z / L.z + 0.5)};
  int g[3] = {G.x, G.y, G.z};
  int f[3];
  float mn[9], dmn[9];
  for (int d = 0; d < 3; d++) {
    f[d] = (int)ss[d];
    float w = (float)(ss[d] - (double)f[d]);
    fillspline_f(order, w, mn, dmn);
    for (int m = 1; m <= order; m++) {
      sm[((size_t)s * order + (m - 1)) * 3 + d] = mn[m];
      sd[((size_t)s * order + (m - 1)) * 3 + d] = dmn[m];
    }
    floor3[3 * s + d] = f[d];
  }
  int cell = (wrapg32(f[0], g[0]) * g[1] + wrapg32(f[1], g[1])) * g[2] + wrapg32(f[2], g[2]);
  int k = atomicAdd(&bcount[cell], 1);
  if (k < gcap) batoms[(size_t)cell * gcap + k] = s;
  else atomicOr(status, ST_GRID_OVERFLOW);
}

__global__ void k_mx_binsort(long K, int gcap, int *__restrict__ bcount, int *__restrict__ batoms) {
  long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= K) return;
  int m = bcount[c];
  if (m > gcap) {
    m = gcap;
    bcount[c] = gcap;
  }
  int *a = batoms + c * gcap;
  for (int i = 1; i < m; i++) {
    int v = a[i], j = i - 1;
    while (j >= 0 && a[j] > v) {
      a[j + 1] = a[j];
      j--;
    }
    a[j + 1] = v;
  }
}

// atom-free gather spreading, one thread per grid point (x, y, z)
__global__ void k_mx_spread(int order, int3 G, const float4 *__restrict__ pos32,
                            const float *__restrict__ sm, int gcap, const int *__restrict__ bcount,
                            const int *__restrict__ batoms, float *__restrict__ grid) {
  long K = (long)G.x * G.y * G.z;
  long id = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= K) return;
  int z = (int)(id % G.z);
  int y = (int)((id / G.z) % G.y);
  int x = (int)(id / ((long)G.z * G.y));
  float sum = 0.f;
  for (int xi = 1; xi <= order; xi++) {
    int fx = wrapg32(x + order - xi, G.x);
    for (int yi = 1; yi <= order; yi++) {
      int fy = wrapg32(y + order - yi, G.y);
      long cb = ((long)fx * G.y + fy) * G.z;
      for (int zi = 1; zi <= order; zi++) {
        int fz = wrapg32(z + order - zi, G.z);
        long c = cb + fz;
        int m = bcount[c];
        const int *at = batoms + c * gcap;
        for (int k = 0; k < m; k++) {
          int j = at[k];
          const float *w = sm + (size_t)j * order * 3;
          sum += w[(xi - 1) * 3] * w[(yi - 1) * 3 + 1] * w[(zi - 1) * 3 + 2] * pos32[j].w;
        }
      }
    }
  }
  grid[id] = sum;
}

__global__ void k_mx_recip(long Kh, const float *__restrict__ eterm, const float *__restrict__ kw,
                           cufftComplex *__restrict__ gk, double *__restrict__ partials) {
  double e = 0.0;
  for (long h = (long)blockIdx.x * blockDim.x + threadIdx.x; h < Kh;
       h += (long)gridDim.x * blockDim.x) {
    cufftComplex v = gk[h];
    float et = eterm[h];
    e += (double)(kw[h] * et * (v.x * v.x + v.y * v.y));
    v.x *= et;
    v.y *= et;
    gk[h] = v;
  }
  double vv[1] = {e};
  block_partials<1>(vv, partials);
}

__global__ void k_mx_gather(int n, int order, int3 G, float3 gl, float qfe,
                            const float4 *__restrict__ pos32, const int *__restrict__ perm,
                            const int *__restrict__ floor3, const float *__restrict__ sm,
                            const float *__restrict__ sd, const float *__restrict__ grid,
                            unsigned long long *__restrict__ fix, double *__restrict__ partials) {
  double sx = 0.0, sy = 0.0, sz = 0.0;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    float fxi = 0.f, fyi = 0.f, fzi = 0.f;
    const float *m = sm + (size_t)s * order * 3;
    const float *dm = sd + (size_t)s * order * 3;
    int xo = floor3[3 * s] - order, yo0 = floor3[3 * s + 1] - order, zo0 = floor3[3 * s + 2] - order;
    for (int xi = 1; xi <= order; xi++) {
      int x = wrapg32(xo + xi, G.x);
      float mx = m[(xi - 1) * 3], dmx = dm[(xi - 1) * 3];
      for (int yi = 1; yi <= order; yi++) {
        int y = wrapg32(yo0 + yi, G.y);
        float my = m[(yi - 1) * 3 + 1], dmy = dm[(yi - 1) * 3 + 1];
        const float *row = grid + ((long)x * G.y + y) * G.z;
        for (int zi = 1; zi <= order; zi++) {
          int z = wrapg32(zo0 + zi, G.z);
          float mz = m[(zi - 1) * 3 + 2], dmz = dm[(zi - 1) * 3 + 2];
          float term = row[z];
          fxi -= dmx * my * mz * term;
          fyi -= mx * dmy * mz * term;
          fzi -= mx * my * dmz * term;
        }
      }
    }
    float fac = pos32[s].w * qfe;
    fxi *= fac * gl.x;
    fyi *= fac * gl.y;
    fzi *= fac * gl.z;
    int oi = perm[s];
    atomicAdd(&fix[3 * oi], (unsigned long long)to_fix(fxi));
    atomicAdd(&fix[3 * oi + 1], (unsigned long long)to_fix(fyi));
    atomicAdd(&fix[3 * oi + 2], (unsigned long long)to_fix(fzi));
    sx += (double)to_fix(fxi);
    sy += (double)to_fix(fyi);
    sz += (double)to_fix(fzi);
  }
  double v[3] = {sx, sy, sz};
  block_partials<3>(v, partials);
}

// FP64 forces from the fixed-point sums, minus the mean reciprocal force
__global__ void k_mx_finalize(int n, const unsigned long long *__restrict__ fix,
                              const double *__restrict__ scal, double *__restrict__ ff) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * n) return;
  double mean = scal[SC_FMEAN + i % 3] / kFixScale / (double)n;
  ff[i] = (double)(long long)fix[i] / kFixScale - mean;
}

// ---------------------------------------------------------------------------

int mixed_setup(Box *b) {
  Mixed &M = *b->mx;
  int n = b->n;
  // cell grid of edge >= rlist / 2
  double half = 0.5 * (b->p.rclist > b->p.rclist_ew ? b->p.rclist : b->p.rclist_ew);
  M.ncells = 1;
  for (int d = 0; d < 3; d++) {
    int m = (int)(b->p.L[d] / half);
    M.nc[d] = m < 1 ? 1 : m;
    M.h[d] = b->p.L[d] / M.nc[d];
    M.ncells *= M.nc[d];
  }
  if (n >= (1 << 22)) {
    set_error("mixed precision supports at most 4,194,303 sites per box");
    return FE_ERR_SIZE;
  }
  FE_CUDA(cudaMalloc(&M.cell_count, sizeof(int) * M.ncells));
  FE_CUDA(cudaMalloc(&M.cell_start, sizeof(int) * (M.ncells + 1)));
  FE_CUDA(cudaMalloc(&M.cell_fill, sizeof(int) * M.ncells));
  FE_CUDA(cudaMalloc(&M.cell_of, sizeof(int) * n));
  FE_CUDA(cudaMalloc(&M.perm, sizeof(int) * n));
  FE_CUDA(cudaMalloc(&M.iperm, sizeof(int) * n));
  FE_CUDA(cudaMalloc(&M.cell_s, sizeof(int) * n));
  FE_CUDA(cudaMalloc(&M.type_s, sizeof(int) * n));
  FE_CUDA(cudaMalloc(&M.pos32, sizeof(float4) * n));
  // full-list row capacity: a sphere of rlist at the box's density, with margin
  double vol = b->p.L[0] * b->p.L[1] * b->p.L[2];
  double rl = b->p.rclist;
  double expect = 4.0 / 3.0 * kPI * rl * rl * rl * (double)n / vol;
  int cap = (int)(1.6 * expect + 64.0);
  if (b->p.max_neighbors > 0) cap = b->p.max_neighbors;
  cap = (cap + 31) / 32 * 32;
  if (cap > n) cap = (n + 31) / 32 * 32;
  M.cap = cap;
  FE_CUDA(cudaMalloc(&M.count, sizeof(int) * n));
  FE_CUDA(cudaMalloc(&M.ent, sizeof(int) * (size_t)n * cap));
  FE_CUDA(cudaMalloc(&M.fix, sizeof(unsigned long long) * 3 * n));
  // image-shift table: o * h as a hi + lo float pair per component
  std::vector<float> tab(kCodes * 6);
  for (int ox = -3; ox <= 3; ox++)
    for (int oy = -3; oy <= 3; oy++)
      for (int oz = -3; oz <= 3; oz++) {
        int c = ((ox + 3) * 7 + (oy + 3)) * 7 + (oz + 3);
        double v[3] = {ox * M.h[0], oy * M.h[1], oz * M.h[2]};
        for (int d = 0; d < 3; d++) {
          float hi = (float)v[d];
          tab[c * 6 + d] = hi;
          tab[c * 6 + 3 + d] = (float)(v[d] - (double)hi);
        }
      }
  FE_CUDA(cudaMalloc(&M.shift_tab, sizeof(float) * tab.size()));
  FE_CUDA(cudaMemcpy(M.shift_tab, tab.data(), sizeof(float) * tab.size(), cudaMemcpyHostToDevice));
  // LJ table: eps, sig^2, and the energy shift constant (sr12s - 2 sr6s)
  int nt = b->nt;
  std::vector<double> eps(nt * nt), sig(nt * nt);
  FE_CUDA(cudaMemcpy(eps.data(), b->lj_eps, sizeof(double) * nt * nt, cudaMemcpyDeviceToHost));
  FE_CUDA(cudaMemcpy(sig.data(), b->lj_sig, sizeof(double) * nt * nt, cudaMemcpyDeviceToHost));
  std::vector<float> lj(nt * nt * 3);
  double rc2 = b->p.rc * b->p.rc;
  for (int k = 0; k < nt * nt; k++) {
    double s2 = sig[k] * sig[k];
    double sr2s = s2 / rc2, sr6s = sr2s * sr2s * sr2s;
    bool on = (eps[k] * sig[k]) != 0.0;
    lj[3 * k] = on ? (float)eps[k] : 0.f;
    lj[3 * k + 1] = (float)s2;
    lj[3 * k + 2] = (float)(sr6s * sr6s - 2.0 * sr6s);
  }
  FE_CUDA(cudaMalloc(&M.lj_tab, sizeof(float) * lj.size()));
  FE_CUDA(cudaMemcpy(M.lj_tab, lj.data(), sizeof(float) * lj.size(), cudaMemcpyHostToDevice));
  // exclusion pair list (xint), for the correction kernel
  M.nexcl = b->p.nexcl;
  FE_CUDA(cudaMalloc(&M.excl_ab, sizeof(int) * 2 * (M.nexcl ? M.nexcl : 1)));
  FE_CUDA(cudaMalloc(&M.excl_flag, sizeof(int) * (M.nexcl ? M.nexcl : 1)));
  if (M.nexcl) {
    FE_CUDA(cudaMemcpy(M.excl_ab, b->p.excl_ab, sizeof(int) * 2 * M.nexcl, cudaMemcpyHostToDevice));
    FE_CUDA(cudaMemcpy(M.excl_flag, b->p.excl_flag, sizeof(int) * M.nexcl, cudaMemcpyHostToDevice));
  }
  // SPME, FP32
  long K = b->K, Kh = b->Kh;
  std::vector<double> et(Kh), kw(Kh);
  FE_CUDA(cudaMemcpy(et.data(), b->eterm, sizeof(double) * Kh, cudaMemcpyDeviceToHost));
  FE_CUDA(cudaMemcpy(kw.data(), b->kweight, sizeof(double) * Kh, cudaMemcpyDeviceToHost));
  std::vector<float> etf(Kh), kwf(Kh);
  for (long i = 0; i < Kh; i++) {
    etf[i] = (float)et[i];
    kwf[i] = (float)kw[i];
  }
  FE_CUDA(cudaMalloc(&M.eterm32, sizeof(float) * Kh));
  FE_CUDA(cudaMalloc(&M.kw32, sizeof(float) * Kh));
  FE_CUDA(cudaMemcpy(M.eterm32, etf.data(), sizeof(float) * Kh, cudaMemcpyHostToDevice));
  FE_CUDA(cudaMemcpy(M.kw32, kwf.data(), sizeof(float) * Kh, cudaMemcpyHostToDevice));
  FE_CUDA(cudaMalloc(&M.grid32, sizeof(float) * K));
  FE_CUDA(cudaMalloc(&M.grid32k, sizeof(cufftComplex) * Kh));
  FE_CUDA(cudaMalloc(&M.floor3, sizeof(int) * 3 * n));
  FE_CUDA(cudaMalloc(&M.sm, sizeof(float) * 3 * (size_t)n * b->order));
  FE_CUDA(cudaMalloc(&M.sd, sizeof(float) * 3 * (size_t)n * b->order));
  cufftResult r = cufftPlan3d(&M.plan_r2c, b->G[0], b->G[1], b->G[2], CUFFT_R2C);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftPlan3d R2C");
  r = cufftPlan3d(&M.plan_c2r, b->G[0], b->G[1], b->G[2], CUFFT_C2R);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftPlan3d C2R");
  M.plans = true;
  return FE_OK;
}

void mixed_free(Box *b) {
  if (!b->mx) return;
  Mixed &M = *b->mx;
  void *ptrs[] = {M.cell_count, M.cell_start, M.cell_fill, M.cell_of, M.perm, M.iperm, M.cell_s,
                  M.type_s, M.pos32, M.count, M.ent, M.fix, M.shift_tab, M.lj_tab, M.excl_ab,
                  M.excl_flag, M.eterm32, M.kw32, M.grid32, M.grid32k, M.floor3, M.sm, M.sd};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  if (M.plans) {
    cufftDestroy(M.plan_r2c);
    cufftDestroy(M.plan_c2r);
  }
  delete b->mx;
  b->mx = nullptr;
}

__global__ void k_mx_types(int n, const int *__restrict__ perm, const int *__restrict__ type,
                           int *__restrict__ type_s) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n) type_s[s] = type[perm[s]];
}

static int launch_convert(Box *b) {
  Mixed &M = *b->mx;
  double3 L = make_double3(b->p.L[0], b->p.L[1], b->p.L[2]);
  double3 h = make_double3(M.h[0], M.h[1], M.h[2]);
  int3 nc = make_int3(M.nc[0], M.nc[1], M.nc[2]);
  k_mx_convert<<<(b->n + 255) / 256, 256, 0, b->stream>>>(b->n, b->pos_q, M.perm, M.cell_s, L, h, nc,
                                                          M.pos32);
  FE_LAUNCH_CHECK("k_mx_convert");
  return FE_OK;
}

int launch_mixed_list(Box *b) {
  Mixed &M = *b->mx;
  int n = b->n;
  double3 L = make_double3(b->p.L[0], b->p.L[1], b->p.L[2]);
  double3 h = make_double3(M.h[0], M.h[1], M.h[2]);
  int3 nc = make_int3(M.nc[0], M.nc[1], M.nc[2]);
  FE_CUDA(cudaMemsetAsync(M.cell_count, 0, sizeof(int) * M.ncells, b->stream));
  k_mx_cell<<<(n + 255) / 256, 256, 0, b->stream>>>(n, b->pos_q, L, h, nc, M.cell_of, M.cell_count);
  FE_LAUNCH_CHECK("k_mx_cell");
  k_cell_scan_ext(M.cell_count, M.ncells, M.cell_start, M.cell_fill, b->stream);
  k_mx_fill<<<(n + 255) / 256, 256, 0, b->stream>>>(n, M.cell_of, M.cell_start, M.cell_fill, M.perm);
  FE_LAUNCH_CHECK("k_mx_fill");
  k_mx_cellsort<<<M.ncells, 256, 0, b->stream>>>(M.cell_start, M.perm, M.iperm, M.cell_s, b->status);
  FE_LAUNCH_CHECK("k_mx_cellsort");
  k_mx_types<<<(n + 255) / 256, 256, 0, b->stream>>>(n, M.perm, b->type, M.type_s);
  FE_LAUNCH_CHECK("k_mx_types");
  int rc = launch_convert(b);
  if (rc) return rc;
  float3 hf = make_float3((float)M.h[0], (float)M.h[1], (float)M.h[2]);
  float3 Lf = make_float3((float)b->p.L[0], (float)b->p.L[1], (float)b->p.L[2]);
  float rl = (float)(b->p.rclist < b->p.rclist_ew ? b->p.rclist : b->p.rclist_ew);
  int blocks = (n + kMxWarps - 1) / kMxWarps;
  if (blocks > 152 * 8) blocks = 152 * 8;
  k_mx_list<<<blocks, kMxWarps * 32, 0, b->stream>>>(n, M.pos32, M.perm, M.cell_s, M.cell_start, nc,
                                                     hf, Lf, rl * rl, b->x_start, b->x_partner,
                                                     M.cap, M.count, M.ent, b->status);
  FE_LAUNCH_CHECK("k_mx_list");
  b->have_list = true;
  return FE_OK;
}

const int *mixed_counts(Box *b) { return b->mx->count; }

static int pair_blocks(Box *b) {
  int blocks = (b->n + kMxWarps - 1) / kMxWarps;
  return blocks > 2048 ? 2048 : blocks;
}

int launch_mx_pair_only(Box *b) {
  Mixed &M = *b->mx;
  int n = b->n;
  MxPair P;
  P.n = n;
  P.nt = b->nt;
  P.cap = M.cap;
  P.rc2 = (float)(b->p.rc * b->p.rc);
  P.kappa = (float)b->p.kappa;
  P.c2k = (float)(2.0 * b->p.kappa / sqrt(kPI));
  double qf = kELEC * kELEQ * kELEQ * kNA * 1.0E-3;
  P.qfe = (float)(qf / b->p.epsRF);
  double ron2 = b->p.r_switch > 0.0 ? b->p.r_switch * b->p.r_switch : 0.0;
  double rc2 = b->p.rc * b->p.rc;
  P.ron2 = (float)ron2;
  P.sw_den = ron2 > 0.0 ? (float)((rc2 - ron2) * (rc2 - ron2) * (rc2 - ron2)) : 0.f;
  int blocks = pair_blocks(b);
  size_t shm = sizeof(float) * (kCodes * 6 + b->nt * b->nt * 3);
  k_mx_pair<<<blocks, kMxWarps * 32, shm, b->stream>>>(P, M.pos32, M.type_s, M.perm, M.count, M.ent,
                                                      M.shift_tab, M.lj_tab, M.fix, b->partials);
  FE_LAUNCH_CHECK("k_mx_pair");
  return FE_OK;
}

int launch_mx_spread_only(Box *b) {
  Mixed &M = *b->mx;
  int3 G = make_int3(b->G[0], b->G[1], b->G[2]);
  k_mx_spread<<<(unsigned)((b->K + 127) / 128), 128, 0, b->stream>>>(
      b->order, G, M.pos32, M.sm, b->gcap, b->gbin_count, b->gbin_atoms, M.grid32);
  FE_LAUNCH_CHECK("k_mx_spread");
  return FE_OK;
}

int forces_mixed(Box *b) {
  Mixed &M = *b->mx;
  int n = b->n;
  int rc;
  if ((rc = launch_convert(b))) return rc;
  FE_CUDA(cudaMemsetAsync(M.fix, 0, sizeof(unsigned long long) * 3 * n, b->stream));
  if ((rc = launch_mx_pair_only(b))) return rc;
  if ((rc = launch_reduce(b, b->partials, pair_blocks(b), 4, SC_MX_PAIR, 1.0))) return rc;
  double qf = kELEC * kELEQ * kELEQ * kNA * 1.0E-3;
  // exclusions
  double3 L = make_double3(b->p.L[0], b->p.L[1], b->p.L[2]);
  int xb = (M.nexcl + 255) / 256;
  if (xb > 1024) xb = 1024;
  if (xb < 1) xb = 1;
  k_mx_excl<<<xb, 256, 0, b->stream>>>(M.nexcl, M.excl_ab, M.excl_flag, b->pos_q, b->type, L, b->nt,
                                       M.lj_tab, (float)(b->p.rc * b->p.rc), (float)b->p.kappa,
                                       (float)(2.0 * b->p.kappa / sqrt(kPI)), (float)qf,
                                       (float)b->p.epsRF, M.fix, b->partials);
  FE_LAUNCH_CHECK("k_mx_excl");
  if ((rc = launch_reduce(b, b->partials, xb, 5, SC_MX_EXCL, 1.0))) return rc;
  // bonded
  int tot = b->nbond + b->nbend;
  int bb = (tot + 255) / 256;
  if (bb > 1024) bb = 1024;
  if (bb < 1) bb = 1;
  k_mx_bonded<<<bb, 256, 0, b->stream>>>(b->nbond, b->nbend, L, b->pos_q, b->bond_ab, b->bond_req,
                                         b->bond_k, b->bend_abc, b->bend_t0, b->bend_k, M.fix,
                                         b->partials);
  FE_LAUNCH_CHECK("k_mx_bonded");
  if ((rc = launch_reduce(b, b->partials, bb, 2, SC_BOND, 1.0))) return rc;
  // SPME
  int3 G = make_int3(b->G[0], b->G[1], b->G[2]);
  FE_CUDA(cudaMemsetAsync(b->gbin_count, 0, sizeof(int) * b->K, b->stream));
  k_mx_splines<<<(n + 127) / 128, 128, 0, b->stream>>>(n, b->order, G, L, b->pos_q, M.perm, M.floor3,
                                                       M.sm, M.sd, b->gcap, b->gbin_count,
                                                       b->gbin_atoms, b->status);
  FE_LAUNCH_CHECK("k_mx_splines");
  k_mx_binsort<<<(unsigned)((b->K + 255) / 256), 256, 0, b->stream>>>(b->K, b->gcap, b->gbin_count,
                                                                     b->gbin_atoms);
  FE_LAUNCH_CHECK("k_mx_binsort");
  k_mx_spread<<<(unsigned)((b->K + 127) / 128), 128, 0, b->stream>>>(
      b->order, G, M.pos32, M.sm, b->gcap, b->gbin_count, b->gbin_atoms, M.grid32);
  FE_LAUNCH_CHECK("k_mx_spread");
  cufftResult r = cufftSetStream(M.plan_r2c, b->stream);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftSetStream");
  r = cufftExecR2C(M.plan_r2c, M.grid32, M.grid32k);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftExecR2C");
  int kb = (int)((b->Kh + 255) / 256);
  if (kb > 1024) kb = 1024;
  k_mx_recip<<<kb, 256, 0, b->stream>>>(b->Kh, M.eterm32, M.kw32, M.grid32k, b->partials);
  FE_LAUNCH_CHECK("k_mx_recip");
  if ((rc = launch_reduce(b, b->partials, kb, 1, SC_ENREC, 1.0))) return rc;
  r = cufftSetStream(M.plan_c2r, b->stream);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftSetStream");
  r = cufftExecC2R(M.plan_c2r, M.grid32k, M.grid32);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftExecC2R");
  float3 gl = make_float3((float)(b->G[0] / b->p.L[0]), (float)(b->G[1] / b->p.L[1]),
                          (float)(b->G[2] / b->p.L[2]));
  int gb = (n + 127) / 128;
  if (gb > 1024) gb = 1024;
  float qfe = (float)(qf / b->p.epsRF);
  k_mx_gather<<<gb, 128, 0, b->stream>>>(n, b->order, G, gl, qfe, M.pos32, M.perm, M.floor3, M.sm,
                                         M.sd, M.grid32, M.fix, b->partials);
  FE_LAUNCH_CHECK("k_mx_gather");
  if ((rc = launch_reduce(b, b->partials, gb, 3, SC_FMEAN, 1.0))) return rc;
  k_mx_finalize<<<(3 * n + 255) / 256, 256, 0, b->stream>>>(n, M.fix, b->scal, b->ff);
  FE_LAUNCH_CHECK("k_mx_finalize");
  return launch_mixed_assemble(b);
}

// combine the mixed kernels' sums into the reference's slots, then assemble
__global__ void k_mx_slots(double *__restrict__ s, double erfc_rc_over_rc) {
  if (threadIdx.x != 0) return;
  s[SC_LJ] = s[SC_MX_PAIR + 0] + s[SC_MX_EXCL + 0];
  s[SC_LJS] = s[SC_MX_PAIR + 1] + s[SC_MX_EXCL + 1];
  s[SC_REAL] = s[SC_MX_PAIR + 2] + s[SC_MX_EXCL + 2];
  s[SC_REALS] = (s[SC_MX_PAIR + 3] + s[SC_MX_EXCL + 3]) * erfc_rc_over_rc;
  s[SC_INTRA] = s[SC_MX_EXCL + 4];
}

int launch_mixed_assemble(Box *b) {
  k_mx_slots<<<1, 32, 0, b->stream>>>(b->scal, b->mx->erfc_rc_over_rc);
  FE_LAUNCH_CHECK("k_mx_slots");
  return launch_assemble_energies(b, 1);
}

}  // namespace fe
