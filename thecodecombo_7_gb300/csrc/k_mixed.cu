// k_mixed.cu -- the mixed-precision force engine: FP32 pair and SPME math,
// 64-bit fixed-point force sums (exact, so the result does not depend on the
// order of summation), FP64 integration and energy reductions.
//
// Layout (rebuilt with the list, every nlist steps):
//   * sites are sorted by a cell grid of edge h >= rlist/3 (cells assigned
//     from the same 32-bit fractions as below); perm[s] is the original
//     index of sorted slot s;
//   * every step, posfx[s] = (x, y, z) as unsigned 32-bit fractions of the box
//     length (x/L + 1/2 scaled by 2^32) and the charge: the difference of two
//     coordinates taken in 32-bit integer arithmetic wraps around, which IS the
//     minimum image for |d| < L/2, and converts to FP32 with a relative error
//     of 2^-24 (~2e-7 A at 3 A) -- no image shifts, no cell-relative frames;
//   * the OUTER list is full (both directions, no Newton-3 scatter): row s
//     holds every non-excluded j within rlist, pairs with an LJ term at the
//     front and the rest at the back.  It is built per unit of 8 sorted
//     sites: the candidates near the unit's bounding box are loaded once and
//     tested against all 8 sites;
//   * the pair kernel reads an INNER list (rc + skin, skin 0.8 A): it prunes
//     the outer rows into it while computing forces after every list
//     rebuild and whenever some site has moved skin/2 since the last prune
//     (measured every step against a snapshot of the positions), so every
//     pair within rc is always in it -- the forces are those of the outer
//     list, with ~27 % fewer entries walked;
//   * excluded / 1-4 pairs (xint) are handled with the bonded terms, one
//     thread per molecule when molecules are contiguous runs of sites, else
//     by kernels over the exclusion list (cnonbond_nblist.c:245-263, 416-437
//     semantics);
//   * SPME spreading adds every site's spline contributions to 64-bit
//     fixed-point grid sums with integer reductions (order independent),
//     converted once per step to the FP32 grid for cuFFT; at order 4 the
//     spline weights are computed where they are used (spreading, gather).
// In the pair kernel one warp walks a row (rows handed out from a device
// counter) with coalesced entry loads; the row's FP32 partial sums are added
// over the warp in a fixed butterfly and converted once to the fixed-point
// accumulators (2^32 per kJ/mol/A) -- deterministic.
#include <algorithm>
#include <climits>
#include <cstring>
#include <cmath>
#include <vector>

#include "fe_device.cuh"
#include "fe_df.cuh"
#include "fe_mixed.h"

namespace fe {

constexpr double kFixScale = 4294967296.0;  // 2^32
constexpr float kFixScaleF = 4294967296.0f;
constexpr int kMxWarps = 8;                 // warps per block of the list build
constexpr int kMxMaxCellAtoms = 2048;       // sites per cell a sort block handles

__device__ __forceinline__ long long to_fix(float v) { return __float2ll_rn(v * kFixScaleF); }

// v in [-g, 2g) wrapped into [0, g) without a division
__device__ __forceinline__ int wrap1(int v, int g) { return v < 0 ? v + g : (v >= g ? v - g : v); }

// minimum-image separation from 32-bit fractional coordinates
__device__ __forceinline__ float fx_delta(unsigned a, unsigned b, float scale) {
  return __int2float_rn((int)(a - b)) * scale;
}

// a fixed-point coordinate difference in A, in FP64 (the integer difference
// is exact; sd = L / 2^32 in double)
__device__ __forceinline__ double fx_delta_d(unsigned a, unsigned b, double sd) {
  return (double)(int)(a - b) * sd;
}

// ---------------------------------------------------------------------------
// sorting by cells

// x / L + 1/2 as an unsigned 32-bit fraction (wraps: -L/2 and +L/2 coincide)
__device__ __forceinline__ unsigned frac32(double x, double invL) {
  return (unsigned)(unsigned long long)llrint((x * invL + 0.5) * kFixScale);
}

// cell of each site from the same 32-bit fractions the kernels see, so that
// cell membership and fixed-point coordinates always agree
__device__ __forceinline__ void k_mx_cell_body(VBlk vb_, int n, const double4 *__restrict__ pos, double3 invL, int3 nc,
                          int *__restrict__ cell_of, int *__restrict__ count) {
  int i = vb_.id * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double4 p = pos[i];
  int cx = (int)(((unsigned long long)frac32(p.x, invL.x) * (unsigned)nc.x) >> 32);
  int cy = (int)(((unsigned long long)frac32(p.y, invL.y) * (unsigned)nc.y) >> 32);
  int cz = (int)(((unsigned long long)frac32(p.z, invL.z) * (unsigned)nc.z) >> 32);
  int c = (cx * nc.y + cy) * nc.z + cz;
  cell_of[i] = c;
  atomicAdd(&count[c], 1);
}

__global__ void k_mx_cell(int n, const double4 *__restrict__ pos, double3 invL, int3 nc,
                          int *__restrict__ cell_of, int *__restrict__ count) {
  k_mx_cell_body(vblk_self(), n, pos, invL, nc, cell_of, count);
}

__device__ __forceinline__ void k_mx_fill_body(VBlk vb_, int n, const int *__restrict__ cell_of, const int *__restrict__ start,
                          int *__restrict__ fill, int *__restrict__ perm) {
  int i = vb_.id * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int c = cell_of[i];
  int s = atomicAdd(&fill[c], 1);
  perm[start[c] + s] = i;
}

__global__ void k_mx_fill(int n, const int *__restrict__ cell_of, const int *__restrict__ start,
                          int *__restrict__ fill, int *__restrict__ perm) {
  k_mx_fill_body(vblk_self(), n, cell_of, start, fill, perm);
}

// order each cell's sites by original index (deterministic layout): cells of up
// to 32 sites by rank within one warp, larger ones by a bitonic sort
__device__ __forceinline__ void k_mx_cellsort_body(VBlk vb_, const int *__restrict__ start, int *__restrict__ perm,
                              int *__restrict__ iperm, int *__restrict__ cell_s,
                              const int *__restrict__ type, int *__restrict__ type_s,
                              int *__restrict__ status) {
  __shared__ int buf[kMxMaxCellAtoms];
  int c = vb_.id;
  int s0 = start[c], s1 = start[c + 1];
  int m = s1 - s0;
  if (m > kMxMaxCellAtoms) {
    if (threadIdx.x == 0) atomicOr(status, ST_CELL_OVERFLOW);
    m = kMxMaxCellAtoms;
  }
  if (m <= 32 && blockDim.x == 32) {
    // one site per lane: its rank among the cell's original indices
    const int lane = threadIdx.x;
    int v = lane < m ? perm[s0 + lane] : INT_MAX;
    int rank = 0;
#pragma unroll
    for (int src = 0; src < 32; src++) rank += __shfl_sync(0xffffffffu, v, src) < v ? 1 : 0;
    if (lane < m) {
      perm[s0 + rank] = v;
      iperm[v] = s0 + rank;
      cell_s[s0 + rank] = c;
      type_s[s0 + rank] = type[v];
    }
    return;
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
    type_s[s0 + i] = type[o];
  }
}

__global__ void k_mx_cellsort(const int *__restrict__ start, int *__restrict__ perm,
                              int *__restrict__ iperm, int *__restrict__ cell_s,
                              const int *__restrict__ type, int *__restrict__ type_s,
                              int *__restrict__ status) {
  k_mx_cellsort_body(vblk_self(), start, perm, iperm, cell_s, type, type_s, status);
}

// per step: sorted fixed-point coordinates and charge; with `snap`, also the
// largest squared displacement (A^2) of any site since the inner list was
// last pruned (float bits, atomicMax: non-negative floats order as integers)
__device__ __forceinline__ void k_mx_convert_body(VBlk vb_, int n, const double4 *__restrict__ pos, const int *__restrict__ perm,
                             double3 invL, int4 *__restrict__ posfx,
                             const int4 *__restrict__ snap, float3 sc,
                             unsigned *__restrict__ dmax2) {
  int s = vb_.id * blockDim.x + threadIdx.x;
  float d2 = 0.f;
  if (s < n) {
    double4 p = pos[perm[s]];
    int4 q = make_int4((int)frac32(p.x, invL.x), (int)frac32(p.y, invL.y),
                       (int)frac32(p.z, invL.z), __float_as_int((float)p.w));
    posfx[s] = q;
    if (snap) {
      int4 o = snap[s];
      float dx = fx_delta((unsigned)q.x, (unsigned)o.x, sc.x);
      float dy = fx_delta((unsigned)q.y, (unsigned)o.y, sc.y);
      float dz = fx_delta((unsigned)q.z, (unsigned)o.z, sc.z);
      d2 = dx * dx + dy * dy + dz * dz;
    }
  }
  if (snap) {
#pragma unroll
    for (int o = 16; o; o >>= 1) d2 = fmaxf(d2, __shfl_xor_sync(0xffffffffu, d2, o));
    if ((threadIdx.x & 31) == 0 && d2 > 0.f) atomicMax(dmax2, __float_as_uint(d2));
  }
}

// fix_zero (optional): the force sums to clear for the evaluation that follows
__global__ void k_mx_convert(int n, const double4 *__restrict__ pos, const int *__restrict__ perm,
                             double3 invL, int4 *__restrict__ posfx,
                             const int4 *__restrict__ snap, float3 sc,
                             unsigned *__restrict__ dmax2, unsigned long long *__restrict__ fix_zero) {
  if (fix_zero) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < n) {
      fix_zero[3 * s] = 0ull;
      fix_zero[3 * s + 1] = 0ull;
      fix_zero[3 * s + 2] = 0ull;
    }
  }
  k_mx_convert_body(vblk_self(), n, pos, perm, invL, posfx, snap, sc, dmax2);
}

__device__ __forceinline__ int mx_is_excluded(const int *__restrict__ xs, const int *__restrict__ xp,
                                              int a, int b) {
  for (int p = xs[a]; p < xs[a + 1]; p++)
    if (xp[p] == b) return 1;
  return 0;
}

// ---------------------------------------------------------------------------
// lists

// Appends the candidates that pass to a row: LJ pairs at the front
// (ascending), the rest at the back (descending).
struct RowCursor {
  int nlj, nnl;
};

__device__ __forceinline__ void row_push(bool ok, bool lj, int entry, int lane, int cap,
                                         int *__restrict__ row, RowCursor &rc) {
  unsigned mlj = __ballot_sync(0xffffffffu, ok && lj);
  unsigned mnl = __ballot_sync(0xffffffffu, ok && !lj);
  unsigned lt = (1u << lane) - 1u;
  if (ok) {
    if (lj) {
      int p = rc.nlj + __popc(mlj & lt);
      if (p + rc.nnl < cap) row[p] = entry;
    } else {
      int p = rc.nnl + __popc(mnl & lt);
      if (p + rc.nlj < cap) row[cap - 1 - p] = entry;
    }
  }
  rc.nlj += __popc(mlj);
  rc.nnl += __popc(mnl);
}

__device__ __forceinline__ void row_close(const RowCursor &rc, int cap, int s, int lane,
                                          int *__restrict__ cnt_lj, int *__restrict__ cnt_nl,
                                          int *__restrict__ status) {
  if (lane != 0) return;
  if (rc.nlj + rc.nnl > cap) {
    atomicOr(status, ST_LIST_OVERFLOW);
    int keep = min(rc.nlj, cap);
    cnt_lj[s] = keep;
    cnt_nl[s] = cap - keep;
  } else {
    cnt_lj[s] = rc.nlj;
    cnt_nl[s] = rc.nnl;
  }
}

constexpr int kListUnit = 8;  // consecutive sorted sites one warp lists together
// cells per rlist along each axis: finer cells trim the candidates of a unit
// (rlist/2: ~3000 per unit of 8 water sites, rlist/3: ~2250), coarser ones
// make fewer, longer contiguous ranges; 3 measured fastest of 2, 3, 4
constexpr double kListCellsPerReach = 3.0;
constexpr int kListExcl = 4;  // excluded partners per site handled by lane masks
constexpr int kListBlocksPerSM = 3;  // register budget of the list build (no spills at 74)
static_assert(kListUnit * kListExcl == 32, "one lane per (site, excluded partner)");

__device__ __forceinline__ float warp_fmin(float v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ float warp_fmax(float v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ int wrap_mod(int v, int g) {
  v %= g;
  return v < 0 ? v + g : v;
}

// gap between the interval [lo, hi] and cell c of edge h along one axis
__device__ __forceinline__ float cell_gap(int c, float h, float lo, float hi) {
  return fmaxf(fmaxf(c * h - hi, lo - (c + 1) * h), 0.f);
}

// Appends one chunk's passing candidates to a row without divergent branches.
__device__ __forceinline__ void row_push_bf(bool ok, bool lj, int entry, unsigned lt, int cap,
                                            int *__restrict__ row, RowCursor &rc) {
  unsigned mlj = __ballot_sync(0xffffffffu, ok && lj);
  unsigned mnl = __ballot_sync(0xffffffffu, ok && !lj);
  if ((mlj | mnl) == 0u) return;  // warp-uniform: nothing to append
  int p = lj ? rc.nlj + __popc(mlj & lt) : rc.nnl + __popc(mnl & lt);
  int other = lj ? rc.nnl : rc.nlj;
  int idx = lj ? p : cap - 1 - p;
  if (ok && p + other < cap) row[idx] = entry;
  rc.nlj += __popc(mlj);
  rc.nnl += __popc(mnl);
}

// One chunk of candidates (one per lane) against every site of the unit.
// FAST: the FP32 frame of the unit's first site covers every pair, the
// sites have at most kListExcl excluded partners and nt <= 32; otherwise
// the exact fixed-point differences, the exclusion lists and the type table
// are used.  Sites past the end of the unit carry NaN offsets: no pair passes.
template <bool FAST>
__device__ __forceinline__ void list_chunk(
    int j, int js, int4 pj, float fjx, float fjy, float fjz, int tj, unsigned mj, unsigned ebit,
    unsigned lanebit, unsigned lt, const float4 (&site)[kListUnit], const int4 (&spk)[kListUnit],
    float3 sc, float rl2, int nt, const unsigned char *__restrict__ lj_on,
    const int *__restrict__ xs, const int *__restrict__ xp, int ok_orig, int oj, int cap,
    int *__restrict__ row0, RowCursor (&rc)[kListUnit]) {
#pragma unroll
  for (int k = 0; k < kListUnit; k++) {
    unsigned exm = __shfl_sync(0xffffffffu, ebit, 4 * k);
    float4 si = site[k];
    int tik = __float_as_int(si.w);
    float dx, dy, dz;
    if (FAST) {
      dx = fjx - si.x;
      dy = fjy - si.y;
      dz = fjz - si.z;
    } else {
      int4 pik = spk[k];
      dx = fx_delta((unsigned)pj.x, (unsigned)pik.x, sc.x);
      dy = fx_delta((unsigned)pj.y, (unsigned)pik.y, sc.y);
      dz = fx_delta((unsigned)pj.z, (unsigned)pik.z, sc.z);
      if (si.x != si.x) dx = si.x;  // padding site
    }
    float r2 = dx * dx + dy * dy + dz * dz;
    bool ok = r2 < rl2 && js != k && (exm & lanebit) == 0u;
    bool lj;
    if (FAST) {
      lj = ((mj >> tik) & 1u) != 0u;
    } else {
      int oi = __shfl_sync(0xffffffffu, ok_orig, k);
      if (ok) ok = !mx_is_excluded(xs, xp, oi, oj);
      lj = lj_on[tik * nt + tj] != 0;
    }
    row_push_bf(ok, lj, j, lt, cap, row0 + (size_t)k * cap, rc[k]);
  }
}

// Outer list: one warp per UNIT of kListUnit consecutive sorted sites (mostly
// one or two neighbouring cells).  The warp takes the bounding box of the
// unit's sites (minimum-image offsets from its first site, in A), walks the
// cell columns within reach of it -- 32 columns at a time, one per lane, each
// with the z cells within rlist of the box as one or two contiguous sorted
// ranges -- and packs those ranges into full 32-lane chunks of candidates.
// Every candidate is loaded once and tested against all sites of the unit.
// Excluded partners are turned into per-chunk lane masks (lane 4k+q owns the
// q-th partner of site k and locates it among the candidates once per column
// batch), so the per-pair test is a distance, a mask bit and a ballot.
// Rows come out in a fixed (column, slot) order: deterministic.
__device__ __forceinline__ void k_mx_list_body(VBlk vb_, int n, const int4 *__restrict__ posfx, const int *__restrict__ perm,
          const int *__restrict__ iperm, const int *__restrict__ cell_s,
          const int *__restrict__ type_s, const int *__restrict__ cstart, int3 nc, float3 sc,
          float3 Lf, float rlist, int nt, const unsigned *__restrict__ lj_row,
          const unsigned char *__restrict__ lj_on, const int *__restrict__ xs,
          const int *__restrict__ xp, int cap, int *__restrict__ cnt_lj,
          int *__restrict__ cnt_nl, int *__restrict__ ent, int *__restrict__ status) {
  const unsigned full = 0xffffffffu;
  __shared__ float4 s_site[kMxWarps][kListUnit];
  __shared__ int4 s_pk[kMxWarps][kListUnit];
  int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  unsigned lanebit = 1u << lane, lt = lanebit - 1u;
  float rl2 = rlist * rlist;
  // reach of the cell walk: rlist plus a margin for the FP32 frame's rounding
  float ra = rlist + 1e-3f + 4e-6f * fmaxf(Lf.x, fmaxf(Lf.y, Lf.z));
  float ra2 = ra * ra;
  float3 hc = make_float3(Lf.x / nc.x, Lf.y / nc.y, Lf.z / nc.z);
  float3 ihc = make_float3(nc.x / Lf.x, nc.y / Lf.y, nc.z / Lf.z);
  int nunits = (n + kListUnit - 1) / kListUnit;
  for (int u = vb_.id * kMxWarps + wib; u < nunits; u += vb_.n * kMxWarps) {
    int s0 = u * kListUnit, nk = min(kListUnit, n - s0);
    int sl = s0 + min(lane, nk - 1);  // lanes past the unit repeat its last site
    int4 pk = posfx[sl];
    int tk = type_s[sl];
    int ok_orig = perm[sl];
    unsigned r0x = __shfl_sync(full, (unsigned)pk.x, 0), r0y = __shfl_sync(full, (unsigned)pk.y, 0),
             r0z = __shfl_sync(full, (unsigned)pk.z, 0);
    float ox = fx_delta((unsigned)pk.x, r0x, sc.x), oy = fx_delta((unsigned)pk.y, r0y, sc.y),
          oz = fx_delta((unsigned)pk.z, r0z, sc.z);
    float lox = warp_fmin(ox), hix = warp_fmax(ox), loy = warp_fmin(oy), hiy = warp_fmax(oy),
          loz = warp_fmin(oz), hiz = warp_fmax(oz);
    // the FP32 frame of the first site gives the minimum image of every pair
    // within reach when offsets + reach stay under half the box
    bool frame = fmaxf(-lox, hix) + ra < 0.5f * Lf.x && fmaxf(-loy, hiy) + ra < 0.5f * Lf.y &&
                 fmaxf(-loz, hiz) + ra < 0.5f * Lf.z;
    // the unit's sites for the per-pair tests: offsets and type, and the
    // fixed-point coordinates for units the FP32 frame does not cover
    __syncwarp();
    if (lane < kListUnit) {
      float pad = lane < nk ? 0.f : __int_as_float(0x7fc00000);  // NaN: no pair passes
      s_site[wib][lane] = make_float4(ox + pad, oy + pad, oz + pad, __int_as_float(tk));
      s_pk[wib][lane] = pk;
    }
    __syncwarp();
    // lane 4k+q: q-th excluded partner of site k (sorted slot, -1 if none)
    int ek = lane >> 2, eq = lane & 3, exs = -1;
    bool many_l = false;
    if (ek < nk) {
      int o = perm[s0 + ek];
      int a = xs[o], m = xs[o + 1] - a;
      if (eq < m) exs = iperm[xp[a + eq]];
      many_l = eq == 0 && m > kListExcl;
    }
    bool fast = frame && lj_row != nullptr && !__any_sync(full, many_l);
    int *row0 = ent + (size_t)s0 * cap;
    int ecx = 0, ecy = 0;
    if (exs >= 0) {
      int c = cell_s[exs];
      ecy = (c / nc.z) % nc.y;
      ecx = c / (nc.z * nc.y);
    }
    // cell window of the unit, unwrapped (the whole axis when it wraps onto itself)
    float X0 = __uint2float_rn(r0x) * sc.x, Y0 = __uint2float_rn(r0y) * sc.y,
          Z0 = __uint2float_rn(r0z) * sc.z;
    float Xlo = X0 + lox, Xhi = X0 + hix, Ylo = Y0 + loy, Yhi = Y0 + hiy, Zlo = Z0 + loz,
          Zhi = Z0 + hiz;
    int xa = __float2int_rd((Xlo - ra) * ihc.x), xb = __float2int_rd((Xhi + ra) * ihc.x);
    int ya = __float2int_rd((Ylo - ra) * ihc.y), yb = __float2int_rd((Yhi + ra) * ihc.y);
    bool allx = xb - xa + 1 >= nc.x, ally = yb - ya + 1 >= nc.y;
    if (allx) {
      xa = 0;
      xb = nc.x - 1;
    }
    if (ally) {
      ya = 0;
      yb = nc.y - 1;
    }
    int nx = xb - xa + 1, ny = yb - ya + 1, ncol = nx * ny;
    // column of the excluded partner within the window (-1: outside)
    int eqcol = -1;
    if (exs >= 0) {
      int dx = wrap_mod(ecx - xa, nc.x), dy = wrap_mod(ecy - ya, nc.y);
      if (dx < nx && dy < ny) eqcol = dx * ny + dy;
    }
    RowCursor rc[kListUnit];
#pragma unroll
    for (int k = 0; k < kListUnit; k++) rc[k] = {0, 0};
    for (int q0 = 0; q0 < ncol; q0 += 32) {
      int q = q0 + lane;
      int a0 = 0, la = 0, b0 = 0, lb = 0;
      if (q < ncol) {
        int x = xa + q / ny, y = ya + q % ny;
        float gx = allx ? 0.f : cell_gap(x, hc.x, Xlo, Xhi);
        float gy = ally ? 0.f : cell_gap(y, hc.y, Ylo, Yhi);
        float g2 = gx * gx + gy * gy;
        if (g2 < ra2) {
          float rho = sqrtf(ra2 - g2);
          int za = __float2int_rd((Zlo - rho) * ihc.z), zb = __float2int_rd((Zhi + rho) * ihc.z);
          const int *cs = cstart + (wrap_mod(x, nc.x) * nc.y + wrap_mod(y, nc.y)) * nc.z;
          if (zb - za + 1 >= nc.z) {
            a0 = cs[0];
            la = cs[nc.z] - a0;
          } else {
            int zaw = wrap_mod(za, nc.z), zbw = wrap_mod(zb, nc.z);
            a0 = cs[zaw];
            if (zaw <= zbw) {
              la = cs[zbw + 1] - a0;
            } else {
              la = cs[nc.z] - a0;
              b0 = cs[0];
              lb = cs[zbw + 1] - b0;
            }
          }
        }
      }
      // exclusive prefix of the columns' candidate counts
      int len = la + lb, incl = len;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(full, incl, o);
        if (lane >= o) incl += t;
      }
      int P = incl - len, T = __shfl_sync(full, incl, 31);
      // virtual index of this lane's excluded partner among the batch's candidates
      bool here = eqcol >= q0 && eqcol < q0 + 32;
      int src = here ? eqcol - q0 : 0;
      int eP = __shfl_sync(full, P, src), ea0 = __shfl_sync(full, a0, src),
          ela = __shfl_sync(full, la, src), eb0 = __shfl_sync(full, b0, src),
          elb = __shfl_sync(full, lb, src);
      int ve = -1;
      if (here) {
        if (exs >= ea0 && exs < ea0 + ela) ve = eP + exs - ea0;
        else if (exs >= eb0 && exs < eb0 + elb) ve = eP + ela + exs - eb0;
      }
      for (int vb = 0; vb < T; vb += 32) {
        int v = vb + lane;
        bool valid = v < T;
        int c = 0;
#pragma unroll
        for (int st = 16; st; st >>= 1) {
          int Pt = __shfl_sync(full, P, c + st);
          if (Pt <= v) c += st;
        }
        int Pc = __shfl_sync(full, P, c), a0c = __shfl_sync(full, a0, c),
            lac = __shfl_sync(full, la, c), b0c = __shfl_sync(full, b0, c);
        int off = v - Pc;
        int j = off < lac ? a0c + off : b0c + (off - lac);
        if (!valid) j = s0;
        int4 pj = posfx[j];
        int tj = type_s[j];
        float fjx = fx_delta((unsigned)pj.x, r0x, sc.x), fjy = fx_delta((unsigned)pj.y, r0y, sc.y),
              fjz = fx_delta((unsigned)pj.z, r0z, sc.z);
        unsigned te = (unsigned)(ve - vb);
        unsigned ebit = (ve >= 0 && te < 32u) ? 1u << te : 0u;
        ebit |= __shfl_xor_sync(full, ebit, 1);
        ebit |= __shfl_xor_sync(full, ebit, 2);
        int js = valid ? j - s0 : -1;  // this lane's candidate is site js of the unit
        if (fast) {
          list_chunk<true>(j, js, pj, fjx, fjy, fjz, tj, lj_row[tj], ebit, lanebit, lt,
                           s_site[wib], s_pk[wib], sc, valid ? rl2 : -1.f, nt, lj_on, xs, xp,
                           ok_orig, 0, cap, row0, rc);
        } else {
          list_chunk<false>(j, js, pj, fjx, fjy, fjz, tj, 0u, ebit, lanebit, lt, s_site[wib],
                            s_pk[wib], sc, valid ? rl2 : -1.f, nt, lj_on, xs, xp, ok_orig,
                            perm[j], cap, row0, rc);
        }
      }
    }
#pragma unroll
    for (int k = 0; k < kListUnit; k++)
      if (k < nk) row_close(rc[k], cap, s0 + k, lane - k, cnt_lj, cnt_nl, status);
  }
}

__global__ void __launch_bounds__(kMxWarps * 32, kListBlocksPerSM)
k_mx_list(int n, const int4 *__restrict__ posfx, const int *__restrict__ perm,
          const int *__restrict__ iperm, const int *__restrict__ cell_s,
          const int *__restrict__ type_s, const int *__restrict__ cstart, int3 nc, float3 sc,
          float3 Lf, float rlist, int nt, const unsigned *__restrict__ lj_row,
          const unsigned char *__restrict__ lj_on, const int *__restrict__ xs,
          const int *__restrict__ xp, int cap, int *__restrict__ cnt_lj,
          int *__restrict__ cnt_nl, int *__restrict__ ent, int *__restrict__ status) {
  k_mx_list_body(vblk_self(), n, posfx, perm, iperm, cell_s, type_s, cstart, nc, sc, Lf, rlist, nt, lj_row, lj_on, xs, xp, cap, cnt_lj, cnt_nl, ent, status);
}


// ---------------------------------------------------------------------------
// pair kernel

constexpr int kPairGrab = 2;  // rows a warp takes from the row counter at a time

struct MxPair {
  int n, nt, cap;
  float rc2, kappa, c2k, qfe;  // c2k = 2 kappa / sqrt(pi); qfe = QFACTOR / epsRF
  float ron2, inv_sw_den;  // switch start^2 and 1 / (rc^2 - ron^2)^3
  float3 sc;                   // L / 2^32 per axis
  int cubic;                   // Lx = Ly = Lz: distances formed in lattice units
  float s2;                    // sc.x^2 (cubic boxes)
  // inner list: radius^2 (rc + skin)^2, and the squared displacement that
  // forces a prune ((skin / 2)^2, less a rounding margin)
  float rp2, thresh2;
  int inner_on;                // 0: rows always come from the outer list
};


// the reference's erfc (ewald.c:817-836, Numerical Recipes "erfcc") in FP32;
// ex = exp(-z^2) is shared with the force term
__device__ __forceinline__ float erfc_nr_f(float z, float ex) {
  float t = __fdividef(1.0f, 1.0f + 0.5f * z);
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

// 2^x by the SFU's ex2.approx (PTX ISA): the exponential of the pair terms
__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
constexpr float kLog2e = 1.44269504f;

// the same fit as erfc_nr_f, erfc(z) = t exp(-z^2 + P(t)), with the two
// exponents merged: t 2^(P(t) log2 e + q2), q2 = -z^2 log2 e given
__device__ __forceinline__ float erfc_nr_q(float z, float q2) {
  float t = __fdividef(1.0f, fmaf(0.5f, z, 1.0f));
  float p = fmaf(t, 0.17087277f, -0.82215223f);
  p = fmaf(t, p, 1.48851587f);
  p = fmaf(t, p, -1.13520398f);
  p = fmaf(t, p, 0.27886807f);
  p = fmaf(t, p, -0.18628806f);
  p = fmaf(t, p, 0.09678418f);
  p = fmaf(t, p, 0.37409196f);
  p = fmaf(t, p, 1.00002368f);
  p = fmaf(t, p, -1.26551223f);
  return t * ex2_approx(fmaf(p, kLog2e, q2));
}

struct PairAcc {
  float fx, fy, fz, e_lj, e_ljs, e_real, qsum;
};

// one list entry j of row i: Ewald real space always, LJ when WITH_LJ
// one pair with its separation (dx, dy, dz), r2 already formed
template <bool WITH_LJ>
__device__ __forceinline__ void mx_pair_core(const MxPair &P, float qi, int j, int4 pj, float dx,
                                             float dy, float dz, float r2,
                                             const float *__restrict__ ljrow,
                                             const int *__restrict__ type_s, PairAcc &a) {
  if (r2 > P.rc2) return;
  float rinv = rsqrtf(r2);
  float r = r2 * rinv;
  float rinv2 = rinv * rinv;
  float qq = qi * __int_as_float(pj.w);
  float qr = qq * rinv;
  float kr = P.kappa * r;
  float q2 = (kr * -kLog2e) * kr;
  float ex = ex2_approx(q2);  // exp(-(kappa r)^2)
  float erfckr = erfc_nr_q(kr, q2);
  float F = qr * rinv2 * fmaf(P.c2k * r, ex, erfckr);
  a.e_real = fmaf(qr, erfckr, a.e_real);
  a.qsum += qq;
  if (WITH_LJ) {
    const float *lj = ljrow + type_s[j] * 3;
    float eps = lj[0];
    float sr2 = lj[1] * rinv2;
    float sr6 = sr2 * sr2 * sr2;
    float sr12 = sr6 * sr6;
    float flj = 12.f * eps * rinv2 * (sr12 - sr6);
    float elj = eps * (sr12 - 2.f * sr6);
    if (P.ron2 > 0.f) {
      if (r2 > P.ron2) {
        float c = P.rc2 - r2;
        float sw = c * c * (P.rc2 + 2.f * r2 - 3.f * P.ron2) * P.inv_sw_den;
        float dsw = 12.f * c * (r2 - P.ron2) * P.inv_sw_den;
        flj = flj * sw + elj * dsw;
        elj = elj * sw;
      }
    } else {
      a.e_ljs = fmaf(eps, lj[2], a.e_ljs);
    }
    F += flj;
    a.e_lj += elj;
  }
  a.fx = fmaf(F, dx, a.fx);
  a.fy = fmaf(F, dy, a.fy);
  a.fz = fmaf(F, dz, a.fz);
}

// the separation of sites pi and pj: in A, or (CUBIC) in lattice units of
// L / 2^32 with r2 in A^2 -- the force sums are then scaled once per row
template <bool CUBIC>
__device__ __forceinline__ float mx_sep(const MxPair &P, int4 pi, int4 pj, float &dx, float &dy,
                                        float &dz) {
  if (CUBIC) {
    dx = __int2float_rn((int)((unsigned)pi.x - (unsigned)pj.x));
    dy = __int2float_rn((int)((unsigned)pi.y - (unsigned)pj.y));
    dz = __int2float_rn((int)((unsigned)pi.z - (unsigned)pj.z));
    return P.s2 * fmaf(dx, dx, fmaf(dy, dy, dz * dz));
  }
  dx = fx_delta((unsigned)pi.x, (unsigned)pj.x, P.sc.x);
  dy = fx_delta((unsigned)pi.y, (unsigned)pj.y, P.sc.y);
  dz = fx_delta((unsigned)pi.z, (unsigned)pj.z, P.sc.z);
  return dx * dx + dy * dy + dz * dz;
}

template <bool WITH_LJ, bool CUBIC>
__device__ __forceinline__ void mx_pair_one(const MxPair &P, int4 pi, float qi, int j, int4 pj,
                                            const float *__restrict__ ljrow,
                                            const int *__restrict__ type_s, PairAcc &a) {
  float dx, dy, dz;
  float r2 = mx_sep<CUBIC>(P, pi, pj, dx, dy, dz);
  mx_pair_core<WITH_LJ>(P, qi, j, pj, dx, dy, dz, r2, ljrow, type_s, a);
}

// Walks entries b0 + lane, b0 + lane + 32, ... of a row with a two-deep
// software pipeline: the entry two iterations ahead and the j position one
// iteration ahead are in flight while the current pair is computed.  The loop
// body covers two entries, so the in-flight values change registers without
// copies.
template <bool WITH_LJ, bool CUBIC>
__device__ __forceinline__ void mx_segment(const MxPair &P, int4 pi, float qi,
                                           const int *__restrict__ row, int b0, int b1, int lane,
                                           const int4 *__restrict__ posfx,
                                           const float *__restrict__ ljrow,
                                           const int *__restrict__ type_s, PairAcc &a) {
  int i = b0 + lane;
  if (i >= b1) return;
  int e0 = row[i];
  int e1 = i + 32 < b1 ? row[i + 32] : -1;
  int4 p0 = posfx[e0];
  while (true) {
    int e2 = (e1 >= 0 && i + 64 < b1) ? row[i + 64] : -1;
    int4 p1 = make_int4(0, 0, 0, 0);
    if (e1 >= 0) p1 = posfx[e1];
    mx_pair_one<WITH_LJ, CUBIC>(P, pi, qi, e0, p0, ljrow, type_s, a);
    if (e1 < 0) break;
    int e3 = (e2 >= 0 && i + 96 < b1) ? row[i + 96] : -1;
    if (e2 >= 0) p0 = posfx[e2];
    mx_pair_one<WITH_LJ, CUBIC>(P, pi, qi, e1, p1, ljrow, type_s, a);
    if (e2 < 0) break;
    e0 = e2;
    e1 = e3;
    i += 64;
  }
}

// The same walk over an OUTER row while writing the inner row: entries
// within rc + skin are appended to `irow` (same LJ-front / rest-back layout).
// Each lane visits the same entries in the same order as mx_segment (and the
// same two-deep pipeline), but the loop runs the warp's common trip count so
// that the appends can use warp ballots; lanes past the row end compute
// nothing and append nothing.
template <bool WITH_LJ, bool CUBIC>
__device__ __forceinline__ void mx_segment_prune(const MxPair &P, int4 pi, float qi,
                                                 const int *__restrict__ row, int b0, int b1,
                                                 int lane, unsigned lt,
                                                 const int4 *__restrict__ posfx,
                                                 const float *__restrict__ ljrow,
                                                 const int *__restrict__ type_s,
                                                 int *__restrict__ irow, RowCursor &rc,
                                                 PairAcc &a) {
  int i = b0 + lane;
  int e_cur = i < b1 ? row[i] : 0;
  int e_nxt = i + 32 < b1 ? row[i + 32] : 0;
  int4 p_cur = posfx[e_cur];
  for (int base = b0; base < b1; base += 32, i += 32) {
    int e_nn = i + 64 < b1 ? row[i + 64] : 0;
    int4 p_nxt = posfx[e_nxt];
    bool v = i < b1;
    float dx, dy, dz;
    float r2 = mx_sep<CUBIC>(P, pi, p_cur, dx, dy, dz);
    if (v) mx_pair_core<WITH_LJ>(P, qi, e_cur, p_cur, dx, dy, dz, r2, ljrow, type_s, a);
    row_push_bf(v && r2 < P.rp2, WITH_LJ, e_cur, lt, P.cap, irow, rc);
    e_cur = e_nxt;
    p_cur = p_nxt;
    e_nxt = e_nn;
  }
}

// NW warps per block and a register budget of 65536 / (RW * 32) per thread
// for RW resident warps per SM (48: 40 registers, 32: 64 registers): a
// launch shape chosen by mixed_autotune.
// Two variants run one after the other every evaluation and read the same
// device state.  PRUNE walks the outer rows, rewrites the inner ones and
// adds its block sums to the energy accumulators; it returns at once when no
// prune is due.  The plain variant walks the inner rows (nothing when the
// PRUNE variant ran), finishes the energies and clears the state.
template <int NW, int RW, bool PRUNE>
__device__ __forceinline__ void k_mx_pair_body(VBlk vb_, MxPair P, const int4 *__restrict__ posfx, const int *__restrict__ type_s,
          const int *__restrict__ perm, const int *__restrict__ cnt_lj,
          const int *__restrict__ cnt_nl, const int *__restrict__ ent,
          int *__restrict__ icnt_lj, int *__restrict__ icnt_nl, int *__restrict__ ient,
          int4 *__restrict__ snap, MxPruneState *__restrict__ ps,
          const float *__restrict__ lj_tab, unsigned long long *__restrict__ fix,
          unsigned long long *__restrict__ facc, unsigned *__restrict__ ticket,
          double *__restrict__ out, int *__restrict__ status) {
  // prune (read the outer list, rewrite the inner one) after a list rebuild
  // or when some site has moved half the skin since the last prune; between
  // prunes no pair can come within rc from beyond rc + skin
  const bool prune = !P.inner_on || ps->need != 0 || __uint_as_float(ps->dmax2) >= P.thresh2;
  if (PRUNE && !prune) return;
  const bool work = PRUNE || !prune;
  extern __shared__ float s_lj[];  // nt*nt*3: eps, sig^2, shift constant
  for (int i = threadIdx.x; i < P.nt * P.nt * 3; i += blockDim.x) s_lj[i] = lj_tab[i];
  __syncthreads();
  int lane = threadIdx.x & 31;
  unsigned lt = (1u << lane) - 1u;
  if (PRUNE && P.inner_on && vb_.id == 0 && threadIdx.x == 0) atomicAdd(&ps->prunes, 1ull);
  const int *rlj = PRUNE ? cnt_lj : icnt_lj;
  const int *rnl = PRUNE ? cnt_nl : icnt_nl;
  const int *rent = PRUNE ? ent : ient;
  PairAcc a;
  // energies per row in FP32, then exact fixed-point sums across rows (kept
  // in shared memory by each warp's lane 0): the totals do not depend on how
  // rows are spread over warps (the launch shape)
  __shared__ long long weq[NW][4];
  if (lane < 4) weq[threadIdx.x >> 5][lane] = 0;
  __syncwarp();
  // rows are taken kPairGrab at a time from a device counter: warps finish
  // together whatever their rows' lengths (the per-row energies are exact
  // fixed-point sums, so the results do not depend on which warp took a row)
  while (work) {
    int s0 = 0;
    if (lane == 0) s0 = atomicAdd(&ps->next_row, kPairGrab);
    s0 = __shfl_sync(0xffffffffu, s0, 0);
    if (s0 >= P.n) break;
    const int s1 = min(s0 + kPairGrab, P.n);
    for (int s = s0; s < s1; s++) {
    int4 pi = posfx[s];
    float qi = __int_as_float(pi.w) * P.qfe;
    const float *ljrow = s_lj + type_s[s] * P.nt * 3;
    const int *row = rent + (size_t)s * P.cap;
    a.fx = a.fy = a.fz = 0.f;
    a.e_lj = a.e_ljs = a.e_real = a.qsum = 0.f;
    if (PRUNE && P.inner_on) {
      int *irow = ient + (size_t)s * P.cap;
      RowCursor rc = {0, 0};
      if (P.cubic) {
        mx_segment_prune<true, true>(P, pi, qi, row, 0, rlj[s], lane, lt, posfx, ljrow, type_s,
                                     irow, rc, a);
        mx_segment_prune<false, true>(P, pi, qi, row, P.cap - rnl[s], P.cap, lane, lt, posfx,
                                      ljrow, type_s, irow, rc, a);
      } else {
        mx_segment_prune<true, false>(P, pi, qi, row, 0, rlj[s], lane, lt, posfx, ljrow, type_s,
                                      irow, rc, a);
        mx_segment_prune<false, false>(P, pi, qi, row, P.cap - rnl[s], P.cap, lane, lt, posfx,
                                       ljrow, type_s, irow, rc, a);
      }
      row_close(rc, P.cap, s, lane, icnt_lj, icnt_nl, status);
      if (lane == 0) snap[s] = pi;
    } else {
      if (P.cubic) {
        mx_segment<true, true>(P, pi, qi, row, 0, rlj[s], lane, posfx, ljrow, type_s, a);
        mx_segment<false, true>(P, pi, qi, row, P.cap - rnl[s], P.cap, lane, posfx, ljrow,
                                type_s, a);
      } else {
        mx_segment<true, false>(P, pi, qi, row, 0, rlj[s], lane, posfx, ljrow, type_s, a);
        mx_segment<false, false>(P, pi, qi, row, P.cap - rnl[s], P.cap, lane, posfx, ljrow,
                                 type_s, a);
      }
    }
    // the row's force: a fixed butterfly of FP32 partial sums (deterministic),
    // converted once to the fixed-point accumulators
    float fx = a.fx, fy = a.fy, fz = a.fz;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      fx += __shfl_xor_sync(0xffffffffu, fx, o);
      fy += __shfl_xor_sync(0xffffffffu, fy, o);
      fz += __shfl_xor_sync(0xffffffffu, fz, o);
    }
    if (P.cubic) {  // lattice units to A
      fx *= P.sc.x;
      fy *= P.sc.x;
      fz *= P.sc.x;
    }
    // every pair is visited from both ends: half of each row's energy
    float e[4] = {0.5f * a.e_lj, 0.5f * a.e_ljs, 0.5f * a.e_real, 0.5f * a.qsum};
#pragma unroll
    for (int t = 0; t < 4; t++) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) e[t] += __shfl_xor_sync(0xffffffffu, e[t], o);
    }
    if (lane == 0) {
      int oi = perm[s];
      atomicAdd(&fix[3 * oi], (unsigned long long)to_fix(fx));
      atomicAdd(&fix[3 * oi + 1], (unsigned long long)to_fix(fy));
      atomicAdd(&fix[3 * oi + 2], (unsigned long long)to_fix(fz));
#pragma unroll
      for (int t = 0; t < 4; t++) weq[threadIdx.x >> 5][t] += to_fix(e[t]);
    }
    }
  }
  __syncwarp();
  long long eq[4] = {0, 0, 0, 0};
  if (lane == 0)
#pragma unroll
    for (int t = 0; t < 4; t++) eq[t] = weq[threadIdx.x >> 5][t];
  if (PRUNE) {
    block_fix_add<4>(eq, 32, facc);
    return;
  }
  // the last block: both variants have read the prune state and every row
  // has been taken, clear both
  if (block_fix_final<4>(eq, 32, facc, ticket, out, vb_) && threadIdx.x == 0) {
    ps->need = 0;
    ps->dmax2 = 0u;
    ps->next_row = 0;
  }
}

template <int NW, int RW, bool PRUNE>
__global__ void __launch_bounds__(NW * 32, RW / NW)
k_mx_pair(MxPair P, const int4 *__restrict__ posfx, const int *__restrict__ type_s,
          const int *__restrict__ perm, const int *__restrict__ cnt_lj,
          const int *__restrict__ cnt_nl, const int *__restrict__ ent,
          int *__restrict__ icnt_lj, int *__restrict__ icnt_nl, int *__restrict__ ient,
          int4 *__restrict__ snap, MxPruneState *__restrict__ ps,
          const float *__restrict__ lj_tab, unsigned long long *__restrict__ fix,
          unsigned long long *__restrict__ facc, unsigned *__restrict__ ticket,
          double *__restrict__ out, int *__restrict__ status) {
  k_mx_pair_body<NW, RW, PRUNE>(vblk_self(), P, posfx, type_s, perm, cnt_lj, cnt_nl, ent, icnt_lj, icnt_nl, ient, snap, ps, lj_tab, fix, facc, ticket, out, status);
}

// qq (1 - erfc(kappa r)) / r of an excluded pair in double-float, from the
// exact integer separation of the 32-bit fractional coordinates and the FP64
// charges (the term eewald_intra of cnonbond_nblist.c:416-437)
__device__ __forceinline__ dfl intra_energy_df(const DfIntra &D, int4 A, int4 B, double qa,
                                               double qb, float qscale,
                                               const float2 *__restrict__ exptab) {
  dfl r2 = {0.f, 0.f};
  int dd[3] = {(int)((unsigned)A.x - (unsigned)B.x), (int)((unsigned)A.y - (unsigned)B.y),
               (int)((unsigned)A.z - (unsigned)B.z)};
#pragma unroll
  for (int c = 0; c < 3; c++) {
    dfl d = df_mul(df_from_ll((long long)dd[c]), {D.sl[c].x, D.sl[c].y});
    r2 = df_add(r2, df_mul(d, d));
  }
  dfl r = df_sqrt(r2);
  dfl z = df_mul(r, {D.kappa.x, D.kappa.y});
  dfl erf = df_add({1.0f, 0.0f}, df_neg(df_erfc_nr(z, D.C, exptab)));
  dfl qq = df_mul(df_mul(df_from_double(qa), df_from_double(qb)), {D.qf.x, D.qf.y});
  qq = df_mul_f(qq, qscale);
  return df_mul(df_mul(qq, erf), df_recip(r));
}

__device__ __forceinline__ long long df_to_fixed(dfl v, int shift) {
  return to_fixed(v.hi, shift) + to_fixed(v.lo, shift);
}

// excluded and 1-4 pairs (xint), cnonbond_nblist.c:245-263 and 416-437:
// inside rc an excluded pair contributes no LJ and no real-space term but the
// intra correction -qq (1 - erfc(kr)) / r; a 1-4 pair gets LJ, real space
// scaled by E14FAC and the correction with (1 - E14FAC)
__global__ void k_mx_excl(int nexcl, const int *__restrict__ ab, const int *__restrict__ flag,
                          const int4 *__restrict__ posfx, const int *__restrict__ iperm,
                          const int *__restrict__ type, float3 sL, int nt, const float *__restrict__ lj_tab, float rc2, float kappa,
                          float c2k, float qf, float epsRF, const double4 *__restrict__ pos_q,
                          const float2 *__restrict__ exptab, DfIntra D,
                          unsigned long long *__restrict__ fix,
                          unsigned long long *__restrict__ facc, unsigned *__restrict__ ticket,
                          double *__restrict__ out) {
  float e_lj = 0.f, e_ljs = 0.f, e_real = 0.f, qsum = 0.f;
  long long q_intra = 0;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nexcl; t += gridDim.x * blockDim.x) {
    int a = ab[2 * t], b = ab[2 * t + 1], xf = flag[t];
    if (xf == 0) continue;
    int4 A = posfx[iperm[a]], B = posfx[iperm[b]];
    float dx = fx_delta((unsigned)A.x, (unsigned)B.x, sL.x);
    float dy = fx_delta((unsigned)A.y, (unsigned)B.y, sL.y);
    float dz = fx_delta((unsigned)A.z, (unsigned)B.z, sL.z);
    float r2 = dx * dx + dy * dy + dz * dz;
    if (r2 > rc2) continue;
    float rinv = rsqrtf(r2), r = r2 * rinv, rinv2 = rinv * rinv;
    float kr = kappa * r;
    float ex = __expf(-kr * kr);
    float erfckr = erfc_nr_f(kr, ex);
    float qqab = __int_as_float(A.w) * __int_as_float(B.w) * qf;
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
    q_intra += df_to_fixed(intra_energy_df(D, A, B, pos_q[a].w, pos_q[b].w,
                                           xf == 4 ? (float)(1.0 - kE14FAC) : 1.f, exptab),
                           32);
    F -= qcorr * rinv * rinv2 * (erfkr - c2k * r * ex);
    long long fxq = to_fix(F * dx), fyq = to_fix(F * dy), fzq = to_fix(F * dz);
    atomicAdd(&fix[3 * a], (unsigned long long)fxq);
    atomicAdd(&fix[3 * a + 1], (unsigned long long)fyq);
    atomicAdd(&fix[3 * a + 2], (unsigned long long)fzq);
    atomicAdd(&fix[3 * b], (unsigned long long)(-fxq));
    atomicAdd(&fix[3 * b + 1], (unsigned long long)(-fyq));
    atomicAdd(&fix[3 * b + 2], (unsigned long long)(-fzq));
  }
  long long v[5] = {to_fixed(e_lj, 32), to_fixed(e_ljs, 32), to_fixed(e_real, 32),
                    to_fixed(qsum, 32), q_intra};
  block_fix_final<5>(v, 32, facc, ticket, out);
}

// bonded terms from the fixed-point coordinates (cbond.c, cbend.c): the
// stretch, the angle and the energies in FP64 as in intra_bond / intra_bend,
// the forces in FP32 (sd: the length scale L / 2^32 in FP64)
__global__ void k_mx_bonded(int nbond, int nbend, float3 sL, double3 sd,
                            const int4 *__restrict__ posfx,
                            const int *__restrict__ iperm,
                            const int *__restrict__ bond_ab, const double *__restrict__ bond_req,
                            const double *__restrict__ bond_k, const int *__restrict__ bend_abc,
                            const double *__restrict__ bend_t0, const double *__restrict__ bend_k,
                            unsigned long long *__restrict__ fix,
                            unsigned long long *__restrict__ facc, unsigned *__restrict__ ticket,
                            double *__restrict__ out) {
  double eb = 0.0, ea = 0.0;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nbond + nbend;
       t += gridDim.x * blockDim.x) {
    if (t < nbond) {
      int ia = bond_ab[2 * t], ib = bond_ab[2 * t + 1];
      int4 A = posfx[iperm[ia]], B = posfx[iperm[ib]];
      float dx = fx_delta((unsigned)B.x, (unsigned)A.x, sL.x);
      float dy = fx_delta((unsigned)B.y, (unsigned)A.y, sL.y);
      float dz = fx_delta((unsigned)B.z, (unsigned)A.z, sL.z);
      float dr = sqrtf(dx * dx + dy * dy + dz * dz);
      const double ex = fx_delta_d((unsigned)B.x, (unsigned)A.x, sd.x);
      const double ey = fx_delta_d((unsigned)B.y, (unsigned)A.y, sd.y);
      const double ez = fx_delta_d((unsigned)B.z, (unsigned)A.z, sd.z);
      const double rrd = sqrt(ex * ex + ey * ey + ez * ez) - bond_req[t];
      eb += bond_k[t] * rrd * rrd;
      float fr = -(float)bond_k[t] * (float)rrd * 2.f;
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
      int4 A = posfx[iperm[ia]], B = posfx[iperm[ib]], Cc = posfx[iperm[ic]];
      float dax = fx_delta((unsigned)A.x, (unsigned)B.x, sL.x);
      float day = fx_delta((unsigned)A.y, (unsigned)B.y, sL.y);
      float daz = fx_delta((unsigned)A.z, (unsigned)B.z, sL.z);
      float dcx = fx_delta((unsigned)Cc.x, (unsigned)B.x, sL.x);
      float dcy = fx_delta((unsigned)Cc.y, (unsigned)B.y, sL.y);
      float dcz = fx_delta((unsigned)Cc.z, (unsigned)B.z, sL.z);
      float drai = rsqrtf(dax * dax + day * day + daz * daz);
      float erax = dax * drai, eray = day * drai, eraz = daz * drai;
      float drci = rsqrtf(dcx * dcx + dcy * dcy + dcz * dcz);
      float ercx = dcx * drci, ercy = dcy * drci, ercz = dcz * drci;
      const double pax = fx_delta_d((unsigned)A.x, (unsigned)B.x, sd.x);
      const double pay = fx_delta_d((unsigned)A.y, (unsigned)B.y, sd.y);
      const double paz = fx_delta_d((unsigned)A.z, (unsigned)B.z, sd.z);
      const double pcx = fx_delta_d((unsigned)Cc.x, (unsigned)B.x, sd.x);
      const double pcy = fx_delta_d((unsigned)Cc.y, (unsigned)B.y, sd.y);
      const double pcz = fx_delta_d((unsigned)Cc.z, (unsigned)B.z, sd.z);
      double cosd = (pax * pcx + pay * pcy + paz * pcz) /
                    sqrt((pax * pax + pay * pay + paz * paz) * (pcx * pcx + pcy * pcy + pcz * pcz));
      cosd = fmin(fmax(cosd, -1.0), 1.0);
      const double rrd = acos(cosd) - bend_t0[u];
      ea += bend_k[u] * rrd * rrd;
      float cosphi = (float)cosd;
      float isinphi = rsqrtf(fmaxf(1.f - cosphi * cosphi, 1e-20f));
      float fr = -(float)bend_k[u] * (float)rrd * 2.f;
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
  double v[2] = {eb, ea};
  block_fix_final<2>(v, 32, facc, ticket, out);
}

// ---------------------------------------------------------------------------
// SPME in FP32

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

// per sorted slot: origin cell and fraction exactly from the 32-bit
// fixed-point coordinate (u G / 2^32: integer part and remainder), FP32
// weights, binning
// B-spline weights and derivatives of every site and its integer spline
// origin (floor of u G, exact from the 32-bit fraction)
__device__ __forceinline__ void k_mx_splines_body(VBlk vb_, int n, int order, int3 G, const int4 *__restrict__ posfx,
                             int *__restrict__ floor3, float *__restrict__ sm,
                             float *__restrict__ sd) {
  int s = vb_.id * blockDim.x + threadIdx.x;
  if (s >= n) return;
  int4 p = posfx[s];
  unsigned u[3] = {(unsigned)p.x, (unsigned)p.y, (unsigned)p.z};
  int g[3] = {G.x, G.y, G.z};
  float mn[9], dmn[9];
  for (int d = 0; d < 3; d++) {
    unsigned long long t = (unsigned long long)u[d] * (unsigned)g[d];
    float w = (float)(unsigned)(t & 0xffffffffull) * 0x1p-32f;
    fillspline_f(order, w, mn, dmn);
    for (int m = 1; m <= order; m++) {
      sm[((size_t)s * order + (m - 1)) * 3 + d] = mn[m];
      sd[((size_t)s * order + (m - 1)) * 3 + d] = dmn[m];
    }
    floor3[3 * s + d] = (int)(t >> 32);
  }
}

__global__ void k_mx_splines(int n, int order, int3 G, const int4 *__restrict__ posfx,
                             int *__restrict__ floor3, float *__restrict__ sm,
                             float *__restrict__ sd) {
  k_mx_splines_body(vblk_self(), n, order, G, posfx, floor3, sm, sd);
}

// Spreading by fixed-point reductions: thread (site, mx) adds the
// contributions q wx wy wz of its site's spline slab mx (order x order
// points) to a 64-bit fixed-point grid (2^40 per unit) with fire-and-forget
// integer reductions.  Integer sums do not depend on the order of the
// additions, so the grid is bitwise reproducible; sites in sorted (spatial)
// order keep neighbouring threads on neighbouring grid lines.
constexpr float kSpRedFix = 1099511627776.0f;  // 2^40

__device__ __forceinline__ void k_mx_spread_red_body(VBlk vb_, int n, int order, int3 G, const int4 *__restrict__ posfx,
                                const float *__restrict__ sm, const int *__restrict__ floor3,
                                unsigned long long *__restrict__ gfix) {
  int t = vb_.id * blockDim.x + threadIdx.x;
  int s = t / order, mx = t - s * order;
  if (s >= n) return;
  const float *w = sm + (size_t)s * order * 3;
  float qwx = __int_as_float(posfx[s].w) * w[mx * 3];
  int x = floor3[3 * s] - order + 1 + mx, y0 = floor3[3 * s + 1] - order + 1,
      z0 = floor3[3 * s + 2] - order + 1;
  if (x < 0) x += G.x;
  unsigned long long *gx = gfix + (size_t)x * G.y * G.z;
  for (int my = 0; my < order; my++) {
    int y = y0 + my;
    if (y < 0) y += G.y;
    float v = qwx * w[my * 3 + 1];
    unsigned long long *gy = gx + (size_t)y * G.z;
    for (int mz = 0; mz < order; mz++) {
      int z = z0 + mz;
      if (z < 0) z += G.z;
      atomicAdd(gy + z, (unsigned long long)__float2ll_rn(v * w[mz * 3 + 2] * kSpRedFix));
    }
  }
}

__global__ void k_mx_spread_red(int n, int order, int3 G, const int4 *__restrict__ posfx,
                                const float *__restrict__ sm, const int *__restrict__ floor3,
                                unsigned long long *__restrict__ gfix) {
  k_mx_spread_red_body(vblk_self(), n, order, G, posfx, sm, floor3, gfix);
}

// Order 4 (the configured workloads): the spline weights are computed where
// they are used, from the site's 32-bit fixed-point coordinate, instead of
// being stored by a separate pass and read back (fillspline_f with a
// constant order unrolls into registers).
__device__ __forceinline__ void spline4_axis(unsigned u, int g, int &fl, float (&m)[5],
                                             float (&dm)[5]) {
  unsigned long long t = (unsigned long long)u * (unsigned)g;
  fl = (int)(t >> 32);
  fillspline_f(4, (float)(unsigned)(t & 0xffffffffull) * 0x1p-32f, m, dm);
}

__device__ __forceinline__ void k_mx_spread_o4_body(VBlk vb_, int n, int3 G,
                                                  const int4 *__restrict__ posfx,
                                                  unsigned long long *__restrict__ gfix) {
  int t = vb_.id * blockDim.x + threadIdx.x;
  int s = t >> 2, mx = t & 3;
  if (s >= n) return;
  int4 p = posfx[s];
  float wx[5], wy[5], wz[5], dd[5];
  int fx, fy, fz;
  spline4_axis((unsigned)p.x, G.x, fx, wx, dd);
  spline4_axis((unsigned)p.y, G.y, fy, wy, dd);
  spline4_axis((unsigned)p.z, G.z, fz, wz, dd);
  float w_mx = mx == 0 ? wx[1] : mx == 1 ? wx[2] : mx == 2 ? wx[3] : wx[4];
  float qwx = __int_as_float(p.w) * w_mx;
  int x = fx - 3 + mx, y0 = fy - 3, z0 = fz - 3;
  if (x < 0) x += G.x;
  unsigned long long *gx = gfix + (size_t)x * G.y * G.z;
#pragma unroll
  for (int my = 0; my < 4; my++) {
    int y = y0 + my;
    if (y < 0) y += G.y;
    float v = qwx * wy[my + 1];
    unsigned long long *gy = gx + (size_t)y * G.z;
#pragma unroll
    for (int mz = 0; mz < 4; mz++) {
      int z = z0 + mz;
      if (z < 0) z += G.z;
      atomicAdd(gy + z, (unsigned long long)__float2ll_rn(v * wz[mz + 1] * kSpRedFix));
    }
  }
}

__global__ void k_mx_spread_o4(int n, int3 G, const int4 *__restrict__ posfx,
                             unsigned long long *__restrict__ gfix) {
  k_mx_spread_o4_body(vblk_self(), n, G, posfx, gfix);
}

// A grid sum (2^40 per unit) as FP32 without the FP64 pipe: the upper 32
// bits hold value x 2^8 and convert exactly while |value| < 2^16 (a grid
// point's charge sum is a few e), the lower 32 bits with one rounding, and
// one fused multiply-add joins them.
__device__ __forceinline__ float grid_fix_to_f32(long long v) {
  int hi = (int)(v >> 32);
  unsigned lo = (unsigned)(v & 0xffffffffll);
  return fmaf((float)hi, 0x1p-8f, __uint2float_rn(lo) * 0x1p-40f);
}

// FP32 grid from the fixed-point sums; the sums are cleared for the next step
// (two points per thread and iteration: 16-byte loads and stores)
__device__ __forceinline__ void k_mx_fix2grid_body(VBlk vb_, long K, unsigned long long *__restrict__ gfix,
                              float *__restrict__ grid) {
  const long K2 = K >> 1;
  longlong2 *g2 = reinterpret_cast<longlong2 *>(gfix);
  float2 *o2 = reinterpret_cast<float2 *>(grid);
  for (long i = (long)vb_.id * blockDim.x + threadIdx.x; i < K2;
       i += (long)vb_.n * blockDim.x) {
    longlong2 v = g2[i];
    o2[i] = make_float2(grid_fix_to_f32(v.x), grid_fix_to_f32(v.y));
    g2[i] = make_longlong2(0, 0);
  }
  if ((K & 1) && vb_.id == 0 && threadIdx.x == 0) {
    grid[K - 1] = grid_fix_to_f32((long long)gfix[K - 1]);
    gfix[K - 1] = 0ull;
  }
}

__global__ void k_mx_fix2grid(long K, unsigned long long *__restrict__ gfix,
                              float *__restrict__ grid) {
  k_mx_fix2grid_body(vblk_self(), K, gfix, grid);
}

__device__ __forceinline__ void k_mx_recip_body(VBlk vb_, long Kh, const float *__restrict__ eterm, const float *__restrict__ kw,
                           cufftComplex *__restrict__ gk, unsigned long long *__restrict__ facc,
                           unsigned *__restrict__ ticket, double *__restrict__ out) {
  float e = 0.f;
  for (long h = (long)vb_.id * blockDim.x + threadIdx.x; h < Kh;
       h += (long)vb_.n * blockDim.x) {
    cufftComplex v = gk[h];
    float et = eterm[h];
    e = fmaf(kw[h] * et, v.x * v.x + v.y * v.y, e);
    v.x *= et;
    v.y *= et;
    gk[h] = v;
  }
  float vv[1] = {e};
  block_fix_final<1>(vv, 24, facc, ticket, out, vb_);
}

__global__ void k_mx_recip(long Kh, const float *__restrict__ eterm, const float *__restrict__ kw,
                           cufftComplex *__restrict__ gk, unsigned long long *__restrict__ facc,
                           unsigned *__restrict__ ticket, double *__restrict__ out) {
  k_mx_recip_body(vblk_self(), Kh, eterm, kw, gk, facc, ticket, out);
}

__device__ __forceinline__ void k_mx_gather_body(VBlk vb_, int n, int order, int3 G, float3 gl, float qfe,
                            const int4 *__restrict__ posfx, const int *__restrict__ perm,
                            const int *__restrict__ floor3, const float *__restrict__ sm,
                            const float *__restrict__ sd, const float *__restrict__ grid,
                            unsigned long long *__restrict__ fix,
                            unsigned long long *__restrict__ facc, unsigned *__restrict__ ticket,
                            double *__restrict__ out) {
  long long sx = 0, sy = 0, sz = 0;
  for (int s = vb_.id * blockDim.x + threadIdx.x; s < n; s += vb_.n * blockDim.x) {
    float fxi = 0.f, fyi = 0.f, fzi = 0.f;
    const float *m = sm + (size_t)s * order * 3;
    const float *dm = sd + (size_t)s * order * 3;
    int xo = floor3[3 * s] - order, yo0 = floor3[3 * s + 1] - order, zo0 = floor3[3 * s + 2] - order;
    for (int xi = 1; xi <= order; xi++) {
      int x = wrap1(xo + xi, G.x);
      float mx = m[(xi - 1) * 3], dmx = dm[(xi - 1) * 3];
      for (int yi = 1; yi <= order; yi++) {
        int y = wrap1(yo0 + yi, G.y);
        float my = m[(yi - 1) * 3 + 1], dmy = dm[(yi - 1) * 3 + 1];
        const float *row = grid + ((long)x * G.y + y) * G.z;
        for (int zi = 1; zi <= order; zi++) {
          int z = wrap1(zo0 + zi, G.z);
          float mz = m[(zi - 1) * 3 + 2], dmz = dm[(zi - 1) * 3 + 2];
          float term = row[z];
          fxi -= dmx * my * mz * term;
          fyi -= mx * dmy * mz * term;
          fzi -= mx * my * dmz * term;
        }
      }
    }
    float fac = __int_as_float(posfx[s].w) * qfe;
    fxi *= fac * gl.x;
    fyi *= fac * gl.y;
    fzi *= fac * gl.z;
    int oi = perm[s];
    long long qx = to_fix(fxi), qy = to_fix(fyi), qz = to_fix(fzi);
    atomicAdd(&fix[3 * oi], (unsigned long long)qx);
    atomicAdd(&fix[3 * oi + 1], (unsigned long long)qy);
    atomicAdd(&fix[3 * oi + 2], (unsigned long long)qz);
    sx += qx;
    sy += qy;
    sz += qz;
  }
  long long v[3] = {sx, sy, sz};
  block_fix_final<3>(v, 0, facc, ticket, out, vb_);
}

__global__ void k_mx_gather(int n, int order, int3 G, float3 gl, float qfe,
                            const int4 *__restrict__ posfx, const int *__restrict__ perm,
                            const int *__restrict__ floor3, const float *__restrict__ sm,
                            const float *__restrict__ sd, const float *__restrict__ grid,
                            unsigned long long *__restrict__ fix,
                            unsigned long long *__restrict__ facc, unsigned *__restrict__ ticket,
                            double *__restrict__ out) {
  k_mx_gather_body(vblk_self(), n, order, G, gl, qfe, posfx, perm, floor3, sm, sd, grid, fix, facc, ticket, out);
}

// gather with the order-4 weights and derivatives computed in registers
__device__ __forceinline__ void k_mx_gather_o4_body(VBlk vb_, int n, int3 G, float3 gl, float qfe,
                                                  const int4 *__restrict__ posfx,
                                                  const int *__restrict__ perm,
                                                  const float *__restrict__ grid,
                                                  unsigned long long *__restrict__ fix,
                                                  unsigned long long *__restrict__ facc,
                                                  unsigned *__restrict__ ticket,
                                                  double *__restrict__ out) {
  long long sx = 0, sy = 0, sz = 0;
  for (int s = vb_.id * blockDim.x + threadIdx.x; s < n; s += vb_.n * blockDim.x) {
    int4 p = posfx[s];
    float m[3][5], dm[3][5];
    int fl[3];
    spline4_axis((unsigned)p.x, G.x, fl[0], m[0], dm[0]);
    spline4_axis((unsigned)p.y, G.y, fl[1], m[1], dm[1]);
    spline4_axis((unsigned)p.z, G.z, fl[2], m[2], dm[2]);
    float fxi = 0.f, fyi = 0.f, fzi = 0.f;
    int xo = fl[0] - 4, yo0 = fl[1] - 4, zo0 = fl[2] - 4;
#pragma unroll
    for (int xi = 1; xi <= 4; xi++) {
      int x = wrap1(xo + xi, G.x);
      float mx = m[0][xi], dmx = dm[0][xi];
#pragma unroll
      for (int yi = 1; yi <= 4; yi++) {
        int y = wrap1(yo0 + yi, G.y);
        float my = m[1][yi], dmy = dm[1][yi];
        const float *row = grid + ((long)x * G.y + y) * G.z;
#pragma unroll
        for (int zi = 1; zi <= 4; zi++) {
          int z = wrap1(zo0 + zi, G.z);
          float mz = m[2][zi], dmz = dm[2][zi];
          float term = row[z];
          fxi -= dmx * my * mz * term;
          fyi -= mx * dmy * mz * term;
          fzi -= mx * my * dmz * term;
        }
      }
    }
    float fac = __int_as_float(p.w) * qfe;
    fxi *= fac * gl.x;
    fyi *= fac * gl.y;
    fzi *= fac * gl.z;
    int oi = perm[s];
    long long qx = to_fix(fxi), qy = to_fix(fyi), qz = to_fix(fzi);
    atomicAdd(&fix[3 * oi], (unsigned long long)qx);
    atomicAdd(&fix[3 * oi + 1], (unsigned long long)qy);
    atomicAdd(&fix[3 * oi + 2], (unsigned long long)qz);
    sx += qx;
    sy += qy;
    sz += qz;
  }
  long long v[3] = {sx, sy, sz};
  block_fix_final<3>(v, 0, facc, ticket, out, vb_);
}

__global__ void k_mx_gather_o4(int n, int3 G, float3 gl, float qfe, const int4 *__restrict__ posfx,
                             const int *__restrict__ perm, const float *__restrict__ grid,
                             unsigned long long *__restrict__ fix,
                             unsigned long long *__restrict__ facc, unsigned *__restrict__ ticket,
                             double *__restrict__ out) {
  k_mx_gather_o4_body(vblk_self(), n, G, gl, qfe, posfx, perm, grid, fix, facc, ticket, out);
}

// FP64 forces from the fixed-point sums, minus the mean reciprocal force
__device__ __forceinline__ void k_mx_finalize_body(VBlk vb_, int n, const unsigned long long *__restrict__ fix,
                              const double *__restrict__ scal, double *__restrict__ ff) {
  __shared__ double mean[3];
  if (threadIdx.x < 3) mean[threadIdx.x] = scal[SC_FMEAN + threadIdx.x] / kFixScale / (double)n;
  __syncthreads();
  int i = vb_.id * blockDim.x + threadIdx.x;
  if (i >= 3 * n) return;
  ff[i] = (double)(long long)fix[i] * (1.0 / kFixScale) - mean[i % 3];
}

__global__ void k_mx_finalize(int n, const unsigned long long *__restrict__ fix,
                              const double *__restrict__ scal, double *__restrict__ ff) {
  k_mx_finalize_body(vblk_self(), n, fix, scal, ff);
}

// All intramolecular terms of one molecule per thread: the exclusion
// corrections of k_mx_excl and the bonds and bends of k_mx_bonded, same
// arithmetic, with the molecule's forces summed in registers and added to
// the fixed-point accumulators without atomics (each site belongs to one
// molecule and no other kernel runs concurrently on the accumulators).
// site a of a molecule's register arrays, selected without dynamic indexing
template <int NS>
__device__ __forceinline__ int4 intra_pick(const int4 (&P)[NS], int a) {
  int4 r = P[0];
#pragma unroll
  for (int i = 1; i < NS; i++)
    if (a == i) r = P[i];
  return r;
}
template <int NS>
__device__ __forceinline__ void intra_add(float (&F)[NS][3], int a, float x, float y, float z) {
#pragma unroll
  for (int i = 0; i < NS; i++)
    if (a == i) {
      F[i][0] += x;
      F[i][1] += y;
      F[i][2] += z;
    }
}

template <int NS>
__device__ __forceinline__ int intra_pick_i(const int (&v)[kIntraMaxSites], int a) {
  int r = v[0];
#pragma unroll
  for (int i = 1; i < NS; i++)
    if (a == i) r = v[i];
  return r;
}

// NS: the largest molecule (sites) of the box, so that the molecule's
// positions and forces stay in registers
// UNI: every molecule is T (its terms read from T, unrolled), else the
// per-molecule index lists
// The three kinds of intramolecular term, each adding to the molecule's
// force registers F and the thread's energy sums A.
struct IntraAcc {
  float e_lj = 0.f, e_ljs = 0.f, e_real = 0.f, qsum = 0.f;
  double eb = 0.0, ea = 0.0;  // bond and bend energies (FP64 geometry)
  long long q_intra = 0;
};


// excluded (xf 1-3) or 1-4 (xf 4) pair a-bq: the intra correction, and for
// 1-4 pairs the scaled real-space term and LJ (cnonbond_nblist.c:245-263,
// 416-437); qa, qb the FP64 charges, type_a / type_b the site types
template <int NS>
__device__ __forceinline__ void intra_excl(const int4 (&P)[NS], float (&F)[NS][3], int a, int bq,
                                           int xf, double qa, double qb, int type_a, int type_b,
                                           float3 sL, int nt, const float *__restrict__ lj_tab,
                                           float rc2, float kappa, float c2k, float qf,
                                           float epsRF, const float2 *__restrict__ exptab,
                                           const DfIntra &D, IntraAcc &A) {
  const int4 Pa = intra_pick(P, a), Pb = intra_pick(P, bq);
  float dx = fx_delta((unsigned)Pa.x, (unsigned)Pb.x, sL.x);
  float dy = fx_delta((unsigned)Pa.y, (unsigned)Pb.y, sL.y);
  float dz = fx_delta((unsigned)Pa.z, (unsigned)Pb.z, sL.z);
  float r2 = dx * dx + dy * dy + dz * dz;
  if (r2 > rc2) return;
  float rinv = rsqrtf(r2), r = r2 * rinv, rinv2 = rinv * rinv;
  float kr = kappa * r;
  float ex = __expf(-kr * kr);
  float erfckr = erfc_nr_f(kr, ex);
  float qqab = __int_as_float(Pa.w) * __int_as_float(Pb.w) * qf;
  float Fs = 0.f;
  float qcorr = qqab;
  if (xf == 4) {
    float qq = qqab * (float)kE14FAC / epsRF;
    Fs += qq * rinv * rinv2 * (erfckr + c2k * r * ex);
    A.e_real += qq * erfckr * rinv;
    A.qsum += qq;
    const float *lj = lj_tab + (type_a * nt + type_b) * 3;
    if (lj[0] != 0.f) {
      float sr2 = lj[1] * rinv2, sr6 = sr2 * sr2 * sr2, sr12 = sr6 * sr6;
      Fs += 12.f * lj[0] * rinv2 * (sr12 - sr6);
      A.e_lj += lj[0] * (sr12 - 2.f * sr6);
      A.e_ljs += lj[0] * lj[2];
    }
    qcorr *= (1.f - (float)kE14FAC);
  }
  float erfkr = 1.f - erfckr;
  A.q_intra += df_to_fixed(
      intra_energy_df(D, Pa, Pb, qa, qb, xf == 4 ? (float)(1.0 - kE14FAC) : 1.f, exptab), 32);
  Fs -= qcorr * rinv * rinv2 * (erfkr - c2k * r * ex);
  intra_add(F, a, Fs * dx, Fs * dy, Fs * dz);
  intra_add(F, bq, -Fs * dx, -Fs * dy, -Fs * dz);
}

// cbond.c:27: E = k (r - r0)^2.  The stretch and the energy in FP64 from
// the exact fixed-point differences (a sum of ~1e5 small positive terms
// keeps 1e-7 only if each stretch does: FP32 lengths carry ~1e-7 of r, a
// few 1e-6 of r - r0); the force in FP32 along the FP32 bond vector.
template <int NS>
__device__ __forceinline__ void intra_bond(const int4 (&P)[NS], float (&F)[NS][3], int ia, int ib,
                                           double req, float kb, float3 sL, double3 sd,
                                           IntraAcc &A) {
  const int4 Pa = intra_pick(P, ia), Pb = intra_pick(P, ib);
  const double ex = fx_delta_d((unsigned)Pb.x, (unsigned)Pa.x, sd.x);
  const double ey = fx_delta_d((unsigned)Pb.y, (unsigned)Pa.y, sd.y);
  const double ez = fx_delta_d((unsigned)Pb.z, (unsigned)Pa.z, sd.z);
  const double rr = sqrt(ex * ex + ey * ey + ez * ez) - req;
  A.eb += (double)kb * rr * rr;
  float dx = fx_delta((unsigned)Pb.x, (unsigned)Pa.x, sL.x);
  float dy = fx_delta((unsigned)Pb.y, (unsigned)Pa.y, sL.y);
  float dz = fx_delta((unsigned)Pb.z, (unsigned)Pa.z, sL.z);
  float dr = sqrtf(dx * dx + dy * dy + dz * dz);
  float fr = -kb * (float)rr * 2.f;
  float sc = fr / dr;
  intra_add(F, ia, -sc * dx, -sc * dy, -sc * dz);
  intra_add(F, ib, sc * dx, sc * dy, sc * dz);
}

// cbend.c:24: E = k (theta - theta0)^2.  The angle and the energy in FP64
// (as the stretch above); the force in FP32 from the FP32 unit vectors.
template <int NS>
__device__ __forceinline__ void intra_bend(const int4 (&P)[NS], float (&F)[NS][3], int ia, int ib,
                                           int ic, double t0, float ka, float3 sL, double3 sd,
                                           IntraAcc &A) {
  const int4 Pa = intra_pick(P, ia), Pb = intra_pick(P, ib), Pc = intra_pick(P, ic);
  const double ax = fx_delta_d((unsigned)Pa.x, (unsigned)Pb.x, sd.x);
  const double ay = fx_delta_d((unsigned)Pa.y, (unsigned)Pb.y, sd.y);
  const double az = fx_delta_d((unsigned)Pa.z, (unsigned)Pb.z, sd.z);
  const double cx = fx_delta_d((unsigned)Pc.x, (unsigned)Pb.x, sd.x);
  const double cy = fx_delta_d((unsigned)Pc.y, (unsigned)Pb.y, sd.y);
  const double cz = fx_delta_d((unsigned)Pc.z, (unsigned)Pb.z, sd.z);
  double cosd = (ax * cx + ay * cy + az * cz) /
                sqrt((ax * ax + ay * ay + az * az) * (cx * cx + cy * cy + cz * cz));
  cosd = fmin(fmax(cosd, -1.0), 1.0);
  const double rr = acos(cosd) - t0;
  A.ea += (double)ka * rr * rr;
  float dax = fx_delta((unsigned)Pa.x, (unsigned)Pb.x, sL.x);
  float day = fx_delta((unsigned)Pa.y, (unsigned)Pb.y, sL.y);
  float daz = fx_delta((unsigned)Pa.z, (unsigned)Pb.z, sL.z);
  float dcx = fx_delta((unsigned)Pc.x, (unsigned)Pb.x, sL.x);
  float dcy = fx_delta((unsigned)Pc.y, (unsigned)Pb.y, sL.y);
  float dcz = fx_delta((unsigned)Pc.z, (unsigned)Pb.z, sL.z);
  float drai = rsqrtf(dax * dax + day * day + daz * daz);
  float erax = dax * drai, eray = day * drai, eraz = daz * drai;
  float drci = rsqrtf(dcx * dcx + dcy * dcy + dcz * dcz);
  float ercx = dcx * drci, ercy = dcy * drci, ercz = dcz * drci;
  float cosphi = (float)cosd;
  float isinphi = rsqrtf(fmaxf(1.f - cosphi * cosphi, 1e-20f));
  float fr = -ka * (float)rr * 2.f;
  float irasin = drai * isinphi * fr, ircsin = drci * isinphi * fr;
  float fxa = (erax * cosphi - ercx) * irasin, fya = (eray * cosphi - ercy) * irasin,
        fza = (eraz * cosphi - ercz) * irasin;
  float fxc = (ercx * cosphi - erax) * ircsin, fyc = (ercy * cosphi - eray) * ircsin,
        fzc = (ercz * cosphi - eraz) * ircsin;
  intra_add(F, ia, fxa, fya, fza);
  intra_add(F, ic, fxc, fyc, fzc);
  intra_add(F, ib, -(fxa + fxc), -(fya + fyc), -(fza + fzc));
}

template <int NS, bool UNI = false>
__device__ __forceinline__ void k_mx_intra_body(VBlk vb_, int nmol, const int *__restrict__ mol_first,
                           const int *__restrict__ mol_x, const int *__restrict__ mol_xi,
                           const int *__restrict__ mol_b, const int *__restrict__ mol_bi,
                           const int *__restrict__ mol_a, const int *__restrict__ mol_ai,
                           const int *__restrict__ ab, const int *__restrict__ flag,
                           const int *__restrict__ bond_ab, const double *__restrict__ bond_req,
                           const double *__restrict__ bond_k, const int *__restrict__ bend_abc,
                           const double *__restrict__ bend_t0, const double *__restrict__ bend_k,
                           const int4 *__restrict__ posfx, const int *__restrict__ iperm,
                           const int *__restrict__ type, float3 sL, int nt,
                           const float *__restrict__ lj_tab, float rc2, float kappa, float c2k,
                           float qf, float epsRF, const double4 *__restrict__ pos_q,
                           const float2 *__restrict__ exptab, DfIntra D,
                           unsigned long long *__restrict__ fix,
                           unsigned long long *__restrict__ facc, unsigned *__restrict__ ticket,
                           double *__restrict__ out, const IntraTpl &T = IntraTpl()) {
  IntraAcc A;
  // the length scale per axis, L / 2^32, in FP64 (hi + lo)
  const double3 sd = make_double3((double)D.sl[0].x + (double)D.sl[0].y,
                                  (double)D.sl[1].x + (double)D.sl[1].y,
                                  (double)D.sl[2].x + (double)D.sl[2].y);
  for (int m = vb_.id * blockDim.x + threadIdx.x; m < nmol; m += vb_.n * blockDim.x) {
    const int lb = UNI ? m * T.ns : mol_first[m];
    const int ns = UNI ? T.ns : mol_first[m + 1] - lb;
    int4 P[NS];
    float F[NS][3];
#pragma unroll
    for (int i = 0; i < NS; i++) {
      P[i] = i < ns ? posfx[iperm[lb + i]] : make_int4(0, 0, 0, 0);
      F[i][0] = F[i][1] = F[i][2] = 0.f;
    }
    const int tx0 = UNI ? 0 : mol_x[m], tx1 = UNI ? kTplTerms : mol_x[m + 1];
#pragma unroll
    for (int t = tx0; t < tx1; t++) {
      int a, bq, xf;
      if (UNI) {
        if (t >= T.nx) break;
        a = T.xa[t];
        bq = T.xb[t];
        xf = T.xf[t];
      } else {
        int x = mol_xi[t];
        a = ab[2 * x] - lb;
        bq = ab[2 * x + 1] - lb;
        xf = flag[x];
      }
      if (xf == 0) continue;
      intra_excl<NS>(P, F, a, bq, xf, pos_q[lb + a].w, pos_q[lb + bq].w,
                     UNI ? intra_pick_i<NS>(T.type, a) : type[lb + a],
                     UNI ? intra_pick_i<NS>(T.type, bq) : type[lb + bq], sL, nt, lj_tab, rc2,
                     kappa, c2k, qf, epsRF, exptab, D, A);
    }
    const int tb0 = UNI ? 0 : mol_b[m], tb1 = UNI ? kTplTerms : mol_b[m + 1];
#pragma unroll
    for (int t = tb0; t < tb1; t++) {
      int ia, ib;
      double req;
      float kb;
      if (UNI) {
        if (t >= T.nb) break;
        ia = T.ba[t];
        ib = T.bb[t];
        req = (double)T.breq[t] + (double)T.breq_lo[t];
        kb = T.bk[t];
      } else {
        int u = mol_bi[t];
        ia = bond_ab[2 * u] - lb;
        ib = bond_ab[2 * u + 1] - lb;
        req = bond_req[u];
        kb = (float)bond_k[u];
      }
      intra_bond<NS>(P, F, ia, ib, req, kb, sL, sd, A);
    }
    const int ta0 = UNI ? 0 : mol_a[m], ta1 = UNI ? kTplTerms : mol_a[m + 1];
#pragma unroll
    for (int t = ta0; t < ta1; t++) {
      int ia, ib, ic;
      double t0;
      float ka;
      if (UNI) {
        if (t >= T.na) break;
        ia = T.aa[t];
        ib = T.ab[t];
        ic = T.ac[t];
        t0 = (double)T.at0[t] + (double)T.at0_lo[t];
        ka = T.ak[t];
      } else {
        int u = mol_ai[t];
        ia = bend_abc[3 * u] - lb;
        ib = bend_abc[3 * u + 1] - lb;
        ic = bend_abc[3 * u + 2] - lb;
        t0 = bend_t0[u];
        ka = (float)bend_k[u];
      }
      intra_bend<NS>(P, F, ia, ib, ic, t0, ka, sL, sd, A);
    }
#pragma unroll
    for (int i = 0; i < NS; i++)
      if (i < ns)
#pragma unroll
        for (int c = 0; c < 3; c++) {
          unsigned long long *q = fix + 3 * (size_t)(lb + i) + c;
          atomicAdd(q, (unsigned long long)to_fix(F[i][c]));
        }
  }
  long long v[7] = {to_fixed(A.e_lj, 32), to_fixed(A.e_ljs, 32), to_fixed(A.e_real, 32),
                    to_fixed(A.qsum, 32), A.q_intra, to_fixed(A.eb, 32), to_fixed(A.ea, 32)};
  block_fix_final<7>(v, 32, facc, ticket, out, vb_);
}

template <int NS>
__global__ void k_mx_intra(int nmol, const int *__restrict__ mol_first,
                           const int *__restrict__ mol_x, const int *__restrict__ mol_xi,
                           const int *__restrict__ mol_b, const int *__restrict__ mol_bi,
                           const int *__restrict__ mol_a, const int *__restrict__ mol_ai,
                           const int *__restrict__ ab, const int *__restrict__ flag,
                           const int *__restrict__ bond_ab, const double *__restrict__ bond_req,
                           const double *__restrict__ bond_k, const int *__restrict__ bend_abc,
                           const double *__restrict__ bend_t0, const double *__restrict__ bend_k,
                           const int4 *__restrict__ posfx, const int *__restrict__ iperm,
                           const int *__restrict__ type, float3 sL, int nt,
                           const float *__restrict__ lj_tab, float rc2, float kappa, float c2k,
                           float qf, float epsRF, const double4 *__restrict__ pos_q,
                           const float2 *__restrict__ exptab, DfIntra D,
                           unsigned long long *__restrict__ fix,
                           unsigned long long *__restrict__ facc, unsigned *__restrict__ ticket,
                           double *__restrict__ out) {
  k_mx_intra_body<NS>(vblk_self(), nmol, mol_first, mol_x, mol_xi, mol_b, mol_bi, mol_a, mol_ai, ab, flag, bond_ab, bond_req, bond_k, bend_abc, bend_t0, bend_k, posfx, iperm, type, sL, nt, lj_tab, rc2, kappa, c2k, qf, epsRF, pos_q, exptab, D, fix, facc, ticket, out);
}

// the same for a box of identical molecules (their topology in T)
template <int NS>
__global__ void k_mx_intra_uni(int nmol, IntraTpl T, const int4 *__restrict__ posfx,
                               const int *__restrict__ iperm, float3 sL, int nt,
                               const float *__restrict__ lj_tab, float rc2, float kappa,
                               float c2k, float qf, float epsRF,
                               const double4 *__restrict__ pos_q,
                               const float2 *__restrict__ exptab, DfIntra D,
                               unsigned long long *__restrict__ fix,
                               unsigned long long *__restrict__ facc,
                               unsigned *__restrict__ ticket, double *__restrict__ out) {
  k_mx_intra_body<NS, true>(vblk_self(), nmol, nullptr, nullptr, nullptr, nullptr, nullptr,
                            nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                            nullptr, nullptr, nullptr, posfx, iperm, nullptr, sL, nt, lj_tab,
                            rc2, kappa, c2k, qf, epsRF, pos_q, exptab, D, fix, facc, ticket, out,
                            T);
}

// combine the mixed kernels' sums into the reference's slots
__global__ void k_mx_slots(double *__restrict__ s, double erfc_rc_over_rc, int fused) {
  if (threadIdx.x != 0) return;
  mixed_slots_dev(s, erfc_rc_over_rc, fused);
}

// ---------------------------------------------------------------------------
// host side

static int up(int **dst, const std::vector<int> &v) {
  FE_CUDA(cudaMalloc(dst, sizeof(int) * (v.empty() ? 1 : v.size())));
  if (!v.empty())
    FE_CUDA(cudaMemcpy(*dst, v.data(), sizeof(int) * v.size(), cudaMemcpyHostToDevice));
  return FE_OK;
}

int mixed_setup(Box *b) {
  Mixed &M = *b->mx;
  int n = b->n;
  FE_CUDA(cudaDeviceGetAttribute(&M.nsm, cudaDevAttrMultiProcessorCount, b->dev));
  FE_CUDA(cudaStreamCreateWithFlags(&M.s2, cudaStreamNonBlocking));
  FE_CUDA(cudaEventCreateWithFlags(&M.ev_fork, cudaEventDisableTiming));
  FE_CUDA(cudaEventCreateWithFlags(&M.ev_join, cudaEventDisableTiming));
  FE_CUDA(cudaMalloc(&M.facc2, sizeof(unsigned long long) * kFaccSlots));
  FE_CUDA(cudaMemset(M.facc2, 0, sizeof(unsigned long long) * kFaccSlots));
  FE_CUDA(cudaMalloc(&M.ticket2, sizeof(unsigned)));
  FE_CUDA(cudaMemset(M.ticket2, 0, sizeof(unsigned)));
  // cell grid of edge >= rlist / kListCellsPerReach
  double edge = (b->p.rclist > b->p.rclist_ew ? b->p.rclist : b->p.rclist_ew) / kListCellsPerReach;
  M.ncells = 1;
  for (int d = 0; d < 3; d++) {
    int m = (int)(b->p.L[d] / edge);
    M.nc[d] = m < 1 ? 1 : m;
    M.h[d] = b->p.L[d] / M.nc[d];
    M.ncells *= M.nc[d];
  }
  // the minimum image from wrapped 32-bit fractions needs |d| < L/2
  double rl = b->p.rclist;
  for (int d = 0; d < 3; d++)
    if (rl >= 0.5 * b->p.L[d]) {
      set_error("mixed precision needs rclist < L/2 in every direction");
      return FE_ERR_ARG;
    }
  FE_CUDA(cudaMalloc(&M.cell_count, sizeof(int) * M.ncells));
  // the counts are zero between list builds: each build clears them after
  // its scan (launch_mixed_list, k_b_mx_scan)
  FE_CUDA(cudaMemset(M.cell_count, 0, sizeof(int) * M.ncells));
  FE_CUDA(cudaMalloc(&M.cell_start, sizeof(int) * (M.ncells + 1)));
  FE_CUDA(cudaMalloc(&M.cell_fill, sizeof(int) * M.ncells));
  FE_CUDA(cudaMalloc(&M.cell_of, sizeof(int) * n));
  FE_CUDA(cudaMalloc(&M.perm, sizeof(int) * n));
  FE_CUDA(cudaMalloc(&M.iperm, sizeof(int) * n));
  FE_CUDA(cudaMalloc(&M.cell_s, sizeof(int) * n));
  FE_CUDA(cudaMalloc(&M.type_s, sizeof(int) * n));
  FE_CUDA(cudaMalloc(&M.posfx, sizeof(int4) * n));
  // full-list row capacity: a sphere of rlist at the box's density, with margin
  double vol = b->p.L[0] * b->p.L[1] * b->p.L[2];
  double expect = 4.0 / 3.0 * kPI * rl * rl * rl * (double)n / vol;
  int cap = (int)(1.6 * expect + 64.0);
  if (b->p.max_neighbors > 0) cap = b->p.max_neighbors;
  cap = (cap + 31) / 32 * 32;
  if (cap > n) cap = (n + 31) / 32 * 32;
  M.cap = cap;
  FE_CUDA(cudaMalloc(&M.cnt_lj, sizeof(int) * n));
  FE_CUDA(cudaMalloc(&M.cnt_nl, sizeof(int) * n));
  FE_CUDA(cudaMalloc(&M.ent, sizeof(int) * (size_t)n * cap));
  FE_CUDA(cudaMalloc(&M.icnt_lj, sizeof(int) * n));
  FE_CUDA(cudaMalloc(&M.icnt_nl, sizeof(int) * n));
  FE_CUDA(cudaMalloc(&M.ient, sizeof(int) * (size_t)n * cap));
  FE_CUDA(cudaMalloc(&M.snap, sizeof(int4) * n));
  FE_CUDA(cudaMalloc(&M.ps, sizeof(MxPruneState)));
  FE_CUDA(cudaMemset(M.ps, 0, sizeof(MxPruneState)));
  M.inner_on = b->p.rc + M.skin < (b->p.rclist < b->p.rclist_ew ? b->p.rclist : b->p.rclist_ew);
  FE_CUDA(cudaMalloc(&M.fix, sizeof(unsigned long long) * 3 * n));
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
  std::vector<unsigned char> on(nt * nt);
  for (int k = 0; k < nt * nt; k++) on[k] = lj[3 * k] != 0.f ? 1 : 0;
  FE_CUDA(cudaMalloc(&M.lj_on, on.size()));
  FE_CUDA(cudaMemcpy(M.lj_on, on.data(), on.size(), cudaMemcpyHostToDevice));
  if (nt <= 32) {  // lj_row[t'] bit t: pair (t, t') has an LJ term
    std::vector<unsigned> row(nt, 0u);
    for (int t = 0; t < nt; t++)
      for (int t2 = 0; t2 < nt; t2++)
        if (on[t * nt + t2]) row[t2] |= 1u << t;
    FE_CUDA(cudaMalloc(&M.lj_row, sizeof(unsigned) * nt));
    FE_CUDA(cudaMemcpy(M.lj_row, row.data(), sizeof(unsigned) * nt, cudaMemcpyHostToDevice));
  }
  // exclusion pair list (xint), for the correction kernel
  M.nexcl = b->p.nexcl;
  FE_CUDA(cudaMalloc(&M.excl_ab, sizeof(int) * 2 * (M.nexcl ? M.nexcl : 1)));
  FE_CUDA(cudaMalloc(&M.excl_flag, sizeof(int) * (M.nexcl ? M.nexcl : 1)));
  if (M.nexcl) {
    FE_CUDA(cudaMemcpy(M.excl_ab, b->p.excl_ab, sizeof(int) * 2 * M.nexcl, cudaMemcpyHostToDevice));
    FE_CUDA(cudaMemcpy(M.excl_flag, b->p.excl_flag, sizeof(int) * M.nexcl, cudaMemcpyHostToDevice));
  }  {
    // molecules for the fused intramolecular kernel: connected components of
    // bonds, bends and exclusions; usable when each is a contiguous run of
    // at most kIntraMaxSites sites
    std::vector<int> par(n);
    for (int i = 0; i < n; i++) par[i] = i;
    auto find = [&](int x) {
      while (par[x] != x) x = par[x] = par[par[x]];
      return x;
    };
    auto unite = [&](int x, int y) {
      x = find(x);
      y = find(y);
      if (x != y) par[x > y ? x : y] = x < y ? x : y;
    };
    const fe_box_params &pp = b->p;
    for (int t = 0; t < pp.nbond; t++) unite(pp.bond_ab[2 * t], pp.bond_ab[2 * t + 1]);
    for (int t = 0; t < pp.nbend; t++) {
      unite(pp.bend_abc[3 * t], pp.bend_abc[3 * t + 1]);
      unite(pp.bend_abc[3 * t + 1], pp.bend_abc[3 * t + 2]);
    }
    for (int t = 0; t < pp.nexcl; t++) unite(pp.excl_ab[2 * t], pp.excl_ab[2 * t + 1]);
    std::vector<int> first, mol_of(n);
    bool ok = true;
    for (int i = 0; i < n && ok; i++) {
      int r = find(i);
      if (i == 0 || r != find(i - 1)) {
        if (r != i) ok = false;  // a component that does not start here: not contiguous
        first.push_back(i);
      }
      mol_of[i] = (int)first.size() - 1;
    }
    first.push_back(n);
    int nm = (int)first.size() - 1;
    for (int m = 0; m < nm && ok; m++)
      if (first[m + 1] - first[m] > kIntraMaxSites) ok = false;
    if (ok && nm > 0) {
      auto csr = [&](int count, auto mol_fn, std::vector<int> &off, std::vector<int> &idx) {
        off.assign(nm + 1, 0);
        for (int t = 0; t < count; t++) off[mol_fn(t) + 1]++;
        for (int m = 0; m < nm; m++) off[m + 1] += off[m];
        std::vector<int> fill(off.begin(), off.end() - 1);
        idx.assign(count > 0 ? count : 1, 0);
        for (int t = 0; t < count; t++) idx[fill[mol_fn(t)]++] = t;
      };
      std::vector<int> xo, xi, bo, bi, ao, ai;
      csr(pp.nexcl, [&](int t) { return mol_of[pp.excl_ab[2 * t]]; }, xo, xi);
      csr(pp.nbond, [&](int t) { return mol_of[pp.bond_ab[2 * t]]; }, bo, bi);
      csr(pp.nbend, [&](int t) { return mol_of[pp.bend_abc[3 * t]]; }, ao, ai);
      int rc;
      if ((rc = up(&M.mol_first, first))) return rc;
      if ((rc = up(&M.mol_x, xo)) || (rc = up(&M.mol_xi, xi))) return rc;
      if ((rc = up(&M.mol_b, bo)) || (rc = up(&M.mol_bi, bi))) return rc;
      if ((rc = up(&M.mol_a, ao)) || (rc = up(&M.mol_ai, ai))) return rc;
      M.nmol = nm;
      M.intra_maxs = 1;
      for (int m = 0; m < nm; m++)
        if (first[m + 1] - first[m] > M.intra_maxs) M.intra_maxs = first[m + 1] - first[m];
      // all molecules alike?  (same size and, at the same relative sites,
      // the same exclusions, bonds, bends and site types)
      IntraTpl &T = M.tpl;
      memset(&T, 0, sizeof T);
      const int ns0 = first[1] - first[0];
      bool uni = xo[1] - xo[0] <= kTplTerms && bo[1] - bo[0] <= kTplTerms &&
                 ao[1] - ao[0] <= kTplTerms;
      T.ns = ns0;
      T.nx = xo[1] - xo[0];
      T.nb = bo[1] - bo[0];
      T.na = ao[1] - ao[0];
      for (int m = 0; m < nm && uni; m++) {
        const int lb = first[m];
        if (first[m + 1] - lb != ns0 || lb != m * ns0 || xo[m + 1] - xo[m] != T.nx ||
            bo[m + 1] - bo[m] != T.nb || ao[m + 1] - ao[m] != T.na) {
          uni = false;
          break;
        }
        for (int i = 0; i < ns0 && uni; i++) {
          if (m == 0) T.type[i] = pp.type[lb + i];
          else if (pp.type[lb + i] != T.type[i]) uni = false;
        }
        for (int k = 0; k < T.nx && uni; k++) {
          int x = xi[xo[m] + k];
          int a = pp.excl_ab[2 * x] - lb, c = pp.excl_ab[2 * x + 1] - lb, f = pp.excl_flag[x];
          if (m == 0) {
            T.xa[k] = a;
            T.xb[k] = c;
            T.xf[k] = f;
          } else if (a != T.xa[k] || c != T.xb[k] || f != T.xf[k]) {
            uni = false;
          }
        }
        for (int k = 0; k < T.nb && uni; k++) {
          int u = bi[bo[m] + k];
          int a = pp.bond_ab[2 * u] - lb, c = pp.bond_ab[2 * u + 1] - lb;
          float req = (float)pp.bond_req[u], kk = (float)pp.bond_k[u];
          float req_lo = (float)(pp.bond_req[u] - (double)req);
          if (m == 0) {
            T.ba[k] = a;
            T.bb[k] = c;
            T.breq[k] = req;
            T.breq_lo[k] = req_lo;
            T.bk[k] = kk;
          } else if (a != T.ba[k] || c != T.bb[k] || req != T.breq[k] ||
                     req_lo != T.breq_lo[k] || kk != T.bk[k]) {
            uni = false;
          }
        }
        for (int k = 0; k < T.na && uni; k++) {
          int u = ai[ao[m] + k];
          int a = pp.bend_abc[3 * u] - lb, c = pp.bend_abc[3 * u + 1] - lb,
              d = pp.bend_abc[3 * u + 2] - lb;
          float t0 = (float)pp.bend_theta0[u], kk = (float)pp.bend_k[u];
          float t0_lo = (float)(pp.bend_theta0[u] - (double)t0);
          if (m == 0) {
            T.aa[k] = a;
            T.ab[k] = c;
            T.ac[k] = d;
            T.at0[k] = t0;
            T.at0_lo[k] = t0_lo;
            T.ak[k] = kk;
          } else if (a != T.aa[k] || c != T.ab[k] || d != T.ac[k] || t0 != T.at0[k] ||
                     t0_lo != T.at0_lo[k] || kk != T.ak[k]) {
            uni = false;
          }
        }
      }
      M.uniform = uni;
    }
  }

  {
    // double-float constants of the intramolecular correction energy
    std::vector<float2> tab(kDfExpN);
    for (int k = kDfExpLo; k <= kDfExpHi; k++) {
      float hi, lo;
      df_split(exp((double)k / 64.0), hi, lo);
      tab[k - kDfExpLo] = make_float2(hi, lo);
    }
    FE_CUDA(cudaMalloc(&M.exptab, sizeof(float2) * kDfExpN));
    FE_CUDA(cudaMemcpy(M.exptab, tab.data(), sizeof(float2) * kDfExpN, cudaMemcpyHostToDevice));
    // ewald.c:817-836, constant term first
    const double c[10] = {-1.26551223, 1.00002368, 0.37409196, 0.09678418, -0.18628806,
                          0.27886807, -1.13520398, 1.48851587, -0.82215223, 0.17087277};
    for (int k = 0; k < 10; k++) df_split(c[k], M.dfi.C.c[k].x, M.dfi.C.c[k].y);
    df_split(b->p.kappa, M.dfi.kappa.x, M.dfi.kappa.y);
    df_split(kELEC * kELEQ * kELEQ * kNA * 1.0E-3, M.dfi.qf.x, M.dfi.qf.y);
    for (int d = 0; d < 3; d++) df_split(b->p.L[d] / kFixScale, M.dfi.sl[d].x, M.dfi.sl[d].y);
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
  FE_CUDA(cudaMalloc(&M.gfix, sizeof(unsigned long long) * b->K));
  FE_CUDA(cudaMemset(M.gfix, 0, sizeof(unsigned long long) * b->K));
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
                  M.type_s, M.posfx, M.cnt_lj, M.cnt_nl, M.ent, M.icnt_lj, M.icnt_nl,
                  M.ient, M.snap, M.ps, M.fix, M.lj_tab, M.lj_on, M.lj_row, M.excl_ab, M.excl_flag, M.eterm32, M.kw32,
                  M.grid32, M.grid32k, M.floor3, M.gfix, M.sm, M.sd, M.mol_first, M.mol_x,
                  M.mol_xi, M.mol_b, M.mol_bi, M.mol_a, M.mol_ai, M.exptab, M.facc2, M.ticket2};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  if (M.ev_fork) cudaEventDestroy(M.ev_fork);
  if (M.ev_join) cudaEventDestroy(M.ev_join);
  if (M.s2) cudaStreamDestroy(M.s2);
  if (M.plans) {
    cufftDestroy(M.plan_r2c);
    cufftDestroy(M.plan_c2r);
  }
  delete b->mx;
  b->mx = nullptr;
}

void mixed_counts(Box *b, const int **lj, const int **rest) {
  *lj = b->mx->cnt_lj;
  *rest = b->mx->cnt_nl;
}

void mixed_inner_counts(Box *b, const int **lj, const int **rest, bool *on) {
  *lj = b->mx->icnt_lj;
  *rest = b->mx->icnt_nl;
  *on = b->mx->inner_on;
}

MxPruneState *mixed_prune_state(Box *b) { return b->mx->ps; }

static float3 fix_scale(Box *b) {
  return make_float3((float)(b->p.L[0] / kFixScale), (float)(b->p.L[1] / kFixScale),
                     (float)(b->p.L[2] / kFixScale));
}

static int launch_convert(Box *b, bool zero_forces = false) {
  Mixed &M = *b->mx;
  double3 invL = make_double3(1.0 / b->p.L[0], 1.0 / b->p.L[1], 1.0 / b->p.L[2]);
  k_mx_convert<<<(b->n + 255) / 256, 256, 0, b->stream>>>(
      b->n, b->pos_q, M.perm, invL, M.posfx, M.inner_on ? M.snap : nullptr, fix_scale(b),
      &M.ps->dmax2, zero_forces ? M.fix : nullptr);
  FE_LAUNCH_CHECK("k_mx_convert");
  return FE_OK;
}



int launch_mixed_list(Box *b) {
  Mixed &M = *b->mx;
  int n = b->n;
  double3 L = make_double3(b->p.L[0], b->p.L[1], b->p.L[2]);
  double3 invL = make_double3(1.0 / b->p.L[0], 1.0 / b->p.L[1], 1.0 / b->p.L[2]);
  int3 nc = make_int3(M.nc[0], M.nc[1], M.nc[2]);
  k_mx_cell<<<(n + 255) / 256, 256, 0, b->stream>>>(n, b->pos_q, invL, nc, M.cell_of,
                                                    M.cell_count);
  FE_LAUNCH_CHECK("k_mx_cell");
  k_cell_scan_ext(M.cell_count, M.ncells, M.cell_start, M.cell_fill, b->stream);
  FE_CUDA(cudaMemsetAsync(M.cell_count, 0, sizeof(int) * M.ncells, b->stream));
  k_mx_fill<<<(n + 255) / 256, 256, 0, b->stream>>>(n, M.cell_of, M.cell_start, M.cell_fill, M.perm);
  FE_LAUNCH_CHECK("k_mx_fill");
  k_mx_cellsort<<<M.ncells, 32, 0, b->stream>>>(M.cell_start, M.perm, M.iperm, M.cell_s,
                                                 b->type, M.type_s, b->status);
  FE_LAUNCH_CHECK("k_mx_cellsort");
  int rc = launch_convert(b);
  if (rc) return rc;
  float3 Lf = make_float3((float)b->p.L[0], (float)b->p.L[1], (float)b->p.L[2]);
  float rl = (float)(b->p.rclist < b->p.rclist_ew ? b->p.rclist : b->p.rclist_ew);
  int units = (n + kListUnit - 1) / kListUnit;
  int blocks = (units + kMxWarps - 1) / kMxWarps;
  k_mx_list<<<blocks < M.nsm * 8 ? blocks : M.nsm * 8, kMxWarps * 32, 0, b->stream>>>(
      n, M.posfx, M.perm, M.iperm, M.cell_s, M.type_s, M.cell_start, nc, fix_scale(b), Lf, rl,
      b->nt, M.lj_row, M.lj_on, b->x_start, b->x_partner, M.cap, M.cnt_lj, M.cnt_nl, M.ent,
      b->status);
  FE_LAUNCH_CHECK("k_mx_list");
  // the inner list and its snapshot belong to the old sort: prune next
  FE_CUDA(cudaMemsetAsync(&M.ps->need, 0x01, sizeof(int), b->stream));
  b->have_list = true;
  return FE_OK;
}

static int pair_blocks(Box *b, int nw) {
  int blocks = (b->n + nw - 1) / nw;
  return blocks > 2048 ? 2048 : blocks;
}

MxPair mx_pair_params(Box *b) {
  Mixed &M = *b->mx;
  MxPair P;
  P.n = b->n;
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
  P.inv_sw_den = ron2 > 0.0 ? (float)(1.0 / ((rc2 - ron2) * (rc2 - ron2) * (rc2 - ron2))) : 0.f;
  P.sc = fix_scale(b);
  P.cubic = (b->p.L[0] == b->p.L[1] && b->p.L[1] == b->p.L[2]) ? 1 : 0;
  P.s2 = P.sc.x * P.sc.x;
  double rp = b->p.rc + M.skin, hs = 0.5 * M.skin - 1e-4;
  P.rp2 = (float)(rp * rp);
  P.thresh2 = (float)(hs * hs);
  P.inner_on = M.inner_on ? 1 : 0;
  return P;
}

int launch_mx_pair_only(Box *b) {
  Mixed &M = *b->mx;
  MxPair P = mx_pair_params(b);
  size_t shm = sizeof(float) * (b->nt * b->nt * 3);
  int nw = M.tune_nw, blocks = M.tune_blocks > 0 ? M.tune_blocks : pair_blocks(b, nw);
#define FE_PAIR_ARGS                                                                          \
  P, M.posfx, M.type_s, M.perm, M.cnt_lj, M.cnt_nl, M.ent, M.icnt_lj, M.icnt_nl, M.ient, M.snap, \
      M.ps, M.lj_tab, M.fix, b->facc, b->ticket, b->scal + SC_MX_PAIR, b->status
  // the pruning variant: 64 registers, one resident wave of 8-warp blocks
  k_mx_pair<8, 32, true><<<M.nsm * 4, 256, shm, b->stream>>>(FE_PAIR_ARGS);
  FE_LAUNCH_CHECK("k_mx_pair<prune>");
#define FE_PAIR_LAUNCH(NWV, RWV) \
  k_mx_pair<NWV, RWV, false><<<blocks, NWV * 32, shm, b->stream>>>(FE_PAIR_ARGS)
  if (M.tune_rw == 32) {
    if (nw == 4) FE_PAIR_LAUNCH(4, 32);
    else if (nw == 16) FE_PAIR_LAUNCH(16, 32);
    else FE_PAIR_LAUNCH(8, 32);
  } else {
    if (nw == 4) FE_PAIR_LAUNCH(4, 48);
    else if (nw == 16) FE_PAIR_LAUNCH(16, 48);
    else FE_PAIR_LAUNCH(8, 48);
  }
#undef FE_PAIR_LAUNCH
#undef FE_PAIR_ARGS
  FE_LAUNCH_CHECK("k_mx_pair");
  return FE_OK;
}

// Chooses the pair kernel's launch shape for this box: warps per block in
// {4, 8, 16}, register budget (40 or 64 per thread) and the grid size
// (multiples of the SM count, or one warp per row), each timed with CUDA
// events on the box's stream over the current (inner) list; the fastest is
// kept.
// Forces and energies must be recomputed after.
int mixed_autotune(Box *b, int *nw_out, int *rw_out, int *blocks_out, double *us_out) {
  Mixed &M = *b->mx;
  int nsm = 0;
  FE_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, b->dev));
  const int nws[3] = {4, 8, 16}, rws[2] = {48, 32};
  cudaEvent_t e0, e1;
  FE_CUDA(cudaEventCreate(&e0));
  FE_CUDA(cudaEventCreate(&e1));
  int best_nw = M.tune_nw, best_blocks = M.tune_blocks, best_rw = M.tune_rw;
  float best = 1e30f;
  int rc = FE_OK;
  for (int c = 0; c < 6 && rc == FE_OK; c++) {
    int nw = nws[c % 3], rw = rws[c / 3];
    int full = (b->n + nw - 1) / nw;
    int grids[6] = {nsm * 4, nsm * 8, nsm * 12, nsm * 16, nsm * 24, full};
    for (int g = 0; g < 6 && rc == FE_OK; g++) {
      int blocks = grids[g] < full ? grids[g] : full;
      M.tune_nw = nw;
      M.tune_rw = rw;
      M.tune_blocks = blocks;
      if ((rc = launch_mx_pair_only(b))) break;  // warm-up
      cudaEventRecord(e0, b->stream);
      for (int r = 0; r < 3 && rc == FE_OK; r++) rc = launch_mx_pair_only(b);
      cudaEventRecord(e1, b->stream);
      cudaError_t e = cudaEventSynchronize(e1);
      if (e != cudaSuccess) {
        rc = cuda_fail(e, "mixed_autotune");
        break;
      }
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (ms < best) {
        best = ms;
        best_nw = nw;
        best_rw = rw;
        best_blocks = blocks;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  M.tune_nw = best_nw;
  M.tune_rw = best_rw;
  M.tune_blocks = best_blocks;
  if (rc) return rc;
  if (nw_out) *nw_out = best_nw;
  if (rw_out) *rw_out = best_rw;
  if (blocks_out) *blocks_out = best_blocks;
  if (us_out) *us_out = 1000.0 * best / 3.0;
  return FE_OK;
}

static int spread_on(Box *b, cudaStream_t st) {
  Mixed &M = *b->mx;
  int3 G = make_int3(b->G[0], b->G[1], b->G[2]);
  long nt = (long)b->n * b->order;
  if (b->order == 4) {
    k_mx_spread_o4<<<(unsigned)((nt + 255) / 256), 256, 0, st>>>(b->n, G, M.posfx, M.gfix);
    FE_LAUNCH_CHECK("k_mx_spread_o4");
  } else {
    k_mx_spread_red<<<(unsigned)((nt + 255) / 256), 256, 0, st>>>(
        b->n, b->order, G, M.posfx, M.sm, M.floor3, M.gfix);
    FE_LAUNCH_CHECK("k_mx_spread_red");
  }
  k_mx_fix2grid<<<M.nsm * 8, 256, 0, st>>>(b->K, M.gfix, M.grid32);
  FE_LAUNCH_CHECK("k_mx_fix2grid");
  return FE_OK;
}

int launch_mx_spread_only(Box *b) { return spread_on(b, b->stream); }

// The reciprocal-space forces and energy (pme_calc's work) on stream st with
// the reduction slots facc / ticket: [splines,] spreading, FFT, convolution,
// inverse FFT, gather.  It reads the fixed-point coordinates and adds to the
// force sums with integer atomics, so it may run beside the pair kernel.
static int spme_on(Box *b, cudaStream_t st, unsigned long long *facc, unsigned *ticket) {
  Mixed &M = *b->mx;
  const int n = b->n;
  int rc;
  int3 G = make_int3(b->G[0], b->G[1], b->G[2]);
  if (b->order != 4) {  // order 4 computes its weights inside spreading and gathering
    k_mx_splines<<<(n + 127) / 128, 128, 0, st>>>(n, b->order, G, M.posfx, M.floor3, M.sm,
                                                  M.sd);
    FE_LAUNCH_CHECK("k_mx_splines");
  }
  if ((rc = spread_on(b, st))) return rc;
  cufftResult r = cufftSetStream(M.plan_r2c, st);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftSetStream");
  r = cufftExecR2C(M.plan_r2c, M.grid32, M.grid32k);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftExecR2C");
  int kb = (int)((b->Kh + 255) / 256);
  if (kb > 1024) kb = 1024;
  k_mx_recip<<<kb, 256, 0, st>>>(b->Kh, M.eterm32, M.kw32, M.grid32k, facc, ticket,
                                 b->scal + SC_ENREC);
  FE_LAUNCH_CHECK("k_mx_recip");
  r = cufftSetStream(M.plan_c2r, st);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftSetStream");
  r = cufftExecC2R(M.plan_c2r, M.grid32k, M.grid32);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftExecC2R");
  double qf = kELEC * kELEQ * kELEQ * kNA * 1.0E-3;
  float3 gl = make_float3((float)(b->G[0] / b->p.L[0]), (float)(b->G[1] / b->p.L[1]),
                          (float)(b->G[2] / b->p.L[2]));
  int gb = (n + 127) / 128;
  if (gb > 1024) gb = 1024;
  float qfe = (float)(qf / b->p.epsRF);
  if (b->order == 4) {
    k_mx_gather_o4<<<gb, 128, 0, st>>>(n, G, gl, qfe, M.posfx, M.perm, M.grid32, M.fix, facc,
                                       ticket, b->scal + SC_FMEAN);
    FE_LAUNCH_CHECK("k_mx_gather_o4");
  } else {
    k_mx_gather<<<gb, 128, 0, st>>>(n, b->order, G, gl, qfe, M.posfx, M.perm, M.floor3, M.sm,
                                    M.sd, M.grid32, M.fix, facc, ticket, b->scal + SC_FMEAN);
    FE_LAUNCH_CHECK("k_mx_gather");
  }
  return FE_OK;
}

// The intramolecular terms (exclusion corrections, 1-4 pairs, bonds, bends)
// on stream st with the reduction slots facc / ticket: one thread per
// molecule when the topology allows, else kernels over the exclusion and
// bonded lists.  Integer atomics into the force sums.
static int intra_on(Box *b, cudaStream_t st, unsigned long long *facc, unsigned *ticket) {
  Mixed &M = *b->mx;
  double qf = kELEC * kELEQ * kELEQ * kNA * 1.0E-3;
  // intramolecular terms: one thread per molecule when the topology allows,
  // else the exclusion and bonded kernels
  float3 sL = fix_scale(b);
  const DfIntra &dfi = M.dfi;
  if (M.nmol > 0) {
    int mb = (M.nmol + 127) / 128;
    if (mb > 2048) mb = 2048;
#define FE_INTRA_ARGS                                                                           \
  M.nmol, M.mol_first, M.mol_x, M.mol_xi, M.mol_b, M.mol_bi, M.mol_a, M.mol_ai, M.excl_ab,        \
      M.excl_flag, b->bond_ab, b->bond_req, b->bond_k, b->bend_abc, b->bend_t0, b->bend_k,        \
      M.posfx, M.iperm, b->type, sL, b->nt, M.lj_tab, (float)(b->p.rc * b->p.rc),                 \
      (float)b->p.kappa, (float)(2.0 * b->p.kappa / sqrt(kPI)), (float)qf, (float)b->p.epsRF,     \
      b->pos_q, M.exptab, dfi, M.fix, facc, ticket, b->scal + SC_MX_INTRA
    if (M.uniform && M.tpl.ns == 3) {
      k_mx_intra_uni<3><<<mb, 128, 0, st>>>(
          M.nmol, M.tpl, M.posfx, M.iperm, sL, b->nt, M.lj_tab, (float)(b->p.rc * b->p.rc),
          (float)b->p.kappa, (float)(2.0 * b->p.kappa / sqrt(kPI)), (float)qf,
          (float)b->p.epsRF, b->pos_q, M.exptab, dfi, M.fix, facc, ticket,
          b->scal + SC_MX_INTRA);
    }
    else if (M.intra_maxs <= 3) k_mx_intra<3><<<mb, 128, 0, st>>>(FE_INTRA_ARGS);
    else if (M.intra_maxs <= 4) k_mx_intra<4><<<mb, 128, 0, st>>>(FE_INTRA_ARGS);
    else k_mx_intra<kIntraMaxSites><<<mb, 128, 0, st>>>(FE_INTRA_ARGS);
#undef FE_INTRA_ARGS
    FE_LAUNCH_CHECK("k_mx_intra");
  } else {
    int xb = (M.nexcl + 255) / 256;
    if (xb > 1024) xb = 1024;
    if (xb < 1) xb = 1;
    k_mx_excl<<<xb, 256, 0, st>>>(M.nexcl, M.excl_ab, M.excl_flag, M.posfx, M.iperm,
                                         b->type, sL, b->nt, M.lj_tab,
                                         (float)(b->p.rc * b->p.rc), (float)b->p.kappa,
                                         (float)(2.0 * b->p.kappa / sqrt(kPI)), (float)qf,
                                         (float)b->p.epsRF, b->pos_q, M.exptab, dfi, M.fix,
                                         facc, ticket, b->scal + SC_MX_EXCL);
    FE_LAUNCH_CHECK("k_mx_excl");
    int tot = b->nbond + b->nbend;
    int bb = (tot + 255) / 256;
    if (bb > 1024) bb = 1024;
    if (bb < 1) bb = 1;
    const double3 sd = make_double3((double)dfi.sl[0].x + (double)dfi.sl[0].y,
                                    (double)dfi.sl[1].x + (double)dfi.sl[1].y,
                                    (double)dfi.sl[2].x + (double)dfi.sl[2].y);
    k_mx_bonded<<<bb, 256, 0, st>>>(b->nbond, b->nbend, sL, sd, M.posfx, M.iperm, b->bond_ab,
                                           b->bond_req, b->bond_k, b->bend_abc, b->bend_t0,
                                           b->bend_k, M.fix, facc, ticket,
                                           b->scal + SC_BOND);
    FE_LAUNCH_CHECK("k_mx_bonded");
  }
  return FE_OK;
}

int forces_mixed(Box *b) {
  Mixed &M = *b->mx;
  int n = b->n;
  int rc;
  if ((rc = launch_convert(b, true))) return rc;  // also clears the force sums
  // reciprocal space on the second stream, beside the pair kernel (the
  // intramolecular terms there measured slower: they follow the pair kernel)
  FE_CUDA(cudaEventRecord(M.ev_fork, b->stream));
  FE_CUDA(cudaStreamWaitEvent(M.s2, M.ev_fork, 0));
  if ((rc = spme_on(b, M.s2, M.facc2, M.ticket2))) return rc;
  FE_CUDA(cudaEventRecord(M.ev_join, M.s2));
  if ((rc = launch_mx_pair_only(b))) return rc;
  if ((rc = intra_on(b, b->stream, b->facc, b->ticket))) return rc;
  // Urey-Bradley, torsions and impropers (FP64, into the fixed-point sums)
  if ((rc = launch_bonded_ext(b, true))) return rc;
  FE_CUDA(cudaStreamWaitEvent(b->stream, M.ev_join, 0));
  if (b->fold_tail) return FE_OK;  // finalised inside the second half kick
  k_mx_finalize<<<(3 * n + 255) / 256, 256, 0, b->stream>>>(n, M.fix, b->scal, b->ff);
  FE_LAUNCH_CHECK("k_mx_finalize");
  return launch_mixed_assemble(b);
}

// ---------------------------------------------------------------------------
// Replica batches: every box's force evaluation in one launch per kernel.
// Box r of a launch owns blocks off[r] .. off[r+1]-1 and runs the same kernel
// body as its own launch would, on its own buffers (the per-box arguments
// are kept in device memory); its reductions finish in its own last block.
// The grids of boxes of equal shape sit side by side so that one batched
// cuFFT plan transforms them all.

struct BMxArgs {
  int n, nt, nmol, order;
  const double4 *pos;
  const int *perm, *iperm, *type, *type_s;
  double3 invL;
  int4 *posfx;
  int4 *snap;
  float3 sc;
  MxPruneState *ps;
  unsigned long long *fix, *facc, *facc2;  // facc2 / ticket2: the reciprocal branch's
  unsigned *ticket, *ticket2;
  double *scal;
  int *status;
  // pair
  MxPair P;
  const int *cnt_lj, *cnt_nl, *ent;
  int *icnt_lj, *icnt_nl, *ient;
  const float *lj_tab;
  // intramolecular
  const int *mol_first, *mol_x, *mol_xi, *mol_b, *mol_bi, *mol_a, *mol_ai, *excl_ab, *excl_flag;
  const int *bond_ab, *bend_abc;
  const double *bond_req, *bond_k, *bend_t0, *bend_k;
  float rc2, kappa, c2k, qf, epsRF;
  const float2 *exptab;
  DfIntra D;
  // list rebuild
  int3 nc;
  int ncells;
  int *cell_count, *cell_start, *cell_fill, *cell_of, *cell_s;
  int *perm_w, *iperm_w, *type_s_w;
  float3 Lf;
  float rlist;
  const unsigned *lj_row;
  const unsigned char *lj_on;
  const int *x_start, *x_partner;
  int cap;
  int *cnt_lj_w, *cnt_nl_w, *ent_w;
  // SPME
  int3 G;
  long K, Kh;
  int *floor3;
  float *sm, *sd;
  unsigned long long *gfix;
  float *grid32;
  cufftComplex *grid32k;
  const float *eterm32, *kw32;
  float3 gl;
  float qfe;
  double *ff;
};

__global__ void k_b_mx_convert(const BMxArgs *__restrict__ A, const int *__restrict__ off,
                               int nbox) {
  const int r = vblk_box(off, nbox);
  const BMxArgs &a = A[r];
  const VBlk vb = vblk_of(off, r);
  int s = vb.id * blockDim.x + threadIdx.x;
  if (s < a.n) {  // the force sums start from zero (forces_mixed's memset)
    a.fix[3 * s] = 0ull;
    a.fix[3 * s + 1] = 0ull;
    a.fix[3 * s + 2] = 0ull;
  }
  k_mx_convert_body(vb, a.n, a.pos, a.perm, a.invL, a.posfx,
                    a.P.inner_on ? a.snap : nullptr, a.sc, &a.ps->dmax2);
}

template <bool PRUNE>
__global__ void __launch_bounds__(256, PRUNE ? 4 : 6)
k_b_mx_pair(const BMxArgs *__restrict__ A, const int *__restrict__ off, int nbox) {
  const int r = vblk_box(off, nbox);
  const BMxArgs &a = A[r];
  k_mx_pair_body<8, PRUNE ? 32 : 48, PRUNE>(
      vblk_of(off, r), a.P, a.posfx, a.type_s, a.perm, a.cnt_lj, a.cnt_nl, a.ent, a.icnt_lj,
      a.icnt_nl, a.ient, a.snap, a.ps, a.lj_tab, a.fix, a.facc, a.ticket, a.scal + SC_MX_PAIR,
      a.status);
}

template <int NS>
__global__ void k_b_mx_intra(const BMxArgs *__restrict__ A, const int *__restrict__ off,
                             int nbox) {
  const int r = vblk_box(off, nbox);
  const BMxArgs &a = A[r];
  k_mx_intra_body<NS>(vblk_of(off, r), a.nmol, a.mol_first, a.mol_x, a.mol_xi, a.mol_b, a.mol_bi,
                      a.mol_a, a.mol_ai, a.excl_ab, a.excl_flag, a.bond_ab, a.bond_req, a.bond_k,
                      a.bend_abc, a.bend_t0, a.bend_k, a.posfx, a.iperm, a.type, a.sc, a.nt,
                      a.lj_tab, a.rc2, a.kappa, a.c2k, a.qf, a.epsRF, a.pos, a.exptab, a.D, a.fix,
                      a.facc, a.ticket, a.scal + SC_MX_INTRA);
}

__global__ void k_b_mx_splines(const BMxArgs *__restrict__ A, const int *__restrict__ off,
                               int nbox) {
  const int r = vblk_box(off, nbox);
  const BMxArgs &a = A[r];
  k_mx_splines_body(vblk_of(off, r), a.n, a.order, a.G, a.posfx, a.floor3, a.sm, a.sd);
}

__global__ void k_b_mx_spread(const BMxArgs *__restrict__ A, const int *__restrict__ off,
                              int nbox) {
  const int r = vblk_box(off, nbox);
  const BMxArgs &a = A[r];
  k_mx_spread_red_body(vblk_of(off, r), a.n, a.order, a.G, a.posfx, a.sm, a.floor3, a.gfix);
}

__global__ void k_b_mx_spread_o4(const BMxArgs *__restrict__ A, const int *__restrict__ off,
                               int nbox) {
  const int r = vblk_box(off, nbox);
  const BMxArgs &a = A[r];
  k_mx_spread_o4_body(vblk_of(off, r), a.n, a.G, a.posfx, a.gfix);
}

__global__ void k_b_mx_gather_o4(const BMxArgs *__restrict__ A, const int *__restrict__ off,
                               int nbox) {
  const int r = vblk_box(off, nbox);
  const BMxArgs &a = A[r];
  k_mx_gather_o4_body(vblk_of(off, r), a.n, a.G, a.gl, a.qfe, a.posfx, a.perm, a.grid32, a.fix,
                    a.facc2, a.ticket2, a.scal + SC_FMEAN);
}

__global__ void k_b_mx_fix2grid(const BMxArgs *__restrict__ A, const int *__restrict__ off,
                                int nbox) {
  const int r = vblk_box(off, nbox);
  const BMxArgs &a = A[r];
  k_mx_fix2grid_body(vblk_of(off, r), a.K, a.gfix, a.grid32);
}

__global__ void k_b_mx_recip(const BMxArgs *__restrict__ A, const int *__restrict__ off,
                             int nbox) {
  const int r = vblk_box(off, nbox);
  const BMxArgs &a = A[r];
  k_mx_recip_body(vblk_of(off, r), a.Kh, a.eterm32, a.kw32, a.grid32k, a.facc2, a.ticket2,
                  a.scal + SC_ENREC);
}

__global__ void k_b_mx_gather(const BMxArgs *__restrict__ A, const int *__restrict__ off,
                              int nbox) {
  const int r = vblk_box(off, nbox);
  const BMxArgs &a = A[r];
  k_mx_gather_body(vblk_of(off, r), a.n, a.order, a.G, a.gl, a.qfe, a.posfx, a.perm, a.floor3,
                   a.sm, a.sd, a.grid32, a.fix, a.facc2, a.ticket2, a.scal + SC_FMEAN);
}

__global__ void k_b_mx_finalize(const BMxArgs *__restrict__ A, const int *__restrict__ off,
                                int nbox) {
  const int r = vblk_box(off, nbox);
  const BMxArgs &a = A[r];
  k_mx_finalize_body(vblk_of(off, r), a.n, a.fix, a.scal, a.ff);
}

// list rebuild of every box: cells, scan, fill, sort within cells, the
// fixed-point coordinates and the outer list (launch_mixed_list for each box)
__global__ void k_b_mx_cell(const BMxArgs *__restrict__ A, const int *__restrict__ off, int nbox) {
  const int r = vblk_box(off, nbox);
  const BMxArgs &a = A[r];
  k_mx_cell_body(vblk_of(off, r), a.n, a.pos, a.invL, a.nc, a.cell_of, a.cell_count);
}

// exclusive prefix of the cell counts (one block of 1024 threads per box,
// as k_cell_scan); fill counters cleared, counts cleared for the next build
__global__ void __launch_bounds__(1024) k_b_mx_scan(const BMxArgs *__restrict__ A) {
  const BMxArgs &a = A[blockIdx.x];
  int t = threadIdx.x, T = blockDim.x;
  int chunk = (a.ncells + T - 1) / T;
  int lo = min(t * chunk, a.ncells), hi = min(lo + chunk, a.ncells);
  int sum = 0;
  for (int c = lo; c < hi; c++) sum += a.cell_count[c];
  int total;
  int acc = block_exclusive_scan(sum, &total);
  if (t == 0) a.cell_start[a.ncells] = total;
  for (int c = lo; c < hi; c++) {
    a.cell_start[c] = acc;
    a.cell_fill[c] = 0;
    acc += a.cell_count[c];
    a.cell_count[c] = 0;
  }
}

__global__ void k_b_mx_fill(const BMxArgs *__restrict__ A, const int *__restrict__ off, int nbox) {
  const int r = vblk_box(off, nbox);
  const BMxArgs &a = A[r];
  k_mx_fill_body(vblk_of(off, r), a.n, a.cell_of, a.cell_start, a.cell_fill, a.perm_w);
}

__global__ void k_b_mx_cellsort(const BMxArgs *__restrict__ A, const int *__restrict__ off,
                                int nbox) {
  const int r = vblk_box(off, nbox);
  const BMxArgs &a = A[r];
  const VBlk vb = vblk_of(off, r);
  // the inner list and its snapshot belong to the old sort: prune next
  if (vb.id == 0 && threadIdx.x == 0) a.ps->need = 1;
  k_mx_cellsort_body(vb, a.cell_start, a.perm_w, a.iperm_w, a.cell_s, a.type, a.type_s_w,
                     a.status);
}

__global__ void k_b_mx_convert_only(const BMxArgs *__restrict__ A, const int *__restrict__ off,
                                    int nbox) {
  const int r = vblk_box(off, nbox);
  const BMxArgs &a = A[r];
  k_mx_convert_body(vblk_of(off, r), a.n, a.pos, a.perm, a.invL, a.posfx,
                    a.P.inner_on ? a.snap : nullptr, a.sc, &a.ps->dmax2);
}

__global__ void __launch_bounds__(kMxWarps * 32, kListBlocksPerSM)
k_b_mx_list(const BMxArgs *__restrict__ A, const int *__restrict__ off, int nbox) {
  const int r = vblk_box(off, nbox);
  const BMxArgs &a = A[r];
  k_mx_list_body(vblk_of(off, r), a.n, a.posfx, a.perm, a.iperm, a.cell_s, a.type_s,
                 a.cell_start, a.nc, a.sc, a.Lf, a.rlist, a.nt, a.lj_row, a.lj_on, a.x_start,
                 a.x_partner, a.cap, a.cnt_lj_w, a.cnt_nl_w, a.ent_w, a.status);
}

struct BMxGroup {
  int G[3];
  int count = 0;
  float *real = nullptr;
  cufftComplex *cplx = nullptr;
  cufftHandle r2c = 0, c2r = 0;
  bool plans = false;
};

// block offsets of one kernel over the batch (device copy)
struct BMxRange {
  int *d_off = nullptr;
  int total = 0;
};

struct BMxPlan {
  int nbox = 0;
  BMxArgs *d_args = nullptr;
  BMxRange convert, prune, pair, intra, splines, spread, fix2grid, recip, gather, finalize;
  BMxRange cell, fill, cellsort, list;
  int intra_ns = 3;
  bool order4 = true;  // every box has B-spline order 4: weights computed in place
  // the reciprocal branch's stream and its fork / join events
  cudaStream_t s2 = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  size_t pair_shm = 0;
  std::vector<BMxGroup> groups;
};

static int bmx_range(BMxRange &R, const std::vector<int> &blocks) {
  std::vector<int> off(blocks.size() + 1, 0);
  for (size_t r = 0; r < blocks.size(); r++) off[r + 1] = off[r] + blocks[r];
  R.total = off.back();
  FE_CUDA(cudaMalloc(&R.d_off, sizeof(int) * off.size()));
  FE_CUDA(cudaMemcpy(R.d_off, off.data(), sizeof(int) * off.size(), cudaMemcpyHostToDevice));
  return FE_OK;
}

void mixed_batch_free(BMxPlan *P) {
  if (!P) return;
  cudaFree(P->d_args);
  BMxRange *rs[] = {&P->convert, &P->prune, &P->pair, &P->intra, &P->splines, &P->spread,
                    &P->fix2grid, &P->recip, &P->gather, &P->finalize, &P->cell, &P->fill,
                    &P->cellsort, &P->list};
  for (BMxRange *r : rs) cudaFree(r->d_off);
  if (P->ev_fork) cudaEventDestroy(P->ev_fork);
  if (P->ev_join) cudaEventDestroy(P->ev_join);
  if (P->s2) cudaStreamDestroy(P->s2);
  for (BMxGroup &g : P->groups) {
    if (g.plans) {
      cufftDestroy(g.r2c);
      cufftDestroy(g.c2r);
    }
    cudaFree(g.real);
    cudaFree(g.cplx);
  }
  delete P;
}

unsigned long long *mixed_force_sums(Box *b) { return b->mx ? b->mx->fix : nullptr; }

void mixed_bint_fields(Box *b, BIntArgs *a) {
  if (!b->mx) return;
  a->erfc_rc_over_rc = b->mx->erfc_rc_over_rc;
  a->mixed_fused = b->mx->nmol > 0 ? 1 : 0;
}

// The batched force evaluation needs mixed-precision boxes whose molecules
// are contiguous runs of sites (the fused intramolecular kernel); otherwise
// FE_ERR_ARG and the batch steps box by box.
int mixed_batch_plan(Box *const *boxes, int nbox, BMxPlan **out) {
  *out = nullptr;
  for (int r = 0; r < nbox; r++)
    if (!boxes[r]->mx || boxes[r]->mx->nmol == 0 || boxes[r]->mx->intra_maxs > kIntraMaxSites) {
      set_error("batched force evaluation: mixed-precision boxes of contiguous molecules only");
      return FE_ERR_ARG;
    }
  for (int r = 0; r < nbox; r++)
    if (boxes[r]->nurey + boxes[r]->ntors + boxes[r]->nimpr > 0) {
      set_error("batched force evaluation: boxes with Urey-Bradley, torsion or improper terms "
                "run box by box");
      return FE_ERR_ARG;
    }
  BMxPlan *P = new BMxPlan();
  P->nbox = nbox;
  FE_CUDA(cudaStreamCreateWithFlags(&P->s2, cudaStreamNonBlocking));
  FE_CUDA(cudaEventCreateWithFlags(&P->ev_fork, cudaEventDisableTiming));
  FE_CUDA(cudaEventCreateWithFlags(&P->ev_join, cudaEventDisableTiming));
  std::vector<BMxArgs> args(nbox);
  std::vector<int> bconv, bprune, bpair, bintra, bspl, bspr, bf2g, brec, bgat, bfin;
  std::vector<int> bcell, bfill, bsort, blist;
  double qf = kELEC * kELEQ * kELEQ * kNA * 1.0E-3;
  int rc = FE_OK;
  for (int r = 0; r < nbox && rc == FE_OK; r++) {
    Box *b = boxes[r];
    Mixed &M = *b->mx;
    BMxArgs &a = args[r];
    memset(&a, 0, sizeof a);
    a.n = b->n;
    a.nt = b->nt;
    a.nmol = M.nmol;
    a.order = b->order;
    a.pos = b->pos_q;
    a.perm = M.perm;
    a.iperm = M.iperm;
    a.type = b->type;
    a.type_s = M.type_s;
    a.invL = make_double3(1.0 / b->p.L[0], 1.0 / b->p.L[1], 1.0 / b->p.L[2]);
    a.posfx = M.posfx;
    a.snap = M.snap;
    a.sc = fix_scale(b);
    a.ps = M.ps;
    a.fix = M.fix;
    a.facc = b->facc;
    a.ticket = b->ticket;
    a.facc2 = M.facc2;
    a.ticket2 = M.ticket2;
    a.scal = b->scal;
    a.status = b->status;
    a.P = mx_pair_params(b);
    a.cnt_lj = M.cnt_lj;
    a.cnt_nl = M.cnt_nl;
    a.ent = M.ent;
    a.icnt_lj = M.icnt_lj;
    a.icnt_nl = M.icnt_nl;
    a.ient = M.ient;
    a.lj_tab = M.lj_tab;
    a.mol_first = M.mol_first;
    a.mol_x = M.mol_x;
    a.mol_xi = M.mol_xi;
    a.mol_b = M.mol_b;
    a.mol_bi = M.mol_bi;
    a.mol_a = M.mol_a;
    a.mol_ai = M.mol_ai;
    a.excl_ab = M.excl_ab;
    a.excl_flag = M.excl_flag;
    a.bond_ab = b->bond_ab;
    a.bend_abc = b->bend_abc;
    a.bond_req = b->bond_req;
    a.bond_k = b->bond_k;
    a.bend_t0 = b->bend_t0;
    a.bend_k = b->bend_k;
    a.rc2 = (float)(b->p.rc * b->p.rc);
    a.kappa = (float)b->p.kappa;
    a.c2k = (float)(2.0 * b->p.kappa / sqrt(kPI));
    a.qf = (float)qf;
    a.epsRF = (float)b->p.epsRF;
    a.exptab = M.exptab;
    a.D = M.dfi;
    a.G = make_int3(b->G[0], b->G[1], b->G[2]);
    a.K = b->K;
    a.Kh = b->Kh;
    a.floor3 = M.floor3;
    a.sm = M.sm;
    a.sd = M.sd;
    a.gfix = M.gfix;
    a.eterm32 = M.eterm32;
    a.kw32 = M.kw32;
    a.gl = make_float3((float)(b->G[0] / b->p.L[0]), (float)(b->G[1] / b->p.L[1]),
                       (float)(b->G[2] / b->p.L[2]));
    a.qfe = (float)(qf / b->p.epsRF);
    a.ff = b->ff;
    a.nc = make_int3(M.nc[0], M.nc[1], M.nc[2]);
    a.ncells = M.ncells;
    a.cell_count = M.cell_count;
    a.cell_start = M.cell_start;
    a.cell_fill = M.cell_fill;
    a.cell_of = M.cell_of;
    a.cell_s = M.cell_s;
    a.perm_w = M.perm;
    a.iperm_w = M.iperm;
    a.type_s_w = M.type_s;
    a.Lf = make_float3((float)b->p.L[0], (float)b->p.L[1], (float)b->p.L[2]);
    a.rlist = (float)(b->p.rclist < b->p.rclist_ew ? b->p.rclist : b->p.rclist_ew);
    a.lj_row = M.lj_row;
    a.lj_on = M.lj_on;
    a.x_start = b->x_start;
    a.x_partner = b->x_partner;
    a.cap = M.cap;
    a.cnt_lj_w = M.cnt_lj;
    a.cnt_nl_w = M.cnt_nl;
    a.ent_w = M.ent;
    // the grid of equal shapes side by side (the group buffers are set below)
    int gi = -1;
    for (size_t g = 0; g < P->groups.size(); g++)
      if (P->groups[g].G[0] == b->G[0] && P->groups[g].G[1] == b->G[1] &&
          P->groups[g].G[2] == b->G[2])
        gi = (int)g;
    if (gi < 0) {
      P->groups.push_back(BMxGroup());
      gi = (int)P->groups.size() - 1;
      for (int d = 0; d < 3; d++) P->groups[gi].G[d] = b->G[d];
    }
    a.grid32 = reinterpret_cast<float *>((size_t)gi);                        // group index,
    a.grid32k = reinterpret_cast<cufftComplex *>((size_t)P->groups[gi].count);  // slot in it
    P->groups[gi].count++;
    if (M.intra_maxs > P->intra_ns) P->intra_ns = M.intra_maxs;
    size_t shm = sizeof(float) * (b->nt * b->nt * 3);
    if (shm > P->pair_shm) P->pair_shm = shm;
    int nsm = M.nsm > 0 ? M.nsm : 152;
    bconv.push_back((b->n + 255) / 256);
    bprune.push_back(std::max(1, std::min(4 * nsm, b->n / 160)));
    bpair.push_back(std::max(1, std::min(2048, b->n / 80)));
    bintra.push_back(std::min(2048, (M.nmol + 127) / 128));
    bspl.push_back((b->n + 127) / 128);
    bspr.push_back((int)(((long)b->n * b->order + 255) / 256));
    bf2g.push_back((int)std::min<long>(8L * nsm, (b->K / 2 + 255) / 256 + 1));
    brec.push_back((int)std::min<long>(1024L, (b->Kh + 255) / 256));
    bgat.push_back(std::min(1024, (b->n + 127) / 128));
    bfin.push_back((3 * b->n + 255) / 256);
    if (b->order != 4) P->order4 = false;
    bcell.push_back((b->n + 255) / 256);
    bfill.push_back((b->n + 255) / 256);
    bsort.push_back(M.ncells);
    int units = (b->n + kListUnit - 1) / kListUnit;
    int lb = (units + kMxWarps - 1) / kMxWarps;
    blist.push_back(std::max(1, std::min(lb, nsm * 8)));
  }
  // group buffers and batched plans; each box's grid points into its group.
  // Real grids start every Kpad floats (K rounded up to 4: 16-byte aligned,
  // as the grid kernels' paired float stores need for odd K).
  for (BMxGroup &g : P->groups) {
    if (rc) break;
    long K = (long)g.G[0] * g.G[1] * g.G[2], Kh = (long)g.G[0] * g.G[1] * (g.G[2] / 2 + 1);
    long Kpad = (K + 3) / 4 * 4;
    if (cudaMalloc(&g.real, sizeof(float) * Kpad * g.count) != cudaSuccess ||
        cudaMalloc(&g.cplx, sizeof(cufftComplex) * Kh * g.count) != cudaSuccess) {
      rc = cuda_fail(cudaGetLastError(), "batch grid buffers");
      break;
    }
    int nn[3] = {g.G[0], g.G[1], g.G[2]};
    int nh[3] = {g.G[0], g.G[1], g.G[2] / 2 + 1};
    cufftResult fr = cufftPlanMany(&g.r2c, 3, nn, nn, 1, (int)Kpad, nh, 1, (int)Kh, CUFFT_R2C,
                                   g.count);
    if (fr == CUFFT_SUCCESS)
      fr = cufftPlanMany(&g.c2r, 3, nn, nh, 1, (int)Kh, nn, 1, (int)Kpad, CUFFT_C2R, g.count);
    if (fr != CUFFT_SUCCESS) {
      rc = cufft_fail(fr, "cufftPlanMany (batch)");
      break;
    }
    g.plans = true;
  }
  if (rc == FE_OK)
    for (int r = 0; r < nbox; r++) {
      size_t gi = reinterpret_cast<size_t>(args[r].grid32);
      size_t slot = reinterpret_cast<size_t>(args[r].grid32k);
      BMxGroup &g = P->groups[gi];
      long K = (long)g.G[0] * g.G[1] * g.G[2], Kh = (long)g.G[0] * g.G[1] * (g.G[2] / 2 + 1);
      long Kpad = (K + 3) / 4 * 4;
      args[r].grid32 = g.real + slot * Kpad;
      args[r].grid32k = g.cplx + slot * Kh;
    }
  if (rc == FE_OK && cudaMalloc(&P->d_args, sizeof(BMxArgs) * nbox) != cudaSuccess)
    rc = cuda_fail(cudaGetLastError(), "batch arguments");
  if (rc == FE_OK &&
      cudaMemcpy(P->d_args, args.data(), sizeof(BMxArgs) * nbox, cudaMemcpyHostToDevice) !=
          cudaSuccess)
    rc = cuda_fail(cudaGetLastError(), "batch arguments");
  if (rc == FE_OK) rc = bmx_range(P->convert, bconv);
  if (rc == FE_OK) rc = bmx_range(P->prune, bprune);
  if (rc == FE_OK) rc = bmx_range(P->pair, bpair);
  if (rc == FE_OK) rc = bmx_range(P->intra, bintra);
  if (rc == FE_OK) rc = bmx_range(P->splines, bspl);
  if (rc == FE_OK) rc = bmx_range(P->spread, bspr);
  if (rc == FE_OK) rc = bmx_range(P->fix2grid, bf2g);
  if (rc == FE_OK) rc = bmx_range(P->recip, brec);
  if (rc == FE_OK) rc = bmx_range(P->gather, bgat);
  if (rc == FE_OK) rc = bmx_range(P->finalize, bfin);
  if (rc == FE_OK) rc = bmx_range(P->cell, bcell);
  if (rc == FE_OK) rc = bmx_range(P->fill, bfill);
  if (rc == FE_OK) rc = bmx_range(P->cellsort, bsort);
  if (rc == FE_OK) rc = bmx_range(P->list, blist);
  if (rc) {
    mixed_batch_free(P);
    return rc;
  }
  *out = P;
  return FE_OK;
}

// The list rebuild of every box (launch_mixed_list for each); the cell
// counts are zero on entry and left at zero by the scan.
int mixed_batch_list(BMxPlan *P, cudaStream_t s) {
  const int nb = P->nbox;
  k_b_mx_cell<<<P->cell.total, 256, 0, s>>>(P->d_args, P->cell.d_off, nb);
  FE_LAUNCH_CHECK("k_b_mx_cell");
  k_b_mx_scan<<<nb, 1024, 0, s>>>(P->d_args);
  FE_LAUNCH_CHECK("k_b_mx_scan");
  k_b_mx_fill<<<P->fill.total, 256, 0, s>>>(P->d_args, P->fill.d_off, nb);
  FE_LAUNCH_CHECK("k_b_mx_fill");
  k_b_mx_cellsort<<<P->cellsort.total, 32, 0, s>>>(P->d_args, P->cellsort.d_off, nb);
  FE_LAUNCH_CHECK("k_b_mx_cellsort");
  k_b_mx_convert_only<<<P->convert.total, 256, 0, s>>>(P->d_args, P->convert.d_off, nb);
  FE_LAUNCH_CHECK("k_b_mx_convert_only");
  k_b_mx_list<<<P->list.total, kMxWarps * 32, 0, s>>>(P->d_args, P->list.d_off, nb);
  FE_LAUNCH_CHECK("k_b_mx_list");
  return FE_OK;
}

// One force evaluation of every box (forces_mixed for each, energies
// assembled later by the batched second half kick).
int mixed_batch_forces(BMxPlan *P, cudaStream_t s) {
  const int nb = P->nbox;
  k_b_mx_convert<<<P->convert.total, 256, 0, s>>>(P->d_args, P->convert.d_off, nb);
  FE_LAUNCH_CHECK("k_b_mx_convert");
  // reciprocal space of every box on the second stream, beside the pair kernel
  cudaStream_t s2 = P->s2;
  FE_CUDA(cudaEventRecord(P->ev_fork, s));
  FE_CUDA(cudaStreamWaitEvent(s2, P->ev_fork, 0));
  if (P->order4) {
    k_b_mx_spread_o4<<<P->spread.total, 256, 0, s2>>>(P->d_args, P->spread.d_off, nb);
    FE_LAUNCH_CHECK("k_b_mx_spread_o4");
  } else {
    k_b_mx_splines<<<P->splines.total, 128, 0, s2>>>(P->d_args, P->splines.d_off, nb);
    FE_LAUNCH_CHECK("k_b_mx_splines");
    k_b_mx_spread<<<P->spread.total, 256, 0, s2>>>(P->d_args, P->spread.d_off, nb);
    FE_LAUNCH_CHECK("k_b_mx_spread");
  }
  k_b_mx_fix2grid<<<P->fix2grid.total, 256, 0, s2>>>(P->d_args, P->fix2grid.d_off, nb);
  FE_LAUNCH_CHECK("k_b_mx_fix2grid");
  for (BMxGroup &g : P->groups) {
    cufftResult r = cufftSetStream(g.r2c, s2);
    if (r == CUFFT_SUCCESS) r = cufftExecR2C(g.r2c, g.real, g.cplx);
    if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftExecR2C (batch)");
  }
  k_b_mx_recip<<<P->recip.total, 256, 0, s2>>>(P->d_args, P->recip.d_off, nb);
  FE_LAUNCH_CHECK("k_b_mx_recip");
  for (BMxGroup &g : P->groups) {
    cufftResult r = cufftSetStream(g.c2r, s2);
    if (r == CUFFT_SUCCESS) r = cufftExecC2R(g.c2r, g.cplx, g.real);
    if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftExecC2R (batch)");
  }
  if (P->order4) {
    k_b_mx_gather_o4<<<P->gather.total, 128, 0, s2>>>(P->d_args, P->gather.d_off, nb);
    FE_LAUNCH_CHECK("k_b_mx_gather_o4");
  } else {
    k_b_mx_gather<<<P->gather.total, 128, 0, s2>>>(P->d_args, P->gather.d_off, nb);
    FE_LAUNCH_CHECK("k_b_mx_gather");
  }
  FE_CUDA(cudaEventRecord(P->ev_join, s2));
  // real space and the intramolecular terms
  k_b_mx_pair<true><<<P->prune.total, 256, P->pair_shm, s>>>(P->d_args, P->prune.d_off, nb);
  FE_LAUNCH_CHECK("k_b_mx_pair<prune>");
  k_b_mx_pair<false><<<P->pair.total, 256, P->pair_shm, s>>>(P->d_args, P->pair.d_off, nb);
  FE_LAUNCH_CHECK("k_b_mx_pair");
  if (P->intra_ns <= 3) k_b_mx_intra<3><<<P->intra.total, 128, 0, s>>>(P->d_args, P->intra.d_off, nb);
  else if (P->intra_ns <= 4) k_b_mx_intra<4><<<P->intra.total, 128, 0, s>>>(P->d_args, P->intra.d_off, nb);
  else k_b_mx_intra<kIntraMaxSites><<<P->intra.total, 128, 0, s>>>(P->d_args, P->intra.d_off, nb);
  FE_LAUNCH_CHECK("k_b_mx_intra");
  FE_CUDA(cudaStreamWaitEvent(s, P->ev_join, 0));
  k_b_mx_finalize<<<P->finalize.total, 256, 0, s>>>(P->d_args, P->finalize.d_off, nb);
  FE_LAUNCH_CHECK("k_b_mx_finalize");
  return FE_OK;
}

int launch_mixed_assemble(Box *b) {
  k_mx_slots<<<1, 32, 0, b->stream>>>(b->scal, b->mx->erfc_rc_over_rc, b->mx->nmol > 0 ? 1 : 0);
  FE_LAUNCH_CHECK("k_mx_slots");
  return launch_assemble_energies(b, 1);
}

}  // namespace fe
