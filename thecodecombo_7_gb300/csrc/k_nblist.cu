// k_nblist.cu -- the Verlet-list build of nblist(ibox) (nblist.c:32-592) on
// the device.  Compiled with -fmad=false: the distance test below performs
// exactly the reference's roundings, so the pair set is bit-exact.
//
// Layout: a cell grid of nc[0] x nc[1] x nc[2] cells whose edge is at least
// max(rclist, rclist_ew), binned as CSR (count -> scan -> fill).  One warp per
// site a gathers every b > a from the (deduplicated, periodic) 27-cell
// neighbourhood that passes the reference's test, sorts the row by b in
// shared memory (bitonic) and writes it into the padded row
// nl_ent[a * max_nb ...] -- the layout of the reference's
// nlist[k].list[a][max_num_neighbors] -- with the xint flag packed as
// entry = b * 8 + xflag (nblist.c:149-183).
#include <climits>

#include "fe_device.cuh"

namespace fe {

constexpr int kListWarps = 4;        // warps per block
constexpr int kListBuf = 2048;       // candidates a warp can hold (per row)

__global__ void k_cell_count(const double4 *__restrict__ pos, int n, double3 L, int3 nc,
                             int *__restrict__ cell_of, int *__restrict__ cell_count) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double4 p = pos[i];
  int cx = (int)floor((p.x + 0.5 * L.x) / L.x * nc.x);
  int cy = (int)floor((p.y + 0.5 * L.y) / L.y * nc.y);
  int cz = (int)floor((p.z + 0.5 * L.z) / L.z * nc.z);
  cx = min(max(cx, 0), nc.x - 1);
  cy = min(max(cy, 0), nc.y - 1);
  cz = min(max(cz, 0), nc.z - 1);
  int c = (cx * nc.y + cy) * nc.z + cz;
  cell_of[i] = c;
  atomicAdd(&cell_count[c], 1);
}

// exclusive scan of cell_count into cell_start[0..ncells] (one block)
__global__ void k_cell_scan(const int *__restrict__ count, int ncells, int *__restrict__ start,
                            int *__restrict__ fill) {
  int t = threadIdx.x, T = blockDim.x;
  int chunk = (ncells + T - 1) / T;
  int lo = min(t * chunk, ncells), hi = min(lo + chunk, ncells);
  int s = 0;
  for (int c = lo; c < hi; c++) s += count[c];
  int total;
  int acc = block_exclusive_scan(s, &total);
  if (t == 0) start[ncells] = total;
  for (int c = lo; c < hi; c++) {
    start[c] = acc;
    fill[c] = 0;
    acc += count[c];
  }
}

__global__ void k_cell_fill(int n, const int *__restrict__ cell_of, const int *__restrict__ start,
                            int *__restrict__ fill, int *__restrict__ atoms) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int c = cell_of[i];
  int s = atomicAdd(&fill[c], 1);
  atoms[start[c] + s] = i;
}

__device__ __forceinline__ int excl_flag_of(const int *__restrict__ xs, const int *__restrict__ xp,
                                            const int *__restrict__ xf, int a, int b) {
  // the last matching xint entry wins, as in the hash scan of nblist.c:160-172
  int f = 0;
  for (int p = xs[a]; p < xs[a + 1]; p++)
    if (xp[p] == b) f = xf[p];
  return f;
}

__global__ void __launch_bounds__(kListWarps * 32)
k_list(const double4 *__restrict__ pos, int n, double3 L, double rcut, double rcut2,
       double rcut2_ew, int3 nc, const int *__restrict__ cell_of, const int *__restrict__ cstart,
       const int *__restrict__ catoms, const int *__restrict__ xs, const int *__restrict__ xp,
       const int *__restrict__ xf, int max_nb, int *__restrict__ count, int *__restrict__ ent,
       int *__restrict__ status) {
  __shared__ int sbuf[kListWarps][kListBuf];
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int *buf = sbuf[w];
  const double hx = L.x / 2.0, hy = L.y / 2.0, hz = L.z / 2.0;
  for (int a = blockIdx.x * kListWarps + w; a < n; a += gridDim.x * kListWarps) {
    double4 pa = pos[a];
    int ca = cell_of[a];
    int cz = ca % nc.z, cy = (ca / nc.z) % nc.y, cx = ca / (nc.z * nc.y);
    int nxs = nc.x >= 3 ? 3 : nc.x, nys = nc.y >= 3 ? 3 : nc.y, nzs = nc.z >= 3 ? 3 : nc.z;
    int cnt = 0;
    for (int ix = 0; ix < nxs; ix++) {
      int x = nc.x >= 3 ? (cx + ix - 1 + nc.x) % nc.x : ix;
      for (int iy = 0; iy < nys; iy++) {
        int y = nc.y >= 3 ? (cy + iy - 1 + nc.y) % nc.y : iy;
        for (int iz = 0; iz < nzs; iz++) {
          int z = nc.z >= 3 ? (cz + iz - 1 + nc.z) % nc.z : iz;
          int c = (x * nc.y + y) * nc.z + z;
          int s0 = cstart[c], s1 = cstart[c + 1];
          for (int base = s0; base < s1; base += 32) {
            int j = base + lane;
            bool ok = false;
            int b = 0;
            if (j < s1) {
              b = catoms[j];
              if (b > a) {
                // nblist.c:116-141, component rejections then dr2
                double4 pb = pos[b];
                double dx = fabs(pa.x - pb.x);
                if (dx > hx) dx -= L.x;
                if (!(dx > rcut)) {
                  double dy = fabs(pa.y - pb.y);
                  if (dy > hy) dy -= L.y;
                  if (!(dy > rcut)) {
                    double dz = fabs(pa.z - pb.z);
                    if (dz > hz) dz -= L.z;
                    if (!(dz > rcut)) {
                      double dr2 = dx * dx + dy * dy + dz * dz;
                      ok = (dr2 < rcut2_ew) && (dr2 < rcut2);  // nblist.c:145,178
                    }
                  }
                }
              }
            }
            unsigned m = __ballot_sync(0xffffffffu, ok);
            if (ok) {
              int p = cnt + __popc(m & ((1u << lane) - 1u));
              if (p < kListBuf) buf[p] = b;
            }
            cnt += __popc(m);
          }
        }
      }
    }
    __syncwarp();
    int mcount = cnt < kListBuf ? cnt : kListBuf;
    int P = 1;
    while (P < mcount) P <<= 1;
    for (int i = mcount + lane; i < P; i += 32) buf[i] = INT_MAX;
    __syncwarp();
    for (int k = 2; k <= P; k <<= 1) {
      for (int jj = k >> 1; jj > 0; jj >>= 1) {
        for (int i = lane; i < P; i += 32) {
          int ixj = i ^ jj;
          if (ixj > i) {
            int vi = buf[i], vj = buf[ixj];
            bool up = (i & k) == 0;
            if ((vi > vj) == up) {
              buf[i] = vj;
              buf[ixj] = vi;
            }
          }
        }
        __syncwarp();
      }
    }
    int rowlen = mcount < max_nb ? mcount : max_nb;
    if (cnt > max_nb || cnt > kListBuf) {
      if (lane == 0) atomicOr(status, ST_LIST_OVERFLOW);
    }
    int *row = ent + (size_t)a * max_nb;
    for (int i = lane; i < rowlen; i += 32) {
      int b = buf[i];
      row[i] = b * 8 + excl_flag_of(xs, xp, xf, a, b);
    }
    if (lane == 0) count[a] = rowlen;
    __syncwarp();
  }
}

void k_cell_scan_ext(const int *count, int ncells, int *start, int *fill, cudaStream_t s) {
  k_cell_scan<<<1, 1024, 0, s>>>(count, ncells, start, fill);
  ++g_launches;
}

int nblist_setup(Box *b) {
  double cut = b->p.rclist > b->p.rclist_ew ? b->p.rclist : b->p.rclist_ew;
  cut *= (1.0 + 1e-9);
  b->ncells = 1;
  for (int d = 0; d < 3; d++) {
    int m = (int)(b->p.L[d] / cut);
    b->nc[d] = m < 1 ? 1 : m;
    b->ncells *= b->nc[d];
  }
  FE_CUDA(cudaMalloc(&b->cell_count, sizeof(int) * b->ncells));
  FE_CUDA(cudaMalloc(&b->cell_start, sizeof(int) * (b->ncells + 1)));
  FE_CUDA(cudaMalloc(&b->cell_fill, sizeof(int) * b->ncells));
  FE_CUDA(cudaMalloc(&b->cell_atoms, sizeof(int) * b->n));
  FE_CUDA(cudaMalloc(&b->cell_of, sizeof(int) * b->n));
  int mnb = b->p.max_neighbors;
  if (mnb <= 0) mnb = b->n < 2000 ? b->n : 1500;  // allocate.c:321-322
  if (mnb > kListBuf) mnb = kListBuf;
  if (mnb < 1) mnb = 1;
  b->max_nb = mnb;
  FE_CUDA(cudaMalloc(&b->nl_count, sizeof(int) * b->n));
  FE_CUDA(cudaMalloc(&b->nl_ent, sizeof(int) * (size_t)b->n * mnb));
  FE_CUDA(cudaMemsetAsync(b->nl_count, 0, sizeof(int) * b->n, b->stream));
  return FE_OK;
}

// nblist.c:607-647 (DLIST): whether any site of [lb, ub) has moved more than
// (rclist - rc) / 4 from its position at the last list build, along one axis
// or in distance, with the reference's per-axis image rule (|d| > half box:
// subtract the box length)
__global__ void k_nl_check(int lb, int ub, double3 L, double3 H, double rcut, double rcut2,
                           const double4 *__restrict__ pos, const double4 *__restrict__ pos0,
                           int *__restrict__ flag) {
  int i = lb + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ub) return;
  double4 p = pos[i], q = pos0[i];
  double dx = fabs(p.x - q.x);
  if (dx > H.x) dx -= L.x;
  double dy = fabs(p.y - q.y);
  if (dy > H.y) dy -= L.y;
  double dz = fabs(p.z - q.z);
  if (dz > H.z) dz -= L.z;
  if (dx > rcut || dy > rcut || dz > rcut || dx * dx + dy * dy + dz * dz > rcut2) atomicOr(flag, 1);
}

int launch_nl_check(Box *b, int lb, int ub, int *dflag) {
  if (ub <= lb) return FE_OK;
  double3 L = make_double3(b->p.L[0], b->p.L[1], b->p.L[2]);
  double3 H = make_double3(b->p.L[0] / 2.0, b->p.L[1] / 2.0, b->p.L[2] / 2.0);
  double rcut = (b->p.rclist - b->p.rc) / 4.0;
  k_nl_check<<<(ub - lb + 255) / 256, 256, 0, b->stream>>>(lb, ub, L, H, rcut, rcut * rcut,
                                                           b->pos_q, b->pos_list0, dflag);
  FE_LAUNCH_CHECK("k_nl_check");
  return FE_OK;
}

int launch_nblist(Box *b) {
  int n = b->n;
  double3 L = make_double3(b->p.L[0], b->p.L[1], b->p.L[2]);
  int3 nc = make_int3(b->nc[0], b->nc[1], b->nc[2]);
  FE_CUDA(cudaMemsetAsync(b->cell_count, 0, sizeof(int) * b->ncells, b->stream));
  k_cell_count<<<(n + 255) / 256, 256, 0, b->stream>>>(b->pos_q, n, L, nc, b->cell_of, b->cell_count);
  FE_LAUNCH_CHECK("k_cell_count");
  k_cell_scan<<<1, 1024, 0, b->stream>>>(b->cell_count, b->ncells, b->cell_start, b->cell_fill);
  FE_LAUNCH_CHECK("k_cell_scan");
  k_cell_fill<<<(n + 255) / 256, 256, 0, b->stream>>>(n, b->cell_of, b->cell_start, b->cell_fill,
                                                      b->cell_atoms);
  FE_LAUNCH_CHECK("k_cell_fill");
  double rcut = b->p.rclist;
  double rcut2 = b->p.rclist * b->p.rclist;
  double rcut2_ew = b->p.rclist_ew * b->p.rclist_ew;
  int blocks = (n + kListWarps - 1) / kListWarps;
  if (blocks > 152 * 16) blocks = 152 * 16;
  k_list<<<blocks, kListWarps * 32, 0, b->stream>>>(
      b->pos_q, n, L, rcut, rcut2, rcut2_ew, nc, b->cell_of, b->cell_start, b->cell_atoms,
      b->x_start, b->x_partner, b->x_flag, b->max_nb, b->nl_count, b->nl_ent, b->status);
  FE_LAUNCH_CHECK("k_list");
  b->have_list = true;
  return FE_OK;
}

}  // namespace fe
