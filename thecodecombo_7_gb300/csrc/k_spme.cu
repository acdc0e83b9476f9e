// k_spme.cu -- FP64 smooth particle-mesh Ewald of pme_calc (pme_calc.c:18-279)
// on the device: B-spline weights (pme_spline.c:10-49, pme_qgrid.c:26-70),
// atom-free sorted spreading, cuFFT real<->complex transforms, the
// reciprocal-space convolution and the force gather with mean-force removal.
//
// Spreading is a gather: sites are binned by the grid cell of their spline
// origin (int)(ss) and each grid point sums the <= order^3 neighbouring bins
// in a fixed order (bins sorted by site index), so the grid is deterministic
// and needs no atomics.
//
// FFT: the reference transforms the real charge grid Q with FFTW_BACKWARD,
// scales by eterm (index 0 left alone), transforms FFTW_FORWARD and reads the
// real part.  For real Q that equals  real_out = C2R(eterm * R2C(Q))  with
// cuFFT's conventions (R2C: exp(-i...), C2R: exp(+i...), both unnormalised),
// which is what runs here on the half spectrum.  |S|^2 is the same for both
// signs, so the energy sum is unchanged (weight 2 for the mirrored half).
#include <cmath>
#include <vector>

#include "fe_device.cuh"

namespace fe {

constexpr int kMaxOrder = 8;

// pme_spline.c:10-49, same operation order; array/darray indices 0..order
__host__ __device__ inline void fillspline(int order, double w, double *array, double *darray) {
  for (int i = 3; i <= order; i++) array[i] = 0.0;
  array[2] = w;
  array[1] = 1.0 - w;
  array[0] = 0.0;
  for (int i = 3; i <= order - 1; i++) {
    double div = (double)(1.0 / (i - 1));
    array[i] = div * w * array[i - 1];
    double di = (double)(i);
    for (int j = 1; j <= (i - 2); j++) {
      double dj = (double)(j);
      array[i - j] = div * ((w + dj) * array[i - j - 1] + (di - dj - w) * array[i - j]);
    }
    array[1] *= div * (1.0 - w);
  }
  darray[0] = 0.0;
  darray[1] = -array[1];
  for (int i = 2; i <= order; i++) darray[i] = array[i - 1] - array[i];
  int kk = order;
  double div = (double)(1.0 / (kk - 1));
  array[kk] = div * w * array[kk - 1];
  double dkk = (double)(kk);
  for (int i = 1; i <= (kk - 2); i++) {
    double di = (double)(i);
    array[kk - i] = div * ((w + di) * array[kk - i - 1] + (dkk - di - w) * array[kk - i]);
  }
  array[1] *= div * (1.0 - w);
}

__device__ __forceinline__ int wrapg(int v, int g) {
  v %= g;
  return v < 0 ? v + g : v;
}

// per site: scaled coordinates, spline origin, weights and derivatives;
// bins the site under its origin cell
__global__ void k_splines(int n, int order, int3 G, double3 L, const double4 *__restrict__ pos,
                          int *__restrict__ floor3, double *__restrict__ sm,
                          double *__restrict__ sd, int gcap, int *__restrict__ bcount,
                          int *__restrict__ batoms, int *__restrict__ status) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double4 p = pos[i];
  double ssv[3];
  ssv[0] = G.x * (p.x / L.x + 0.5);  // pme_qgrid.c:27-33
  ssv[1] = G.y * (p.y / L.y + 0.5);
  ssv[2] = G.z * (p.z / L.z + 0.5);
  int g[3] = {G.x, G.y, G.z};
  int f[3];
  double mn[kMaxOrder + 1], dmn[kMaxOrder + 1];
  for (int d = 0; d < 3; d++) {
    f[d] = (int)(ssv[d]);
    double w = ssv[d] - (int)(ssv[d]);
    fillspline(order, w, mn, dmn);
    for (int m = 1; m <= order; m++) {
      sm[((size_t)i * order + (m - 1)) * 3 + d] = mn[m];
      sd[((size_t)i * order + (m - 1)) * 3 + d] = dmn[m];
    }
    floor3[3 * i + d] = f[d];
  }
  int cell = (wrapg(f[0], g[0]) * g[1] + wrapg(f[1], g[1])) * g[2] + wrapg(f[2], g[2]);
  int s = atomicAdd(&bcount[cell], 1);
  if (s < gcap) batoms[(size_t)cell * gcap + s] = i;
  else atomicOr(status, ST_GRID_OVERFLOW);
}

// order each bin by site index (bins hold a handful of sites)
__global__ void k_bin_sort(long K, int gcap, int *__restrict__ bcount, int *__restrict__ batoms) {
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

// grid point (x, y, z) receives w = mm[xi].x * mm[yi].y * mm[zi].z * q from each
// site whose origin is (x + order - xi, ...) (mod G), pme_qgrid.c:77-112
__global__ void k_spread(int order, int3 G, const double4 *__restrict__ pos,
                         const double *__restrict__ sm, int gcap, const int *__restrict__ bcount,
                         const int *__restrict__ batoms, double *__restrict__ grid) {
  long K = (long)G.x * G.y * G.z;
  long id = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= K) return;
  int z = (int)(id % G.z);
  int y = (int)((id / G.z) % G.y);
  int x = (int)(id / ((long)G.z * G.y));
  double sum = 0.0;
  for (int xi = 1; xi <= order; xi++) {
    int fx = wrapg(x + order - xi, G.x);
    for (int yi = 1; yi <= order; yi++) {
      int fy = wrapg(y + order - yi, G.y);
      for (int zi = 1; zi <= order; zi++) {
        int fz = wrapg(z + order - zi, G.z);
        long c = ((long)fx * G.y + fy) * G.z + fz;
        int m = bcount[c];
        const int *at = batoms + c * gcap;
        for (int s = 0; s < m; s++) {
          int j = at[s];
          double mxi = sm[((size_t)j * order + (xi - 1)) * 3 + 0];
          double myi = sm[((size_t)j * order + (yi - 1)) * 3 + 1];
          double mzi = sm[((size_t)j * order + (zi - 1)) * 3 + 2];
          sum += mxi * myi * mzi * pos[j].w;
        }
      }
    }
  }
  grid[id] = sum;
}

// half spectrum: energy sum and scaling by eterm (pme_calc.c:52-93)
__global__ void k_recip(long Kh, const double *__restrict__ eterm, const double *__restrict__ kw,
                        cufftDoubleComplex *__restrict__ gk, double *__restrict__ partials) {
  double e = 0.0;
  for (long h = (long)blockIdx.x * blockDim.x + threadIdx.x; h < Kh;
       h += (long)gridDim.x * blockDim.x) {
    cufftDoubleComplex v = gk[h];
    double et = eterm[h];
    double struc2 = v.x * v.x + v.y * v.y;
    e += kw[h] * (et * struc2);
    v.x *= et;
    v.y *= et;
    gk[h] = v;
  }
  double vv[1] = {e};
  block_partials<1>(vv, partials);
}

// pme_force (pme_calc.c:122-265): per-site gather from the convolved grid
__global__ void k_gather(int n, int order, int3 G, double3 L, double epsRF,
                         const double4 *__restrict__ pos, const int *__restrict__ floor3,
                         const double *__restrict__ sm, const double *__restrict__ sd,
                         const double *__restrict__ grid, double *__restrict__ fp,
                         double *__restrict__ partials) {
  double sx = 0.0, sy = 0.0, sz = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double fxi = 0.0, fyi = 0.0, fzi = 0.0;
    int xxo = floor3[3 * i] - order, yyo = floor3[3 * i + 1] - order,
        zzo = floor3[3 * i + 2] - order;
    const double *m = sm + (size_t)i * order * 3;
    const double *dm = sd + (size_t)i * order * 3;
    int xo = xxo;
    for (int xi = 1; xi <= order; xi++) {
      xo++;
      int x = wrapg(xo, G.x);
      double mxi = m[(xi - 1) * 3 + 0], dmxi = dm[(xi - 1) * 3 + 0];
      int yo = yyo;
      for (int yi = 1; yi <= order; yi++) {
        yo++;
        int y = wrapg(yo, G.y);
        double myi = m[(yi - 1) * 3 + 1], dmyi = dm[(yi - 1) * 3 + 1];
        int zo = zzo;
        for (int zi = 1; zi <= order; zi++) {
          zo++;
          int z = wrapg(zo, G.z);
          double mzi = m[(zi - 1) * 3 + 2], dmzi = dm[(zi - 1) * 3 + 2];
          double term = grid[((long)x * G.y + y) * G.z + z];
          fxi -= dmxi * myi * mzi * term;
          fyi -= mxi * dmyi * mzi * term;
          fzi -= mxi * myi * dmzi * term;
        }
      }
    }
    double fac = qfactor_mul(pos[i].w) / epsRF;
    fxi *= fac * G.x / L.x;
    fyi *= fac * G.y / L.y;
    fzi *= fac * G.z / L.z;
    fp[3 * i] = fxi;
    fp[3 * i + 1] = fyi;
    fp[3 * i + 2] = fzi;
    sx += fxi;
    sy += fyi;
    sz += fzi;
  }
  double v[3] = {sx, sy, sz};
  block_partials<3>(v, partials);
}

int spme_setup(Box *b) {
  int GX = b->p.grid[0], GY = b->p.grid[1], GZ = b->p.grid[2];
  b->G[0] = GX;
  b->G[1] = GY;
  b->G[2] = GZ;
  b->order = b->p.order;
  b->K = (long)GX * GY * GZ;
  b->Kh = (long)GX * GY * (GZ / 2 + 1);
  int order = b->order;
  // B-spline moduli (pme_setup.c:86-130), host arithmetic as the reference
  double mn[kMaxOrder + 2], dmn[kMaxOrder + 2];
  fillspline(order, 0.0, mn, dmn);
  int gm = GX > GY ? (GX > GZ ? GX : GZ) : (GY > GZ ? GY : GZ);
  std::vector<double> barr(gm + 8, 0.0);
  for (int i = 2; i <= order + 1; i++) barr[i] = mn[i - 1];
  auto dftmod = [&](int grid) {
    std::vector<double> bm(grid + 2, 0.0);
    double twopi = 2.0 * kPI;
    for (int i = 1; i <= grid; i++) {
      double sum1 = 0.0, sum2 = 0.0;
      for (int j = 1; j <= grid; j++) {
        double arg = twopi * (i - 1) * (j - 1) / grid;
        sum1 += barr[j] * cos(arg);
        sum2 += barr[j] * sin(arg);
      }
      bm[i] = sum1 * sum1 + sum2 * sum2;
    }
    return bm;
  };
  std::vector<double> bx = dftmod(GX), by = dftmod(GY), bz = dftmod(GZ);
  // eterm on the half spectrum (pme_calc.c:52-71)
  double blx = b->p.L[0], bly = b->p.L[1], blz = b->p.L[2];
  double vol = blx * bly * blz;
  double kap = b->p.kappa;
  double fac = kPI * kPI / kap / kap;
  int GZh = GZ / 2 + 1;
  std::vector<double> et(b->Kh), kw(b->Kh);
  for (int k1 = 0; k1 < GX; k1++)
    for (int k2 = 0; k2 < GY; k2++)
      for (int k3 = 0; k3 < GZh; k3++) {
        long h = ((long)k1 * GY + k2) * GZh + k3;
        if (k1 == 0 && k2 == 0 && k3 == 0) {
          et[h] = 1.0;  // the reference never scales index 0
          kw[h] = 0.0;
          continue;
        }
        int mx = k1 - (k1 > GX / 2 ? GX : 0);
        int my = k2 - (k2 > GY / 2 ? GY : 0);
        int mz = k3 - (k3 > GZ / 2 ? GZ : 0);
        double mhatx = mx / blx, mhaty = my / bly, mhatz = mz / blz;
        double mm = mhatx * mhatx + mhaty * mhaty + mhatz * mhatz;
        double bb = bx[k1 + 1] * by[k2 + 1] * bz[k3 + 1];
        double den = kPI * vol * mm * bb;
        et[h] = exp(-fac * mm) / den;
        kw[h] = (k3 == 0 || (GZ % 2 == 0 && k3 == GZ / 2)) ? 1.0 : 2.0;
      }
  FE_CUDA(cudaMalloc(&b->eterm, sizeof(double) * b->Kh));
  FE_CUDA(cudaMalloc(&b->kweight, sizeof(double) * b->Kh));
  FE_CUDA(cudaMemcpy(b->eterm, et.data(), sizeof(double) * b->Kh, cudaMemcpyHostToDevice));
  FE_CUDA(cudaMemcpy(b->kweight, kw.data(), sizeof(double) * b->Kh, cudaMemcpyHostToDevice));
  FE_CUDA(cudaMalloc(&b->grid, sizeof(double) * b->K));
  FE_CUDA(cudaMalloc(&b->grid_k, sizeof(cufftDoubleComplex) * b->Kh));
  FE_CUDA(cudaMalloc(&b->spl_floor, sizeof(int) * 3 * b->n));
  FE_CUDA(cudaMalloc(&b->spl_m, sizeof(double) * 3 * (size_t)b->n * order));
  FE_CUDA(cudaMalloc(&b->spl_d, sizeof(double) * 3 * (size_t)b->n * order));
  FE_CUDA(cudaMalloc(&b->fp, sizeof(double) * 3 * b->n));
  // bin capacity: ~ mean occupancy with a wide margin
  double cellvol = vol / (double)b->K;
  double mean = cellvol * (double)b->n / vol;
  int cap = (int)(8.0 * mean + 12.0);
  if (cap < 12) cap = 12;
  if (cap > 256) cap = 256;
  b->gcap = cap;
  FE_CUDA(cudaMalloc(&b->gbin_count, sizeof(int) * b->K));
  FE_CUDA(cudaMalloc(&b->gbin_atoms, sizeof(int) * (size_t)b->K * cap));
  cufftResult r = cufftPlan3d(&b->plan_r2c, GX, GY, GZ, CUFFT_D2Z);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftPlan3d D2Z");
  r = cufftPlan3d(&b->plan_c2r, GX, GY, GZ, CUFFT_Z2D);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftPlan3d Z2D");
  b->plans = true;
  return FE_OK;
}

int launch_charge_grid64(Box *b) {
  int3 G = make_int3(b->G[0], b->G[1], b->G[2]);
  double3 L = make_double3(b->p.L[0], b->p.L[1], b->p.L[2]);
  FE_CUDA(cudaMemsetAsync(b->gbin_count, 0, sizeof(int) * b->K, b->stream));
  k_splines<<<(b->n + 127) / 128, 128, 0, b->stream>>>(b->n, b->order, G, L, b->pos_q, b->spl_floor,
                                                       b->spl_m, b->spl_d, b->gcap, b->gbin_count,
                                                       b->gbin_atoms, b->status);
  FE_LAUNCH_CHECK("k_splines");
  k_bin_sort<<<(unsigned)((b->K + 255) / 256), 256, 0, b->stream>>>(b->K, b->gcap, b->gbin_count,
                                                                   b->gbin_atoms);
  FE_LAUNCH_CHECK("k_bin_sort");
  k_spread<<<(unsigned)((b->K + 127) / 128), 128, 0, b->stream>>>(
      b->order, G, b->pos_q, b->spl_m, b->gcap, b->gbin_count, b->gbin_atoms, b->grid);
  FE_LAUNCH_CHECK("k_spread");
  return FE_OK;
}

int launch_pme64(Box *b) {
  int rc = launch_charge_grid64(b);
  if (rc) return rc;
  cufftResult r = cufftSetStream(b->plan_r2c, b->stream);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftSetStream");
  r = cufftExecD2Z(b->plan_r2c, b->grid, b->grid_k);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftExecD2Z");
  int blocks = (int)((b->Kh + 255) / 256);
  if (blocks > 1024) blocks = 1024;
  k_recip<<<blocks, 256, 0, b->stream>>>(b->Kh, b->eterm, b->kweight, b->grid_k, b->partials);
  FE_LAUNCH_CHECK("k_recip");
  rc = launch_reduce(b, b->partials, blocks, 1, SC_ENREC, 1.0);
  if (rc) return rc;
  r = cufftSetStream(b->plan_c2r, b->stream);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftSetStream");
  r = cufftExecZ2D(b->plan_c2r, b->grid_k, b->grid);
  if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftExecZ2D");
  return launch_pme_gather64(b);
}

// pme_force (pme_calc.c:122-206): the reciprocal forces into fp from the
// convolved grid and the splines of the last charge_grid, their sum into
// SC_FMEAN (the mean removal is launch_apply_pme)
int launch_pme_gather64(Box *b) {
  int3 G = make_int3(b->G[0], b->G[1], b->G[2]);
  double3 L = make_double3(b->p.L[0], b->p.L[1], b->p.L[2]);
  int gb = (b->n + 127) / 128;
  if (gb > 1024) gb = 1024;
  k_gather<<<gb, 128, 0, b->stream>>>(b->n, b->order, G, L, b->p.epsRF, b->pos_q, b->spl_floor,
                                      b->spl_m, b->spl_d, b->grid, b->fp, b->partials);
  FE_LAUNCH_CHECK("k_gather");
  return launch_reduce(b, b->partials, gb, 3, SC_FMEAN, 1.0);
}

}  // namespace fe
