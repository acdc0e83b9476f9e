// k_noalloc.cu -- classic-Ewald reciprocal-space energy for callers that
// cannot allocate device memory.
//
// Some hosts of this engine do not own device memory: the MC driver may run
// inside a larger program whose device memory is handed out by another
// allocator (a framework's caching allocator, or a pool reserved once at
// start-up under a fixed memory budget), and that program forbids its plug-ins
// from calling cudaMalloc/cudaFree behind its back.  Such a caller can still
// pass device buffers it got from its own allocator, but every temporary must
// come from somewhere else.  This entry point takes the sites and the output
// from the caller and keeps its only temporary -- one partial sum per
// candidate k-vector -- in a file-scope __device__ array of fixed size, so it
// performs no allocation of any kind (no cudaMalloc, no cudaFree, no library
// routine that allocates).
//
// The array lives in every GPU that loads this library until the process
// exits.  All calls share it and it keeps the last call's contents; each
// call writes every slot it later reads, so nothing has to start at zero.
// Two calls whose kernels overlap on the GPU (different streams, or
// different host threads on one device) race on the array and must be
// serialised by the caller.  The first call on each device must come before
// any stream capture (its address lookup may load the module).  Host
// pointers are refused on the host (FE_ERR_ARG) before anything is launched.
#include <cmath>
#include <cstdint>
#include <mutex>

#include "fe_device.cuh"

namespace fe {

// candidate k-vectors of one call: (kmax+1) * (2 kmax+1)^2 <= this
constexpr int kNoAllocMaxK = 8192;
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) double g_kspace_partial[kNoAllocMaxK];

// device addresses of g_kspace_partial from the last lookup on each device
// (used inside stream captures)
static double *g_partial_addr[kNoAllocMaxDevices];
static bool g_partial_ready[kNoAllocMaxDevices];
static std::mutex g_partial_mu;

// one block per candidate (kx, ky, kz) of ewald.c:104-118; the block sums
// S(k) = sum_i q_i exp(i k.r_i) in a fixed order and writes
// w_k * kvec_k * |S(k)|^2 * fconv (w = 1 on the kx = 0 plane, 2 above it,
// ewald_mc.c:186-287), or 0 for a vector outside the sphere
__global__ void k_na_kspace(const double *__restrict__ xyzq, int n, double3 L, double kappa,
                            int kmax, int mks, double *__restrict__ partial) {
  int b = blockIdx.x;
  int side = 2 * kmax + 1;
  int kz = b % side - kmax;
  int ky = (b / side) % side - kmax;
  int kx = b / (side * side);
  int ksq = kx * kx + ky * ky + kz * kz;
  bool on = ksq <= mks && ksq != 0;
  __shared__ double shr[256], shi[256];
  double sr = 0.0, si = 0.0;
  const double two_pi = 2.0 * kPI;
  double gx = two_pi * (double)kx / L.x, gy = two_pi * (double)ky / L.y,
         gz = two_pi * (double)kz / L.z;
  if (on) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const double *p = xyzq + 4 * (size_t)i;
      double s, c;
      sincos(gx * p[0] + gy * p[1] + gz * p[2], &s, &c);
      sr += p[3] * c;
      si += p[3] * s;
    }
  }
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
  if (threadIdx.x == 0) {
    double e = 0.0;
    if (on) {
      double rksq = gx * gx + gy * gy + gz * gz;
      double vol = L.x * L.y * L.z;
      double kvec = two_pi * exp(-(0.25 / (kappa * kappa)) * rksq) / rksq / vol;
      double fconv = (kELEC * kELEQ * kELEQ * kNA * 0.001);
      e = (kx == 0 ? 1.0 : 2.0) * kvec * (shr[0] * shr[0] + shi[0] * shi[0]) * fconv;
    }
    partial[b] = e;
  }
}

// fixed-order sum of the per-k partials into the caller's output
__global__ void k_na_sum(const double *__restrict__ partial, int nb, double *__restrict__ out) {
  __shared__ double sh[256];
  double s = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) s += partial[b];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

// Device address of the scratch array in the current context.  Outside a
// stream capture it is looked up on every call (a symbol lookup allocates
// nothing), so a context that the host program reset or replaced since the
// last call gets the address of its own copy of the array.  Inside a capture
// the lookup is not made (the first lookup in a context may load the module,
// which a capture forbids) and the address of the last lookup on this device
// is used: the first call on each device must come before any capture.
static int scratch_for_current_device(cudaStream_t s, double **out) {
  int dev = 0;
  FE_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoAllocMaxDevices) {
    set_error("fe_ewald_kspace_energy_noalloc: device ordinal beyond 63");
    return FE_ERR_SIZE;
  }
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaError_t ce = cudaStreamIsCapturing(s, &cap);
  if (ce != cudaSuccess) {
    cudaGetLastError();
    cap = cudaStreamCaptureStatusActive;  // cannot tell: do nothing a capture forbids
  }
  std::lock_guard<std::mutex> lock(g_partial_mu);
  if (cap == cudaStreamCaptureStatusNone) {
    void *ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_kspace_partial);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_kspace_partial)");
    g_partial_addr[dev] = static_cast<double *>(ptr);
    g_partial_ready[dev] = true;
  } else if (!g_partial_ready[dev]) {
    set_error("fe_ewald_kspace_energy_noalloc: first call on this device inside a stream "
              "capture (make one call before capturing)");
    return FE_ERR_STATE;
  }
  *out = g_partial_addr[dev];
  return FE_OK;
}

// The caller's buffers must be device memory: a host pointer handed to the
// kernels would fault the GPU, so it is refused here, on the host.
static bool is_device_buffer(const void *p, size_t align) {
  if (reinterpret_cast<uintptr_t>(p) % align != 0) return false;
  cudaPointerAttributes a;
  cudaError_t e = cudaPointerGetAttributes(&a, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

}  // namespace fe

using namespace fe;

extern "C" int fe_ewald_kspace_energy_noalloc(const double *xyzq, int n, const double *L,
                                              double kappa, int kmax, int max_k_square,
                                              double *energy, void *stream) {
  if (!xyzq || !L || !energy || n < 1 || kmax < 1 || max_k_square < 1 || !(kappa > 0.0) ||
      !(L[0] > 0.0) || !(L[1] > 0.0) || !(L[2] > 0.0)) {
    set_error("fe_ewald_kspace_energy_noalloc: need device xyzq and energy, n >= 1, "
              "kmax >= 1, max_k_square >= 1, kappa > 0, L > 0");
    return FE_ERR_ARG;
  }
  // (kmax+1)(2kmax+1)^2 <= 8192 holds exactly for kmax <= 12; test kmax first
  // so that the product below cannot overflow
  long nb = kmax <= 12 ? ((long)kmax + 1) * (2L * kmax + 1) * (2L * kmax + 1) : kNoAllocMaxK + 1L;
  if (nb > kNoAllocMaxK) {
    set_error("fe_ewald_kspace_energy_noalloc: (kmax+1)*(2*kmax+1)^2 exceeds 8192 "
              "candidate k-vectors (kmax <= 12)");
    return FE_ERR_SIZE;
  }
  if (!is_device_buffer(xyzq, alignof(double)) || !is_device_buffer(energy, alignof(double))) {
    set_error("fe_ewald_kspace_energy_noalloc: xyzq and energy must be 8-byte aligned device "
              "(or managed) memory");
    return FE_ERR_ARG;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  double *partial = nullptr;
  int rc = scratch_for_current_device(s, &partial);
  if (rc) return rc;
  double3 Ld = make_double3(L[0], L[1], L[2]);
  k_na_kspace<<<(unsigned)nb, 256, 0, s>>>(xyzq, n, Ld, kappa, kmax, max_k_square, partial);
  FE_LAUNCH_CHECK("k_na_kspace");
  k_na_sum<<<1, 256, 0, s>>>(partial, (int)nb, energy);
  FE_LAUNCH_CHECK("k_na_sum");
  return FE_OK;
}
