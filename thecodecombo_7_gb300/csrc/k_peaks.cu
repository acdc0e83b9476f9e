// k_peaks.cu -- measured arithmetic peaks of the device the engine runs on:
// FP32 FMA, FP64 FMA and the special-function unit (ex2.approx), the
// denominators of the pipe fractions reported for the pair, SPME and
// integrator kernels.  No counterpart in the reference.
//
// Each thread runs kChains independent dependency chains so that the
// pipeline of every SM sub-partition stays full; the grid is a whole number
// of waves (SMs x resident blocks).  The operands keep every chain finite
// (a <- a*b + c with |b| < 1 converges), and the result is stored so that
// nothing is eliminated.
#include "fe_internal.h"

namespace fe {

constexpr int kChains = 8;

template <typename T>
__global__ void __launch_bounds__(256) k_peak_fma(int iters, T b, T c, T *__restrict__ out) {
  T a[kChains];
#pragma unroll
  for (int k = 0; k < kChains; k++) a[k] = (T)(threadIdx.x + k) * (T)1e-3;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int u = 0; u < 16; u++)
#pragma unroll
      for (int k = 0; k < kChains; k++) a[k] = fma(a[k], b, c);
  }
  T s = 0;
#pragma unroll
  for (int k = 0; k < kChains; k++) s += a[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// one special-function op and one FP32 multiply per step of each chain
__global__ void __launch_bounds__(256) k_peak_mufu(int iters, float b, float *__restrict__ out) {
  float a[kChains];
#pragma unroll
  for (int k = 0; k < kChains; k++) a[k] = -1e-3f * (float)(threadIdx.x + k);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int u = 0; u < 16; u++)
#pragma unroll
      for (int k = 0; k < kChains; k++) a[k] = -ex2_approx(a[k]) * b;
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < kChains; k++) s += a[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace fe

using namespace fe;

// which: 0 FP32 FMA, 1 FP64 FMA (TFLOP/s, an FMA counted as 2), 2 ex2.approx
// (Tops/s).  Best of three timed launches after one warm-up.
extern "C" int fe_pipe_peak(int device, int which, double *tera_per_s) {
  if (!tera_per_s || which < 0 || which > 2) {
    set_error("fe_pipe_peak: which in 0..2 and a result pointer");
    return FE_ERR_ARG;
  }
  FE_CUDA(cudaSetDevice(device));
  int nsm = 0;
  FE_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device));
  const int threads = 256, blocks = nsm * 8;
  const int iters = which == 1 ? 64 : 2048;
  void *out = nullptr;
  FE_CUDA(cudaMalloc(&out, sizeof(double) * blocks * threads));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  int rc = FE_OK;
  for (int r = 0; r < 4 && rc == FE_OK; r++) {
    cudaEventRecord(e0, 0);
    if (which == 0)
      k_peak_fma<float><<<blocks, threads>>>(iters, 0.999f, 1e-3f, static_cast<float *>(out));
    else if (which == 1)
      k_peak_fma<double><<<blocks, threads>>>(iters, 0.999, 1e-3, static_cast<double *>(out));
    else
      k_peak_mufu<<<blocks, threads>>>(iters, 0.5f, static_cast<float *>(out));
    cudaEventRecord(e1, 0);
    cudaError_t e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
      rc = cuda_fail(e, "fe_pipe_peak");
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (r > 0 && ms < best) best = ms;  // launch 0 is the warm-up
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (rc) return rc;
  double ops = (double)blocks * threads * iters * 16.0 * kChains * (which == 2 ? 1.0 : 2.0);
  *tera_per_s = ops / (best * 1e-3) / 1e12;
  return FE_OK;
}
