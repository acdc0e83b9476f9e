// k_mlp.cu -- the Monte Carlo surrogate network, trained and evaluated with
// hand-written BF16-in / FP32-accumulate kernels; every matrix product runs
// on the 5th-generation tensor cores (tcgen05.mma, accumulator in tensor
// memory).
//
// Network: g(x) = w3 . silu(W2 silu(W1 x' + b1) + b2) + b3 with 64 inputs,
// two hidden layers of 128 and one output; x' = (x - mean) / std per input.
// A trial move is scored by the difference g(x_new) - g(x_old) of its
// descriptors after and before the move, which makes the predicted energy
// change antisymmetric under reversing the move (what the delayed-acceptance
// second stage relies on).  Training minimises the mean squared error of
// that difference against the exact reciprocal-space energy change with
// Adam (Kingma & Ba 2015).
//
// GEMM kernel: one CTA of 4 warps computes a 128 x N tile of D = A B^T
// (A: M x K, B: N x K, both bf16 with K contiguous; D fp32).  K is streamed
// through shared memory in chunks of 64; thread 0 issues the MMAs (K = 16
// each) and commits them to an mbarrier that all threads wait on (bounded),
// then each warp reads its 32 accumulator rows from tensor memory.
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "fe_internal.h"
#include "fe_rng.cuh"
#include "fe_tc.cuh"

namespace fe {

constexpr int kMlpIn = 64, kMlpH = 128;
constexpr int kOffW1 = 0, kOffB1 = kOffW1 + kMlpH * kMlpIn, kOffW2 = kOffB1 + kMlpH,
              kOffB2 = kOffW2 + kMlpH * kMlpH, kOffW3 = kOffB2 + kMlpH, kOffB3 = kOffW3 + kMlpH,
              kMlpParams = kOffB3 + 1;
constexpr int kTcKc = 64;  // K per shared-memory chunk
constexpr long kTcWaitPolls = 1L << 20;

typedef __nv_bfloat16 bf16;

// ---------------------------------------------------------------------------
// D[M x N] (row stride ldd) = A[M x K] B[N x K]^T + bias; M % 128 == 0,
// N in {32, 64, 96, 128, ..., 256}, K % 64 == 0; rows 16-byte aligned.
__global__ void __launch_bounds__(128) k_gemm_tc(const bf16 *__restrict__ A, int lda,
                                                 const bf16 *__restrict__ B, int ldb,
                                                 const float *__restrict__ bias,
                                                 float *__restrict__ D, int ldd, int N, int K,
                                                 int *__restrict__ err) {
  extern __shared__ __align__(1024) unsigned char tc_smem[];
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_base;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * 128;
  const uint32_t ncols = N <= 32 ? 32u : N <= 64 ? 64u : N <= 128 ? 128u : 256u;
  unsigned char *sA = tc_smem;
  unsigned char *sB = tc_smem + 128 * kTcKc * 2;
  if (warp == 0) {
    tc::tmem_alloc(tc::smem_u32(&tmem_base), ncols);
    tc::tmem_relinquish();
  }
  if (tid == 0) tc::mbar_init(tc::smem_u32(&mbar), 1);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_base;
  const uint32_t idesc = tc::idesc_bf16_f32(128, N);
  uint32_t phase = 0;
  bool ok = true;
  for (int k0 = 0; k0 < K && ok; k0 += kTcKc) {
    for (int u = tid; u < 128 * (kTcKc / 8); u += blockDim.x) {
      int r = u / (kTcKc / 8), c = u % (kTcKc / 8);
      uint4 v = *reinterpret_cast<const uint4 *>(A + (size_t)(m0 + r) * lda + k0 + c * 8);
      *reinterpret_cast<uint4 *>(sA + tc::tile_offset(r, c * 8, kTcKc)) = v;
    }
    for (int u = tid; u < N * (kTcKc / 8); u += blockDim.x) {
      int r = u / (kTcKc / 8), c = u % (kTcKc / 8);
      uint4 v = *reinterpret_cast<const uint4 *>(B + (size_t)r * ldb + k0 + c * 8);
      *reinterpret_cast<uint4 *>(sB + tc::tile_offset(r, c * 8, kTcKc)) = v;
    }
    tc::fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc::fence_after_sync();
#pragma unroll
      for (int ks = 0; ks < kTcKc / 16; ks++) {
        uint64_t ad = tc::smem_desc(tc::smem_u32(sA) + ks * 2 * tc::kLbo, tc::kLbo,
                                    tc::sbo_bytes(kTcKc));
        uint64_t bd = tc::smem_desc(tc::smem_u32(sB) + ks * 2 * tc::kLbo, tc::kLbo,
                                    tc::sbo_bytes(kTcKc));
        tc::mma_bf16(tmem, ad, bd, idesc, (k0 > 0 || ks > 0) ? 1u : 0u);
      }
      tc::mma_commit(tc::smem_u32(&mbar));
    }
    // the chunk buffers are rewritten next: wait for the MMAs to finish
    ok = tc::mbar_wait(tc::smem_u32(&mbar), phase, kTcWaitPolls);
    phase ^= 1u;
    ok = __syncthreads_and(ok ? 1 : 0) != 0;
  }
  if (ok) {
    tc::fence_after_sync();
    const int row = m0 + warp * 32 + lane;
    for (int cg = 0; cg < N / 32; cg++) {
      float v[32];
      tc::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(cg * 32), v);
      float *d = D + (size_t)row * ldd + cg * 32;
#pragma unroll
      for (int j = 0; j < 32; j++) d[j] = v[j] + (bias ? bias[cg * 32 + j] : 0.f);
    }
  } else {
    // give the tensor core a last bounded chance to finish before freeing its memory
    if (tid == 0) atomicExch(err, 1);
    tc::mbar_wait(tc::smem_u32(&mbar), phase ^ 1u, kTcWaitPolls);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

static int gemm_tc(cudaStream_t st, const bf16 *A, int lda, const bf16 *B, int ldb,
                   const float *bias, float *D, int ldd, int M, int N, int K, int *err) {
  if (M % 128 || N % 32 || N < 32 || N > 256 || K % kTcKc || lda % 8 || ldb % 8) {
    set_error("tensor-core GEMM: M % 128, N in 32..256 step 32, K % 64 and 8-element strides");
    return FE_ERR_ARG;
  }
  size_t smem = (size_t)(128 + N) * kTcKc * 2;
  static bool attr = false;
  if (!attr) {
    FE_CUDA(cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)((128 + 256) * kTcKc * 2)));
    attr = true;
  }
  k_gemm_tc<<<M / 128, 128, smem, st>>>(A, lda, B, ldb, bias, D, ldd, N, K, err);
  FE_LAUNCH_CHECK("k_gemm_tc");
  return FE_OK;
}

// ---------------------------------------------------------------------------
// training pipeline kernels

__device__ __forceinline__ float sigm(float z) { return 1.f / (1.f + __expf(-z)); }

// rows r < B are the "before" descriptors of sample idx[r], rows B + r the
// "after" ones; normalised, rounded to bf16, stored row-major and transposed
__global__ void k_mlp_pack(int B, const int *__restrict__ idx, const float *__restrict__ data,
                           const float *__restrict__ y, const float *__restrict__ mean,
                           const float *__restrict__ istd, bf16 *__restrict__ X,
                           bf16 *__restrict__ Xt, float *__restrict__ yb) {
  int R = 2 * B;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= R * kMlpIn) return;
  int r = t / kMlpIn, f = t % kMlpIn;
  int s = idx[r % B];
  float v = data[(size_t)s * 2 * kMlpIn + (r >= B ? kMlpIn : 0) + f];
  bf16 h = __float2bfloat16_rn((v - mean[f]) * istd[f]);
  X[(size_t)r * kMlpIn + f] = h;
  Xt[(size_t)f * R + r] = h;
  if (f == 0 && r < B) yb[r] = y[s];
}

__global__ void k_mlp_silu(int R, const float *__restrict__ Z, bf16 *__restrict__ H,
                           bf16 *__restrict__ Ht) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= R * kMlpH) return;
  int r = t / kMlpH, u = t % kMlpH;
  float z = Z[t];
  bf16 h = __float2bfloat16_rn(z * sigm(z));
  H[t] = h;
  if (Ht) Ht[(size_t)u * R + r] = h;
}

// output head and the loss gradient: one thread per sample s (rows s, B + s)
__global__ void k_mlp_head(int B, const float *__restrict__ Z2, const float *__restrict__ P,
                           const float *__restrict__ yb, float *__restrict__ out,
                           float *__restrict__ dout, float *__restrict__ err2) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= B) return;
  const float *w3 = P + kOffW3;
  float o[2];
  for (int h = 0; h < 2; h++) {
    const float *z = Z2 + (size_t)(s + h * B) * kMlpH;
    float acc = P[kOffB3];
    for (int u = 0; u < kMlpH; u++) acc = fmaf(w3[u], z[u] * sigm(z[u]), acc);
    o[h] = acc;
    out[s + h * B] = acc;
  }
  float e = (o[1] - o[0]) - yb[s];
  err2[s] = e * e;
  float g = 2.f * e / (float)B;
  dout[B + s] = g;
  dout[s] = -g;
}

// dZ2 = dout w3 silu'(Z2): fp32 row-major and bf16 row-major + transposed
__global__ void k_mlp_dz2(int R, const float *__restrict__ Z2, const float *__restrict__ P,
                          const float *__restrict__ dout, float *__restrict__ dZf,
                          bf16 *__restrict__ dZ, bf16 *__restrict__ dZt) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= R * kMlpH) return;
  int r = t / kMlpH, u = t % kMlpH;
  float z = Z2[t], sg = sigm(z);
  float g = dout[r] * P[kOffW3 + u] * sg * (1.f + z * (1.f - sg));
  dZf[t] = g;
  bf16 h = __float2bfloat16_rn(g);
  dZ[t] = h;
  dZt[(size_t)u * R + r] = h;
}

// dZ1 = dH1 silu'(Z1): fp32 row-major and bf16 transposed
__global__ void k_mlp_dz1(int R, const float *__restrict__ Z1, const float *__restrict__ dH,
                          float *__restrict__ dZf, bf16 *__restrict__ dZt) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= R * kMlpH) return;
  int r = t / kMlpH, u = t % kMlpH;
  float z = Z1[t], sg = sigm(z);
  float g = dH[t] * sg * (1.f + z * (1.f - sg));
  dZf[t] = g;
  dZt[(size_t)u * R + r] = __float2bfloat16_rn(g);
}

// column sums in a fixed order: bias gradients, dw3 and db3, the batch loss
__global__ void k_mlp_colsum(int R, int B, const float *__restrict__ dZ1f,
                             const float *__restrict__ dZ2f, const float *__restrict__ Z2,
                             const float *__restrict__ dout, const float *__restrict__ err2,
                             float *__restrict__ G, float *__restrict__ loss) {
  int u = threadIdx.x;  // blockDim = 128
  int which = blockIdx.x;
  float acc = 0.f;
  if (which == 0) {
    for (int r = 0; r < R; r++) acc += dZ1f[(size_t)r * kMlpH + u];
    G[kOffB1 + u] = acc;
  } else if (which == 1) {
    for (int r = 0; r < R; r++) acc += dZ2f[(size_t)r * kMlpH + u];
    G[kOffB2 + u] = acc;
  } else if (which == 2) {
    for (int r = 0; r < R; r++) {
      float z = Z2[(size_t)r * kMlpH + u];
      acc = fmaf(dout[r], z * sigm(z), acc);
    }
    G[kOffW3 + u] = acc;
  } else if (u == 0) {
    for (int r = 0; r < R; r++) acc += dout[r];
    G[kOffB3] = acc;
    float l = 0.f;
    for (int s = 0; s < B; s++) l += err2[s];
    *loss = l / (float)B;
  }
}

__global__ void k_mlp_adam(int n, float *__restrict__ P, const float *__restrict__ G,
                           float *__restrict__ m, float *__restrict__ v, float lr, float b1,
                           float b2, float c1, float c2, float eps) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float g = G[i];
  float mi = b1 * m[i] + (1.f - b1) * g;
  float vi = b2 * v[i] + (1.f - b2) * g * g;
  m[i] = mi;
  v[i] = vi;
  P[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// bf16 weight copies for the GEMMs: W1 [128 x 64], W2 [128 x 128], W2^T
__global__ void k_mlp_refresh(const float *__restrict__ P, bf16 *__restrict__ W1b,
                              bf16 *__restrict__ W2b, bf16 *__restrict__ W2tb) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < kMlpH * kMlpIn) W1b[t] = __float2bfloat16_rn(P[kOffW1 + t]);
  if (t < kMlpH * kMlpH) {
    int j = t / kMlpH, i = t % kMlpH;
    bf16 h = __float2bfloat16_rn(P[kOffW2 + t]);
    W2b[t] = h;
    W2tb[(size_t)i * kMlpH + j] = h;
  }
}

// ---------------------------------------------------------------------------

struct Mlp {
  int dev = 0;
  cudaStream_t st = nullptr;
  int cap = 0;  // rows (2B) capacity
  float *P = nullptr, *G = nullptr, *Am = nullptr, *Av = nullptr;
  long long step = 0;
  float *mean = nullptr, *istd = nullptr;
  bf16 *W1b = nullptr, *W2b = nullptr, *W2tb = nullptr;
  bf16 *X = nullptr, *Xt = nullptr, *H1 = nullptr, *H1t = nullptr, *dZ2 = nullptr,
       *dZ2t = nullptr, *dZ1t = nullptr;
  float *Z1 = nullptr, *Z2 = nullptr, *dZ2f = nullptr, *dH1 = nullptr, *dZ1f = nullptr;
  float *out = nullptr, *dout = nullptr, *err2 = nullptr, *yb = nullptr, *loss = nullptr;
  int *idx = nullptr, *err = nullptr;
  float *data = nullptr, *y = nullptr;  // uploaded samples
  long long ndata = 0, data_cap = 0;
};

static void mlp_free_buffers(Mlp *m) {
  void *p[] = {m->X, m->Xt, m->H1, m->H1t, m->dZ2, m->dZ2t, m->dZ1t, m->Z1, m->Z2, m->dZ2f,
               m->dH1, m->dZ1f, m->out, m->dout, m->err2, m->yb, m->idx};
  for (void *q : p)
    if (q) cudaFree(q);
  m->X = m->Xt = m->H1 = m->H1t = m->dZ2 = m->dZ2t = m->dZ1t = nullptr;
  m->Z1 = m->Z2 = m->dZ2f = m->dH1 = m->dZ1f = m->out = m->dout = m->err2 = m->yb = nullptr;
  m->idx = nullptr;
  m->cap = 0;
}

static void mlp_free(Mlp *m) {
  mlp_free_buffers(m);
  void *p[] = {m->P, m->G, m->Am, m->Av, m->mean, m->istd, m->W1b, m->W2b, m->W2tb,
               m->loss, m->err, m->data, m->y};
  for (void *q : p)
    if (q) cudaFree(q);
  if (m->st) cudaStreamDestroy(m->st);
}

static int mlp_reserve(Mlp *m, int R) {
  if (R <= m->cap) return FE_OK;
  mlp_free_buffers(m);
  size_t rh = (size_t)R * kMlpH, ri = (size_t)R * kMlpIn;
  FE_CUDA(cudaMalloc(&m->X, ri * 2));
  FE_CUDA(cudaMalloc(&m->Xt, ri * 2));
  FE_CUDA(cudaMalloc(&m->H1, rh * 2));
  FE_CUDA(cudaMalloc(&m->H1t, rh * 2));
  FE_CUDA(cudaMalloc(&m->dZ2, rh * 2));
  FE_CUDA(cudaMalloc(&m->dZ2t, rh * 2));
  FE_CUDA(cudaMalloc(&m->dZ1t, rh * 2));
  FE_CUDA(cudaMalloc(&m->Z1, rh * 4));
  FE_CUDA(cudaMalloc(&m->Z2, rh * 4));
  FE_CUDA(cudaMalloc(&m->dZ2f, rh * 4));
  FE_CUDA(cudaMalloc(&m->dH1, rh * 4));
  FE_CUDA(cudaMalloc(&m->dZ1f, rh * 4));
  FE_CUDA(cudaMalloc(&m->out, (size_t)R * 4));
  FE_CUDA(cudaMalloc(&m->dout, (size_t)R * 4));
  FE_CUDA(cudaMalloc(&m->err2, (size_t)R * 4));
  FE_CUDA(cudaMalloc(&m->yb, (size_t)R * 4));
  FE_CUDA(cudaMalloc(&m->idx, (size_t)R * 4));
  m->cap = R;
  return FE_OK;
}

static int mlp_refresh(Mlp *m) {
  k_mlp_refresh<<<(kMlpH * kMlpH + 255) / 256, 256, 0, m->st>>>(m->P, m->W1b, m->W2b, m->W2tb);
  FE_LAUNCH_CHECK("k_mlp_refresh");
  return FE_OK;
}

static int mlp_create(Mlp *m, int dev, uint64_t seed) {
  m->dev = dev;
  FE_CUDA(cudaSetDevice(dev));
  FE_CUDA(cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking));
  FE_CUDA(cudaMalloc(&m->P, sizeof(float) * kMlpParams));
  FE_CUDA(cudaMalloc(&m->G, sizeof(float) * kMlpParams));
  FE_CUDA(cudaMalloc(&m->Am, sizeof(float) * kMlpParams));
  FE_CUDA(cudaMalloc(&m->Av, sizeof(float) * kMlpParams));
  FE_CUDA(cudaMalloc(&m->mean, sizeof(float) * kMlpIn));
  FE_CUDA(cudaMalloc(&m->istd, sizeof(float) * kMlpIn));
  FE_CUDA(cudaMalloc(&m->W1b, 2 * kMlpH * kMlpIn));
  FE_CUDA(cudaMalloc(&m->W2b, 2 * kMlpH * kMlpH));
  FE_CUDA(cudaMalloc(&m->W2tb, 2 * kMlpH * kMlpH));
  FE_CUDA(cudaMalloc(&m->loss, sizeof(float)));
  FE_CUDA(cudaMalloc(&m->err, sizeof(int)));
  FE_CUDA(cudaMemset(m->err, 0, sizeof(int)));
  FE_CUDA(cudaMemset(m->G, 0, sizeof(float) * kMlpParams));
  FE_CUDA(cudaMemset(m->Am, 0, sizeof(float) * kMlpParams));
  FE_CUDA(cudaMemset(m->Av, 0, sizeof(float) * kMlpParams));
  // Glorot-uniform weights from Philox draws, zero biases, identity normalisation
  std::vector<float> P(kMlpParams, 0.f), mean(kMlpIn, 0.f), istd(kMlpIn, 1.f);
  auto fill = [&](int off, int fan_out, int fan_in, uint32_t tag) {
    float a = sqrtf(6.f / (float)(fan_in + fan_out));
    for (int i = 0; i < fan_out * fan_in; i++)
      P[off + i] = (float)((2.0 * fe_uniform(seed, tag, (uint64_t)i, 0) - 1.0) * a);
  };
  fill(kOffW1, kMlpH, kMlpIn, 0x4D4C5031u);
  fill(kOffW2, kMlpH, kMlpH, 0x4D4C5032u);
  fill(kOffW3, 1, kMlpH, 0x4D4C5033u);
  FE_CUDA(cudaMemcpy(m->P, P.data(), sizeof(float) * kMlpParams, cudaMemcpyHostToDevice));
  FE_CUDA(cudaMemcpy(m->mean, mean.data(), sizeof(float) * kMlpIn, cudaMemcpyHostToDevice));
  FE_CUDA(cudaMemcpy(m->istd, istd.data(), sizeof(float) * kMlpIn, cudaMemcpyHostToDevice));
  int rc = mlp_refresh(m);
  if (rc) return rc;
  FE_CUDA(cudaStreamSynchronize(m->st));
  return FE_OK;
}

// forward + backward of one batch (indices already in m->idx); gradients in m->G
static int mlp_fwd_bwd(Mlp *m, int B, const float *data, const float *y) {
  int R = 2 * B, rc;
  cudaStream_t st = m->st;
  int nb = (R * kMlpIn + 255) / 256, nh = (R * kMlpH + 255) / 256;
  k_mlp_pack<<<nb, 256, 0, st>>>(B, m->idx, data, y, m->mean, m->istd, m->X, m->Xt, m->yb);
  FE_LAUNCH_CHECK("k_mlp_pack");
  if ((rc = gemm_tc(st, m->X, kMlpIn, m->W1b, kMlpIn, m->P + kOffB1, m->Z1, kMlpH, R, kMlpH,
                    kMlpIn, m->err)))
    return rc;
  k_mlp_silu<<<nh, 256, 0, st>>>(R, m->Z1, m->H1, m->H1t);
  FE_LAUNCH_CHECK("k_mlp_silu");
  if ((rc = gemm_tc(st, m->H1, kMlpH, m->W2b, kMlpH, m->P + kOffB2, m->Z2, kMlpH, R, kMlpH,
                    kMlpH, m->err)))
    return rc;
  k_mlp_head<<<(B + 127) / 128, 128, 0, st>>>(B, m->Z2, m->P, m->yb, m->out, m->dout, m->err2);
  FE_LAUNCH_CHECK("k_mlp_head");
  k_mlp_dz2<<<nh, 256, 0, st>>>(R, m->Z2, m->P, m->dout, m->dZ2f, m->dZ2, m->dZ2t);
  FE_LAUNCH_CHECK("k_mlp_dz2");
  // dW2 = dZ2^T H1 ; dH1 = dZ2 W2
  if ((rc = gemm_tc(st, m->dZ2t, R, m->H1t, R, nullptr, m->G + kOffW2, kMlpH, kMlpH, kMlpH, R,
                    m->err)))
    return rc;
  if ((rc = gemm_tc(st, m->dZ2, kMlpH, m->W2tb, kMlpH, nullptr, m->dH1, kMlpH, R, kMlpH, kMlpH,
                    m->err)))
    return rc;
  k_mlp_dz1<<<nh, 256, 0, st>>>(R, m->Z1, m->dH1, m->dZ1f, m->dZ1t);
  FE_LAUNCH_CHECK("k_mlp_dz1");
  // dW1 = dZ1^T X
  if ((rc = gemm_tc(st, m->dZ1t, R, m->Xt, R, nullptr, m->G + kOffW1, kMlpIn, kMlpH, kMlpIn, R,
                    m->err)))
    return rc;
  k_mlp_colsum<<<4, 128, 0, st>>>(R, B, m->dZ1f, m->dZ2f, m->Z2, m->dout, m->err2, m->G, m->loss);
  FE_LAUNCH_CHECK("k_mlp_colsum");
  return FE_OK;
}

static int mlp_check_err(Mlp *m) {
  int e = 0;
  FE_CUDA(cudaMemcpyAsync(&e, m->err, sizeof(int), cudaMemcpyDeviceToHost, m->st));
  FE_CUDA(cudaStreamSynchronize(m->st));
  if (e) {
    set_error("tensor-core GEMM: an MMA completion wait ran out");
    FE_CUDA(cudaMemset(m->err, 0, sizeof(int)));
    return FE_ERR_DEVICE;
  }
  return FE_OK;
}

static int mlp_upload(Mlp *m, const float *data, const float *y, long long n) {
  if (n > m->data_cap) {
    if (m->data) cudaFree(m->data);
    if (m->y) cudaFree(m->y);
    m->data = nullptr;
    m->y = nullptr;
    FE_CUDA(cudaMalloc(&m->data, sizeof(float) * 2 * kMlpIn * (size_t)n));
    FE_CUDA(cudaMalloc(&m->y, sizeof(float) * (size_t)n));
    m->data_cap = n;
  }
  FE_CUDA(cudaMemcpyAsync(m->data, data, sizeof(float) * 2 * kMlpIn * (size_t)n,
                          cudaMemcpyHostToDevice, m->st));
  FE_CUDA(cudaMemcpyAsync(m->y, y, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice, m->st));
  m->ndata = n;
  return FE_OK;
}

// Trains on n samples resident on the device (data: n x [64 before | 64
// after], y: n).  Epochs of shuffled batches (Philox permutation keys);
// loss_hist[e] = mean batch loss of epoch e.
int mlp_train_device(Mlp *m, const float *data, const float *y, long long n, int epochs, int B,
                     float lr, uint64_t seed, float *loss_hist) {
  if (B < 64 || B % 64 || n < B || epochs < 1) {
    set_error("fe_mlp_train: batch must be a multiple of 64 and at most the sample count");
    return FE_ERR_ARG;
  }
  int rc;
  if ((rc = mlp_reserve(m, 2 * B))) return rc;
  // per-feature normalisation from the samples (both halves)
  {
    std::vector<float> h((size_t)n * 2 * kMlpIn);
    FE_CUDA(cudaMemcpyAsync(h.data(), data, sizeof(float) * h.size(), cudaMemcpyDeviceToHost, m->st));
    FE_CUDA(cudaStreamSynchronize(m->st));
    std::vector<float> mean(kMlpIn), istd(kMlpIn);
    for (int f = 0; f < kMlpIn; f++) {
      double s = 0.0, s2 = 0.0;
      for (long long i = 0; i < 2 * n; i++) {
        double v = h[(size_t)(i / 2) * 2 * kMlpIn + (i & 1) * kMlpIn + f];
        s += v;
        s2 += v * v;
      }
      double mu = s / (2.0 * n), var = s2 / (2.0 * n) - mu * mu;
      mean[f] = (float)mu;
      istd[f] = (float)(var > 1e-12 ? 1.0 / sqrt(var) : 1.0);
    }
    FE_CUDA(cudaMemcpy(m->mean, mean.data(), sizeof(float) * kMlpIn, cudaMemcpyHostToDevice));
    FE_CUDA(cudaMemcpy(m->istd, istd.data(), sizeof(float) * kMlpIn, cudaMemcpyHostToDevice));
  }
  std::vector<int> perm((size_t)n);
  long long nbatch = n / B;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int e = 0; e < epochs; e++) {
    // Fisher-Yates with Philox draws
    for (long long i = 0; i < n; i++) perm[(size_t)i] = (int)i;
    for (long long i = n - 1; i > 0; i--) {
      long long j = (long long)(fe_uniform(seed, 0x50524D31u, (uint64_t)e * (uint64_t)n + i, 0) *
                                (double)(i + 1));
      if (j > i) j = i;
      std::swap(perm[(size_t)i], perm[(size_t)j]);
    }
    double lsum = 0.0;
    for (long long bi = 0; bi < nbatch; bi++) {
      FE_CUDA(cudaMemcpyAsync(m->idx, perm.data() + bi * B, sizeof(int) * B,
                              cudaMemcpyHostToDevice, m->st));
      if ((rc = mlp_fwd_bwd(m, B, data, y))) return rc;
      m->step++;
      float c1 = 1.f - powf(b1, (float)m->step), c2 = 1.f - powf(b2, (float)m->step);
      k_mlp_adam<<<(kMlpParams + 255) / 256, 256, 0, m->st>>>(kMlpParams, m->P, m->G, m->Am, m->Av,
                                                            lr, b1, b2, c1, c2, eps);
      FE_LAUNCH_CHECK("k_mlp_adam");
      if ((rc = mlp_refresh(m))) return rc;
      float l = 0.f;
      FE_CUDA(cudaMemcpyAsync(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->st));
      FE_CUDA(cudaStreamSynchronize(m->st));
      lsum += l;
    }
    if (loss_hist) loss_hist[e] = (float)(lsum / (double)nbatch);
  }
  return mlp_check_err(m);
}

}  // namespace fe

using namespace fe;

struct fe_mlp {
  Mlp m;
};

namespace fe {
Mlp *mlp_from_handle(fe_mlp *h) { return &h->m; }
}  // namespace fe

extern "C" {

int fe_mlp_create(fe_mlp **out, int device, uint64_t seed) {
  if (!out) return FE_ERR_ARG;
  fe_mlp *h = new fe_mlp();
  int rc = mlp_create(&h->m, device, seed);
  if (rc) {
    mlp_free(&h->m);
    delete h;
    return rc;
  }
  *out = h;
  return FE_OK;
}

void fe_mlp_destroy(fe_mlp *h) {
  if (!h) return;
  if (h->m.st) cudaStreamSynchronize(h->m.st);
  mlp_free(&h->m);
  delete h;
}

int fe_mlp_param_count(void) { return kMlpParams; }

int fe_mlp_set_params(fe_mlp *h, const float *params, const float *mean, const float *istd) {
  if (!h || !params) return FE_ERR_ARG;
  Mlp *m = &h->m;
  FE_CUDA(cudaMemcpyAsync(m->P, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice, m->st));
  if (mean)
    FE_CUDA(cudaMemcpyAsync(m->mean, mean, sizeof(float) * kMlpIn, cudaMemcpyHostToDevice, m->st));
  if (istd)
    FE_CUDA(cudaMemcpyAsync(m->istd, istd, sizeof(float) * kMlpIn, cudaMemcpyHostToDevice, m->st));
  int rc = mlp_refresh(m);
  if (rc) return rc;
  FE_CUDA(cudaStreamSynchronize(m->st));
  return FE_OK;
}

int fe_mlp_get_params(fe_mlp *h, float *params, float *mean, float *istd) {
  if (!h) return FE_ERR_ARG;
  Mlp *m = &h->m;
  if (params)
    FE_CUDA(cudaMemcpyAsync(params, m->P, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, m->st));
  if (mean)
    FE_CUDA(cudaMemcpyAsync(mean, m->mean, sizeof(float) * kMlpIn, cudaMemcpyDeviceToHost, m->st));
  if (istd)
    FE_CUDA(cudaMemcpyAsync(istd, m->istd, sizeof(float) * kMlpIn, cudaMemcpyDeviceToHost, m->st));
  FE_CUDA(cudaStreamSynchronize(m->st));
  return FE_OK;
}

// Gradient of the batch loss at the current parameters (no update): B
// samples of 128 inputs (64 before, 64 after) and targets y; B % 64 == 0.
int fe_mlp_grad(fe_mlp *h, const float *data, const float *y, int B, float *grad, float *loss,
                float *out2B) {
  if (!h || !data || !y || B < 64 || B % 64) return FE_ERR_ARG;
  Mlp *m = &h->m;
  int rc;
  if ((rc = mlp_reserve(m, 2 * B))) return rc;
  if ((rc = mlp_upload(m, data, y, B))) return rc;
  std::vector<int> id(B);
  for (int i = 0; i < B; i++) id[i] = i;
  FE_CUDA(cudaMemcpyAsync(m->idx, id.data(), sizeof(int) * B, cudaMemcpyHostToDevice, m->st));
  if ((rc = mlp_fwd_bwd(m, B, m->data, m->y))) return rc;
  if (grad)
    FE_CUDA(cudaMemcpyAsync(grad, m->G, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost, m->st));
  if (loss) FE_CUDA(cudaMemcpyAsync(loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->st));
  if (out2B)
    FE_CUDA(cudaMemcpyAsync(out2B, m->out, sizeof(float) * 2 * B, cudaMemcpyDeviceToHost, m->st));
  FE_CUDA(cudaStreamSynchronize(m->st));
  return mlp_check_err(m);
}

int fe_mlp_train(fe_mlp *h, const float *data, const float *y, int64_t n, int epochs, int batch,
                 float lr, uint64_t seed, float *loss_hist) {
  if (!h || !data || !y || n < 1) return FE_ERR_ARG;
  Mlp *m = &h->m;
  int rc;
  if ((rc = mlp_upload(m, data, y, n))) return rc;
  return mlp_train_device(m, m->data, m->y, n, epochs, batch, lr, seed, loss_hist);
}

// Test entry for the tensor-core GEMM alone: D = A B^T (+ bias), host arrays,
// A: M x K, B: N x K bf16 bit patterns, D: M x N fp32.
int fe_tc_gemm_bf16(const uint16_t *A, const uint16_t *B, const float *bias, float *D, int M,
                    int N, int K) {
  if (!A || !B || !D) return FE_ERR_ARG;
  bf16 *dA = nullptr, *dB = nullptr;
  float *dD = nullptr, *dbias = nullptr;
  int *derr = nullptr;
  int rc = FE_OK;
  cudaError_t e = cudaSuccess;
  do {
    if ((e = cudaMalloc(&dA, 2 * (size_t)M * K))) break;
    if ((e = cudaMalloc(&dB, 2 * (size_t)N * K))) break;
    if ((e = cudaMalloc(&dD, 4 * (size_t)M * N))) break;
    if ((e = cudaMalloc(&derr, sizeof(int)))) break;
    if ((e = cudaMemset(derr, 0, sizeof(int)))) break;
    if (bias && (e = cudaMalloc(&dbias, 4 * (size_t)N))) break;
    if ((e = cudaMemcpy(dA, A, 2 * (size_t)M * K, cudaMemcpyHostToDevice))) break;
    if ((e = cudaMemcpy(dB, B, 2 * (size_t)N * K, cudaMemcpyHostToDevice))) break;
    if (bias && (e = cudaMemcpy(dbias, bias, 4 * (size_t)N, cudaMemcpyHostToDevice))) break;
    rc = gemm_tc(0, dA, K, dB, K, dbias, dD, N, M, N, K, derr);
    if (rc) break;
    if ((e = cudaDeviceSynchronize())) break;
    int he = 0;
    if ((e = cudaMemcpy(&he, derr, sizeof(int), cudaMemcpyDeviceToHost))) break;
    if (he) {
      set_error("tensor-core GEMM: an MMA completion wait ran out");
      rc = FE_ERR_DEVICE;
      break;
    }
    e = cudaMemcpy(D, dD, 4 * (size_t)M * N, cudaMemcpyDeviceToHost);
  } while (0);
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dD);
  cudaFree(dbias);
  cudaFree(derr);
  if (e != cudaSuccess) return cuda_fail(e, "fe_tc_gemm_bf16");
  return rc;
}

}  // extern "C"
