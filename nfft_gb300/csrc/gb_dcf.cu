// gb_dcf.cu -- density-compensation weights for the inverse NFFT: the
// fixed-point iteration on the GPU transforms, per-node features, and a small
// MLP (8 -> 64 -> 64 -> 1, GELU, FP32) with hand-written forward, backward
// and Adam kernels that learns the weights from the features.
//
// No counterpart in the reference: the reference solver takes weights from
// the caller (solver_plan_complex::w with PRECOMPUTE_WEIGHT,
// kernel/solver/solver.c:69-70, 91-104).  The weights produced here are meant
// for exactly that field.
//
// Fixed point: w <- w / |A A^H w| (A = trafo, A^H = adjoint of the plan),
// started at w = 1.
// Features of node j (2-D): log(1 + c_r) for the number c_r of nodes in the
// (2r+1)^2 cells of the oversampled grid around the node's cell, r = 1, 2, 4;
// the radius 2|x_j|; cos / sin of its angle and of twice its angle.
// MLP parameters (floats): W1[8][64], b1[64], W2[64][64], b2[64], W3[64], b3.
#include <algorithm>
#include <cmath>

#include "../../include/nfft_gb300.h"
#include "gb_internal.h"

namespace gb {

static constexpr int F_IN = 8, H1 = 64, H2 = 64;
static constexpr int P_W1 = 0, P_B1 = P_W1 + F_IN * H1, P_W2 = P_B1 + H1, P_B2 = P_W2 + H1 * H2,
                     P_W3 = P_B2 + H2, P_B3 = P_W3 + H2, P_COUNT = P_B3 + 1;

__device__ __forceinline__ float gelu(float a) { return 0.5f * a * (1.f + erff(a * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float a)
{
  const float cdf = 0.5f * (1.f + erff(a * 0.70710678118654752f));
  const float pdf = 0.39894228040143268f * expf(-0.5f * a * a);
  return cdf + a * pdf;
}

// ---------------------------------------------------------------- features
__global__ void k_cell_counts(const float *__restrict__ x, int M, int n0, int n1, int *__restrict__ cnt)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= M) return;
  int c0 = (int)floorf((x[2 * j] + 0.5f) * n0);
  int c1 = (int)floorf((x[2 * j + 1] + 0.5f) * n1);
  c0 = wrap(c0, n0);
  c1 = wrap(c1, n1);
  atomicAdd(&cnt[c0 * n1 + c1], 1);
}

__global__ void k_features(const float *__restrict__ x, int M, int n0, int n1, const int *__restrict__ cnt,
                           float *__restrict__ feat)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= M) return;
  const float x0 = x[2 * j], x1 = x[2 * j + 1];
  const int c0 = wrap((int)floorf((x0 + 0.5f) * n0), n0);
  const int c1 = wrap((int)floorf((x1 + 0.5f) * n1), n1);
  const int radii[3] = {1, 2, 4};
  float *o = feat + (long long)j * F_IN;
  for (int q = 0; q < 3; ++q) {
    const int r = radii[q];
    int s = 0;
    for (int a = -r; a <= r; ++a)
      for (int b = -r; b <= r; ++b) s += cnt[wrap(c0 + a, n0) * n1 + wrap(c1 + b, n1)];
    o[q] = log1pf((float)s);
  }
  const float rad = sqrtf(x0 * x0 + x1 * x1);
  const float th = atan2f(x1, x0);
  o[3] = 2.f * rad;
  o[4] = cosf(th);
  o[5] = sinf(th);
  o[6] = cosf(2.f * th);
  o[7] = sinf(2.f * th);
}

// ---------------------------------------------------------------- MLP forward
static constexpr int MLP_THREADS = 128;

__global__ void __launch_bounds__(MLP_THREADS) k_mlp_forward(const float *__restrict__ params,
                                                             const float *__restrict__ feat, int M,
                                                             float *__restrict__ out)
{
  // the weights in shared memory, read four outputs at a time (one 16-byte
  // broadcast load feeds four FMAs; each output's sum keeps its order)
  __shared__ __align__(16) float P[P_COUNT];
  static_assert(P_W1 % 4 == 0 && P_W2 % 4 == 0 && H1 % 4 == 0 && H2 % 4 == 0, "16-byte weight rows");
  for (int i = threadIdx.x; i < P_COUNT; i += blockDim.x) P[i] = params[i];
  __syncthreads();
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < M; s += gridDim.x * blockDim.x) {
    float xin[F_IN];
#pragma unroll
    for (int i = 0; i < F_IN; ++i) xin[i] = feat[(long long)s * F_IN + i];
    float h1[H1];
#pragma unroll
    for (int k = 0; k < H1; k += 4) {
      float a0 = P[P_B1 + k], a1 = P[P_B1 + k + 1], a2 = P[P_B1 + k + 2], a3 = P[P_B1 + k + 3];
#pragma unroll
      for (int i = 0; i < F_IN; ++i) {
        const float4 w = *reinterpret_cast<const float4 *>(&P[P_W1 + i * H1 + k]);
        a0 += xin[i] * w.x;
        a1 += xin[i] * w.y;
        a2 += xin[i] * w.z;
        a3 += xin[i] * w.w;
      }
      h1[k] = gelu(a0);
      h1[k + 1] = gelu(a1);
      h1[k + 2] = gelu(a2);
      h1[k + 3] = gelu(a3);
    }
    float o = P[P_B3];
    for (int j = 0; j < H2; j += 4) {
      float a0 = P[P_B2 + j], a1 = P[P_B2 + j + 1], a2 = P[P_B2 + j + 2], a3 = P[P_B2 + j + 3];
#pragma unroll
      for (int k = 0; k < H1; ++k) {
        const float4 w = *reinterpret_cast<const float4 *>(&P[P_W2 + k * H2 + j]);
        a0 += h1[k] * w.x;
        a1 += h1[k] * w.y;
        a2 += h1[k] * w.z;
        a3 += h1[k] * w.w;
      }
      o += P[P_W3 + j] * gelu(a0);
      o += P[P_W3 + j + 1] * gelu(a1);
      o += P[P_W3 + j + 2] * gelu(a2);
      o += P[P_W3 + j + 3] * gelu(a3);
    }
    out[s] = o;
  }
}

// ---------------------------------------------------------------- MLP gradient
// Mean squared error 1/M sum (out - target)^2 and its gradient with respect to
// the parameters.  A CTA takes tiles of MLP_THREADS samples: every thread runs
// its sample forward and back and leaves x, h1, h2, dL/dpre1, dL/dpre2 and
// dL/dout in shared memory (one padded row per sample, so that the per-sample
// writes and the later column reads are both free of bank conflicts); the
// weight gradients are then contracted over the tile by the whole CTA, each
// thread owning every MLP_THREADS-th parameter and keeping its running sums
// in registers over all the CTA's tiles; the CTA adds them to the global
// gradient once.
static constexpr int G_SLICE = (P_COUNT + MLP_THREADS - 1) / MLP_THREADS;  // 38
static constexpr int SX = F_IN + 1, SH = H1 + 1;                           // padded row strides

__host__ __device__ constexpr int mlp_grad_smem_floats()
{
  return P_COUNT + MLP_THREADS * (SX + 4 * SH + 1);
}

__global__ void __launch_bounds__(MLP_THREADS) k_mlp_grad(const float *__restrict__ params,
                                                          const float *__restrict__ feat,
                                                          const float *__restrict__ target, int M,
                                                          float *__restrict__ grad, float *__restrict__ loss)
{
  extern __shared__ float sm[];
  float *P = sm;                        // parameters
  float *X = P + P_COUNT;               // [T][SX]  x
  float *Hh = X + MLP_THREADS * SX;     // [T][SH]  h1
  float *G2 = Hh + MLP_THREADS * SH;    // [T][SH]  h2
  float *D2 = G2 + MLP_THREADS * SH;    // [T][SH]  dL/dpre2
  float *D1 = D2 + MLP_THREADS * SH;    // [T][SH]  dL/dpre1
  float *DO = D1 + MLP_THREADS * SH;    // [T]      dL/dout
  __shared__ float red[MLP_THREADS / 32];
  const int tid = threadIdx.x;
  for (int i = tid; i < P_COUNT; i += blockDim.x) P[i] = params[i];
  float acc[G_SLICE];
#pragma unroll
  for (int q = 0; q < G_SLICE; ++q) acc[q] = 0.f;
  float lsum = 0.f;
  const float inv_m = 1.f / (float)M;
  __syncthreads();
  for (int t0 = blockIdx.x * MLP_THREADS; t0 < M; t0 += gridDim.x * MLP_THREADS) {
    const int s = t0 + tid;
    const bool valid = s < M;
    float xin[F_IN];
#pragma unroll
    for (int i = 0; i < F_IN; ++i) {
      xin[i] = valid ? feat[(long long)s * F_IN + i] : 0.f;
      X[tid * SX + i] = xin[i];
    }
    float pre1[H1], h1[H1];
#pragma unroll
    for (int k = 0; k < H1; ++k) {
      float a = P[P_B1 + k];
#pragma unroll
      for (int i = 0; i < F_IN; ++i) a += xin[i] * P[P_W1 + i * H1 + k];
      pre1[k] = a;
      h1[k] = gelu(a);
      Hh[tid * SH + k] = h1[k];
    }
    float o = P[P_B3];
    for (int j = 0; j < H2; ++j) {
      float a = P[P_B2 + j];
#pragma unroll
      for (int k = 0; k < H1; ++k) a += h1[k] * P[P_W2 + k * H2 + j];
      const float h2 = gelu(a);
      G2[tid * SH + j] = h2;
      D2[tid * SH + j] = a;  // pre2, turned into dL/dpre2 below
      o += P[P_W3 + j] * h2;
    }
    const float diff = valid ? (o - target[s]) : 0.f;
    lsum += diff * diff;
    const float dout = 2.f * diff * inv_m;
    DO[tid] = dout;
    for (int j = 0; j < H2; ++j) D2[tid * SH + j] = dout * P[P_W3 + j] * gelu_grad(D2[tid * SH + j]);
#pragma unroll
    for (int k = 0; k < H1; ++k) {
      float a = 0.f;
      for (int j = 0; j < H2; ++j) a += P[P_W2 + k * H2 + j] * D2[tid * SH + j];
      D1[tid * SH + k] = a * gelu_grad(pre1[k]);
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < G_SLICE; ++q) {
      const int p = tid + q * MLP_THREADS;
      if (p >= P_COUNT) break;
      float g = 0.f;
      if (p < P_B1) {  // W1[i][k] = sum_r x[r][i] dpre1[r][k]
        const int i = p / H1, k = p - i * H1;
        for (int r = 0; r < MLP_THREADS; ++r) g += X[r * SX + i] * D1[r * SH + k];
      } else if (p < P_W2) {  // b1[k]
        const int k = p - P_B1;
        for (int r = 0; r < MLP_THREADS; ++r) g += D1[r * SH + k];
      } else if (p < P_B2) {  // W2[k][j] = sum_r h1[r][k] dpre2[r][j]
        const int k = (p - P_W2) / H2, j = (p - P_W2) - k * H2;
        for (int r = 0; r < MLP_THREADS; ++r) g += Hh[r * SH + k] * D2[r * SH + j];
      } else if (p < P_W3) {  // b2[j]
        const int j = p - P_B2;
        for (int r = 0; r < MLP_THREADS; ++r) g += D2[r * SH + j];
      } else if (p < P_B3) {  // W3[j] = sum_r dout[r] h2[r][j]
        const int j = p - P_W3;
        for (int r = 0; r < MLP_THREADS; ++r) g += DO[r] * G2[r * SH + j];
      } else {  // b3
        for (int r = 0; r < MLP_THREADS; ++r) g += DO[r];
      }
      acc[q] += g;
    }
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < G_SLICE; ++q) {
    const int p = tid + q * MLP_THREADS;
    if (p < P_COUNT) atomicAdd(&grad[p], acc[q]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_down_sync(0xffffffffu, lsum, o);
  if ((tid & 31) == 0) red[tid >> 5] = lsum;
  __syncthreads();
  if (tid == 0) {
    float t = 0.f;
    for (int i = 0; i < MLP_THREADS / 32; ++i) t += red[i];
    atomicAdd(loss, t * inv_m);
  }
}

__global__ void k_adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m1,
                       float *__restrict__ m2, int n, float lr, float b1, float b2, float eps, float c1, float c2)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float a = b1 * m1[i] + (1.f - b1) * gi;
  const float b = b2 * m2[i] + (1.f - b2) * gi * gi;
  m1[i] = a;
  m2[i] = b;
  p[i] -= lr * (a / c1) / (sqrtf(b / c2) + eps);
}

// ---------------------------------------------------------------- fixed point
__global__ void k_real_to_complex(const float *__restrict__ w, float2 *__restrict__ f, int M)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < M) f[j] = make_float2(w[j], 0.f);
}

__global__ void k_dcf_update(float *__restrict__ w, const float2 *__restrict__ f, int M)
{
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= M) return;
  const float a = sqrtf(f[j].x * f[j].x + f[j].y * f[j].y);
  w[j] = a > 0.f ? w[j] / a : w[j];
}

}  // namespace gb

using namespace gb;

extern "C" {

int nfft_gb_mlp_param_count(void) { return P_COUNT; }

int nfft_gb_dcf_features(const float *x_dev, int M, int n0, int n1, float *feat_dev, void *stream)
{
  if (M < 0 || n0 < 1 || n1 < 1) return -1;
  if (M == 0) return 0;
  cudaStream_t s = (cudaStream_t)stream;
  // the cell counts in stream-ordered scratch: no device-wide synchronisation,
  // the features are ready in stream order like the other entry points' results
  int *cnt = nullptr;
  GB_CUDA(cudaMallocAsync(reinterpret_cast<void **>(&cnt), (size_t)n0 * n1 * sizeof(int), s));
  GB_CUDA(cudaMemsetAsync(cnt, 0, (size_t)n0 * n1 * sizeof(int), s));
  k_cell_counts<<<(M + 255) / 256, 256, 0, s>>>(x_dev, M, n0, n1, cnt);
  GB_LAUNCHED("cell_counts");
  k_features<<<(M + 255) / 256, 256, 0, s>>>(x_dev, M, n0, n1, cnt, feat_dev);
  GB_LAUNCHED("features");
  GB_CUDA(cudaFreeAsync(cnt, s));
  return 0;
}

int nfft_gb_mlp_forward(const float *params, const float *feat, int M, float *out, void *stream)
{
  if (M <= 0) return M < 0 ? -1 : 0;
  const int blocks = std::min((M + MLP_THREADS - 1) / MLP_THREADS, 152 * 8);
  k_mlp_forward<<<blocks, MLP_THREADS, 0, (cudaStream_t)stream>>>(params, feat, M, out);
  GB_LAUNCHED("mlp_forward");
  return 0;
}

// grad (P_COUNT floats) and loss (1 float) are overwritten
int nfft_gb_mlp_grad(const float *params, const float *feat, const float *target, int M, float *grad,
                     float *loss, void *stream)
{
  cudaStream_t s = (cudaStream_t)stream;
  GB_CUDA(cudaMemsetAsync(grad, 0, P_COUNT * sizeof(float), s));
  GB_CUDA(cudaMemsetAsync(loss, 0, sizeof(float), s));
  if (M <= 0) return M < 0 ? -1 : 0;
  const size_t smem = mlp_grad_smem_floats() * sizeof(float);
  set_smem_limit((const void *)k_mlp_grad, smem);
  const int blocks = std::min((M + MLP_THREADS - 1) / MLP_THREADS, 152);
  k_mlp_grad<<<blocks, MLP_THREADS, smem, s>>>(params, feat, target, M, grad, loss);
  GB_LAUNCHED("mlp_grad");
  return 0;
}

int nfft_gb_mlp_adam(float *params, const float *grad, float *m1, float *m2, int step, float lr, float beta1,
                     float beta2, float eps, void *stream)
{
  const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
  k_adam<<<(P_COUNT + 255) / 256, 256, 0, (cudaStream_t)stream>>>(params, grad, m1, m2, P_COUNT, lr, beta1,
                                                                    beta2, eps, c1, c2);
  GB_LAUNCHED("adam");
  return 0;
}

// w_dev (M reals, device): in = start weights, out = after `iters` steps of
// w <- w / |A A^H w| with the plan's transforms (nodes already set up).
int nfftf_gb_dcf_fixed_point(nfftf_plan *p, float *w_dev, int iters)
{
  const int M = (int)p->M_total;
  cudaStream_t s = (cudaStream_t)nfftf_gb_get_stream(p);
  float2 *f = (float2 *)nfftf_gb_device_f(p);
  for (int it = 0; it < iters; ++it) {
    k_real_to_complex<<<(M + 255) / 256, 256, 0, s>>>(w_dev, f, M);
    GB_LAUNCHED("real_to_complex");
    nfftf_gb_adjoint_device(p);  // f_hat = A^H w
    nfftf_gb_trafo_device(p);    // f = A A^H w
    k_dcf_update<<<(M + 255) / 256, 256, 0, s>>>(w_dev, f, M);
    GB_LAUNCHED("dcf_update");
  }
  GB_CUDA(cudaStreamSynchronize(s));
  return 0;
}

}  // extern "C"

namespace gb {
// a[r][c] = a[r][c] * scale[c] + shift[c] (feature standardisation)
struct Affine8 {
  float s[8], t[8];
};
__global__ void k_affine_columns(float *__restrict__ a, long long rows, int cols, Affine8 aff)
{
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows * cols) return;
  const int c = (int)(i % cols);
  a[i] = a[i] * aff.s[c] + aff.t[c];
}
}  // namespace gb

extern "C" int nfft_gb_affine_columns(float *a, long long rows, int cols, const float *scale,
                                      const float *shift, void *stream)
{
  if (cols < 1 || cols > 8 || rows < 0) return -1;
  gb::Affine8 aff;
  for (int c = 0; c < 8; ++c) {
    aff.s[c] = c < cols ? scale[c] : 1.f;
    aff.t[c] = c < cols ? shift[c] : 0.f;
  }
  const long long n = rows * cols;
  if (n == 0) return 0;
  gb::k_affine_columns<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(a, rows, cols, aff);
  GB_LAUNCHED("affine_columns");
  return 0;
}
