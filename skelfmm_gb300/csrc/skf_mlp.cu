// Rank predictor of the learned-rank build: a 3-layer perceptron
//   h1 = bf16(relu(W1 x + b1)), h2 = bf16(relu(W2 h1 + b2)), y = w3 . h2 + b3
// with width 128, BF16 weights and activations, FP32 arithmetic, FP32
// gradients and FP32 Adam master weights.  Training minimises the mean
// squared error against log2(rank + 1) of the pivoted-QR build.
//
// Parameter vector (FP32 master `theta`, BF16 mirror `theta16`):
//   W1 [128 x nin] | b1 [128] | W2 [128 x 128] | b2 [128] | w3 [128] | b3 [1]
//
// One CTA of 128 threads owns a tile of 64 samples; thread o owns output
// unit o of every layer.  The per-tile gradient goes to a scratch row and a
// second kernel adds the rows in a fixed order and applies Adam, so training
// is deterministic.  The whole network (34 K parameters) is tiny next to the
// build it serves; FP32 FMA on the CUDA cores is enough.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "skf_internal.cuh"

namespace skf {

constexpr int kH = 128;       // hidden width
constexpr int kTile = 64;     // samples per CTA
constexpr int kMaxIn = 32;    // input features
constexpr int kLd = kH + 1;   // padded smem row (floats)

__host__ __device__ constexpr int64_t mlp_params(int nin) { return (int64_t)kH * nin + kH + kH * kH + kH + kH + 1; }

struct MlpOffsets {
  int w1, b1, w2, b2, w3, b3;
};
__host__ __device__ inline MlpOffsets mlp_offsets(int nin) {
  MlpOffsets o;
  o.w1 = 0;
  o.b1 = kH * nin;
  o.w2 = o.b1 + kH;
  o.b2 = o.w2 + kH * kH;
  o.w3 = o.b2 + kH;
  o.b3 = o.w3 + kH;
  return o;
}

__device__ __forceinline__ float bf(const __nv_bfloat16 v) { return __bfloat162float(v); }
__device__ __forceinline__ float round_bf16(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

// shared-memory layout of one tile (floats)
struct MlpSmem {
  float* x;   // [kTile][kMaxIn]
  float* w2;  // [kH][kLd]  W2 (row o = output o)
  float* h1;  // [kTile][kLd]
  float* h2;  // [kTile][kLd]
  float* d2;  // [kTile][kLd]  dL/d(pre-activation 2)
  float* y;   // [kTile]
};

__host__ __device__ constexpr size_t mlp_smem_floats() {
  return (size_t)kTile * kMaxIn + (size_t)kH * kLd + 3 * (size_t)kTile * kLd + kTile;
}

__device__ inline MlpSmem carve(float* sm) {
  MlpSmem s;
  s.x = sm;
  s.w2 = s.x + kTile * kMaxIn;
  s.h1 = s.w2 + kH * kLd;
  s.h2 = s.h1 + kTile * kLd;
  s.d2 = s.h2 + kTile * kLd;
  s.y = s.d2 + kTile * kLd;
  return s;
}

// Forward pass of one tile; leaves x, W2, h1, h2 and y in shared memory.
__device__ void mlp_forward_tile(const __nv_bfloat16* __restrict__ th, int nin, const __nv_bfloat16* __restrict__ X,
                                 int64_t s0, int ns, const MlpSmem& s) {
  const MlpOffsets of = mlp_offsets(nin);
  const int o = threadIdx.x;
  for (int i = threadIdx.x; i < kTile * kMaxIn; i += blockDim.x) {
    const int r = i / kMaxIn, f = i % kMaxIn;
    s.x[i] = (r < ns && f < nin) ? bf(X[(s0 + r) * nin + f]) : 0.f;
  }
  for (int i = threadIdx.x; i < kH * kH; i += blockDim.x) s.w2[(i / kH) * kLd + i % kH] = bf(th[of.w2 + i]);
  __syncthreads();
  // layer 1: unit o
  float w1[kMaxIn];
#pragma unroll
  for (int f = 0; f < kMaxIn; ++f) w1[f] = f < nin ? bf(th[of.w1 + o * nin + f]) : 0.f;
  const float b1 = bf(th[of.b1 + o]);
  for (int r = 0; r < kTile; ++r) {
    float acc = b1;
#pragma unroll
    for (int f = 0; f < kMaxIn; ++f) acc = fmaf(w1[f], s.x[r * kMaxIn + f], acc);
    s.h1[r * kLd + o] = round_bf16(fmaxf(acc, 0.f));
  }
  __syncthreads();
  // layer 2: unit o, 16 samples at a time
  const float b2 = bf(th[of.b2 + o]);
  for (int r0 = 0; r0 < kTile; r0 += 16) {
    float acc[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) acc[i] = b2;
    for (int k = 0; k < kH; ++k) {
      const float w = s.w2[o * kLd + k];
#pragma unroll
      for (int i = 0; i < 16; ++i) acc[i] = fmaf(s.h1[(r0 + i) * kLd + k], w, acc[i]);
    }
#pragma unroll
    for (int i = 0; i < 16; ++i) s.h2[(r0 + i) * kLd + o] = round_bf16(fmaxf(acc[i], 0.f));
  }
  __syncthreads();
  // output: one warp per 16 samples, lanes over the 128 inputs
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const float b3 = bf(th[of.b3]);
  for (int r = warp; r < kTile; r += blockDim.x >> 5) {
    float acc = 0.f;
    for (int k = lane; k < kH; k += 32) acc = fmaf(bf(th[of.w3 + k]), s.h2[r * kLd + k], acc);
    for (int sh = 16; sh > 0; sh >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, sh);
    if (lane == 0) s.y[r] = acc + b3;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(kH) k_mlp_predict(const __nv_bfloat16* __restrict__ th, int nin,
                                                    const __nv_bfloat16* __restrict__ X, int64_t n,
                                                    float* __restrict__ y) {
  extern __shared__ float sm[];
  const MlpSmem s = carve(sm);
  const int64_t s0 = (int64_t)blockIdx.x * kTile;
  const int ns = (int)(n - s0 < kTile ? n - s0 : kTile);
  mlp_forward_tile(th, nin, X, s0, ns, s);
  for (int r = threadIdx.x; r < ns; r += blockDim.x) y[s0 + r] = s.y[r];
}

// Gradient of 1/n sum (y - t)^2 over this tile, written to part[blockIdx.x][P];
// part[..][P] holds the tile's sum of squared errors.
__global__ void __launch_bounds__(kH) k_mlp_grad_tile(const __nv_bfloat16* __restrict__ th, int nin,
                                                      const __nv_bfloat16* __restrict__ X,
                                                      const float* __restrict__ t, int64_t n,
                                                      float* __restrict__ part) {
  extern __shared__ float sm[];
  const MlpSmem s = carve(sm);
  const MlpOffsets of = mlp_offsets(nin);
  const int64_t P = mlp_params(nin);
  const int64_t s0 = (int64_t)blockIdx.x * kTile;
  const int ns = (int)(n - s0 < kTile ? n - s0 : kTile);
  mlp_forward_tile(th, nin, X, s0, ns, s);
  float* g = part + (int64_t)blockIdx.x * (P + 1);
  const int o = threadIdx.x;
  const float inv_n = 1.f / (float)n;
  // dL/dy in s.y (reused), squared error
  __shared__ float s_sse[kTile];
  if (threadIdx.x < kTile) {
    const int r = threadIdx.x;
    const float e = r < ns ? s.y[r] - t[s0 + r] : 0.f;
    s_sse[r] = e * e;
    s.y[r] = 2.f * e * inv_n;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float sse = 0.f;
    for (int r = 0; r < kTile; ++r) sse += s_sse[r];
    g[P] = sse;
  }
  // output layer and dL/d(pre2)
  const float w3o = bf(th[of.w3 + o]);
  float gw3 = 0.f, gb3 = 0.f, gb2 = 0.f;
  for (int r = 0; r < kTile; ++r) {
    const float dy = s.y[r];
    const float h = s.h2[r * kLd + o];
    gw3 = fmaf(dy, h, gw3);
    gb3 += dy;
    const float d = h > 0.f ? dy * w3o : 0.f;
    s.d2[r * kLd + o] = d;
    gb2 += d;
  }
  g[of.w3 + o] = gw3;
  g[of.b2 + o] = gb2;
  if (o == 0) g[of.b3] = gb3;
  __syncthreads();
  // dW2[o][k] = sum_r d2[r][o] h1[r][k]
  for (int k0 = 0; k0 < kH; k0 += 16) {
    float acc[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) acc[i] = 0.f;
    for (int r = 0; r < kTile; ++r) {
      const float d = s.d2[r * kLd + o];
#pragma unroll
      for (int i = 0; i < 16; ++i) acc[i] = fmaf(d, s.h1[r * kLd + k0 + i], acc[i]);
    }
#pragma unroll
    for (int i = 0; i < 16; ++i) g[of.w2 + o * kH + k0 + i] = acc[i];
  }
  // dL/d(pre1)[r][k] for unit k = o: sum_j d2[r][j] W2[j][k], masked by h1 > 0
  float gb1 = 0.f;
  float gw1[kMaxIn];
#pragma unroll
  for (int f = 0; f < kMaxIn; ++f) gw1[f] = 0.f;
  for (int r = 0; r < kTile; ++r) {
    float acc = 0.f;
    for (int j = 0; j < kH; ++j) acc = fmaf(s.d2[r * kLd + j], s.w2[j * kLd + o], acc);
    const float d1 = s.h1[r * kLd + o] > 0.f ? acc : 0.f;
    gb1 += d1;
#pragma unroll
    for (int f = 0; f < kMaxIn; ++f) gw1[f] = fmaf(d1, s.x[r * kMaxIn + f], gw1[f]);
  }
  g[of.b1 + o] = gb1;
  for (int f = 0; f < nin; ++f) g[of.w1 + o * nin + f] = gw1[f];
}

// grad = sum over tiles (fixed order); then Adam on the FP32 master weights
// and the BF16 mirror.  loss_out = mean squared error of the batch.
__global__ void k_mlp_reduce_adam(int64_t P, int ntiles, const float* __restrict__ part, float* __restrict__ grad,
                                  float* __restrict__ theta, __nv_bfloat16* __restrict__ th16, float* __restrict__ m,
                                  float* __restrict__ v, int step, float lr, float beta1, float beta2, float eps,
                                  int apply, int64_t n, float* __restrict__ loss_out) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p > P) return;
  float acc = 0.f;
  for (int i = 0; i < ntiles; ++i) acc += part[(int64_t)i * (P + 1) + p];
  if (p == P) {
    if (loss_out) *loss_out = acc / (float)n;
    return;
  }
  grad[p] = acc;
  if (!apply) return;
  const float mm = beta1 * m[p] + (1.f - beta1) * acc;
  const float vv = beta2 * v[p] + (1.f - beta2) * acc * acc;
  m[p] = mm;
  v[p] = vv;
  const float mh = mm / (1.f - powf(beta1, (float)step));
  const float vh = vv / (1.f - powf(beta2, (float)step));
  const float w = theta[p] - lr * mh / (sqrtf(vh) + eps);
  theta[p] = w;
  th16[p] = __float2bfloat16_rn(w);
}

__global__ void k_f32_to_bf16(const float* __restrict__ a, __nv_bfloat16* __restrict__ b, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = __float2bfloat16_rn(a[i]);
}

// Geometric moments of the rank network's features: per box, the mean
// offset of its points from the box centre and their second central
// moments, in units of the box width.  One block per box, FP64 sums.
// out[9 b ..]: mean x y z, then xx yy zz xy xz yz.
constexpr int kMomThreads = 128;
__global__ void __launch_bounds__(kMomThreads) k_box_moments(const int64_t* __restrict__ off,
                                                             const double* __restrict__ x, int ndim,
                                                             const double* __restrict__ centers, double width,
                                                             double* __restrict__ out) {
  const int b = blockIdx.x;
  const int64_t o0 = off[b], o1 = off[b + 1];
  double c[3] = {0.0, 0.0, 0.0};
  for (int d = 0; d < ndim; ++d) c[d] = centers[(int64_t)b * ndim + d];
  double s[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) s[q] = 0.0;
  for (int64_t i = o0 + threadIdx.x; i < o1; i += kMomThreads) {
    double r[3] = {0.0, 0.0, 0.0};
    for (int d = 0; d < ndim; ++d) r[d] = (x[i * ndim + d] - c[d]) / width;
    s[0] += r[0];
    s[1] += r[1];
    s[2] += r[2];
    s[3] += r[0] * r[0];
    s[4] += r[1] * r[1];
    s[5] += r[2] * r[2];
    s[6] += r[0] * r[1];
    s[7] += r[0] * r[2];
    s[8] += r[1] * r[2];
  }
  __shared__ double red[kMomThreads / 32][9];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < 9; ++q) {
    double v = s[q];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[w][q] = v;
  }
  __syncthreads();
  if (threadIdx.x < 9) {
    const int q = threadIdx.x;
    double t = 0.0;
    for (int k = 0; k < kMomThreads / 32; ++k) t += red[k][q];
    red[0][q] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const double n = o1 > o0 ? (double)(o1 - o0) : 1.0;
    double m[3];
    for (int d = 0; d < 3; ++d) m[d] = red[0][d] / n;
    double* o = out + (int64_t)9 * b;
    o[0] = m[0];
    o[1] = m[1];
    o[2] = m[2];
    o[3] = red[0][3] / n - m[0] * m[0];
    o[4] = red[0][4] / n - m[1] * m[1];
    o[5] = red[0][5] / n - m[2] * m[2];
    o[6] = red[0][6] / n - m[0] * m[1];
    o[7] = red[0][7] / n - m[0] * m[2];
    o[8] = red[0][8] / n - m[1] * m[2];
  }
}

static int mlp_smem_attr(const void* fn) {
  const size_t bytes = mlp_smem_floats() * sizeof(float);
  SKF_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  return SKF_OK;
}

}  // namespace skf

using namespace skf;

extern "C" {

int64_t skf_mlp_num_params(int32_t nin) { return (nin <= 0 || nin > kMaxIn) ? -1 : mlp_params(nin); }

int64_t skf_mlp_scratch_floats(int32_t nin, int64_t n) {
  if (nin <= 0 || nin > kMaxIn || n < 0) return -1;
  const int64_t tiles = (n + kTile - 1) / kTile;
  return tiles * (mlp_params(nin) + 1);
}

int skf_mlp_bf16(const float* src, void* dst, int64_t n, void* stream) {
  if (n < 0 || (n > 0 && (!src || !dst))) return SKF_ERR_ARG;
  if (n == 0) return SKF_OK;
  const int g = (int)std::min<int64_t>((n + 255) / 256, 152 * 8);
  k_f32_to_bf16<<<g, 256, 0, static_cast<cudaStream_t>(stream)>>>(src, static_cast<__nv_bfloat16*>(dst), n);
  SKF_CUDA_TRY(cudaGetLastError());
  return SKF_OK;
}

int skf_mlp_predict(int32_t nin, const void* theta16, const void* x16, int64_t n, float* y, void* stream) {
  if (nin <= 0 || nin > kMaxIn || n < 0) return SKF_ERR_ARG;
  if (n == 0) return SKF_OK;
  if (!theta16 || !x16 || !y) return SKF_ERR_ARG;
  if (mlp_smem_attr((const void*)k_mlp_predict) != SKF_OK) return SKF_ERR_CUDA;
  const int64_t tiles = (n + kTile - 1) / kTile;
  if (tiles > 0x7fffffff) return SKF_ERR_ARG;
  k_mlp_predict<<<(unsigned)tiles, kH, mlp_smem_floats() * sizeof(float), static_cast<cudaStream_t>(stream)>>>(
      static_cast<const __nv_bfloat16*>(theta16), nin, static_cast<const __nv_bfloat16*>(x16), n, y);
  SKF_CUDA_TRY(cudaGetLastError());
  return SKF_OK;
}

int skf_mlp_train_step(int32_t nin, float* theta, void* theta16, const void* x16, const float* target, int64_t n,
                       float* scratch, float* grad, float* adam_m, float* adam_v, int32_t step, float lr,
                       float beta1, float beta2, float eps, int32_t apply, float* loss, void* stream) {
  if (nin <= 0 || nin > kMaxIn || n <= 0 || step < 1) return SKF_ERR_ARG;
  if (!theta16 || !x16 || !target || !scratch || !grad) return SKF_ERR_ARG;
  if (apply && (!theta || !adam_m || !adam_v)) return SKF_ERR_ARG;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (mlp_smem_attr((const void*)k_mlp_grad_tile) != SKF_OK) return SKF_ERR_CUDA;
  const int64_t tiles = (n + kTile - 1) / kTile;
  if (tiles > 0x7fffffff) return SKF_ERR_ARG;
  const int64_t P = mlp_params(nin);
  k_mlp_grad_tile<<<(unsigned)tiles, kH, mlp_smem_floats() * sizeof(float), st>>>(
      static_cast<const __nv_bfloat16*>(theta16), nin, static_cast<const __nv_bfloat16*>(x16), target, n, scratch);
  SKF_CUDA_TRY(cudaGetLastError());
  k_mlp_reduce_adam<<<(unsigned)((P + 1 + 255) / 256), 256, 0, st>>>(
      P, (int)tiles, scratch, grad, theta, static_cast<__nv_bfloat16*>(theta16), adam_m, adam_v, step, lr, beta1,
      beta2, eps, apply, n, loss);
  SKF_CUDA_TRY(cudaGetLastError());
  return SKF_OK;
}

int skf_box_moments(int32_t nbox, int32_t ndim, const int64_t* off, const double* x, const double* centers,
                    double width, double* out, void* stream) {
  if (nbox < 0 || (ndim != 2 && ndim != 3) || !(width > 0.0)) return SKF_ERR_ARG;
  if (nbox == 0) return SKF_OK;
  if (!off || !x || !centers || !out) return SKF_ERR_ARG;
  k_box_moments<<<nbox, kMomThreads, 0, static_cast<cudaStream_t>(stream)>>>(off, x, ndim, centers, width, out);
  SKF_CUDA_TRY(cudaGetLastError());
  return SKF_OK;
}

}  // extern "C"
