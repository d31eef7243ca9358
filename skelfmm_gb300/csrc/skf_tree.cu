// skf_tree.cu — the point-level front end of the tree build on the device:
// integer cell coordinates of every point on the finest grid of the root box
// and their interleaved (Morton) keys.  The host tree (skelfmm_gb300/tree.py,
// the stand-in for simpletree.BalancedTree called at skelfmm/skel_fmm.py:150)
// sorts by these keys and refines box ranges level by level; computing them
// here gives bit-identical keys (same FP64 operations in the same order, no
// contraction) at HBM speed.
#include <cuda_runtime.h>
#include <stdint.h>

#include "skf_internal.cuh"

namespace skf {

// bit b of v moved to bit b * ndim (v < 2^depth)
__device__ __forceinline__ uint64_t spread_bits(uint64_t v, int ndim, int depth) {
  uint64_t out = 0;
#pragma unroll 4
  for (int b = 0; b < depth; ++b) out |= ((v >> b) & 1ull) << (b * ndim);
  return out;
}

// One thread per point: q = clamp(floor((x - corner) / L0 * 2^depth), 0,
// 2^depth - 1) per axis (FP64, correctly rounded at every step), and the
// key with axis 0 in the most significant bit of every ndim-bit group.
__global__ void k_morton_keys(int ndim, int64_t n, const double* __restrict__ x, const double* __restrict__ corner,
                              double L0, int depth, uint64_t* __restrict__ keys, int64_t* __restrict__ q) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double scale = (double)(1ll << depth);
  const double top = (double)((1ll << depth) - 1);
  uint64_t key = 0;
  for (int d = 0; d < ndim; ++d) {
    double t = __dsub_rn(x[i * ndim + d], corner[d]);
    t = __ddiv_rn(t, L0);
    t = __dmul_rn(t, scale);
    t = floor(t);
    t = fmin(t, top);
    t = fmax(t, 0.0);
    const int64_t c = (int64_t)t;
    if (q) q[i * ndim + d] = c;
    key |= spread_bits((uint64_t)c, ndim, depth) << (ndim - 1 - d);
  }
  keys[i] = key;
}

}  // namespace skf

extern "C" int skf_morton_keys(int32_t ndim, int64_t n, const double* x, const double* corner, double L0,
                               int32_t depth, uint64_t* keys, int64_t* q, void* stream) {
  if ((ndim != 2 && ndim != 3) || n < 0 || !(L0 > 0) || depth < 1 || depth * ndim > 63) return SKF_ERR_ARG;
  if (n == 0) return SKF_OK;
  if (!x || !corner || !keys) return SKF_ERR_ARG;
  const int64_t blocks = (n + 255) / 256;
  skf::k_morton_keys<<<(unsigned)blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(ndim, n, x, corner, L0, depth,
                                                                                      keys, q);
  SKF_CUDA_TRY(cudaGetLastError());
  return SKF_OK;
}
