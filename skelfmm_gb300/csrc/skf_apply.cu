// skf_apply.cu — the apply of a built skeletonization on one GPU.
//
// Restates SkelFMMBatched.matvec (skelfmm/batched_fmm.py:539-564) as five
// kernel phases over a ragged (CSR) layout, all on the device:
//   1. permute in      q[leaf entries] = x[points]        (get_qorig, :442-447)
//   2. upward, per level, deepest first:
//        qskel[:r] = q[:r] + T q[r:bs], scattered into the parent's entries
//                                             (compute_qskel, :403-467)
//   3. translations, one launch for every level: each target box owns its
//      rows and accumulates u and uskel over its interaction list, with the
//      kernel evaluated on the fly               (addto_uvec + subtract_from_uskel,
//                                                 :219-302, :496-534)
//   4. downward, per level, coarsest first:
//        uskel[:r] += u(parent entries); u[:r] += uskel[:r]; u[r:] += T^T uskel[:r]
//                                             (resultvec_from_uskel, :469-483)
//   5. permute out     y[points] = u[leaf entries]      (get_result, :487-490)
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "skf_internal.cuh"
#include "skf_kernels.cuh"
#include "skf_translate.cuh"

namespace skf {

// ------------------------------------------------------------------ permute
template <bool C>
__global__ void k_permute_in(const int64_t* __restrict__ pe, const int64_t* __restrict__ pp, int64_t n,
                             const double* __restrict__ x, double* __restrict__ q) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = pe[i], p = pp[i];
    if (C) {
      reinterpret_cast<double2*>(q)[e] = reinterpret_cast<const double2*>(x)[p];
    } else {
      q[e] = x[p];
    }
  }
}

template <bool C>
__global__ void k_permute_out(const int64_t* __restrict__ pe, const int64_t* __restrict__ pp, int64_t n,
                              const double* __restrict__ u, double* __restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = pe[i], p = pp[i];
    if (C) {
      reinterpret_cast<double2*>(y)[p] = reinterpret_cast<const double2*>(u)[e];
    } else {
      y[p] = u[e];
    }
  }
}

// FP32 effective charges for the mixed translations (see skf_plan::q32):
// rounded once from the FP64 vectors, with q - qskel formed in FP64.
__global__ void k_charges32(int64_t n, int W, const int32_t* __restrict__ skel, const double* __restrict__ q,
                            const double* __restrict__ qh, float* __restrict__ q32, float* __restrict__ qhn32,
                            float* __restrict__ qd32) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const bool sk = skel[i / W] != 0;
    const double v = q[i];
    q32[i] = (float)v;
    qhn32[i] = sk ? (float)(-qh[i]) : 0.f;
    qd32[i] = sk ? (float)(v - qh[i]) : (float)v;
  }
}

// ------------------------------------------------------------------ T passes
template <typename T>
struct Acc;
template <>
struct Acc<double> {
  using type = double;
};
template <>
struct Acc<float> {
  using type = float;
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// One block per box: qskel[:r] = q[:r] + T q[r:bs]; each skeleton entry is
// also written into its slot of the parent box's q.
template <bool C, typename TT>
__global__ void __launch_bounds__(256) k_up(const int32_t* __restrict__ boxes, const int64_t* __restrict__ box_off,
                                            const int32_t* __restrict__ box_rank, const int64_t* __restrict__ t_off,
                                            const TT* __restrict__ tdat, const int64_t* __restrict__ pslot,
                                            double* __restrict__ q, double* __restrict__ qh) {
  extern __shared__ double sm_up[];
  const int b = boxes[blockIdx.x];
  const int64_t off = box_off[b];
  const int bs = (int)(box_off[b + 1] - off);
  const int r = box_rank[b];
  const int nred = bs - r;
  const int W = C ? 2 : 1;
  for (int c = threadIdx.x; c < nred * W; c += blockDim.x) sm_up[c] = q[(off + r) * W + c];
  __syncthreads();
  const TT* T = tdat + t_off[b] * W;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int i = warp; i < r; i += nw) {
    const TT* row = T + (int64_t)i * nred * W;
    typename Acc<TT>::type ar = 0, ai = 0;
    for (int c = lane; c < nred; c += 32) {
      if (C) {
        const TT tr = row[2 * c], ti = row[2 * c + 1];
        const TT xr = (TT)sm_up[2 * c], xi = (TT)sm_up[2 * c + 1];
        ar += tr * xr - ti * xi;
        ai += tr * xi + ti * xr;
      } else {
        ar += row[c] * (TT)sm_up[c];
      }
    }
    double sr = warp_sum((double)ar);
    double si = C ? warp_sum((double)ai) : 0.0;
    if (lane == 0) {
      const int64_t e = off + i;
      const int64_t ps = pslot[e];
      if (C) {
        const double vr = q[2 * e] + sr, vi = q[2 * e + 1] + si;
        qh[2 * e] = vr;
        qh[2 * e + 1] = vi;
        if (ps >= 0) {
          q[2 * ps] = vr;
          q[2 * ps + 1] = vi;
        }
      } else {
        const double v = q[e] + sr;
        qh[e] = v;
        if (ps >= 0) q[ps] = v;
      }
    }
  }
}

// ---- float-float variants for the mixed apply ------------------------------
// GB300's FP64 pipe runs the T / T^T products of the FP64-T kernels above at
// its peak; here T is held as an FP32 pair (hi = fl32(T), lo = fl32(T - hi))
// and the vector as a pair likewise, products are formed exactly with FMA
// (p = a*b, e = fma(a, b, -p)) plus the two cross terms, and sums are
// carried as (s, c) pairs with Knuth's TwoSum: ~2^-44 relative, all on the
// FP32 pipes, same 8 bytes of T per scalar.
struct FF {
  float s = 0.f, c = 0.f;
};
__device__ __forceinline__ void ff_add_prod(FF& acc, float ah, float al, float bh, float bl) {
  const float p = ah * bh;
  const float e = fmaf(ah, bh, -p);
  const float x = fmaf(ah, bl, al * bh);
  const float t = acc.s + p;
  const float z = t - acc.s;
  const float err = (acc.s - (t - z)) + (p - z);
  acc.s = t;
  acc.c += err + e + x;
}
__device__ __forceinline__ void ff_sub_prod(FF& acc, float ah, float al, float bh, float bl) {
  ff_add_prod(acc, -ah, -al, bh, bl);
}
// Warp sum of float-float values on the FP32 pipes (xor butterfly, TwoSum of
// the leading parts): lane 0's result is the same on every run.
__device__ __forceinline__ double ff_warp_sum(FF a) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float s2 = __shfl_xor_sync(0xffffffffu, a.s, o);
    const float c2 = __shfl_xor_sync(0xffffffffu, a.c, o);
    const float t = a.s + s2;
    const float z = t - a.s;
    const float err = (a.s - (t - z)) + (s2 - z);
    a.s = t;
    a.c = (a.c + c2) + err;
  }
  return (double)a.s + (double)a.c;
}
// Sum of float-float values over aligned groups of g lanes (g a power of
// two): every lane of a group holds the group's sum, in a fixed order.
__device__ __forceinline__ FF ff_group_sum(FF a, int g) {
  for (int o = g >> 1; o > 0; o >>= 1) {
    const float s2 = __shfl_xor_sync(0xffffffffu, a.s, o);
    const float c2 = __shfl_xor_sync(0xffffffffu, a.c, o);
    const float t = a.s + s2;
    const float z = t - a.s;
    const float err = (a.s - (t - z)) + (s2 - z);
    a.s = t;
    a.c = (a.c + c2) + err;
  }
  return a;
}
__device__ __forceinline__ FF ff_add(FF a, FF b) {
  const float t = a.s + b.s;
  const float z = t - a.s;
  const float err = (a.s - (t - z)) + (b.s - z);
  FF r;
  r.s = t;
  r.c = (a.c + b.c) + err;
  return r;
}
__device__ __forceinline__ void split_f64(double v, float& h, float& l) {
  h = (float)v;
  l = (float)(v - (double)h);
}

template <bool C>
__global__ void __launch_bounds__(256) k_up_ff(const int32_t* __restrict__ boxes, const int64_t* __restrict__ box_off,
                                               const int32_t* __restrict__ box_rank, const int64_t* __restrict__ t_off,
                                               const float* __restrict__ thi, const float* __restrict__ tlo,
                                               const int64_t* __restrict__ pslot, double* __restrict__ q,
                                               double* __restrict__ qh) {
  extern __shared__ float sm_upf[];  // [2 * nred * W]: hi, lo
  const int b = boxes[blockIdx.x];
  const int64_t off = box_off[b];
  const int bs = (int)(box_off[b + 1] - off);
  const int r = box_rank[b];
  const int nred = bs - r;
  const int W = C ? 2 : 1;
  float* xh = sm_upf;
  float* xl = sm_upf + nred * W;
  for (int c = threadIdx.x; c < nred * W; c += blockDim.x) split_f64(q[(off + r) * W + c], xh[c], xl[c]);
  __syncthreads();
  const float* Th = thi + t_off[b] * W;
  const float* Tl = tlo + t_off[b] * W;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  // g lanes per row (about 8+ columns a lane), 32 / g rows per warp; two
  // accumulators per lane (alternate column strides) for independent chains
  const int g = nred > 256 ? 32 : (nred > 128 ? 16 : (nred > 32 ? 8 : 4));
  const int rows = 32 / g, lg = lane & (g - 1);
  for (int i0 = warp * rows; i0 < r; i0 += nw * rows) {
    const int i = i0 + lane / g;
    const int64_t rb = (int64_t)min(i, r - 1) * nred * W;
    FF ar, ai, br, bi;
    if (i < r) {
      int c = lg;
      for (; c + g < nred; c += 2 * g) {
        if (C) {
          const float trh = Th[rb + 2 * c], tih = Th[rb + 2 * c + 1];
          const float trl = Tl[rb + 2 * c], til = Tl[rb + 2 * c + 1];
          const float xrh = xh[2 * c], xih = xh[2 * c + 1], xrl = xl[2 * c], xil = xl[2 * c + 1];
          const int d = c + g;
          const float urh = Th[rb + 2 * d], uih = Th[rb + 2 * d + 1];
          const float url = Tl[rb + 2 * d], uil = Tl[rb + 2 * d + 1];
          const float yrh = xh[2 * d], yih = xh[2 * d + 1], yrl = xl[2 * d], yil = xl[2 * d + 1];
          ff_add_prod(ar, trh, trl, xrh, xrl);
          ff_sub_prod(ar, tih, til, xih, xil);
          ff_add_prod(ai, trh, trl, xih, xil);
          ff_add_prod(ai, tih, til, xrh, xrl);
          ff_add_prod(br, urh, url, yrh, yrl);
          ff_sub_prod(br, uih, uil, yih, yil);
          ff_add_prod(bi, urh, url, yih, yil);
          ff_add_prod(bi, uih, uil, yrh, yrl);
        } else {
          const float t0h = Th[rb + c], t0l = Tl[rb + c], t1h = Th[rb + c + g], t1l = Tl[rb + c + g];
          ff_add_prod(ar, t0h, t0l, xh[c], xl[c]);
          ff_add_prod(br, t1h, t1l, xh[c + g], xl[c + g]);
        }
      }
      if (c < nred) {
        if (C) {
          const float trh = Th[rb + 2 * c], tih = Th[rb + 2 * c + 1];
          const float trl = Tl[rb + 2 * c], til = Tl[rb + 2 * c + 1];
          const float xrh = xh[2 * c], xih = xh[2 * c + 1], xrl = xl[2 * c], xil = xl[2 * c + 1];
          ff_add_prod(ar, trh, trl, xrh, xrl);
          ff_sub_prod(ar, tih, til, xih, xil);
          ff_add_prod(ai, trh, trl, xih, xil);
          ff_add_prod(ai, tih, til, xrh, xrl);
        } else {
          ff_add_prod(ar, Th[rb + c], Tl[rb + c], xh[c], xl[c]);
        }
      }
    }
    const FF tr = ff_group_sum(ff_add(ar, br), g);
    const FF ti = C ? ff_group_sum(ff_add(ai, bi), g) : FF();
    const double sr = (double)tr.s + (double)tr.c;
    const double si = C ? (double)ti.s + (double)ti.c : 0.0;
    if (lg == 0 && i < r) {
      const int64_t e = off + i;
      const int64_t ps = pslot[e];
      if (C) {
        const double vr = q[2 * e] + sr, vi = q[2 * e + 1] + si;
        qh[2 * e] = vr;
        qh[2 * e + 1] = vi;
        if (ps >= 0) {
          q[2 * ps] = vr;
          q[2 * ps + 1] = vi;
        }
      } else {
        const double v = q[e] + sr;
        qh[e] = v;
        if (ps >= 0) q[ps] = v;
      }
    }
  }
}

template <bool C>
__global__ void __launch_bounds__(256) k_down_ff(const int32_t* __restrict__ boxes,
                                                 const int64_t* __restrict__ box_off,
                                                 const int32_t* __restrict__ box_rank,
                                                 const int64_t* __restrict__ t_off, const float* __restrict__ thi,
                                                 const float* __restrict__ tlo, const int64_t* __restrict__ pslot,
                                                 double* __restrict__ u, double* __restrict__ uh) {
  extern __shared__ float sm_dnf[];  // [2 * r * W]: hi, lo
  const int b = boxes[blockIdx.x];
  const int64_t off = box_off[b];
  const int bs = (int)(box_off[b + 1] - off);
  const int r = box_rank[b];
  const int nred = bs - r;
  const int W = C ? 2 : 1;
  float* hh = sm_dnf;
  float* hl = sm_dnf + r * W;
  for (int i = threadIdx.x; i < r; i += blockDim.x) {
    const int64_t e = off + i;
    const int64_t ps = pslot[e];
    if (C) {
      double hr = uh[2 * e], hi = uh[2 * e + 1];
      if (ps >= 0) {
        hr += u[2 * ps];
        hi += u[2 * ps + 1];
      }
      uh[2 * e] = hr;
      uh[2 * e + 1] = hi;
      u[2 * e] += hr;
      u[2 * e + 1] += hi;
      split_f64(hr, hh[2 * i], hl[2 * i]);
      split_f64(hi, hh[2 * i + 1], hl[2 * i + 1]);
    } else {
      double h = uh[e];
      if (ps >= 0) h += u[ps];
      uh[e] = h;
      u[e] += h;
      split_f64(h, hh[i], hl[i]);
    }
  }
  __syncthreads();
  const float* Th = thi + t_off[b] * W;
  const float* Tl = tlo + t_off[b] * W;
  for (int c = threadIdx.x; c < nred; c += blockDim.x) {
    FF ar, ai;
    if constexpr (C) {
      // complex: two chains (even and odd rows) for independent work
      FF br, bi;
      int i = 0;
      for (; i + 1 < r; i += 2) {
        const int64_t k = ((int64_t)i * nred + c) * W, k2 = k + (int64_t)nred * W;
        const float trh = Th[k], tih = Th[k + 1], trl = Tl[k], til = Tl[k + 1];
        const float urh = Th[k2], uih = Th[k2 + 1], url = Tl[k2], uil = Tl[k2 + 1];
        ff_add_prod(ar, trh, trl, hh[2 * i], hl[2 * i]);
        ff_sub_prod(ar, tih, til, hh[2 * i + 1], hl[2 * i + 1]);
        ff_add_prod(ai, trh, trl, hh[2 * i + 1], hl[2 * i + 1]);
        ff_add_prod(ai, tih, til, hh[2 * i], hl[2 * i]);
        ff_add_prod(br, urh, url, hh[2 * i + 2], hl[2 * i + 2]);
        ff_sub_prod(br, uih, uil, hh[2 * i + 3], hl[2 * i + 3]);
        ff_add_prod(bi, urh, url, hh[2 * i + 3], hl[2 * i + 3]);
        ff_add_prod(bi, uih, uil, hh[2 * i + 2], hl[2 * i + 2]);
      }
      if (i < r) {
        const int64_t k = ((int64_t)i * nred + c) * W;
        const float trh = Th[k], tih = Th[k + 1], trl = Tl[k], til = Tl[k + 1];
        ff_add_prod(ar, trh, trl, hh[2 * i], hl[2 * i]);
        ff_sub_prod(ar, tih, til, hh[2 * i + 1], hl[2 * i + 1]);
        ff_add_prod(ai, trh, trl, hh[2 * i + 1], hl[2 * i + 1]);
        ff_add_prod(ai, tih, til, hh[2 * i], hl[2 * i]);
      }
      ar = ff_add(ar, br);
      ai = ff_add(ai, bi);
    } else {
      for (int i = 0; i < r; ++i) {
        const int64_t k = (int64_t)i * nred + c;
        ff_add_prod(ar, Th[k], Tl[k], hh[i], hl[i]);
      }
    }
    const int64_t e = off + r + c;
    if (C) {
      u[2 * e] += (double)ar.s + (double)ar.c;
      u[2 * e + 1] += (double)ai.s + (double)ai.c;
    } else {
      u[e] += (double)ar.s + (double)ar.c;
    }
  }
}

// One block per box: uskel[:r] += u(parent slots); u[:r] += uskel[:r];
// u[r:bs] += T^T uskel[:r].
template <bool C, typename TT>
__global__ void __launch_bounds__(256) k_down(const int32_t* __restrict__ boxes, const int64_t* __restrict__ box_off,
                                              const int32_t* __restrict__ box_rank, const int64_t* __restrict__ t_off,
                                              const TT* __restrict__ tdat, const int64_t* __restrict__ pslot,
                                              double* __restrict__ u, double* __restrict__ uh) {
  extern __shared__ double sm_dn[];
  const int b = boxes[blockIdx.x];
  const int64_t off = box_off[b];
  const int bs = (int)(box_off[b + 1] - off);
  const int r = box_rank[b];
  const int nred = bs - r;
  const int W = C ? 2 : 1;
  for (int i = threadIdx.x; i < r; i += blockDim.x) {
    const int64_t e = off + i;
    const int64_t ps = pslot[e];
    if (C) {
      double hr = uh[2 * e], hi = uh[2 * e + 1];
      if (ps >= 0) {
        hr += u[2 * ps];
        hi += u[2 * ps + 1];
      }
      uh[2 * e] = hr;
      uh[2 * e + 1] = hi;
      u[2 * e] += hr;
      u[2 * e + 1] += hi;
      sm_dn[2 * i] = hr;
      sm_dn[2 * i + 1] = hi;
    } else {
      double h = uh[e];
      if (ps >= 0) h += u[ps];
      uh[e] = h;
      u[e] += h;
      sm_dn[i] = h;
    }
  }
  __syncthreads();
  const TT* T = tdat + t_off[b] * W;
  for (int c = threadIdx.x; c < nred; c += blockDim.x) {
    typename Acc<TT>::type ar = 0, ai = 0;
    for (int i = 0; i < r; ++i) {
      if (C) {
        const TT tr = T[((int64_t)i * nred + c) * 2], ti = T[((int64_t)i * nred + c) * 2 + 1];
        const TT hr = (TT)sm_dn[2 * i], hi = (TT)sm_dn[2 * i + 1];
        ar += tr * hr - ti * hi;
        ai += tr * hi + ti * hr;
      } else {
        ar += T[(int64_t)i * nred + c] * (TT)sm_dn[i];
      }
    }
    const int64_t e = off + r + c;
    if (C) {
      u[2 * e] += (double)ar;
      u[2 * e + 1] += (double)ai;
    } else {
      u[e] += (double)ar;
    }
  }
}

// ------------------------------------------------------------------ dispatch
template <int OP, int TS, int MINB>
static void launch_sym(const SymArgs& c, int n, cudaStream_t st) {
  constexpr size_t smem = sym_smem_bytes(TS);
  static bool attr = false;  // per instantiation
  if (!attr) {
    cudaFuncSetAttribute(k_translate_sym<OP, TS, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = true;
  }
  k_translate_sym<OP, TS, MINB><<<n, 128, smem, st>>>(c);
}

template <int OP>
static void launch_symw(const SymArgs& c, int n, int* queue, cudaStream_t st) {
  constexpr size_t smem = symw_smem_bytes();
  static bool attr = false;  // per instantiation
  if (!attr) {
    cudaFuncSetAttribute(k_translate_symw<OP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(k_translate_symw_queue<OP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = true;
  }
  if (queue == nullptr) {
    k_translate_symw<OP><<<n, kSymwWarps * 32, smem, st>>>(c);
  } else {
    int dev = 0, nsm = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaMemsetAsync(queue, 0, sizeof(int), st);
    k_translate_symw_queue<OP><<<std::min(n, 3 * nsm), kSymwWarps * 32, smem, st>>>(c, n, queue);
  }
}

template <int TS, int MINB>
static void launch_sym_helm(const SymArgs& c, float kappa, int n, cudaStream_t st) {
  constexpr size_t smem = symh_smem_bytes(TS);
  static bool attr = false;  // per instantiation
  if (!attr) {
    cudaFuncSetAttribute(k_translate_sym_helm<TS, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = true;
  }
  k_translate_sym_helm<TS, MINB><<<n, 128, smem, st>>>(c, kappa);
}

template <int OP>
static void launch_translate(const skf_plan* p, bool mixed, cudaStream_t st) {
  TransArgs a;
  a.box_off = p->box_off;
  a.box_rank = p->box_rank;
  a.list_off = p->list_off;
  a.list_src = p->list_src;
  a.list_kind = p->list_kind;
  a.xyz64 = p->xyz64;
  a.geom64 = p->geom64;
  a.hi32 = p->hi32;
  a.lo32 = p->lo32;
  a.geom32 = p->geom32;
  a.q = p->q;
  a.qh = p->qh;
  a.u = p->u;
  a.uh = p->uh;
  a.kappa = p->kappa;
  if (mixed) {
    TransArgs32 b;
    b.work_box = p->work32.box;
    b.work_row = p->work32.row;
    b.box_off = p->box_off;
    b.box_rank = p->box_rank;
    b.list_off = p->list_off;
    b.list_src = p->list_src;
    b.list_kind = p->list_kind;
    b.hi32 = p->hi32;
    b.lo32 = p->lo32;
    b.geom32 = p->geom32;
    b.geom32lo = p->geom32lo;
    b.q32 = p->q32;
    b.qhn32 = p->qhn32;
    b.qd32 = p->qd32;
    b.u = p->u;
    b.uh = p->uh;
    b.kappa = (float)p->kappa;
    static_assert(kT32Threads * kRowsPerThreadF32 == 256, "mixed work items are 256-row tiles");
    if (p->work32.n > 0) {
      if constexpr (OP == SKF_LAPLACE_2D || OP == SKF_LAPLACE_3D || OP == SKF_HELMHOLTZ_3D) {
        if (!p->scalar_mixed && p->sym_ok && p->sym_on) {
          SymArgs c;
          c.work_box = p->worksym.box;
          c.work_row = p->worksym.row;
          c.box_off = p->box_off;
          c.box_rank = p->box_rank;
          c.list_off = p->sym_list_off;
          c.list_src = p->sym_list_src;
          c.list_kind = p->sym_list_kind;
          c.list_poff = p->sym_list_poff;
          c.box_pbase = p->box_pbase;
          c.box_pstride = p->box_pstride;
          c.hi32 = p->hi32;
          c.lo32 = p->lo32;
          c.q32 = p->q32;
          c.qhn32 = p->qhn32;
          c.qd32 = p->qd32;
          c.pbuf = p->pbuf;
          c.u = p->u;
          c.uh = p->uh;
          c.work_part = p->symw_part;
          c.box_ntiles = p->box_ntiles;
          c.box_nparts = p->box_nparts;
          c.box_apart = p->box_apart;
          if constexpr (OP == SKF_HELMHOLTZ_3D) {
            if (p->worksym.n > 0) {
              // tile shape: 0 = 32 sources, 3 blocks/SM; 1 = 64 sources, 2 blocks/SM;
              // 2 = 32 sources, 4 blocks/SM; 3 = 16 sources, 4 blocks/SM
              switch (p->sym_shape) {
                case 1: launch_sym_helm<64, 2>(c, (float)p->kappa, p->worksym.n, st); break;
                case 2: launch_sym_helm<32, 4>(c, (float)p->kappa, p->worksym.n, st); break;
                case 3: launch_sym_helm<16, 4>(c, (float)p->kappa, p->worksym.n, st); break;
                default: launch_sym_helm<32, 3>(c, (float)p->kappa, p->worksym.n, st); break;
              }
            }
            k_sym_reduce_c<<<dim3(p->nboxes, (p->max_bs + 255) / 256), 256, 0, st>>>(
                p->box_off, p->box_rank, p->in_off, p->in_blk, p->pbuf, p->u, p->uh);
          } else if (p->sym_shape == 4 || p->sym_shape == 5) {
            // warps split the source tiles (k_translate_symw): its own items
            // and incoming partial lists (A-side partials of split items);
            // shape 5 takes the items from a queue with persistent blocks
            c.work_box = p->worksymw.box;
            c.work_row = p->worksymw.row;
            if (p->worksymw.n > 0) launch_symw<OP>(c, p->worksymw.n, p->sym_shape == 5 ? p->symw_queue : nullptr, st);
            if (p->red.n > 0)
              k_sym_reduce<OP == SKF_LAPLACE_2D><<<p->red.n, 256, 0, st>>>(
                  p->red.box, p->red.row, p->box_off, p->box_rank, p->in_off_w, p->in_blk_w, p->pbuf, p->u, p->uh);
          } else {
            if (p->worksym.n > 0) {
              // tile shape: 0 = 64 sources, 5 blocks/SM; 1 = 128 sources, 3 blocks/SM;
              // 2 = 64 sources, 4 blocks/SM; 3 = 32 sources, 5 blocks/SM
              switch (p->sym_shape) {
                case 1: launch_sym<OP, 128, 3>(c, p->worksym.n, st); break;
                case 2: launch_sym<OP, 64, 4>(c, p->worksym.n, st); break;
                case 3: launch_sym<OP, 32, 5>(c, p->worksym.n, st); break;
                default: launch_sym<OP, 64, 5>(c, p->worksym.n, st); break;
              }
            }
            if (p->red.n > 0)
              k_sym_reduce<OP == SKF_LAPLACE_2D><<<p->red.n, 256, 0, st>>>(
                  p->red.box, p->red.row, p->box_off, p->box_rank, p->in_off, p->in_blk, p->pbuf, p->u, p->uh);
          }
          return;
        }
        if constexpr (OP != SKF_HELMHOLTZ_3D) {
          if (!p->scalar_mixed) {
            // packed kernel geometry: warps per block x row pairs per thread
            switch (p->x2_config) {
              case 3: {
                TransArgs32 bs = b;
                bs.work_box = p->work32s.box;
                bs.work_row = p->work32s.row;
                if (p->work32s.n > 0) k_translate_f32x2<OP, 1, 1><<<p->work32s.n, 32, 0, st>>>(bs);
                break;
              }
              case 1: k_translate_f32x2<OP, 1, 4><<<p->work32.n, 32, 0, st>>>(b); break;
              case 2: k_translate_f32x2<OP, 2, 2><<<p->work32.n, 64, 0, st>>>(b); break;
              default: k_translate_f32x2<OP, 4, 1><<<p->work32.n, 128, 0, st>>>(b); break;
            }
            return;
          }
        }
      }
      if constexpr (OP == SKF_HELMHOLTZ_3D) {
        if (!p->scalar_mixed) {
          switch (p->x2_config) {
            case 3: {
              TransArgs32 bs = b;
              bs.work_box = p->work32s.box;
              bs.work_row = p->work32s.row;
              if (p->work32s.n > 0) k_translate_helm_x2<1, 1><<<p->work32s.n, 32, 0, st>>>(bs);
              break;
            }
            case 1: k_translate_helm_x2<1, 4><<<p->work32.n, 32, 0, st>>>(b); break;
            case 2: k_translate_helm_x2<2, 2><<<p->work32.n, 64, 0, st>>>(b); break;
            default: k_translate_helm_x2<4, 1><<<p->work32.n, 128, 0, st>>>(b); break;
          }
          return;
        }
      }
      k_translate_f32<OP><<<p->work32.n, kT32Threads, 0, st>>>(b);
    }
  } else {
    a.work_box = p->work64.box;
    a.work_row = p->work64.row;
    if (p->work64.n > 0) k_translate_f64<OP><<<p->work64.n, kTransThreads, 0, st>>>(a);
  }
}

static void translate_dispatch(const skf_plan* p, bool mixed, cudaStream_t st) {
  switch (p->op) {
    case SKF_LAPLACE_2D: launch_translate<SKF_LAPLACE_2D>(p, mixed, st); break;
    case SKF_LAPLACE_3D: launch_translate<SKF_LAPLACE_3D>(p, mixed, st); break;
    case SKF_HELMHOLTZ_2D: launch_translate<SKF_HELMHOLTZ_2D>(p, mixed, st); break;
    case SKF_HELMHOLTZ_3D: launch_translate<SKF_HELMHOLTZ_3D>(p, mixed, st); break;
    case SKF_LAPLACE_DOUBLE_LAYER_3D: launch_translate<SKF_LAPLACE_DOUBLE_LAYER_3D>(p, mixed, st); break;
    case SKF_LAPLACE_ADJOINT_DOUBLE_LAYER_3D: launch_translate<SKF_LAPLACE_ADJOINT_DOUBLE_LAYER_3D>(p, mixed, st); break;
    case SKF_HELMHOLTZ_DOUBLE_LAYER_3D: launch_translate<SKF_HELMHOLTZ_DOUBLE_LAYER_3D>(p, mixed, st); break;
    case SKF_HELMHOLTZ_ADJOINT_DOUBLE_LAYER_3D: launch_translate<SKF_HELMHOLTZ_ADJOINT_DOUBLE_LAYER_3D>(p, mixed, st); break;
    default: break;
  }
}

static int grid_for(int64_t n, int threads) {
  int64_t g = (n + threads - 1) / threads;
  if (g < 1) g = 1;
  if (g > 152 * 32) g = 152 * 32;
  return (int)g;
}

__global__ void k_f64_to_f32(const double* __restrict__ src, float* __restrict__ dst, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (float)src[i];
}

// dst[dst_off[s] + i] = src[src_off[s] + i] for i < len[s]; elements of
// 8 (W = 1) or 16 (W = 2) bytes.  One block per segment (grid-strided).
template <int W>
__global__ void k_copy_segments(int64_t nseg, const int64_t* __restrict__ src_off,
                                const int64_t* __restrict__ dst_off, const int64_t* __restrict__ len,
                                const double* __restrict__ src, double* __restrict__ dst) {
  for (int64_t sgi = blockIdx.x; sgi < nseg; sgi += gridDim.x) {
    const int64_t so = src_off[sgi] * W, d0 = dst_off[sgi] * W, n = len[sgi] * W;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) dst[d0 + i] = src[so + i];
  }
}

int copy_segments(int64_t nseg, const int64_t* src_off, const int64_t* dst_off, const int64_t* len,
                  const void* src, void* dst, int elem_bytes, cudaStream_t st) {
  if (nseg <= 0) return SKF_OK;
  const int g = (int)std::min<int64_t>(nseg, 152 * 16);
  if (elem_bytes == 8)
    k_copy_segments<1><<<g, 256, 0, st>>>(nseg, src_off, dst_off, len, static_cast<const double*>(src),
                                          static_cast<double*>(dst));
  else
    k_copy_segments<2><<<g, 256, 0, st>>>(nseg, src_off, dst_off, len, static_cast<const double*>(src),
                                          static_cast<double*>(dst));
  SKF_CUDA_TRY(cudaGetLastError());
  return SKF_OK;
}

__global__ void k_f64_split(const double* __restrict__ src, float* __restrict__ hi, float* __restrict__ lo, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float h = (float)src[i];
    hi[i] = h;
    lo[i] = (float)(src[i] - (double)h);
  }
}

int split_f64(const double* src, float* hi, float* lo, int64_t n, cudaStream_t st) {
  if (n <= 0) return SKF_OK;
  k_f64_split<<<grid_for(n, 256), 256, 0, st>>>(src, hi, lo, n);
  SKF_CUDA_TRY(cudaGetLastError());
  SKF_CUDA_TRY(cudaStreamSynchronize(st));
  return SKF_OK;
}

int convert_f64_f32(const double* src, float* dst, int64_t n, cudaStream_t st) {
  if (n <= 0) return SKF_OK;
  k_f64_to_f32<<<grid_for(n, 256), 256, 0, st>>>(src, dst, n);
  SKF_CUDA_TRY(cudaGetLastError());
  SKF_CUDA_TRY(cudaStreamSynchronize(st));
  return SKF_OK;
}

// precision: SKF_PREC_FP64, SKF_PREC_MIXED (FP32 kernel evaluation, FP64 T),
// SKF_PREC_MIXED_T32 (FP32 kernel evaluation, FP32 T).
int plan_apply_device(skf_plan* p, const double* x, double* y, int precision, cudaStream_t st) {
  const int W = p->cplx ? 2 : 1;
  const bool mixed = precision != SKF_PREC_FP64;
  const bool t32 = precision == SKF_PREC_MIXED_T32;
  const bool ff = precision == SKF_PREC_MIXED;  // float-float T / T^T
  SKF_CUDA_TRY(cudaMemsetAsync(p->u, 0, sizeof(double) * p->E * W, st));
  SKF_CUDA_TRY(cudaMemsetAsync(p->uh, 0, sizeof(double) * p->E * W, st));
  const int g = grid_for(p->nperm, 256);
  if (p->cplx) k_permute_in<true><<<g, 256, 0, st>>>(p->perm_entry, p->perm_point, p->nperm, x, p->q);
  else k_permute_in<false><<<g, 256, 0, st>>>(p->perm_entry, p->perm_point, p->nperm, x, p->q);
  // upward
  for (int lev = p->nlevels - 1; lev > p->root_level; --lev) {
    const LevelBoxes& L = p->levels[lev];
    if (L.n == 0) continue;
    const size_t sm = sizeof(double) * (size_t)std::max(L.max_red, 1) * W;
    if (ff) {
      if (p->cplx) k_up_ff<true><<<L.n, 256, sm, st>>>(L.dev, p->box_off, p->box_rank, p->t_off, p->t32, p->t32lo, p->pslot, p->q, p->qh);
      else k_up_ff<false><<<L.n, 256, sm, st>>>(L.dev, p->box_off, p->box_rank, p->t_off, p->t32, p->t32lo, p->pslot, p->q, p->qh);
    } else if (p->cplx) {
      if (t32) k_up<true, float><<<L.n, 256, sm, st>>>(L.dev, p->box_off, p->box_rank, p->t_off, p->t32, p->pslot, p->q, p->qh);
      else k_up<true, double><<<L.n, 256, sm, st>>>(L.dev, p->box_off, p->box_rank, p->t_off, p->t64, p->pslot, p->q, p->qh);
    } else {
      if (t32) k_up<false, float><<<L.n, 256, sm, st>>>(L.dev, p->box_off, p->box_rank, p->t_off, p->t32, p->pslot, p->q, p->qh);
      else k_up<false, double><<<L.n, 256, sm, st>>>(L.dev, p->box_off, p->box_rank, p->t_off, p->t64, p->pslot, p->q, p->qh);
    }
  }
  if (mixed) {
    const int gc = grid_for(p->E * W, 256);
    k_charges32<<<gc, 256, 0, st>>>(p->E * W, W, p->entry_skel, p->q, p->qh, p->q32, p->qhn32, p->qd32);
  }
  translate_dispatch(p, mixed, st);
  // downward
  for (int lev = p->root_level + 1; lev < p->nlevels; ++lev) {
    const LevelBoxes& L = p->levels[lev];
    if (L.n == 0) continue;
    const size_t sm = sizeof(double) * (size_t)std::max(L.max_rank, 1) * W;
    if (ff) {
      if (p->cplx) k_down_ff<true><<<L.n, 256, sm, st>>>(L.dev, p->box_off, p->box_rank, p->t_off, p->t32, p->t32lo, p->pslot, p->u, p->uh);
      else k_down_ff<false><<<L.n, 256, sm, st>>>(L.dev, p->box_off, p->box_rank, p->t_off, p->t32, p->t32lo, p->pslot, p->u, p->uh);
    } else if (p->cplx) {
      if (t32) k_down<true, float><<<L.n, 256, sm, st>>>(L.dev, p->box_off, p->box_rank, p->t_off, p->t32, p->pslot, p->u, p->uh);
      else k_down<true, double><<<L.n, 256, sm, st>>>(L.dev, p->box_off, p->box_rank, p->t_off, p->t64, p->pslot, p->u, p->uh);
    } else {
      if (t32) k_down<false, float><<<L.n, 256, sm, st>>>(L.dev, p->box_off, p->box_rank, p->t_off, p->t32, p->pslot, p->u, p->uh);
      else k_down<false, double><<<L.n, 256, sm, st>>>(L.dev, p->box_off, p->box_rank, p->t_off, p->t64, p->pslot, p->u, p->uh);
    }
  }
  if (p->cplx) k_permute_out<true><<<g, 256, 0, st>>>(p->perm_entry, p->perm_point, p->nperm, p->u, y);
  else k_permute_out<false><<<g, 256, 0, st>>>(p->perm_entry, p->perm_point, p->nperm, p->u, y);
  SKF_CUDA_TRY(cudaGetLastError());
  return SKF_OK;
}

int plan_time_translations(skf_plan* p, bool mixed, int reps, cudaStream_t st, float* ms) {
  cudaEvent_t e0, e1;
  SKF_CUDA_TRY(cudaEventCreate(&e0));
  SKF_CUDA_TRY(cudaEventCreate(&e1));
  SKF_CUDA_TRY(cudaEventRecord(e0, st));
  for (int i = 0; i < reps; ++i) translate_dispatch(p, mixed, st);
  SKF_CUDA_TRY(cudaEventRecord(e1, st));
  SKF_CUDA_TRY(cudaEventSynchronize(e1));
  float t = 0;
  SKF_CUDA_TRY(cudaEventElapsedTime(&t, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms = t / std::max(reps, 1);
  SKF_CUDA_TRY(cudaGetLastError());
  return SKF_OK;
}

// ------------------------------------------------------------------ kernel-apply seam
template <int OP, bool MIXED>
__global__ void k_block_apply(int npairs, int mmax, int nmax, const int32_t* __restrict__ m,
                              const int32_t* __restrict__ n, const double* __restrict__ xt,
                              const double* __restrict__ xs, const double* __restrict__ gt,
                              const double* __restrict__ gs, const double* __restrict__ q,
                              const int8_t* __restrict__ self_flag, double* __restrict__ out, double kappa) {
  constexpr bool C = OpTraits<OP>::kComplex;
  constexpr int D = OpTraits<OP>::kDim;
  constexpr int G = OpTraits<OP>::kGeom;
  const int pr = blockIdx.x;
  const int i = blockIdx.y * blockDim.x + threadIdx.x;
  if (pr >= npairs || i >= m[pr]) return;
  const int nn = n[pr];
  const bool self = self_flag != nullptr && self_flag[pr] != 0;
  const double* xi = xt + ((int64_t)pr * mmax + i) * D;
  double ar = 0, ai = 0;
  const float kf = (float)kappa;
  for (int j = 0; j < nn; ++j) {
    const double* yj = xs + ((int64_t)pr * nmax + j) * D;
    double gx = 0, gy = 0, gz = 0;
    if (G == 1) {
      const double* g = gs + ((int64_t)pr * nmax + j) * 3;
      gx = g[0]; gy = g[1]; gz = g[2];
    } else if (G == 2) {
      const double* g = gt + ((int64_t)pr * mmax + i) * 3;
      gx = g[0]; gy = g[1]; gz = g[2];
    }
    double kr, ki;
    if (MIXED) {
      // the difference as an FP32 pair dh + dl of the FP64 difference (the
      // plan's binade-shifted hi/lo split gives the same pair to ~2^-48)
      float d[3] = {0, 0, 0}, dh[3] = {0, 0, 0}, dl[3] = {0, 0, 0};
#pragma unroll
      for (int c = 0; c < D; ++c) {
        const double dd = xi[c] - yj[c];
        dh[c] = (float)dd;
        dl[c] = (float)(dd - (double)dh[c]);
        d[c] = dh[c] + dl[c];
      }
      float rotn = 0.f;
      if (G != 0) {
        const float nh[3] = {(float)gx, (float)gy, (float)gz};
        rotn = dot_dn(dh[0], dh[1], dh[2], dl[0], dl[1], dl[2], nh[0], nh[1], nh[2], (float)(gx - (double)nh[0]),
                      (float)(gy - (double)nh[1]), (float)(gz - (double)nh[2]));
      }
      float fr, fi;
      eval_f32<OP>(d[0], d[1], d[2], rotn, kf, fr, fi);
      kr = fr;
      ki = fi;
    } else {
      const double dz = (D == 3) ? xi[2] - yj[2] : 0.0;
      eval_f64<OP>(xi[0] - yj[0], xi[1] - yj[1], dz, gx, gy, gz, kappa, kr, ki);
    }
    if (self && j == i) {
      kr = 0;
      ki = 0;
    }
    const int64_t qi = (int64_t)pr * nmax + j;
    if (C) {
      const double qr = q[2 * qi], qim = q[2 * qi + 1];
      ar += kr * qr - ki * qim;
      ai += kr * qim + ki * qr;
    } else {
      ar += kr * q[qi];
    }
  }
  const int64_t o = (int64_t)pr * mmax + i;
  if (C) {
    out[2 * o] = ar;
    out[2 * o + 1] = ai;
  } else {
    out[o] = ar;
  }
}

template <int OP>
static void launch_block(int npairs, int mmax, int nmax, const int32_t* m, const int32_t* n, const double* xt,
                         const double* xs, const double* gt, const double* gs, const double* q, const int8_t* sf,
                         double* out, double kappa, bool mixed, cudaStream_t st) {
  dim3 grid(npairs, (mmax + 127) / 128);  // pairs on x (2^31 - 1), row tiles on y
  if (mixed) k_block_apply<OP, true><<<grid, 128, 0, st>>>(npairs, mmax, nmax, m, n, xt, xs, gt, gs, q, sf, out, kappa);
  else k_block_apply<OP, false><<<grid, 128, 0, st>>>(npairs, mmax, nmax, m, n, xt, xs, gt, gs, q, sf, out, kappa);
}

int kernel_apply(int op, double kappa, int npairs, int mmax, int nmax, const int32_t* m, const int32_t* n,
                 const double* xt, const double* xs, const double* gt, const double* gs, const double* q,
                 const int8_t* sf, double* out, bool mixed, cudaStream_t st) {
  switch (op) {
#define SKF_CASE(OPID) \
  case OPID: launch_block<OPID>(npairs, mmax, nmax, m, n, xt, xs, gt, gs, q, sf, out, kappa, mixed, st); break;
    SKF_CASE(SKF_LAPLACE_2D)
    SKF_CASE(SKF_LAPLACE_3D)
    SKF_CASE(SKF_HELMHOLTZ_2D)
    SKF_CASE(SKF_HELMHOLTZ_3D)
    SKF_CASE(SKF_LAPLACE_DOUBLE_LAYER_3D)
    SKF_CASE(SKF_LAPLACE_ADJOINT_DOUBLE_LAYER_3D)
    SKF_CASE(SKF_HELMHOLTZ_DOUBLE_LAYER_3D)
    SKF_CASE(SKF_HELMHOLTZ_ADJOINT_DOUBLE_LAYER_3D)
#undef SKF_CASE
    default: return SKF_ERR_ARG;
  }
  SKF_CUDA_TRY(cudaGetLastError());
  return SKF_OK;
}

}  // namespace skf
