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

// ------------------------------------------------------------------ translations
struct TransArgs {
  const int32_t* work_box;
  const int32_t* work_row;
  const int64_t* box_off;
  const int32_t* box_rank;
  const int64_t* list_off;
  const int32_t* list_src;
  const int8_t* list_kind;
  const double4_32a* xyz64;
  const double4_32a* geom64;
  const float4* hi32;
  const float4* lo32;
  const float4* geom32;
  const double* q;
  const double* qh;
  double* u;
  double* uh;
  double kappa;
};

// Effective source charges of entry j of source box s for a translation kind:
// acc_u += K * c1 ; acc_h += K * c2 (acc_h only kept for the target's skeleton rows).
__device__ __forceinline__ void kind_charges(int kind, int j, int rs, double q, double qh, double& c1, double& c2) {
  const bool sk = j < rs;
  switch (kind) {
    case SKF_KIND_COLLEAGUE:
      c1 = q;
      c2 = sk ? -qh : 0.0;
      break;
    case SKF_KIND_COARSE_UP:
      c1 = q;
      c2 = -q;
      break;
    case SKF_KIND_COARSE_DOWN:
      c1 = sk ? q - qh : q;
      c2 = 0.0;
      break;
    default:
      c1 = q;
      c2 = 0.0;
      break;
  }
}

// FP64 translation kernel: one block per (target box, 128-row tile).
template <int OP>
__global__ void __launch_bounds__(kTransThreads) k_translate_f64(TransArgs a) {
  constexpr bool C = OpTraits<OP>::kComplex;
  constexpr int G = OpTraits<OP>::kGeom;
  constexpr int TS = kTileSrcF64;
  __shared__ double2 sA[TS];  // x, y
  __shared__ double2 sB[TS];  // z, c1r
  __shared__ double2 sC[TS];  // c2r, c1i
  __shared__ double2 sD[TS];  // c2i, gx
  __shared__ double2 sE[TS];  // gy, gz

  const int U = a.work_box[blockIdx.x];
  const int row0 = a.work_row[blockIdx.x];
  const int64_t offU = a.box_off[U];
  const int bsU = (int)(a.box_off[U + 1] - offU);
  const int rU = a.box_rank[U];
  const int row = row0 + threadIdx.x;
  const bool valid = row < bsU;
  const int64_t eT = offU + (valid ? row : bsU - 1);
  const double4_32a tp = a.xyz64[eT];
  double4_32a tg = make_double4_32a(0, 0, 0, 0);
  if (G == 2) tg = a.geom64[eT];
  const bool need_h = (row0 + (threadIdx.x & ~31)) < rU;

  double aur = 0, aui = 0, ahr = 0, ahi = 0;
  const int64_t l0 = a.list_off[U], l1 = a.list_off[U + 1];
  for (int64_t l = l0; l < l1; ++l) {
    const int s = a.list_src[l];
    const int kind = a.list_kind[l];
    const int64_t offS = a.box_off[s];
    const int bsS = (int)(a.box_off[s + 1] - offS);
    const int rS = a.box_rank[s];
    const int nh = (kind == SKF_KIND_COLLEAGUE) ? rS : ((kind == SKF_KIND_COARSE_UP) ? bsS : 0);
    for (int t0 = 0; t0 < bsS; t0 += TS) {
      const int nt = min(TS, bsS - t0);
      __syncthreads();
      for (int j = threadIdx.x; j < nt; j += blockDim.x) {
        const int js = t0 + j;
        const int64_t e = offS + js;
        const double4_32a p = a.xyz64[e];
        double c1r, c2r, c1i = 0, c2i = 0;
        if (C) {
          kind_charges(kind, js, rS, a.q[2 * e], a.qh[2 * e], c1r, c2r);
          kind_charges(kind, js, rS, a.q[2 * e + 1], a.qh[2 * e + 1], c1i, c2i);
        } else {
          kind_charges(kind, js, rS, a.q[e], a.qh[e], c1r, c2r);
        }
        sA[j] = make_double2(p.x, p.y);
        sB[j] = make_double2(p.z, c1r);
        sC[j] = make_double2(c2r, c1i);
        double4_32a g = make_double4_32a(0, 0, 0, 0);
        if (G == 1) g = a.geom64[e];
        sD[j] = make_double2(c2i, g.x);
        sE[j] = make_double2(g.y, g.z);
      }
      __syncthreads();
      const bool doh = need_h && (t0 < nh);
      for (int j = 0; j < nt; ++j) {
        const double2 A = sA[j], B = sB[j];
        const double dx = tp.x - A.x, dy = tp.y - A.y, dz = tp.z - B.x;
        double gx = 0, gy = 0, gz = 0;
        if (G == 1) {
          gx = sD[j].y;
          const double2 E = sE[j];
          gy = E.x;
          gz = E.y;
        } else if (G == 2) {
          gx = tg.x;
          gy = tg.y;
          gz = tg.z;
        }
        double kr, ki;
        eval_f64<OP>(dx, dy, dz, gx, gy, gz, a.kappa, kr, ki);
        const double2 Cc = sC[j];
        if (C) {
          const double c1i = Cc.y;
          aur = fma(kr, B.y, fma(-ki, c1i, aur));
          aui = fma(kr, c1i, fma(ki, B.y, aui));
          if (doh) {
            const double c2i = sD[j].x;
            ahr = fma(kr, Cc.x, fma(-ki, c2i, ahr));
            ahi = fma(kr, c2i, fma(ki, Cc.x, ahi));
          }
        } else {
          aur = fma(kr, B.y, aur);
          if (doh) ahr = fma(kr, Cc.x, ahr);
        }
      }
    }
  }
  if (valid) {
    const bool sk = row < rU;
    if (C) {
      a.u[2 * eT] = aur;
      a.u[2 * eT + 1] = aui;
      a.uh[2 * eT] = sk ? ahr : 0.0;
      a.uh[2 * eT + 1] = sk ? ahi : 0.0;
    } else {
      a.u[eT] = aur;
      a.uh[eT] = sk ? ahr : 0.0;
    }
  }
}

// Mixed translation kernel: FP32 kernel evaluation with accurate, level-
// independent differences (hi/lo split coordinates), FP32 partial sums per
// source tile, FP64 accumulation across tiles.  Two target rows per thread.
template <int OP>
__global__ void __launch_bounds__(kTransThreads) k_translate_f32(TransArgs a) {
  constexpr bool C = OpTraits<OP>::kComplex;
  constexpr int G = OpTraits<OP>::kGeom;
  constexpr int TS = kTileSrcF32;
  constexpr int RPT = kRowsPerThreadF32;
  __shared__ float4 sA[TS];  // hx, hy, hz, c1r
  __shared__ float4 sB[TS];  // lx, ly, lz, c2r
  __shared__ float4 sC[(C || G == 1) ? TS : 1];  // c1i, c2i, gx, gy
  __shared__ float sD[(G == 1) ? TS : 1];        // gz

  const int U = a.work_box[blockIdx.x];
  const int row0 = a.work_row[blockIdx.x];
  const int64_t offU = a.box_off[U];
  const int bsU = (int)(a.box_off[U + 1] - offU);
  const int rU = a.box_rank[U];
  const float kappa = (float)a.kappa;

  float4 th[RPT], tl[RPT], tg[RPT];
  int64_t eT[RPT];
  bool valid[RPT];
#pragma unroll
  for (int k = 0; k < RPT; ++k) {
    const int row = row0 + threadIdx.x + k * kTransThreads;
    valid[k] = row < bsU;
    eT[k] = offU + (valid[k] ? row : bsU - 1);
    th[k] = a.hi32[eT[k]];
    tl[k] = a.lo32[eT[k]];
    tg[k] = (G == 2) ? a.geom32[eT[k]] : make_float4(0, 0, 0, 0);
  }
  const bool need_h = (row0 + (threadIdx.x & ~31)) < rU;

  double aur[RPT], aui[RPT], ahr[RPT], ahi[RPT];
#pragma unroll
  for (int k = 0; k < RPT; ++k) aur[k] = aui[k] = ahr[k] = ahi[k] = 0.0;

  const int64_t l0 = a.list_off[U], l1 = a.list_off[U + 1];
  for (int64_t l = l0; l < l1; ++l) {
    const int s = a.list_src[l];
    const int kind = a.list_kind[l];
    const int64_t offS = a.box_off[s];
    const int bsS = (int)(a.box_off[s + 1] - offS);
    const int rS = a.box_rank[s];
    const int nh = (kind == SKF_KIND_COLLEAGUE) ? rS : ((kind == SKF_KIND_COARSE_UP) ? bsS : 0);
    for (int t0 = 0; t0 < bsS; t0 += TS) {
      const int nt = min(TS, bsS - t0);
      __syncthreads();
      for (int j = threadIdx.x; j < nt; j += blockDim.x) {
        const int js = t0 + j;
        const int64_t e = offS + js;
        const float4 h = a.hi32[e], lo = a.lo32[e];
        double c1r, c2r, c1i = 0, c2i = 0;
        if (C) {
          kind_charges(kind, js, rS, a.q[2 * e], a.qh[2 * e], c1r, c2r);
          kind_charges(kind, js, rS, a.q[2 * e + 1], a.qh[2 * e + 1], c1i, c2i);
        } else {
          kind_charges(kind, js, rS, a.q[e], a.qh[e], c1r, c2r);
        }
        sA[j] = make_float4(h.x, h.y, h.z, (float)c1r);
        sB[j] = make_float4(lo.x, lo.y, lo.z, (float)c2r);
        if (C || G == 1) {
          float4 g = (G == 1) ? a.geom32[e] : make_float4(0, 0, 0, 0);
          sC[j] = make_float4((float)c1i, (float)c2i, g.x, g.y);
          if (G == 1) sD[j] = g.z;
        }
      }
      __syncthreads();
      const bool doh = need_h && (t0 < nh);
      float pur[RPT], pui[RPT], phr[RPT], phi[RPT];
#pragma unroll
      for (int k = 0; k < RPT; ++k) pur[k] = pui[k] = phr[k] = phi[k] = 0.f;
      if (doh) {
#pragma unroll 2
        for (int j = 0; j < nt; ++j) {
          const float4 A = sA[j], B = sB[j];
          float4 Cc = make_float4(0, 0, 0, 0);
          if (C || G == 1) Cc = sC[j];
#pragma unroll
          for (int k = 0; k < RPT; ++k) {
            const float dx = (th[k].x - A.x) + (tl[k].x - B.x);
            const float dy = (th[k].y - A.y) + (tl[k].y - B.y);
            const float dz = (th[k].z - A.z) + (tl[k].z - B.z);
            float gx = 0, gy = 0, gz = 0;
            if (G == 1) {
              gx = Cc.z;
              gy = Cc.w;
              gz = sD[j];
            } else if (G == 2) {
              gx = tg[k].x;
              gy = tg[k].y;
              gz = tg[k].z;
            }
            float kr, ki;
            eval_f32<OP>(dx, dy, dz, gx, gy, gz, kappa, kr, ki);
            if (C) {
              pur[k] = fmaf(kr, A.w, fmaf(-ki, Cc.x, pur[k]));
              pui[k] = fmaf(kr, Cc.x, fmaf(ki, A.w, pui[k]));
              phr[k] = fmaf(kr, B.w, fmaf(-ki, Cc.y, phr[k]));
              phi[k] = fmaf(kr, Cc.y, fmaf(ki, B.w, phi[k]));
            } else {
              pur[k] = fmaf(kr, A.w, pur[k]);
              phr[k] = fmaf(kr, B.w, phr[k]);
            }
          }
        }
      } else {
#pragma unroll 2
        for (int j = 0; j < nt; ++j) {
          const float4 A = sA[j], B = sB[j];
          float4 Cc = make_float4(0, 0, 0, 0);
          if (C || G == 1) Cc = sC[j];
#pragma unroll
          for (int k = 0; k < RPT; ++k) {
            const float dx = (th[k].x - A.x) + (tl[k].x - B.x);
            const float dy = (th[k].y - A.y) + (tl[k].y - B.y);
            const float dz = (th[k].z - A.z) + (tl[k].z - B.z);
            float gx = 0, gy = 0, gz = 0;
            if (G == 1) {
              gx = Cc.z;
              gy = Cc.w;
              gz = sD[j];
            } else if (G == 2) {
              gx = tg[k].x;
              gy = tg[k].y;
              gz = tg[k].z;
            }
            float kr, ki;
            eval_f32<OP>(dx, dy, dz, gx, gy, gz, kappa, kr, ki);
            if (C) {
              pur[k] = fmaf(kr, A.w, fmaf(-ki, Cc.x, pur[k]));
              pui[k] = fmaf(kr, Cc.x, fmaf(ki, A.w, pui[k]));
            } else {
              pur[k] = fmaf(kr, A.w, pur[k]);
            }
          }
        }
      }
#pragma unroll
      for (int k = 0; k < RPT; ++k) {
        aur[k] += (double)pur[k];
        ahr[k] += (double)phr[k];
        if (C) {
          aui[k] += (double)pui[k];
          ahi[k] += (double)phi[k];
        }
      }
    }
  }
#pragma unroll
  for (int k = 0; k < RPT; ++k) {
    if (!valid[k]) continue;
    const int row = row0 + threadIdx.x + k * kTransThreads;
    const bool sk = row < rU;
    const int64_t e = eT[k];
    if (C) {
      a.u[2 * e] = aur[k];
      a.u[2 * e + 1] = aui[k];
      a.uh[2 * e] = sk ? ahr[k] : 0.0;
      a.uh[2 * e + 1] = sk ? ahi[k] : 0.0;
    } else {
      a.u[e] = aur[k];
      a.uh[e] = sk ? ahr[k] : 0.0;
    }
  }
}

// ------------------------------------------------------------------ dispatch
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
    a.work_box = p->work32.box;
    a.work_row = p->work32.row;
    if (p->work32.n > 0) k_translate_f32<OP><<<p->work32.n, kTransThreads, 0, st>>>(a);
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

int plan_apply_device(skf_plan* p, const double* x, double* y, bool mixed, cudaStream_t st) {
  const int W = p->cplx ? 2 : 1;
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
    if (p->cplx) {
      if (mixed) k_up<true, float><<<L.n, 256, sm, st>>>(L.dev, p->box_off, p->box_rank, p->t_off, p->t32, p->pslot, p->q, p->qh);
      else k_up<true, double><<<L.n, 256, sm, st>>>(L.dev, p->box_off, p->box_rank, p->t_off, p->t64, p->pslot, p->q, p->qh);
    } else {
      if (mixed) k_up<false, float><<<L.n, 256, sm, st>>>(L.dev, p->box_off, p->box_rank, p->t_off, p->t32, p->pslot, p->q, p->qh);
      else k_up<false, double><<<L.n, 256, sm, st>>>(L.dev, p->box_off, p->box_rank, p->t_off, p->t64, p->pslot, p->q, p->qh);
    }
  }
  translate_dispatch(p, mixed, st);
  // downward
  for (int lev = p->root_level + 1; lev < p->nlevels; ++lev) {
    const LevelBoxes& L = p->levels[lev];
    if (L.n == 0) continue;
    const size_t sm = sizeof(double) * (size_t)std::max(L.max_rank, 1) * W;
    if (p->cplx) {
      if (mixed) k_down<true, float><<<L.n, 256, sm, st>>>(L.dev, p->box_off, p->box_rank, p->t_off, p->t32, p->pslot, p->u, p->uh);
      else k_down<true, double><<<L.n, 256, sm, st>>>(L.dev, p->box_off, p->box_rank, p->t_off, p->t64, p->pslot, p->u, p->uh);
    } else {
      if (mixed) k_down<false, float><<<L.n, 256, sm, st>>>(L.dev, p->box_off, p->box_rank, p->t_off, p->t32, p->pslot, p->u, p->uh);
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
  const int pr = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
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
      float d[3] = {0, 0, 0};
#pragma unroll
      for (int c = 0; c < D; ++c) {
        const float hx = (float)xi[c], hy = (float)yj[c];
        const float lx = (float)(xi[c] - (double)hx), ly = (float)(yj[c] - (double)hy);
        d[c] = (hx - hy) + (lx - ly);
      }
      float fr, fi;
      eval_f32<OP>(d[0], d[1], d[2], (float)gx, (float)gy, (float)gz, kf, fr, fi);
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
  dim3 grid((mmax + 127) / 128, npairs);
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
