// skf_translate.cuh — the translation kernels (near field + skeleton
// translations of every level in one launch).
//
// One thread block owns a tile of target rows of one box U and walks U's
// interaction list (colleagues incl. U itself, coarse-up, coarse-down, root);
// for every source box it stages the sources in shared memory and
// accumulates, per target row,
//   u  += sum_j K(x_i, y_j) c1_j           (all rows)
//   uh += sum_j K(x_i, y_j) c2_j           (U's skeleton rows)
// with the effective charges c1/c2 of the translation kind (kind_charges).
// No atomics: a row is written by exactly one block, so applies are bitwise
// reproducible.  Coincident points only meet in U's self pair (identical
// points share a box at every level), so only self pairs test r == 0.
#pragma once
#include <type_traits>

#include "skf_internal.cuh"
#include "skf_kernels.cuh"

namespace skf {

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
// acc_u += K * c1 ; acc_h += K * c2.
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

// ------------------------------------------------------------------ FP64
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
    const bool self = (s == U);
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
        if (self) {
          eval_f64<OP>(dx, dy, dz, gx, gy, gz, a.kappa, kr, ki);
        } else {
          eval_f64<OP, false>(dx, dy, dz, gx, gy, gz, a.kappa, kr, ki);
        }
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

// ------------------------------------------------------------------ mixed (FP32)
// FP32 kernel evaluation.  Differences are formed from hi/lo split
// coordinates, d = (hi_i - hi_j) + (lo_i - lo_j), which is accurate to FP32
// rounding of d itself and identical for a pair at every level (so the add at
// a parent level and the subtract at the child level cancel exactly).  Each
// thread owns kRowsPerThreadF32 consecutive rows, so one broadcast
// shared-memory read of a source feeds that many kernel evaluations.  Tile
// sums are FP32 and are accumulated with Knuth's TwoSum (a compensated FP32
// pair), which keeps the FP64 pipe out of the loop.
template <int OP, bool H, bool SELF, int RPT>
__device__ __forceinline__ void t32_tile(const float4* __restrict__ sA, const float4* __restrict__ sB,
                                         const float4* __restrict__ sC, const float* __restrict__ sD,
                                         const float4* __restrict__ sE, int nt, const float4 (&th)[RPT],
                                         const float4 (&tl)[RPT], const float4 (&tg)[RPT],
                                         const float4 (&tgl)[RPT], float kappa, float (&pur)[RPT],
                                         float (&pui)[RPT], float (&phr)[RPT], float (&phi)[RPT]) {
  constexpr bool C = OpTraits<OP>::kComplex;
  constexpr int G = OpTraits<OP>::kGeom;
#pragma unroll 4
  for (int j = 0; j < nt; ++j) {
    const float4 A = sA[j], B = sB[j];
    float4 Cc = make_float4(0, 0, 0, 0);
    if (C || G == 1) Cc = sC[j];
    float gzs = 0;
    float4 gl = make_float4(0, 0, 0, 0);
    if (G == 1) {
      gzs = sD[j];
      gl = sE[j];
    }
#pragma unroll
    for (int k = 0; k < RPT; ++k) {
      const float dhx = th[k].x - A.x, dlx = tl[k].x - B.x;
      const float dhy = th[k].y - A.y, dly = tl[k].y - B.y;
      const float dhz = th[k].z - A.z, dlz = tl[k].z - B.z;
      const float dx = dhx + dlx, dy = dhy + dly, dz = dhz + dlz;
      float rotn = 0.f;
      if (G == 1) rotn = dot_dn(dhx, dhy, dhz, dlx, dly, dlz, Cc.z, Cc.w, gzs, gl.x, gl.y, gl.z);
      else if (G == 2)
        rotn = dot_dn(dhx, dhy, dhz, dlx, dly, dlz, tg[k].x, tg[k].y, tg[k].z, tgl[k].x, tgl[k].y, tgl[k].z);
      float kr, ki;
      eval_f32<OP, SELF>(dx, dy, dz, rotn, kappa, kr, ki);
      if (C) {
        pur[k] = fmaf(kr, A.w, fmaf(-ki, Cc.x, pur[k]));
        pui[k] = fmaf(kr, Cc.x, fmaf(ki, A.w, pui[k]));
        if (H) {
          phr[k] = fmaf(kr, B.w, fmaf(-ki, Cc.y, phr[k]));
          phi[k] = fmaf(kr, Cc.y, fmaf(ki, B.w, phi[k]));
        }
      } else {
        pur[k] = fmaf(kr, A.w, pur[k]);
        if (H) phr[k] = fmaf(kr, B.w, phr[k]);
      }
    }
  }
}

// s + c += p, with the rounding error of the sum carried in c (TwoSum).
__device__ __forceinline__ void two_sum_add(float& s, float& c, float p) {
  const float t = s + p;
  const float z = t - s;
  c += (s - (t - z)) + (p - z);
  s = t;
}

struct TransArgs32 {
  const int32_t* work_box;
  const int32_t* work_row;
  const int64_t* box_off;
  const int32_t* box_rank;
  const int64_t* list_off;
  const int32_t* list_src;
  const int8_t* list_kind;
  const float4* hi32;
  const float4* lo32;
  const float4* geom32;
  const float4* geom32lo;
  const float* q32;
  const float* qhn32;
  const float* qd32;
  double* u;
  double* uh;
  float kappa;
};

template <int OP>
__global__ void __launch_bounds__(kT32Threads) k_translate_f32(TransArgs32 a) {
  constexpr bool C = OpTraits<OP>::kComplex;
  constexpr int G = OpTraits<OP>::kGeom;
  constexpr int TS = kTileSrcF32;
  constexpr int RPT = kRowsPerThreadF32;
  constexpr int W = C ? 2 : 1;
  __shared__ float4 sA[TS];  // hx, hy, hz, c1r
  __shared__ float4 sB[TS];  // lx, ly, lz, c2r
  __shared__ float4 sC[(C || G == 1) ? TS : 1];  // c1i, c2i, gx, gy
  __shared__ float sD[(G == 1) ? TS : 1];        // gz
  __shared__ float4 sE[(G == 1) ? TS : 1];       // lo parts of the normal

  const int U = a.work_box[blockIdx.x];
  const int row0 = a.work_row[blockIdx.x];
  const int64_t offU = a.box_off[U];
  const int bsU = (int)(a.box_off[U + 1] - offU);
  const int rU = a.box_rank[U];
  const int rowt = row0 + RPT * threadIdx.x;  // first row of this thread

  float4 th[RPT], tl[RPT], tg[RPT], tgl[RPT];
#pragma unroll
  for (int k = 0; k < RPT; ++k) {
    const int row = rowt + k;
    const int64_t e = offU + (row < bsU ? row : bsU - 1);
    th[k] = a.hi32[e];
    tl[k] = a.lo32[e];
    tg[k] = (G == 2) ? a.geom32[e] : make_float4(0, 0, 0, 0);
    tgl[k] = (G == 2) ? a.geom32lo[e] : make_float4(0, 0, 0, 0);
  }
  // skeleton rows need uh; decided per warp so the branch stays uniform
  const bool need_h = (row0 + RPT * (threadIdx.x & ~31)) < rU;

  // compensated FP32 accumulators: value s, error c
  float sur[RPT], cur[RPT], sui[RPT], cui[RPT], shr[RPT], chr[RPT], shi[RPT], chi[RPT];
#pragma unroll
  for (int k = 0; k < RPT; ++k) sur[k] = cur[k] = sui[k] = cui[k] = shr[k] = chr[k] = shi[k] = chi[k] = 0.f;

  const int64_t l0 = a.list_off[U], l1 = a.list_off[U + 1];
  for (int64_t l = l0; l < l1; ++l) {
    const int s = a.list_src[l];
    const int kind = a.list_kind[l];
    const int64_t offS = a.box_off[s];
    const int bsS = (int)(a.box_off[s + 1] - offS);
    const int rS = a.box_rank[s];
    // sources [0, nh) carry a non-zero uh charge; tiles are cut at nh
    const int nh = (kind == SKF_KIND_COLLEAGUE) ? rS : ((kind == SKF_KIND_COARSE_UP) ? bsS : 0);
    const bool self = (s == U);
    const float* c1src = (kind == SKF_KIND_COARSE_DOWN) ? a.qd32 : a.q32;
    for (int t0 = 0; t0 < bsS;) {
      const bool hseg = t0 < nh;
      const int nt = min(TS, (hseg ? nh : bsS) - t0);
      __syncthreads();
      for (int j = threadIdx.x; j < nt; j += blockDim.x) {
        const int64_t e = offS + t0 + j;
        const float4 h = a.hi32[e], lo = a.lo32[e];
        float c1r = c1src[e * W], c1i = C ? c1src[e * W + 1] : 0.f;
        float c2r = 0.f, c2i = 0.f;
        if (kind == SKF_KIND_COLLEAGUE) {
          c2r = a.qhn32[e * W];
          if (C) c2i = a.qhn32[e * W + 1];
        } else if (kind == SKF_KIND_COARSE_UP) {
          c2r = -c1r;
          c2i = -c1i;
        }
        sA[j] = make_float4(h.x, h.y, h.z, c1r);
        sB[j] = make_float4(lo.x, lo.y, lo.z, c2r);
        if (C || G == 1) {
          const float4 g = (G == 1) ? a.geom32[e] : make_float4(0, 0, 0, 0);
          sC[j] = make_float4(c1i, c2i, g.x, g.y);
          if (G == 1) {
            sD[j] = g.z;
            sE[j] = a.geom32lo[e];
          }
        }
      }
      __syncthreads();
      float pur[RPT], pui[RPT], phr[RPT], phi[RPT];
#pragma unroll
      for (int k = 0; k < RPT; ++k) pur[k] = pui[k] = phr[k] = phi[k] = 0.f;
      const bool doh = need_h && hseg;
      if (doh) {
        if (self) t32_tile<OP, true, true, RPT>(sA, sB, sC, sD, sE, nt, th, tl, tg, tgl, a.kappa, pur, pui, phr, phi);
        else t32_tile<OP, true, false, RPT>(sA, sB, sC, sD, sE, nt, th, tl, tg, tgl, a.kappa, pur, pui, phr, phi);
      } else {
        if (self) t32_tile<OP, false, true, RPT>(sA, sB, sC, sD, sE, nt, th, tl, tg, tgl, a.kappa, pur, pui, phr, phi);
        else t32_tile<OP, false, false, RPT>(sA, sB, sC, sD, sE, nt, th, tl, tg, tgl, a.kappa, pur, pui, phr, phi);
      }
#pragma unroll
      for (int k = 0; k < RPT; ++k) {
        two_sum_add(sur[k], cur[k], pur[k]);
        if (C) two_sum_add(sui[k], cui[k], pui[k]);
        if (doh) {
          two_sum_add(shr[k], chr[k], phr[k]);
          if (C) two_sum_add(shi[k], chi[k], phi[k]);
        }
      }
      t0 += nt;
    }
  }
#pragma unroll
  for (int k = 0; k < RPT; ++k) {
    const int row = rowt + k;
    if (row >= bsU) continue;
    const bool sk = row < rU;
    const int64_t e = offU + row;
    if (C) {
      a.u[2 * e] = (double)sur[k] + (double)cur[k];
      a.u[2 * e + 1] = (double)sui[k] + (double)cui[k];
      a.uh[2 * e] = sk ? (double)shr[k] + (double)chr[k] : 0.0;
      a.uh[2 * e + 1] = sk ? (double)shi[k] + (double)chi[k] : 0.0;
    } else {
      a.u[e] = (double)sur[k] + (double)cur[k];
      a.uh[e] = sk ? (double)shr[k] + (double)chr[k] : 0.0;
    }
  }
}

}  // namespace skf

namespace skf {

// ------------------------------------------------------------------ mixed, packed FP32x2
// Laplace 2D/3D translations with Blackwell's packed FP32x2 arithmetic
// (add/mul/fma.rn.f32x2): every instruction works on two target rows, which
// halves the issue slots per kernel evaluation; rsqrt/lg2 stay scalar (MUFU).
// One warp per block, kX2Rows rows per thread (row0 + lane + 32 k), sources
// staged in shared memory pre-negated and duplicated into both halves.
// Same arithmetic per evaluation as k_translate_f32 (hi/lo differences,
// compensated FP32 sums), so results agree with it to FP32 rounding order.
typedef unsigned long long f2_t;  // two FP32 values in one 64-bit register

__device__ __forceinline__ f2_t f2_add(f2_t a, f2_t b) {
  f2_t d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2_t f2_mul(f2_t a, f2_t b) {
  f2_t d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2_t f2_fma(f2_t a, f2_t b, f2_t c) {
  f2_t d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ f2_t f2_pack(float lo, float hi) {
  f2_t d;
  asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(lo), "f"(hi));
  return d;
}
__device__ __forceinline__ void f2_unpack(f2_t v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}

// NP packed row pairs per thread: lane l of warp w owns rows
// row0 + 64 NP w + 32 k + l, k < 2 NP; row pair p = (k = 2p, 2p + 1).
template <int D, int NP, bool H, bool SELF, bool LOG>
__device__ __forceinline__ void x2_tile(const ulonglong2* __restrict__ s0, const ulonglong2* __restrict__ s1,
                                        const ulonglong2* __restrict__ s2, const ulonglong2* __restrict__ s3, int nt,
                                        const f2_t (&thx)[NP], const f2_t (&thy)[NP], const f2_t (&thz)[NP],
                                        const f2_t (&tlx)[NP], const f2_t (&tly)[NP], const f2_t (&tlz)[NP],
                                        f2_t (&pu)[NP], f2_t (&ph)[NP]) {
#pragma unroll 4
  for (int j = 0; j < nt; ++j) {
    const ulonglong2 A = s0[j];   // (-hx,-hx), (-hy,-hy)
    const ulonglong2 B = s1[j];   // (-hz,-hz), (-lx,-lx)
    const ulonglong2 Cc = s2[j];  // (-ly,-ly), (-lz,-lz)
    const ulonglong2 Q = s3[j];   // (c1,c1), (c2,c2)
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      const f2_t dx = f2_add(f2_add(thx[p], A.x), f2_add(tlx[p], B.y));
      const f2_t dy = f2_add(f2_add(thy[p], A.y), f2_add(tly[p], Cc.x));
      f2_t r2 = f2_mul(dx, dx);
      r2 = f2_fma(dy, dy, r2);
      if (D == 3) {
        const f2_t dz = f2_add(f2_add(thz[p], B.x), f2_add(tlz[p], Cc.y));
        r2 = f2_fma(dz, dz, r2);
      }
      float ra, rb;
      f2_unpack(r2, ra, rb);
      float ka = LOG ? lg2_approx(ra) : rsqrt_approx(ra);
      float kb = LOG ? lg2_approx(rb) : rsqrt_approx(rb);
      if (SELF) {
        ka = ra > 0.f ? ka : 0.f;
        kb = rb > 0.f ? kb : 0.f;
      }
      const f2_t k = f2_pack(ka, kb);
      pu[p] = f2_fma(k, Q.x, pu[p]);
      if (H) ph[p] = f2_fma(k, Q.y, ph[p]);
    }
  }
}

// s + c += p for both halves (TwoSum, see two_sum_add).
__device__ __forceinline__ void f2_two_sum(f2_t& s, f2_t& c, f2_t p) {
  const f2_t t = f2_add(s, p);
  const f2_t neg = f2_pack(-1.f, -1.f);
  const f2_t z = f2_fma(s, neg, t);                               // t - s
  const f2_t tz = f2_fma(z, neg, t);                              // t - z
  const f2_t e = f2_add(f2_fma(tz, neg, s), f2_fma(z, neg, p));  // (s - (t - z)) + (p - z)
  c = f2_add(c, e);
  s = t;
}

// NW warps per block share one staged source tile; a block covers
// 64 NW NP = 256 rows.  Warps whose rows all lie past the box skip the
// arithmetic, so a partial tile wastes at most 63 rows.
template <int OP, int NW, int NP>
__global__ void __launch_bounds__(NW * 32) k_translate_f32x2(TransArgs32 a) {
  constexpr int D = OpTraits<OP>::kDim;
  constexpr bool LOG = (OP == SKF_LAPLACE_2D);
  // 64-source tiles for the one-warp shape: 4 KB of staged sources per
  // block, so more blocks fit an SM
  constexpr int TS = (NW == 1 && NP == 1) ? 64 : kTileSrcF32;
  // a work item is a tile of 64 * NW * NP rows (256, or 64 for the 1 x 1 shape)
  static_assert(64 * NW * NP == 256 || (NW == 1 && NP == 1), "work items are 256- or 64-row tiles");
  __shared__ ulonglong2 s0[TS], s1[TS], s2[TS], s3[TS];

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int U = a.work_box[blockIdx.x];
  const int row0 = a.work_row[blockIdx.x];
  const int64_t offU = a.box_off[U];
  const int bsU = (int)(a.box_off[U + 1] - offU);
  const int rU = a.box_rank[U];
  const int wrow0 = row0 + 64 * NP * warp;  // first row of this warp
  const bool active = wrow0 < bsU;

  f2_t thx[NP], thy[NP], thz[NP], tlx[NP], tly[NP], tlz[NP];
#pragma unroll
  for (int p = 0; p < NP; ++p) {
    const int ra = wrow0 + lane + 64 * p, rb = ra + 32;
    const int64_t ea = offU + max(0, min(ra, bsU - 1)), eb = offU + max(0, min(rb, bsU - 1));
    const float4 ha = a.hi32[ea], hb = a.hi32[eb];
    const float4 la = a.lo32[ea], lb = a.lo32[eb];
    thx[p] = f2_pack(ha.x, hb.x);
    thy[p] = f2_pack(ha.y, hb.y);
    thz[p] = f2_pack(ha.z, hb.z);
    tlx[p] = f2_pack(la.x, lb.x);
    tly[p] = f2_pack(la.y, lb.y);
    tlz[p] = f2_pack(la.z, lb.z);
  }
  const bool need_h = wrow0 < rU;
  const f2_t zero = f2_pack(0.f, 0.f);
  f2_t su[NP], cu[NP], sh[NP], ch[NP];
#pragma unroll
  for (int p = 0; p < NP; ++p) su[p] = cu[p] = sh[p] = ch[p] = zero;

  const int64_t l0 = a.list_off[U], l1 = a.list_off[U + 1];
  for (int64_t l = l0; l < l1; ++l) {
    const int s = a.list_src[l];
    const int kind = a.list_kind[l];
    const int64_t offS = a.box_off[s];
    const int bsS = (int)(a.box_off[s + 1] - offS);
    const int rS = a.box_rank[s];
    const int nh = (kind == SKF_KIND_COLLEAGUE) ? rS : ((kind == SKF_KIND_COARSE_UP) ? bsS : 0);
    const bool self = (s == U);
    const float* c1src = (kind == SKF_KIND_COARSE_DOWN) ? a.qd32 : a.q32;
    for (int t0 = 0; t0 < bsS;) {
      const bool hseg = t0 < nh;
      const int nt = min(TS, (hseg ? nh : bsS) - t0);
      __syncthreads();
      for (int j = threadIdx.x; j < nt; j += NW * 32) {
        const int64_t e = offS + t0 + j;
        const float4 h = a.hi32[e], lo = a.lo32[e];
        const float c1 = c1src[e];
        float c2 = 0.f;
        if (kind == SKF_KIND_COLLEAGUE) c2 = a.qhn32[e];
        else if (kind == SKF_KIND_COARSE_UP) c2 = -c1;
        s0[j] = make_ulonglong2(f2_pack(-h.x, -h.x), f2_pack(-h.y, -h.y));
        s1[j] = make_ulonglong2(f2_pack(-h.z, -h.z), f2_pack(-lo.x, -lo.x));
        s2[j] = make_ulonglong2(f2_pack(-lo.y, -lo.y), f2_pack(-lo.z, -lo.z));
        s3[j] = make_ulonglong2(f2_pack(c1, c1), f2_pack(c2, c2));
      }
      __syncthreads();
      if (active) {
        f2_t pu[NP], ph[NP];
#pragma unroll
        for (int p = 0; p < NP; ++p) pu[p] = ph[p] = zero;
        const bool doh = need_h && hseg;
        if (doh) {
          if (self) x2_tile<D, NP, true, true, LOG>(s0, s1, s2, s3, nt, thx, thy, thz, tlx, tly, tlz, pu, ph);
          else x2_tile<D, NP, true, false, LOG>(s0, s1, s2, s3, nt, thx, thy, thz, tlx, tly, tlz, pu, ph);
        } else {
          if (self) x2_tile<D, NP, false, true, LOG>(s0, s1, s2, s3, nt, thx, thy, thz, tlx, tly, tlz, pu, ph);
          else x2_tile<D, NP, false, false, LOG>(s0, s1, s2, s3, nt, thx, thy, thz, tlx, tly, tlz, pu, ph);
        }
#pragma unroll
        for (int p = 0; p < NP; ++p) {
          f2_two_sum(su[p], cu[p], pu[p]);
          if (doh) f2_two_sum(sh[p], ch[p], ph[p]);
        }
      }
      t0 += nt;
    }
  }
  if (!active) return;
  // log r = (ln 2 / 2) log2(r^2): the constant is applied once to the sums
  const double scale = LOG ? 0.34657359027997264 : 1.0;
#pragma unroll
  for (int p = 0; p < NP; ++p) {
    float sua, sub, cua, cub, sha, shb, cha, chb;
    f2_unpack(su[p], sua, sub);
    f2_unpack(cu[p], cua, cub);
    f2_unpack(sh[p], sha, shb);
    f2_unpack(ch[p], cha, chb);
    const int ra = wrow0 + lane + 64 * p, rb = ra + 32;
    if (ra < bsU) {
      a.u[offU + ra] = scale * ((double)sua + (double)cua);
      a.uh[offU + ra] = ra < rU ? scale * ((double)sha + (double)cha) : 0.0;
    }
    if (rb < bsU) {
      a.u[offU + rb] = scale * ((double)sub + (double)cub);
      a.uh[offU + rb] = rb < rU ? scale * ((double)shb + (double)chb) : 0.0;
    }
  }
}

// ------------------------------------------------------------------ Helmholtz 3D, packed
// exp(i kappa r) / r with complex charges, two target rows per FP32x2
// instruction: differences, r^2, r, the phase in turns, its one-turn
// remainder, the scalings by 1/r and the four complex multiply-adds are
// packed; rsqrt, rint, sin and cos stay per lane.  Sources are staged
// pre-negated and duplicated, with the charges as (c1r, c1i), (-c1i, c2r),
// (c2i, -c2i).  Same arithmetic per evaluation as k_translate_f32 (hi/lo
// differences, one-turn phase reduction, compensated FP32 sums).
template <int NP, bool H, bool SELF>
__device__ __forceinline__ void hx2_tile(const ulonglong2* __restrict__ s0, const ulonglong2* __restrict__ s1,
                                         const ulonglong2* __restrict__ s2, const ulonglong2* __restrict__ s3,
                                         const ulonglong2* __restrict__ s4, const ulonglong2* __restrict__ s5, int nt,
                                         const f2_t (&thx)[NP], const f2_t (&thy)[NP], const f2_t (&thz)[NP],
                                         const f2_t (&tlx)[NP], const f2_t (&tly)[NP], const f2_t (&tlz)[NP],
                                         f2_t kc2, f2_t (&pur)[NP], f2_t (&pui)[NP], f2_t (&phr)[NP],
                                         f2_t (&phi)[NP]) {
  const f2_t two_pi = f2_pack(6.283185307179586f, 6.283185307179586f);
#pragma unroll 4
  for (int j = 0; j < nt; ++j) {
    const ulonglong2 A = s0[j];   // (-hx), (-hy)
    const ulonglong2 B = s1[j];   // (-hz), (-lx)
    const ulonglong2 Cc = s2[j];  // (-ly), (-lz)
    const ulonglong2 Q1 = s3[j];  // c1r, c1i
    const ulonglong2 Q2 = s4[j];  // -c1i, c2r
    const ulonglong2 Q3 = s5[j];  // c2i, -c2i
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      const f2_t dx = f2_add(f2_add(thx[p], A.x), f2_add(tlx[p], B.y));
      const f2_t dy = f2_add(f2_add(thy[p], A.y), f2_add(tly[p], Cc.x));
      const f2_t dz = f2_add(f2_add(thz[p], B.x), f2_add(tlz[p], Cc.y));
      f2_t r2 = f2_mul(dx, dx);
      r2 = f2_fma(dy, dy, r2);
      r2 = f2_fma(dz, dz, r2);
      float ra, rb;
      f2_unpack(r2, ra, rb);
      float ia = rsqrt_approx(ra), ib = rsqrt_approx(rb);
      if (SELF) {
        ia = ra > 0.f ? ia : 0.f;
        ib = rb > 0.f ? ib : 0.f;
      }
      const f2_t ir = f2_pack(ia, ib);
      const f2_t t = f2_mul(f2_mul(r2, ir), kc2);  // phase in turns: kappa r / (2 pi)
      float ta, tb;
      f2_unpack(t, ta, tb);
      const f2_t ang = f2_mul(f2_add(t, f2_pack(-rintf(ta), -rintf(tb))), two_pi);
      float aa, ab;
      f2_unpack(ang, aa, ab);
      float sa, ca, sb, cb;
      asm("sin.approx.ftz.f32 %0, %1;" : "=f"(sa) : "f"(aa));
      asm("cos.approx.ftz.f32 %0, %1;" : "=f"(ca) : "f"(aa));
      asm("sin.approx.ftz.f32 %0, %1;" : "=f"(sb) : "f"(ab));
      asm("cos.approx.ftz.f32 %0, %1;" : "=f"(cb) : "f"(ab));
      const f2_t kr = f2_mul(f2_pack(ca, cb), ir);
      const f2_t ki = f2_mul(f2_pack(sa, sb), ir);
      pur[p] = f2_fma(ki, Q2.x, f2_fma(kr, Q1.x, pur[p]));
      pui[p] = f2_fma(ki, Q1.x, f2_fma(kr, Q1.y, pui[p]));
      if (H) {
        phr[p] = f2_fma(ki, Q3.y, f2_fma(kr, Q2.y, phr[p]));
        phi[p] = f2_fma(ki, Q2.y, f2_fma(kr, Q3.x, phi[p]));
      }
    }
  }
}

template <int NW, int NP>
__global__ void __launch_bounds__(NW * 32) k_translate_helm_x2(TransArgs32 a) {
  constexpr int TS = kTileSrcF32;
  // a work item is a tile of 64 * NW * NP rows (256, or 64 for the 1 x 1 shape)
  static_assert(64 * NW * NP == 256 || (NW == 1 && NP == 1), "work items are 256- or 64-row tiles");
  __shared__ ulonglong2 s0[TS], s1[TS], s2[TS], s3[TS], s4[TS], s5[TS];

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int U = a.work_box[blockIdx.x];
  const int row0 = a.work_row[blockIdx.x];
  const int64_t offU = a.box_off[U];
  const int bsU = (int)(a.box_off[U + 1] - offU);
  const int rU = a.box_rank[U];
  const int wrow0 = row0 + 64 * NP * warp;
  const bool active = wrow0 < bsU;
  const float kc = a.kappa * 0.15915494309189535f;
  const f2_t kc2 = f2_pack(kc, kc);

  f2_t thx[NP], thy[NP], thz[NP], tlx[NP], tly[NP], tlz[NP];
#pragma unroll
  for (int p = 0; p < NP; ++p) {
    const int ra = wrow0 + lane + 64 * p, rb = ra + 32;
    const int64_t ea = offU + max(0, min(ra, bsU - 1)), eb = offU + max(0, min(rb, bsU - 1));
    const float4 ha = a.hi32[ea], hb = a.hi32[eb];
    const float4 la = a.lo32[ea], lb = a.lo32[eb];
    thx[p] = f2_pack(ha.x, hb.x);
    thy[p] = f2_pack(ha.y, hb.y);
    thz[p] = f2_pack(ha.z, hb.z);
    tlx[p] = f2_pack(la.x, lb.x);
    tly[p] = f2_pack(la.y, lb.y);
    tlz[p] = f2_pack(la.z, lb.z);
  }
  const bool need_h = wrow0 < rU;
  const f2_t zero = 0ull;
  f2_t sur[NP], cur[NP], sui[NP], cui[NP], shr[NP], chr[NP], shi[NP], chi[NP];
#pragma unroll
  for (int p = 0; p < NP; ++p) sur[p] = cur[p] = sui[p] = cui[p] = shr[p] = chr[p] = shi[p] = chi[p] = zero;

  const int64_t l0 = a.list_off[U], l1 = a.list_off[U + 1];
  for (int64_t l = l0; l < l1; ++l) {
    const int s = a.list_src[l];
    const int kind = a.list_kind[l];
    const int64_t offS = a.box_off[s];
    const int bsS = (int)(a.box_off[s + 1] - offS);
    const int rS = a.box_rank[s];
    const int nh = (kind == SKF_KIND_COLLEAGUE) ? rS : ((kind == SKF_KIND_COARSE_UP) ? bsS : 0);
    const bool self = (s == U);
    const float* c1src = (kind == SKF_KIND_COARSE_DOWN) ? a.qd32 : a.q32;
    for (int t0 = 0; t0 < bsS;) {
      const bool hseg = t0 < nh;
      const int nt = min(TS, (hseg ? nh : bsS) - t0);
      __syncthreads();
      for (int j = threadIdx.x; j < nt; j += NW * 32) {
        const int64_t e = offS + t0 + j;
        const float4 h = a.hi32[e], lo = a.lo32[e];
        const float c1r = c1src[2 * e], c1i = c1src[2 * e + 1];
        float c2r = 0.f, c2i = 0.f;
        if (kind == SKF_KIND_COLLEAGUE) {
          c2r = a.qhn32[2 * e];
          c2i = a.qhn32[2 * e + 1];
        } else if (kind == SKF_KIND_COARSE_UP) {
          c2r = -c1r;
          c2i = -c1i;
        }
        s0[j] = make_ulonglong2(f2_pack(-h.x, -h.x), f2_pack(-h.y, -h.y));
        s1[j] = make_ulonglong2(f2_pack(-h.z, -h.z), f2_pack(-lo.x, -lo.x));
        s2[j] = make_ulonglong2(f2_pack(-lo.y, -lo.y), f2_pack(-lo.z, -lo.z));
        s3[j] = make_ulonglong2(f2_pack(c1r, c1r), f2_pack(c1i, c1i));
        s4[j] = make_ulonglong2(f2_pack(-c1i, -c1i), f2_pack(c2r, c2r));
        s5[j] = make_ulonglong2(f2_pack(c2i, c2i), f2_pack(-c2i, -c2i));
      }
      __syncthreads();
      if (active) {
        f2_t pur[NP], pui[NP], phr[NP], phi[NP];
#pragma unroll
        for (int p = 0; p < NP; ++p) pur[p] = pui[p] = phr[p] = phi[p] = zero;
        const bool doh = need_h && hseg;
        if (doh) {
          if (self) hx2_tile<NP, true, true>(s0, s1, s2, s3, s4, s5, nt, thx, thy, thz, tlx, tly, tlz, kc2, pur, pui, phr, phi);
          else hx2_tile<NP, true, false>(s0, s1, s2, s3, s4, s5, nt, thx, thy, thz, tlx, tly, tlz, kc2, pur, pui, phr, phi);
        } else {
          if (self) hx2_tile<NP, false, true>(s0, s1, s2, s3, s4, s5, nt, thx, thy, thz, tlx, tly, tlz, kc2, pur, pui, phr, phi);
          else hx2_tile<NP, false, false>(s0, s1, s2, s3, s4, s5, nt, thx, thy, thz, tlx, tly, tlz, kc2, pur, pui, phr, phi);
        }
#pragma unroll
        for (int p = 0; p < NP; ++p) {
          f2_two_sum(sur[p], cur[p], pur[p]);
          f2_two_sum(sui[p], cui[p], pui[p]);
          if (doh) {
            f2_two_sum(shr[p], chr[p], phr[p]);
            f2_two_sum(shi[p], chi[p], phi[p]);
          }
        }
      }
      t0 += nt;
    }
  }
  if (!active) return;
#pragma unroll
  for (int p = 0; p < NP; ++p) {
    float a0, b0, a1, b1;
    const int ra = wrow0 + lane + 64 * p, rb = ra + 32;
    double ur[2], ui[2], hr[2], hi[2];
    f2_unpack(sur[p], a0, b0);
    f2_unpack(cur[p], a1, b1);
    ur[0] = (double)a0 + (double)a1;
    ur[1] = (double)b0 + (double)b1;
    f2_unpack(sui[p], a0, b0);
    f2_unpack(cui[p], a1, b1);
    ui[0] = (double)a0 + (double)a1;
    ui[1] = (double)b0 + (double)b1;
    f2_unpack(shr[p], a0, b0);
    f2_unpack(chr[p], a1, b1);
    hr[0] = (double)a0 + (double)a1;
    hr[1] = (double)b0 + (double)b1;
    f2_unpack(shi[p], a0, b0);
    f2_unpack(chi[p], a1, b1);
    hi[0] = (double)a0 + (double)a1;
    hi[1] = (double)b0 + (double)b1;
    const int rows[2] = {ra, rb};
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int row = rows[q];
      if (row >= bsU) continue;
      const int64_t e = offU + row;
      const bool sk = row < rU;
      a.u[2 * e] = ur[q];
      a.u[2 * e + 1] = ui[q];
      a.uh[2 * e] = sk ? hr[q] : 0.0;
      a.uh[2 * e + 1] = sk ? hi[q] : 0.0;
    }
  }
}

}  // namespace skf

namespace skf {

// ------------------------------------------------------------------ symmetric (mixed, packed)
// Symmetric point kernels (K(x,y) = K(y,x)) and symmetric lists: every
// translation (A <- B, kind k) has a mirror (B <- A, mirror kind:
// colleague <-> colleague, coarse-up <-> coarse-down, root <-> root) that uses
// the same kernel block transposed.  Box A owns its pairs with B > A: one
// evaluation of K(X_A, X_B) feeds both
//   rows of A:    u_A[i] += sum_j K_ij c1_j(k),   uh_A[i] += sum_j K_ij c2_j(k)
//   rows of B:    u_B[j] += sum_i K_ij c1_i(k'),  uh_B[j] += sum_i K_ij c2_i(k')
// The B-side sums of one work item (its 256 rows of A) go to a partial buffer
// (fixed slot per item, list entry and source), and k_sym_reduce adds them in
// a fixed order: deterministic, no atomics.  Self pairs are evaluated once as
// before.
//
// Lane layout per warp (64 rows of A): lane = 16 ls + lr; lane (lr, ls) owns
// rows wrow0 + lr + 16k (k < 4, packed in pairs (0,1), (2,3)) and the
// sources j = t0 + ls + 2g of each tile.  Row sums are combined across the 2
// ls lanes at the end; a source's B-side sums (one per lane, over its 4
// rows) go to a padded shared tile and are added over the 16 lr lanes and
// the 4 warps after the tile.
struct SymArgs {
  const int32_t* work_box;
  const int32_t* work_row;
  const int64_t* box_off;
  const int32_t* box_rank;
  const int64_t* list_off;   // symmetric lists: self + owned entries
  const int32_t* list_src;
  const int8_t* list_kind;
  const int64_t* list_poff;  // offset of the entry's partial block within a tile region
  const int64_t* box_pbase;  // first partial of the box's tile regions
  const int64_t* box_pstride;  // partials per tile region of the box
  const float4* hi32;
  const float4* lo32;
  const float* q32;
  const float* qhn32;
  const float* qd32;
  float* pbuf;
  double* u;
  double* uh;
  // source-split items (k_translate_symw only)
  const int32_t* work_part;
  const int32_t* box_ntiles;
  const int32_t* box_nparts;
  const int64_t* box_apart;
};

constexpr int kSymPairs = 2;  // packed row pairs per lane (4 rows)
// Sources per shared-memory tile (TS, a multiple of 32) and the row stride of
// the B-side partial tile, TS + 2 = 2 (mod 32): the lanes (lr, ls) of a warp
// write 32 distinct banks.
__host__ __device__ constexpr int sym_ld(int ts) { return ts + 2; }
__host__ __device__ constexpr size_t sym_smem_bytes(int ts) {
  return 4 * sizeof(ulonglong2) * (size_t)ts + 2 * 4 * 16 * sizeof(float) * (size_t)sym_ld(ts);
}

// One tile: lane (lr, ls) evaluates its 4 rows against sources j = 2g + ls.
// Row sums accumulate in registers; the lane's B-side sum for source j (its 4
// rows) goes to sTu[lr][j] / sTh[lr][j] and is reduced after the tile.
template <int D, bool HR, bool HT, bool TR, bool SELF, bool LOG, int LD>
__device__ __forceinline__ void sym_tile(const ulonglong2* __restrict__ s0, const ulonglong2* __restrict__ s1,
                                         const ulonglong2* __restrict__ s2, const ulonglong2* __restrict__ s3,
                                         int nt, int ls, int lr, const f2_t (&thx)[kSymPairs],
                                         const f2_t (&thy)[kSymPairs], const f2_t (&thz)[kSymPairs],
                                         const f2_t (&tlx)[kSymPairs], const f2_t (&tly)[kSymPairs],
                                         const f2_t (&tlz)[kSymPairs], const f2_t (&c1T)[kSymPairs],
                                         const f2_t (&c2T)[kSymPairs], f2_t (&pu)[kSymPairs],
                                         f2_t (&ph)[kSymPairs], float* __restrict__ sTu,
                                         float* __restrict__ sTh) {
#pragma unroll 4
  for (int j = ls; j < nt; j += 2) {
    const ulonglong2 A = s0[j];   // (-hx,-hx), (-hy,-hy)
    const ulonglong2 B = s1[j];   // (-hz,-hz), (-lx,-lx)
    const ulonglong2 Cc = s2[j];  // (-ly,-ly), (-lz,-lz)
    const ulonglong2 Q = s3[j];   // (c1,c1), (c2,c2)
    f2_t tu = 0ull, th = 0ull;
#pragma unroll
    for (int p = 0; p < kSymPairs; ++p) {
      const f2_t dx = f2_add(f2_add(thx[p], A.x), f2_add(tlx[p], B.y));
      const f2_t dy = f2_add(f2_add(thy[p], A.y), f2_add(tly[p], Cc.x));
      f2_t r2 = f2_mul(dx, dx);
      r2 = f2_fma(dy, dy, r2);
      if (D == 3) {
        const f2_t dz = f2_add(f2_add(thz[p], B.x), f2_add(tlz[p], Cc.y));
        r2 = f2_fma(dz, dz, r2);
      }
      float ra, rb;
      f2_unpack(r2, ra, rb);
      float ka = LOG ? lg2_approx(ra) : rsqrt_approx(ra);
      float kb = LOG ? lg2_approx(rb) : rsqrt_approx(rb);
      if (SELF) {
        ka = ra > 0.f ? ka : 0.f;
        kb = rb > 0.f ? kb : 0.f;
      }
      const f2_t k = f2_pack(ka, kb);
      pu[p] = f2_fma(k, Q.x, pu[p]);
      if (HR) ph[p] = f2_fma(k, Q.y, ph[p]);
      if (TR) {
        tu = p == 0 ? f2_mul(k, c1T[p]) : f2_fma(k, c1T[p], tu);
        if (HT) th = p == 0 ? f2_mul(k, c2T[p]) : f2_fma(k, c2T[p], th);
      }
    }
    if (TR) {
      float a, b;
      f2_unpack(tu, a, b);
      sTu[lr * LD + j] = a + b;
      if (HT) {
        f2_unpack(th, a, b);
        sTh[lr * LD + j] = a + b;
      }
    }
  }
}

template <int OP, int TS, int MINB>
__global__ void __launch_bounds__(128, MINB) k_translate_sym(SymArgs a) {
  constexpr int D = OpTraits<OP>::kDim;
  constexpr bool LOG = (OP == SKF_LAPLACE_2D);
  constexpr int NW = 4;
  constexpr int LD = sym_ld(TS);
  extern __shared__ __align__(16) unsigned char sym_sm[];
  ulonglong2* s0 = reinterpret_cast<ulonglong2*>(sym_sm);
  ulonglong2* s1 = s0 + TS;
  ulonglong2* s2 = s1 + TS;
  ulonglong2* s3 = s2 + TS;
  float* sTu = reinterpret_cast<float*>(s3 + TS);  // [NW][16][LD]
  float* sTh = sTu + NW * 16 * LD;

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int lr = lane & 15, ls = lane >> 4;
  const int U = a.work_box[blockIdx.x];
  const int row0 = a.work_row[blockIdx.x];
  const int64_t offU = a.box_off[U];
  const int bsU = (int)(a.box_off[U + 1] - offU);
  const int rU = a.box_rank[U];
  const int wrow0 = row0 + 64 * warp;
  const bool active = wrow0 < bsU;
  const int64_t pbase = a.box_pbase[U] + (int64_t)(row0 / 256) * a.box_pstride[U];

  // rows of this lane: wrow0 + lr + 16 k, k < 4, packed pairs (0,1), (2,3)
  f2_t thx[kSymPairs], thy[kSymPairs], thz[kSymPairs], tlx[kSymPairs], tly[kSymPairs], tlz[kSymPairs];
#pragma unroll
  for (int p = 0; p < kSymPairs; ++p) {
    const int ra = wrow0 + lr + 32 * p, rb = ra + 16;
    const int64_t ea = offU + max(0, min(ra, bsU - 1)), eb = offU + max(0, min(rb, bsU - 1));
    const float4 ha = a.hi32[ea], hb = a.hi32[eb];
    const float4 la = a.lo32[ea], lb = a.lo32[eb];
    thx[p] = f2_pack(ha.x, hb.x);
    thy[p] = f2_pack(ha.y, hb.y);
    thz[p] = f2_pack(ha.z, hb.z);
    tlx[p] = f2_pack(la.x, lb.x);
    tly[p] = f2_pack(la.y, lb.y);
    tlz[p] = f2_pack(la.z, lb.z);
  }
  const bool skel_rows = wrow0 < rU;
  const f2_t zero = 0ull;
  f2_t su[kSymPairs], cu[kSymPairs], sh[kSymPairs], ch[kSymPairs];
#pragma unroll
  for (int p = 0; p < kSymPairs; ++p) su[p] = cu[p] = sh[p] = ch[p] = zero;

  const int64_t l0 = a.list_off[U], l1 = a.list_off[U + 1];
  for (int64_t l = l0; l < l1; ++l) {
    const int s = a.list_src[l];
    const int kind = a.list_kind[l];
    const int64_t offS = a.box_off[s];
    const int bsS = (int)(a.box_off[s + 1] - offS);
    const int rS = a.box_rank[s];
    const bool self = (s == U);
    const int nh = (kind == SKF_KIND_COLLEAGUE || kind == SKF_KIND_COARSE_DOWN)
                       ? rS
                       : ((kind == SKF_KIND_COARSE_UP) ? bsS : 0);
    const float* c1src = (kind == SKF_KIND_COARSE_DOWN) ? a.qd32 : a.q32;
    // charges of A's rows seen from B (mirror kind), for the B-side sums
    f2_t c1T[kSymPairs], c2T[kSymPairs];
#pragma unroll
    for (int p = 0; p < kSymPairs; ++p) c1T[p] = c2T[p] = zero;
    if (!self) {
      const float* t1 = (kind == SKF_KIND_COARSE_UP) ? a.qd32 : a.q32;
#pragma unroll
      for (int p = 0; p < kSymPairs; ++p) {
        const int ra = wrow0 + lr + 32 * p, rb = ra + 16;
        const float ca = ra < bsU ? t1[offU + ra] : 0.f, cb = rb < bsU ? t1[offU + rb] : 0.f;
        c1T[p] = f2_pack(ca, cb);
        float da = 0.f, db = 0.f;
        if (kind == SKF_KIND_COLLEAGUE) {
          da = ra < bsU ? a.qhn32[offU + ra] : 0.f;
          db = rb < bsU ? a.qhn32[offU + rb] : 0.f;
        } else if (kind == SKF_KIND_COARSE_DOWN) {
          da = -ca;
          db = -cb;
        }
        c2T[p] = f2_pack(da, db);
      }
    }
    const bool row_h_kind = kind == SKF_KIND_COLLEAGUE || kind == SKF_KIND_COARSE_UP;
    const bool t_h_kind = kind == SKF_KIND_COLLEAGUE ? skel_rows : kind == SKF_KIND_COARSE_DOWN;
    const int64_t pblk = self ? 0 : pbase + a.list_poff[l];
    for (int t0 = 0; t0 < bsS;) {
      const bool hseg = t0 < nh;
      const int nt = min(TS, (hseg ? nh : bsS) - t0);
      __syncthreads();
      for (int j = threadIdx.x; j < nt; j += NW * 32) {
        const int64_t e = offS + t0 + j;
        const float4 h = a.hi32[e], lo = a.lo32[e];
        const float c1 = c1src[e];
        float c2 = 0.f;
        if (kind == SKF_KIND_COLLEAGUE) c2 = a.qhn32[e];
        else if (kind == SKF_KIND_COARSE_UP) c2 = -c1;
        s0[j] = make_ulonglong2(f2_pack(-h.x, -h.x), f2_pack(-h.y, -h.y));
        s1[j] = make_ulonglong2(f2_pack(-h.z, -h.z), f2_pack(-lo.x, -lo.x));
        s2[j] = make_ulonglong2(f2_pack(-lo.y, -lo.y), f2_pack(-lo.z, -lo.z));
        s3[j] = make_ulonglong2(f2_pack(c1, c1), f2_pack(c2, c2));
      }
      __syncthreads();
      const bool hr = active && hseg && row_h_kind && skel_rows;
      const bool ht = active && hseg && t_h_kind;
      f2_t pu[kSymPairs], ph[kSymPairs];
#pragma unroll
      for (int p = 0; p < kSymPairs; ++p) pu[p] = ph[p] = zero;
      float* tu = sTu + warp * 16 * LD;
      float* thp = sTh + warp * 16 * LD;
      if (active) {
        if (self) {
          if (hr) sym_tile<D, true, false, false, true, LOG, LD>(s0, s1, s2, s3, nt, ls, lr, thx, thy, thz, tlx, tly, tlz, c1T, c2T, pu, ph, tu, thp);
          else sym_tile<D, false, false, false, true, LOG, LD>(s0, s1, s2, s3, nt, ls, lr, thx, thy, thz, tlx, tly, tlz, c1T, c2T, pu, ph, tu, thp);
        } else if (hr) {
          if (ht) sym_tile<D, true, true, true, false, LOG, LD>(s0, s1, s2, s3, nt, ls, lr, thx, thy, thz, tlx, tly, tlz, c1T, c2T, pu, ph, tu, thp);
          else sym_tile<D, true, false, true, false, LOG, LD>(s0, s1, s2, s3, nt, ls, lr, thx, thy, thz, tlx, tly, tlz, c1T, c2T, pu, ph, tu, thp);
        } else {
          if (ht) sym_tile<D, false, true, true, false, LOG, LD>(s0, s1, s2, s3, nt, ls, lr, thx, thy, thz, tlx, tly, tlz, c1T, c2T, pu, ph, tu, thp);
          else sym_tile<D, false, false, true, false, LOG, LD>(s0, s1, s2, s3, nt, ls, lr, thx, thy, thz, tlx, tly, tlz, c1T, c2T, pu, ph, tu, thp);
        }
#pragma unroll
        for (int p = 0; p < kSymPairs; ++p) {
          f2_two_sum(su[p], cu[p], pu[p]);
          if (hr) f2_two_sum(sh[p], ch[p], ph[p]);
        }
      }
      if (!self) {
        // warps without rows, or without a B-side uh sum, contribute zeros
        if (!active || !ht) {
          for (int k = lane; k < 16 * TS; k += 32) {
            const int rr = k / TS, jj = k - rr * TS;
            if (jj < nt) {
              if (!active) tu[rr * LD + jj] = 0.f;
              thp[rr * LD + jj] = 0.f;
            }
          }
        }
        __syncthreads();
        // index i < TS: u partials of source j = i, TS <= i < 2 TS: the uh
        // partials of source i - TS; 4 warps x 16 lanes each, consecutive j
        // per thread
        for (int i = threadIdx.x; i < 2 * TS; i += NW * 32) {
          const int j = i & (TS - 1);
          const bool hpart = i >= TS;
          if (j < nt) {
            const float* src = hpart ? sTh : sTu;
            float v0 = 0.f, v1 = 0.f, v2 = 0.f, v3 = 0.f;
#pragma unroll
            for (int r = 0; r < 16; ++r) {
              v0 += src[(0 * 16 + r) * LD + j];
              v1 += src[(1 * 16 + r) * LD + j];
              v2 += src[(2 * 16 + r) * LD + j];
              v3 += src[(3 * 16 + r) * LD + j];
            }
            a.pbuf[pblk + (hpart ? bsS : 0) + t0 + j] = (v0 + v1) + (v2 + v3);
          }
        }
      }
      t0 += nt;
    }
  }
  // combine the row sums of the 2 lanes sharing rows (ls = 0, 1), in FP64
#pragma unroll
  for (int p = 0; p < kSymPairs; ++p) {
    float sua, sub, cua, cub, sha, shb, cha, chb;
    f2_unpack(su[p], sua, sub);
    f2_unpack(cu[p], cua, cub);
    f2_unpack(sh[p], sha, shb);
    f2_unpack(ch[p], cha, chb);
    double v[4] = {(double)sua + (double)cua, (double)sub + (double)cub, (double)sha + (double)cha,
                   (double)shb + (double)chb};
#pragma unroll
    for (int q = 0; q < 4; ++q) v[q] += __shfl_xor_sync(0xffffffffu, v[q], 16);
    if (active && ls == 0) {
      const double scale = LOG ? 0.34657359027997264 : 1.0;
      const int ra = wrow0 + lr + 32 * p, rb = ra + 16;
      if (ra < bsU) {
        a.u[offU + ra] = scale * v[0];
        a.uh[offU + ra] = ra < rU ? scale * v[2] : 0.0;
      }
      if (rb < bsU) {
        a.u[offU + rb] = scale * v[1];
        a.uh[offU + rb] = rb < rU ? scale * v[3] : 0.0;
      }
    }
  }
}

// ------------------------------------------------------------------ symmetric, warps split the sources
// Same arithmetic and partial-buffer layout as k_translate_sym, organised so
// that the source tiles need no thread-block barrier.  A block owns one part
// of a 256-row work item: its share of the item's source tiles (32 sources,
// numbered across the list entries; boxes with long lists split them into
// box_nparts contiguous parts).  Each warp holds all 256 rows (8 per lane:
// rows row0 + lane + 32 k, k < 8, packed in pairs (2p, 2p + 1)) and takes
// every fourth tile of the part.  A warp stages its own tiles in a private,
// double-buffered shared-memory area (the next tile is loaded into registers
// while the current one is evaluated), so the B-side sums of a tile cover all
// 256 rows inside one warp: lane l writes its sum for source j (over its 8
// rows) to sT[j][l] (row stride 33: no bank conflicts either way) and, after
// a warp barrier, lane j adds up row j and writes the tile's partial (uh
// partials only where the tile carries uh sums; the others stay zero).  The
// warps' row sums (compensated FP32 pairs) are added in FP64 in warp order
// after one block barrier at the end; the first part writes u / uh, the
// others float-float partials that k_sym_reduce adds: deterministic, no
// atomics.
constexpr int kSymwPairs = 4;   // packed row pairs per lane (8 rows)
constexpr int kSymwWarps = 4;   // warps per block, splitting the part's source tiles
__host__ __device__ constexpr int symw_ts() { return 32; }
__host__ __device__ constexpr size_t symw_warp_bytes(int ts) {
  return 2 * 4 * sizeof(ulonglong2) * (size_t)ts + 2 * sizeof(float) * (size_t)ts * 33;
}
__host__ __device__ constexpr size_t symw_smem_bytes() {
  // per-warp tiles; the final row-sum exchange (warps x 256 rows x 4 floats) reuses them
  return kSymwWarps * symw_warp_bytes(symw_ts()) > (size_t)kSymwWarps * 256 * 4 * sizeof(float)
             ? kSymwWarps * symw_warp_bytes(symw_ts())
             : (size_t)kSymwWarps * 256 * 4 * sizeof(float);
}

// NPA: packed row pairs that hold rows of the item (items shorter than 256
// rows skip the pairs past their last row)
template <int D, bool HR, bool HT, bool TR, bool SELF, bool LOG, int NPA>
__device__ __forceinline__ void symw_tile(const ulonglong2* __restrict__ sb, int nt, int lane,
                                          const f2_t (&thx)[kSymwPairs], const f2_t (&thy)[kSymwPairs],
                                          const f2_t (&thz)[kSymwPairs], const f2_t (&tlx)[kSymwPairs],
                                          const f2_t (&tly)[kSymwPairs], const f2_t (&tlz)[kSymwPairs],
                                          const f2_t (&c1T)[kSymwPairs], const f2_t (&c2T)[kSymwPairs],
                                          f2_t (&pu)[kSymwPairs], f2_t (&ph)[kSymwPairs], float* __restrict__ sTu,
                                          float* __restrict__ sTh) {
#pragma unroll 4
  for (int j = 0; j < nt; ++j) {
    const ulonglong2 A = sb[j];                     // (-hx,-hx), (-hy,-hy)
    const ulonglong2 B = sb[symw_ts() + j];         // (-hz,-hz), (-lx,-lx)
    const ulonglong2 Cc = sb[2 * symw_ts() + j];    // (-ly,-ly), (-lz,-lz)
    const ulonglong2 Q = sb[3 * symw_ts() + j];     // (c1,c1), (c2,c2)
    f2_t tu = 0ull, th = 0ull;
#pragma unroll
    for (int p = 0; p < NPA; ++p) {
      const f2_t dx = f2_add(f2_add(thx[p], A.x), f2_add(tlx[p], B.y));
      const f2_t dy = f2_add(f2_add(thy[p], A.y), f2_add(tly[p], Cc.x));
      f2_t r2 = f2_mul(dx, dx);
      r2 = f2_fma(dy, dy, r2);
      if (D == 3) {
        const f2_t dz = f2_add(f2_add(thz[p], B.x), f2_add(tlz[p], Cc.y));
        r2 = f2_fma(dz, dz, r2);
      }
      float ra, rb;
      f2_unpack(r2, ra, rb);
      float ka = LOG ? lg2_approx(ra) : rsqrt_approx(ra);
      float kb = LOG ? lg2_approx(rb) : rsqrt_approx(rb);
      if (SELF) {
        ka = ra > 0.f ? ka : 0.f;
        kb = rb > 0.f ? kb : 0.f;
      }
      const f2_t k = f2_pack(ka, kb);
      pu[p] = f2_fma(k, Q.x, pu[p]);
      if (HR) ph[p] = f2_fma(k, Q.y, ph[p]);
      if (TR) {
        tu = p == 0 ? f2_mul(k, c1T[p]) : f2_fma(k, c1T[p], tu);
        if (HT) th = p == 0 ? f2_mul(k, c2T[p]) : f2_fma(k, c2T[p], th);
      }
    }
    if (TR) {
      float a, b;
      f2_unpack(tu, a, b);
      sTu[j * 33 + lane] = a + b;
      if (HT) {
        f2_unpack(th, a, b);
        sTh[j * 33 + lane] = a + b;
      }
    }
  }
}

template <int OP>
__device__ __forceinline__ void symw_item(const SymArgs& a, int item) {
  constexpr int D = OpTraits<OP>::kDim;
  constexpr bool LOG = (OP == SKF_LAPLACE_2D);
  constexpr int TS = symw_ts();
  constexpr int NP = kSymwPairs;
  constexpr int NW = kSymwWarps;
  extern __shared__ __align__(16) unsigned char symw_sm[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned char* wsm = symw_sm + (size_t)warp * symw_warp_bytes(TS);
  ulonglong2* sbuf = reinterpret_cast<ulonglong2*>(wsm);  // [2][TS][4]
  float* sTu = reinterpret_cast<float*>(sbuf + 2 * 4 * TS);  // [TS][33]
  float* sTh = sTu + TS * 33;

  const int U = a.work_box[item];
  const int row0 = a.work_row[item];
  const int part = a.work_part[item];
  const int64_t offU = a.box_off[U];
  const int bsU = (int)(a.box_off[U + 1] - offU);
  const int rU = a.box_rank[U];
  const int64_t pbase = a.box_pbase[U] + (int64_t)(row0 / 256) * a.box_pstride[U];
  // this part's tiles of the box's list: [g0, g1) in list order
  const int ntot = a.box_ntiles[U], nparts = a.box_nparts[U];
  const int g0 = (int)((int64_t)part * ntot / nparts), g1 = (int)((int64_t)(part + 1) * ntot / nparts);

  f2_t thx[NP], thy[NP], thz[NP], tlx[NP], tly[NP], tlz[NP];
#pragma unroll
  for (int p = 0; p < NP; ++p) {
    const int ra = row0 + lane + 64 * p, rb = ra + 32;
    const int64_t ea = offU + min(ra, bsU - 1), eb = offU + min(rb, bsU - 1);
    const float4 ha = a.hi32[ea], hb = a.hi32[eb];
    const float4 la = a.lo32[ea], lb = a.lo32[eb];
    thx[p] = f2_pack(ha.x, hb.x);
    thy[p] = f2_pack(ha.y, hb.y);
    thz[p] = f2_pack(ha.z, hb.z);
    tlx[p] = f2_pack(la.x, lb.x);
    tly[p] = f2_pack(la.y, lb.y);
    tlz[p] = f2_pack(la.z, lb.z);
  }
  const bool skel_rows = row0 < rU;
  // packed pairs holding rows of this item: pair p holds rows 64 p .. 64 p + 63
  const int nrows = min(256, bsU - row0);
  const int npa = nrows <= 64 ? 1 : (nrows <= 128 ? 2 : 4);
  const f2_t zero = 0ull;
  f2_t su[NP], cu[NP], sh[NP], ch[NP];
#pragma unroll
  for (int p = 0; p < NP; ++p) su[p] = cu[p] = sh[p] = ch[p] = zero;

  int gbase = 0;  // tiles of the earlier list entries (the warp of tile g is g % NW)
  const int64_t l0 = a.list_off[U], l1 = a.list_off[U + 1];
  for (int64_t l = l0; l < l1 && gbase < g1; ++l) {
    const int s = a.list_src[l];
    const int64_t offS = a.box_off[s];
    const int bsS = (int)(a.box_off[s + 1] - offS);
    if (bsS == 0) continue;
    const int kind = a.list_kind[l];
    const int rS = a.box_rank[s];
    const bool self = (s == U);
    const int nh = (kind == SKF_KIND_COLLEAGUE || kind == SKF_KIND_COARSE_DOWN)
                       ? rS
                       : ((kind == SKF_KIND_COARSE_UP) ? bsS : 0);
    // tiles: [0, nh) and [nh, bsS) in chunks of TS (sources past nh carry no
    // uh charge); the plan counts them the same way (box_ntiles)
    const int nth = (nh + TS - 1) / TS;
    const int ntiles = nth + (bsS - nh + TS - 1) / TS;
    // this warp's tiles of the entry: local k with gbase + k in [g0, g1), = warp (mod NW)
    const int kmin = max(0, g0 - gbase), kend = min(ntiles, g1 - gbase);
    int k = kmin + ((warp - (gbase + kmin)) % NW + NW) % NW;
    gbase += ntiles;
    if (k >= kend) continue;
    auto tile_t0 = [&](int kk) { return kk < nth ? kk * TS : nh + (kk - nth) * TS; };
    auto tile_len = [&](int kk) { return kk < nth ? min(TS, nh - kk * TS) : min(TS, bsS - tile_t0(kk)); };
    const float* c1src = (kind == SKF_KIND_COARSE_DOWN) ? a.qd32 : a.q32;
    // charges of this item's rows seen from the source box (mirror kind)
    f2_t c1T[NP], c2T[NP];
#pragma unroll
    for (int p = 0; p < NP; ++p) c1T[p] = c2T[p] = zero;
    if (!self) {
      const float* t1 = (kind == SKF_KIND_COARSE_UP) ? a.qd32 : a.q32;
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        const int ra = row0 + lane + 64 * p, rb = ra + 32;
        const float ca = ra < bsU ? t1[offU + ra] : 0.f, cb = rb < bsU ? t1[offU + rb] : 0.f;
        c1T[p] = f2_pack(ca, cb);
        float da = 0.f, db = 0.f;
        if (kind == SKF_KIND_COLLEAGUE) {
          da = ra < bsU ? a.qhn32[offU + ra] : 0.f;
          db = rb < bsU ? a.qhn32[offU + rb] : 0.f;
        } else if (kind == SKF_KIND_COARSE_DOWN) {
          da = -ca;
          db = -cb;
        }
        c2T[p] = f2_pack(da, db);
      }
    }
    const bool row_h_kind = kind == SKF_KIND_COLLEAGUE || kind == SKF_KIND_COARSE_UP;
    const bool t_h_kind = kind == SKF_KIND_COLLEAGUE ? skel_rows : kind == SKF_KIND_COARSE_DOWN;
    const bool hr_kind = row_h_kind && skel_rows;
    const int64_t pblk = self ? 0 : pbase + a.list_poff[l];
    // source j of tile kk, as loaded by lane j
    float4 nh4 = make_float4(0, 0, 0, 0), nl4 = nh4;
    float nc1 = 0.f, nc2 = 0.f;
    auto load_src = [&](int kk) {
      if (lane < tile_len(kk)) {
        const int64_t e = offS + tile_t0(kk) + lane;
        nh4 = a.hi32[e];
        nl4 = a.lo32[e];
        nc1 = c1src[e];
        nc2 = kind == SKF_KIND_COLLEAGUE ? a.qhn32[e] : (kind == SKF_KIND_COARSE_UP ? -nc1 : 0.f);
      }
    };
    auto store_src = [&](ulonglong2* dst) {  // planes [4][TS]
      dst[lane] = make_ulonglong2(f2_pack(-nh4.x, -nh4.x), f2_pack(-nh4.y, -nh4.y));
      dst[TS + lane] = make_ulonglong2(f2_pack(-nh4.z, -nh4.z), f2_pack(-nl4.x, -nl4.x));
      dst[2 * TS + lane] = make_ulonglong2(f2_pack(-nl4.y, -nl4.y), f2_pack(-nl4.z, -nl4.z));
      dst[3 * TS + lane] = make_ulonglong2(f2_pack(nc1, nc1), f2_pack(nc2, nc2));
    };
    int buf = 0;
    load_src(k);
    __syncwarp();
    store_src(sbuf);
    for (; k < kend; k += NW) {
      const int t0 = tile_t0(k);
      const int nt = tile_len(k);
      const bool hseg = k < nth;
      const bool more = k + NW < kend;
      if (more) load_src(k + NW);  // this warp's next tile, in flight during this one
      __syncwarp();
      const ulonglong2* sb = sbuf + buf * 4 * TS;
      const bool hr = hseg && hr_kind;
      const bool ht = hseg && t_h_kind;
      f2_t pu[NP], ph[NP];
#pragma unroll
      for (int p = 0; p < NP; ++p) pu[p] = ph[p] = zero;
      auto run = [&](auto npa_tag) {
        constexpr int NPA = decltype(npa_tag)::value;
        if (self) {
          if (hr) symw_tile<D, true, false, false, true, LOG, NPA>(sb, nt, lane, thx, thy, thz, tlx, tly, tlz, c1T, c2T, pu, ph, sTu, sTh);
          else symw_tile<D, false, false, false, true, LOG, NPA>(sb, nt, lane, thx, thy, thz, tlx, tly, tlz, c1T, c2T, pu, ph, sTu, sTh);
        } else if (hr) {
          if (ht) symw_tile<D, true, true, true, false, LOG, NPA>(sb, nt, lane, thx, thy, thz, tlx, tly, tlz, c1T, c2T, pu, ph, sTu, sTh);
          else symw_tile<D, true, false, true, false, LOG, NPA>(sb, nt, lane, thx, thy, thz, tlx, tly, tlz, c1T, c2T, pu, ph, sTu, sTh);
        } else {
          if (ht) symw_tile<D, false, true, true, false, LOG, NPA>(sb, nt, lane, thx, thy, thz, tlx, tly, tlz, c1T, c2T, pu, ph, sTu, sTh);
          else symw_tile<D, false, false, true, false, LOG, NPA>(sb, nt, lane, thx, thy, thz, tlx, tly, tlz, c1T, c2T, pu, ph, sTu, sTh);
        }
      };
      if (npa == 4) run(std::integral_constant<int, 4>());
      else if (npa == 2) run(std::integral_constant<int, 2>());
      else run(std::integral_constant<int, 1>());
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        f2_two_sum(su[p], cu[p], pu[p]);
        if (hr) f2_two_sum(sh[p], ch[p], ph[p]);
      }
      __syncwarp();
      if (!self && lane < nt) {
        // lane j: the tile's B-side sums of source j over the item's 256 rows
        float vu = 0.f, vh = 0.f;
#pragma unroll 8
        for (int r = 0; r < 32; ++r) vu += sTu[lane * 33 + r];
        if (ht) {
#pragma unroll 8
          for (int r = 0; r < 32; ++r) vh += sTh[lane * 33 + r];
        }
        a.pbuf[pblk + t0 + lane] = vu;
        // uh partials of tiles without uh charges stay at the zeros the
        // plan wrote when it allocated the buffer (the same slots every apply)
        if (ht) a.pbuf[pblk + bsS + t0 + lane] = vh;
      }
      if (more) store_src(sbuf + (buf ^ 1) * 4 * TS);
      __syncwarp();
      buf ^= 1;
    }
  }
  // row sums of the warps, added in FP64 in warp order
  __syncthreads();
  float* ex = reinterpret_cast<float*>(symw_sm);  // [NW][256][4]: su, cu, sh, ch
#pragma unroll
  for (int p = 0; p < NP; ++p) {
    float v[8];
    f2_unpack(su[p], v[0], v[4]);
    f2_unpack(cu[p], v[1], v[5]);
    f2_unpack(sh[p], v[2], v[6]);
    f2_unpack(ch[p], v[3], v[7]);
    const int ra = lane + 64 * p, rb = ra + 32;
    *reinterpret_cast<float4*>(ex + ((size_t)warp * 256 + ra) * 4) = make_float4(v[0], v[1], v[2], v[3]);
    *reinterpret_cast<float4*>(ex + ((size_t)warp * 256 + rb) * 4) = make_float4(v[4], v[5], v[6], v[7]);
  }
  __syncthreads();
  const double scale = LOG ? 0.34657359027997264 : 1.0;
  // the first part owns u / uh; later parts leave float-float partials
  // (hi region, then lo region) that k_sym_reduce adds in a fixed order
  float* apart = part > 0 ? a.pbuf + a.box_apart[U] + (int64_t)(part - 1) * 4 * bsU : nullptr;
  for (int r = threadIdx.x; r < 256; r += NW * 32) {
    const int row = row0 + r;
    if (row >= bsU) continue;
    double vu = 0.0, vh = 0.0;
#pragma unroll
    for (int w = 0; w < NW; ++w) {
      const float4 e = *reinterpret_cast<const float4*>(ex + ((size_t)w * 256 + r) * 4);
      vu += (double)e.x + (double)e.y;
      vh += (double)e.z + (double)e.w;
    }
    if (row >= rU) vh = 0.0;
    if (part == 0) {
      a.u[offU + row] = scale * vu;
      a.uh[offU + row] = scale * vh;
    } else {
      const float hu = (float)vu, hh = (float)vh;
      apart[row] = hu;
      apart[bsU + row] = hh;
      apart[2 * bsU + row] = (float)(vu - (double)hu);
      apart[3 * bsU + row] = (float)(vh - (double)hh);
    }
  }
}

// One block per item of the (costliest-first) item list.
template <int OP>
__global__ void __launch_bounds__(kSymwWarps * 32, 3) k_translate_symw(SymArgs a) {
  symw_item<OP>(a, blockIdx.x);
}

// Persistent form: one block per resident slot (3 per SM) takes items from
// a queue counter (zeroed before the launch) in list order until it is
// exhausted.  Which block takes an item changes from run to run; what an
// item writes (its rows, its partial slots) does not, so results are the
// same bit for bit.
template <int OP>
__global__ void __launch_bounds__(kSymwWarps * 32, 3) k_translate_symw_queue(SymArgs a, int nitems, int* queue) {
  __shared__ int s_item;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(queue, 1);
    __syncthreads();
    const int item = s_item;
    __syncthreads();  // all threads read s_item (and finished the last item) first
    if (item >= nitems) break;
    symw_item<OP>(a, item);
  }
}

// ------------------------------------------------------------------ symmetric Helmholtz 3D (mixed, packed)
// exp(i kappa r) / r is symmetric too: the owned pairs of the symmetric
// lists are evaluated once for both directions as in k_translate_sym, with
// the arithmetic of k_translate_helm_x2 per evaluation (hi/lo differences,
// one-turn phase reduction, sin/cos.approx) and complex charges and sums.
// Same lane layout (lane = 16 ls + lr, 4 rows per lane in 2 packed pairs),
// tiles and fixed-order B-side partials, with four partial arrays per
// source (u re, u im, uh re, uh im).
__host__ __device__ constexpr size_t symh_smem_bytes(int ts) {
  return 6 * sizeof(ulonglong2) * (size_t)ts + 4 * 4 * 16 * sizeof(float) * (size_t)sym_ld(ts);
}

// Charges of the A rows seen from B (mirror kind) for the B-side sums,
// packed per row pair: c1 = (r, i) and -i, c2 likewise.
struct SymhCharges {
  f2_t c1r[kSymPairs], c1i[kSymPairs], m1i[kSymPairs];
  f2_t c2r[kSymPairs], c2i[kSymPairs], m2i[kSymPairs];
};

template <bool HR, bool HT, bool TR, bool SELF, int LD>
__device__ __forceinline__ void symh_tile(const ulonglong2* __restrict__ s0, const ulonglong2* __restrict__ s1,
                                          const ulonglong2* __restrict__ s2, const ulonglong2* __restrict__ s3,
                                          const ulonglong2* __restrict__ s4, const ulonglong2* __restrict__ s5,
                                          int nt, int ls, int lr, const f2_t (&thx)[kSymPairs],
                                          const f2_t (&thy)[kSymPairs], const f2_t (&thz)[kSymPairs],
                                          const f2_t (&tlx)[kSymPairs], const f2_t (&tly)[kSymPairs],
                                          const f2_t (&tlz)[kSymPairs], f2_t kc2, const SymhCharges& cT,
                                          f2_t (&pur)[kSymPairs], f2_t (&pui)[kSymPairs], f2_t (&phr)[kSymPairs],
                                          f2_t (&phi)[kSymPairs], float* __restrict__ sT) {
  const f2_t two_pi = f2_pack(6.283185307179586f, 6.283185307179586f);
  constexpr int PS = 4 * 16 * LD;  // stride between the four partial arrays
#pragma unroll 2
  for (int j = ls; j < nt; j += 2) {
    const ulonglong2 A = s0[j];   // (-hx), (-hy)
    const ulonglong2 B = s1[j];   // (-hz), (-lx)
    const ulonglong2 Cc = s2[j];  // (-ly), (-lz)
    const ulonglong2 Q1 = s3[j];  // c1r, c1i
    const ulonglong2 Q2 = s4[j];  // -c1i, c2r
    const ulonglong2 Q3 = s5[j];  // c2i, -c2i
    f2_t tur = 0ull, tui = 0ull, thr = 0ull, thi = 0ull;
#pragma unroll
    for (int p = 0; p < kSymPairs; ++p) {
      const f2_t dx = f2_add(f2_add(thx[p], A.x), f2_add(tlx[p], B.y));
      const f2_t dy = f2_add(f2_add(thy[p], A.y), f2_add(tly[p], Cc.x));
      const f2_t dz = f2_add(f2_add(thz[p], B.x), f2_add(tlz[p], Cc.y));
      f2_t r2 = f2_mul(dx, dx);
      r2 = f2_fma(dy, dy, r2);
      r2 = f2_fma(dz, dz, r2);
      float ra, rb;
      f2_unpack(r2, ra, rb);
      float ia = rsqrt_approx(ra), ib = rsqrt_approx(rb);
      if (SELF) {
        ia = ra > 0.f ? ia : 0.f;
        ib = rb > 0.f ? ib : 0.f;
      }
      const f2_t ir = f2_pack(ia, ib);
      const f2_t t = f2_mul(f2_mul(r2, ir), kc2);  // phase in turns: kappa r / (2 pi)
      float ta, tb;
      f2_unpack(t, ta, tb);
      const f2_t ang = f2_mul(f2_add(t, f2_pack(-rintf(ta), -rintf(tb))), two_pi);
      float aa, ab;
      f2_unpack(ang, aa, ab);
      float sa, ca, sb, cb;
      asm("sin.approx.ftz.f32 %0, %1;" : "=f"(sa) : "f"(aa));
      asm("cos.approx.ftz.f32 %0, %1;" : "=f"(ca) : "f"(aa));
      asm("sin.approx.ftz.f32 %0, %1;" : "=f"(sb) : "f"(ab));
      asm("cos.approx.ftz.f32 %0, %1;" : "=f"(cb) : "f"(ab));
      const f2_t kr = f2_mul(f2_pack(ca, cb), ir);
      const f2_t ki = f2_mul(f2_pack(sa, sb), ir);
      pur[p] = f2_fma(ki, Q2.x, f2_fma(kr, Q1.x, pur[p]));
      pui[p] = f2_fma(ki, Q1.x, f2_fma(kr, Q1.y, pui[p]));
      if (HR) {
        phr[p] = f2_fma(ki, Q3.y, f2_fma(kr, Q2.y, phr[p]));
        phi[p] = f2_fma(ki, Q2.y, f2_fma(kr, Q3.x, phi[p]));
      }
      if (TR) {
        tur = f2_fma(ki, cT.m1i[p], f2_fma(kr, cT.c1r[p], tur));
        tui = f2_fma(ki, cT.c1r[p], f2_fma(kr, cT.c1i[p], tui));
        if (HT) {
          thr = f2_fma(ki, cT.m2i[p], f2_fma(kr, cT.c2r[p], thr));
          thi = f2_fma(ki, cT.c2r[p], f2_fma(kr, cT.c2i[p], thi));
        }
      }
    }
    if (TR) {
      float a, b;
      f2_unpack(tur, a, b);
      sT[lr * LD + j] = a + b;
      f2_unpack(tui, a, b);
      sT[PS + lr * LD + j] = a + b;
      if (HT) {
        f2_unpack(thr, a, b);
        sT[2 * PS + lr * LD + j] = a + b;
        f2_unpack(thi, a, b);
        sT[3 * PS + lr * LD + j] = a + b;
      }
    }
  }
}

template <int TS, int MINB>
__global__ void __launch_bounds__(128, MINB) k_translate_sym_helm(SymArgs a, float kappa) {
  constexpr int NW = 4;
  constexpr int LD = sym_ld(TS);
  constexpr int PS = NW * 16 * LD;
  extern __shared__ __align__(16) unsigned char symh_sm[];
  ulonglong2* s0 = reinterpret_cast<ulonglong2*>(symh_sm);
  ulonglong2* s1 = s0 + TS;
  ulonglong2* s2 = s1 + TS;
  ulonglong2* s3 = s2 + TS;
  ulonglong2* s4 = s3 + TS;
  ulonglong2* s5 = s4 + TS;
  float* sT = reinterpret_cast<float*>(s5 + TS);  // [4][NW][16][LD]

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int lr = lane & 15, ls = lane >> 4;
  const int U = a.work_box[blockIdx.x];
  const int row0 = a.work_row[blockIdx.x];
  const int64_t offU = a.box_off[U];
  const int bsU = (int)(a.box_off[U + 1] - offU);
  const int rU = a.box_rank[U];
  const int wrow0 = row0 + 64 * warp;
  const bool active = wrow0 < bsU;
  const int64_t pbase = a.box_pbase[U] + (int64_t)(row0 / 256) * a.box_pstride[U];
  const float kc = kappa * 0.15915494309189535f;
  const f2_t kc2 = f2_pack(kc, kc);

  f2_t thx[kSymPairs], thy[kSymPairs], thz[kSymPairs], tlx[kSymPairs], tly[kSymPairs], tlz[kSymPairs];
#pragma unroll
  for (int p = 0; p < kSymPairs; ++p) {
    const int ra = wrow0 + lr + 32 * p, rb = ra + 16;
    const int64_t ea = offU + max(0, min(ra, bsU - 1)), eb = offU + max(0, min(rb, bsU - 1));
    const float4 ha = a.hi32[ea], hb = a.hi32[eb];
    const float4 la = a.lo32[ea], lb = a.lo32[eb];
    thx[p] = f2_pack(ha.x, hb.x);
    thy[p] = f2_pack(ha.y, hb.y);
    thz[p] = f2_pack(ha.z, hb.z);
    tlx[p] = f2_pack(la.x, lb.x);
    tly[p] = f2_pack(la.y, lb.y);
    tlz[p] = f2_pack(la.z, lb.z);
  }
  const bool skel_rows = wrow0 < rU;
  const f2_t zero = 0ull;
  f2_t sur[kSymPairs], cur[kSymPairs], sui[kSymPairs], cui[kSymPairs];
  f2_t shr[kSymPairs], chr[kSymPairs], shi[kSymPairs], chi[kSymPairs];
#pragma unroll
  for (int p = 0; p < kSymPairs; ++p) sur[p] = cur[p] = sui[p] = cui[p] = shr[p] = chr[p] = shi[p] = chi[p] = zero;

  const int64_t l0 = a.list_off[U], l1 = a.list_off[U + 1];
  for (int64_t l = l0; l < l1; ++l) {
    const int s = a.list_src[l];
    const int kind = a.list_kind[l];
    const int64_t offS = a.box_off[s];
    const int bsS = (int)(a.box_off[s + 1] - offS);
    const int rS = a.box_rank[s];
    const bool self = (s == U);
    const int nh = (kind == SKF_KIND_COLLEAGUE || kind == SKF_KIND_COARSE_DOWN)
                       ? rS
                       : ((kind == SKF_KIND_COARSE_UP) ? bsS : 0);
    const float* c1src = (kind == SKF_KIND_COARSE_DOWN) ? a.qd32 : a.q32;
    // complex charges of A's rows seen from B (mirror kind), for the B-side sums
    SymhCharges cT;
#pragma unroll
    for (int p = 0; p < kSymPairs; ++p) cT.c1r[p] = cT.c1i[p] = cT.m1i[p] = cT.c2r[p] = cT.c2i[p] = cT.m2i[p] = zero;
    if (!self) {
      const float* t1 = (kind == SKF_KIND_COARSE_UP) ? a.qd32 : a.q32;
#pragma unroll
      for (int p = 0; p < kSymPairs; ++p) {
        const int ra = wrow0 + lr + 32 * p, rb = ra + 16;
        float ar = 0.f, ai = 0.f, br = 0.f, bi = 0.f;
        if (ra < bsU) {
          ar = t1[2 * (offU + ra)];
          ai = t1[2 * (offU + ra) + 1];
        }
        if (rb < bsU) {
          br = t1[2 * (offU + rb)];
          bi = t1[2 * (offU + rb) + 1];
        }
        cT.c1r[p] = f2_pack(ar, br);
        cT.c1i[p] = f2_pack(ai, bi);
        cT.m1i[p] = f2_pack(-ai, -bi);
        float dr = 0.f, di = 0.f, er = 0.f, ei = 0.f;
        if (kind == SKF_KIND_COLLEAGUE) {
          if (ra < bsU) {
            dr = a.qhn32[2 * (offU + ra)];
            di = a.qhn32[2 * (offU + ra) + 1];
          }
          if (rb < bsU) {
            er = a.qhn32[2 * (offU + rb)];
            ei = a.qhn32[2 * (offU + rb) + 1];
          }
        } else if (kind == SKF_KIND_COARSE_DOWN) {
          dr = -ar;
          di = -ai;
          er = -br;
          ei = -bi;
        }
        cT.c2r[p] = f2_pack(dr, er);
        cT.c2i[p] = f2_pack(di, ei);
        cT.m2i[p] = f2_pack(-di, -ei);
      }
    }
    const bool row_h_kind = kind == SKF_KIND_COLLEAGUE || kind == SKF_KIND_COARSE_UP;
    const bool t_h_kind = kind == SKF_KIND_COLLEAGUE ? skel_rows : kind == SKF_KIND_COARSE_DOWN;
    const int64_t pblk = self ? 0 : pbase + a.list_poff[l];
    for (int t0 = 0; t0 < bsS;) {
      const bool hseg = t0 < nh;
      const int nt = min(TS, (hseg ? nh : bsS) - t0);
      __syncthreads();
      for (int j = threadIdx.x; j < nt; j += NW * 32) {
        const int64_t e = offS + t0 + j;
        const float4 h = a.hi32[e], lo = a.lo32[e];
        const float c1r = c1src[2 * e], c1i = c1src[2 * e + 1];
        float c2r = 0.f, c2i = 0.f;
        if (kind == SKF_KIND_COLLEAGUE) {
          c2r = a.qhn32[2 * e];
          c2i = a.qhn32[2 * e + 1];
        } else if (kind == SKF_KIND_COARSE_UP) {
          c2r = -c1r;
          c2i = -c1i;
        }
        s0[j] = make_ulonglong2(f2_pack(-h.x, -h.x), f2_pack(-h.y, -h.y));
        s1[j] = make_ulonglong2(f2_pack(-h.z, -h.z), f2_pack(-lo.x, -lo.x));
        s2[j] = make_ulonglong2(f2_pack(-lo.y, -lo.y), f2_pack(-lo.z, -lo.z));
        s3[j] = make_ulonglong2(f2_pack(c1r, c1r), f2_pack(c1i, c1i));
        s4[j] = make_ulonglong2(f2_pack(-c1i, -c1i), f2_pack(c2r, c2r));
        s5[j] = make_ulonglong2(f2_pack(c2i, c2i), f2_pack(-c2i, -c2i));
      }
      __syncthreads();
      const bool hr = active && hseg && row_h_kind && skel_rows;
      const bool ht = active && hseg && t_h_kind;
      f2_t pur[kSymPairs], pui[kSymPairs], phr[kSymPairs], phi[kSymPairs];
#pragma unroll
      for (int p = 0; p < kSymPairs; ++p) pur[p] = pui[p] = phr[p] = phi[p] = zero;
      float* tw = sT + warp * 16 * LD;
      if (active) {
        if (self) {
          if (hr) symh_tile<true, false, false, true, LD>(s0, s1, s2, s3, s4, s5, nt, ls, lr, thx, thy, thz, tlx, tly, tlz, kc2, cT, pur, pui, phr, phi, tw);
          else symh_tile<false, false, false, true, LD>(s0, s1, s2, s3, s4, s5, nt, ls, lr, thx, thy, thz, tlx, tly, tlz, kc2, cT, pur, pui, phr, phi, tw);
        } else if (hr) {
          if (ht) symh_tile<true, true, true, false, LD>(s0, s1, s2, s3, s4, s5, nt, ls, lr, thx, thy, thz, tlx, tly, tlz, kc2, cT, pur, pui, phr, phi, tw);
          else symh_tile<true, false, true, false, LD>(s0, s1, s2, s3, s4, s5, nt, ls, lr, thx, thy, thz, tlx, tly, tlz, kc2, cT, pur, pui, phr, phi, tw);
        } else {
          if (ht) symh_tile<false, true, true, false, LD>(s0, s1, s2, s3, s4, s5, nt, ls, lr, thx, thy, thz, tlx, tly, tlz, kc2, cT, pur, pui, phr, phi, tw);
          else symh_tile<false, false, true, false, LD>(s0, s1, s2, s3, s4, s5, nt, ls, lr, thx, thy, thz, tlx, tly, tlz, kc2, cT, pur, pui, phr, phi, tw);
        }
#pragma unroll
        for (int p = 0; p < kSymPairs; ++p) {
          f2_two_sum(sur[p], cur[p], pur[p]);
          f2_two_sum(sui[p], cui[p], pui[p]);
          if (hr) {
            f2_two_sum(shr[p], chr[p], phr[p]);
            f2_two_sum(shi[p], chi[p], phi[p]);
          }
        }
      }
      if (!self) {
        // warps without rows, or without B-side uh sums, contribute zeros
        if (!active || !ht) {
          for (int k = lane; k < 16 * TS; k += 32) {
            const int rr = k / TS, jj = k - rr * TS;
            if (jj < nt) {
              if (!active) {
                tw[rr * LD + jj] = 0.f;
                tw[PS + rr * LD + jj] = 0.f;
              }
              tw[2 * PS + rr * LD + jj] = 0.f;
              tw[3 * PS + rr * LD + jj] = 0.f;
            }
          }
        }
        __syncthreads();
        // item i < 4 TS: partial array i / TS (u re, u im, uh re, uh im) of
        // source i % TS; 4 warps x 16 lanes each
        for (int i = threadIdx.x; i < 4 * TS; i += NW * 32) {
          const int part = i / TS, j = i - part * TS;
          if (j < nt) {
            const float* src = sT + part * PS;
            float v0 = 0.f, v1 = 0.f, v2 = 0.f, v3 = 0.f;
#pragma unroll
            for (int r = 0; r < 16; ++r) {
              v0 += src[(0 * 16 + r) * LD + j];
              v1 += src[(1 * 16 + r) * LD + j];
              v2 += src[(2 * 16 + r) * LD + j];
              v3 += src[(3 * 16 + r) * LD + j];
            }
            a.pbuf[pblk + (int64_t)part * bsS + t0 + j] = (v0 + v1) + (v2 + v3);
          }
        }
      }
      t0 += nt;
    }
  }
  // combine the row sums of the 2 lanes sharing rows (ls = 0, 1), in FP64
#pragma unroll
  for (int p = 0; p < kSymPairs; ++p) {
    double v[8];
    float x0, x1, y0, y1;
    f2_unpack(sur[p], x0, x1);
    f2_unpack(cur[p], y0, y1);
    v[0] = (double)x0 + (double)y0;
    v[1] = (double)x1 + (double)y1;
    f2_unpack(sui[p], x0, x1);
    f2_unpack(cui[p], y0, y1);
    v[2] = (double)x0 + (double)y0;
    v[3] = (double)x1 + (double)y1;
    f2_unpack(shr[p], x0, x1);
    f2_unpack(chr[p], y0, y1);
    v[4] = (double)x0 + (double)y0;
    v[5] = (double)x1 + (double)y1;
    f2_unpack(shi[p], x0, x1);
    f2_unpack(chi[p], y0, y1);
    v[6] = (double)x0 + (double)y0;
    v[7] = (double)x1 + (double)y1;
#pragma unroll
    for (int q = 0; q < 8; ++q) v[q] += __shfl_xor_sync(0xffffffffu, v[q], 16);
    if (active && ls == 0) {
      const int ra = wrow0 + lr + 32 * p, rb = ra + 16;
      if (ra < bsU) {
        const int64_t e = offU + ra;
        const bool sk = ra < rU;
        a.u[2 * e] = v[0];
        a.u[2 * e + 1] = v[2];
        a.uh[2 * e] = sk ? v[4] : 0.0;
        a.uh[2 * e + 1] = sk ? v[6] : 0.0;
      }
      if (rb < bsU) {
        const int64_t e = offU + rb;
        const bool sk = rb < rU;
        a.u[2 * e] = v[1];
        a.u[2 * e + 1] = v[3];
        a.uh[2 * e] = sk ? v[5] : 0.0;
        a.uh[2 * e + 1] = sk ? v[7] : 0.0;
      }
    }
  }
}

// Complex form of k_sym_reduce: a partial block holds u re, u im, uh re,
// uh im of the box's entries back to back.
__global__ void __launch_bounds__(256) k_sym_reduce_c(const int64_t* __restrict__ box_off,
                                                      const int32_t* __restrict__ box_rank,
                                                      const int64_t* __restrict__ in_off,
                                                      const int64_t* __restrict__ in_blk,
                                                      const float* __restrict__ pbuf, double* __restrict__ u,
                                                      double* __restrict__ uh) {
  const int B = blockIdx.x;
  const int64_t off = box_off[B];
  const int bs = (int)(box_off[B + 1] - off);
  const int j = blockIdx.y * blockDim.x + threadIdx.x;
  const int64_t k0 = in_off[B], k1 = in_off[B + 1];
  if (j >= bs || k0 == k1) return;
  const int r = box_rank[B];
  double ur[2] = {0.0, 0.0}, ui[2] = {0.0, 0.0}, hr[2] = {0.0, 0.0}, hi[2] = {0.0, 0.0};
  int64_t k = k0;
  for (; k + 1 < k1; k += 2) {
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int64_t b = in_blk[k + q];
      ur[q] += (double)pbuf[b + j];
      ui[q] += (double)pbuf[b + bs + j];
      hr[q] += (double)pbuf[b + 2 * bs + j];
      hi[q] += (double)pbuf[b + 3 * bs + j];
    }
  }
  if (k < k1) {
    const int64_t b = in_blk[k];
    ur[0] += (double)pbuf[b + j];
    ui[0] += (double)pbuf[b + bs + j];
    hr[0] += (double)pbuf[b + 2 * bs + j];
    hi[0] += (double)pbuf[b + 3 * bs + j];
  }
  u[2 * (off + j)] += ur[0] + ur[1];
  u[2 * (off + j) + 1] += ui[0] + ui[1];
  if (j < r) {
    uh[2 * (off + j)] += hr[0] + hr[1];
    uh[2 * (off + j) + 1] += hi[0] + hi[1];
  }
}

// Adds the B-side partial sums into u / uh in a fixed order.  Block i of the
// launch takes item (box, chunk) = (red_box[i], red_chunk[i]): entries
// [256 chunk, 256 chunk + 256) of a box that receives partials (the plan
// lists only those); uh partials are read only for skeleton entries.
template <bool LOG>
__global__ void __launch_bounds__(256) k_sym_reduce(const int32_t* __restrict__ red_box,
                                                    const int32_t* __restrict__ red_chunk,
                                                    const int64_t* __restrict__ box_off,
                                                    const int32_t* __restrict__ box_rank,
                                                    const int64_t* __restrict__ in_off,
                                                    const int64_t* __restrict__ in_blk,
                                                    const float* __restrict__ pbuf, double* __restrict__ u,
                                                    double* __restrict__ uh) {
  const int B = red_box[blockIdx.x];
  const int64_t off = box_off[B];
  const int bs = (int)(box_off[B + 1] - off);
  const int j = red_chunk[blockIdx.x] * blockDim.x + threadIdx.x;
  const int64_t k0 = in_off[B], k1 = in_off[B + 1];
  if (j >= bs || k0 == k1) return;
  const int r = box_rank[B];
  const bool skel = j < r;
  const double scale = LOG ? 0.34657359027997264 : 1.0;
  // four independent chains keep eight loads in flight per thread; the
  // grouping is fixed, so the sum is deterministic
  // four chains of compensated FP32 sums (TwoSum: value and rounding error,
  // ~2^-48 relative, as an FP64 sum; the FP32 pipes instead of the FP64 pipe)
  float su[4] = {0.f, 0.f, 0.f, 0.f}, cu[4] = {0.f, 0.f, 0.f, 0.f};
  float sh[4] = {0.f, 0.f, 0.f, 0.f}, ch[4] = {0.f, 0.f, 0.f, 0.f};
  int64_t k = k0;
  for (; k + 3 < k1; k += 4) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int64_t b = in_blk[k + q];
      two_sum_add(su[q], cu[q], pbuf[b + j]);
      if (skel) two_sum_add(sh[q], ch[q], pbuf[b + bs + j]);
    }
  }
  for (int q = 0; k < k1; ++k, ++q) {
    const int64_t b = in_blk[k];
    two_sum_add(su[q], cu[q], pbuf[b + j]);
    if (skel) two_sum_add(sh[q], ch[q], pbuf[b + bs + j]);
  }
  double vu = 0.0, vh = 0.0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    vu += (double)su[q] + (double)cu[q];
    vh += (double)sh[q] + (double)ch[q];
  }
  u[off + j] += scale * vu;
  if (skel) uh[off + j] += scale * vh;
}

}  // namespace skf
