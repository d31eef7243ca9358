// skf_build.cu — proxy-surface interpolative decompositions of one tree level.
//
// Replaces util.skel_box_helper (skelfmm/util.py:404-437) as driven by
// RecursiveSkeletonization.skel_tree (skelfmm/recursive_skel.py:412-492):
// for every box of a level, in one launch (one thread block per box),
//   1. the stacked proxy matrix (util.py:87-124): symmetric point kernels use
//      K(x_box, proxy)^T (nproxy x bs) — the reference stacks that block twice,
//      which scales R by sqrt(2) and leaves ranks, pivots and T unchanged —
//      geometry kernels use [K(proxy, x_box); K(x_box, proxy)^T] (2 nproxy x bs);
//   2. a column-pivoted Householder QR in FP64 (Businger & Golub, 1965) with
//      the partial-norm downdating safeguard of Drmac & Bujanovic (LAPACK
//      Working Note 176), stopped at the first |R_kk| <= tol |R_00|
//      (util.py:25-35 counts |R_ii| > tol |R_00|; the diagonal of a
//      column-pivoted QR is non-increasing);
//   3. T = R11^{-1} R12 by column-oriented back substitution (util.py:41-49).
// The proxy matrix lives column-major in a global workspace (L2-resident for
// leaf-sized boxes); one warp owns a column during each trailing update.
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstdio>
#include <cmath>
#include <random>
#include <type_traits>
#include <vector>

#include "skf_internal.cuh"
#include "skf_kernels.cuh"

namespace skf {

// Proxy surfaces of side 1 centred at the origin, matching
// skelfmm_gb300.tree.get_cube_surface / get_sphere_surface.
static std::vector<double> proxy_template(int ndim, bool sphere, int nproxy) {
  std::vector<double> t;
  const double length = 1.0, h = 0.5;
  if (!sphere) {
    if (ndim == 2) {
      const int n = std::max(1, (int)std::ceil(nproxy / 4.0));
      for (int side = 0; side < 4; ++side)
        for (int k = 0; k < n; ++k) {
          const double s = -h + length * (double)k / n;
          double x = 0, y = 0;
          if (side == 0) { x = s; y = -h; }
          if (side == 1) { x = h; y = s; }
          if (side == 2) { x = -s; y = h; }
          if (side == 3) { x = -h; y = -s; }
          t.push_back(x);
          t.push_back(y);
        }
    } else {
      const int n = std::max(1, (int)std::ceil(std::sqrt(nproxy / 6.0)));
      for (int axis = 0; axis < 3; ++axis) {
        int o0 = axis == 0 ? 1 : 0, o1 = axis == 2 ? 1 : 2;
        for (int sg = 0; sg < 2; ++sg)
          for (int a = 0; a < n; ++a)
            for (int b = 0; b < n; ++b) {
              double p[3];
              p[axis] = sg == 0 ? -h : h;
              p[o0] = -h + length * (a + 0.5) / n;
              p[o1] = -h + length * (b + 0.5) / n;
              t.push_back(p[0]);
              t.push_back(p[1]);
              t.push_back(p[2]);
            }
      }
    }
  } else {
    const int n = std::max(1, nproxy);
    if (ndim == 2) {
      for (int k = 0; k < n; ++k) {
        const double th = 2.0 * M_PI * k / n;
        t.push_back(h * std::cos(th));
        t.push_back(h * std::sin(th));
      }
    } else {
      const double ga = M_PI * (3.0 - std::sqrt(5.0));
      for (int k = 0; k < n; ++k) {
        const double kk = k + 0.5;
        const double z = 1.0 - 2.0 * kk / n;
        const double rho = std::sqrt(std::max(0.0, 1.0 - z * z));
        const double phi = ga * kk;
        t.push_back(h * rho * std::cos(phi));
        t.push_back(h * rho * std::sin(phi));
        t.push_back(h * z);
      }
    }
  }
  return t;
}

struct SkelArgs {
  const int64_t* off;
  const double* x;
  const double* geom;
  const double* centers;
  const double* tmpl;  // [np * ndim] unit proxy surface
  int np;              // proxy points
  int mrows;           // rows of the proxy matrix (np or 2 np)
  double plen;         // proxy side = 2.95 * box length
  const double* box_len;  // per-box side lengths (boxes of several trees), or NULL: plen for all
  double kappa;
  double tol;
  double* ws;          // column-major workspace
  const int64_t* ws_off;
  int32_t* rank;
  int32_t* perm;
  const int64_t* t_off_out;
  double* t_out;
  int first_box;
  // randomized mode: box b with kpred[b] > 0 first factors the sketch
  // Y = S K of its proxy matrix, kpred[b] + oversample rows of the launch's
  // sparse sign matrix S (`rho` entries +-1 per row, drawn on the host from
  // `seed`, shared by all boxes: S does not depend on K).  If the rank found
  // on Y (|R_kk| <= sketch_tol |R_00|) comes within oversample / 2 of the
  // sketch size the sketch is saturated; otherwise the ID is checked on nchk
  // hashed rows of K and kept when its relative Frobenius residual is <=
  // resid_tol.  Saturated or rejected boxes run the full pivoted-QR ID of K.
  const int32_t* kpred;
  int oversample;
  int rho;
  uint64_t seed;
  int nchk;
  double sketch_tol;
  double resid_tol;
  double* resid;    // [nbox] residual of the randomized ID (-1: not tried)
  int8_t* status;   // [nbox] 0 full QR; else 10 * sketch rounds + (1 kept, 2 rejected)
  const int32_t* sk_tab;  // [sk_rows * rho] sketch entries: proxy row | sign bit 31
  const int32_t* order;  // block -> box of the batch, longest first (NULL: identity)
  // deferred fallback: a rejected randomized ID writes only its status and
  // residual; its pivoted-QR ID runs in a second launch over the rejects
  int defer;
  // sketch round of a randomized launch (1: the predicted rank, 2: the
  // larger sketch a first-round reject retries with), in the status code
  int round;
  // set to 1 by any block whose proxy matrix has a non-finite entry or whose
  // points (normals) are not finite; NULL: unchecked
  int* nonfinite;
};

constexpr int kSkelThreads = 256;

__device__ __forceinline__ double block_sum(double v, double* red) {
  v = warp_sum_d(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  double s = 0;
  for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[i];
  return s;
}

// 1/sqrt(x) from the hardware estimate and one Newton step (relative error
// ~2^-44): proxy matrices that only feed a sketch and its residual check.
__device__ __forceinline__ double rsqrt_f64_1(double x) {
  double y;
  asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  const double e = fma(-x * y, y, 1.0);
  return fma(0.5 * y, e, y);
}

// 3D Laplace proxy-matrix entries on the FP32 pipes (GB300 issues FP64 at
// 1/64 of the FP32 rate): 1/|x - p| as an unevaluated FP32 pair hi + lo with
// relative error ~1e-13, from u = x - c and v = p - c (c the box centre)
// held as FP32 pairs.  d = u - v by TwoSum (Knuth) plus the low parts; r^2
// from exact squares (FMA residuals) and TwoSums; 1/r from the hardware
// estimate y0 and one Newton step in pair arithmetic, y = y0 + y0 (1 -
// r^2 y0^2) / 2, where 1 - fl(r^2 y0^2) is exact (Sterbenz).  Used for the
// matrices that feed a sketch and its residual check (randomized IDs).
__device__ __forceinline__ void two_sum_f(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ float2 lap3d_pair(const float (&uh)[3], const float (&ul)[3], const float* vh,
                                             const float* vl) {
  float dh[3], dl[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    two_sum_f(uh[k], -vh[k], dh[k], dl[k]);
    dl[k] = __fadd_rn(dl[k], __fsub_rn(ul[k], vl[k]));
  }
  // r^2 = sum dh^2 + 2 dh dl (dl^2 below the pair's precision)
  float p[3], pe[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    p[k] = __fmul_rn(dh[k], dh[k]);
    pe[k] = __fmaf_rn(dh[k], dh[k], -p[k]);
  }
  float h, e1, e2;
  two_sum_f(p[0], p[1], h, e1);
  two_sum_f(h, p[2], h, e2);
  float l = __fadd_rn(__fadd_rn(e1, e2), __fadd_rn(__fadd_rn(pe[0], pe[1]), pe[2]));
  l = __fmaf_rn(__fmul_rn(2.f, dh[0]), dl[0], l);
  l = __fmaf_rn(__fmul_rn(2.f, dh[1]), dl[1], l);
  l = __fmaf_rn(__fmul_rn(2.f, dh[2]), dl[2], l);
  const float H = __fadd_rn(h, l);
  const float L = __fsub_rn(l, __fsub_rn(H, h));
  // 1/r: y0 ~ 1/sqrt(H), then one Newton step with t = r^2 y0^2 in pairs
  const float y0 = rsqrtf(H);
  const float a = __fmul_rn(y0, y0);
  const float b = __fmaf_rn(y0, y0, -a);
  const float t = __fmul_rn(H, a);
  const float te = __fmaf_rn(H, a, -t);
  const float rest = __fmaf_rn(L, a, __fmaf_rn(H, b, te));
  const float delta = __fsub_rn(__fsub_rn(1.f, t), rest);
  return make_float2(y0, __fmul_rn(__fmul_rn(0.5f, y0), delta));
}

__device__ __forceinline__ double pair_to_f64(float2 v) { return __dadd_rn((double)v.x, (double)v.y); }

// Entry (row i, box point x) of the stacked proxy matrix: rows [0, np) are
// K(x, p_i) (target = box point), rows [np, 2 np) of the geometry operators
// K(p_i, x) (target = proxy).  Sphere proxies carry radial normals.  `pts`
// holds the box's proxy points (NULL: from the template).  FAST: 3D Laplace
// entries from rsqrt_f64_1.
template <int OP, bool FAST = false>
__device__ __forceinline__ void proxy_entry(const SkelArgs& a, const double (&c)[3], double plen, const double* pts,
                                            int i, const double* xj, const double* gj, double& kr, double& ki) {
  constexpr int D = OpTraits<OP>::kDim;
  constexpr int G = OpTraits<OP>::kGeom;
  const int pi = (i < a.np) ? i : i - a.np;
  double p[3] = {0, 0, 0};
  if (pts) {
    for (int d = 0; d < D; ++d) p[d] = pts[pi * D + d];
  } else {
    for (int d = 0; d < D; ++d) p[d] = c[d] + plen * a.tmpl[pi * D + d];
  }
  if constexpr (FAST && OP == SKF_LAPLACE_3D) {
    const double dx = xj[0] - p[0], dy = xj[1] - p[1], dz = xj[2] - p[2];
    kr = rsqrt_f64_1(fma(dx, dx, fma(dy, dy, dz * dz)));
    ki = 0.0;
    return;
  }
  double gx = 0, gy = 0, gz = 0;
  double pn[3] = {0, 0, 0};
  if (G != 0) {
    double nn = 0;
    for (int d = 0; d < D; ++d) {
      pn[d] = p[d] - c[d];
      nn += pn[d] * pn[d];
    }
    nn = sqrt(nn);
    for (int d = 0; d < D; ++d) pn[d] /= nn;
  }
  if (G == 0 || i >= a.np) {
    // K(x_j, p_i): target = box point, source = proxy
    if (G == 1) { gx = pn[0]; gy = pn[1]; gz = pn[2]; }
    if (G == 2) { gx = gj[0]; gy = gj[1]; gz = gj[2]; }
    eval_f64<OP>(xj[0] - p[0], xj[1] - p[1], D == 3 ? xj[2] - p[2] : 0.0, gx, gy, gz, a.kappa, kr, ki);
  } else {
    // K(p_i, x_j): target = proxy, source = box point
    if (G == 1) { gx = gj[0]; gy = gj[1]; gz = gj[2]; }
    if (G == 2) { gx = pn[0]; gy = pn[1]; gz = pn[2]; }
    eval_f64<OP>(p[0] - xj[0], p[1] - xj[1], D == 3 ? p[2] - xj[2] : 0.0, gx, gy, gz, a.kappa, kr, ki);
  }
}

// A box takes the randomized ID when its sketch has at most 3/4 of the
// proxy matrix's rows (the factorization's cost is proportional to the rows).
__host__ __device__ __forceinline__ bool sketch_fits(int64_t s, int64_t m) { return 4 * s <= 3 * m; }

// 64-bit mixing function (splitmix64 finaliser) for the sketch's indices.
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

struct QrScratch {
  double* vn1;  // [n] squared partial column norms
  double* vn2;  // [n] squared norms at the last recomputation
  double* vv;   // [m * W] Householder vector
  double* red;  // [64] reduction scratch
  int* piv;     // [n] column permutation
};

// Real reflector I - tau v v^T on rows k..m-1 of columns held in registers.
// A group of G lanes (G = 4, 8, 16 or 32, group lane sl) holds one column, CR
// rows per lane (row k + sl + G q, m - k <= G CR), loaded with every load in
// flight: a step costs one round trip to L2 per column.  The narrowest group
// whose registers hold the slice is used, so the FP64 instructions issued per
// column follow the slice length (a short sketch column takes a quarter of a
// warp) instead of the register capacity.
constexpr int kColRegs = 24;

// Applies the reflector to the group's column (live: the group has a
// column); returns its updated row-k entry on every lane of the group.
template <int G, int CR>
__device__ __forceinline__ double group_reflect(double* __restrict__ cj, bool live, const double* __restrict__ vv,
                                                int k, int m, double tau, int sl, double (&cr)[CR]) {
#pragma unroll
  for (int q = 0; q < CR; ++q) {
    const int i = k + sl + G * q;
    cr[q] = (live && i < m) ? cj[i] : 0.0;
  }
  double w0 = 0, w1 = 0;
#pragma unroll
  for (int q = 0; q < CR; q += 2) {
    const int i = k + sl + G * q;
    w0 = fma(i < m ? vv[i] : 0.0, cr[q], w0);
    if (q + 1 < CR) w1 = fma(i + G < m ? vv[i + G] : 0.0, cr[q + 1], w1);
  }
  double w = w0 + w1;
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
  const double f = tau * w;
#pragma unroll
  for (int q = 0; q < CR; ++q) {
    const int i = k + sl + G * q;
    if (i < m) {
      const double v = fma(-vv[i], f, cr[q]);
      cr[q] = v;
      if (live) cj[i] = v;
    }
  }
  const int lane = threadIdx.x & 31;
  return __shfl_sync(0xffffffffu, cr[0], lane - sl);
}

// Squared norm of rows > k of the group's updated column (group-reduced).
template <int G, int CR>
__device__ __forceinline__ double group_norm_below(const double (&cr)[CR], int k, int m, int sl) {
  double p = 0;
#pragma unroll
  for (int q = 0; q < CR; ++q) {
    const int i = k + sl + G * q;
    if (i > k && i < m) p = fma(cr[q], cr[q], p);
  }
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) p += __shfl_xor_sync(0xffffffffu, p, o);
  return p;
}

// Partial-norm downdate of column j after step k (LAWN 176, squared form):
// vn1 - |r_kj|^2, recomputed from the column when it falls to
// sqrt(eps) vn2.  `norm()` is evaluated by the whole warp only when some
// group of the warp recomputes.
template <typename NormFn>
__device__ __forceinline__ void downdate_norm(bool live, int j, bool lead, double akj, double* vn1, double* vn2,
                                              double tol3z, NormFn norm) {
  double v1 = 0.0, rem = 0.0;
  bool rc = false;
  if (live) {
    v1 = vn1[j];
    rem = v1 - akj * akj;
    rc = v1 != 0.0 && rem <= tol3z * vn2[j];
  }
  double p = 0.0;
  if (__any_sync(0xffffffffu, rc)) p = norm();
  if (live && lead) {
    if (rc) {
      vn1[j] = p;
      vn2[j] = p;
    } else if (v1 != 0.0) {
      vn1[j] = rem;
    }
  }
}

// Trailing update of columns k+1..n-1 of the column-major m x n matrix A,
// 32 / G columns per warp pass.
template <int G, int CR>
__device__ __noinline__ void reflect_trailing(double* A, int m, int n, int k, const double* __restrict__ vv, double tau,
                                 double* vn1, double* vn2, double tol3z) {
  constexpr int NG = 32 / G;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int g = lane / G, sl = lane - g * G;
  for (int j0 = k + 1 + NG * warp; j0 < n; j0 += NG * nw) {
    const int j = j0 + g;
    const bool live = j < n;
    double cr[CR];
    const double akj = group_reflect<G, CR>(A + (int64_t)(live ? j : j0) * m, live, vv, k, m, tau, sl, cr);
    downdate_norm(live, j, sl == 0, akj, vn1, vn2, tol3z, [&] { return group_norm_below<G, CR>(cr, k, m, sl); });
  }
}

// Picks the lane group and register count for rows k..m-1; false when the
// slice exceeds 32 kColRegs rows.
__device__ __forceinline__ bool reflect_trailing_regs(double* A, int m, int n, int k, const double* vv, double tau,
                                                      double* vn1, double* vn2, double tol3z) {
  const int len = m - k;
  if (len <= 4 * kColRegs) {
    const int cr = (len + 3) / 4;
    if (cr <= 4) reflect_trailing<4, 4>(A, m, n, k, vv, tau, vn1, vn2, tol3z);
    else if (cr <= 8) reflect_trailing<4, 8>(A, m, n, k, vv, tau, vn1, vn2, tol3z);
    else if (cr <= 12) reflect_trailing<4, 12>(A, m, n, k, vv, tau, vn1, vn2, tol3z);
    else if (cr <= 16) reflect_trailing<4, 16>(A, m, n, k, vv, tau, vn1, vn2, tol3z);
    else if (cr <= 20) reflect_trailing<4, 20>(A, m, n, k, vv, tau, vn1, vn2, tol3z);
    else reflect_trailing<4, 24>(A, m, n, k, vv, tau, vn1, vn2, tol3z);
  } else if (len <= 8 * kColRegs) {
    const int cr = (len + 7) / 8;
    if (cr <= 16) reflect_trailing<8, 16>(A, m, n, k, vv, tau, vn1, vn2, tol3z);
    else if (cr <= 20) reflect_trailing<8, 20>(A, m, n, k, vv, tau, vn1, vn2, tol3z);
    else reflect_trailing<8, 24>(A, m, n, k, vv, tau, vn1, vn2, tol3z);
  } else if (len <= 16 * kColRegs) {
    const int cr = (len + 15) / 16;
    if (cr <= 16) reflect_trailing<16, 16>(A, m, n, k, vv, tau, vn1, vn2, tol3z);
    else if (cr <= 20) reflect_trailing<16, 20>(A, m, n, k, vv, tau, vn1, vn2, tol3z);
    else reflect_trailing<16, 24>(A, m, n, k, vv, tau, vn1, vn2, tol3z);
  } else if (len <= 32 * kColRegs) {
    const int cr = (len + 31) / 32;
    if (cr <= 16) reflect_trailing<32, 16>(A, m, n, k, vv, tau, vn1, vn2, tol3z);
    else if (cr <= 20) reflect_trailing<32, 20>(A, m, n, k, vv, tau, vn1, vn2, tol3z);
    else reflect_trailing<32, 24>(A, m, n, k, vv, tau, vn1, vn2, tol3z);
  } else {
    return false;
  }
  return true;
}

// Column-pivoted Householder QR of the m x n column-major matrix A (leading
// dimension m), stopped at rank kfix (> 0) or at |R_kk| <= tol |R_00|.
// Businger-Golub pivoting (first index of the largest partial norm), partial
// norms downdated as in LAPACK's xLAQP2 (LAWN 176), kept squared: the
// downdate vn1^2 - |r_kj|^2 and LAPACK's recompute test
// (1 - (|r_kj| / vn1)^2) (vn1 / vn2)^2 <= sqrt(eps), i.e.
// vn1^2 - |r_kj|^2 <= sqrt(eps) vn2^2, need no division or square root.
// On return A holds R in its upper triangle (rows < rank) and the updated
// trailing block; piv the column order.  Returns the rank.
template <int OP>
__device__ int pivoted_qr(double* A, int m, int n, double tol, int kfix, const QrScratch& q) {
  constexpr bool C = OpTraits<OP>::kComplex;
  constexpr int W = C ? 2 : 1;
  __shared__ int s_k;
  __shared__ double s_scal[4];
  double* vn1 = q.vn1;
  double* vn2 = q.vn2;
  double* vv = q.vv;
  double* red = q.red;
  int* piv = q.piv;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int j = warp; j < n; j += nw) {
    double s = 0;
    const double* col = A + (int64_t)j * m * W;
    for (int i = lane; i < m * W; i += 32) s += col[i] * col[i];
    s = warp_sum_d(s);
    if (lane == 0) {
      vn1[j] = s;
      vn2[j] = s;
    }
  }
  for (int j = threadIdx.x; j < n; j += blockDim.x) piv[j] = j;
  __syncthreads();

  const int kmax = min(m, n);
  const bool fixed = kfix > 0;
  const int rank_fixed = fixed ? min(kfix, kmax) : kmax;
  double r00 = 0.0;
  int rank = 0;
  const double tol3z = sqrt(2.220446049250313e-16);
  for (int k = 0; k < kmax; ++k) {
    // pivot: first index of the largest partial norm
    double best = -1.0;
    int bi = k;
    for (int j = k + threadIdx.x; j < n; j += blockDim.x) {
      const double v = vn1[j];
      if (v > best) {
        best = v;
        bi = j;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ob > best || (ob == best && oi < bi)) {
        best = ob;
        bi = oi;
      }
    }
    __syncthreads();
    if (lane == 0) {
      red[warp] = best;
      reinterpret_cast<int*>(red + 32)[warp] = bi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double bb = red[0];
      int bj = reinterpret_cast<int*>(red + 32)[0];
      for (int w = 1; w < nw; ++w) {
        const double ob = red[w];
        const int oi = reinterpret_cast<int*>(red + 32)[w];
        if (ob > bb || (ob == bb && oi < bj)) {
          bb = ob;
          bj = oi;
        }
      }
      s_k = bj;
    }
    __syncthreads();
    const int p = s_k;
    if (p != k) {
      double* ck = A + (int64_t)k * m * W;
      double* cp = A + (int64_t)p * m * W;
      for (int i = threadIdx.x; i < m * W; i += blockDim.x) {
        const double t = ck[i];
        ck[i] = cp[i];
        cp[i] = t;
      }
      if (threadIdx.x == 0) {
        const int t = piv[k];
        piv[k] = piv[p];
        piv[p] = t;
        vn1[p] = vn1[k];
        vn2[p] = vn2[k];
      }
    }
    __syncthreads();
    // Householder reflector for column k, rows k..m-1 (complex: LAPACK zlarfg form)
    double* ck = A + (int64_t)k * m * W;
    double s = 0;
    for (int i = k + 1 + threadIdx.x; i < m; i += blockDim.x) {
      s += ck[i * W] * ck[i * W];
      if (C) s += ck[i * W + 1] * ck[i * W + 1];
    }
    const double xnorm2 = block_sum(s, red);
    if (threadIdx.x == 0) {
      const double ar = ck[k * W], ai = C ? ck[k * W + 1] : 0.0;
      double beta, taur = 0, taui = 0, scr = 0, sci = 0;
      if (xnorm2 == 0.0 && ai == 0.0) {
        beta = ar;  // H = I
        taur = 0;
        scr = 0;
      } else {
        const double nrm = sqrt(ar * ar + ai * ai + xnorm2);
        beta = ar >= 0 ? -nrm : nrm;
        taur = (beta - ar) / beta;
        taui = -ai / beta;
        // scale = 1 / (alpha - beta)
        const double dr = ar - beta, di = ai;
        const double dd = dr * dr + di * di;
        scr = dr / dd;
        sci = -di / dd;
      }
      s_scal[0] = beta;
      s_scal[1] = taur;
      s_scal[2] = taui;
      s_scal[3] = 0;
      red[60] = scr;
      red[61] = sci;
    }
    __syncthreads();
    const double beta = s_scal[0], taur = s_scal[1], taui = s_scal[2];
    const double scr = red[60], sci = red[61];
    if (k == 0) r00 = fabs(beta);
    const double rkk = fabs(beta);
    const bool stop = fixed ? (k >= rank_fixed) : (!(rkk > tol * r00) || r00 == 0.0);
    if (stop) {
      rank = k;
      break;
    }
    rank = k + 1;
    // v = [1; x(k+1:) * scale]
    for (int i = k + threadIdx.x; i < m; i += blockDim.x) {
      if (i == k) {
        vv[i * W] = 1.0;
        if (C) vv[i * W + 1] = 0.0;
      } else {
        const double xr = ck[i * W], xi = C ? ck[i * W + 1] : 0.0;
        vv[i * W] = xr * scr - xi * sci;
        if (C) vv[i * W + 1] = xr * sci + xi * scr;
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      ck[k * W] = beta;
      if (C) ck[k * W + 1] = 0.0;
    }
    // trailing update: A(k:, j) -= conj(tau) v (v^H A(k:, j)), one warp per column
    if constexpr (!C) {
      if (reflect_trailing_regs(A, m, n, k, vv, taur, vn1, vn2, tol3z)) {
        __syncthreads();
        continue;
      }
    }
    for (int j = k + 1 + warp; j < n; j += nw) {
      double* cj = A + (int64_t)j * m * W;
      double wr = 0, wi = 0;
      for (int i = k + lane; i < m; i += 32) {
        const double vr = vv[i * W], vi = C ? vv[i * W + 1] : 0.0;
        const double ar = cj[i * W], ai = C ? cj[i * W + 1] : 0.0;
        // conj(v) * a
        wr += vr * ar + vi * ai;
        if (C) wi += vr * ai - vi * ar;
      }
      wr = warp_sum_d(wr);
      if (C) wi = warp_sum_d(wi);
      // f = conj(tau) * w  (H^H applied: LAPACK zgeqp3 applies H(k)^H = I - conj(tau) v v^H)
      const double fr = taur * wr + taui * wi;
      const double fi = C ? (taur * wi - taui * wr) : 0.0;
      double part = 0;
      for (int i = k + lane; i < m; i += 32) {
        const double vr = vv[i * W], vi = C ? vv[i * W + 1] : 0.0;
        double ar = cj[i * W] - (vr * fr - vi * fi);
        cj[i * W] = ar;
        if (C) {
          double ai = cj[i * W + 1] - (vr * fi + vi * fr);
          cj[i * W + 1] = ai;
          if (i > k) part += ar * ar + ai * ai;
        } else if (i > k) {
          part += ar * ar;
        }
      }
      // partial-norm downdate (LAWN 176): every lane takes the same decision
      __syncwarp();
      double akj2;
      {
        const double ar = cj[k * W], ai = C ? cj[k * W + 1] : 0.0;
        akj2 = ar * ar + ai * ai;
      }
      const double v1 = vn1[j];
      const double rem = v1 - akj2;
      const bool recompute = v1 != 0.0 && rem <= tol3z * vn2[j];
      if (recompute) {
        part = warp_sum_d(part);
        if (lane == 0) {
          vn1[j] = part;
          vn2[j] = part;
        }
      } else if (lane == 0 && v1 != 0.0) {
        vn1[j] = rem;
      }
      __syncwarp();
    }
    __syncthreads();
  }
  __syncthreads();
  return rank;
}

// T = R11^{-1} R12 (row-major rank x (n - rank)) from the R that pivoted_qr
// left in A: column back substitution, one warp per right-hand side.
template <int OP>
__device__ void write_T(double* A, int m, int n, int rank, double* T, double* rinv) {
  constexpr bool C = OpTraits<OP>::kComplex;
  constexpr int W = C ? 2 : 1;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int nr = n - rank;
  // reciprocals of the diagonal of R11 (rinv: [rank * W] shared scratch)
  for (int i = threadIdx.x; i < rank; i += blockDim.x) {
    const double rr = A[((int64_t)i * m + i) * W], ri = C ? A[((int64_t)i * m + i) * W + 1] : 0.0;
    if (C) {
      const double dd = rr * rr + ri * ri;
      rinv[2 * i] = rr / dd;
      rinv[2 * i + 1] = -ri / dd;
    } else {
      rinv[i] = 1.0 / rr;
    }
  }
  __syncthreads();
  if (rank > 0 && nr > 0) {
    for (int cidx = warp; cidx < nr; cidx += nw) {
      double* bcol = A + (int64_t)(rank + cidx) * m * W;  // R12(:, c), overwritten by t
      for (int i = rank - 1; i >= 0; --i) {
        const double* ci = A + (int64_t)i * m * W;
        double tr, ti = 0;
        {
          const double br = bcol[i * W], bi = C ? bcol[i * W + 1] : 0.0;
          if (C) {
            const double qr = rinv[2 * i], qi = rinv[2 * i + 1];
            tr = br * qr - bi * qi;
            ti = br * qi + bi * qr;
          } else {
            tr = br * rinv[i];
          }
        }
        __syncwarp();
        if (lane == 0) {
          bcol[i * W] = tr;
          if (C) bcol[i * W + 1] = ti;
        }
        for (int l = lane; l < i; l += 32) {
          const double rr = ci[l * W], ri = C ? ci[l * W + 1] : 0.0;
          bcol[l * W] -= rr * tr - ri * ti;
          if (C) bcol[l * W + 1] -= rr * ti + ri * tr;
        }
        __syncwarp();
      }
      for (int i = lane; i < rank; i += 32) {
        T[((int64_t)i * nr + cidx) * W] = bcol[i * W];
        if (C) T[((int64_t)i * nr + cidx) * W + 1] = bcol[i * W + 1];
      }
    }
  }
  __syncthreads();
}

// RAND: the launch carries randomized boxes (a.kpred).
template <int OP, int NT, bool RAND>
__global__ void __launch_bounds__(NT, NT <= 256 ? 2 : 1) k_skel_box(SkelArgs a) {
  constexpr bool C = OpTraits<OP>::kComplex;
  constexpr int D = OpTraits<OP>::kDim;
  constexpr int W = C ? 2 : 1;  // scalars per matrix entry
  extern __shared__ double sm[];
  const int lb = a.order ? a.order[blockIdx.x] : (int)blockIdx.x;  // box within the batch
  const int b = a.first_box + lb;
  const int64_t off = a.off[b];
  const int n = (int)(a.off[b + 1] - off);
  const int m = a.mrows;
  const int kp = (RAND && a.kpred) ? a.kpred[b] : 0;
  // randomized ID while the sketch is well below the proxy matrix
  int s = kp > 0 ? min(kp, n) + a.oversample : 0;
  const bool sketch = kp > 0 && sketch_fits(s, m);
  // smem: vn1[n], vn2[n], v[m * W], red[64], proxy points[np * D], piv[n]
  QrScratch q;
  q.vn1 = sm;
  q.vn2 = q.vn1 + n;
  q.vv = q.vn2 + n;
  q.red = q.vv + (size_t)m * W;
  double* pts = q.red + 64;
  q.piv = reinterpret_cast<int*>(pts + (size_t)a.np * D);

  double* A = a.ws + a.ws_off[lb];
  double c[3] = {0, 0, 0};
  for (int d = 0; d < D; ++d) c[d] = a.centers[(int64_t)b * D + d];
  const double plen = a.box_len ? 2.95 * a.box_len[b] : a.plen;
  // 3D Laplace boxes of a randomized launch keep K as FP32 pairs (lap3d_pair)
  // in the FP64 slots: it only feeds the sketch and the residual check
  const bool pairs = RAND && OP == SKF_LAPLACE_3D && sketch && m == a.np;
  float* vh = reinterpret_cast<float*>(pts);  // pairs: p_i - c as FP32 pairs
  float* vl = vh + a.np * 3;
  if (pairs) {
    for (int i = threadIdx.x; i < a.np * 3; i += blockDim.x) {
      const double v = plen * a.tmpl[i];
      const float h = __double2float_rn(v);
      vh[i] = h;
      vl[i] = __double2float_rn(v - (double)h);
    }
  } else {
    for (int i = threadIdx.x; i < a.np * D; i += blockDim.x) pts[i] = c[i % D] + plen * a.tmpl[i];
  }
  __syncthreads();

  // ---- 1. proxy matrix, column j = box point j (a warp per column)
  {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int j = warp; j < n; j += nw) {
      const double* xj = a.x + (off + j) * D;
      const double* gj = a.geom ? a.geom + (off + j) * 3 : nullptr;
      double* col = A + (int64_t)j * m * W;
      // a non-finite point (or normal) would read as a zero column where
      // the kernel masks r == 0, so the inputs are checked as well
      bool bad = false;
      for (int d = 0; d < D; ++d) bad |= !isfinite(xj[d]);
      if (gj) bad |= !(isfinite(gj[0]) && isfinite(gj[1]) && isfinite(gj[2]));
      if (pairs) {
        float uh[3], ul[3];
        for (int d = 0; d < 3; ++d) {
          const double u = xj[d] - c[d];
          uh[d] = __double2float_rn(u);
          ul[d] = __double2float_rn(u - (double)uh[d]);
        }
        float2* colp = reinterpret_cast<float2*>(col);
        for (int i = lane; i < m; i += 32) {
          const float2 k = lap3d_pair(uh, ul, vh + 3 * i, vl + 3 * i);
          colp[i] = k;
          bad |= !isfinite(k.x);
        }
      } else {
        for (int i = lane; i < m; i += 32) {
          double kr, ki;
          proxy_entry<OP, RAND>(a, c, plen, pts, i, xj, gj, kr, ki);
          col[i * W] = kr;
          if (C) col[i * W + 1] = ki;
          bad |= !isfinite(kr) || (C && !isfinite(ki));
        }
      }
      if (bad && a.nonfinite) *a.nonfinite = 1;
    }
  }
  __syncthreads();
  // K(row, column j) as FP64 (either storage)
  auto kval = [&](int j, int row) -> double {
    return pairs ? pair_to_f64(reinterpret_cast<const float2*>(A)[(int64_t)j * m + row])
                 : A[((int64_t)j * m + row) * W];
  };

  double* T = a.t_out + a.t_off_out[b] * W;
  int rank = 0;
  bool done = false;
  if (sketch) {
    // ---- 2a. sketches Y = S K (s x n, after K in the workspace): row t of
    // S has rho entries +-1 at hashed proxy rows
    double* Y = A + (int64_t)m * n * W;
    const int guard = max(2, a.oversample / 2);
    bool ok = false;
    const int rounds = a.round > 0 ? a.round : 1;
    {
      for (int64_t idx = threadIdx.x; idx < (int64_t)s * n; idx += blockDim.x) {
        const int j = (int)(idx / s), t = (int)(idx % s);
        double yr = 0, yi = 0;
        const double* col = A + (int64_t)j * m * W;
        const int32_t* row = a.sk_tab + (int64_t)t * a.rho;
        if (pairs) {
          // signed sum of FP32 pairs, compensated in FP32 (TwoSum)
          const float2* colp = reinterpret_cast<const float2*>(col);
          float sh = 0.f, sl = 0.f;
          for (int u = 0; u < a.rho; ++u) {
            const int32_t e = row[u];
            float2 v = colp[e & 0x7fffffff];
            if (e < 0) v = make_float2(-v.x, -v.y);
            float err;
            two_sum_f(sh, v.x, sh, err);
            sl = __fadd_rn(sl, __fadd_rn(err, v.y));
          }
          Y[(int64_t)j * s + t] = pair_to_f64(make_float2(sh, sl));
          continue;
        }
        for (int u = 0; u < a.rho; ++u) {
          const int32_t e = row[u];
          const int i = e & 0x7fffffff;
          if (e < 0) {
            yr -= col[(int64_t)i * W];
            if (C) yi -= col[(int64_t)i * W + 1];
          } else {
            yr += col[(int64_t)i * W];
            if (C) yi += col[(int64_t)i * W + 1];
          }
        }
        Y[((int64_t)j * s + t) * W] = yr;
        if (C) Y[((int64_t)j * s + t) * W + 1] = yi;
      }
      __syncthreads();
      rank = pivoted_qr<OP>(Y, s, n, a.sketch_tol, 0, q);
      ok = !(rank < n && rank > s - guard);  // saturated: the sketch hides rank
    }
    if (ok) {
      write_T<OP>(Y, s, n, rank, T, q.vn1);
      // ---- 2b. residual on nchk hashed rows of K (K is still intact)
      const uint64_t key = mix64(a.seed ^ ((uint64_t)b << 20));
      const int nr = n - rank;
      double e2 = 0.0, z2 = 0.0;
      for (int qi = 0; qi < a.nchk; ++qi) {
        const int row = (int)__umulhi((unsigned)(mix64(key ^ (0xC0FFEEull + (uint64_t)qi)) >> 32), (unsigned)m);
        for (int jr = threadIdx.x; jr < n; jr += blockDim.x) {
          const int pj = q.piv[jr];
          const double zr = kval(pj, row), zi = C ? A[((int64_t)pj * m + row) * W + 1] : 0.0;
          z2 += zr * zr + zi * zi;
          if (jr < rank) continue;
          double er = zr, ei = zi;
          for (int i = 0; i < rank; ++i) {
            const int pi = q.piv[i];
            const double sr = kval(pi, row), si = C ? A[((int64_t)pi * m + row) * W + 1] : 0.0;
            const double tr = T[((int64_t)i * nr + (jr - rank)) * W];
            const double ti = C ? T[((int64_t)i * nr + (jr - rank)) * W + 1] : 0.0;
            er -= sr * tr - si * ti;
            if (C) ei -= sr * ti + si * tr;
          }
          e2 += er * er + ei * ei;
        }
      }
      e2 = block_sum(e2, q.red);
      z2 = block_sum(z2, q.red);
      const double res = z2 > 0.0 ? sqrt(e2 / z2) : 0.0;
      done = res <= a.resid_tol;
      if (threadIdx.x == 0 && a.resid) a.resid[b] = res;
    } else if (threadIdx.x == 0 && a.resid) {
      a.resid[b] = -2.0;  // the sketch saturated
    }
    if (threadIdx.x == 0 && a.status) a.status[b] = (int8_t)(10 * rounds + (done ? 1 : 2));
    __syncthreads();
  } else if (threadIdx.x == 0) {
    if (a.resid) a.resid[b] = -1.0;
    if (a.status) a.status[b] = 0;
  }
  if (!done) {
    if (a.defer) return;
    if (pairs) {
      // K back to FP64 in place (each thread converts its own entries)
      for (int64_t idx = threadIdx.x; idx < (int64_t)m * n; idx += blockDim.x) {
        const float2 v = reinterpret_cast<const float2*>(A)[idx];
        A[idx] = pair_to_f64(v);
      }
      __syncthreads();
    }
    // ---- 3. full column-pivoted QR ID of K
    rank = pivoted_qr<OP>(A, m, n, a.tol >= 1.0 ? 0.0 : a.tol, a.tol >= 1.0 ? (int)a.tol : 0, q);
    write_T<OP>(A, m, n, rank, T, q.vn1);
  }
  if (threadIdx.x == 0) a.rank[b] = rank;
  for (int j = threadIdx.x; j < n; j += blockDim.x) a.perm[off + j] = q.piv[j];
}

// ---- one box on a thread-block cluster -------------------------------------
// The costliest boxes of a level (candidate sets of ~1,000-1,500 points) set
// the level's time when one block factors each.  Here a cluster of
// kClusterCTAs blocks, each on its own SM, factors one box: block r owns the
// physical columns j = r (mod kClusterCTAs) of the column-major proxy matrix
// in global memory.  Per elimination step: every block publishes its best
// candidate (squared partial norm, position) in shared memory; after a
// cluster barrier every block reads all candidates through distributed
// shared memory and applies the same logical swap of positions k and p; the
// pivot column's owner builds the Householder vector and publishes it; after
// a second cluster barrier every block copies it and updates its own
// columns.  Same pivoting rule (first position of the largest norm), stopping
// rule, squared-norm downdate and outputs as pivoted_qr + write_T.  Every
// block runs the same steps and cluster barriers: the stop decision reads the
// published |R_kk| after a barrier, so it is uniform over the cluster.
constexpr int kClusterCTAs = 8;

// Shared-memory scratch of one block of a cluster.
struct ClusterScratch {
  double* vsh;   // [m] Householder vector published by the pivot's owner
  double* vloc;  // [m] local copy (later: reciprocal diagonal)
  double* red;   // [64]
  double* pub;   // [8] candidate norm, candidate position, beta, tau, residual sums
  double* vn1;   // [ncl] squared partial norms of the owned columns
  double* vn2;   // [ncl]
  int* piv;      // [n] position -> physical column
  int* posof;    // [n] physical column -> position
};

// Column-pivoted QR of the column-major m x n matrix M (leading dimension
// m) on a cluster: block r owns the physical columns j = r (mod
// kClusterCTAs).  Stopped at rank kfix (> 0) or at |R_kk| <= tol |R_00|;
// the rank is uniform over the cluster.  On return M holds R (rows < rank
// of the pivot columns), piv / posof the column order, and every update is
// visible to the cluster.
__device__ int cluster_pivoted_qr(cooperative_groups::cluster_group& cl, double* M, int m, int n, double tol,
                                  int kfix, const ClusterScratch& s) {
  constexpr int NC = kClusterCTAs;
  const int cr = (int)cl.block_rank();
  const int ncl = (n + NC - 1) / NC;
  double* vsh = s.vsh;
  double* vloc = s.vloc;
  double* red = s.red;
  double* pub = s.pub;
  double* vn1 = s.vn1;
  double* vn2 = s.vn2;
  int* piv = s.piv;
  int* posof = s.posof;
  __shared__ int s_col;
  __shared__ double s_h[3];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    piv[j] = j;
    posof[j] = j;
  }
  for (int jl = warp; jl < ncl; jl += nw) {
    const int j = cr + NC * jl;
    if (j >= n) continue;
    const double* col = M + (int64_t)j * m;
    double sq = 0;
    for (int i = lane; i < m; i += 32) sq += col[i] * col[i];
    sq = warp_sum_d(sq);
    if (lane == 0) {
      vn1[jl] = sq;
      vn2[jl] = sq;
    }
  }
  __syncthreads();

  const int kmax = min(m, n);
  const bool fixed = kfix > 0;
  const int rank_fixed = fixed ? min(kfix, kmax) : kmax;
  const double tol3z = sqrt(2.220446049250313e-16);
  double r00 = 0.0;
  int rank = 0;
  for (int k = 0; k < kmax; ++k) {
    // ---- this block's candidate: largest norm, first position on ties
    double best = -1.0;
    int bpos = 0x7fffffff;
    for (int jl = threadIdx.x; jl < ncl; jl += blockDim.x) {
      const int j = cr + NC * jl;
      if (j >= n) continue;
      const int pos = posof[j];
      if (pos < k) continue;
      const double v = vn1[jl];
      if (v > best || (v == best && pos < bpos)) {
        best = v;
        bpos = pos;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int op = __shfl_xor_sync(0xffffffffu, bpos, o);
      if (ob > best || (ob == best && op < bpos)) {
        best = ob;
        bpos = op;
      }
    }
    if (lane == 0) {
      red[warp] = best;
      reinterpret_cast<int*>(red + 32)[warp] = bpos;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double bb = red[0];
      int bp = reinterpret_cast<int*>(red + 32)[0];
      for (int w = 1; w < nw; ++w) {
        const double ob = red[w];
        const int op = reinterpret_cast<int*>(red + 32)[w];
        if (ob > bb || (ob == bb && op < bp)) {
          bb = ob;
          bp = op;
        }
      }
      pub[0] = bb;
      pub[1] = (double)bp;
    }
    cl.sync();  // candidates published
    // ---- the cluster's pivot and the logical swap of positions k and p
    if (threadIdx.x == 0) {
      double gb = -1.0;
      int gp = 0x7fffffff;
      for (int r = 0; r < NC; ++r) {
        const double* rp = cl.map_shared_rank(pub, r);
        const double v = rp[0];
        const int p = (int)rp[1];
        if (v > gb || (v == gb && p < gp)) {
          gb = v;
          gp = p;
        }
      }
      const int ck = piv[k], cp = piv[gp];
      piv[k] = cp;
      piv[gp] = ck;
      posof[cp] = k;
      posof[ck] = gp;
      s_col = cp;
    }
    __syncthreads();
    const int col = s_col;
    const int owner = col % NC;
    if (cr == owner) {
      // Householder reflector of column col, rows k..m-1 (real zlarfg form)
      double* ckc = M + (int64_t)col * m;
      double sq = 0;
      for (int i = k + 1 + threadIdx.x; i < m; i += blockDim.x) sq += ckc[i] * ckc[i];
      const double xnorm2 = block_sum(sq, red);
      if (threadIdx.x == 0) {
        const double ar = ckc[k];
        double beta = ar, tau = 0, scl = 0;
        if (xnorm2 != 0.0) {
          const double nrm = sqrt(ar * ar + xnorm2);
          beta = ar >= 0 ? -nrm : nrm;
          tau = (beta - ar) / beta;
          scl = 1.0 / (ar - beta);
        }
        s_h[0] = beta;
        s_h[1] = tau;
        s_h[2] = scl;
        pub[2] = beta;
        pub[3] = tau;
      }
      __syncthreads();
      const double scl = s_h[2];
      for (int i = k + threadIdx.x; i < m; i += blockDim.x) vsh[i] = (i == k) ? 1.0 : ckc[i] * scl;
      __syncthreads();
      if (threadIdx.x == 0) ckc[k] = s_h[0];
    }
    cl.sync();  // reflector published
    const double* opub = cl.map_shared_rank(pub, owner);
    const double beta = opub[2], tau = opub[3];
    if (k == 0) r00 = fabs(beta);
    const bool stop = fixed ? (k >= rank_fixed) : (!(fabs(beta) > tol * r00) || r00 == 0.0);
    if (stop) {
      rank = k;
      break;
    }
    rank = k + 1;
    const double* ov = cl.map_shared_rank(vsh, owner);
    for (int i = k + threadIdx.x; i < m; i += blockDim.x) vloc[i] = ov[i];
    __syncthreads();
    // ---- trailing update of the owned columns at positions > k (one warp
    // per column, register count by the slice length)
    auto update_regs = [&](auto regs) {
      constexpr int CRN = decltype(regs)::value;
      for (int jl = warp; jl < ncl; jl += nw) {
        const int j = cr + NC * jl;
        if (j >= n || posof[j] <= k) continue;
        double c[CRN];
        const double akj = group_reflect<32, CRN>(M + (int64_t)j * m, true, vloc, k, m, tau, lane, c);
        downdate_norm(true, jl, lane == 0, akj, vn1, vn2, tol3z,
                      [&] { return group_norm_below<32, CRN>(c, k, m, lane); });
      }
    };
    const int len = m - k;
    if (len <= 32 * 8) {
      update_regs(std::integral_constant<int, 8>());
    } else if (len <= 32 * 16) {
      update_regs(std::integral_constant<int, 16>());
    } else if (len <= 32 * 20) {
      update_regs(std::integral_constant<int, 20>());
    } else if (len <= 32 * kColRegs) {
      update_regs(std::integral_constant<int, kColRegs>());
    } else {
      for (int jl = warp; jl < ncl; jl += nw) {
        const int j = cr + NC * jl;
        if (j >= n || posof[j] <= k) continue;
        double* cj = M + (int64_t)j * m;
        double w = 0;
        for (int i = k + lane; i < m; i += 32) w += vloc[i] * cj[i];
        w = warp_sum_d(w);
        const double f = tau * w;
        double part = 0;
        for (int i = k + lane; i < m; i += 32) {
          const double v = cj[i] - vloc[i] * f;
          cj[i] = v;
          if (i > k) part += v * v;
        }
        __syncwarp();
        const double akj = cj[k];
        downdate_norm(true, jl, lane == 0, akj, vn1, vn2, tol3z, [&] { return warp_sum_d(part); });
        __syncwarp();
      }
    }
    __syncthreads();
  }
  cl.sync();  // every update of M is visible; no remote reads follow
  return rank;
}

// T = R11^{-1} R12 (row-major rank x (n - rank)) for this block's redundant
// columns, from the R that cluster_pivoted_qr left in M (leading dimension m).
__device__ void cluster_write_T(double* M, int m, int n, int rank, double* T, const ClusterScratch& s, int cr) {
  constexpr int NC = kClusterCTAs;
  const int nr = n - rank;
  if (rank == 0 || nr == 0) return;
  const int ncl = (n + NC - 1) / NC;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  double* rinv = s.vloc;
  for (int i = threadIdx.x; i < rank; i += blockDim.x) rinv[i] = 1.0 / M[(int64_t)s.piv[i] * m + i];
  __syncthreads();
  for (int jl = warp; jl < ncl; jl += nw) {
    const int j = cr + NC * jl;
    if (j >= n) continue;
    const int pos = s.posof[j];
    if (pos < rank) continue;
    const int cidx = pos - rank;
    double* bcol = M + (int64_t)j * m;  // R12 column, overwritten by t
    for (int i = rank - 1; i >= 0; --i) {
      const double* ci = M + (int64_t)s.piv[i] * m;
      const double t = bcol[i] * rinv[i];
      __syncwarp();
      if (lane == 0) bcol[i] = t;
      for (int l = lane; l < i; l += 32) bcol[l] -= ci[l] * t;
      __syncwarp();
    }
    for (int i = lane; i < rank; i += 32) T[(int64_t)i * nr + cidx] = bcol[i];
  }
}

// RAND: boxes with a predicted rank first try the randomized ID on the
// cluster (sketch of the owned columns, pivoted QR of the sketch, residual
// on hashed rows of the proxy matrix reduced over the cluster), the same
// steps and outputs as k_skel_box's randomized branch; a rejected box takes
// the full pivoted-QR ID right away.
template <int OP, bool RAND>
__global__ void __cluster_dims__(kClusterCTAs, 1, 1) __launch_bounds__(kSkelThreads)
    k_skel_box_cluster(SkelArgs a) {
  static_assert(!OpTraits<OP>::kComplex, "real operators only");
  namespace cg = cooperative_groups;
  constexpr int D = OpTraits<OP>::kDim;
  constexpr int NC = kClusterCTAs;
  cg::cluster_group cl = cg::this_cluster();
  const int cr = (int)cl.block_rank();
  const int lb = a.order[blockIdx.x / NC];
  const int b = a.first_box + lb;
  const int64_t off = a.off[b];
  const int n = (int)(a.off[b + 1] - off);
  const int m = a.mrows;
  const int ncl = (n + NC - 1) / NC;
  double* A = a.ws + a.ws_off[lb];
  extern __shared__ double smc[];
  ClusterScratch s;
  s.vsh = smc;
  s.vloc = s.vsh + m;
  s.red = s.vloc + m;
  s.pub = s.red + 64;
  s.vn1 = s.pub + 8;
  s.vn2 = s.vn1 + ncl;
  s.piv = reinterpret_cast<int*>(s.vn2 + ncl);
  s.posof = s.piv + n;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  double c[3] = {0, 0, 0};
  for (int d = 0; d < D; ++d) c[d] = a.centers[(int64_t)b * D + d];
  const double plen = a.box_len ? 2.95 * a.box_len[b] : a.plen;
  // randomized 3D Laplace: K from FP32-pair entries (lap3d_pair, relative
  // error ~1e-13), rounded to FP64 (the fallback factors K in place)
  constexpr bool kPairs = RAND && OP == SKF_LAPLACE_3D;
  const bool pairs = kPairs && m == a.np;
  float* vh = reinterpret_cast<float*>(s.posof + n);
  float* vl = vh + 3 * a.np;
  if (pairs) {
    for (int i = threadIdx.x; i < a.np * 3; i += blockDim.x) {
      const double v = plen * a.tmpl[i];
      const float h = __double2float_rn(v);
      vh[i] = h;
      vl[i] = __double2float_rn(v - (double)h);
    }
    __syncthreads();
  }

  // ---- proxy matrix, owned columns only (a warp per column)
  for (int jl = warp; jl < ncl; jl += nw) {
    const int j = cr + NC * jl;
    if (j >= n) continue;
    const double* xj = a.x + (off + j) * D;
    const double* gj = a.geom ? a.geom + (off + j) * 3 : nullptr;
    bool bad = false;
    for (int d = 0; d < D; ++d) bad |= !isfinite(xj[d]);
    if (gj) bad |= !(isfinite(gj[0]) && isfinite(gj[1]) && isfinite(gj[2]));
    if (pairs) {
      float uh[3], ul[3];
      for (int d = 0; d < 3; ++d) {
        const double u = xj[d] - c[d];
        uh[d] = __double2float_rn(u);
        ul[d] = __double2float_rn(u - (double)uh[d]);
      }
      for (int i = lane; i < m; i += 32) {
        const float2 k = lap3d_pair(uh, ul, vh + 3 * i, vl + 3 * i);
        A[(int64_t)j * m + i] = pair_to_f64(k);
        bad |= !isfinite(k.x);
      }
    } else {
      for (int i = lane; i < m; i += 32) {
        double kr, ki;
        proxy_entry<OP>(a, c, plen, nullptr, i, xj, gj, kr, ki);
        A[(int64_t)j * m + i] = kr;
        bad |= !isfinite(kr);
      }
    }
    if (bad && a.nonfinite) *a.nonfinite = 1;
  }
  __syncthreads();

  double* T = a.t_out + a.t_off_out[b];
  int rank = 0;
  bool done = false;
  int8_t code = 0;
  double resid = -1.0;
  if constexpr (RAND) {
    const int kp = a.kpred ? a.kpred[b] : 0;
    const int sr = min(kp, n) + a.oversample;
    if (kp > 0 && sketch_fits(sr, m)) {
      // ---- sketch Y = S K of the owned columns (sr x n, after K)
      double* Y = A + (int64_t)m * n;
      for (int jl = warp; jl < ncl; jl += nw) {
        const int j = cr + NC * jl;
        if (j >= n) continue;
        const double* col = A + (int64_t)j * m;
        double* ycol = Y + (int64_t)j * sr;
        for (int t = lane; t < sr; t += 32) {
          const int32_t* row = a.sk_tab + (int64_t)t * a.rho;
          double y = 0;
          for (int u = 0; u < a.rho; ++u) {
            const int32_t e = row[u];
            const double v = col[e & 0x7fffffff];
            y += e < 0 ? -v : v;
          }
          ycol[t] = y;
        }
      }
      __syncthreads();
      rank = cluster_pivoted_qr(cl, Y, sr, n, a.sketch_tol, 0, s);
      const int guard = max(2, a.oversample / 2);
      if (rank < n && rank > sr - guard) {
        resid = -2.0;  // the sketch saturated
      } else {
        cluster_write_T(Y, sr, n, rank, T, s, cr);
        cl.sync();  // T visible to the cluster
        // ---- residual on nchk hashed rows of K
        const uint64_t key = mix64(a.seed ^ ((uint64_t)b << 20));
        const int nr = n - rank;
        double e2 = 0.0, z2 = 0.0;
        for (int qi = 0; qi < a.nchk; ++qi) {
          const int row = (int)__umulhi((unsigned)(mix64(key ^ (0xC0FFEEull + (uint64_t)qi)) >> 32), (unsigned)m);
          for (int jl = threadIdx.x; jl < ncl; jl += blockDim.x) {
            const int j = cr + NC * jl;
            if (j >= n) continue;
            const double z = A[(int64_t)j * m + row];
            z2 += z * z;
            const int pos = s.posof[j];
            if (pos < rank) continue;
            double e = z;
            for (int i = 0; i < rank; ++i) e -= A[(int64_t)s.piv[i] * m + row] * T[(int64_t)i * nr + (pos - rank)];
            e2 += e * e;
          }
        }
        e2 = block_sum(e2, s.red);
        z2 = block_sum(z2, s.red);
        if (threadIdx.x == 0) {
          s.pub[4] = e2;
          s.pub[5] = z2;
        }
        cl.sync();  // residual sums published
        double E2 = 0.0, Z2 = 0.0;
        for (int r = 0; r < NC; ++r) {
          const double* rp = cl.map_shared_rank(s.pub, r);
          E2 += rp[4];
          Z2 += rp[5];
        }
        resid = Z2 > 0.0 ? sqrt(E2 / Z2) : 0.0;
        done = resid <= a.resid_tol;
        cl.sync();  // remote reads of pub done before it is reused
      }
      code = (int8_t)(10 * (a.round > 0 ? a.round : 1) + (done ? 1 : 2));
    }
  }
  if (!done) {
    // ---- full column-pivoted QR ID of K
    rank = cluster_pivoted_qr(cl, A, m, n, a.tol >= 1.0 ? 0.0 : a.tol, a.tol >= 1.0 ? (int)a.tol : 0, s);
    cluster_write_T(A, m, n, rank, T, s, cr);
  }
  if (cr == 0) {
    if (threadIdx.x == 0) {
      a.rank[b] = rank;
      if (a.status) a.status[b] = code;
      if (a.resid) a.resid[b] = resid;
    }
    for (int pos = threadIdx.x; pos < n; pos += blockDim.x) a.perm[off + pos] = s.piv[pos];
  }
}

// Dynamic shared memory above this needs the opt-in attribute: 48 KB less
// a margin for the kernels' static shared variables.
constexpr size_t kSmemNoOptIn = 46 * 1024;

__global__ void k_fill_f64(double* __restrict__ p, int n, double v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

template <int OP, bool RAND>
static int launch_skel_cluster_t(const SkelArgs& a, int nbox, size_t smem, cudaStream_t st) {
  if (smem > kSmemNoOptIn)
    SKF_CUDA_TRY(
        cudaFuncSetAttribute(k_skel_box_cluster<OP, RAND>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_skel_box_cluster<OP, RAND><<<nbox * kClusterCTAs, kSkelThreads, smem, st>>>(a);
  SKF_CUDA_TRY(cudaGetLastError());
  return SKF_OK;
}

template <int OP>
static int launch_skel_cluster(const SkelArgs& a, int nbox, int maxn, cudaStream_t st) {
  const int ncl = (maxn + kClusterCTAs - 1) / kClusterCTAs;
  size_t smem = sizeof(double) * ((size_t)2 * a.mrows + 64 + 8 + 2 * (size_t)ncl) + sizeof(int) * 2 * (size_t)maxn;
  // randomized 3D Laplace: the proxies relative to the centre as FP32 pairs
  if (a.kpred && OP == SKF_LAPLACE_3D) smem += sizeof(float) * 6 * (size_t)a.np;
  if (smem > 200 * 1024) return SKF_ERR_UNSUPPORTED;
  return a.kpred ? launch_skel_cluster_t<OP, true>(a, nbox, smem, st) : launch_skel_cluster_t<OP, false>(a, nbox, smem, st);
}

template <int OP, int NT>
static int launch_skel_nt(const SkelArgs& a, int nbox, size_t smem, cudaStream_t st) {
  if (a.kpred) {
    if (smem > kSmemNoOptIn)
      SKF_CUDA_TRY(cudaFuncSetAttribute(k_skel_box<OP, NT, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_skel_box<OP, NT, true><<<nbox, NT, smem, st>>>(a);
  } else {
    if (smem > kSmemNoOptIn)
      SKF_CUDA_TRY(cudaFuncSetAttribute(k_skel_box<OP, NT, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_skel_box<OP, NT, false><<<nbox, NT, smem, st>>>(a);
  }
  SKF_CUDA_TRY(cudaGetLastError());
  return SKF_OK;
}

// One batch of boxes.  With nbig > 0 the first nbig boxes of a.order (the
// most expensive) run on `side` — one thread-block cluster per box for real
// operators (full pivoted-QR ID), one 1024-thread block otherwise —
// concurrently with the rest as 256-thread blocks on `st`; `st` then waits
// for `side`.
template <int OP>
static int launch_skel(SkelArgs a, int nbox, int maxn, int maxm, cudaStream_t st, int nbig = 0,
                       cudaStream_t side = nullptr, cudaEvent_t e0 = nullptr, cudaEvent_t e1 = nullptr) {
  constexpr int W = OpTraits<OP>::kComplex ? 2 : 1;
  const size_t smem = sizeof(double) * ((size_t)2 * maxn + (size_t)maxm * W + 64 + (size_t)a.np * OpTraits<OP>::kDim) +
                      sizeof(int) * (size_t)maxn;
  if (smem > 200 * 1024) return SKF_ERR_UNSUPPORTED;
  if (nbig <= 0 || !side || !a.order) return launch_skel_nt<OP, kSkelThreads>(a, nbox, smem, st);
  if (nbig >= nbox) {
    // every box is big: all of them take the big-box path on `st`
    if constexpr (!OpTraits<OP>::kComplex) return launch_skel_cluster<OP>(a, nbox, maxn, st);
    else return launch_skel_nt<OP, 1024>(a, nbox, smem, st);
  }
  SKF_CUDA_TRY(cudaEventRecord(e0, st));
  SKF_CUDA_TRY(cudaStreamWaitEvent(side, e0, 0));
  int status;
  if constexpr (!OpTraits<OP>::kComplex) status = launch_skel_cluster<OP>(a, nbig, maxn, side);
  else status = launch_skel_nt<OP, 1024>(a, nbig, smem, side);
  SkelArgs rest = a;
  rest.order = a.order + nbig;
  if (status == SKF_OK) status = launch_skel_nt<OP, kSkelThreads>(rest, nbox - nbig, smem, st);
  SKF_CUDA_TRY(cudaEventRecord(e1, side));
  SKF_CUDA_TRY(cudaStreamWaitEvent(st, e1, 0));
  return status;
}

int proxy_rows(int op, int nproxy) {
  const int ndim = (op == SKF_LAPLACE_2D || op == SKF_HELMHOLTZ_2D) ? 2 : 3;
  const bool geom_op = op >= SKF_LAPLACE_DOUBLE_LAYER_3D;
  const int np = (int)(proxy_template(ndim, geom_op, nproxy).size() / ndim);
  return geom_op ? 2 * np : np;
}

struct RandomizedArgs {
  const int32_t* kpred = nullptr;  // DEVICE [nbox], <= 0: full QR
  int oversample = 10;
  int rho = 24;
  uint64_t seed = 0;
  int nchk = 16;
  double sketch_tol = 0.0;
  double resid_tol = 0.0;
  double* resid = nullptr;
  int8_t* status = nullptr;
};

// The ID workspaces come from the device's default memory pool, whose
// default release threshold hands freed memory back at every
// synchronization: the next level then maps its gigabytes again.  The
// builds keep it in the pool instead, and trim_workspace returns it once a
// build is done.
static void keep_pool_memory() {
  int dev = 0;
  cudaMemPool_t pool;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetDefaultMemPool(&pool, dev) != cudaSuccess) return;
  uint64_t thr = UINT64_MAX;
  cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
}

int trim_workspace() {
  int dev = 0;
  cudaMemPool_t pool;
  SKF_CUDA_TRY(cudaGetDevice(&dev));
  SKF_CUDA_TRY(cudaDeviceGetDefaultMemPool(&pool, dev));
  uint64_t thr = 0;
  SKF_CUDA_TRY(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
  SKF_CUDA_TRY(cudaMemPoolTrimTo(pool, 0));
  return SKF_OK;
}

static int skel_boxes_impl(int op, double kappa, int nbox, const int64_t* off, const double* x, const double* geom,
                           const double* centers, double box_length, const double* box_lens, int nproxy, double tol,
                           const RandomizedArgs& ra, int32_t* rank, int32_t* perm, const int64_t* t_off_out,
                           void* t_out, cudaStream_t st) {
  const int ndim = (op == SKF_LAPLACE_2D || op == SKF_HELMHOLTZ_2D) ? 2 : 3;
  const bool geom_op = op >= SKF_LAPLACE_DOUBLE_LAYER_3D;
  const bool cplx = op == SKF_HELMHOLTZ_2D || op == SKF_HELMHOLTZ_3D || op == SKF_HELMHOLTZ_DOUBLE_LAYER_3D ||
                    op == SKF_HELMHOLTZ_ADJOINT_DOUBLE_LAYER_3D;
  const int W = cplx ? 2 : 1;
  keep_pool_memory();
  std::vector<double> tmpl = proxy_template(ndim, geom_op, nproxy);
  const int np = (int)(tmpl.size() / ndim);
  const int mrows = geom_op ? 2 * np : np;
  std::vector<int64_t> hoff(nbox + 1);
  SKF_CUDA_TRY(cudaMemcpyAsync(hoff.data(), off, sizeof(int64_t) * (nbox + 1), cudaMemcpyDeviceToHost, st));
  std::vector<int32_t> hk;
  if (ra.kpred) {
    hk.resize(nbox);
    SKF_CUDA_TRY(cudaMemcpyAsync(hk.data(), ra.kpred, sizeof(int32_t) * nbox, cudaMemcpyDeviceToHost, st));
  }
  SKF_CUDA_TRY(cudaStreamSynchronize(st));
  // the sketch rank of a box is its predicted rank capped at its size (the
  // kernels apply the same cap)
  for (int b = 0; b < (int)hk.size(); ++b) hk[b] = (int32_t)std::min<int64_t>(hk[b], hoff[b + 1] - hoff[b]);
  // A first-round reject retries once with a larger sketch (rank k +
  // max(k / 2, 2 oversample), capped at the box size) when that still fits;
  // hk2 = 0: no retry.
  std::vector<int32_t> hk2(hk.size(), 0);
  for (int b = 0; b < (int)hk.size(); ++b) {
    if (hk[b] <= 0 || !sketch_fits(hk[b] + ra.oversample, mrows)) continue;
    const int64_t n = hoff[b + 1] - hoff[b];
    const int32_t k2 =
        (int32_t)std::min<int64_t>((int64_t)hk[b] + std::max<int64_t>(hk[b] / 2, 2 * ra.oversample), n);
    if (k2 > hk[b] && sketch_fits(k2 + ra.oversample, mrows)) hk2[b] = k2;
  }
  // workspace rows per box: K, plus the (retry's) sketch when the box is randomized
  auto box_rows = [&](int b) -> int64_t {
    if (!ra.kpred || hk[b] <= 0) return mrows;
    const int64_t s = (int64_t)std::max(hk[b], hk2[b]) + ra.oversample;
    return sketch_fits((int64_t)hk[b] + ra.oversample, mrows) ? mrows + s : mrows;  // K and the sketch
  };

  double* dtmpl = nullptr;
  SKF_CUDA_TRY(cudaMallocAsync(&dtmpl, sizeof(double) * tmpl.size(), st));
  SKF_CUDA_TRY(cudaMemcpyAsync(dtmpl, tmpl.data(), sizeof(double) * tmpl.size(), cudaMemcpyHostToDevice, st));
  // sparse sign sketch shared by the launch: sk_rows x rho entries, each a
  // uniform proxy row with a random sign (bit 31)
  int32_t* dtab = nullptr;
  std::vector<int32_t> tab;
  if (ra.kpred) {
    int sk_rows = 1;
    for (int b = 0; b < nbox; ++b)
      if (hk[b] > 0 && sketch_fits(hk[b] + ra.oversample, mrows))
        sk_rows = std::max<int>(sk_rows, std::max(hk[b], hk2[b]) + ra.oversample);
    tab.resize((size_t)sk_rows * ra.rho);
    std::mt19937_64 gen(ra.seed);
    for (auto& e : tab) {
      const uint64_t h = gen();
      const int32_t i = (int32_t)((h >> 1) % (uint64_t)mrows);
      e = (h & 1) ? (int32_t)((uint32_t)i | 0x80000000u) : i;
    }
    SKF_CUDA_TRY(cudaMallocAsync(&dtab, sizeof(int32_t) * tab.size(), st));
    SKF_CUDA_TRY(cudaMemcpyAsync(dtab, tab.data(), sizeof(int32_t) * tab.size(), cudaMemcpyHostToDevice, st));
  }

  // every box reports status 0 and residual -1 unless its randomized ID is
  // tried; the status also drives the second (pivoted-QR) launch
  int8_t* dstat = ra.status;
  int8_t* own_stat = nullptr;
  if (ra.kpred && nbox > 0) {
    if (!dstat) {
      SKF_CUDA_TRY(cudaMallocAsync(&own_stat, (size_t)nbox, st));
      dstat = own_stat;
    }
    SKF_CUDA_TRY(cudaMemsetAsync(dstat, 0, (size_t)nbox, st));
    if (ra.resid) {
      k_fill_f64<<<(nbox + 255) / 256, 256, 0, st>>>(ra.resid, nbox, -1.0);
      SKF_CUDA_TRY(cudaGetLastError());
    }
  }

  int32_t* dk2 = nullptr;  // retry sketch ranks
  if (ra.kpred && nbox > 0) {
    SKF_CUDA_TRY(cudaMallocAsync(&dk2, sizeof(int32_t) * nbox, st));
    SKF_CUDA_TRY(cudaMemcpyAsync(dk2, hk2.data(), sizeof(int32_t) * nbox, cudaMemcpyHostToDevice, st));
  }

  int* dbad = nullptr;  // non-finite proxy entries seen by any block
  SKF_CUDA_TRY(cudaMallocAsync(&dbad, sizeof(int), st));
  SKF_CUDA_TRY(cudaMemsetAsync(dbad, 0, sizeof(int), st));

  // workspace in batches of boxes bounded by a quarter of the free device
  // memory, at most 16 GiB (a level in one batch has one launch tail, not
  // one per batch), at least 1 GiB
  int64_t budget = (int64_t)4 << 30;
  {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess)
      budget = std::max<int64_t>((int64_t)1 << 30, std::min<int64_t>((int64_t)16 << 30, (int64_t)(free_b / 4)));
  }
  int status = SKF_OK;
  cudaStream_t side = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int b0 = 0;
  while (b0 < nbox && status == SKF_OK) {
    std::vector<int64_t> wso;
    int64_t acc = 0;
    int b1 = b0;
    while (b1 < nbox) {
      const int64_t need = box_rows(b1) * (hoff[b1 + 1] - hoff[b1]) * W * (int64_t)sizeof(double);
      if (b1 > b0 && acc + need > budget) break;
      wso.push_back(acc / (int64_t)sizeof(double));
      acc += need;
      ++b1;
    }
    // Boxes of the batch whose randomized ID is tried (sketch well below the
    // proxy matrix); the others take the pivoted-QR ID directly.
    auto sketched = [&](int b) {
      return ra.kpred && hk[b] > 0 && sketch_fits(hk[b] + ra.oversample, mrows);
    };
    // cost ~ rows x n x min(rows, n), rows = the sketch or the proxy matrix
    const std::vector<int32_t>* cost_k = &hk;  // sketch ranks of the launch being ordered
    auto box_cost = [&](int b, bool sketch) {
      const double n = (double)(hoff[b + 1] - hoff[b]);
      const double rows = sketch ? (double)(*cost_k)[b] + ra.oversample : (double)mrows;
      return rows * n * std::min(rows, n);
    };
    double* ws = nullptr;
    int64_t* dwso = nullptr;
    int32_t* dord = nullptr;
    const size_t nb = (size_t)(b1 - b0);
    cudaError_t e = cudaMallocAsync(&ws, std::max<int64_t>(acc, 8), st);
    if (e == cudaSuccess) e = cudaMallocAsync(&dwso, sizeof(int64_t) * wso.size(), st);
    if (e == cudaSuccess) e = cudaMallocAsync(&dord, sizeof(int32_t) * 2 * nb, st);
    if (e != cudaSuccess) {
      set_last_cuda_error(e);
      status = SKF_ERR_OOM;
      if (ws) cudaFreeAsync(ws, st);
      if (dwso) cudaFreeAsync(dwso, st);
      break;
    }
    e = cudaMemcpyAsync(dwso, wso.data(), sizeof(int64_t) * wso.size(), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) {
      set_last_cuda_error(e);
      status = SKF_ERR_CUDA;
    }
    SkelArgs a{};
    a.off = off;
    a.x = x;
    a.geom = geom;
    a.centers = centers;
    a.tmpl = dtmpl;
    a.np = np;
    a.mrows = mrows;
    a.plen = 2.95 * box_length;
    a.box_len = box_lens;
    a.kappa = kappa;
    a.tol = tol;
    a.ws = ws;
    a.ws_off = dwso;
    a.rank = rank;
    a.perm = perm;
    a.t_off_out = t_off_out;
    a.t_out = static_cast<double*>(t_out);
    a.first_box = b0;
    a.sk_tab = dtab;
    a.oversample = ra.oversample;
    a.rho = ra.rho;
    a.seed = ra.seed;
    a.nchk = ra.nchk;
    a.sketch_tol = ra.sketch_tol;
    a.resid_tol = ra.resid_tol;
    a.nonfinite = dbad;
    int maxn_batch = 1;
    for (int b = b0; b < b1; ++b) maxn_batch = std::max<int>(maxn_batch, (int)(hoff[b + 1] - hoff[b]));
    // Launches the boxes `list` (batch-local) longest first; boxes far above
    // an even share of the launch's work get a thread-block cluster (real
    // operators, from twice an even share) or a 1024-thread block on `side`.
    auto launch_list = [&](SkelArgs la, std::vector<int32_t> list, bool sketch, int32_t* dlist,
                           std::vector<int32_t>* clustered = nullptr) -> int {
      if (list.empty()) return SKF_OK;
      std::vector<double> cost(list.size());
      for (size_t i = 0; i < list.size(); ++i) cost[i] = box_cost(b0 + list[i], sketch);
      std::vector<int32_t> idx(list.size());
      for (size_t i = 0; i < idx.size(); ++i) idx[i] = (int32_t)i;
      std::stable_sort(idx.begin(), idx.end(), [&](int32_t p, int32_t q) { return cost[p] > cost[q]; });
      std::vector<int32_t> ord(list.size());
      double total = 0.0;
      for (size_t i = 0; i < idx.size(); ++i) {
        ord[i] = list[idx[i]];
        total += cost[idx[i]];
      }
      // (in a randomized launch the big boxes of real operators take the
      // clustered pivoted-QR ID: 8 SMs on the full matrix beat one block on
      // the sketch)
      int nbig = 0;
      const double big = (W == 1 ? 2.0 : 4.0) * total / (152.0 * 4.0);
      while (nbig < (int)ord.size() && cost[idx[nbig]] > big && hoff[b0 + ord[nbig] + 1] - hoff[b0 + ord[nbig]] >= 192)
        ++nbig;
      if (nbig > 0 && !side) {
        if (cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&ev0, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&ev1, cudaEventDisableTiming) != cudaSuccess)
          nbig = 0;
      }
      if (clustered && W == 1) clustered->assign(ord.begin(), ord.begin() + nbig);
      SKF_CUDA_TRY(cudaMemcpyAsync(dlist, ord.data(), sizeof(int32_t) * ord.size(), cudaMemcpyHostToDevice, st));
      la.order = dlist;
      switch (op) {
#define SKF_CASE(OPID) \
  case OPID: return launch_skel<OPID>(la, (int)ord.size(), maxn_batch, mrows, st, nbig, side, ev0, ev1);
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
    };
    std::vector<int32_t> rnd, full;
    for (int b = b0; b < b1; ++b) (sketched(b) ? rnd : full).push_back(b - b0);
    if (status == SKF_OK && !rnd.empty()) {
      // phase 1: randomized IDs; rejects only report their status
      SkelArgs r = a;
      r.kpred = ra.kpred;
      r.resid = ra.resid;
      r.status = dstat;
      r.defer = 1;
      // (boxes on clusters, real operators, finish their fallback in place)
      std::vector<int32_t> clustered;
      status = launch_list(r, rnd, true, dord, &clustered);
      if (status == SKF_OK) {
        std::vector<int8_t> hs(nb), done(nb, 0);
        for (int32_t lb : clustered) done[lb] = 1;
        cudaError_t ce = cudaMemcpyAsync(hs.data(), dstat + b0, nb, cudaMemcpyDeviceToHost, st);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
        if (ce != cudaSuccess) {
          set_last_cuda_error(ce);
          status = SKF_ERR_CUDA;
        }
        std::vector<int32_t> retry;
        for (int32_t lb : rnd)
          if (hs[lb] % 10 == 2 && !done[lb]) (hk2[b0 + lb] > 0 ? retry : full).push_back(lb);
        if (status == SKF_OK && !retry.empty()) {
          // phase 2: the rejects retry with the larger sketch
          SkelArgs r2 = r;
          r2.kpred = dk2;
          r2.round = 2;
          std::vector<int32_t> clustered2;
          cost_k = &hk2;
          status = launch_list(r2, retry, true, dord + nb, &clustered2);
          cost_k = &hk;
          if (status == SKF_OK) {
            for (int32_t lb : clustered2) done[lb] = 1;
            ce = cudaMemcpyAsync(hs.data(), dstat + b0, nb, cudaMemcpyDeviceToHost, st);
            if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
            if (ce != cudaSuccess) {
              set_last_cuda_error(ce);
              status = SKF_ERR_CUDA;
            }
            for (int32_t lb : retry)
              if (hs[lb] % 10 == 2 && !done[lb]) full.push_back(lb);
          }
        }
      }
    }
    // phase 3: pivoted-QR IDs of the other boxes and of the rejects
    if (status == SKF_OK) status = launch_list(a, full, false, dord + nb);
    cudaFreeAsync(ws, st);
    cudaFreeAsync(dwso, st);
    cudaFreeAsync(dord, st);
    b0 = b1;
  }
  if (status == SKF_OK) {
    int bad = 0;
    cudaError_t ce = cudaMemcpyAsync(&bad, dbad, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce != cudaSuccess) {
      set_last_cuda_error(ce);
      status = SKF_ERR_CUDA;
    } else if (bad) {
      status = SKF_ERR_ID;
    }
  }
  cudaFreeAsync(dbad, st);
  if (dk2) cudaFreeAsync(dk2, st);
  cudaFreeAsync(dtmpl, st);
  if (dtab) cudaFreeAsync(dtab, st);
  if (own_stat) cudaFreeAsync(own_stat, st);
  if (side) {
    cudaStreamDestroy(side);
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
  }
  if (status == SKF_OK) SKF_CUDA_TRY(cudaGetLastError());
  return status;
}

int skel_boxes(int op, double kappa, int nbox, const int64_t* off, const double* x, const double* geom,
               const double* centers, double box_length, const double* box_lens, int nproxy, double tol,
               int32_t* rank, int32_t* perm, const int64_t* t_off_out, void* t_out, cudaStream_t st) {
  RandomizedArgs ra;
  return skel_boxes_impl(op, kappa, nbox, off, x, geom, centers, box_length, box_lens, nproxy, tol, ra, rank, perm,
                         t_off_out, t_out, st);
}

int skel_boxes_randomized(int op, double kappa, int nbox, const int64_t* off, const double* x, const double* geom,
                          const double* centers, double box_length, int nproxy, double tol, const int32_t* kpred,
                          int oversample, int rho, uint64_t seed, int nchk, double sketch_tol, double resid_tol,
                          double* resid, int8_t* status, int32_t* rank, int32_t* perm, const int64_t* t_off_out,
                          void* t_out, cudaStream_t st) {
  RandomizedArgs ra;
  ra.kpred = kpred;
  ra.oversample = oversample;
  ra.rho = rho;
  ra.seed = seed;
  ra.nchk = nchk;
  ra.sketch_tol = sketch_tol;
  ra.resid_tol = resid_tol;
  ra.resid = resid;
  ra.status = status;
  return skel_boxes_impl(op, kappa, nbox, off, x, geom, centers, box_length, nullptr, nproxy, tol, ra, rank, perm,
                         t_off_out, t_out, st);
}

// Same work as skel_boxes, with the proxy template, the per-box workspace
// offsets and the workspaces carved out of a caller-provided device buffer of
// `cap` doubles instead of stream-ordered allocations.  Boxes are processed
// in batches that fit the buffer, in stream order.  Returns SKF_ERR_SCRATCH,
// before any kernel launch or scratch write, when one box's proxy matrix does
// not fit; SKF_ERR_ID when a proxy matrix (a point or normal) is not finite.
int skel_boxes_scratch(int op, double kappa, int nbox, const int64_t* off, const double* x, const double* geom,
                       const double* centers, double box_length, int nproxy, double tol, int32_t* rank,
                       int32_t* perm, const int64_t* t_off_out, void* t_out, double* scratch, int64_t cap,
                       cudaStream_t st) {
  const int ndim = (op == SKF_LAPLACE_2D || op == SKF_HELMHOLTZ_2D) ? 2 : 3;
  const bool geom_op = op >= SKF_LAPLACE_DOUBLE_LAYER_3D;
  const bool cplx = op == SKF_HELMHOLTZ_2D || op == SKF_HELMHOLTZ_3D || op == SKF_HELMHOLTZ_DOUBLE_LAYER_3D ||
                    op == SKF_HELMHOLTZ_ADJOINT_DOUBLE_LAYER_3D;
  const int W = cplx ? 2 : 1;
  std::vector<double> tmpl = proxy_template(ndim, geom_op, nproxy);
  const int np = (int)(tmpl.size() / ndim);
  const int mrows = geom_op ? 2 * np : np;
  constexpr int64_t kMaxBatch = 4096;  // workspace-offset slots
  constexpr int64_t kFlagSlots = 32;   // the non-finite flag (one int in a 256-byte slot)
  const int64_t tsz = ((int64_t)tmpl.size() + 31) / 32 * 32;
  const int64_t wcap = cap - tsz - kMaxBatch - kFlagSlots;
  if (wcap <= 0) return SKF_ERR_SCRATCH;
  std::vector<int64_t> hoff(nbox + 1);
  SKF_CUDA_TRY(cudaMemcpyAsync(hoff.data(), off, sizeof(int64_t) * (nbox + 1), cudaMemcpyDeviceToHost, st));
  SKF_CUDA_TRY(cudaStreamSynchronize(st));
  for (int b = 0; b < nbox; ++b)
    if ((int64_t)mrows * (hoff[b + 1] - hoff[b]) * W > wcap) return SKF_ERR_SCRATCH;

  double* dtmpl = scratch;
  int64_t* dwso = reinterpret_cast<int64_t*>(scratch + tsz);
  int* dbad = reinterpret_cast<int*>(scratch + tsz + kMaxBatch);
  double* ws = scratch + tsz + kMaxBatch + kFlagSlots;
  SKF_CUDA_TRY(cudaMemcpyAsync(dtmpl, tmpl.data(), sizeof(double) * tmpl.size(), cudaMemcpyHostToDevice, st));
  SKF_CUDA_TRY(cudaMemsetAsync(dbad, 0, sizeof(int), st));
  int status = SKF_OK;
  int b0 = 0;
  while (b0 < nbox && status == SKF_OK) {
    std::vector<int64_t> wso;
    int64_t acc = 0;
    int b1 = b0;
    while (b1 < nbox && (int64_t)wso.size() < kMaxBatch) {
      const int64_t need = (int64_t)mrows * (hoff[b1 + 1] - hoff[b1]) * W;
      if (acc + need > wcap) break;
      wso.push_back(acc);
      acc += need;
      ++b1;
    }
    // pageable source: the copy is staged before this call returns, and it is
    // ordered after the previous batch's kernel on the stream
    SKF_CUDA_TRY(cudaMemcpyAsync(dwso, wso.data(), sizeof(int64_t) * wso.size(), cudaMemcpyHostToDevice, st));
    SkelArgs a{};
    a.off = off;
    a.x = x;
    a.geom = geom;
    a.centers = centers;
    a.tmpl = dtmpl;
    a.np = np;
    a.mrows = mrows;
    a.plen = 2.95 * box_length;
    a.kappa = kappa;
    a.tol = tol;
    a.ws = ws;
    a.ws_off = dwso;
    a.rank = rank;
    a.perm = perm;
    a.t_off_out = t_off_out;
    a.t_out = static_cast<double*>(t_out);
    a.first_box = b0;
    a.nonfinite = dbad;
    int maxn_batch = 1;
    for (int b = b0; b < b1; ++b) maxn_batch = std::max<int>(maxn_batch, (int)(hoff[b + 1] - hoff[b]));
    switch (op) {
#define SKF_CASE(OPID) \
  case OPID: status = launch_skel<OPID>(a, b1 - b0, maxn_batch, mrows, st); break;
      SKF_CASE(SKF_LAPLACE_2D)
      SKF_CASE(SKF_LAPLACE_3D)
      SKF_CASE(SKF_HELMHOLTZ_2D)
      SKF_CASE(SKF_HELMHOLTZ_3D)
      SKF_CASE(SKF_LAPLACE_DOUBLE_LAYER_3D)
      SKF_CASE(SKF_LAPLACE_ADJOINT_DOUBLE_LAYER_3D)
      SKF_CASE(SKF_HELMHOLTZ_DOUBLE_LAYER_3D)
      SKF_CASE(SKF_HELMHOLTZ_ADJOINT_DOUBLE_LAYER_3D)
#undef SKF_CASE
      default: status = SKF_ERR_ARG;
    }
    b0 = b1;
  }
  if (status == SKF_OK) {
    int bad = 0;
    SKF_CUDA_TRY(cudaMemcpyAsync(&bad, dbad, sizeof(int), cudaMemcpyDeviceToHost, st));
    SKF_CUDA_TRY(cudaStreamSynchronize(st));
    if (bad) status = SKF_ERR_ID;
  }
  if (status == SKF_OK) SKF_CUDA_TRY(cudaGetLastError());
  return status;
}

}  // namespace skf
