// skf_kernels.cuh — point-kernel evaluation for the eight built-in operators,
// in FP64 (parity path) and FP32 (mixed path).
//
// Kernel formulas follow the reference's dense kernels (skelfmm/util.py:128-377)
// and batched kernels (skelfmm/util_batched.py:240-656):
//   LAPLACE_2D      log r                              (no 1/2pi factor)
//   LAPLACE_3D      1/r                                (no 1/4pi factor)
//   HELMHOLTZ_2D    J0(k r) + i Y0(k r)
//   HELMHOLTZ_3D    exp(i k r) / r
//   LAPLACE_DL      -(1/4pi) (x-y).n_y / r^3           (source normals)
//   LAPLACE_ADL     +(1/4pi) (x-y).n_x / r^3           (target normals)
//   HELMHOLTZ_DL    +(1/4pi) (x-y).n_y e^{ikr}(ikr-1)/r^3
//   HELMHOLTZ_ADL   -(1/4pi) (x-y).n_x e^{ikr}(ikr-1)/r^3
// Every kernel is 0 for coincident points (r == 0), which reproduces the
// reference's zeroed self-interaction diagonal (util_batched.py:154-172) and
// its dense kernels' handling of coincident pairs.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/skf.h"

namespace skf {

constexpr double kInv4Pi = 0.07957747154594767;  // 1/(4 pi)

template <int OP>
struct OpTraits {
  static constexpr bool kComplex = (OP == SKF_HELMHOLTZ_2D || OP == SKF_HELMHOLTZ_3D ||
                                    OP == SKF_HELMHOLTZ_DOUBLE_LAYER_3D ||
                                    OP == SKF_HELMHOLTZ_ADJOINT_DOUBLE_LAYER_3D);
  static constexpr int kDim = (OP == SKF_LAPLACE_2D || OP == SKF_HELMHOLTZ_2D) ? 2 : 3;
  // 0: none, 1: source normals, 2: target normals
  static constexpr int kGeom =
      (OP == SKF_LAPLACE_DOUBLE_LAYER_3D || OP == SKF_HELMHOLTZ_DOUBLE_LAYER_3D)
          ? 1
          : ((OP == SKF_LAPLACE_ADJOINT_DOUBLE_LAYER_3D ||
              OP == SKF_HELMHOLTZ_ADJOINT_DOUBLE_LAYER_3D)
                 ? 2
                 : 0);
};

// ---------------------------------------------------------------- FP32 helpers
__device__ __forceinline__ float rsqrt_approx(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float lg2_approx(float x) {
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
// sin / cos of the phase 2 pi t: t is first reduced to the nearest-integer
// remainder in [-1/2, 1/2] turn (exact in FP32), then the hardware
// sin.approx / cos.approx (absolute error ~5e-7 on [-pi, pi]) take 2 pi f.
__device__ __forceinline__ void sincos_turns(float t, float& s, float& c) {
  const float f = t - rintf(t);
  const float a = f * 6.283185307179586f;
  asm("sin.approx.ftz.f32 %0, %1;" : "=f"(s) : "f"(a));
  asm("cos.approx.ftz.f32 %0, %1;" : "=f"(c) : "f"(a));
}

// ---------------------------------------------------------------- FP64 helpers
// 1/sqrt(x): hardware estimate refined by two Newton-Raphson steps
// y <- y + y*(1 - x*y^2)/2 (quadratic convergence; the second step brings a
// ~2^-22 estimate to the limit of double rounding).
__device__ __forceinline__ double rsqrt_f64(double x) {
  double y;
  asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  double e = fma(-x * y, y, 1.0);
  y = fma(0.5 * y, e, y);
  e = fma(-x * y, y, 1.0);
  y = fma(0.5 * y, e, y);
  return y;
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---------------------------------------------------------------- evaluation
// d = x_target - y_source; gs/gt = source/target normals (3D geometry kernels).
// Output: kr (real part) and ki (imag part, complex kernels only).
// MASK: test r == 0 (needed only where coincident points can meet).
template <int OP, bool MASK = true>
__device__ __forceinline__ void eval_f64(double dx, double dy, double dz, double gx, double gy,
                                         double gz, double kappa, double& kr, double& ki) {
  const double r2 = fma(dx, dx, fma(dy, dy, dz * dz));
  if (MASK && !(r2 > 0.0)) {
    kr = 0.0;
    ki = 0.0;
    return;
  }
  if constexpr (OP == SKF_LAPLACE_2D) {
    kr = 0.5 * log(r2);
    ki = 0.0;
  } else if constexpr (OP == SKF_LAPLACE_3D) {
    kr = rsqrt_f64(r2);
    ki = 0.0;
  } else if constexpr (OP == SKF_HELMHOLTZ_2D) {
    const double r = sqrt(r2);
    kr = j0(kappa * r);
    ki = y0(kappa * r);
  } else if constexpr (OP == SKF_HELMHOLTZ_3D) {
    const double ir = rsqrt_f64(r2);
    const double r = r2 * ir;
    double s, c;
    sincos(kappa * r, &s, &c);
    kr = c * ir;
    ki = s * ir;
  } else {
    const double ir = rsqrt_f64(r2);
    const double ir3 = ir * ir * ir;
    const double rotn = dx * gx + dy * gy + dz * gz;
    if constexpr (OP == SKF_LAPLACE_DOUBLE_LAYER_3D) {
      kr = -kInv4Pi * rotn * ir3;
      ki = 0.0;
    } else if constexpr (OP == SKF_LAPLACE_ADJOINT_DOUBLE_LAYER_3D) {
      kr = kInv4Pi * rotn * ir3;
      ki = 0.0;
    } else {
      const double r = r2 * ir;
      const double kr_ = kappa * r;
      double s, c;
      sincos(kr_, &s, &c);
      // e^{ikr}(ikr - 1) = (c + i s)(-1 + i kr) = (-c - s kr) + i (c kr - s)
      const double fr = (-c - s * kr_) * ir3;
      const double fi = (c * kr_ - s) * ir3;
      const double sg = (OP == SKF_HELMHOLTZ_DOUBLE_LAYER_3D) ? kInv4Pi : -kInv4Pi;
      kr = sg * rotn * fr;
      ki = sg * rotn * fi;
    }
  }
}

// (x - y).n of the double-layer kernels to FP32 rounding of the result.
// For points on a surface |(x - y).n| ~ r^2 while its terms are ~r, so a
// plain FP32 dot product loses ~2^-24 / r relatively.  Here d = dh + dl with
// dh exact (the hi parts of both points lie on one FP32 grid) and
// n = nh + nl (FP32 pair): the products dh*nh are split exactly with FMA
// residuals and summed with TwoSum (the Dot2 scheme of Ogita, Rump & Oishi,
// "Accurate sum and dot product", SIAM J. Sci. Comput. 26, 2005); the cross
// terms dh*nl + dl*nh, ~2^-24 of the products, need only FP32.  The _rn
// intrinsics keep the compiler from contracting the error-free steps.
__device__ __forceinline__ float dot_dn(float dhx, float dhy, float dhz, float dlx, float dly, float dlz,
                                        float nhx, float nhy, float nhz, float nlx, float nly, float nlz) {
  float p = __fmul_rn(dhx, nhx);
  float s = fmaf(dhx, nhx, -p);
  float h = __fmul_rn(dhy, nhy);
  float e = fmaf(dhy, nhy, -h);
  float t = __fadd_rn(p, h);
  float z = __fsub_rn(t, p);
  s = __fadd_rn(s, __fadd_rn(__fadd_rn(__fsub_rn(p, __fsub_rn(t, z)), __fsub_rn(h, z)), e));
  p = t;
  h = __fmul_rn(dhz, nhz);
  e = fmaf(dhz, nhz, -h);
  t = __fadd_rn(p, h);
  z = __fsub_rn(t, p);
  s = __fadd_rn(s, __fadd_rn(__fadd_rn(__fsub_rn(p, __fsub_rn(t, z)), __fsub_rn(h, z)), e));
  p = t;
  s = fmaf(dhx, nlx, s);
  s = fmaf(dhy, nly, s);
  s = fmaf(dhz, nlz, s);
  s = fmaf(dlx, nhx, s);
  s = fmaf(dly, nhy, s);
  s = fmaf(dlz, nhz, s);
  return __fadd_rn(p, s);
}

// FP32 evaluation from an accurate difference vector (see the translation
// kernel: differences are formed from hi/lo split coordinates).  rotn =
// (x - y).n for the double-layer kernels (dot_dn), unused otherwise.
template <int OP, bool MASK = true>
__device__ __forceinline__ void eval_f32(float dx, float dy, float dz, float rotn, float kappa, float& kr,
                                         float& ki) {
  const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
  if constexpr (OP == SKF_LAPLACE_2D) {
    // log r = (ln 2 / 2) * log2(r^2)
    const float v = 0.34657359027997264f * lg2_approx(r2);
    kr = (!MASK || r2 > 0.f) ? v : 0.f;
    ki = 0.f;
  } else if constexpr (OP == SKF_LAPLACE_3D) {
    const float v = rsqrt_approx(r2);
    kr = (!MASK || r2 > 0.f) ? v : 0.f;
    ki = 0.f;
  } else if constexpr (OP == SKF_HELMHOLTZ_2D) {
    if (!MASK || r2 > 0.f) {
      const float r = sqrtf(r2);
      kr = j0f(kappa * r);
      ki = y0f(kappa * r);
    } else {
      kr = 0.f;
      ki = 0.f;
    }
  } else if constexpr (OP == SKF_HELMHOLTZ_3D) {
    if (!MASK || r2 > 0.f) {
      const float ir = rsqrt_approx(r2);
      const float r = r2 * ir;
      float s, c;
      sincos_turns(kappa * 0.15915494309189535f * r, s, c);
      kr = c * ir;
      ki = s * ir;
    } else {
      kr = 0.f;
      ki = 0.f;
    }
  } else {
    if (!MASK || r2 > 0.f) {
      const float ir = rsqrt_approx(r2);
      const float ir3 = ir * ir * ir;
      if constexpr (OP == SKF_LAPLACE_DOUBLE_LAYER_3D) {
        kr = -float(kInv4Pi) * rotn * ir3;
        ki = 0.f;
      } else if constexpr (OP == SKF_LAPLACE_ADJOINT_DOUBLE_LAYER_3D) {
        kr = float(kInv4Pi) * rotn * ir3;
        ki = 0.f;
      } else {
        const float r = r2 * ir;
        const float kr_ = kappa * r;
        float s, c;
        sincos_turns(kappa * 0.15915494309189535f * r, s, c);
        const float fr = (-c - s * kr_) * ir3;
        const float fi = (c * kr_ - s) * ir3;
        const float sg = (OP == SKF_HELMHOLTZ_DOUBLE_LAYER_3D) ? float(kInv4Pi) : -float(kInv4Pi);
        kr = sg * rotn * fr;
        ki = sg * rotn * fi;
      }
    } else {
      kr = 0.f;
      ki = 0.f;
    }
  }
}

}  // namespace skf
