// trax_math.h -- single-precision math shared, byte for byte, by the CPU
// oracle (g++) and the sm_103a kernels (nvcc).
//
// The triplet-seeding cuts compare FP32 quantities built from atan2, acos,
// atan and asinh against cut values.  For the pair, candidate and triplet
// sets of the GPU path to equal the oracle's bit for bit, both must evaluate
// every one of those functions with the same sequence of IEEE-754
// round-to-nearest operations.  Vendor libraries (glibc libm, CUDA's libdevice)
// differ from each other in the last bits, so this header provides its own
// implementations built only from + - * / sqrt, comparisons and integer bit
// manipulation, evaluated without contraction, and the polynomial steps as
// explicit fused multiply-adds (fmaf: one rounding, IEEE-754's fusedMultiplyAdd,
// so the same bits on the CPU and the GPU):
//   * nvcc: -fmad=false -prec-div=true -prec-sqrt=true -ftz=false
//   * g++ : -ffp-contract=off (and no -ffast-math)
//
// Methods (published, coefficients fitted by fit_math_coeffs.py):
//   atan   : three-interval reduction (|x| > tan(3pi/8): -1/x + pi/2,
//            |x| > tan(pi/8): (x-1)/(x+1) + pi/4), odd polynomial on
//            |t| <= tan(pi/8) -- the reduction used by Cephes' atanf
//            (S. L. Moshier, "Methods and Programs for Mathematical
//            Functions", 1989).
//   atan2  : quadrant folding onto atan of a ratio in [0, 1] with C99
//            Annex F special cases.
//   acos   : acos(x) = pi/2 - asin(x) for |x| <= 1/2, otherwise the half-angle
//            identity acos(x) = 2 asin(sqrt((1-x)/2)) (and pi minus it for x<0).
//   log    : x = 2^k m, m in [sqrt(1/2), sqrt(2)), log m = 2 atanh(s),
//            s = (m-1)/(m+1).
//   asinh  : odd polynomial for |x| <= 1, log(|x| + sqrt(x^2+1)) above,
//            log(2|x|) for |x| > 2^12.
// Multi-part constants (pi = PI_HI + PI_LO) keep the final additions within
// about one ulp.  Accuracy is tested against float64 (tests/test_math.py) and
// against CUDA's own atan2f/acosf/atanf/asinhf on the GPU, where the device
// build must also give the CPU build's bits (tests/test_gpu_math.py).
//
// The header also restates, with fixed semantics, the OpenCL C built-ins the
// reference kernels use (sign, max, normalize, cross, float->integer
// conversion), because their vendor-defined corner cases decide bits.
#pragma once

#include <stdint.h>
#include <string.h>

#include <cmath>

#include "trax_math_coeffs.h"

#if defined(__CUDACC__)
#define TRAX_HD __host__ __device__ __forceinline__
#else
#define TRAX_HD inline
#endif

namespace trax {

// ---------------------------------------------------------------- constants
// float nearest to pi (OpenCL M_PI_F) and the remainder pi - PI_HI.
#define TRAX_PI_F 3.14159274101257324e+00f
#define TRAX_PI_LO (-8.74227765734758577e-08f)
#define TRAX_PIO2_HI 1.57079637050628662e+00f
#define TRAX_PIO2_LO (-4.37113882867379289e-08f)
#define TRAX_PIO4_HI 7.85398185253143311e-01f
#define TRAX_PIO4_LO (-2.18556941433689644e-08f)
#define TRAX_LN2_HI 6.93145752e-01f      // 0x3f317200: 15 significant bits, k*LN2_HI exact
#define TRAX_LN2_LO 1.42860682030941723e-06f  // ln 2 - LN2_HI
#define TRAX_TAN_3PI_8 2.41421356237309504880f
#define TRAX_TAN_PI_8 0.41421356237309504880f

// ---------------------------------------------------------------- bit casts
TRAX_HD uint32_t f2bits(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(x);
#else
  uint32_t u;
  memcpy(&u, &x, sizeof(u));
  return u;
#endif
}

TRAX_HD float bits2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float x;
  memcpy(&x, &u, sizeof(x));
  return x;
#endif
}

TRAX_HD bool is_nan(float x) { return (f2bits(x) & 0x7fffffffu) > 0x7f800000u; }
TRAX_HD bool is_inf(float x) { return (f2bits(x) & 0x7fffffffu) == 0x7f800000u; }
TRAX_HD bool sign_bit(float x) { return (f2bits(x) >> 31) != 0u; }
TRAX_HD float fabs_(float x) { return bits2f(f2bits(x) & 0x7fffffffu); }
TRAX_HD float copysign_(float mag, float sgn) {
  return bits2f((f2bits(mag) & 0x7fffffffu) | (f2bits(sgn) & 0x80000000u));
}

// IEEE correctly rounded square root and floor (exact on both sides).
TRAX_HD float sqrt_(float x) {
#if defined(__CUDA_ARCH__)
  return __fsqrt_rn(x);
#else
  return __builtin_sqrtf(x);
#endif
}

TRAX_HD float floor_(float x) {
#if defined(__CUDA_ARCH__)
  return floorf(x);
#else
  return __builtin_floorf(x);
#endif
}

// IEEE correctly rounded division (explicit on the device so that the result
// does not depend on -prec-div).
TRAX_HD float div_(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fdiv_rn(a, b);
#else
  return a / b;
#endif
}

// -------------------------------------------------- float -> integer casts
// C/C++ leave out-of-range and NaN conversions undefined and OpenCL leaves
// them implementation-defined.  Both sides use this saturating definition:
// truncate toward zero, NaN -> 0, clamp to the destination range.
// On the device this is one conversion instruction: PTX's cvt.rzi from
// f32 to an integer type truncates, clamps to the destination range and
// turns NaN into 0.  tests/test_gpu_math.py holds the two builds equal.
TRAX_HD uint32_t f2u_sat(float x) {
#if defined(__CUDA_ARCH__)
  return __float2uint_rz(x);
#else
  if (!(x > -1.0f)) return 0u;                  // NaN, -inf and x <= -1
  if (x >= 4294967296.0f) return 0xffffffffu;
  if (x < 1.0f) return 0u;                       // (-1, 1) truncates to 0
  return (uint32_t)x;
#endif
}

TRAX_HD int32_t f2i_sat(float x) {
#if defined(__CUDA_ARCH__)
  return __float2int_rz(x);
#else
  if (is_nan(x)) return 0;
  if (x >= 2147483648.0f) return 2147483647;
  if (x <= -2147483648.0f) return (int32_t)(-2147483647 - 1);
  return (int32_t)x;
#endif
}

// ------------------------------------------------------ OpenCL restatements
// sign(x): 1 for x > 0, -1 for x < 0, x itself for +-0, 0 for NaN.
TRAX_HD float cl_sign(float x) {
  if (x > 0.0f) return 1.0f;
  if (x < 0.0f) return -1.0f;
  if (is_nan(x)) return 0.0f;
  return x;
}

// max(x, y) for floats: y if x < y, otherwise x.
TRAX_HD float cl_max(float x, float y) { return (x < y) ? y : x; }

// ------------------------------------------------------ polynomial kernels
// P(u) by Horner, one rounding per step: p = fma(p, u, c[k]).
template <int N>
TRAX_HD float horner(const float (&c)[N], float u) {
  float p = c[N - 1];
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
  for (int k = N - 2; k >= 0; --k) p = fmaf(p, u, c[k]);
  return p;
}

// t + t^3 P(t^2)
template <int N>
TRAX_HD float odd_series(const float (&c)[N], float t) {
  float u = t * t;
  float p = horner(c, u);
  float t3 = t * u;
  return t + t3 * p;
}

TRAX_HD float atan_kernel(float t) {  // |t| <= tan(pi/8)
  const float c[TRAX_ATAN_NCOEF] = TRAX_ATAN_COEFS;
  return odd_series(c, t);
}

TRAX_HD float asin_kernel(float t) {  // |t| <= 1/2
  const float c[TRAX_ASIN_NCOEF] = TRAX_ASIN_COEFS;
  return odd_series(c, t);
}

TRAX_HD float atanh_kernel(float t) {  // |t| <= (sqrt2-1)/(sqrt2+1)
  const float c[TRAX_ATANH_NCOEF] = TRAX_ATANH_COEFS;
  return odd_series(c, t);
}

TRAX_HD float asinh_kernel(float t) {  // |t| <= 1
  const float c[TRAX_ASINH_NCOEF] = TRAX_ASINH_COEFS;
  return odd_series(c, t);
}

// ------------------------------------------------------------------- atan
// atan(a) for a >= 0 (a may be +inf).
TRAX_HD float atan_pos(float a) {
  if (a > TRAX_TAN_3PI_8) {
    // pi/2 - atan(1/a)
    float t = div_(-1.0f, a);
    return TRAX_PIO2_HI + (atan_kernel(t) + TRAX_PIO2_LO);
  }
  if (a > TRAX_TAN_PI_8) {
    float t = div_(a - 1.0f, a + 1.0f);
    return TRAX_PIO4_HI + (atan_kernel(t) + TRAX_PIO4_LO);
  }
  return atan_kernel(a);
}

// atan_pos without branches, for callers whose neighbouring lanes fall in
// different intervals (atan2 of arbitrary directions): the interval selects
// the operands of one division and the constants around one polynomial.
// Every lane performs the operations of atan_pos above (a / 1 == a), so the
// result is the same.
TRAX_HD float atan_pos_select(float a) {
  const bool big = a > TRAX_TAN_3PI_8;
  const bool mid = !big && a > TRAX_TAN_PI_8;
  const float t = div_(big ? -1.0f : (mid ? a - 1.0f : a), big ? a : (mid ? a + 1.0f : 1.0f));
  const float p = atan_kernel(t);
  const float hi = big ? TRAX_PIO2_HI : TRAX_PIO4_HI;
  const float lo = big ? TRAX_PIO2_LO : TRAX_PIO4_LO;
  return (big || mid) ? hi + (p + lo) : p;
}

TRAX_HD float atan_(float x) {
  if (is_nan(x)) return x;
  float r = atan_pos(fabs_(x));
  return copysign_(r, x);
}

// ------------------------------------------------------------------ atan2
TRAX_HD float atan2_(float y, float x) {
  if (is_nan(x) || is_nan(y)) return x + y;
  float ax = fabs_(x), ay = fabs_(y);
  float r;
  if (ay == 0.0f) {
    // +-0 for x > 0 or x == +0, +-pi for x < 0 or x == -0
    r = sign_bit(x) ? TRAX_PI_F : 0.0f;
    return copysign_(r, y);
  }
  if (is_inf(ax)) {
    if (is_inf(ay)) {
      r = sign_bit(x) ? (3.0f * TRAX_PIO4_HI) : TRAX_PIO4_HI;
    } else {
      r = sign_bit(x) ? TRAX_PI_F : 0.0f;
    }
    return copysign_(r, y);
  }
  if (is_inf(ay) || ax == 0.0f) {
    return copysign_(TRAX_PIO2_HI, y);
  }
  // [0, pi/4] from atan(ay / ax), (pi/4, pi/2) as pi/2 - atan(ax / ay): one
  // division and one atan_pos_select for either half
  const bool lower = ay <= ax;
  const float rp = atan_pos_select(div_(lower ? ay : ax, lower ? ax : ay));
  r = lower ? rp : TRAX_PIO2_HI - (rp - TRAX_PIO2_LO);
  if (sign_bit(x)) {
    r = TRAX_PI_F - (r - TRAX_PI_LO);
  }
  return copysign_(r, y);
}

// ------------------------------------------------------------------- acos
TRAX_HD float acos_(float x) {
  if (is_nan(x)) return x;
  float ax = fabs_(x);
  if (ax > 1.0f) return bits2f(0x7fc00000u);
  if (ax <= 0.5f) {
    // pi/2 - asin(x) = (PIO2_HI - x) - (x^3 P(x^2) - PIO2_LO)
    float u = x * x;
    const float c[TRAX_ASIN_NCOEF] = TRAX_ASIN_COEFS;
    float p = horner(c, u);
    float x3p = (x * u) * p;
    return (TRAX_PIO2_HI - x) - (x3p - TRAX_PIO2_LO);
  }
  if (x > 0.0f) {
    float z = (1.0f - x) * 0.5f;  // exact
    float s = sqrt_(z);
    return 2.0f * asin_kernel(s);
  }
  float z = (1.0f + x) * 0.5f;  // exact
  float s = sqrt_(z);
  float a2 = 2.0f * asin_kernel(s);
  return TRAX_PI_F - (a2 - TRAX_PI_LO);
}

// -------------------------------------------------------------------- log
// Natural logarithm for finite x > 0 (x <= 0 gives -inf/NaN, +inf gives +inf).
TRAX_HD float log_(float x) {
  if (is_nan(x)) return x;
  if (x < 0.0f) return bits2f(0x7fc00000u);
  if (x == 0.0f) return bits2f(0xff800000u);
  if (is_inf(x)) return x;
  uint32_t b = f2bits(x);
  int32_t k = 0;
  if (b < 0x00800000u) {  // subnormal: scale by 2^25 (exact)
    x = x * 33554432.0f;
    b = f2bits(x);
    k = -25;
  }
  k += (int32_t)(b >> 23) - 127;
  float m = bits2f((b & 0x007fffffu) | 0x3f800000u);  // [1, 2)
  if (m > 1.41421356237309504880f) {
    m = m * 0.5f;  // exact
    k += 1;
  }
  float s = div_(m - 1.0f, m + 1.0f);  // m - 1 exact (Sterbenz)
  float lm = 2.0f * atanh_kernel(s);   // log m
  float kf = (float)k;
  return kf * TRAX_LN2_HI + (lm + kf * TRAX_LN2_LO);
}

// ------------------------------------------------------------------ asinh
TRAX_HD float asinh_(float x) {
  if (is_nan(x) || is_inf(x)) return x;
  float a = fabs_(x);
  float r;
  if (a < 2.44140625e-04f) {  // 2^-12: asinh(x) = x to within 2^-25 relative
    return x;
  } else if (a <= 1.0f) {
    r = asinh_kernel(a);
  } else if (a > 4096.0f) {
    r = log_(a) + 6.93147180559945309e-01f;
  } else {
    r = log_(a + sqrt_(a * a + 1.0f));
  }
  return copysign_(r, x);
}

// ------------------------------------------------------ vector built-ins
struct f3 {
  float x, y, z;
};

TRAX_HD f3 make_f3(float x, float y, float z) {
  f3 r;
  r.x = x;
  r.y = y;
  r.z = z;
  return r;
}

TRAX_HD f3 sub3(f3 a, f3 b) { return make_f3(a.x - b.x, a.y - b.y, a.z - b.z); }

// dot(a, b) = (a.x b.x + a.y b.y) + a.z b.z
TRAX_HD float dot3(f3 a, f3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }

TRAX_HD f3 cross3(f3 a, f3 b) {
  return make_f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// normalize(v) = v / sqrt(dot(v, v)), component by component.
TRAX_HD f3 normalize3(f3 v) {
  float l = sqrt_(dot3(v, v));
  return make_f3(div_(v.x, l), div_(v.y, l), div_(v.z, l));
}

// 2-component normalize: v / sqrt(v.x v.x + v.y v.y)
TRAX_HD void normalize2(float& vx, float& vy) {
  float l = sqrt_(vx * vx + vy * vy);
  vx = div_(vx, l);
  vy = div_(vy, l);
}

// ------------------------------------------- the dphi cut away from its edge
// The filter's dphi cut (TripletThetaPhiFilter.h:118-128) compares the
// wrapped difference of atan2(v) and atan2(u), u = B - A and v = C - B in the
// transverse plane, with dPhiCut.  Away from the cut the answer follows from
// the cross and dot products of u and v alone:
// - the evaluated difference is within 2.1e-6 rad of the true angle between
//   u and v: atan2_ is within 3 ulp of each direction (7.2e-7 rad below pi),
//   the subtraction and the +-2 pi_f wrap round by 2.4e-7 rad each, and
//   pi_f is 8.7e-8 from pi;
// - the FP32 cross and dot products, a difference and a sum of two rounded
//   products, are within 2^-23 |u| |v| of the exact ones, which for angles up
//   to 1 rad puts the angle they give within 6e-7 rad of the true one, as
//   long as |u| |v| stays far from the under- and overflow limits.
// With a margin of TRAX_DPHI_MARGIN rad on both sides of the cut,
// cross <= dot tan(cut - margin) means the cut passes and
// cross >= dot tan(cut + margin) means it fails.  Candidates in between,
// degenerate or non-finite vectors, and cuts outside [0, 1] rad (whose
// tanHi is infinite) are left to the atan2 evaluation.
// Returns 1 (passes), 0 (fails) or -1 (undecided).
#define TRAX_DPHI_MARGIN 1e-4

TRAX_HD int dphi_decide(float tanLo, float tanHi, float ux, float uy, float vx, float vy) {
  if (!(tanHi < bits2f(0x7f800000u))) return -1;
  const float nm = (fabs_(ux) + fabs_(uy)) * (fabs_(vx) + fabs_(vy));
  if (!(nm >= 1e-30f && nm <= 1e30f)) return -1;
  const float cr = fabs_(ux * vy - uy * vx), dt = ux * vx + uy * vy;
  if (dt <= 0.0f) return 0;  // at least pi/2 - 6e-7 rad apart
  if (cr <= dt * tanLo) return 1;
  if (cr >= dt * tanHi) return 0;
  return -1;
}

// tan(cut -+ margin) of a dphi cut, or (-1, inf) for a cut outside [0, 1] rad
// (host side; the kernels read the pair from the configuration)
inline void dphi_tan_bounds(float cut, float& tanLo, float& tanHi) {
  if (cut >= 0.0f && cut <= 1.0f) {
    tanLo = (float)std::tan((double)cut - TRAX_DPHI_MARGIN);
    tanHi = (float)std::tan((double)cut + TRAX_DPHI_MARGIN);
  } else {
    tanLo = -1.0f;
    tanHi = bits2f(0x7f800000u);
  }
}

}  // namespace trax
