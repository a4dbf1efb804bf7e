// k_fit.cu -- differentiable FP32 triplet circle/helix fit with a
// hand-written adjoint, for the alignment of the detector layers.
//
// No counterpart in the reference.  The per-triplet geometry follows its
// fitters: the circle through three points (TrackletCircleFitter.h:32-97,
// FastCircle.h:41-118) and a straight line in the (arc length, z) plane
// (FastLine.h:15-42).  Per triplet, with hits corrected by their layer's
// shifts (dr, dz, dphi):
//   circle through the three points: centre C, radius R (curvature 1/R)
//   d0  = |C| - R, the signed transverse impact parameter
//   s_i = 2 R asin(r_i / 2R), r_i = |P_i| = r + dr: arc length from the beam
//         line (exact for a helix through it; the part of a nonzero d0 that
//         is linear in s is absorbed by the line fit)
//   least-squares line z = z0 + cot(theta) s through (s_i, z_i)
//   chi2 = d0^2 / sigma_tip^2 + sum_i e_i^2 / sigma_z^2
// Everything per triplet is FP32; the sums over triplets are FP64, each in a
// fixed order (per-thread, then per-block, then one block over the blocks).
//
// Precision: the three points enter relative to the first one, and the
// alignment enters as small corrections added to those differences, so that
// the circle of a nearly straight triplet is not computed from rounded
// absolute coordinates.  The arc lengths depend on a hit through its radius
// only, and the adjoint carries that dependence as a radial derivative: a
// rotation changes no radius, so the z residuals reach dphi only through the
// circle, and the tangential projection of a large, nearly radial Cartesian
// gradient (which loses the small dphi part to rounding) never happens.  The
// asin of the arc lengths and of their R derivative are Taylor series below
// r / 2R = 1/2 (the correction to s = r is then summed on its own), and the
// line fit takes the raw coordinates and the shifts apart (see below).  The line
// fit's (z0, cot theta) are least-squares optimal, so the adjoint moves chi2
// with z_i and s_i at fixed line parameters (their own gradient terms
// vanish).
#include "trax_kernels.h"

namespace trax {

namespace {

constexpr int FIT_THREADS = 256;

// correction of one hit on layer l: (dX, dY) = (X - x, Y - y)
struct Corr {
  float r, f, xr, yr, dX, dY;
};

__device__ __forceinline__ Corr correct(const FitConfig& c, uint32_t l, float x, float y) {
  Corr k;
  k.r = sqrtf(x * x + y * y);
  const float sn = c.sn[l], cm1 = c.cm1[l];
  const float rx = x * cm1 - y * sn;  // rotated minus original
  const float ry = x * sn + y * cm1;
  k.xr = x + rx;
  k.yr = y + ry;
  const float fr = c.dr[l] / k.r;  // f - 1
  k.f = 1.0f + fr;
  k.dX = rx + fr * k.xr;
  k.dY = ry + fr * k.yr;
  return k;
}

struct FitState {
  float X1, Y1, Z[3];
  float u[3], v[3];  // P_i - P_1 (u[0] = v[0] = 0)
  float q2, q3, D, a, b, R, Cx, Cy, Cn, num, d0;
  float rho[3], sq[3], ds[3], dsdR[3];  // corrected radius, sqrt(1 - x^2), s_i - mean s, d s / d R
  float t, z0, e[3];
};

// Maclaurin coefficients: asin(x) / x - 1 = sum_k A_k x^(2k), A_k = C(2k, k) / (4^k (2k + 1));
// asin(x) - x / sqrt(1 - x^2) = -sum_k B_k x^(2k+1), B_k = C(2k, k) / 4^k * 2k / (2k + 1).
// Twelve terms reach 2e-9 at x = 1/2.
__device__ __constant__ float kAsinA[12] = {1.666666667e-01f, 7.500000000e-02f, 4.464285714e-02f, 3.038194444e-02f,
                                            2.237215909e-02f, 1.735276442e-02f, 1.396484375e-02f, 1.155180090e-02f,
                                            9.761609529e-03f, 8.390335810e-03f, 7.312525874e-03f, 6.447210312e-03f};
__device__ __constant__ float kAsinB[12] = {3.333333333e-01f, 3.000000000e-01f, 2.678571429e-01f, 2.430555556e-01f,
                                            2.237215909e-01f, 2.082331731e-01f, 1.955078125e-01f, 1.848288143e-01f,
                                            1.757089715e-01f, 1.678067162e-01f, 1.608755692e-01f, 1.547330475e-01f};

// a + b = s + err exactly (Knuth's two-sum; no fused operations)
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& err) {
  const float t = a + b;
  const float bb = t - a;
  err = (a - (t - bb)) + (b - bb);
  s = t;
}

// arc length s = 2R asin(r / 2R) as r + c (c returned; small next to r) and
// ds/dR = 2 asin(x) - 2x / sqrt(1 - x^2), x = r / 2R
__device__ __forceinline__ void arc_length(float r, float R, float& c, float& dsdR, float& sq) {
  const float x = fminf(r / (2.0f * R), 1.0f);
  const float x2 = x * x;
  sq = sqrtf(fmaxf(1.0f - x2, 1e-30f));
  if (x <= 0.5f) {
    float pa = kAsinA[11], pb = kAsinB[11];
#pragma unroll
    for (int k = 10; k >= 0; --k) {
      pa = pa * x2 + kAsinA[k];
      pb = pb * x2 + kAsinB[k];
    }
    c = r * (x2 * pa);             // s = r (1 + x^2 P(x^2))
    dsdR = -2.0f * x * (x2 * pb);  // -2 x^3 Q(x^2)
  } else {
    const float as = asinf(x);
    c = 2.0f * R * as - r;
    dsdR = 2.0f * as - 2.0f * x / sq;
  }
}

// forward of one triplet; false when the fit is not finite
__device__ __forceinline__ bool fit_forward(const FitConfig& c, uint32_t lt, const float4 h[3], Corr k[3],
                                            FitState& f) {
  for (int i = 0; i < 3; ++i) k[i] = correct(c, c.layer[i][lt], h[i].x, h[i].y);
  f.X1 = h[0].x + k[0].dX;
  f.Y1 = h[0].y + k[0].dY;
  f.u[0] = f.v[0] = 0.0f;
  // the chords P_i - P_1 as unevaluated sums hi + lo: the raw difference
  // exactly (two_sum), the alignment correction added to the low part
  float ul[3], vl[3];
  ul[0] = vl[0] = 0.0f;
  for (int i = 1; i < 3; ++i) {
    two_sum(h[i].x, -h[0].x, f.u[i], ul[i]);
    two_sum(f.u[i], ul[i] + (k[i].dX - k[0].dX), f.u[i], ul[i]);
    two_sum(h[i].y, -h[0].y, f.v[i], vl[i]);
    two_sum(f.v[i], vl[i] + (k[i].dY - k[0].dY), f.v[i], vl[i]);
  }
  for (int i = 0; i < 3; ++i) f.Z[i] = h[i].z + c.dz[c.layer[i][lt]];
  const float u2 = f.u[1], v2 = f.v[1], u3 = f.u[2], v3 = f.v[2];
  f.q2 = u2 * u2 + v2 * v2;
  f.q3 = u3 * u3 + v3 * v3;
  // D = 2 (u2 v3 - u3 v2): for a nearly straight triplet the two products
  // almost cancel (by about the chord length over 2R), so D takes the exact
  // errors of both products (FMA) and the chords' low parts; the curvature
  // then stays within about 1e-6 of FP64
  const float p23 = u2 * v3, p32 = u3 * v2;
  const float e23 = __fmaf_rn(u2, v3, -p23), e32 = __fmaf_rn(u3, v2, -p32);
  const float corr = (e23 - e32) + ((u2 * vl[2] + ul[1] * v3) - (u3 * vl[1] + ul[2] * v2));
  f.D = 2.0f * ((p23 - p32) + corr);
  f.a = (v3 * f.q2 - v2 * f.q3) / f.D;
  f.b = (u2 * f.q3 - u3 * f.q2) / f.D;
  f.R = sqrtf(f.a * f.a + f.b * f.b);
  f.Cx = f.X1 + f.a;
  f.Cy = f.Y1 + f.b;
  f.Cn = sqrtf(f.Cx * f.Cx + f.Cy * f.Cy);
  f.num = f.X1 * f.X1 + f.Y1 * f.Y1 + 2.0f * (f.X1 * f.a + f.Y1 * f.b);
  f.d0 = f.num / (f.Cn + f.R);
  // Line fit in (s, z) relative to the first hit.  Arc lengths are r + c,
  // the raw radii kept apart from the shifts and the small arc correction,
  // and z is the raw z plus the shift; the raw and the shift parts go
  // through the (linear) line fit separately, so that no shift is rounded
  // into a large coordinate.
  float cc[3];
  for (int i = 0; i < 3; ++i) {
    f.rho[i] = k[i].r + c.dr[c.layer[i][lt]];  // |P_i|: a rotation keeps the radius
    arc_length(f.rho[i], f.R, cc[i], f.dsdR[i], f.sq[i]);
  }
  float sr[3], zr[3], zc[3];
  sr[0] = zr[0] = zc[0] = 0.0f;
  const float dr0 = c.dr[c.layer[0][lt]], dz0 = c.dz[c.layer[0][lt]];
  for (int i = 1; i < 3; ++i) {
    sr[i] = (k[i].r - k[0].r) + ((c.dr[c.layer[i][lt]] - dr0) + (cc[i] - cc[0]));
    zr[i] = h[i].z - h[0].z;
    zc[i] = c.dz[c.layer[i][lt]] - dz0;
  }
  const float sb = (sr[1] + sr[2]) * (1.0f / 3.0f);
  const float zbr = (zr[1] + zr[2]) * (1.0f / 3.0f);
  const float zbc = (zc[1] + zc[2]) * (1.0f / 3.0f);
  float Sss = 0.0f, Szr = 0.0f, Szc = 0.0f;
  for (int i = 0; i < 3; ++i) {
    f.ds[i] = sr[i] - sb;
    Sss += f.ds[i] * f.ds[i];
    Szr += f.ds[i] * (zr[i] - zbr);
    Szc += f.ds[i] * (zc[i] - zbc);
  }
  const float tr = Szr / Sss, tc = Szc / Sss;
  f.t = tr + tc;
  for (int i = 0; i < 3; ++i) f.e[i] = ((zr[i] - zbr) - tr * f.ds[i]) + ((zc[i] - zbc) - tc * f.ds[i]);
  // z at s = 0: the first hit's z, minus the line's rise from s = 0 to s_1
  f.z0 = f.Z[0] + ((zbr + zbc) - f.t * sb) - f.t * (f.rho[0] + cc[0]);
  // usable: finite, the hits well inside the circle's reach (r < 0.9 * 2R, so
  // that the arc length and its derivatives stay smooth), three distinct
  // directions
  const bool inside = f.rho[0] < 1.8f * f.R && f.rho[1] < 1.8f * f.R && f.rho[2] < 1.8f * f.R;
  const bool bent = fabsf(f.D) > 1e-7f * sqrtf(f.q2 * f.q3);
  return isfinite(f.d0) && isfinite(f.t) && isfinite(f.e[0]) && isfinite(f.e[1]) && isfinite(f.e[2]) &&
         isfinite(f.R) && inside && bent;
}

__device__ __forceinline__ float fit_chi2(const FitConfig& c, uint32_t lt, const FitState& f) {
  return c.wTip[lt] * f.d0 * f.d0 + c.wZ * (f.e[0] * f.e[0] + f.e[1] * f.e[1] + f.e[2] * f.e[2]);
}

// reverse pass from d(.)/d d0 = seedD0 and d(.)/d e_i = seedE[i] (line
// parameters at their least-squares optimum) to the corrected hits: the
// Cartesian part d(.)/d(X_i, Y_i) through the circle, the radial part
// d(.)/d r_i through the arc lengths, and d(.)/d Z_i
__device__ __forceinline__ void fit_adjoint(const FitState& f, float seedD0, const float seedE[3], float gX[3],
                                            float gY[3], float gR[3], float gZ[3]) {
  float g_R = 0.0f;
  for (int i = 0; i < 3; ++i) {
    gZ[i] = seedE[i];
    const float g_s = -f.t * seedE[i];
    gR[i] = g_s / f.sq[i];  // ds / dr = 1 / sqrt(1 - x^2)
    g_R += g_s * f.dsdR[i];
  }
  const float g_d0 = seedD0;
  // d0 = num / (Cn + R)
  const float den = f.Cn + f.R;
  const float g_num = g_d0 / den;
  const float g_Cn = -g_d0 * f.d0 / den;
  g_R -= g_d0 * f.d0 / den;
  // num = X1^2 + Y1^2 + 2 (X1 a + Y1 b)
  float g_X1 = g_num * 2.0f * (f.X1 + f.a);
  float g_Y1 = g_num * 2.0f * (f.Y1 + f.b);
  float g_a = g_num * 2.0f * f.X1, g_b = g_num * 2.0f * f.Y1;
  // Cn = |C|, C = P1 + (a, b)
  const float g_Cx = g_Cn * f.Cx / f.Cn;
  const float g_Cy = g_Cn * f.Cy / f.Cn;
  g_X1 += g_Cx;
  g_Y1 += g_Cy;
  g_a += g_Cx;
  g_b += g_Cy;
  // R = |(a, b)|
  g_a += g_R * f.a / f.R;
  g_b += g_R * f.b / f.R;
  // a = (v3 q2 - v2 q3) / D, b = (u2 q3 - u3 q2) / D, D = 2 (u2 v3 - u3 v2)
  const float u2 = f.u[1], v2 = f.v[1], u3 = f.u[2], v3 = f.v[2];
  const float iD = 1.0f / f.D;
  const float g_D = -(g_a * f.a + g_b * f.b) * iD;
  const float g_q2 = (g_a * v3 - g_b * u3) * iD;
  const float g_q3 = (-g_a * v2 + g_b * u2) * iD;
  const float g_v3 = g_a * f.q2 * iD + 2.0f * g_D * u2 + 2.0f * v3 * g_q3;
  const float g_v2 = -g_a * f.q3 * iD - 2.0f * g_D * u3 + 2.0f * v2 * g_q2;
  const float g_u2 = g_b * f.q3 * iD + 2.0f * g_D * v3 + 2.0f * u2 * g_q2;
  const float g_u3 = -g_b * f.q2 * iD - 2.0f * g_D * v2 + 2.0f * u3 * g_q3;
  // u_i = X_i - X_1
  gX[1] = g_u2;
  gY[1] = g_v2;
  gX[2] = g_u3;
  gY[2] = g_v3;
  gX[0] = g_X1 - g_u2 - g_u3;
  gY[0] = g_Y1 - g_v2 - g_v3;
}

__device__ __forceinline__ uint32_t fit_seg(const DevConfig& cfg, DevHits hits, uint32_t h1) {
  return hits.evt[h1] * cfg.nLT + (hits.layer[h1] - 1);
}

__global__ void fit_select_kernel(FitConfig fc, DevConfig cfg, DevHits hits, TripletView t, uint32_t nT,
                                  int truthOnly, uint32_t* ok, uint32_t* segCount) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nT; i += gridDim.x * blockDim.x) {
    const uint32_t a = t.h1[i], b = t.h2[i], c = t.h3[i];
    const uint32_t lt = hits.layer[a] - 1;
    bool good = lt < fc.nLT && hits.layer[a] - 1 == fc.layer[0][lt] && hits.layer[b] - 1 == fc.layer[1][lt] &&
                hits.layer[c] - 1 == fc.layer[2][lt];
    if (good && truthOnly) {
      const uint32_t id = hits.hid[a];
      good = id != 0 && hits.hid[b] == id && hits.hid[c] == id;
    }
    if (good) {
      const float4 h[3] = {hits.xyzp[a], hits.xyzp[b], hits.xyzp[c]};
      Corr k[3];
      FitState f;
      good = fit_forward(fc, lt, h, k, f);
    }
    ok[i] = good ? 1u : 0u;
    if (good) atomicAdd(&segCount[fit_seg(cfg, hits, a)], 1u);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) ok[nT] = 0u;
}

__global__ void fit_scatter_kernel(DevConfig cfg, DevHits hits, TripletView t, uint32_t nT, const uint32_t* okScan,
                                   const int32_t* segDelta, uint32_t* rows) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nT; i += gridDim.x * blockDim.x) {
    if (okScan[i + 1] == okScan[i]) continue;
    const uint32_t s = fit_seg(cfg, hits, t.h1[i]);
    rows[(uint32_t)((int64_t)okScan[i] + segDelta[s])] = i;
  }
}

__device__ __forceinline__ double warp_sum(double v) {
  for (int d = 16; d > 0; d >>= 1) v += __shfl_down_sync(0xffffffffu, v, d);
  return v;
}

template <bool GRAD>
__global__ void __launch_bounds__(FIT_THREADS)
    fit_eval_kernel(FitConfig fc, DevHits hits, TripletView t, const uint32_t* __restrict__ rows,
                    double* partials, float* params, double* dHits) {
  __shared__ double s_acc[FIT_THREADS / 32][TRAX_FIT_SLOTS];
  const uint32_t blk = blockIdx.x;
  uint32_t lt = 0;
  while (lt + 1 < fc.nLT && blk >= fc.blkStart[lt + 1]) ++lt;
  const uint32_t begin = fc.ltBase[lt] + (blk - fc.blkStart[lt]) * TRAX_FIT_CHUNK;
  const uint32_t end = min(begin + TRAX_FIT_CHUNK, fc.ltBase[lt + 1]);
  double acc[TRAX_FIT_SLOTS];
#pragma unroll
  for (int k = 0; k < TRAX_FIT_SLOTS; ++k) acc[k] = 0.0;
  for (uint32_t r = begin + threadIdx.x; r < end; r += FIT_THREADS) {
    const uint32_t ti = rows[r];
    const uint32_t hi[3] = {t.h1[ti], t.h2[ti], t.h3[ti]};
    const float4 h[3] = {hits.xyzp[hi[0]], hits.xyzp[hi[1]], hits.xyzp[hi[2]]};
    Corr k[3];
    FitState f;
    if (!fit_forward(fc, lt, h, k, f)) {
      // a row selected at other shifts whose fit is not usable at these: it
      // contributes nothing (reported as NaN parameters)
      if (params) reinterpret_cast<float4*>(params)[r] = make_float4(NAN, NAN, NAN, NAN);
      continue;
    }
    acc[0] += (double)fit_chi2(fc, lt, f);
    if (params) {
      reinterpret_cast<float4*>(params)[r] = make_float4(1.0f / f.R, f.d0, f.z0, f.t);
    }
    if (GRAD) {
      float gX[3], gY[3], gR[3], gZ[3];
      const float seedE[3] = {2.0f * fc.wZ * f.e[0], 2.0f * fc.wZ * f.e[1], 2.0f * fc.wZ * f.e[2]};
      fit_adjoint(f, 2.0f * fc.wTip[lt] * f.d0, seedE, gX, gY, gR, gZ);
      // approximate Gauss-Newton diagonal (a preconditioner): d d0 / d align
      // squared over sigma_tip^2 for dr and dphi; the z residuals' projector
      // diagonal P_kk = (2/3 - ds_k^2 / S_ss) / sigma_z^2 for dz, and
      // cot(theta)^2 P_kk for dr (a radial shift slides the hit along its arc)
      float hX[3], hY[3], hR[3], hZ[3];
      const float zero3[3] = {0.0f, 0.0f, 0.0f};
      fit_adjoint(f, 1.0f, zero3, hX, hY, hR, hZ);
      const float Sss = f.ds[0] * f.ds[0] + f.ds[1] * f.ds[1] + f.ds[2] * f.ds[2];
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const Corr& c = k[i];
        // d(X, Y)/d dr = (xr, yr) / r, d(X, Y)/d dphi = f (-yr, xr), dZ/d dz = 1
        // the radial part: r_i = r + dr
        const float gdr = (gX[i] * c.xr + gY[i] * c.yr) / c.r + gR[i];
        const float gdp = c.f * (gY[i] * c.xr - gX[i] * c.yr);
        acc[1 + 3 * i] += (double)gdr;
        acc[2 + 3 * i] += (double)gZ[i];
        acc[3 + 3 * i] += (double)gdp;
        const float hdr = (hX[i] * c.xr + hY[i] * c.yr) / c.r;
        const float hdp = c.f * (hY[i] * c.xr - hX[i] * c.yr);
        const float pkk = fc.wZ * (2.0f / 3.0f - f.ds[i] * f.ds[i] / Sss);
        const float tq = f.t / f.sq[i];
        acc[10 + 3 * i] += (double)(fc.wTip[lt] * hdr * hdr + tq * tq * pkk);
        acc[11 + 3 * i] += (double)pkk;
        acc[12 + 3 * i] += (double)(fc.wTip[lt] * hdp * hdp);
        if (dHits) {
          // raw-hit Jacobian: X = f (x c - y s), Y = f (x s + y c), f = 1 + dr / r
          const uint32_t l = fc.layer[i][lt];
          const float cs = 1.0f + fc.cm1[l], sn = fc.sn[l];
          const float r3 = c.r * c.r * c.r;
          const float dfx = -fc.dr[l] * h[i].x / r3, dfy = -fc.dr[l] * h[i].y / r3;
          const float gx = gX[i] * (c.f * cs + c.xr * dfx) + gY[i] * (c.f * sn + c.yr * dfx) + gR[i] * h[i].x / c.r;
          const float gy = gX[i] * (-c.f * sn + c.xr * dfy) + gY[i] * (c.f * cs + c.yr * dfy) + gR[i] * h[i].y / c.r;
          double* o = dHits + 3 * (size_t)hi[i];
          atomicAdd(o + 0, (double)gx);
          atomicAdd(o + 1, (double)gy);
          atomicAdd(o + 2, (double)gZ[i]);
        }
      }
    }
  }
  // block sums in a fixed order
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < TRAX_FIT_SLOTS; ++k) {
    const double v = warp_sum(acc[k]);
    if (lane == 0) s_acc[warp][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < TRAX_FIT_SLOTS) {
    double v = 0.0;
    for (int w = 0; w < FIT_THREADS / 32; ++w) v += s_acc[w][threadIdx.x];
    partials[(size_t)blk * TRAX_FIT_SLOTS + threadIdx.x] = v;
  }
}

// one thread per output: chi2, then (dr, dz, dphi) of every layer, then
// their squared per-triplet sums
__global__ void fit_reduce_kernel(FitConfig fc, const double* __restrict__ partials, double* out) {
  const uint32_t nOut = 1 + 6 * fc.L;
  for (uint32_t o = threadIdx.x; o < nOut; o += blockDim.x) {
    double v = 0.0;
    if (o == 0) {
      for (uint32_t b = 0; b < fc.nBlocks; ++b) v += partials[(size_t)b * TRAX_FIT_SLOTS];
    } else {
      const uint32_t sq = o > 3 * fc.L ? 9u : 0u;  // squared sums follow the sums
      const uint32_t q = o - 1 - (sq ? 3 * fc.L : 0u);
      const uint32_t l = q / 3, p = q % 3;
      for (uint32_t lt = 0; lt < fc.nLT; ++lt)
        for (int slot = 0; slot < 3; ++slot) {
          if (fc.layer[slot][lt] != l) continue;
          for (uint32_t b = fc.blkStart[lt]; b < fc.blkStart[lt + 1]; ++b)
            v += partials[(size_t)b * TRAX_FIT_SLOTS + 1 + sq + 3 * slot + p];
        }
    }
    out[o] = v;
  }
}

__global__ void fit_hits_out_kernel(const double* __restrict__ dHits, const uint32_t* __restrict__ orig,
                                    uint64_t nHits, float* out) {
  for (uint64_t h = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; h < nHits;
       h += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t o = orig ? orig[h] : h;
    out[3 * o + 0] = (float)dHits[3 * h + 0];
    out[3 * o + 1] = (float)dHits[3 * h + 1];
    out[3 * o + 2] = (float)dHits[3 * h + 2];
  }
}

// corrected coordinates written over the uploaded hits
__global__ void fit_apply_kernel(FitConfig fc, float* x, float* y, float* z, const uint32_t* layer, uint64_t n) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t l = layer[i] - 1;
    if (l >= fc.L) continue;
    const Corr k = correct(fc, l, x[i], y[i]);
    x[i] += k.dX;
    y[i] += k.dY;
    z[i] += fc.dz[l];
  }
}

int blocks_for(uint64_t n, int threads) {
  uint64_t b = (n + threads - 1) / threads;
  const uint64_t cap = (uint64_t)sm_count() * 8;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (int)b;
}

}  // namespace

cudaError_t fit_select(const FitConfig& fc, const DevConfig& cfg, DevHits hits, TripletView t, uint64_t nT,
                       int truthOnly, uint32_t* ok, uint32_t* segCount, cudaStream_t st, uint32_t* launches) {
  fit_select_kernel<<<blocks_for(nT + 1, 256), 256, 0, st>>>(fc, cfg, hits, t, (uint32_t)nT, truthOnly, ok,
                                                              segCount);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

cudaError_t fit_scatter(const DevConfig& cfg, DevHits hits, TripletView t, uint64_t nT, const uint32_t* okScan,
                        const int32_t* segDelta, uint32_t* rows, cudaStream_t st, uint32_t* launches) {
  if (nT == 0) return cudaSuccess;
  fit_scatter_kernel<<<blocks_for(nT, 256), 256, 0, st>>>(cfg, hits, t, (uint32_t)nT, okScan, segDelta, rows);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

cudaError_t fit_eval(const FitConfig& fc, bool grad, DevHits hits, TripletView t, const uint32_t* rows,
                     double* partials, float* params, double* dHits, cudaStream_t st, uint32_t* launches) {
  if (fc.nBlocks == 0) return cudaSuccess;
  if (grad)
    fit_eval_kernel<true><<<fc.nBlocks, FIT_THREADS, 0, st>>>(fc, hits, t, rows, partials, params, dHits);
  else
    fit_eval_kernel<false><<<fc.nBlocks, FIT_THREADS, 0, st>>>(fc, hits, t, rows, partials, params, nullptr);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

cudaError_t fit_reduce(const FitConfig& fc, const double* partials, double* out, cudaStream_t st,
                       uint32_t* launches) {
  fit_reduce_kernel<<<1, 128, 0, st>>>(fc, partials, out);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

cudaError_t fit_apply(const FitConfig& fc, float* x, float* y, float* z, const uint32_t* layer, uint64_t n,
                      cudaStream_t st, uint32_t* launches) {
  if (n == 0) return cudaSuccess;
  fit_apply_kernel<<<blocks_for(n, 256), 256, 0, st>>>(fc, x, y, z, layer, n);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

cudaError_t fit_hits_out(const double* dHits, const uint32_t* orig, uint64_t nHits, float* out, cudaStream_t st,
                         uint32_t* launches) {
  if (nHits == 0) return cudaSuccess;
  fit_hits_out_kernel<<<blocks_for(nHits, 256), 256, 0, st>>>(dHits, orig, nHits, out);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

}  // namespace trax
