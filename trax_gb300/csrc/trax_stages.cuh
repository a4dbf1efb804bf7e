// trax_stages.cuh -- per-pair prediction window and per-candidate filter
// predicates, shared by the kernels of the prediction and filter stages
// so that every pass evaluates exactly the same float operations.
#pragma once

#include "trax_device.cuh"

namespace trax {

// Third-hit window of one pair (predictCount / predictStore,
// TripletThetaPhiPredictor.h:111-185 and :286-355).  The two kernels differ
// only in how rOrigin is rounded (Q4); both z windows are kept, the phi
// window is common.
struct PredWindow {
  float zLow[2], zHigh[2];           // [0] count variant, [1] store variant
  uint32_t zLoSec[2], zHiSec[2];
  float phiLow, phiHigh;
  uint32_t pL, pH, wrap;
  bool same;                         // both variants give the same window
};

__device__ __forceinline__ void pred_z_bounds(float p1z, float p2z, float rOrigin, float r2t, float tip2,
                                              float minR, float maxR, float sigmaZ, float& zLow, float& zHigh) {
  const float cotTheta = div_(p2z - p1z, r2t - rOrigin);
  float tmp = p1z + (sqrt_(maxR * maxR - tip2) - rOrigin) * cotTheta;
  zLow = p1z + (sqrt_(minR * minR - tip2) - rOrigin) * cotTheta;
  zHigh = (float)(tmp > zLow) * tmp + (float)(tmp < zLow) * zLow;
  zLow = (float)(tmp > zLow) * zLow + (float)(tmp < zLow) * tmp;
  zLow -= sigmaZ;
  zHigh += sigmaZ;
}

// The z rows of a window: its first row, and its last row without the
// clamp to nZ (0xffffffff when the bound lies beyond 2^32 rows).
__device__ __forceinline__ uint32_t pred_row_lo(const DevConfig& cfg, float zLow) {
  return (uint32_t)max(f2i_sat(floor_(div_(zLow - cfg.minZ, cfg.sZ))), 0);
}
__device__ __forceinline__ uint32_t pred_row_hi_raw(const DevConfig& cfg, float zHigh) {
  return f2u_sat(floor_(div_(zHigh - cfg.minZ, cfg.sZ)));
}

// The candidates the prediction count captures for pair gid, slot q at
// p[q * stride].  Interleaved (IL, keep_interleaved: 16 or more slots per
// pair, or the fine z grid), the slots of a warp's 32 consecutive pairs
// share lines (stride 32: slot q of those pairs is one 128-byte line, which
// the lanes fill and read together); otherwise a pair's slots are
// consecutive (stride 1: one or two 32-byte sectors per pair, mostly
// holding one candidate).  The layout is a template parameter of the
// kernels that touch the slots, chosen on the host.
template <bool IL, class T>
struct KeepSlots {
  T* p;
  __device__ __forceinline__ T& operator[](uint32_t q) const { return p[(size_t)q * (IL ? 32u : 1u)]; }
};
template <bool IL, class T>
__device__ __forceinline__ KeepSlots<IL, T> keep_slots(T* keep, uint32_t gid, uint32_t nKeep) {
  return KeepSlots<IL, T>{IL ? keep + (((size_t)(gid >> 5) * nKeep) << 5) + (gid & 31u) : keep + (size_t)gid * nKeep};
}

// Row of z in the fine grid, given G, z's row in the grid clamped to
// [0, nZ): h = floor((z - minZ) * fineScale) clamped into G's block
// [G fineRows, G fineRows + fineRows).  Both h and G are non-decreasing in
// z, so the fine row is too (a larger G puts it in a later block, an equal
// G clamps a larger h into the same block), and a hit's fine row lies in
// the block of its grid row.
__device__ __forceinline__ uint32_t fine_row(const DevConfig& cfg, float z, uint32_t G) {
  const uint32_t h = f2u_sat(floor_((z - cfg.minZ) * cfg.fineScale));
  const uint32_t lo = G * cfg.fineRows;
  return min(max(h, lo), lo + cfg.fineRows - 1u);
}

__device__ __forceinline__ void pred_z_window(const DevConfig& cfg, float p1z, float p2z, float rOrigin,
                                              float r2t, float tip2, float minR, float maxR, float sigmaZ,
                                              float& zLow, float& zHigh, uint32_t& lo, uint32_t& hi) {
  pred_z_bounds(p1z, p2z, rOrigin, r2t, tip2, minR, maxR, sigmaZ, zLow, zHigh);
  lo = pred_row_lo(cfg, zLow);
  hi = min(pred_row_hi_raw(cfg, zHigh) + 1u, cfg.nZ);
}

// The phi window of one pair (TripletThetaPhiPredictor.h:151-185).
__device__ __forceinline__ void pred_phi_window(const DevConfig& cfg, uint32_t lt, uint32_t layer, float4 h1,
                                                float4 h2, float& phiLowOut, float& phiHighOut, uint32_t& pL,
                                                uint32_t& pH, uint32_t& wrap) {
  const float sigmaPhi = cfg.sigmaPhi[lt];
  const float p1x = h1.x, p1y = h1.y;
  const float p2x = h2.x, p2y = h2.y;
  const float phi = h2.w;  // atan2(p2.y, p2.x)
  float dPhi = phi - h1.w;
  dPhi += (dPhi > TRAX_PI_F) ? -2 * TRAX_PI_F : (dPhi < -TRAX_PI_F) ? 2 * TRAX_PI_F : 0;
  dPhi = fabs_(dPhi);
  const float dHits = sqrt_((p2x - p1x) * (p2x - p1x) + (p2y - p1y) * (p2y - p1y));
  const float twoR = 2 * cfg.minRcurv;
  const float aH = acos_(div_(dHits, twoR));
  float tmp = fabs_(aH - cfg.acosMaxR[layer]);
  float phiLow = fabs_(aH - cfg.acosMinR[layer]);
  dPhi = cl_max(dPhi, cl_max(tmp, phiLow));
  float phiHigh = phi + dPhi + sigmaPhi;
  phiLow = phi - dPhi - sigmaPhi;
  const bool wrapAround = phiLow < -TRAX_PI_F || phiHigh > TRAX_PI_F || phiLow > TRAX_PI_F || phiHigh < -TRAX_PI_F;
  // (float)((x > pi) * 2) * pi is 2 pi (exact) or +0, as a select
  phiLow -= (phiLow > TRAX_PI_F) ? 2.0f * TRAX_PI_F : 0.0f;
  phiLow += (phiLow < -TRAX_PI_F) ? 2.0f * TRAX_PI_F : 0.0f;
  phiHigh -= (phiHigh > TRAX_PI_F) ? 2.0f * TRAX_PI_F : 0.0f;
  phiHigh += (phiHigh < -TRAX_PI_F) ? 2.0f * TRAX_PI_F : 0.0f;
  phiLowOut = phiLow;
  phiHighOut = phiHigh;
  pL = f2u_sat(floor_(div_(phiLow - cfg.minPhi, cfg.sP)));
  pH = min(f2u_sat(floor_(div_(phiHigh - cfg.minPhi, cfg.sP))) + 1u, cfg.nP);
  wrap = wrapAround ? 1u : 0u;
}

// h1, h2: (x, y, z, phi) of the pair's hits; layer = third layer (0-based)
__device__ __forceinline__ PredWindow pred_window(const DevConfig& cfg, uint32_t lt, uint32_t layer, float4 h1,
                                                  float4 h2) {
  PredWindow w;
  const float sigmaZ = cfg.sigmaZ[lt];
  const float minR = cfg.minR[layer];
  const float maxR = cfg.maxR[layer];
  const float p1x = h1.x, p1y = h1.y, p1z = h1.z;
  const float p2x = h2.x, p2y = h2.y, p2z = h2.z;
  float tip2 = p1y * (p2x - p1x) - p1x * (p2y - p1y);
  tip2 *= tip2;
  tip2 = div_(tip2, (p2x - p1x) * (p2x - p1x) + (p2y - p1y) * (p2y - p1y));
  const float rr = p1x * p1x + p1y * p1y;
  const float rOc = sqrt_(rr - tip2);  // :130-131
  const float r1 = sqrt_(rr);
  const float rOs = sqrt_(r1 * r1 - tip2);  // :305-306
  const float r2t = sqrt_(p2x * p2x + p2y * p2y - tip2);
  pred_z_window(cfg, p1z, p2z, rOc, r2t, tip2, minR, maxR, sigmaZ, w.zLow[0], w.zHigh[0], w.zLoSec[0], w.zHiSec[0]);
  w.same = f2bits(rOc) == f2bits(rOs);
  if (w.same) {
    w.zLow[1] = w.zLow[0];
    w.zHigh[1] = w.zHigh[0];
    w.zLoSec[1] = w.zLoSec[0];
    w.zHiSec[1] = w.zHiSec[0];
  } else {
    pred_z_window(cfg, p1z, p2z, rOs, r2t, tip2, minR, maxR, sigmaZ, w.zLow[1], w.zHigh[1], w.zLoSec[1],
                  w.zHiSec[1]);
  }
  pred_phi_window(cfg, lt, layer, h1, h2, w.phiLow, w.phiHigh, w.pL, w.pH, w.wrap);
  return w;
}

// The store variant alone (predictStore, TripletThetaPhiPredictor.h:286-355:
// rOrigin = sqrt(sqrt(x^2+y^2)^2 - tip2)), for the store pass's re-walks;
// both entries of the window hold it.
__device__ __forceinline__ PredWindow pred_store_window(const DevConfig& cfg, uint32_t lt, uint32_t layer,
                                                        float4 h1, float4 h2) {
  PredWindow w;
  const float p1x = h1.x, p1y = h1.y, p1z = h1.z;
  const float p2x = h2.x, p2y = h2.y, p2z = h2.z;
  float tip2 = p1y * (p2x - p1x) - p1x * (p2y - p1y);
  tip2 *= tip2;
  tip2 = div_(tip2, (p2x - p1x) * (p2x - p1x) + (p2y - p1y) * (p2y - p1y));
  const float r1 = sqrt_(p1x * p1x + p1y * p1y);
  const float rOs = sqrt_(r1 * r1 - tip2);
  const float r2t = sqrt_(p2x * p2x + p2y * p2y - tip2);
  pred_z_window(cfg, p1z, p2z, rOs, r2t, tip2, cfg.minR[layer], cfg.maxR[layer], cfg.sigmaZ[lt], w.zLow[1],
                w.zHigh[1], w.zLoSec[1], w.zHiSec[1]);
  w.zLow[0] = w.zLow[1];
  w.zHigh[0] = w.zHigh[1];
  w.zLoSec[0] = w.zLoSec[1];
  w.zHiSec[0] = w.zHiSec[1];
  w.same = true;
  pred_phi_window(cfg, lt, layer, h1, h2, w.phiLow, w.phiHigh, w.pL, w.pH, w.wrap);
  return w;
}

// The count pass's window: both variants' z bounds and one row range, the
// union of their rows.  A hit's row is g(z) = floor(div(z - minZ, sZ)),
// saturated, and a variant's rows are [g(zLow), g(zHigh) + 1) clamped to
// [0, nZ): g is monotone, so a hit in the grid that passes a variant's test
// zLow <= z <= zHigh lies in that variant's rows, and walking the union with
// each variant's own test changes no outcome and no visit order.  The union
// of the rows is the rows of [min zLow, max zHigh], two divisions instead of
// four.  A variant with a NaN bound (its test never passes) or with rows
// past 2^32 (the reference's hi wraps to 0: no rows) is switched off by the
// bounds (+inf, -inf); the union is then taken over the other variant.
struct PredUnionWindow {
  float zLow[2], zHigh[2];  // [0] count variant, [1] store variant
  uint32_t zLo, zHi;        // rows of both
  float phiLow, phiHigh;
  uint32_t pL, pH, wrap;
};

__device__ __forceinline__ PredUnionWindow pred_union_window(const DevConfig& cfg, uint32_t lt, uint32_t layer,
                                                             float4 h1, float4 h2) {
  PredUnionWindow w;
  const float sigmaZ = cfg.sigmaZ[lt];
  const float minR = cfg.minR[layer];
  const float maxR = cfg.maxR[layer];
  const float p1x = h1.x, p1y = h1.y, p1z = h1.z;
  const float p2x = h2.x, p2y = h2.y, p2z = h2.z;
  float tip2 = p1y * (p2x - p1x) - p1x * (p2y - p1y);
  tip2 *= tip2;
  tip2 = div_(tip2, (p2x - p1x) * (p2x - p1x) + (p2y - p1y) * (p2y - p1y));
  const float rr = p1x * p1x + p1y * p1y;
  const float rOc = sqrt_(rr - tip2);  // :130-131
  const float r1 = sqrt_(rr);
  const float rOs = sqrt_(r1 * r1 - tip2);  // :305-306
  const float r2t = sqrt_(p2x * p2x + p2y * p2y - tip2);
  // both variants for every pair: with rOs == rOc the same operations give
  // the same bounds, and no branch splits the warp
  pred_z_bounds(p1z, p2z, rOc, r2t, tip2, minR, maxR, sigmaZ, w.zLow[0], w.zHigh[0]);
  pred_z_bounds(p1z, p2z, rOs, r2t, tip2, minR, maxR, sigmaZ, w.zLow[1], w.zHigh[1]);
  const float inf = __int_as_float(0x7f800000);
  bool on0 = !is_nan(w.zLow[0]) && !is_nan(w.zHigh[0]);
  bool on1 = !is_nan(w.zLow[1]) && !is_nan(w.zHigh[1]);
  float zl = on0 ? (on1 ? fminf(w.zLow[0], w.zLow[1]) : w.zLow[0]) : w.zLow[1];
  float zh = on0 ? (on1 ? fmaxf(w.zHigh[0], w.zHigh[1]) : w.zHigh[0]) : w.zHigh[1];
  uint32_t hiRaw = pred_row_hi_raw(cfg, zh);
  if (hiRaw == 0xffffffffu) {  // a variant whose rows wrap: only far outside the grid
    on0 = on0 && pred_row_hi_raw(cfg, w.zHigh[0]) != 0xffffffffu;
    on1 = on1 && pred_row_hi_raw(cfg, w.zHigh[1]) != 0xffffffffu;
    zl = on0 ? (on1 ? fminf(w.zLow[0], w.zLow[1]) : w.zLow[0]) : w.zLow[1];
    zh = on0 ? (on1 ? fmaxf(w.zHigh[0], w.zHigh[1]) : w.zHigh[0]) : w.zHigh[1];
    hiRaw = pred_row_hi_raw(cfg, zh);
  }
  if (!on0) {
    w.zLow[0] = inf;
    w.zHigh[0] = -inf;
  }
  if (!on1) {
    w.zLow[1] = inf;
    w.zHigh[1] = -inf;
  }
  if (on0 || on1) {
    w.zLo = pred_row_lo(cfg, zl);
    w.zHi = min(hiRaw + 1u, cfg.nZ);
  } else {
    w.zLo = w.zHi = 0u;
  }
  pred_phi_window(cfg, lt, layer, h1, h2, w.phiLow, w.phiHigh, w.pL, w.pH, w.wrap);
  return w;
}

// phi part of the candidate test (TripletThetaPhiPredictor.h:211-214)
__device__ __forceinline__ bool pred_phi_ok(const PredWindow& w, float actPhi) {
  return (!w.wrap && (w.phiLow <= actPhi && actPhi <= w.phiHigh)) ||
         (w.wrap && ((w.phiLow <= actPhi && actPhi <= TRAX_PI_F) || (-TRAX_PI_F <= actPhi && actPhi <= w.phiHigh)));
}

__device__ __forceinline__ bool pred_valid(const PredWindow& w, int v, float4 h) {
  const bool valid = w.zLow[v] <= h.z && h.z <= w.zHigh[v];
  return valid && pred_phi_ok(w, h.w);
}

// Visit ranges of one z row of the third layer (the reference's j loop with
// index = j - (j >= zEnd) * len, zEnd being the next row's start -- Q8): the
// loop visits P1 = [J0, min(end2, zEnd)) and then P2 = [max(J0, zEnd) - len, end2 - len).
template <class Window>  // PredWindow or PredUnionWindow
__device__ __forceinline__ void pred_row_parts(const Window& w, const uint32_t* lG, uint32_t C, uint32_t nP,
                                               uint32_t zs, uint32_t& a1, uint32_t& b1, uint32_t& a2, uint32_t& b2) {
  const uint32_t row = zs * (nP + 1);
  const uint32_t zStart = cell_at(lG, row, C);
  const uint32_t zEnd = cell_at(lG, row + nP + 1, C);
  const uint32_t len = zEnd - zStart;
  const uint32_t J0 = cell_at(lG, row + w.pL, C);
  const uint32_t end2 = w.wrap * zEnd + cell_at(lG, row + w.pH, C) - w.wrap * zStart;
  a1 = J0;
  b1 = min(end2, zEnd);
  if (b1 < a1) b1 = a1;
  const uint32_t j2 = max(J0, zEnd);
  if (j2 < end2) {
    a2 = j2 - len;
    b2 = end2 - len;
  } else {
    a2 = b2 = 0;
  }
}

// filterCount (TripletThetaPhiFilter.h:84-154) is the AND of four predicates
// that share no state, so they can be evaluated in any order.  The dphi
// part (:118-128): the transverse angles of the two segments.
__device__ __forceinline__ bool filter_dphi(float dPhiCut, float4 A, float4 B, float4 Cc) {
  const float phi1 = atan2_((B.y - A.y), (B.x - A.x));
  const float phi2 = atan2_((Cc.y - B.y), (Cc.x - B.x));
  float delta = phi2 - phi1;
  delta += (delta > TRAX_PI_F) ? -2 * TRAX_PI_F : (delta < -TRAX_PI_F) ? 2 * TRAX_PI_F : 0;
  return fabs_(delta) <= dPhiCut;
}

// The dphi part decided from cross and dot products where that is certain
// (dphi_decide), else by the atan2 evaluation above.
__device__ __forceinline__ bool filter_dphi_fast(const DevConfig& cfg, uint32_t lt, float4 A, float4 B, float4 Cc) {
  const int q = dphi_decide(cfg.dPhiTanLo[lt], cfg.dPhiTanHi[lt], B.x - A.x, B.y - A.y, Cc.x - B.x, Cc.y - B.y);
  return q > 0 || (q < 0 && filter_dphi(cfg.dPhiCut[lt], A, B, Cc));
}

// The dtheta part (:84-117): the polar angles of the two segments.
__device__ __forceinline__ bool filter_dtheta(const DevConfig& cfg, uint32_t lt, float4 A, float4 B, float4 Cc) {
  const float theta1 = atan2_(sqrt_((B.x - A.x) * (B.x - A.x) + (B.y - A.y) * (B.y - A.y)), (B.z - A.z));
  const float angle2 = atan2_(sqrt_((Cc.x - B.x) * (Cc.x - B.x) + (Cc.y - B.y) * (Cc.y - B.y)), (Cc.z - B.z));
  const float delta = fabs_(div_(angle2, theta1));
  return 1 - cfg.dThetaCut[lt] <= delta && delta <= 1 + cfg.dThetaCut[lt];
}

// The TIP and curvature parts (:130-154): the circle through the three hits
// from the paraboloid plane, its point closest to the beam line and radius.
__device__ __forceinline__ bool filter_circle(const DevConfig& cfg, uint32_t lt, float4 A, float4 B, float4 Cc) {
  const f3 pP1 = make_f3(A.x, A.y, A.x * A.x + A.y * A.y);
  const f3 pP2 = make_f3(B.x, B.y, B.x * B.x + B.y * B.y);
  const f3 pP3 = make_f3(Cc.x, Cc.y, Cc.x * Cc.x + Cc.y * Cc.y);
  const f3 a = sub3(pP2, pP1);
  const f3 b = sub3(pP3, pP1);
  const f3 n = normalize3(cross3(a, b));
  const float cOx = div_(-n.x, 2 * n.z);
  const float cOy = div_(-n.y, 2 * n.z);
  const float cc = -(n.x * pP1.x + n.y * pP1.y + n.z * pP1.z);
  const float cR = sqrt_(div_(1 - n.z * n.z - 4 * cc * n.z, 4 * n.z * n.z));
  float vx = -cOx, vy = -cOy;
  normalize2(vx, vy);
  const float pCAx = cOx + cR * vx;
  const float pCAy = cOy + cR * vy;
  const float tip_squared = pCAx * pCAx + pCAy * pCAy;
  const float tipCut = cfg.tipCut[lt];
  return tip_squared <= (tipCut * tipCut) && cR >= cfg.minRcurv;
}

// The dtheta, TIP and curvature parts together.
__device__ __forceinline__ bool filter_rest(const DevConfig& cfg, uint32_t lt, float4 A, float4 B, float4 Cc) {
  const bool dtheta = filter_dtheta(cfg, lt, A, B, Cc);
  return filter_circle(cfg, lt, A, B, Cc) && dtheta;
}

}  // namespace trax
