// k_triplets.cu -- third-hit prediction and the dtheta/dphi/TIP filter.
//
// Prediction replaces predictCount / predictStore / predictOffsetMonotonizeStore
// (TripletThetaPhiPredictor.h:49-447, .cpp:10-168): one thread per pair, the
// count pass with predictCount's rOrigin and the store pass with
// predictStore's (Q4: sqrt(x^2+y^2-tip2) vs sqrt(sqrt(x^2+y^2)^2-tip2)), the
// store capped at the count exactly like `pos < nextThread`.  Slots the store
// pass cannot fill (the reference leaves them unwritten) get the candidate
// (pair, 0xffffffff), which the filter rejects.
//
// The filter replaces filterCount / filterPopCount / PrefixSum / filterStore /
// filterOffsetStore / filterOffsetMonotonizeStore (TripletThetaPhiFilter.h:50-280,
// .cpp:10-206): a flag per candidate, a scan of the flags and a stable
// scatter of (h1, h2, h3) keep the candidate order of the reference.
#include "trax_kernels.h"

namespace trax {

namespace {

constexpr int PRED_THREADS = 128;

int grid_for(uint64_t items, int threads) {
  uint64_t blocks = (items + threads - 1) / threads;
  uint64_t cap = (uint64_t)sm_count() * 16;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  return (int)blocks;
}

template <bool STORE>
__global__ void __launch_bounds__(PRED_THREADS)
    predict_kernel(DevConfig cfg, const uint32_t* __restrict__ grid, const float4* __restrict__ hits,
                   const uint32_t* __restrict__ hitEvt, const uint32_t* __restrict__ hitLayer,
                   const uint2* __restrict__ pairs, const uint32_t* __restrict__ nPairsDev, uint32_t* candCount,
                   uint2* cands, uint32_t capCands, uint32_t* sentinels) {
  const uint32_t nPairs = *nPairsDev;
  const uint32_t C = cfg.C, nP = cfg.nP;
  for (uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x; gid < nPairs; gid += gridDim.x * blockDim.x) {
    const uint2 pr = pairs[gid];
    uint32_t pos = 0, limit = 0;
    uint2* out = nullptr;
    if (STORE) {
      pos = candCount[gid];
      limit = candCount[gid + 1] - pos;
      if (pos >= capCands) limit = 0;
      else if (limit > capCands - pos) limit = capCands - pos;
      out = cands + pos;
    }
    uint32_t nFound = 0;
    if (pr.x != TRAX_SENTINEL) {
      const uint32_t firstHit = pr.x, secondHit = pr.y;
      const uint32_t event = hitEvt[firstHit];
      const uint32_t layerTriplet = hitLayer[firstHit] - 1;  // Q7
      const uint32_t layer = cfg.layer3[layerTriplet] - 1;
      const uint32_t* lGrid3 = grid + ((size_t)event * cfg.L + layer) * C;
      const float sigmaZ = cfg.sigmaZ[layerTriplet];
      const float sigmaPhi = cfg.sigmaPhi[layerTriplet];
      const float minLayerRadius = cfg.minR[layer];
      const float maxLayerRadius = cfg.maxR[layer];
      const float4 h1 = hits[firstHit], h2 = hits[secondHit];
      const float p1x = h1.x, p1y = h1.y, p1z = h1.z;
      const float p2x = h2.x, p2y = h2.y, p2z = h2.z;
      float tip2 = p1y * (p2x - p1x) - p1x * (p2y - p1y);
      tip2 *= tip2;
      tip2 = div_(tip2, (p2x - p1x) * (p2x - p1x) + (p2y - p1y) * (p2y - p1y));
      float rOrigin;
      if (!STORE) {
        rOrigin = p1x * p1x + p1y * p1y;
        rOrigin = sqrt_(rOrigin - tip2);
      } else {
        rOrigin = sqrt_(p1x * p1x + p1y * p1y);
        rOrigin = sqrt_(rOrigin * rOrigin - tip2);
      }
      const float cotTheta = div_(p2z - p1z, sqrt_(p2x * p2x + p2y * p2y - tip2) - rOrigin);
      float tmp = p1z + (sqrt_(maxLayerRadius * maxLayerRadius - tip2) - rOrigin) * cotTheta;
      float zLow = p1z + (sqrt_(minLayerRadius * minLayerRadius - tip2) - rOrigin) * cotTheta;
      float zHigh = (float)(tmp > zLow) * tmp + (float)(tmp < zLow) * zLow;
      zLow = (float)(tmp > zLow) * zLow + (float)(tmp < zLow) * tmp;
      zLow -= sigmaZ;
      zHigh += sigmaZ;
      const uint32_t zLowSector = (uint32_t)max(f2i_sat(floor_(div_(zLow - cfg.minZ, cfg.sZ))), 0);
      const uint32_t zHighSector = min(f2u_sat(floor_(div_(zHigh - cfg.minZ, cfg.sZ))) + 1u, cfg.nZ);
      const float phi = h2.w;  // atan2(p2.y, p2.x)
      tmp = h1.w;              // atan2(p1.y, p1.x)
      float dPhi = phi - tmp;
      dPhi += (dPhi > TRAX_PI_F) ? -2 * TRAX_PI_F : (dPhi < -TRAX_PI_F) ? 2 * TRAX_PI_F : 0;
      dPhi = fabs_(dPhi);
      const float dHits = sqrt_((p2x - p1x) * (p2x - p1x) + (p2y - p1y) * (p2y - p1y));
      const float twoR = 2 * cfg.minRcurv;
      tmp = fabs_(acos_(div_(dHits, twoR)) - acos_(div_(maxLayerRadius, twoR)));
      float phiLow = fabs_(acos_(div_(dHits, twoR)) - acos_(div_(minLayerRadius, twoR)));
      dPhi = cl_max(dPhi, cl_max(tmp, phiLow));
      float phiHigh = phi + dPhi + sigmaPhi;
      phiLow = phi - dPhi - sigmaPhi;
      const bool wrapAround = phiLow < -TRAX_PI_F || phiHigh > TRAX_PI_F || phiLow > TRAX_PI_F || phiHigh < -TRAX_PI_F;
      phiLow -= (float)((phiLow > TRAX_PI_F) * 2) * TRAX_PI_F;
      phiLow += (float)((phiLow < -TRAX_PI_F) * 2) * TRAX_PI_F;
      phiHigh -= (float)((phiHigh > TRAX_PI_F) * 2) * TRAX_PI_F;
      phiHigh += (float)((phiHigh < -TRAX_PI_F) * 2) * TRAX_PI_F;
      const uint32_t phiLowSector = f2u_sat(floor_(div_(phiLow - cfg.minPhi, cfg.sP)));
      const uint32_t phiHighSector = min(f2u_sat(floor_(div_(phiHigh - cfg.minPhi, cfg.sP))) + 1u, nP);
      const uint32_t w = wrapAround ? 1u : 0u;
      for (uint32_t zs = zLowSector; zs < zHighSector; ++zs) {
        const uint32_t row = zs * (nP + 1);
        const uint32_t zSectorStart = cell_at(lGrid3, row, C);
        const uint32_t zSectorEnd = cell_at(lGrid3, row + nP + 1, C);  // Q8
        const uint32_t len = zSectorEnd - zSectorStart;
        const uint32_t end2 = w * zSectorEnd + cell_at(lGrid3, row + phiHighSector, C) - w * zSectorStart;
        for (uint32_t j = cell_at(lGrid3, row + phiLowSector, C); j < end2; ++j) {
          const uint32_t index = j - (uint32_t)(j >= zSectorEnd) * len;
          const float4 h = hits[index];
          bool valid = zLow <= h.z && h.z <= zHigh;
          const float actPhi = h.w;
          valid = valid && ((!wrapAround && (phiLow <= actPhi && actPhi <= phiHigh)) ||
                            (wrapAround && ((phiLow <= actPhi && actPhi <= TRAX_PI_F) ||
                                            (-TRAX_PI_F <= actPhi && actPhi <= phiHigh))));
          if (STORE && valid) {
            if (nFound < limit) out[nFound] = make_uint2(gid, index);
          }
          nFound += valid;
          if (STORE && nFound >= limit) break;  // pos < nextThread (:376-377)
        }
        if (STORE && nFound >= limit) break;
      }
    }
    if (!STORE) {
      candCount[gid] = nFound;
      if (gid == 0) candCount[nPairs] = 0u;
    } else if (nFound < limit) {
      atomicAdd(sentinels, limit - nFound);
      for (uint32_t q = nFound; q < limit; ++q) out[q] = make_uint2(gid, TRAX_SENTINEL);
    }
  }
}

// tripletOffsets of predictStore (:404-418); monotonized afterwards
__global__ void predict_offsets_kernel(DevConfig cfg, const uint32_t* __restrict__ hitEvt,
                                       const uint32_t* __restrict__ hitLayer, const uint2* __restrict__ pairs,
                                       const uint32_t* nPairsDev, const uint32_t* candStart, uint32_t* offsets) {
  const uint32_t nPairs = *nPairsDev;
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < nPairs; g += gridDim.x * blockDim.x) {
    const uint2 p = pairs[g];
    if (p.x == TRAX_SENTINEL) continue;
    const uint32_t event = hitEvt[p.x];
    const uint32_t lt = hitLayer[p.x] - 1;
    const uint32_t next = candStart[g + 1];
    if (g < nPairs - 1) {
      const uint2 q = pairs[g + 1];
      const uint32_t nextEvent = q.x == TRAX_SENTINEL ? TRAX_SENTINEL : hitEvt[q.x];
      const uint32_t nextLT = q.x == TRAX_SENTINEL ? TRAX_SENTINEL : hitLayer[q.x] - 1;
      if (lt != nextLT || event != nextEvent) offsets[(size_t)event * cfg.nLT + lt + 1] = next;
    } else {
      offsets[(size_t)event * cfg.nLT + lt + 1] = next;
    }
  }
}

// filterCount (TripletThetaPhiFilter.h:65-154) for one candidate
__device__ __forceinline__ bool filter_one(const DevConfig& cfg, const float4* hits, const uint32_t* hitLayer,
                                           const uint2* pairs, uint2 cand) {
  const uint32_t thirdHit = cand.y;
  if (thirdHit == TRAX_SENTINEL) return false;
  const uint2 pr = pairs[cand.x];
  const uint32_t firstHit = pr.x, secondHit = pr.y;
  const uint32_t layerTriplet = hitLayer[firstHit] - 1;
  const float dThetaCut = cfg.dThetaCut[layerTriplet];
  const float dPhiCut = cfg.dPhiCut[layerTriplet];
  const float tipCut = cfg.tipCut[layerTriplet];
  const float4 A = hits[firstHit], B = hits[secondHit], Cc = hits[thirdHit];
  bool valid = true;
  float angle1 = atan2_(sqrt_((B.x - A.x) * (B.x - A.x) + (B.y - A.y) * (B.y - A.y)), (B.z - A.z));
  float angle2 = atan2_(sqrt_((Cc.x - B.x) * (Cc.x - B.x) + (Cc.y - B.y) * (Cc.y - B.y)), (Cc.z - B.z));
  float delta = fabs_(div_(angle2, angle1));
  valid = valid && (1 - dThetaCut <= delta && delta <= 1 + dThetaCut);
  angle1 = atan2_((B.y - A.y), (B.x - A.x));
  angle2 = atan2_((Cc.y - B.y), (Cc.x - B.x));
  delta = angle2 - angle1;
  delta += (delta > TRAX_PI_F) ? -2 * TRAX_PI_F : (delta < -TRAX_PI_F) ? 2 * TRAX_PI_F : 0;
  valid = valid && (fabs_(delta) <= dPhiCut);
  f3 pP1 = make_f3(A.x, A.y, A.x * A.x + A.y * A.y);
  f3 pP2 = make_f3(B.x, B.y, B.x * B.x + B.y * B.y);
  f3 pP3 = make_f3(Cc.x, Cc.y, Cc.x * Cc.x + Cc.y * Cc.y);
  f3 a = sub3(pP2, pP1);
  f3 b = sub3(pP3, pP1);
  f3 n = normalize3(cross3(a, b));
  const float cOx = div_(-n.x, 2 * n.z);
  const float cOy = div_(-n.y, 2 * n.z);
  const float cc = -(n.x * pP1.x + n.y * pP1.y + n.z * pP1.z);
  const float cR = sqrt_(div_(1 - n.z * n.z - 4 * cc * n.z, 4 * n.z * n.z));
  float vx = -cOx, vy = -cOy;
  normalize2(vx, vy);
  const float pCAx = cOx + cR * vx;
  const float pCAy = cOy + cR * vy;
  const float tip_squared = pCAx * pCAx + pCAy * pCAy;
  valid = valid && (tip_squared <= (tipCut * tipCut));
  valid = valid && (cR >= cfg.minRcurv);
  return valid;
}

__global__ void __launch_bounds__(256)
    filter_kernel(DevConfig cfg, const float4* __restrict__ hits, const uint32_t* __restrict__ hitLayer,
                  const uint2* __restrict__ pairs, const uint2* __restrict__ cands, const uint32_t* nCandsDev,
                  uint32_t* flags) {
  const uint32_t n = *nCandsDev;
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < n; g += gridDim.x * blockDim.x)
    flags[g] = filter_one(cfg, hits, hitLayer, pairs, cands[g]) ? 1u : 0u;
  if (blockIdx.x == 0 && threadIdx.x == 0) flags[n] = 0u;
}

__global__ void filter_store_kernel(const uint2* __restrict__ pairs, const uint2* __restrict__ cands,
                                    const uint32_t* nCandsDev, const uint32_t* __restrict__ scan, uint32_t* h1,
                                    uint32_t* h2, uint32_t* h3, uint32_t capT) {
  const uint32_t n = *nCandsDev;
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < n; g += gridDim.x * blockDim.x) {
    const uint32_t pos = scan[g];
    if (scan[g + 1] != pos && pos < capT) {
      const uint2 c = cands[g];
      const uint2 p = pairs[c.x];
      h1[pos] = p.x;
      h2[pos] = p.y;
      h3[pos] = c.y;
    }
  }
}

// filterOffsetStore (TripletThetaPhiFilter.h:221-257)
__global__ void triplet_offsets_kernel(DevConfig cfg, const uint32_t* __restrict__ hitEvt,
                                       const uint32_t* __restrict__ hitLayer, const uint32_t* __restrict__ h1,
                                       const uint32_t* nTDev, uint32_t* offsets) {
  const uint32_t nT = *nTDev;
  for (uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x; gid < nT; gid += gridDim.x * blockDim.x) {
    const uint32_t hitId = h1[gid];
    const uint32_t layerTriplet = hitLayer[hitId];
    const uint32_t event = hitEvt[hitId];
    if (gid > 0) {
      const uint32_t prev = h1[gid - 1];
      if (layerTriplet != hitLayer[prev] || event != hitEvt[prev])
        offsets[(size_t)event * cfg.nLT + layerTriplet - 1] = gid;
      if ((gid + 1) == nT) offsets[(size_t)event * cfg.nLT + layerTriplet] = gid;
    } else {
      offsets[(size_t)event * cfg.nLT + layerTriplet - 1] = gid;
    }
  }
}

}  // namespace

cudaError_t predict_pairs(const DevConfig& cfg, bool emit, const uint32_t* grid, DevHits hits, const uint2* pairs,
                          const uint32_t* nPairsDev, uint64_t maxPairs, uint32_t* candCount, uint2* cands,
                          uint64_t capCands, uint32_t* sentinels, uint32_t* err, cudaStream_t st,
                          uint32_t* launches) {
  (void)err;
  if (maxPairs == 0) return cudaSuccess;
  const uint32_t cap = capCands > 0xffffffffull ? 0xffffffffu : (uint32_t)capCands;
  const int blocks = grid_for(maxPairs, PRED_THREADS);
  if (emit)
    predict_kernel<true><<<blocks, PRED_THREADS, 0, st>>>(cfg, grid, hits.xyzp, hits.evt, hits.layer, pairs,
                                                          nPairsDev, candCount, cands, cap, sentinels);
  else
    predict_kernel<false><<<blocks, PRED_THREADS, 0, st>>>(cfg, grid, hits.xyzp, hits.evt, hits.layer, pairs,
                                                           nPairsDev, candCount, cands, cap, sentinels);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

cudaError_t predict_offsets(const DevConfig& cfg, DevHits hits, const uint2* pairs, const uint32_t* nPairsDev,
                            uint64_t maxPairs, const uint32_t* candStart, uint32_t* candOffsets, cudaStream_t st,
                            uint32_t* launches) {
  const uint32_t S = cfg.E * cfg.nLT;
  cudaError_t e = cudaMemsetAsync(candOffsets, 0, (S + 1) * sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  if (maxPairs > 0) {
    predict_offsets_kernel<<<grid_for(maxPairs, 256), 256, 0, st>>>(cfg, hits.evt, hits.layer, pairs, nPairsDev,
                                                                    candStart, candOffsets);
    if (launches) *launches += 1;
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return max_scan_inclusive(candOffsets, S + 1, st, launches);
}

cudaError_t filter_candidates(const DevConfig& cfg, DevHits hits, const uint2* pairs, const uint2* cands,
                              const uint32_t* nCandsDev, uint64_t maxCands, uint32_t* flags, cudaStream_t st,
                              uint32_t* launches) {
  filter_kernel<<<grid_for(maxCands + 1, 256), 256, 0, st>>>(cfg, hits.xyzp, hits.layer, pairs, cands, nCandsDev,
                                                              flags);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

cudaError_t filter_store(const uint2* pairs, const uint2* cands, const uint32_t* nCandsDev, uint64_t maxCands,
                         const uint32_t* flagScan, uint32_t* h1, uint32_t* h2, uint32_t* h3, uint64_t capT,
                         cudaStream_t st, uint32_t* launches) {
  if (maxCands == 0) return cudaSuccess;
  const uint32_t cap = capT > 0xffffffffull ? 0xffffffffu : (uint32_t)capT;
  filter_store_kernel<<<grid_for(maxCands, 256), 256, 0, st>>>(pairs, cands, nCandsDev, flagScan, h1, h2, h3, cap);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

cudaError_t triplet_offsets(const DevConfig& cfg, DevHits hits, const uint32_t* h1, const uint32_t* nTDev,
                            uint64_t maxT, uint32_t* offsets, cudaStream_t st, uint32_t* launches) {
  const uint32_t S = cfg.E * cfg.nLT;
  cudaError_t e = cudaMemsetAsync(offsets, 0, (S + 1) * sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  if (maxT > 0) {
    triplet_offsets_kernel<<<grid_for(maxT, 256), 256, 0, st>>>(cfg, hits.evt, hits.layer, h1, nTDev, offsets);
    if (launches) *launches += 1;
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return max_scan_inclusive(offsets, S + 1, st, launches);
}

}  // namespace trax
