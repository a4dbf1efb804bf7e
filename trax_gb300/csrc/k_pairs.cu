// k_pairs.cu -- hit-pair generation from beamspot windows.
//
// Replaces pairCount / PrefixSum / pairStore (PairGeneratorBeamspot.h:43-525,
// PairGeneratorBeamspot.cpp:5-183) without the reference's n1 x n2 bit
// "oracle": the count pass counts, per outer hit, the valid visits of the
// reference's cell loop (duplicates included -- that is the reference's
// count), the exclusive scan turns counts into positions, and the store pass
// re-runs the window and writes the DISTINCT valid inner hits in ascending
// index order, which is the order pairStore's bitmap walk produces with one
// work-item per outer hit.  Slots the reference never writes (count larger
// than the distinct hits: windows wider than 2 pi) get the sentinel pair
// (0xffffffff, 0xffffffff).
//
// The visit set of one z row is the reference's j loop
//   for (j = grid[row + pL]; j < end2; ++j) index = j - (j >= zEnd) * len
// rewritten as two index ranges, P1 = [J0, min(end2, zEnd)) and
// P2 = [max(J0, zEnd) - len, end2 - len).  When all ranges of an outer hit
// are disjoint and can be ordered, the store pass walks them in ascending
// order; otherwise (only for NaN/inf or > 2 pi windows) it walks the whole
// inner layer and keeps the indices that some range contains.
#include "trax_kernels.h"

namespace trax {

namespace {


struct PairWindow {
  float zLow, zHigh, phiLow, phiHigh;
  uint32_t zLowSector, zHighSector, pL, pH;
  uint32_t wrap;
};

// The window arithmetic of pairCount (PairGeneratorBeamspot.h:111-162), in
// the reference's operation order (Q1 sigmaPhi bit pattern, Q2 signed
// radius, Q3 atan-then-divide, Q5 select-by-multiply).
__device__ __forceinline__ PairWindow pair_window(const DevConfig& cfg, uint32_t p, float x, float y, float z,
                                                  float phi) {
  const uint32_t layer = cfg.layer1[p] - 1;
  const float z0 = cfg.z0[p];
  const float tip = cfg.tipCut[p];
  const float sigmaZ = cfg.sigmaZ[p];
  const float sigmaPhi = cfg.pairSigmaPhi[p];
  const float minR1 = cfg.minR[layer];
  const float maxR1 = cfg.maxR[layer];
  PairWindow w;
  float signRadius = cl_sign(y);
  float r = signRadius * sqrt_(x * x + y * y);
  float cotThetaHigh = div_(z - z0, r);
  float cotThetaLow = div_(z + z0, r);
  float tmp = signRadius * maxR1 * cotThetaHigh + z0;
  float zHigh = signRadius * minR1 * cotThetaHigh + z0;
  zHigh = (float)(tmp < zHigh) * zHigh + (float)(tmp > zHigh) * tmp;
  tmp = signRadius * maxR1 * cotThetaLow - z0;
  float zLow = signRadius * minR1 * cotThetaLow - z0;
  zLow = (float)(tmp < zLow) * tmp + (float)(tmp > zLow) * zLow;
  zLow -= sigmaZ;
  zHigh += sigmaZ;
  w.zLowSector = (uint32_t)max(f2i_sat(floor_(div_(zLow - cfg.minZ, cfg.sZ))), 0);
  w.zHighSector = min(f2u_sat(floor_(div_(zHigh - cfg.minZ, cfg.sZ))) + 1u, cfg.nZ);
  const float twoR = 2 * cfg.minRcurv;
  const float aR = acos_(div_(r, twoR));
  tmp = fabs_(aR - cfg.acosMaxR[layer]);
  float dPhi = fabs_(aR - cfg.acosMinR[layer]);
  dPhi = (float)(tmp < dPhi) * dPhi + (float)(tmp > dPhi) * tmp;
  tmp = div_(atan_(tip * (r - minR1)), r * minR1);
  float phiHigh = div_(atan_(tip * (r - maxR1)), r * maxR1);
  dPhi += tmp > phiHigh ? tmp : phiHigh;
  float phiLow = phi - dPhi - sigmaPhi;
  phiHigh = phi + dPhi + sigmaPhi;
  const bool wrapAround = phiLow < -TRAX_PI_F || phiHigh > TRAX_PI_F || phiLow > TRAX_PI_F || phiHigh < -TRAX_PI_F;
  // (float)((x > pi) * 2) * pi is 2 pi (exact) or +0, as a select
  phiLow -= (phiLow > TRAX_PI_F) ? 2.0f * TRAX_PI_F : 0.0f;
  phiLow += (phiLow < -TRAX_PI_F) ? 2.0f * TRAX_PI_F : 0.0f;
  phiHigh -= (phiHigh > TRAX_PI_F) ? 2.0f * TRAX_PI_F : 0.0f;
  phiHigh += (phiHigh < -TRAX_PI_F) ? 2.0f * TRAX_PI_F : 0.0f;
  w.pL = f2u_sat(floor_(div_(phiLow - cfg.minPhi, cfg.sP)));
  w.pH = f2u_sat(floor_(div_(phiHigh - cfg.minPhi, cfg.sP)) + 1);
  w.zLow = zLow;
  w.zHigh = zHigh;
  w.phiLow = phiLow;
  w.phiHigh = phiHigh;
  w.wrap = wrapAround ? 1u : 0u;
  return w;
}

// pair_valid on (z, phi) with the phi test as two intervals, the second
// empty unless the window wraps
struct PairTest {
  float zl, zh, a1, b1, a2, b2;
};
__device__ __forceinline__ PairTest pair_test(const PairWindow& w) {
  const float inf = __int_as_float(0x7f800000);
  PairTest t;
  t.zl = w.zLow;
  t.zh = w.zHigh;
  t.a1 = w.phiLow;
  t.b1 = w.wrap ? TRAX_PI_F : w.phiHigh;
  t.a2 = w.wrap ? -TRAX_PI_F : inf;
  t.b2 = w.wrap ? w.phiHigh : -inf;
  return t;
}
__device__ __forceinline__ bool pair_ok(const PairTest& t, float2 h) {
  return t.zl <= h.x && h.x <= t.zh && ((t.a1 <= h.y && h.y <= t.b1) || (t.a2 <= h.y && h.y <= t.b2));
}

// The count pass's form of the window test (PairGeneratorBeamspot.h:192,
// :212-214).  The hits' angles come from atan2_ and lie in [-pi, pi] or are
// NaN, so a wrapped window's `phi <= pi` and `-pi <= phi` always hold: its
// phi test is lo || hi, a plain window's lo && hi (NaN fails both, as in the
// reference's form).  The store pass keeps the forms below, which measured
// faster there.
__device__ __forceinline__ bool pair_count_ok(const PairWindow& w, float4 h) {
  const bool lo = w.phiLow <= h.w, hi = h.w <= w.phiHigh;
  return w.zLow <= h.z && h.z <= w.zHigh && (w.wrap ? (lo || hi) : (lo && hi));
}

__device__ __forceinline__ bool pair_valid(const PairWindow& w, float4 h) {
  bool valid = w.zLow <= h.z && h.z <= w.zHigh;
  const float actPhi = h.w;
  return valid && ((!w.wrap && (w.phiLow <= actPhi && actPhi <= w.phiHigh)) ||
                   (w.wrap && ((w.phiLow <= actPhi && actPhi <= TRAX_PI_F) ||
                               (-TRAX_PI_F <= actPhi && actPhi <= w.phiHigh))));
}

// visit ranges of one z row (pair generation: zEnd is the start of the phi
// overflow column, PairGeneratorBeamspot.h:174-185)
__device__ __forceinline__ void pair_row_parts(const PairWindow& w, const uint32_t* lG, uint32_t C, uint32_t nP,
                                               uint32_t zs, uint32_t& a1, uint32_t& b1, uint32_t& a2,
                                               uint32_t& b2) {
  const uint32_t row = zs * (nP + 1);
  const uint32_t zStart = cell_at(lG, row, C);
  const uint32_t zEnd = cell_at(lG, row + nP, C);  // (zSector+1)*(nP+1)-1
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

// One row of the ordering check: its two ranges are disjoint and both start
// at or after prevEnd, the end of everything before (advanced here).
__device__ __forceinline__ bool rows_in_order(uint32_t a1, uint32_t b1, uint32_t a2, uint32_t b2,
                                              uint32_t& prevEnd) {
  const bool n1 = a1 < b1, n2 = a2 < b2;
  bool ok = true;
  if (n1 && n2) {
    if (b2 <= a1) {
      ok = a2 >= prevEnd;
      prevEnd = b1;
    } else if (b1 <= a2) {
      ok = a1 >= prevEnd;
      prevEnd = b2;
    } else {
      ok = false;
    }
  } else if (n1) {
    ok = a1 >= prevEnd;
    prevEnd = b1;
  } else if (n2) {
    ok = a2 >= prevEnd;
    prevEnd = b2;
  }
  return ok;
}

__device__ __forceinline__ uint32_t find_segment(const uint32_t* taskBase, uint32_t S, uint32_t k) {
  // largest s with taskBase[s] <= k
  uint32_t lo = 0, hi = S;  // taskBase[S] > k
  while (hi - lo > 1) {
    uint32_t mid = (lo + hi) >> 1;
    if (taskBase[mid] <= k) lo = mid;
    else hi = mid;
  }
  return lo;
}

__global__ void segments_kernel(DevConfig cfg, const uint32_t* __restrict__ grid, uint32_t* segOuter,
                                uint32_t* segCount) {
  const uint32_t S = cfg.E * cfg.nLT;
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < S; s += gridDim.x * blockDim.x) {
    const uint32_t e = s / cfg.nLT, p = s % cfg.nLT;
    const uint32_t* lG2 = grid + ((size_t)e * cfg.L + (cfg.layer2[p] - 1)) * cfg.C;
    const uint32_t l2off = lG2[0];
    segOuter[s] = l2off;
    segCount[s] = lG2[cfg.C - 1] - l2off;  // PairGeneratorBeamspot.h:70-73
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) segCount[S] = 0u;
}

template <bool EMIT>
__global__ void __launch_bounds__(TRAX_MAX_TUNED_THREADS)
    pair_kernel(DevConfig cfg, const uint32_t* __restrict__ grid, const float4* __restrict__ hits,
                const uint32_t* __restrict__ segOuter, const uint32_t* __restrict__ taskBase,
                const uint32_t* __restrict__ nTasksDev, uint32_t* taskCount, PairTaskState state, uint2* pairs,
                uint32_t capPairs, uint32_t* sentinels, uint32_t* err) {
  const uint32_t S = cfg.E * cfg.nLT;
  const uint32_t nTasks = *nTasksDev;
  const uint32_t C = cfg.C, nP = cfg.nP;
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nTasks; k += gridDim.x * blockDim.x) {
    uint32_t s, i;
    PairWindow w;
    bool ordered = false;
    if (!EMIT) {
      s = find_segment(taskBase, S, k);
      i = segOuter[s] + (k - taskBase[s]);
      const float4 ho = hits[trax_hit(i, cfg)];
      w = pair_window(cfg, s % cfg.nLT, ho.x, ho.y, ho.z, ho.w);
    } else {
      // the count pass's window, segment and ordering of this task
      const float4 b = state.bounds[k];
      const uint4 q = state.secs[k];
      const uint2 id = state.ids[k];
      i = id.x;
      s = id.y;
      w.zLow = b.x;
      w.zHigh = b.y;
      w.phiLow = b.z;
      w.phiHigh = b.w;
      w.zLowSector = q.x & 0x7fffffffu;
      w.zHighSector = q.y & 0x7fffffffu;
      w.pL = q.z;
      w.pH = q.w;
      w.wrap = q.y >> 31;
      ordered = (q.x >> 31) != 0u;
    }
    const uint32_t e = s / cfg.nLT, p = s % cfg.nLT;
    const uint32_t* lG1 = grid + ((size_t)e * cfg.L + (cfg.layer1[p] - 1)) * C;
    if (!EMIT) {
      uint32_t nFound = 0;
      // whether the rows' ranges are disjoint and ascending, for the store
      bool simple = true;
      uint32_t prevEnd = 0;
      for (uint32_t zs = w.zLowSector; zs < w.zHighSector; ++zs) {
        uint32_t a1, b1, a2, b2;
        pair_row_parts(w, lG1, C, nP, zs, a1, b1, a2, b2);
        if (simple) simple = rows_in_order(a1, b1, a2, b2, prevEnd);
        for (uint32_t j = a1; j < b1; ++j) nFound += pair_count_ok(w, hits[trax_hit(j, cfg)]);
        for (uint32_t j = a2; j < b2; ++j) nFound += pair_count_ok(w, hits[trax_hit(j, cfg)]);
      }
      taskCount[k] = nFound;
      state.bounds[k] = make_float4(w.zLow, w.zHigh, w.phiLow, w.phiHigh);
      state.secs[k] = make_uint4(w.zLowSector | (simple ? 0x80000000u : 0u), w.zHighSector | (w.wrap << 31), w.pL,
                                 w.pH);
      state.ids[k] = make_uint2(i, s);
    } else {
      const uint32_t pos0 = taskCount[k];
      uint32_t limit = taskCount[k + 1] - pos0;
      if (pos0 >= capPairs) limit = 0;
      else if (limit > capPairs - pos0) limit = capPairs - pos0;
      uint2* out = pairs + pos0;
      // the count pass checked the ordering of the ranges
      const bool simple = ordered;
      uint32_t written = 0;
      if (simple) {
        // the common path tests (z, phi) pairs: 8 bytes per visited hit
        const PairTest t = pair_test(w);
        const float2* zphi = reinterpret_cast<const float2*>(hits) + 1;  // (z, phi) of hit j at zphi[2 j]
        for (uint32_t zs = w.zLowSector; zs < w.zHighSector; ++zs) {
          uint32_t a1, b1, a2, b2;
          pair_row_parts(w, lG1, C, nP, zs, a1, b1, a2, b2);
          uint32_t lo0 = a1, hi0 = b1, lo1 = a2, hi1 = b2;
          if (a2 < b2 && b2 <= a1) {  // P2 precedes P1
            lo0 = a2; hi0 = b2; lo1 = a1; hi1 = b1;
          }
          for (uint32_t j = lo0; j < hi0; ++j)
            if (pair_ok(t, __ldg(zphi + 2 * (size_t)trax_hit(j, cfg)))) {
              if (written < limit) out[written] = make_uint2(j, i);
              ++written;
            }
          for (uint32_t j = lo1; j < hi1; ++j)
            if (pair_ok(t, __ldg(zphi + 2 * (size_t)trax_hit(j, cfg)))) {
              if (written < limit) out[written] = make_uint2(j, i);
              ++written;
            }
        }
        if (written != limit) raise_error(err, TRAX_EBIT_BOUNDS);
      } else {
        // exact slow path: every inner index that some visit range contains
        const uint32_t innerBegin = lG1[0], innerEnd = lG1[C - 1];
        for (uint32_t j = innerBegin; j < innerEnd && written < limit; ++j) {
          bool visited = false;
          for (uint32_t zs = w.zLowSector; zs < w.zHighSector && !visited; ++zs) {
            uint32_t a1, b1, a2, b2;
            pair_row_parts(w, lG1, C, nP, zs, a1, b1, a2, b2);
            visited = (a1 <= j && j < b1) || (a2 <= j && j < b2);
          }
          if (visited && pair_valid(w, hits[trax_hit(j, cfg)])) out[written++] = make_uint2(j, i);
        }
      }
      if (written < limit) {
        atomicAdd(sentinels, limit - written);
        for (uint32_t q = written; q < limit; ++q) out[q] = make_uint2(TRAX_SENTINEL, TRAX_SENTINEL);
      }
    }
  }
  if (!EMIT && blockIdx.x == 0 && threadIdx.x == 0) taskCount[nTasks] = 0u;  // the scan's +1 slot
}

__global__ void pair_offsets_kernel(DevConfig cfg, const uint32_t* taskBase, const uint32_t* pairStart,
                                    uint32_t* pairOffsets) {
  const uint32_t S = cfg.E * cfg.nLT;
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s <= S; s += gridDim.x * blockDim.x)
    pairOffsets[s] = s == 0 ? 0u : pairStart[taskBase[s]];
}

int grid_for(uint64_t items, int threads) {
  uint64_t blocks = (items + threads - 1) / threads;
  uint64_t cap = (uint64_t)sm_count() * (4096 / threads);  // two waves at full occupancy
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  return (int)blocks;
}

}  // namespace

cudaError_t pair_segments(const DevConfig& cfg, const uint32_t* grid, uint32_t* segOuter, uint32_t* segCount,
                          cudaStream_t st, uint32_t* launches) {
  const uint32_t S = cfg.E * cfg.nLT;
  segments_kernel<<<grid_for(S + 1, 256), 256, 0, st>>>(cfg, grid, segOuter, segCount);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

cudaError_t pair_tasks(const DevConfig& cfg, bool emit, const uint32_t* grid, DevHits hits, const uint32_t* segOuter,
                       const uint32_t* taskBase, const uint32_t* nTasksDev, uint64_t maxTasks, uint32_t* taskCount,
                       PairTaskState state, uint2* pairs, uint64_t capPairs, uint32_t* sentinels, uint32_t* err,
                       cudaStream_t st, uint32_t* launches) {
  const uint32_t cap = capPairs > 0xffffffffull ? 0xffffffffu : (uint32_t)capPairs;
  if (emit && maxTasks == 0) return cudaSuccess;
  const int threads = (int)cfg.pairThreads;
  const int blocks = grid_for(maxTasks + 1, threads);
  if (emit)
    pair_kernel<true><<<blocks, threads, 0, st>>>(cfg, grid, hits.xyzp, segOuter, taskBase, nTasksDev,
                                                       taskCount, state, pairs, cap, sentinels, err);
  else
    pair_kernel<false><<<blocks, threads, 0, st>>>(cfg, grid, hits.xyzp, segOuter, taskBase, nTasksDev,
                                                        taskCount, state, pairs, cap, sentinels, err);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

cudaError_t pair_offsets(const DevConfig& cfg, const uint32_t* taskBase, const uint32_t* pairStart,
                         uint32_t* pairOffsets, cudaStream_t st, uint32_t* launches) {
  const uint32_t S = cfg.E * cfg.nLT;
  pair_offsets_kernel<<<grid_for(S + 1, 256), 256, 0, st>>>(cfg, taskBase, pairStart, pairOffsets);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

}  // namespace trax
