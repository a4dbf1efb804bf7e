// trax_lookback.cuh -- decoupled look-back between the tiles of a
// single-pass scan (tiles numbered by an atomic ticket in launch order).
//
// Each tile publishes one 64-bit status word: 2 flag bits (0 = nothing yet,
// 1 = tile aggregate, 2 = inclusive prefix) and a 62-bit value, so that sums
// past 2^32 stay exact and a 32-bit overflow can be detected.  Warp 0 of a
// tile reads 32 predecessors at a time until it meets an inclusive prefix.
// The wait for a predecessor is bounded: after TRAX_SPIN_LIMIT polls (or the
// caller's limit) the tile records TRAX_EBIT_TIMEOUT, counts the missing
// predecessors as empty and finishes, so a lost tile can never hang the GPU.
#pragma once

#include "trax_device.cuh"

namespace trax {

constexpr unsigned long long LB_FLAG_AGG = 1ull << 62;
constexpr unsigned long long LB_FLAG_PREFIX = 2ull << 62;
constexpr unsigned long long LB_FLAG_MASK = 3ull << 62;
constexpr unsigned long long LB_VALUE_MASK = ~LB_FLAG_MASK;

__device__ __forceinline__ unsigned long long lb_load(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void lb_store(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Called by all 32 lanes of ONE warp with the tile's aggregate; returns (in
// every lane) the sum of all earlier tiles and publishes this tile's
// inclusive prefix.  `ctl` bounds the waits and names a tile that publishes
// nothing (a test fault).
__device__ __forceinline__ unsigned long long lb_exclusive_prefix(unsigned long long* status, uint32_t tile,
                                                                  unsigned long long agg, uint32_t* err,
                                                                  WaitCtl ctl) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t limit = ctl.spinLimit ? ctl.spinLimit : TRAX_SPIN_LIMIT;
  const bool publish = tile != ctl.skipTile;
  agg &= LB_VALUE_MASK;
  if (tile == 0) {
    if (lane == 0 && publish) lb_store(&status[0], LB_FLAG_PREFIX | agg);
    return 0ull;
  }
  if (lane == 0 && publish) lb_store(&status[tile], LB_FLAG_AGG | agg);
  unsigned long long excl = 0;
  int64_t pred = (int64_t)tile - 1;
  uint32_t spins = 0;
  while (true) {
    const int64_t idx = pred - (int64_t)lane;
    unsigned long long s = (idx >= 0) ? lb_load(&status[idx]) : (LB_FLAG_PREFIX | 0ull);
    unsigned long long flag = s & LB_FLAG_MASK;
    if (__any_sync(0xffffffffu, flag == 0ull)) {
      if (++spins < limit) {
        __nanosleep(64);
        continue;
      }
      if (lane == 0) raise_error(err, TRAX_EBIT_TIMEOUT);
      if (flag == 0ull) s = LB_FLAG_AGG;
      flag = s & LB_FLAG_MASK;
    }
    const unsigned long long val = s & LB_VALUE_MASK;
    const uint32_t pmask = __ballot_sync(0xffffffffu, flag == LB_FLAG_PREFIX);
    unsigned long long contrib = val;
    if (pmask) {
      const uint32_t first = __ffs(pmask) - 1;
      contrib = (lane <= first) ? val : 0ull;
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) contrib += __shfl_down_sync(0xffffffffu, contrib, d);
    excl += __shfl_sync(0xffffffffu, contrib, 0);
    if (pmask) break;
    pred -= 32;
  }
  if (lane == 0 && publish) lb_store(&status[tile], LB_FLAG_PREFIX | ((excl + agg) & LB_VALUE_MASK));
  return excl;
}

}  // namespace trax
