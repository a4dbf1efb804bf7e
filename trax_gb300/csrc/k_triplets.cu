// k_triplets.cu -- third-hit prediction and the dtheta/dphi/TIP filter.
//
// Prediction replaces predictCount / predictStore / predictOffsetMonotonizeStore
// (TripletThetaPhiPredictor.h:49-447, .cpp:10-168): one thread per pair, the
// count pass with predictCount's rOrigin and the store pass with
// predictStore's (Q4: sqrt(x^2+y^2-tip2) vs sqrt(sqrt(x^2+y^2)^2-tip2)), the
// store capped at the count exactly like `pos < nextThread`.  Slots the store
// pass cannot fill (the reference leaves them unwritten) get the candidate
// (pair, 0xffffffff), which the filter rejects.  Both passes can walk a
// finer z grid instead of the grid's rows (fine_walk, cfg.fineRows) with the
// same results.
//
// The filter replaces filterCount / filterPopCount / PrefixSum / filterStore /
// filterOffsetStore / filterOffsetMonotonizeStore (TripletThetaPhiFilter.h:50-280,
// .cpp:10-206): a flag per candidate (one bit of a word of 32), a scan of
// the words' counts and a stable scatter of (h1, h2, h3) keep the candidate
// order of the reference.
#include "trax_kernels.h"
#include "trax_stages.cuh"

namespace trax {

namespace {


int grid_for(uint64_t items, int threads) {
  uint64_t blocks = (items + threads - 1) / threads;
  uint64_t cap = (uint64_t)sm_count() * (4096 / threads);  // two waves at full occupancy
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  return (int)blocks;
}

// The store pass's candidates of pair gid as capture slots: slot q is the
// hit of out[q], written as (gid, hit).
struct CandSlots {
  uint2* out;
  uint32_t gid;
  struct Ref {
    uint2* e;
    uint32_t gid;
    __device__ __forceinline__ operator uint32_t() const { return e->y; }
    __device__ __forceinline__ Ref& operator=(uint32_t v) {
      *e = make_uint2(gid, v);
      return *this;
    }
    __device__ __forceinline__ Ref& operator=(const Ref& o) { return *this = (uint32_t)o; }
  };
  __device__ __forceinline__ Ref operator[](uint32_t q) const { return Ref{out + q, gid}; }
};

// The prediction's walk over the fine z grid (cfg.fineRows rows per z row),
// for windows with pL <= nP, in the count pass and in the store pass's
// re-walks.  It visits the same hits as the walk over the grid, each as
// often, so the counts are the same:
//  - the grid walk visits, in each z row r of [zLo, zHi), the hits of the
//    row's phi columns [pL, pH) (no wrap), or [pL, nP] and then [0, pH)
//    (wrap; both parts when pH > pL, so such hits twice) -- pred_row_parts
//    for pL <= nP, with pH <= nP always;
//  - here, for each of r's parts, the fine rows of r's block that meet
//    [fine_row(zl), fine_row(zh)], the union window's bounds; a hit passing
//    either variant's z test has zl <= z <= zh, and fine_row is monotone
//    and keeps it in its grid row's block, so its fine row is among them.
//    Hits outside those rows fail both z tests, as in the grid walk.
// The captured candidates are the first nKeep store-valid visits in the
// grid walk's order, (row, part, grid index): the visits of one (row, part)
// come here in fine order, so the slots of the current (row, part) are kept
// sorted by grid index -- appended while they come in order (the largest
// is kept in a register), inserted otherwise -- and a visit past the last
// slot replaces the largest of them when it is smaller.  COUNT: count the
// count variant's valid visits too (the count pass); otherwise (the store
// pass's re-walk, both variants the store variant) stop at the first
// (row, part) after nKeep captures, which can add nothing.
template <bool COUNT, class Slots>
__device__ __forceinline__ void fine_walk(const DevConfig& cfg, const PredUnionWindow& w, const FineGrid& fine,
                                          uint32_t event, uint32_t layer, Slots slot, uint32_t nKeep,
                                          uint32_t& count, uint32_t& nStore) {
  const uint32_t F = cfg.fineRows, Cf = cfg.fineC, nP = cfg.nP;
  const uint32_t* lG = fine.grid + ((size_t)event * cfg.L + layer) * Cf;
  // zl, zh as pred_union_window (a switched-off variant holds +inf, -inf);
  // their grid rows are min(zLo, nZ - 1) and zHi - 1 (zHi >= 1 when any)
  const float zl = fminf(w.zLow[0], w.zLow[1]), zh = fmaxf(w.zHigh[0], w.zHigh[1]);
  const uint32_t fLo = fine_row(cfg, zl, min(w.zLo, cfg.nZ - 1u));
  const uint32_t fHi = w.zHi ? fine_row(cfg, zh, w.zHi - 1u) + 1u : 0u;
  const bool wrap = w.wrap != 0u;
  const float zl0 = w.zLow[0], zh0 = w.zHigh[0], zl1 = w.zLow[1], zh1 = w.zHigh[1];
  for (uint32_t r = w.zLo; r < w.zHi; ++r) {
    const uint32_t f0 = max(F * r, fLo), f1 = min(F * r + F, fHi);
    for (uint32_t part = 0; part <= w.wrap; ++part) {
      if (!COUNT && nStore >= nKeep) return;
      const uint32_t cs = nStore;  // the first visit of this (row, part)
      uint32_t last = 0u;          // the largest kept of this (row, part), at min(nStore, nKeep) - 1
      // part 0: columns [pL, pH), or [pL, nP] under wrap; part 1: [0, pH)
      const uint32_t ca = part ? 0u : w.pL;
      const uint32_t cb = (wrap && !part) ? nP + 1u : w.pH;
      for (uint32_t fr = f0; fr < f1; ++fr) {
        const uint32_t row = fr * (nP + 1u);
        const uint32_t a = cell_at(lG, row + ca, Cf);
        const uint32_t b = max(a, cell_at(lG, row + cb, Cf));
#pragma unroll 1  // a few hits per fine row: unrolled by 4 it measured slower (12.8 vs 12.4 ms)
        for (uint32_t jf = a; jf < b; ++jf) {
          const float4 h = __ldg(fine.hits + trax_hit(jf, cfg));  // (z, phi, grid index, 0)
          const bool lo = w.phiLow <= h.y, hi = h.y <= w.phiHigh;
          const bool phiOk = wrap ? (lo || hi) : (lo && hi);
          if (COUNT) count += (phiOk && zl0 <= h.x && h.x <= zh0);
          if (phiOk && zl1 <= h.x && h.x <= zh1) {
            const uint32_t j = __float_as_uint(h.z);
            if (nStore < nKeep) {
              if (nStore == cs || j > last) {  // in grid order: append
                slot[nStore] = j;
                last = j;
              } else {  // before `last`: move the larger ones up (the largest stays `last`)
                uint32_t q = nStore;
                slot[q--] = last;
                while (q > cs && slot[q - 1u] > j) {
                  slot[q] = slot[q - 1u];
                  --q;
                }
                slot[q] = j;
              }
            } else if (cs < nKeep && j < last) {  // replaces the largest kept, at nKeep - 1
              uint32_t q = nKeep - 1u, top = j;
              while (q > cs) {
                const uint32_t v = slot[q - 1u];
                if (v <= j) break;
                slot[q] = v;
                if (q == nKeep - 1u) top = v;
                --q;
              }
              slot[q] = j;
              last = top;
            }
            ++nStore;
          }
        }
      }
    }
  }
}

// Count pass (predictCount, :190-219) that also captures the first
// min(count, cfg.predKeep) candidates the store pass would write (the store
// variant's valid hits, capped at the count; slots it would leave unwritten
// get the sentinel), so that the store pass is a copy for most pairs.
// The prefix sum between predictCount and predictStore is split in two:
// every warp scans its 32 consecutive counts with shuffles and writes the
// exclusive offsets within the warp to candCount and the warp's sum to
// warpSums; only those sums (one per 32 pairs) are then scanned, and a
// pair's position is its warp's scanned sum plus its offset in the warp.
// At most 40 registers (six blocks of 256 threads per SM), where it spills
// nothing; 32 registers (eight blocks) spill and measured slower, as did 48.
//
// FINE: the walk goes over the fine z grid instead (fine_walk), with the
// same counts and captured candidates.  IL: the slots' layout (keep_slots).
template <bool FINE, bool IL>
__global__ void __launch_bounds__(TRAX_MAX_TUNED_THREADS, 6)
    predict_count_kernel(DevConfig cfg, const uint32_t* __restrict__ grid, const float4* __restrict__ hits,
                         const uint32_t* __restrict__ hitEvt, const uint32_t* __restrict__ hitLayer,
                         const uint2* __restrict__ pairs, const uint32_t* __restrict__ nPairsDev, uint32_t* candCount,
                         uint32_t* keep, uint32_t* warpSums, uint32_t* nWarpsOut, uint32_t* err, FineGrid fine) {
  const uint32_t nPairs = *nPairsDev;
  const uint32_t lane = threadIdx.x & 31u;
  // warp-uniform loop: each warp covers 32 consecutive pairs per step
  for (uint32_t base = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < nPairs;
       base += gridDim.x * blockDim.x) {
    const uint32_t gid = base + lane;
    const uint2 pr = gid < nPairs ? pairs[gid] : make_uint2(TRAX_SENTINEL, TRAX_SENTINEL);
    uint32_t count = 0;
    if (pr.x != TRAX_SENTINEL) {
      const uint32_t hx = trax_hit(pr.x, cfg), hy = trax_hit(pr.y, cfg);
      const uint32_t event = hitEvt[hx];
      const uint32_t lt = hitLayer[hx] - 1;  // Q7
      const uint32_t layer = cfg.layer3[lt] - 1;
      const uint32_t* lG3 = grid + ((size_t)event * cfg.L + layer) * cfg.C;
      const PredUnionWindow w = pred_union_window(cfg, lt, layer, hits[hx], hits[hy]);
      // One walk over the union of both variants' z rows with each
      // variant's own z test (pred_union_window: a hit outside a variant's
      // rows fails its test); the phi test is common.  Each variant's valid
      // hits come out in its own visit order.
      const uint32_t C = cfg.C, nP = cfg.nP;
      const uint32_t nKeep = cfg.predKeep;
      const KeepSlots<IL, uint32_t> slot = keep_slots<IL>(keep, gid, nKeep);
      uint32_t nStore = 0;
      // The phi test (TripletThetaPhiPredictor.h:211-214) on hit angles
      // from atan2_, which lie in [-pi, pi] or are NaN: the wrapped window's
      // `phi <= pi` and `-pi <= phi` always hold, so it is lo || hi, the
      // plain one lo && hi (NaN fails both, as in the reference's form).
      const bool wrap = w.wrap != 0u;
      const float zl0 = w.zLow[0], zh0 = w.zHigh[0], zl1 = w.zLow[1], zh1 = w.zHigh[1];
      const float2* zphi = reinterpret_cast<const float2*>(hits) + 1;  // (z, phi) of hit j at zphi[2 j]
      if (FINE && w.pL <= nP) {
        fine_walk<true>(cfg, w, fine, event, layer, slot, nKeep, count, nStore);
      } else
      for (uint32_t zs = w.zLo; zs < w.zHi; ++zs) {
        uint32_t a[2], b[2];
        if (!wrap && w.pL <= nP) {
          // pred_row_parts' result without the row's start and end: a
          // window that does not wrap visits the columns [pL, pH) of the
          // row (pH <= nP), and its second part is empty
          const uint32_t row = zs * (nP + 1);
          a[0] = cell_at(lG3, row + w.pL, C);
          b[0] = max(a[0], cell_at(lG3, row + w.pH, C));
          a[1] = b[1] = 0u;
        } else {
          pred_row_parts(w, lG3, C, nP, zs, a[0], b[0], a[1], b[1]);
        }
#pragma unroll
        for (int part = 0; part < 2; ++part) {
#pragma unroll 4
          for (uint32_t j = a[part]; j < b[part]; ++j) {
            const float2 h = __ldg(zphi + 2 * (size_t)trax_hit(j, cfg));
            const bool lo = w.phiLow <= h.y, hi = h.y <= w.phiHigh;
            const bool phiOk = wrap ? (lo || hi) : (lo && hi);
            count += (phiOk && zl0 <= h.x && h.x <= zh0);
            if (phiOk && zl1 <= h.x && h.x <= zh1) {
              if (nStore < nKeep) slot[nStore] = j;
              ++nStore;
            }
          }
        }
      }
      // the store pass writes at most `count` candidates; missing ones are
      // slots the reference leaves unwritten
      const uint32_t k = min(count, nKeep);
      for (uint32_t q = nStore; q < k; ++q) slot[q] = TRAX_SENTINEL;
    }
    uint32_t incl = count;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= (uint32_t)d) incl += t;
    }
    if (gid < nPairs) candCount[gid] = incl - count;
    // 32 counts can pass 2^32 only if one of them reaches 2^27
    if (__reduce_max_sync(0xffffffffu, count) >= (1u << 27)) {
      unsigned long long sum = count;
      for (int d = 16; d > 0; d >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, d);
      if (lane == 0 && sum > 0xffffffffull) raise_error(err, TRAX_EBIT_OVERFLOW);
    }
    if (lane == 31) warpSums[base >> 5] = incl;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const uint32_t nW = (nPairs + 31u) >> 5;
    warpSums[nW] = 0u;  // the scan's +1 slot
    *nWarpsOut = nW;
  }
}

// The count pass with K pairs per thread.  A warp takes 32 K consecutive
// pairs; lane l owns pairs base + 32 k + l (k < K), so every group of 32
// consecutive pairs is still scanned by one warp as in predict_count_kernel
// and the outputs are the same.  The windows of a lane's K pairs are
// computed first, in lockstep, and staged in shared memory; the lane then
// walks the visit ranges of its K pairs one after the other in one flat
// loop, one visit per step.  The slowest lane of a warp then sets the pace
// of K pairs together instead of each pair separately: per-lane work is a
// sum over K pairs, which varies less between lanes than one pair's visits
// (3.9 visits per pair on average, 8.9 for the slowest lane of a warp on the
// ttbar-like workload).  Each pair's visits keep their order (rows, then
// the two parts of a row, then hits), so the counts and the captured
// candidates equal predict_count_kernel's.
struct PredStage {
  float zLow[2], zHigh[2], phiLow, phiHigh;
  uint32_t sec[2];     // zLoSec | zHiSec << 16 of each variant
  uint32_t pLpH;       // pL | pH << 16
  uint32_t flags;      // bit 0 wrap, bit 1 a real pair
  uint32_t gridOff;    // first cell of the third layer of the pair's event
};

template <int K>
__global__ void __launch_bounds__(TRAX_MAX_TUNED_THREADS, 4)
    predict_count_k_kernel(DevConfig cfg, const uint32_t* __restrict__ grid, const float4* __restrict__ hits,
                           const uint32_t* __restrict__ hitEvt, const uint32_t* __restrict__ hitLayer,
                           const uint2* __restrict__ pairs, const uint32_t* __restrict__ nPairsDev,
                           uint32_t* candCount, uint32_t* keep, uint32_t* warpSums, uint32_t* nWarpsOut,
                           uint32_t* err) {
  extern __shared__ PredStage s_stage[];  // [warp][k][lane]
  const uint32_t nPairs = *nPairsDev;
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t warpsTotal = gridDim.x * (blockDim.x >> 5);
  PredStage* st = s_stage + (size_t)warp * K * 32 + lane;  // st[32 k]: this lane's pair k
  const float inf = __int_as_float(0x7f800000);
  const float2* zphi = reinterpret_cast<const float2*>(hits) + 1;  // (z, phi) of hit j at zphi[2 j]
  const uint32_t C = cfg.C, nP = cfg.nP;
  for (uint32_t base = (blockIdx.x * (blockDim.x >> 5) + warp) * 32u * K; base < nPairs;
       base += warpsTotal * 32u * K) {
    // windows of the K pairs, in lockstep
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const uint32_t gid = base + 32u * k + lane;
      const uint2 pr = gid < nPairs ? pairs[gid] : make_uint2(TRAX_SENTINEL, TRAX_SENTINEL);
      PredStage& ps = st[32 * k];
      if (pr.x != TRAX_SENTINEL) {
        const uint32_t hx = trax_hit(pr.x, cfg), hy = trax_hit(pr.y, cfg);
        const uint32_t event = hitEvt[hx];
        const uint32_t lt = hitLayer[hx] - 1;  // Q7
        const uint32_t layer = cfg.layer3[lt] - 1;
        const PredWindow w = pred_window(cfg, lt, layer, hits[hx], hits[hy]);
        ps.zLow[0] = w.zLow[0];
        ps.zHigh[0] = w.zHigh[0];
        ps.zLow[1] = w.zLow[1];
        ps.zHigh[1] = w.zHigh[1];
        ps.phiLow = w.phiLow;
        ps.phiHigh = w.phiHigh;
        ps.sec[0] = w.zLoSec[0] | (w.zHiSec[0] << 16);
        ps.sec[1] = w.zLoSec[1] | (w.zHiSec[1] << 16);
        ps.pLpH = w.pL | (w.pH << 16);
        ps.flags = w.wrap | 2u;
        ps.gridOff = (event * cfg.L + layer) * C;
      } else {
        ps.flags = 0u;
      }
    }
    // the flat walk over the lane's K pairs
    uint32_t cnt = 0, nStore = 0;  // of the current pair
    int k = -1;
    uint32_t zs = 0, zHi = 0, j = 0, end = 0, a1 = 0, b1 = 0, part = 1;
    uint32_t zlo[2] = {0, 0}, zhi[2] = {0, 0};
    float zl0 = inf, zh0 = -inf, zl1 = inf, zh1 = -inf, pa1 = 0, pb1 = 0, pa2 = inf, pb2 = -inf;
    float zLow0 = 0, zHigh0 = 0, zLow1 = 0, zHigh1 = 0;
    PredWindow rw;  // pL, pH and wrap for pred_row_parts
    rw.pL = rw.pH = rw.wrap = 0;
    const uint32_t* lG3 = grid;
    KeepSlots<false, uint32_t> slot{keep};
    uint32_t counts[K];
#pragma unroll
    for (int q = 0; q < K; ++q) counts[q] = 0;
    // moves to the next non-empty visit range; false when the lane is done
    auto advance = [&]() -> bool {
      for (;;) {
        if (part == 0) {
          part = 1;
          j = a1;
          end = b1;
          if (j < end) return true;
          continue;
        }
        if (k >= 0 && zs + 1 < zHi) {
          ++zs;
        } else {
          if (k >= 0) {
            // the pair's end: store-pass slots past the valid hits get the sentinel
            const uint32_t kk = min(cnt, cfg.predKeep);
            for (uint32_t q = nStore; q < kk; ++q) slot[q] = TRAX_SENTINEL;
#pragma unroll
            for (int q = 0; q < K; ++q)
              if (q == k) counts[q] = cnt;
          }
          // the next real pair with rows to walk
          for (;;) {
            if (++k >= K) return false;
            const PredStage& ps = st[32 * k];
            if (!(ps.flags & 2u)) continue;
            cnt = nStore = 0;
            zLow0 = ps.zLow[0];
            zHigh0 = ps.zHigh[0];
            zLow1 = ps.zLow[1];
            zHigh1 = ps.zHigh[1];
            zlo[0] = ps.sec[0] & 0xffffu;
            zhi[0] = ps.sec[0] >> 16;
            zlo[1] = ps.sec[1] & 0xffffu;
            zhi[1] = ps.sec[1] >> 16;
            rw.pL = ps.pLpH & 0xffffu;
            rw.pH = ps.pLpH >> 16;
            rw.wrap = ps.flags & 1u;
            pa1 = ps.phiLow;
            pb1 = rw.wrap ? TRAX_PI_F : ps.phiHigh;
            pa2 = rw.wrap ? -TRAX_PI_F : inf;
            pb2 = rw.wrap ? ps.phiHigh : -inf;
            lG3 = grid + ps.gridOff;
            slot = keep_slots<false>(keep, base + 32u * k + lane, cfg.predKeep);
            zs = min(zlo[0], zlo[1]);
            zHi = max(zhi[0], zhi[1]);
            if (zs < zHi) break;
            // no rows: the pair counts nothing
#pragma unroll
            for (int q = 0; q < K; ++q)
              if (q == k) counts[q] = 0;
          }
        }
        // a row: each variant's z interval (empty outside its rows) and the two parts
        const bool in0 = zs >= zlo[0] && zs < zhi[0];
        const bool in1 = zs >= zlo[1] && zs < zhi[1];
        zl0 = in0 ? zLow0 : inf;
        zh0 = in0 ? zHigh0 : -inf;
        zl1 = in1 ? zLow1 : inf;
        zh1 = in1 ? zHigh1 : -inf;
        uint32_t a0, b0;
        pred_row_parts(rw, lG3, C, nP, zs, a0, b0, a1, b1);
        part = 0;
        j = a0;
        end = b0;
        if (j < end) return true;
      }
    };
    bool live = advance();
    while (__any_sync(0xffffffffu, live)) {
      if (live) {
        const float2 h = __ldg(zphi + 2 * (size_t)trax_hit(j, cfg));
        const bool phiOk = (pa1 <= h.y && h.y <= pb1) || (pa2 <= h.y && h.y <= pb2);
        cnt += (phiOk && zl0 <= h.x && h.x <= zh0);
        if (phiOk && zl1 <= h.x && h.x <= zh1) {
          if (nStore < cfg.predKeep) slot[nStore] = j;
          ++nStore;
        }
        if (++j >= end) live = advance();
      }
    }
    // the per-32-pair scans, as predict_count_kernel
#pragma unroll
    for (int q = 0; q < K; ++q) {
      const uint32_t gid = base + 32u * q + lane;
      const uint32_t count = counts[q];
      uint32_t incl = count;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= (uint32_t)d) incl += t;
      }
      if (gid < nPairs) candCount[gid] = incl - count;
      if (__reduce_max_sync(0xffffffffu, count) >= (1u << 27)) {
        unsigned long long sum = count;
        for (int d = 16; d > 0; d >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, d);
        if (lane == 0 && sum > 0xffffffffull) raise_error(err, TRAX_EBIT_OVERFLOW);
      }
      if (lane == 31 && base + 32u * q < nPairs) warpSums[(base >> 5) + q] = incl;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const uint32_t nW = (nPairs + 31u) >> 5;
    warpSums[nW] = 0u;  // the scan's +1 slot
    *nWarpsOut = nW;
  }
}

// Store pass (predictStore, :358-402): candidates (pair, hit3) at the
// scanned position; copied from the captured slots, re-walked only when a
// pair has more candidates than slots.
// At most 32 registers: full occupancy hides the latency of the dependent
// loads better than the few spilled bytes cost (0.61 -> 0.49 ms).
// IL: the slots' layout (keep_slots).  FINE: the re-walks go over the fine
// z grid (fine_walk with the store variant as both variants, its captures
// written straight to the pair's candidates), with the same candidates; it
// gets 40 registers, where it spills nothing (pileup batch: 4.03 ms with
// the grid walk, 4.34 ms fine at 32 registers with 80 B spilled, 3.46 ms
// at 40).
template <bool IL, bool FINE>
__global__ void __launch_bounds__(TRAX_MAX_TUNED_THREADS, FINE ? 6 : 8)
    predict_store_kernel(DevConfig cfg, const uint32_t* __restrict__ grid, const float4* __restrict__ hits,
                         const uint32_t* __restrict__ hitEvt, const uint32_t* __restrict__ hitLayer,
                         const uint2* __restrict__ pairs, const uint32_t* __restrict__ nPairsDev,
                         const uint32_t* __restrict__ local, const uint32_t* __restrict__ warpStart,
                         const uint32_t* __restrict__ keep, uint2* cands, uint32_t capCands, uint32_t* sentinels,
                         FineGrid fine) {
  const uint32_t nPairs = *nPairsDev;
  uint32_t sent = 0;
  for (uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x; gid < nPairs; gid += gridDim.x * blockDim.x) {
    const uint32_t wi = gid >> 5;
    const uint32_t off = local[gid];
    const uint32_t pos = warpStart[wi] + off;
    // the next pair's position: the next warp's start after a warp's last pair
    uint32_t limit = ((gid & 31u) == 31u || gid + 1 == nPairs) ? warpStart[wi + 1] - pos : local[gid + 1] - off;
    if (pos >= capCands) limit = 0;
    else if (limit > capCands - pos) limit = capCands - pos;
    if (limit == 0) continue;
    uint2* out = cands + pos;
    if (limit <= cfg.predKeep) {
      const KeepSlots<IL, const uint32_t> slot = keep_slots<IL>(keep, gid, cfg.predKeep);
      for (uint32_t q = 0; q < limit; ++q) {
        const uint32_t h = slot[q];
        sent += h == TRAX_SENTINEL;
        out[q] = make_uint2(gid, h);
      }
      continue;
    }
    const uint2 pr = pairs[gid];
    const uint32_t hx = trax_hit(pr.x, cfg), hy = trax_hit(pr.y, cfg);
    const uint32_t event = hitEvt[hx];
    const uint32_t lt = hitLayer[hx] - 1;
    const uint32_t layer = cfg.layer3[lt] - 1;
    const uint32_t* lG3 = grid + ((size_t)event * cfg.L + layer) * cfg.C;
    const PredWindow w = pred_store_window(cfg, lt, layer, hits[hx], hits[hy]);
    uint32_t n = 0;
    const uint32_t C = cfg.C, nP = cfg.nP;
    if (FINE && w.pL <= nP) {
      PredUnionWindow u;
      u.zLow[0] = u.zLow[1] = w.zLow[1];
      u.zHigh[0] = u.zHigh[1] = w.zHigh[1];
      u.zLo = w.zLoSec[1];
      u.zHi = w.zHiSec[1];
      u.phiLow = w.phiLow;
      u.phiHigh = w.phiHigh;
      u.pL = w.pL;
      u.pH = w.pH;
      u.wrap = w.wrap;
      uint32_t unused = 0;
      fine_walk<false>(cfg, u, fine, event, layer, CandSlots{out, gid}, limit, unused, n);
      n = min(n, limit);
    } else
    for (uint32_t zs = w.zLoSec[1]; zs < w.zHiSec[1] && n < limit; ++zs) {
      uint32_t a[2], b[2];
      pred_row_parts(w, lG3, C, nP, zs, a[0], b[0], a[1], b[1]);
      for (int part = 0; part < 2 && n < limit; ++part)
        for (uint32_t j = a[part]; j < b[part] && n < limit; ++j)
          if (pred_valid(w, 1, hits[trax_hit(j, cfg)])) out[n++] = make_uint2(gid, j);
    }
    sent += limit - n;
    for (; n < limit; ++n) out[n] = make_uint2(gid, TRAX_SENTINEL);
  }
  for (int d = 16; d > 0; d >>= 1) sent += __shfl_down_sync(0xffffffffu, sent, d);
  if ((threadIdx.x & 31u) == 0 && sent) atomicAdd(sentinels, sent);
}

// tripletOffsets of predictStore (:404-418) + predictOffsetMonotonizeStore
// (:432-447).  The last non-sentinel pair of a segment stores the candidate
// position after it, and empty segments inherit their predecessor's value;
// pairs of a segment are contiguous and sentinel pairs count zero
// candidates, so both come down to the candidate position at the segment's
// pair end.
__global__ void predict_offsets_kernel(uint32_t S, const uint32_t* __restrict__ pairOffsets,
                                       const uint32_t* __restrict__ nPairsDev, const uint32_t* __restrict__ local,
                                       const uint32_t* __restrict__ warpStart, uint32_t* offsets) {
  const uint32_t nPairs = *nPairsDev;
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s <= S; s += gridDim.x * blockDim.x) {
    if (s == 0) {
      offsets[0] = 0u;
      continue;
    }
    const uint32_t p = min(pairOffsets[s], nPairs);
    offsets[s] = p == nPairs ? warpStart[(nPairs + 31u) >> 5] : warpStart[p >> 5] + local[p];
  }
}

// The flags in two steps, each warp on its own (no block barriers): a warp
// takes 1024 consecutive candidates, 32 at a time; every candidate takes the
// dphi test, which rejects most of them, and the survivors go to the warp's
// queue in shared memory.  The dphi test is decided from the cross and dot
// products of the two transverse segments wherever the angle is more than
// 1e-4 rad from the cut, which leaves the two atan2 to a few candidates in
// ten thousand (0.87 -> 0.55 ms on the 1000-event batch).  Whenever the queue holds 32 the warp
// runs the dtheta / TIP / curvature tests on them with every lane busy, and
// it empties the queue at the end of its 1024.  The flag is the AND of
// filterCount's four predicates (TripletThetaPhiFilter.h:65-154).
// filterPopCount + PrefixSum run on words of 32 flags: the flags of 32
// consecutive candidates are one word of masks, the number set goes to
// warpSums (+1 slot zeroed, the number of words to *nWordsOut), and only
// those sums are scanned; a triplet's position is its word's scanned sum
// plus the flags set below it in the word.
// At most 32 registers (eight 256-thread blocks per SM): full occupancy
// outweighs the few spilled bytes (0.99 -> 0.86 ms on the 1000-event batch).
__global__ void __launch_bounds__(TRAX_MAX_TUNED_THREADS, 8)
    filter_kernel(DevConfig cfg, const float4* __restrict__ hits, const uint32_t* __restrict__ hitLayer,
                  const uint2* __restrict__ pairs, const uint2* __restrict__ cands, const uint32_t* nCandsDev,
                  uint32_t* masks, uint32_t* warpSums, uint32_t* nWordsOut) {
  constexpr uint32_t WORDS = 32;  // a warp takes 32 words = 1024 candidates at a time
  __shared__ uint32_t s_queue[TRAX_MAX_TUNED_THREADS / 32][64];
  __shared__ uint32_t s_queue2[TRAX_MAX_TUNED_THREADS / 32][64];
  __shared__ uint32_t s_bits[TRAX_MAX_TUNED_THREADS / 32][WORDS];
  const uint32_t n = *nCandsDev;
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  uint32_t* queue = s_queue[warp];
  uint32_t* queue2 = s_queue2[warp];
  uint32_t* bits = s_bits[warp];
  // The cuts after dphi in the order that rejects most first: the circle
  // (TIP and curvature) keeps about a third of the dphi survivors (an eighth
  // in pileup), dtheta nearly all.  The circle's survivors wait in a second
  // per-warp queue, so that dtheta runs 32 at a time on them only.  The four
  // cuts are independent tests of the same candidate, ANDed, so their order
  // changes no outcome.
  struct Cand {
    float4 A, B, C;
    uint32_t lt;
  };
  auto load = [&](uint32_t g) {
    const uint2 c = cands[g];
    const uint2 pr = pairs[c.x];
    const uint32_t hx = trax_hit(pr.x, cfg);
    return Cand{hits[hx], hits[trax_hit(pr.y, cfg)], hits[trax_hit(c.y, cfg)], hitLayer[hx] - 1};
  };
  uint32_t queued2 = 0;  // warp-uniform
  // dtheta on the first 32 queued circle survivors (items of lanes < active)
  auto dtheta_round = [&](uint32_t g0, uint32_t active) {
    if (lane < active) {
      const uint32_t g = queue2[lane];
      const Cand k = load(g);
      if (filter_dtheta(cfg, k.lt, k.A, k.B, k.C)) atomicOr(&bits[(g - g0) >> 5], 1u << (g & 31u));
    }
    __syncwarp();
  };
  // the circle on one dphi survivor per lane (lanes < active); survivors
  // join the second queue, which runs dtheta whenever it holds 32
  auto circle_round = [&](uint32_t g0, uint32_t active) {
    bool ok = false;
    uint32_t g = 0;
    if (lane < active) {
      g = queue[lane];
      const Cand k = load(g);
      ok = filter_circle(cfg, k.lt, k.A, k.B, k.C);
    }
    const uint32_t ballot = __ballot_sync(0xffffffffu, ok);
    if (ok) queue2[queued2 + __popc(ballot & lanemask_lt())] = g;
    queued2 += __popc(ballot);
    __syncwarp();
    if (queued2 >= 32) {
      dtheta_round(g0, 32u);
      if (lane < queued2 - 32) queue2[lane] = queue2[32 + lane];
      queued2 -= 32;
      __syncwarp();
    }
  };
  for (uint32_t g0 = (blockIdx.x * (blockDim.x >> 5) + warp) * (WORDS * 32); g0 < n; g0 += warps * WORDS * 32) {
    bits[lane] = 0u;
    uint32_t queued = 0;  // warp-uniform
    __syncwarp();
    // each lane's next candidate is loaded one step ahead (0.499 -> 0.482 ms
    // on the ttbar-like batch; its pair as well, or 40 registers, were slower)
    uint2 cN = g0 + lane < n ? cands[g0 + lane] : make_uint2(0u, TRAX_SENTINEL);
    for (uint32_t k = 0; k < WORDS; ++k) {
      const uint32_t g = g0 + k * 32 + lane;
      const uint2 c = cN;
      if (k + 1 < WORDS) cN = g + 32 < n ? cands[g + 32] : make_uint2(0u, TRAX_SENTINEL);
      bool pass = false;
      if (c.y != TRAX_SENTINEL) {  // a slot the reference never wrote fails
        const uint2 pr = pairs[c.x];
        const uint32_t hx = trax_hit(pr.x, cfg);
        pass = filter_dphi_fast(cfg, hitLayer[hx] - 1, hits[hx], hits[trax_hit(pr.y, cfg)],
                                hits[trax_hit(c.y, cfg)]);
      }
      const uint32_t ballot = __ballot_sync(0xffffffffu, pass);
      if (pass) queue[queued + __popc(ballot & lanemask_lt())] = g;
      queued += __popc(ballot);
      __syncwarp();
      if (queued >= 32) {  // a full round of the circle cut
        circle_round(g0, 32u);
        if (lane < queued - 32) queue[lane] = queue[32 + lane];
        queued -= 32;
        __syncwarp();
      }
    }
    circle_round(g0, queued);
    dtheta_round(g0, queued2);
    queued2 = 0;
    const uint32_t word = (g0 >> 5) + lane;
    if (g0 + lane * 32 < n) {
      const uint32_t b = bits[lane];
      masks[word] = b;
      warpSums[word] = (uint32_t)__popc(b);
    }
    __syncwarp();
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const uint32_t nW = (n + 31u) >> 5;
    warpSums[nW] = 0u;  // the scan's +1 slot
    *nWordsOut = nW;
  }
}

// filterStore: (h1, h2, h3) of every flagged candidate, in candidate order.
// A warp takes 32 flag words (1024 candidates), whose triplets occupy the
// positions wordStart[w0] + 0, 1, ...: each lane writes one of them per
// step, finding its word by a 5-step search over the words' running counts
// and its candidate by the rank of the bit in the word (0.21 -> 0.15 ms on
// the 1000-event batch against one thread per candidate).
__global__ void filter_store_kernel(const uint2* __restrict__ pairs, const uint2* __restrict__ cands,
                                    const uint32_t* nCandsDev, const uint32_t* __restrict__ masks,
                                    const uint32_t* __restrict__ wordStart, uint32_t* h1, uint32_t* h2, uint32_t* h3,
                                    uint32_t capT) {
  const uint32_t n = *nCandsDev;
  const uint32_t nW = (n + 31u) >> 5;
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t w0 = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 32u; w0 < nW; w0 += warps * 32u) {
    const uint32_t word = w0 + lane < nW ? masks[w0 + lane] : 0u;
    const uint32_t base = wordStart[w0];
    uint32_t incl = (uint32_t)__popc(word);
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= (uint32_t)d) incl += t;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    for (uint32_t k0 = 0; k0 < total; k0 += 32u) {
      const uint32_t k = k0 + lane;
      // the word holding the warp's k-th flag: the first lane whose inclusive count exceeds k
      uint32_t lo = 0;
#pragma unroll
      for (uint32_t step = 16; step > 0; step >>= 1) {
        const uint32_t v = __shfl_sync(0xffffffffu, incl, lo + step - 1u);
        if (v <= k) lo += step;
      }
      const uint32_t wd = __shfl_sync(0xffffffffu, word, lo);
      const uint32_t before = __shfl_sync(0xffffffffu, incl, lo) - (uint32_t)__popc(wd);
      if (k < total) {
        const uint32_t bit = __fns(wd, 0u, (int)(k - before + 1u));
        const uint32_t g = (w0 + lo) * 32u + bit;
        const uint32_t pos = base + k;
        if (pos < capT) {
          const uint2 c = cands[g];
          const uint2 p = pairs[c.x];
          h1[pos] = p.x;
          h2[pos] = p.y;
          h3[pos] = c.y;
        }
      }
    }
  }
}

// filterOffsetStore (TripletThetaPhiFilter.h:221-257)
__global__ void triplet_offsets_kernel(DevConfig cfg, const uint32_t* __restrict__ hitEvt,
                                       const uint32_t* __restrict__ hitLayer, const uint32_t* __restrict__ h1,
                                       const uint32_t* nTDev, uint32_t* offsets) {
  const uint32_t nT = *nTDev;
  for (uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x; gid < nT; gid += gridDim.x * blockDim.x) {
    const uint32_t hitId = trax_hit(h1[gid], cfg);
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

// The staged windows pack the z rows and phi columns into 16 bits and the
// third layer's first cell into 32 bits.
bool pred_k_fits(const DevConfig& cfg) {
  return cfg.nZ < 65536u && cfg.nP < 65536u && (uint64_t)cfg.E * cfg.L * cfg.C < (1ull << 32);
}

}  // namespace

cudaError_t predict_pairs(const DevConfig& cfg, bool emit, const uint32_t* grid, DevHits hits, const uint2* pairs,
                          const uint32_t* nPairsDev, uint64_t maxPairs, uint32_t* candCount, uint32_t* warpSums,
                          uint32_t* nWarpsOut, uint32_t* keep, uint2* cands, uint64_t capCands, uint32_t* sentinels,
                          uint32_t* err, cudaStream_t st, uint32_t* launches, FineGrid fine) {
  const uint32_t cap = capCands > 0xffffffffull ? 0xffffffffu : (uint32_t)capCands;
  const int threads = (int)cfg.predThreads;
  const int blocks = grid_for(maxPairs + 1, threads);
  const bool il = keep_interleaved(cfg);
  if (emit) {
    if (maxPairs == 0) return cudaSuccess;
    if (cfg.fineRows > 0 && fine.grid)
      predict_store_kernel<true, true><<<blocks, threads, 0, st>>>(cfg, grid, hits.xyzp, hits.evt, hits.layer,
                                                                   pairs, nPairsDev, candCount, warpSums, keep,
                                                                   cands, cap, sentinels, fine);
    else if (il)
      predict_store_kernel<true, false><<<blocks, threads, 0, st>>>(cfg, grid, hits.xyzp, hits.evt, hits.layer,
                                                                    pairs, nPairsDev, candCount, warpSums, keep,
                                                                    cands, cap, sentinels, fine);
    else
      predict_store_kernel<false, false><<<blocks, threads, 0, st>>>(cfg, grid, hits.xyzp, hits.evt, hits.layer,
                                                                     pairs, nPairsDev, candCount, warpSums, keep,
                                                                     cands, cap, sentinels, fine);
  } else if (cfg.fineRows > 0 && fine.grid) {
    predict_count_kernel<true, true><<<blocks, threads, 0, st>>>(cfg, grid, hits.xyzp, hits.evt, hits.layer, pairs,
                                                                 nPairsDev, candCount, keep, warpSums, nWarpsOut,
                                                                 err, fine);
  } else if (il) {  // the K-pairs kernel keeps the consecutive layout
    predict_count_kernel<false, true><<<blocks, threads, 0, st>>>(cfg, grid, hits.xyzp, hits.evt, hits.layer, pairs,
                                                                  nPairsDev, candCount, keep, warpSums, nWarpsOut,
                                                                  err, fine);
  } else if (cfg.predPairsPerThread <= 1 || !pred_k_fits(cfg)) {
    predict_count_kernel<false, false><<<blocks, threads, 0, st>>>(cfg, grid, hits.xyzp, hits.evt, hits.layer,
                                                                   pairs, nPairsDev, candCount, keep, warpSums,
                                                                   nWarpsOut, err, fine);
  } else {
    const int K = cfg.predPairsPerThread;
    const size_t smem = (size_t)threads * K * sizeof(PredStage);
    const int kb = grid_for((maxPairs + K - 1) / K + 1, threads);
    if (K == 2)
      predict_count_k_kernel<2><<<kb, threads, smem, st>>>(cfg, grid, hits.xyzp, hits.evt, hits.layer, pairs,
                                                           nPairsDev, candCount, keep, warpSums, nWarpsOut, err);
    else
      predict_count_k_kernel<4><<<kb, threads, smem, st>>>(cfg, grid, hits.xyzp, hits.evt, hits.layer, pairs,
                                                           nPairsDev, candCount, keep, warpSums, nWarpsOut, err);
  }
  if (launches) *launches += 1;
  return cudaGetLastError();
}

cudaError_t predict_offsets(const DevConfig& cfg, const uint32_t* pairOffsets, const uint32_t* nPairsDev,
                            const uint32_t* candCount, const uint32_t* warpStart, uint32_t* candOffsets,
                            cudaStream_t st, uint32_t* launches) {
  const uint32_t S = cfg.E * cfg.nLT;
  predict_offsets_kernel<<<grid_for(S + 1, 256), 256, 0, st>>>(S, pairOffsets, nPairsDev, candCount, warpStart,
                                                               candOffsets);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

cudaError_t filter_candidates(const DevConfig& cfg, DevHits hits, const uint2* pairs, const uint2* cands,
                              const uint32_t* nCandsDev, uint64_t maxCands, uint32_t* masks, uint32_t* warpSums,
                              uint32_t* nWordsOut, cudaStream_t st, uint32_t* launches) {
  const int threads = (int)cfg.filterThreads;
  filter_kernel<<<grid_for(maxCands + 1, threads), threads, 0, st>>>(cfg, hits.xyzp, hits.layer, pairs, cands,
                                                                     nCandsDev, masks, warpSums, nWordsOut);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

cudaError_t filter_store(const uint2* pairs, const uint2* cands, const uint32_t* nCandsDev, uint64_t maxCands,
                         const uint32_t* masks, const uint32_t* wordStart, uint32_t* h1, uint32_t* h2, uint32_t* h3,
                         uint64_t capT, cudaStream_t st, uint32_t* launches) {
  if (maxCands == 0) return cudaSuccess;
  const uint32_t cap = capT > 0xffffffffull ? 0xffffffffu : (uint32_t)capT;
  filter_store_kernel<<<grid_for((maxCands + 1023) / 1024 * 32, 256), 256, 0, st>>>(pairs, cands, nCandsDev, masks,
                                                                                    wordStart, h1, h2, h3, cap);
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
