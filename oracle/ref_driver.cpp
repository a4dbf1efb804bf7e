// ref_driver.cpp -- runs the reference's own kernel text on the CPU with the
// reference's host-side sequences.  TEST INFRASTRUCTURE ONLY: the tests load
// oracle/_ref/libtraxref.so beside the oracle; the product never links it.
//
// ref_extract.py generates ref_kernels.cpp (the OpenCL C of the reference's
// KERNEL_CLASS blocks, compiled against ref_shim.h) and compiles this file,
// which includes it.  This file restates what the OpenCL wrapper and the
// algorithm classes' run() methods do around the kernels (all citations are
// paths inside the reference project):
//   grid build    GridBuilder.cpp:6-161 (local-memory variant by size)
//   prefix sum    PrefixSum.cpp:20-140 (recursive scan, float group counts)
//   pairs         PairGeneratorBeamspot.cpp:5-183
//   prediction    TripletThetaPhiPredictor.cpp:10-168
//   filter        TripletThetaPhiFilter.cpp:10-206
//   connectivity  TripletConnectivityTight.cpp:5-475
//   circle fit    TrackletCircleFitter.cpp (run)
//   CA            CellularAutomaton.cpp:7-465
//   stage order   TripletBuilder.cpp:312-467
// with the reference's argument order, including the binding of the uint
// column pairSpreadPhi to pairCount's float parameter gSigmaPhi
// (PairGeneratorBeamspot.cpp:59, 80).
//
// NDRanges run work-group by work-group.  Inside a work-group, work-items run
// one after the other; a kernel that calls barrier() with more than one
// work-item per group runs its work-items as ucontext fibers that switch at
// every barrier.  The local-memory variants are chosen as the reference
// chooses them, against a device local-memory size given by the caller.
//
// Memory the reference allocates without initialising is filled with 0xff
// bytes here.  Where the reference then reads slots it never wrote (pair
// slots past the distinct bitmap bits; candidate slots left by the two
// rOrigin roundings of predictCount and predictStore), its result is
// undefined.  Those slots are pointed at one extra hit appended after the
// last (x, y, z NaN, layer 1, event 0) -- and an extra pair (that hit twice)
// for candidates -- whose NaN comparisons reject it everywhere, which is
// what the oracle does with its sentinels.  They are counted.
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <ucontext.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <functional>
#include <limits>
#include <map>
#include <string>
#include <thread>
#include <vector>

#include "ref_kernels.cpp"
#include "ref_tracks.cpp"
#include "trax_oracle.h"

namespace refrt {

thread_local ItemState item;

namespace {

struct FiberGroup {
  std::vector<ucontext_t> ctx;
  std::vector<std::vector<char>> stacks;
  std::vector<char> done;
  std::vector<size_t> lid0, lid1, lid2;
};

thread_local ucontext_t t_sched;
thread_local FiberGroup* t_group = nullptr;
thread_local size_t t_cur = 0;
thread_local const std::function<void()>* t_body = nullptr;

void fiber_entry() {
  (*t_body)();
  t_group->done[t_cur] = 1;
}

constexpr size_t kFiberStack = 256 * 1024;

}  // namespace

void barrier_switch() {
  if (!item.fibers) abort();  // a barrier in a group run without fibers
  swapcontext(&t_group->ctx[t_cur], &t_sched);
}

struct NDRange {
  size_t g[3];
  size_t l[3];
};

// Runs body() once per work-item of the NDRange, work-group after work-group
// (dimension 0 fastest).  `barriers`: the kernel calls barrier().
void launch(NDRange r, bool barriers, const std::function<void()>& body) {
  for (int d = 0; d < 3; ++d) {
    if (r.l[d] == 0 || r.g[d] % r.l[d] != 0) abort();
    item.gsz[d] = r.g[d];
    item.lsz[d] = r.l[d];
  }
  const size_t ng[3] = {r.g[0] / r.l[0], r.g[1] / r.l[1], r.g[2] / r.l[2]};
  const size_t items = r.l[0] * r.l[1] * r.l[2];
  item.group_items = items;
  const bool fibers = barriers && items > 1;
  item.fibers = fibers;
  FiberGroup grp;
  if (fibers) {
    grp.ctx.resize(items);
    grp.stacks.assign(items, std::vector<char>(kFiberStack));
    grp.done.assign(items, 0);
  }
  for (size_t g2 = 0; g2 < ng[2]; ++g2)
    for (size_t g1 = 0; g1 < ng[1]; ++g1)
      for (size_t g0 = 0; g0 < ng[0]; ++g0) {
        const size_t gg[3] = {g0, g1, g2};
        auto set_ids = [&](size_t k) {
          size_t l0 = k % r.l[0], l1 = (k / r.l[0]) % r.l[1], l2 = k / (r.l[0] * r.l[1]);
          const size_t ll[3] = {l0, l1, l2};
          for (int d = 0; d < 3; ++d) {
            item.grp[d] = gg[d];
            item.lid[d] = ll[d];
            item.gid[d] = gg[d] * r.l[d] + ll[d];
          }
        };
        if (!fibers) {
          for (size_t k = 0; k < items; ++k) {
            set_ids(k);
            body();
          }
          continue;
        }
        t_group = &grp;
        t_body = &body;
        for (size_t k = 0; k < items; ++k) {
          getcontext(&grp.ctx[k]);
          grp.ctx[k].uc_stack.ss_sp = grp.stacks[k].data();
          grp.ctx[k].uc_stack.ss_size = kFiberStack;
          grp.ctx[k].uc_link = &t_sched;
          makecontext(&grp.ctx[k], fiber_entry, 0);
          grp.done[k] = 0;
        }
        size_t remaining = items;
        while (remaining) {
          for (size_t k = 0; k < items; ++k) {
            if (grp.done[k]) continue;
            set_ids(k);
            t_cur = k;
            swapcontext(&t_sched, &grp.ctx[k]);
            if (grp.done[k]) --remaining;
          }
        }
        t_group = nullptr;
      }
  item.fibers = false;
}

}  // namespace refrt

namespace {

using refk::uint;
using refk::uint2;
using refrt::launch;
using refrt::NDRange;

// Elements after every allocation: they absorb the reference's reads just
// past an array's end and hold the extra pair and the triplet columns' hit.
#ifndef REF_SLACK
#define REF_SLACK 64
#endif
constexpr size_t kSlack = REF_SLACK;
constexpr uint kUninit = 0xffffffffu;

float uninit_f() {
  float f;
  uint u = kUninit;
  memcpy(&f, &u, 4);
  return f;
}

// A device buffer: `count` elements plus slack that absorbs the reference's
// reads one or a few elements past an allocation's end.
template <class T>
struct Buf {
  std::vector<T> v;
  size_t count = 0;
  void alloc(size_t n, T fill, T slack) {
    count = n;
    v.assign(n + kSlack, slack);
    std::fill(v.begin(), v.begin() + n, fill);
  }
  T* p() { return v.data(); }
  const T* p() const { return v.data(); }
  T& operator[](size_t i) { return v[i]; }
  const T& operator[](size_t i) const { return v[i]; }
};

Buf<uint> u_uninit(size_t n) {
  Buf<uint> b;
  b.alloc(n, kUninit, kUninit);
  return b;
}
Buf<uint> u_value(size_t n, uint value) {
  Buf<uint> b;
  b.alloc(n, value, kUninit);
  return b;
}
Buf<float> f_uninit(size_t n) {
  Buf<float> b;
  b.alloc(n, uninit_f(), uninit_f());
  return b;
}
Buf<uint2> u2_uninit(size_t n) {
  Buf<uint2> b;
  b.alloc(n, uint2(kUninit, kUninit), uint2(kUninit, kUninit));
  return b;
}

NDRange r1(size_t g, size_t l) { return NDRange{{g, 1, 1}, {l, 1, 1}}; }
NDRange r3(size_t g0, size_t g1, size_t g2, size_t l0) { return NDRange{{g0, g1, g2}, {l0, 1, 1}}; }

// (uint) std::max(1.0f, ceil(((float) n) / d)): the reference's group counts
uint groups_of(uint n, uint d) {
  return (uint)std::max(1.0f, std::ceil(((float)n) / (float)d));
}

uint next_pow2(uint n) {  // PrefixSum.cpp:61-71
  n--;
  n |= n >> 1;
  n |= n >> 2;
  n |= n >> 4;
  n |= n >> 8;
  n |= n >> 16;
  n++;
  return n;
}

// PrefixSum::run (PrefixSum.cpp:20-140): exclusive scan of `size` elements in
// place with work-groups of `wg` work-items.
struct PrefixSum {
  std::vector<Buf<uint>> partial;

  void create_partial_sums(uint size, uint wg) {  // :47-59
    uint nGroups = (uint)std::max(1.0f, std::ceil(((float)size) / (float)(wg << 1)));
    while (nGroups > 1) {
      partial.push_back(u_value(nGroups, 0));
      nGroups = (uint)std::max(1.0f, std::ceil(((float)nGroups) / (float)(wg << 1)));
    }
  }

  void recursive_scan(uint* input, uint size, uint wg, uint level) {  // :73-140
    uint nGroups = (uint)std::max(1.0f, std::ceil(((float)size) / (float)(wg << 1)));
    uint padding = (wg << 1) / MEMORY_BANK_COUNT;
    std::vector<uint> local((wg << 1) + padding + kSlack);
    if (nGroups == 1) {
      uint localSize = (uint)std::max(1.0f, std::ceil(((float)size) / 2));
      localSize = next_pow2(localSize);
      launch(r1(localSize, localSize), refk::kBarrier_prefixSumWG,
             [&] { refk::prefixSumWG(input, size, local.data()); });
    } else {
      uint* part = partial[level].p();
      launch(r1((size_t)wg * nGroups, wg), refk::kBarrier_prefixSumPartial,
             [&] { refk::prefixSumPartial(input, size, part, local.data()); });
      recursive_scan(part, nGroups, wg, level + 1);
      launch(r1((size_t)wg * nGroups, wg), refk::kBarrier_prefixSumUniformAdd,
             [&] { refk::prefixSumUniformAdd(input, size, part); });
    }
  }

  void run(uint* input, uint size, uint wg) {
    partial.clear();
    create_partial_sums(size, wg);
    recursive_scan(input, size, wg, 0);
  }
};

struct Stats {
  uint pair_sentinels = 0, cand_sentinels = 0, ca_iterations = 0, no_links = 0, ca_chain_broken = 0,
       grid_count_local = 0, grid_store_variant = 0, pair_count_local = 0;
};

struct Run {
  const oracle_input* in = nullptr;
  uint T = 1;              // exec.threads
  size_t localMem = 0;     // the device's local memory size in bytes
  uint E = 0, L = 0, nZ = 0, nP = 0, nLT = 0, C = 0, H = 0;
  float MIN_Z = 0, sZ = 0, MIN_PHI = 0, sP = 0, minRc = 0;
  uint P = 0;  // the appended hit

  Buf<uint> eventOffsets, layerHits, layerOffsets;
  Buf<float> minR, maxR;
  Buf<uint> l1, l2, l3, spreadZ, spreadPhi, nCand;
  Buf<float> dTheta, sigmaZ, dPhi, sigmaPhi, tip, z0;
  Buf<float> x, y, z;
  Buf<uint> layer, det, hit, evt;
  Buf<uint> grid;
  Buf<uint2> pairs;
  Buf<uint> pairOffsets;
  Buf<uint2> cands;
  Buf<uint> candOffsets;
  Buf<uint> t1, t2, t3, tOffsets;
  Buf<float> eta;
  Buf<uint> basis, follower, connectable, nonConnectable;
  Buf<float> pt;
  Buf<uint> states, best, tracks, trackOffsets;
  Stats st;
};


Buf<uint> hit_index_buf(size_t n, uint poison) {  // triplet hit columns: slack holds the appended hit
  Buf<uint> b;
  b.alloc(n, kUninit, poison);
  return b;
}

// LayerGrid::size() (Grid.h): the layer's first and last grid entries, each
// read through GridEntry::idx(), which returns float.
uint layer_grid_size(const Run& R, uint layer, uint e) {
  size_t base = (size_t)e * R.L * R.C + (size_t)(layer - 1) * R.C;
  uint first = (uint)(float)R.grid[base];
  uint last = (uint)(float)R.grid[base + R.C - 1];
  return last - first;
}

// GridBuilder::run (GridBuilder.cpp:6-161)
void grid_build(Run& R) {
  R.grid = u_value((size_t)R.E * R.L * R.C, 0);  // zeroed before the build (TripletBuilder.cpp:296-310)
  const size_t localBytes = sizeof(uint) * R.C;     // local_param(sizeof(cl_uint), cells)
  const NDRange rg = r3(R.T, R.L, R.E, R.T);
  std::vector<uint> lGrid(R.C + kSlack), written(R.C + kSlack);
  if (localBytes < R.localMem) {
    R.st.grid_count_local = 1;
    launch(rg, refk::kBarrier_gridCount, [&] {
      refk::gridCount(R.eventOffsets.p(), R.layerHits.p(), R.layerOffsets.p(), R.L, R.grid.p(), R.MIN_Z, R.sZ,
                      R.nZ, R.MIN_PHI, R.sP, R.nP, R.x.p(), R.y.p(), R.z.p(), lGrid.data());
    });
  } else {
    launch(rg, refk::kBarrier_gridNoLocalCount, [&] {
      refk::gridNoLocalCount(R.eventOffsets.p(), R.layerHits.p(), R.layerOffsets.p(), R.L, R.grid.p(), R.MIN_Z,
                             R.sZ, R.nZ, R.MIN_PHI, R.sP, R.nP, R.x.p(), R.y.p(), R.z.p());
    });
  }
  PrefixSum().run(R.grid.p(), (uint)R.grid.count, R.T);

  // new hit buffers (HitCollection::transfer.initBuffers), one more for the appended hit
  Buf<float> ox = f_uninit(R.H + 1), oy = f_uninit(R.H + 1), oz = f_uninit(R.H + 1);
  Buf<uint> oLayer = u_uninit(R.H + 1), oDet = u_uninit(R.H + 1), oHit = u_uninit(R.H + 1),
            oEvt = u_uninit(R.H + 1);
  if (localBytes * 2 < R.localMem) {
    R.st.grid_store_variant = 2;
    launch(rg, refk::kBarrier_gridStore, [&] {
      refk::gridStore(R.eventOffsets.p(), R.layerHits.p(), R.layerOffsets.p(), R.L, R.grid.p(), R.MIN_Z, R.sZ,
                      R.nZ, R.MIN_PHI, R.sP, R.nP, R.x.p(), R.y.p(), R.z.p(), R.layer.p(), R.det.p(), R.hit.p(),
                      R.evt.p(), ox.p(), oy.p(), oz.p(), oLayer.p(), oDet.p(), oHit.p(), oEvt.p(), lGrid.data(),
                      written.data());
    });
  } else if (localBytes < R.localMem) {
    R.st.grid_store_variant = 1;
    launch(rg, refk::kBarrier_gridWrittenLocalStore, [&] {
      refk::gridWrittenLocalStore(R.eventOffsets.p(), R.layerHits.p(), R.layerOffsets.p(), R.L, R.grid.p(),
                                  R.MIN_Z, R.sZ, R.nZ, R.MIN_PHI, R.sP, R.nP, R.x.p(), R.y.p(), R.z.p(),
                                  R.layer.p(), R.det.p(), R.hit.p(), R.evt.p(), ox.p(), oy.p(), oz.p(),
                                  oLayer.p(), oDet.p(), oHit.p(), oEvt.p(), written.data());
    });
  } else {
    R.st.grid_store_variant = 0;
    Buf<uint> gWritten = u_value(R.grid.count, 0);
    launch(rg, refk::kBarrier_gridNoLocalStore, [&] {
      refk::gridNoLocalStore(R.eventOffsets.p(), R.layerHits.p(), R.layerOffsets.p(), R.L, R.grid.p(), R.MIN_Z,
                             R.sZ, R.nZ, R.MIN_PHI, R.sP, R.nP, R.x.p(), R.y.p(), R.z.p(), R.layer.p(),
                             R.det.p(), R.hit.p(), R.evt.p(), ox.p(), oy.p(), oz.p(), oLayer.p(), oDet.p(),
                             oHit.p(), oEvt.p(), gWritten.p());
    });
  }
  // the appended hit keeps its place after the last one
  ox[R.H] = R.x[R.H];
  oy[R.H] = R.y[R.H];
  oz[R.H] = R.z[R.H];
  oLayer[R.H] = R.layer[R.H];
  oDet[R.H] = R.det[R.H];
  oHit[R.H] = R.hit[R.H];
  oEvt[R.H] = R.evt[R.H];
  R.x = ox;
  R.y = oy;
  R.z = oz;
  R.layer = oLayer;
  R.det = oDet;
  R.hit = oHit;
  R.evt = oEvt;
}

// PairGeneratorBeamspot::run (PairGeneratorBeamspot.cpp:5-183)
void pair_gen(Run& R) {
  std::vector<uint> oracleOffset;
  uint totalMaxPairs = 0;
  for (uint e = 0; e < R.E; ++e) {
    for (uint p = 0; p < R.nLT; ++p) {
      uint nMaxPairs = layer_grid_size(R, R.l1[p], e) * layer_grid_size(R, R.l2[p], e);
      nMaxPairs = (uint)(32 * std::ceil(nMaxPairs / 32.0));
      oracleOffset.push_back(totalMaxPairs);
      totalMaxPairs += nMaxPairs;
    }
  }
  Buf<uint> mOracleOffset = u_value(oracleOffset.size(), 0);
  std::copy(oracleOffset.begin(), oracleOffset.end(), mOracleOffset.v.begin());
  Buf<uint> mOracle = u_value((size_t)std::ceil(totalMaxPairs / 32.0), 0);
  Buf<uint> mPrefixSum = u_value((size_t)R.E * R.nLT * R.T + 1, 0);
  const size_t localBytes = sizeof(uint) * R.C;
  const NDRange rp = r3(R.T, R.nLT, R.E, R.T);
  // the uint column pairSpreadPhi bound to the float parameter gSigmaPhi (:59, :80)
  const float* sigmaPhiArg = reinterpret_cast<const float*>(R.spreadPhi.p());
  if (localBytes < R.localMem) {
    R.st.pair_count_local = 1;
    std::vector<uint> lGrid1(R.C + kSlack);
    launch(rp, refk::kBarrier_pairCount, [&] {
      refk::pairCount(R.minR.p(), R.maxR.p(), R.l1.p(), R.l2.p(), R.L, R.grid.p(), R.MIN_Z, R.sZ, R.nZ, R.MIN_PHI,
                      R.sP, R.nP, R.z0.p(), sigmaPhiArg, R.sigmaZ.p(), R.tip.p(), R.minRc, R.x.p(), R.y.p(), R.z.p(),
                      mOracle.p(), mOracleOffset.p(), mPrefixSum.p(), lGrid1.data());
    });
  } else {
    launch(rp, refk::kBarrier_pairNoLocalCount, [&] {
      refk::pairNoLocalCount(R.minR.p(), R.maxR.p(), R.l1.p(), R.l2.p(), R.L, R.grid.p(), R.MIN_Z, R.sZ, R.nZ,
                             R.MIN_PHI, R.sP, R.nP, R.z0.p(), sigmaPhiArg, R.sigmaZ.p(), R.tip.p(), R.minRc,
                             R.x.p(), R.y.p(), R.z.p(), mOracle.p(), mOracleOffset.p(), mPrefixSum.p());
    });
  }
  PrefixSum().run(mPrefixSum.p(), (uint)mPrefixSum.count, R.T);
  uint nFoundPairs = mPrefixSum[mPrefixSum.count - 1];
  R.pairs = u2_uninit(nFoundPairs);
  R.pairOffsets = u_value((size_t)R.E * R.nLT + 1, 0);
  launch(rp, refk::kBarrier_pairStore, [&] {
    refk::pairStore(R.l1.p(), R.l2.p(), R.L, R.grid.p(), R.nZ, R.nP, mOracle.p(), mOracleOffset.p(),
                    mPrefixSum.p(), R.pairs.p(), R.pairOffsets.p());
  });
  for (uint i = 0; i < nFoundPairs; ++i) {
    if (R.pairs[i].x == kUninit) {
      R.pairs[i] = uint2(R.P, R.P);
      ++R.st.pair_sentinels;
    }
  }
  R.pairs[nFoundPairs] = uint2(R.P, R.P);  // the extra pair, in the slack
}

// TripletThetaPhiPredictor::run (TripletThetaPhiPredictor.cpp:10-168)
void predict(Run& R) {
  const uint nPairs = (uint)R.pairs.count;
  Buf<uint> mPrefixSum = u_value((size_t)nPairs + 1, 0);
  uint nGroups = groups_of(nPairs, R.T);
  // DetectorGeometry / Dictionary buffers: passed, never read by the kernels
  std::vector<refk::uchar> detRadius(kSlack, 0);
  std::vector<float> radiusDict(kSlack, 0.0f);
  const int* hitId = reinterpret_cast<const int*>(R.hit.p());
  launch(r1((size_t)nGroups * R.T, R.T), refk::kBarrier_predictCount, [&] {
    refk::predictCount(detRadius.data(), radiusDict.data(), R.minR.p(), R.maxR.p(), R.grid.p(), R.l3.p(), R.L,
                       R.MIN_Z, R.sZ, R.nZ, R.MIN_PHI, R.sP, R.nP, R.sigmaZ.p(), R.sigmaPhi.p(), R.minRc,
                       R.pairs.p(), nPairs, R.x.p(), R.y.p(), R.z.p(), R.evt.p(), R.layer.p(), R.det.p(), hitId,
                       mPrefixSum.p());
  });
  PrefixSum().run(mPrefixSum.p(), (uint)mPrefixSum.count, R.T);
  uint nFound = mPrefixSum[mPrefixSum.count - 1];
  R.cands = u2_uninit(nFound);
  R.candOffsets = u_value((size_t)R.E * R.nLT + 1, 0);
  launch(r1((size_t)nGroups * R.T, R.T), refk::kBarrier_predictStore, [&] {
    refk::predictStore(detRadius.data(), radiusDict.data(), R.minR.p(), R.maxR.p(), R.grid.p(), R.l3.p(), R.L,
                       R.MIN_Z, R.sZ, R.nZ, R.MIN_PHI, R.sP, R.nP, R.sigmaZ.p(), R.sigmaPhi.p(), R.nLT, R.minRc,
                       R.pairs.p(), nPairs, R.x.p(), R.y.p(), R.z.p(), R.evt.p(), R.layer.p(), R.det.p(),
                       mPrefixSum.p(), R.cands.p(), R.candOffsets.p());
  });
  nGroups = groups_of((uint)R.candOffsets.count, R.T);
  launch(r1((size_t)nGroups * R.T, R.T), refk::kBarrier_predictOffsetMonotonizeStore, [&] {
    refk::predictOffsetMonotonizeStore(R.candOffsets.p(), (uint)R.candOffsets.count);
  });
  for (uint i = 0; i < nFound; ++i) {
    if (R.cands[i].x == kUninit) {
      R.cands[i] = uint2(nPairs, R.P);  // the extra pair and the appended hit
      ++R.st.cand_sentinels;
    }
  }
}

// TripletThetaPhiFilter::run (TripletThetaPhiFilter.cpp:10-206)
void filter(Run& R) {
  const uint nTripletCandidates = (uint)R.cands.count;
  const uint nOracleCount = (uint)std::ceil(nTripletCandidates / 32.0);
  uint nGroups = groups_of(nTripletCandidates, R.T);
  Buf<uint> mOracle = u_value(nOracleCount, 0);
  launch(r1((size_t)nGroups * R.T, R.T), refk::kBarrier_filterCount, [&] {
    refk::filterCount(R.dTheta.p(), R.dPhi.p(), R.tip.p(), R.minRc, R.pairs.p(), R.cands.p(), nTripletCandidates,
                      R.x.p(), R.y.p(), R.z.p(), R.evt.p(), R.layer.p(), mOracle.p());
  });
  Buf<uint> mPrefixSum = u_value((size_t)nOracleCount + 1, 0);
  nGroups = groups_of(nOracleCount, R.T);
  launch(r1((size_t)nGroups * R.T, R.T), refk::kBarrier_filterPopCount,
         [&] { refk::filterPopCount(mOracle.p(), mPrefixSum.p(), nOracleCount); });
  PrefixSum().run(mPrefixSum.p(), (uint)mPrefixSum.count, R.T);
  const uint nFoundTriplets = mPrefixSum[mPrefixSum.count - 1];
  R.t1 = hit_index_buf(nFoundTriplets, R.P);
  R.t2 = hit_index_buf(nFoundTriplets, R.P);
  R.t3 = hit_index_buf(nFoundTriplets, R.P);
  R.tOffsets = u_value((size_t)R.E * R.nLT + 1, 0);
  launch(r1((size_t)nGroups * R.T, R.T), refk::kBarrier_filterStore, [&] {
    refk::filterStore(R.pairs.p(), R.nLT, R.cands.p(), mOracle.p(), nOracleCount, mPrefixSum.p(), R.t1.p(),
                      R.t2.p(), R.t3.p(), R.tOffsets.p());
  });
  nGroups = groups_of(nFoundTriplets, R.T);
  launch(r1((size_t)nGroups * R.T, R.T), refk::kBarrier_filterOffsetStore, [&] {
    refk::filterOffsetStore(R.t1.p(), nFoundTriplets, R.nLT, R.evt.p(), R.layer.p(), R.tOffsets.p());
  });
  nGroups = groups_of((uint)R.tOffsets.count, R.T);
  launch(r1((size_t)nGroups * R.T, R.T), refk::kBarrier_filterOffsetMonotonizeStore, [&] {
    refk::filterOffsetMonotonizeStore(R.tOffsets.p(), (uint)R.tOffsets.count);
  });
}

// TripletConnectivityTight::run (TripletConnectivityTight.cpp:5-475).  Returns
// false where the reference returns its tuple of null pointers (no links).
bool connectivity(Run& R, float dEtaCut) {
  const uint nTracklets = (uint)R.t1.count;
  const uint nGroups = groups_of(nTracklets, R.T);
  const NDRange rt = r1((size_t)nGroups * R.T, R.T);
  R.eta = f_uninit(nTracklets);
  launch(rt, refk::kBarrier_tripletEtaCalculatorStore, [&] {
    refk::tripletEtaCalculatorStore(R.x.p(), R.y.p(), R.z.p(), R.t1.p(), R.t3.p(), R.eta.p(), nTracklets);
  });
  Buf<uint> mOracle = u_value(nTracklets, 0);
  Buf<uint> mFollowerPrefixSum = u_value((size_t)nTracklets + 1, 0);
  const uint nOffsets = (uint)R.tOffsets.count;
  launch(rt, refk::kBarrier_tripletConnectivityTightCount, [&] {
    refk::tripletConnectivityTightCount(R.t2.p(), R.t3.p(), R.t1.p(), R.t2.p(), R.tOffsets.p(), R.evt.p(),
                                        R.layer.p(), R.nLT, nOffsets, R.eta.p(), dEtaCut, mFollowerPrefixSum.p(),
                                        mOracle.p(), nTracklets);
  });
  PrefixSum ps;
  ps.run(mFollowerPrefixSum.p(), (uint)mFollowerPrefixSum.count, R.T);
  const uint nLinks = mFollowerPrefixSum[mFollowerPrefixSum.count - 1];
  if (!nLinks) {
    R.st.no_links = 1;
    return false;
  }
  R.basis = u_uninit(nLinks);
  R.follower = u_uninit(nLinks);
  Buf<uint> pairEvent = u_uninit(nLinks);
  launch(rt, refk::kBarrier_tripletConnectivityTightStore, [&] {
    refk::tripletConnectivityTightStore(R.t2.p(), R.t3.p(), R.t1.p(), R.t2.p(), R.tOffsets.p(), R.evt.p(),
                                        R.layer.p(), R.nLT, nOffsets, R.eta.p(), dEtaCut, mFollowerPrefixSum.p(),
                                        R.basis.p(), R.follower.p(), pairEvent.p(), nTracklets);
  });
  Buf<uint> mInvOracle = u_uninit(nTracklets);
  launch(rt, refk::kBarrier_predicateInversionStore, [&] {
    refk::predicateInversionStore(mOracle.p(), mInvOracle.p(), (uint)mOracle.count - 1);
  });
  ps.run(mOracle.p(), (uint)mOracle.count, R.T);
  const uint nConnectable = mOracle[mOracle.count - 1];
  ps.run(mInvOracle.p(), (uint)mInvOracle.count, R.T);
  const uint nNonConnectable = mInvOracle[mInvOracle.count - 1];
  R.connectable = u_uninit(nConnectable);
  launch(rt, refk::kBarrier_streamCompactionGetValidIndexesStore, [&] {
    refk::streamCompactionGetValidIndexesStore(mOracle.p(), R.connectable.p(), (uint)mOracle.count - 1);
  });
  R.nonConnectable = u_uninit(0);
  if (nNonConnectable > 0) {
    R.nonConnectable = u_uninit(nNonConnectable);
    launch(rt, refk::kBarrier_streamCompactionGetValidIndexesStore, [&] {
      refk::streamCompactionGetValidIndexesStore(mInvOracle.p(), R.nonConnectable.p(), (uint)mInvOracle.count - 1);
    });
  }
  return true;
}

// TrackletCircleFitter::run (TrackletCircleFitter.cpp)
void circle_fit(Run& R) {
  const uint nTracklets = (uint)R.t1.count;
  const uint nGroups = groups_of(nTracklets, R.T);
  R.pt = f_uninit(nTracklets);
  launch(r1((size_t)nGroups * R.T, R.T), refk::kBarrier_trackletCircleFitterStore, [&] {
    refk::trackletCircleFitterStore(R.x.p(), R.y.p(), R.z.p(), R.t1.p(), R.t2.p(), R.t3.p(), R.connectable.p(),
                                    R.pt.p(), (uint)R.connectable.count);
  });
}

// CellularAutomaton::run (CellularAutomaton.cpp:7-465)
void cellular_automaton(Run& R, uint max_iterations) {
  const uint nTripletPairs = (uint)R.basis.count;
  const uint nTriplets = (uint)R.pt.count;
  const uint gT = groups_of(nTriplets, R.T), gP = groups_of(nTripletPairs, R.T);
  const NDRange rt = r1((size_t)gT * R.T, R.T), rl = r1((size_t)gP * R.T, R.T);
  Buf<uint> states = u_value(nTriplets, 1), next = u_value(nTriplets, 1);
  Buf<uint> living = u_uninit((size_t)nTriplets + 1);
  PrefixSum ps;
  uint aliveCells = 0, iterations = 0;
  do {
    ++iterations;
    launch(rt, refk::kBarrier_memset, [&] { refk::memset(living.p(), 0, nTriplets); });
    launch(rl, refk::kBarrier_iteration, [&] {
      refk::iteration(R.basis.p(), R.follower.p(), states.p(), next.p(), living.p(), nTripletPairs);
    });
    ps.run(living.p(), (uint)living.count, R.T);
    aliveCells = living[living.count - 1];
    std::swap(states, next);
  } while (aliveCells > 0 && iterations < max_iterations);
  R.st.ca_iterations = iterations;

  Buf<uint> followerBasisPS = u_value((size_t)nTriplets + 1, 0);
  launch(rl, refk::kBarrier_followerBasisCount, [&] {
    refk::followerBasisCount(R.basis.p(), R.follower.p(), states.p(), followerBasisPS.p(), nTripletPairs);
  });
  ps.run(followerBasisPS.p(), (uint)followerBasisPS.count, R.T);
  const uint total = followerBasisPS[followerBasisPS.count - 1];
  Buf<uint> basisIndices = u_uninit(total);
  Buf<float> ptDiff = f_uninit(total);
  launch(rl, refk::kBarrier_followerBasisStore, [&] {
    refk::followerBasisStore(R.basis.p(), R.follower.p(), states.p(), R.pt.p(), followerBasisPS.p(), ptDiff.p(),
                             basisIndices.p(), nTripletPairs);
  });
  R.best = u_value(nTriplets, std::numeric_limits<uint>::max());
  Buf<uint> isBest = u_value(nTriplets, 0);
  launch(rt, refk::kBarrier_followerBestBasisStore, [&] {
    refk::followerBestBasisStore(followerBasisPS.p(), ptDiff.p(), basisIndices.p(), R.best.p(), isBest.p(),
                                 nTriplets);
  });
  R.trackOffsets = u_uninit((size_t)nTriplets + 1);
  launch(rt, refk::kBarrier_handlersStateStore, [&] {
    refk::handlersStateStore(states.p(), isBest.p(), R.trackOffsets.p(), nTriplets);
  });
  ps.run(R.trackOffsets.p(), (uint)R.trackOffsets.count, R.T);
  const uint length = R.trackOffsets[R.trackOffsets.count - 1];
  R.states = states;
  // trackCollectionStore walks `length` best-basis steps from each handler; a
  // walk that reaches a follower without a best basis (UINT_MAX) would read
  // far past the array in the reference.  Such runs are reported, not run.
  for (uint t = 0; t < nTriplets; ++t) {
    uint len = R.trackOffsets[t + 1] - R.trackOffsets[t];
    uint b = t;
    for (uint i = 0; i < len; ++i) {
      if (b >= nTriplets) {
        ++R.st.ca_chain_broken;
        break;
      }
      b = R.best[b];
    }
  }
  R.tracks = u_uninit(length);
  if (R.st.ca_chain_broken) return;
  launch(rt, refk::kBarrier_trackCollectionStore, [&] {
    refk::trackCollectionStore(R.best.p(), R.trackOffsets.p(), R.tracks.p(), nTriplets);
  });
}

}  // namespace

struct ref_result {
  std::map<std::string, std::vector<uint32_t>> arrays;
};

namespace {

thread_local std::string g_error;

template <class T>
std::vector<uint32_t> words(const Buf<T>& b) {
  std::vector<uint32_t> w(b.count * sizeof(T) / 4);
  if (!w.empty()) memcpy(w.data(), b.v.data(), w.size() * 4);
  return w;
}

template <class T>
Buf<T> upload(const T* src, size_t n, T slack) {
  Buf<T> b;
  b.alloc(n, slack, slack);
  if (n) memcpy(b.v.data(), src, n * sizeof(T));
  return b;
}

}  // namespace

extern "C" {

// Runs the chain on one event group holding all events of `in`, with
// exec.threads = n_threads and a device local-memory size of local_mem_bytes
// (0: the no-local-memory kernel variants).  Returns 0, or -1 with
// ref_last_error() on invalid input.
int ref_run(const oracle_input* in, uint32_t n_threads, uint32_t local_mem_bytes, uint32_t max_ca_iterations,
            ref_result** out) {
  *out = nullptr;
  if (!in || n_threads == 0 || in->n_events == 0 || in->n_layers == 0 || in->n_z == 0 || in->n_phi == 0) {
    g_error = "invalid input";
    return -1;
  }
  Run R;
  R.in = in;
  R.T = n_threads;
  R.localMem = local_mem_bytes;
  R.E = in->n_events;
  R.L = in->n_layers;
  R.nZ = in->n_z;
  R.nP = in->n_phi;
  R.C = (R.nZ + 1) * (R.nP + 1);
  R.nLT = in->n_lt;
  R.H = in->n_hits;
  R.P = R.H;
  // GridConfig (Grid.h): MIN/MAX as float constants, sector sizes in float
  const float MIN_Z = -300, MAX_Z = 300;
  const float MIN_PHI = (float)-M_PI, MAX_PHI = (float)M_PI;
  R.MIN_Z = MIN_Z;
  R.MIN_PHI = MIN_PHI;
  R.sZ = (MAX_Z - MIN_Z) / R.nZ;
  R.sP = (MAX_PHI - MIN_PHI) / R.nP;
  // TripletConfigurations::minRadiusCurvature(minPt, Bz) with the double
  // IDEAL_BZ passed to its float Bz parameter (TripletConfiguration.h:56-70,
  // TripletConfiguration.cpp:36-43)
  {
    const double IDEAL_BZ = 3.8112;
    const float Bz = (float)IDEAL_BZ;
    const double Q = 1.602177E-19;
    const double GEV_C = 5.344286E-19;
    R.minRc = (float)(in->min_pt * GEV_C / (Bz * Q) * 1E2);
  }
  const size_t EL = (size_t)R.E * R.L;
  R.eventOffsets = upload(in->event_offsets, R.E, kUninit);
  R.layerHits = upload(in->layer_hits, EL, kUninit);
  R.layerOffsets = upload(in->layer_offsets, EL, kUninit);
  R.minR = upload(in->min_r, R.L, uninit_f());
  R.maxR = upload(in->max_r, R.L, uninit_f());
  R.l1 = upload(in->lt_layer1, R.nLT, kUninit);
  R.l2 = upload(in->lt_layer2, R.nLT, kUninit);
  R.l3 = upload(in->lt_layer3, R.nLT, kUninit);
  R.spreadZ = upload(in->lt_pair_spread_z, R.nLT, kUninit);
  R.spreadPhi = upload(in->lt_pair_spread_phi, R.nLT, kUninit);
  R.nCand = upload(in->lt_n_candidates, R.nLT, kUninit);
  R.dTheta = upload(in->lt_dtheta_cut, R.nLT, uninit_f());
  R.sigmaZ = upload(in->lt_sigma_z, R.nLT, uninit_f());
  R.dPhi = upload(in->lt_dphi_cut, R.nLT, uninit_f());
  R.sigmaPhi = upload(in->lt_sigma_phi, R.nLT, uninit_f());
  R.tip = upload(in->lt_tip_cut, R.nLT, uninit_f());
  R.z0 = upload(in->lt_z0, R.nLT, uninit_f());
  R.x = upload(in->x, R.H, uninit_f());
  R.y = upload(in->y, R.H, uninit_f());
  R.z = upload(in->z, R.H, uninit_f());
  R.layer = upload(in->layer, R.H, kUninit);
  R.det = upload(in->det_id, R.H, kUninit);
  R.hit = upload(in->hit_id, R.H, kUninit);
  R.evt = upload(in->event, R.H, kUninit);
  // the appended hit: NaN coordinates, layer 1, event 0
  const float nan = std::numeric_limits<float>::quiet_NaN();
  R.x[R.P] = nan;
  R.y[R.P] = nan;
  R.z[R.P] = nan;
  R.layer[R.P] = 1;
  R.det[R.P] = 0;
  R.hit[R.P] = 0;
  R.evt[R.P] = 0;

  grid_build(R);
  pair_gen(R);
  predict(R);
  filter(R);
  auto* res = new ref_result;
  auto& A = res->arrays;
  A["hx"] = words(R.x);
  A["hy"] = words(R.y);
  A["hz"] = words(R.z);
  A["hlayer"] = words(R.layer);
  A["hdet"] = words(R.det);
  A["hhit"] = words(R.hit);
  A["hevt"] = words(R.evt);
  for (auto* k : {"hx", "hy", "hz", "hlayer", "hdet", "hhit", "hevt"}) A[k].resize(R.H);  // drop the appended hit
  A["grid"] = words(R.grid);
  A["pairs"] = words(R.pairs);
  A["pair_offsets"] = words(R.pairOffsets);
  A["cands"] = words(R.cands);
  A["cand_offsets"] = words(R.candOffsets);
  A["trip_h1"] = words(R.t1);
  A["trip_h2"] = words(R.t2);
  A["trip_h3"] = words(R.t3);
  A["trip_offsets"] = words(R.tOffsets);
  if (connectivity(R, in->d_eta_cut)) {
    circle_fit(R);
    cellular_automaton(R, max_ca_iterations);
    A["eta"] = words(R.eta);
    A["link_basis"] = words(R.basis);
    A["link_follower"] = words(R.follower);
    A["connectable"] = words(R.connectable);
    A["non_connectable"] = words(R.nonConnectable);
    A["pt"] = words(R.pt);
    A["ca_states"] = words(R.states);
    A["ca_best"] = words(R.best);
    A["tracks"] = words(R.tracks);
    A["track_offsets"] = words(R.trackOffsets);
  } else {
    A["eta"] = words(R.eta);
  }
  A["stats"] = {R.st.pair_sentinels, R.st.cand_sentinels, R.st.ca_iterations,     R.st.no_links,
                R.st.ca_chain_broken, R.st.grid_count_local, R.st.grid_store_variant, R.st.pair_count_local};
  *out = res;
  return 0;
}

// CellularAutomaton::run alone (CellularAutomaton.h:43-49, .cpp:7-465) on
// given links and pt, with exec.threads = n_threads.
int ref_ca(uint32_t n_triplets, const uint32_t* basis, const uint32_t* follower, uint32_t n_links, const float* pt,
           uint32_t n_threads, uint32_t max_ca_iterations, ref_result** out) {
  *out = nullptr;
  if (n_threads == 0 || n_triplets == 0 || n_links == 0) {
    g_error = "the CA needs triplets, links and work-items";
    return -1;
  }
  Run R;
  R.T = n_threads;
  R.basis = upload(basis, n_links, kUninit);
  R.follower = upload(follower, n_links, kUninit);
  R.pt = upload(pt, n_triplets, uninit_f());
  cellular_automaton(R, max_ca_iterations);
  auto* res = new ref_result;
  auto& A = res->arrays;
  A["ca_states"] = words(R.states);
  A["ca_best"] = words(R.best);
  A["tracks"] = words(R.tracks);
  A["track_offsets"] = words(R.trackOffsets);
  A["stats"] = {R.st.pair_sentinels, R.st.cand_sentinels, R.st.ca_iterations,     R.st.no_links,
                R.st.ca_chain_broken, R.st.grid_count_local, R.st.grid_store_variant, R.st.pair_count_local};
  *out = res;
  return 0;
}

// The reference's CPU path over many events: each event is its own event
// group (the reference's eventGrouping = 1) and the groups run on `workers`
// host threads.  Only the triplet count of each event is returned (in
// triplets[e]); this is what the CPU baseline times.  Returns 0, or -1 on
// invalid input.
int ref_run_events(const oracle_input* in, uint32_t n_threads, uint32_t local_mem_bytes, uint32_t workers,
                   uint64_t* triplets) {
  if (!in || in->n_events == 0 || n_threads == 0) {
    g_error = "invalid input";
    return -1;
  }
  const uint32_t E = in->n_events, L = in->n_layers;
  std::atomic<uint32_t> next{0};
  std::atomic<int> failed{0};
  auto work = [&] {
    for (uint32_t e = next++; e < E; e = next++) {
      const uint32_t first = in->event_offsets[e];
      const uint32_t last = e + 1 < E ? in->event_offsets[e + 1] : in->n_hits;
      oracle_input one = *in;
      std::vector<uint32_t> evt(last - first, 0u);
      const uint32_t zero = 0;
      one.n_hits = last - first;
      one.x = in->x + first;
      one.y = in->y + first;
      one.z = in->z + first;
      one.layer = in->layer + first;
      one.det_id = in->det_id + first;
      one.hit_id = in->hit_id + first;
      one.event = evt.data();
      one.n_events = 1;
      one.event_offsets = &zero;
      one.layer_hits = in->layer_hits + (size_t)e * L;
      one.layer_offsets = in->layer_offsets + (size_t)e * L;
      ref_result* r = nullptr;
      if (ref_run(&one, n_threads, local_mem_bytes, 100000, &r) != 0) {
        failed = 1;
        return;
      }
      triplets[e] = r->arrays["trip_h1"].size();
      delete r;
    }
  };
  std::vector<std::thread> pool;
  for (uint32_t w = 1; w < std::max(workers, 1u); ++w) pool.emplace_back(work);
  work();
  for (auto& t : pool) t.join();
  return failed ? -1 : 0;
}

const char* ref_last_error(void) { return g_error.c_str(); }

int64_t ref_size(const ref_result* r, const char* name) {
  auto it = r->arrays.find(name);
  return it == r->arrays.end() ? -1 : (int64_t)it->second.size();
}

int ref_copy(const ref_result* r, const char* name, void* dst) {
  auto it = r->arrays.find(name);
  if (it == r->arrays.end()) return -1;
  if (!it->second.empty()) memcpy(dst, it->second.data(), it->second.size() * 4);
  return 0;
}

void ref_free(ref_result* r) { delete r; }

// PrefixSum::run over `n` elements in place with work-groups of `wg`
// work-items: the reference's recursive Blelloch scan kernels.
void ref_prefix_sum(uint32_t* data, uint32_t n, uint32_t wg) {
  Buf<uint> b = upload(data, n, kUninit);
  PrefixSum().run(b.p(), n, wg);
  memcpy(data, b.p(), (size_t)n * 4);
}

// The reference's track evaluation on a CA output: its extractTracks,
// cloneRemoval, splitRealFakeTracks and findUniqueRealTracks
// (TripletBuilder.cpp, in ref_tracks.cpp), and the five counts printTracks
// reports from them (TripletBuilder.cpp:1016-1021, 1047-1051): out5 = total, filtered,
// valid, valid unique, fakes.  tracks[n_entries] and track_offsets
// [n_offsets] are the CA's trackCollection and its handler prefix sum;
// h1..h3 the triplets; hit_id the simulated track of every hit.
void ref_track_metrics(const uint32_t* tracks, uint64_t n_entries, const uint32_t* track_offsets,
                       uint64_t n_offsets, const uint32_t* h1, const uint32_t* h2, const uint32_t* h3,
                       const uint32_t* hit_id, uint64_t* out5) {
  using namespace reftr;
  const std::vector<uint> vTrackCollection(tracks, tracks + n_entries);
  const std::vector<uint> vPSum(track_offsets, track_offsets + n_offsets);
  const std::vector<float> vPt;  // unused by extractTracks
  TrackletCollection tracklets;
  tracklets.h1 = h1;
  tracklets.h2 = h2;
  tracklets.h3 = h3;
  HitCollection hits;
  hits.hitId = hit_id;
  TrackCollection reconstructed;
  if (n_offsets > 0) reconstructed = extractTracks(vTrackCollection, vPSum, &tracklets, hits, vPt);
  const TrackCollection filtered = cloneRemoval(reconstructed);
  TrackCollection real, fake;
  std::tie(real, fake) = splitRealFakeTracks(filtered, hits);
  const std::map<uint, Track> unique = findUniqueRealTracks(real, hits);
  out5[0] = reconstructed.size();
  out5[1] = filtered.size();
  out5[2] = real.size();
  out5[3] = unique.size();
  out5[4] = fake.size();
}

}  // extern "C"
