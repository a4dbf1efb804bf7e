// trax_oracle.cpp -- CPU oracle for the triplet-seeding path.  TEST
// INFRASTRUCTURE ONLY: the tests, the smoke check and the CPU-baseline leg of
// the benchmark load it as the checker; the product never links or calls it.
//
// It restates, kernel by kernel and in the reference's own operation order,
// the OpenCL C of JuantAldea/trax (all file:line citations are paths inside
// that project):
//   grid build    src/algorithms/GridBuilder.h:48-427, GridBuilder.cpp:6-161
//   prefix sum    src/algorithms/PrefixSum.h:58-248, PrefixSum.cpp:47-140
//   pairs         src/algorithms/PairGeneratorBeamspot.h:43-525, .cpp:5-183
//   prediction    src/algorithms/TripletThetaPhiPredictor.h:49-447, .cpp:10-168
//   filter        src/algorithms/TripletThetaPhiFilter.h:50-280, .cpp:10-206
//   connectivity  src/algorithms/TripletConnectivityTight.h:47-346, .cpp:5-475
//   circle fit    src/algorithms/TrackletCircleFitter.h:32-97
//   CA            src/algorithms/CellularAutomaton.h:52-327, .cpp:7-465
//   host config   src/datastructures/Grid.h:5-39, TripletConfiguration.cpp:36-43
// Work-items of one NDRange are executed one after the other.  Where the
// reference's result depends on the order of atomics (grid slot allocation,
// CA best-basis ties) the oracle takes the serial order, which is one of the
// orders the reference can produce:
//   * grid: hits keep their input order inside a cell (GridBuilder.h:243-244);
//   * CA: the bases of a follower are scanned in link order, i.e. ascending
//     basis index (CellularAutomaton.h:201, 254-259).
// Where the reference reads memory it never wrote, the oracle writes a
// sentinel and counts the event in the statistics:
//   * pair slots beyond the distinct bitmap hits (duplicate window visits):
//     inner index 0xffffffff, skipped by the predictor;
//   * candidate slots beyond the store kernel's valid count (rOrigin rounding
//     differs between predictCount and predictStore,
//     TripletThetaPhiPredictor.h:130-131 vs 305-306): hit 0xffffffff,
//     rejected by the filter.
// Grid-offset reads whose cell index falls outside the layer (possible only
// for NaN/inf windows, e.g. a hit with y == 0) are clamped to the last cell
// of the layer; the reference reads out of bounds there.
// The offset monotonize kernels (TripletThetaPhiPredictor.h:432-447,
// TripletThetaPhiFilter.h:267-280) run in parallel in the reference and race
// when two consecutive segments are empty; the oracle applies them serially
// (a running maximum), their documented intent.
#include "trax_oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <memory>
#include <vector>

#include "../trax_gb300/csrc/trax_math.h"

using trax::acos_;
using trax::asinh_;
using trax::atan2_;
using trax::atan_;
using trax::div_;
using trax::f2i_sat;
using trax::f2u_sat;
using trax::fabs_;
using trax::floor_;
using trax::sqrt_;
typedef uint32_t uint;

#define M_PI_F TRAX_PI_F

namespace {

std::mutex g_err_mu;
std::string g_last_error;

void set_error(const std::string& s) {
  std::lock_guard<std::mutex> lk(g_err_mu);
  g_last_error = s;
}

const uint SENTINEL = 0xffffffffu;

struct Group {
  std::map<std::string, std::vector<uint32_t>> a;
  std::vector<uint32_t>& u(const char* n) { return a[n]; }
  void put_f(const char* n, const std::vector<float>& v) {
    std::vector<uint32_t>& d = a[n];
    d.resize(v.size());
    if (!v.empty()) memcpy(d.data(), v.data(), v.size() * 4);
  }
};

// exclusive scan in place, total in the last slot (PrefixSum: the element
// count is n+1 and the total is read from index n; uint32 wrap-around)
void exclusive_scan(std::vector<uint>& v, size_t n) {
  uint acc = 0;
  for (size_t i = 0; i < n; ++i) {
    uint t = v[i];
    v[i] = acc;
    acc += t;
  }
}

struct Hits {
  std::vector<float> x, y, z;
  std::vector<uint> layer, det, hid, evt, orig;
};

// Runs f(begin, end, worker) over [0, n) in chunks of at least `grain` on
// `workers` host threads.  Used only where every index writes its own
// outputs (or the same value to a shared flag), so the results do not
// depend on the number of threads.
template <class F>
void parallel_for(uint64_t n, uint workers, uint64_t grain, F&& f) {
  if (workers <= 1 || n <= grain) {
    if (n) f((uint64_t)0, n, 0u);
    return;
  }
  const uint64_t chunk = std::max<uint64_t>(grain, n / ((uint64_t)workers * 16));
  std::atomic<uint64_t> next(0);
  auto run = [&](uint w) {
    for (;;) {
      const uint64_t b = next.fetch_add(chunk);
      if (b >= n) break;
      f(b, std::min(n, b + chunk), w);
    }
  };
  std::vector<std::thread> th;
  for (uint w = 1; w < workers; ++w) th.emplace_back(run, w);
  run(0);
  for (auto& t : th) t.join();
}

struct Ctx {
  const oracle_input* in;
  uint workers = 1;  // host threads inside this event group
  uint E, L, nZ, nP, C, nLT;
  float minZ, sZ, minPhi, sP;
  float minRcurv;
  std::vector<uint> eventOffsets, layerHits, layerOffsets;
  Hits h;  // current hit collection (input order, then grid order)
};

float min_radius_curvature(float minPt) {
  // TripletConfiguration.cpp:36-43: the double IDEAL_BZ (TripletConfiguration.h:70)
  // passes through minRadiusCurvature's float Bz parameter (:56-64)
  const double IDEAL_BZ = 3.8112;
  const float Bz = (float)IDEAL_BZ;
  const double Q = 1.602177E-19;
  const double GEV_C = 5.344286E-19;
  return (float)(minPt * GEV_C / (Bz * Q) * 1E2);
}

// ----------------------------------------------------------------- grid
// GridBuilder.h:48-115 (count), GridBuilder.cpp:58 (scan), GridBuilder.h:172-257 (store)
bool grid_build(Ctx& c, std::vector<uint>& grid, std::string& err) {
  const Hits& h = c.h;
  grid.assign((size_t)c.E * c.L * c.C, 0u);
  std::vector<uint> cell(h.x.size());
  for (uint e = 0; e < c.E; ++e) {
    for (uint l = 0; l < c.L; ++l) {
      uint hits = c.layerHits[e * c.L + l];
      uint offset = c.eventOffsets[e] + c.layerOffsets[e * c.L + l];
      for (uint i = 0; i < hits; ++i) {
        uint k = offset + i;
        uint zSector = f2u_sat(floor_(div_(h.z[k] - c.minZ, c.sZ)));
        float phi = atan2_(h.y[k], h.x[k]);
        uint phiSector = f2u_sat(floor_(div_(phi - c.minPhi, c.sP)));
        if (zSector >= c.nZ || phiSector > c.nP) {
          char buf[160];
          snprintf(buf, sizeof buf, "hit %u outside the grid (z=%g, z row %u of %u)", k,
                   (double)h.z[k], zSector, c.nZ);
          err = buf;
          return false;
        }
        uint cc = zSector * (c.nP + 1) + phiSector;
        cell[k] = cc;
        grid[((size_t)e * c.L + l) * c.C + cc] += 1;
      }
    }
  }
  exclusive_scan(grid, grid.size());
  std::vector<uint> written(grid.size(), 0u);
  Hits o;
  size_t n = h.x.size();
  o.x.resize(n); o.y.resize(n); o.z.resize(n);
  o.layer.resize(n); o.det.resize(n); o.hid.resize(n); o.evt.resize(n); o.orig.resize(n);
  for (uint e = 0; e < c.E; ++e) {
    for (uint l = 0; l < c.L; ++l) {
      uint hits = c.layerHits[e * c.L + l];
      uint offset = c.eventOffsets[e] + c.layerOffsets[e * c.L + l];
      size_t base = ((size_t)e * c.L + l) * c.C;
      for (uint i = 0; i < hits; ++i) {
        uint k = offset + i;
        uint w = grid[base + cell[k]] + written[base + cell[k]]++;
        o.x[w] = h.x[k]; o.y[w] = h.y[k]; o.z[w] = h.z[k];
        o.layer[w] = h.layer[k]; o.det[w] = h.det[k]; o.hid[w] = h.hid[k];
        o.evt[w] = h.evt[k]; o.orig[w] = h.orig[k];
      }
    }
  }
  c.h = o;
  return true;
}

// layer-local grid read, clamped to the last cell of the layer
inline uint cell_at(const uint* lGrid, uint k, uint C) { return lGrid[k < C ? k : C - 1]; }

// ----------------------------------------------------------------- pairs
struct PairOut {
  std::vector<uint> pairs;  // 2 per pair: inner, outer
  std::vector<uint> offsets;
  uint64_t dupSlots = 0;
  uint64_t windowTests = 0;
};

// PairGeneratorBeamspot.h:43-246 (pairCount) and 448-525 (pairStore) for all
// (event, layer triplet) segments, emulating nThreads work-items per segment.
// One (event, layer triplet) segment: its pairs, positions counted from 0.
struct SegmentPairs {
  std::vector<uint> pairs;
  uint64_t windowTests = 0;
};

void pair_segment(const Ctx& c, const std::vector<uint>& grid, uint e, uint p, SegmentPairs& po) {
  const oracle_input* in = c.in;
  const Hits& h = c.h;
  uint running = 0;  // exclusive prefix over this segment's threads
  {
    {
      uint layer = in->lt_layer2[p] - 1;
      const uint* lGrid2 = &grid[((size_t)e * c.L + layer) * c.C];
      uint layer2Offset = lGrid2[0];
      uint end = lGrid2[c.C - 1];
      uint nHits2 = end - layer2Offset;
      layer = in->lt_layer1[p] - 1;
      const uint* lGrid1 = &grid[((size_t)e * c.L + layer) * c.C];
      uint nHits1 = lGrid1[c.C - 1] - lGrid1[0];
      uint offset = lGrid1[0];
      float z0 = in->lt_z0[p];
      float tip = in->lt_tip_cut[p];
      float sigmaZ = in->lt_sigma_z[p];
      float sigmaPhi;  // Q1: the uint column pairSpreadPhi bound to a float* parameter
      memcpy(&sigmaPhi, &in->lt_pair_spread_phi[p], 4);
      float minR1 = in->min_r[layer];
      float maxR1 = in->max_r[layer];
      uint T = in->n_threads ? in->n_threads : std::max(nHits2, 1u);
      std::vector<uint32_t> oracle(((uint64_t)nHits1 * nHits2 + 31) / 32, 0u);
      std::vector<uint> counts(T, 0u);
      for (uint t = 0; t < T; ++t) {
        uint nFound = 0;
        for (uint i = layer2Offset + t; i < end; i += T) {
          float signRadius = trax::cl_sign(h.y[i]);
          float r = signRadius * sqrt_(h.x[i] * h.x[i] + h.y[i] * h.y[i]);
          float cotThetaHigh = div_(h.z[i] - z0, r);
          float cotThetaLow = div_(h.z[i] + z0, r);
          float tmp = signRadius * maxR1 * cotThetaHigh + z0;
          float zHigh = signRadius * minR1 * cotThetaHigh + z0;
          zHigh = (float)(tmp < zHigh) * zHigh + (float)(tmp > zHigh) * tmp;
          tmp = signRadius * maxR1 * cotThetaLow - z0;
          float zLow = signRadius * minR1 * cotThetaLow - z0;
          zLow = (float)(tmp < zLow) * tmp + (float)(tmp > zLow) * zLow;
          zLow -= sigmaZ;
          zHigh += sigmaZ;
          uint zLowSector = (uint)std::max(f2i_sat(floor_(div_(zLow - c.minZ, c.sZ))), 0);
          uint zHighSector = std::min(f2u_sat(floor_(div_(zHigh - c.minZ, c.sZ))) + 1u, c.nZ);
          float phi = atan2_(h.y[i], h.x[i]);
          float twoR = 2 * c.minRcurv;
          tmp = fabs_(acos_(div_(r, twoR)) - acos_(div_(maxR1, twoR)));
          float dPhi = fabs_(acos_(div_(r, twoR)) - acos_(div_(minR1, twoR)));
          dPhi = (float)(tmp < dPhi) * dPhi + (float)(tmp > dPhi) * tmp;
          tmp = div_(atan_(tip * (r - minR1)), r * minR1);               // Q3
          float phiHigh = div_(atan_(tip * (r - maxR1)), r * maxR1);
          dPhi += tmp > phiHigh ? tmp : phiHigh;
          float phiLow = phi - dPhi - sigmaPhi;
          phiHigh = phi + dPhi + sigmaPhi;
          bool wrapAround = phiLow < -M_PI_F || phiHigh > M_PI_F || phiLow > M_PI_F || phiHigh < -M_PI_F;
          phiLow -= (float)((phiLow > M_PI_F) * 2) * M_PI_F;
          phiLow += (float)((phiLow < -M_PI_F) * 2) * M_PI_F;
          phiHigh -= (float)((phiHigh > M_PI_F) * 2) * M_PI_F;
          phiHigh += (float)((phiHigh < -M_PI_F) * 2) * M_PI_F;
          uint phiLowSector = f2u_sat(floor_(div_(phiLow - c.minPhi, c.sP)));
          uint phiHighSector = f2u_sat(floor_(div_(phiHigh - c.minPhi, c.sP)) + 1);
          uint w = wrapAround ? 1u : 0u;
          for (uint zSector = zLowSector; zSector < zHighSector; ++zSector) {
            uint zSectorStart = cell_at(lGrid1, zSector * (c.nP + 1), c.C);
            uint zSectorEnd = cell_at(lGrid1, (zSector + 1) * (c.nP + 1) - 1, c.C);
            uint zSectorLength = zSectorEnd - zSectorStart;
            uint j = cell_at(lGrid1, zSector * (c.nP + 1) + phiLowSector, c.C);
            uint end2 = w * zSectorEnd + cell_at(lGrid1, zSector * (c.nP + 1) + phiHighSector, c.C) -
                        w * zSectorStart;
            for (; j < end2; ++j) {
              uint64_t index = j - (uint)(j >= zSectorEnd) * zSectorLength;
              po.windowTests++;
              bool valid = zLow <= h.z[index] && h.z[index] <= zHigh;
              float actPhi = atan2_(h.y[index], h.x[index]);
              valid = valid && ((!wrapAround && (phiLow <= actPhi && actPhi <= phiHigh)) ||
                                (wrapAround && ((phiLow <= actPhi && actPhi <= M_PI_F) ||
                                                (-M_PI_F <= actPhi && actPhi <= phiHigh))));
              nFound += valid;
              if (valid) {
                uint64_t bit = (index - offset) * (uint64_t)nHits2 + i - layer2Offset;
                oracle[bit / 32] |= (1u << (bit % 32));
              }
            }
          }
        }
        counts[t] = nFound;
      }
      // exclusive scan of the per-thread counts continues the global one
      std::vector<uint> prefix(T + 1);
      for (uint t = 0; t < T; ++t) {
        prefix[t] = running;
        running += counts[t];
      }
      prefix[T] = running;
      po.pairs.resize((size_t)running * 2, SENTINEL);
      // pairStore
      for (uint t = 0; t < T; ++t) {
        uint pos = prefix[t];
        uint nextThread = prefix[t + 1];
        for (uint i = layer2Offset + t; i < end; i += T) {
          for (uint j = 0; j < nHits1 && pos < nextThread; ++j) {
            uint64_t index = (uint64_t)j * nHits2 + i - layer2Offset;
            bool valid = (oracle[index / 32] >> (index % 32)) & 1u;
            if (valid) {
              po.pairs[2 * (size_t)pos] = j + offset;
              po.pairs[2 * (size_t)pos + 1] = i;
            }
            pos += valid;
          }
        }
      }
      // slots the store kernel never reached stay as written above (sentinel)
    }
  }
}

// The segments on the group's threads, concatenated in (event, layer
// triplet) order; pairOffsets[e * nLT + p + 1] is the running total after
// each segment (pairStore's last thread writes it).
void pair_gen(Ctx& c, const std::vector<uint>& grid, PairOut& po) {
  const uint nSeg = c.E * c.nLT;
  std::vector<SegmentPairs> seg(nSeg);
  parallel_for(nSeg, c.workers, 1, [&](uint64_t b, uint64_t e, uint) {
    for (uint64_t k = b; k < e; ++k) pair_segment(c, grid, (uint)(k / c.nLT), (uint)(k % c.nLT), seg[k]);
  });
  po.offsets.assign((size_t)nSeg + 1, 0u);
  size_t total = 0;
  for (uint k = 0; k < nSeg; ++k) total += seg[k].pairs.size();
  po.pairs.reserve(total);
  uint running = 0;
  for (uint k = 0; k < nSeg; ++k) {
    po.pairs.insert(po.pairs.end(), seg[k].pairs.begin(), seg[k].pairs.end());
    running += (uint)(seg[k].pairs.size() / 2);
    po.offsets[k + 1] = running;
    po.windowTests += seg[k].windowTests;
    std::vector<uint>().swap(seg[k].pairs);
  }
  for (size_t k = 0; k < po.pairs.size(); k += 2)
    if (po.pairs[k] == SENTINEL) {
      po.pairs[k + 1] = SENTINEL;
      po.dupSlots++;
    }
}

// ------------------------------------------------------------ prediction
struct PredOut {
  std::vector<uint> cands;  // 2 per candidate: pair index, hit3
  std::vector<uint> offsets;
  uint64_t undefinedSlots = 0;  // store found fewer than count (Q4)
  uint64_t truncated = 0;       // store found more than count (Q4), dropped
  uint64_t windowTests = 0;
};

uint predict_pair(Ctx& c, const std::vector<uint>& grid, const uint* pr, uint gid, bool storeVariant,
                  uint* out, uint limit, uint64_t& tests, uint& wrote) {
  const oracle_input* in = c.in;
  const Hits& h = c.h;
  wrote = 0;
  uint firstHit = pr[0];
  uint secondHit = pr[1];
  if (firstHit == SENTINEL) return 0;
  uint event = h.evt[firstHit];
  uint layerTriplet = h.layer[firstHit] - 1;  // Q7
  uint layer = in->lt_layer3[layerTriplet] - 1;
  const uint* lGrid3 = &grid[((size_t)event * c.L + layer) * c.C];
  uint nFound = 0;
  float sigmaZ = in->lt_sigma_z[layerTriplet];
  float sigmaPhi = in->lt_sigma_phi[layerTriplet];
  float minLayerRadius = in->min_r[layer];
  float maxLayerRadius = in->max_r[layer];
  float p1x = h.x[firstHit], p1y = h.y[firstHit], p1z = h.z[firstHit];
  float p2x = h.x[secondHit], p2y = h.y[secondHit], p2z = h.z[secondHit];
  float tip2 = p1y * (p2x - p1x) - p1x * (p2y - p1y);
  tip2 *= tip2;
  tip2 = div_(tip2, (p2x - p1x) * (p2x - p1x) + (p2y - p1y) * (p2y - p1y));
  float rOrigin;
  if (!storeVariant) {
    rOrigin = p1x * p1x + p1y * p1y;        // :130
    rOrigin = sqrt_(rOrigin - tip2);        // :131
  } else {
    rOrigin = sqrt_(p1x * p1x + p1y * p1y); // :305
    rOrigin = sqrt_(rOrigin * rOrigin - tip2);  // :306
  }
  float cotTheta = div_(p2z - p1z, sqrt_(p2x * p2x + p2y * p2y - tip2) - rOrigin);
  float tmp = p1z + (sqrt_(maxLayerRadius * maxLayerRadius - tip2) - rOrigin) * cotTheta;
  float zLow = p1z + (sqrt_(minLayerRadius * minLayerRadius - tip2) - rOrigin) * cotTheta;
  float zHigh = (float)(tmp > zLow) * tmp + (float)(tmp < zLow) * zLow;
  zLow = (float)(tmp > zLow) * zLow + (float)(tmp < zLow) * tmp;
  zLow -= sigmaZ;
  zHigh += sigmaZ;
  uint zLowSector = (uint)std::max(f2i_sat(floor_(div_(zLow - c.minZ, c.sZ))), 0);
  uint zHighSector = std::min(f2u_sat(floor_(div_(zHigh - c.minZ, c.sZ))) + 1u, c.nZ);
  float phi = atan2_(p2y, p2x);
  tmp = atan2_(p1y, p1x);
  float dPhi = phi - tmp;
  dPhi += (dPhi > M_PI_F) ? -2 * M_PI_F : (dPhi < -M_PI_F) ? 2 * M_PI_F : 0;
  dPhi = fabs_(dPhi);
  float dHits = sqrt_((p2x - p1x) * (p2x - p1x) + (p2y - p1y) * (p2y - p1y));
  float twoR = 2 * c.minRcurv;
  tmp = fabs_(acos_(div_(dHits, twoR)) - acos_(div_(maxLayerRadius, twoR)));
  float phiLow = fabs_(acos_(div_(dHits, twoR)) - acos_(div_(minLayerRadius, twoR)));
  dPhi = trax::cl_max(dPhi, trax::cl_max(tmp, phiLow));
  float phiHigh = phi + dPhi + sigmaPhi;
  phiLow = phi - dPhi - sigmaPhi;
  bool wrapAround = phiLow < -M_PI_F || phiHigh > M_PI_F || phiLow > M_PI_F || phiHigh < -M_PI_F;
  phiLow -= (float)((phiLow > M_PI_F) * 2) * M_PI_F;
  phiLow += (float)((phiLow < -M_PI_F) * 2) * M_PI_F;
  phiHigh -= (float)((phiHigh > M_PI_F) * 2) * M_PI_F;
  phiHigh += (float)((phiHigh < -M_PI_F) * 2) * M_PI_F;
  uint phiLowSector = std::max(f2u_sat(floor_(div_(phiLow - c.minPhi, c.sP))), 0u);
  uint phiHighSector = std::min(f2u_sat(floor_(div_(phiHigh - c.minPhi, c.sP))) + 1u, c.nP);
  uint w = wrapAround ? 1u : 0u;
  uint pos = 0;
  for (uint zSector = zLowSector; zSector < zHighSector; ++zSector) {
    uint zSectorStart = cell_at(lGrid3, zSector * (c.nP + 1), c.C);
    uint zSectorEnd = cell_at(lGrid3, (zSector + 1) * (c.nP + 1), c.C);  // Q8
    uint zSectorLength = zSectorEnd - zSectorStart;
    uint end2 = w * zSectorEnd + cell_at(lGrid3, zSector * (c.nP + 1) + phiHighSector, c.C) -
                w * zSectorStart;
    // The store kernel stops at pos == nextThread (:376-377).  The loop below
    // keeps counting past that point without writing, only so that the
    // statistics can report how many valid hits were dropped.
    for (uint j = cell_at(lGrid3, zSector * (c.nP + 1) + phiLowSector, c.C); j < end2; ++j) {
      uint64_t index = j - (uint)(j >= zSectorEnd) * zSectorLength;
      tests++;
      bool valid = zLow <= h.z[index] && h.z[index] <= zHigh;
      float actPhi = atan2_(h.y[index], h.x[index]);
      valid = valid && ((!wrapAround && (phiLow <= actPhi && actPhi <= phiHigh)) ||
                        (wrapAround && ((phiLow <= actPhi && actPhi <= M_PI_F) ||
                                        (-M_PI_F <= actPhi && actPhi <= phiHigh))));
      if (storeVariant && valid && pos < limit) {
        out[2 * pos] = gid;
        out[2 * pos + 1] = (uint)index;
        wrote++;
      }
      pos += valid;
      nFound += valid;
    }
  }
  return nFound;
}

// TripletThetaPhiPredictor::run (.cpp:10-168)
void predict(Ctx& c, const std::vector<uint>& grid, const PairOut& po, PredOut& pr) {
  uint nPairs = (uint)(po.pairs.size() / 2);
  std::vector<uint> prefix((size_t)nPairs + 1, 0u);
  std::vector<uint64_t> tests(c.workers, 0), truncated(c.workers, 0), undefinedSlots(c.workers, 0);
  parallel_for(nPairs, c.workers, 4096, [&](uint64_t b, uint64_t e, uint w) {
    for (uint g = (uint)b; g < (uint)e; ++g) {
      uint wrote;
      prefix[g] = predict_pair(c, grid, &po.pairs[2 * (size_t)g], g, false, nullptr, 0, tests[w], wrote);
    }
  });
  for (uint64_t t : tests) pr.windowTests += t;
  exclusive_scan(prefix, prefix.size());
  uint total = prefix[nPairs];
  pr.cands.assign((size_t)total * 2, SENTINEL);
  pr.offsets.assign((size_t)c.E * c.nLT + 1, 0u);
  parallel_for(nPairs, c.workers, 4096, [&](uint64_t b, uint64_t e, uint w) {
   uint64_t dummy = 0;
   for (uint g = (uint)b; g < (uint)e; ++g) {
    uint pos = prefix[g], next = prefix[g + 1];
    uint wrote = 0;
    uint storeValid =
        predict_pair(c, grid, &po.pairs[2 * (size_t)g], g, true,
                     next > pos ? &pr.cands[2 * (size_t)pos] : nullptr, next - pos, dummy, wrote);
    if (storeValid > next - pos) truncated[w] += storeValid - (next - pos);
    if (wrote < next - pos) {
      undefinedSlots[w] += (next - pos) - wrote;
      for (uint k = pos + wrote; k < next; ++k) {
        pr.cands[2 * (size_t)k] = g;
        pr.cands[2 * (size_t)k + 1] = SENTINEL;
      }
    }
    // tripletOffsets (:405-418)
    const uint* p = &po.pairs[2 * (size_t)g];
    if (p[0] == SENTINEL) continue;
    uint event = c.h.evt[p[0]];
    uint layerTriplet = c.h.layer[p[0]] - 1;
    if (g < nPairs - 1) {
      const uint* q = &po.pairs[2 * (size_t)(g + 1)];
      uint nextEvent = q[0] == SENTINEL ? SENTINEL : c.h.evt[q[0]];
      uint nextLT = q[0] == SENTINEL ? SENTINEL : c.h.layer[q[0]] - 1;
      if (layerTriplet != nextLT || event != nextEvent)
        pr.offsets[(size_t)event * c.nLT + layerTriplet + 1] = next;
    } else {
      pr.offsets[(size_t)event * c.nLT + layerTriplet + 1] = next;
    }
   }
  });
  for (uint w = 0; w < c.workers; ++w) {
    pr.truncated += truncated[w];
    pr.undefinedSlots += undefinedSlots[w];
  }
  for (size_t k = 1; k < pr.offsets.size(); ++k)
    if (pr.offsets[k] == 0) pr.offsets[k] = pr.offsets[k - 1];
}

}  // namespace

namespace {

// ---------------------------------------------------------------- filter
struct FilterOut {
  std::vector<uint> h1, h2, h3;
  std::vector<uint> offsets;
};

// TripletThetaPhiFilter.h:50-162 (filterCount) for one candidate.
bool filter_one(const Ctx& c, const PairOut& po, const uint* cand) {
  const oracle_input* in = c.in;
  const Hits& h = c.h;
  uint thirdHit = cand[1];
  if (thirdHit == SENTINEL) return false;  // slot the reference never wrote
  uint firstHit = po.pairs[2 * (size_t)cand[0]];
  uint secondHit = po.pairs[2 * (size_t)cand[0] + 1];
  uint layerTriplet = h.layer[firstHit] - 1;  // Q7
  float dThetaCut = in->lt_dtheta_cut[layerTriplet];
  float dPhiCut = in->lt_dphi_cut[layerTriplet];
  float tipCut = in->lt_tip_cut[layerTriplet];
  bool valid = true;
  const float* X = h.x.data();
  const float* Y = h.y.data();
  const float* Z = h.z.data();
  float angle1 = atan2_(sqrt_((X[secondHit] - X[firstHit]) * (X[secondHit] - X[firstHit]) +
                              (Y[secondHit] - Y[firstHit]) * (Y[secondHit] - Y[firstHit])),
                        (Z[secondHit] - Z[firstHit]));
  float angle2 = atan2_(sqrt_((X[thirdHit] - X[secondHit]) * (X[thirdHit] - X[secondHit]) +
                              (Y[thirdHit] - Y[secondHit]) * (Y[thirdHit] - Y[secondHit])),
                        (Z[thirdHit] - Z[secondHit]));
  float delta = fabs_(div_(angle2, angle1));
  valid = valid && (1 - dThetaCut <= delta && delta <= 1 + dThetaCut);
  angle1 = atan2_((Y[secondHit] - Y[firstHit]), (X[secondHit] - X[firstHit]));
  angle2 = atan2_((Y[thirdHit] - Y[secondHit]), (X[thirdHit] - X[secondHit]));
  delta = angle2 - angle1;
  delta += (delta > M_PI_F) ? -2 * M_PI_F : (delta < -M_PI_F) ? 2 * M_PI_F : 0;
  valid = valid && (fabs_(delta) <= dPhiCut);
  // circle fit on the paraboloid (Strandlie et al.)
  trax::f3 pP1 = trax::make_f3(X[firstHit], Y[firstHit], X[firstHit] * X[firstHit] + Y[firstHit] * Y[firstHit]);
  trax::f3 pP2 = trax::make_f3(X[secondHit], Y[secondHit], X[secondHit] * X[secondHit] + Y[secondHit] * Y[secondHit]);
  trax::f3 pP3 = trax::make_f3(X[thirdHit], Y[thirdHit], X[thirdHit] * X[thirdHit] + Y[thirdHit] * Y[thirdHit]);
  trax::f3 a = trax::sub3(pP2, pP1);
  trax::f3 b = trax::sub3(pP3, pP1);
  trax::f3 n = trax::cross3(a, b);
  n = trax::normalize3(n);
  float cOx = div_(-n.x, 2 * n.z);
  float cOy = div_(-n.y, 2 * n.z);
  float cc = -(n.x * pP1.x + n.y * pP1.y + n.z * pP1.z);
  float cR = sqrt_(div_(1 - n.z * n.z - 4 * cc * n.z, 4 * n.z * n.z));
  float vx = -cOx, vy = -cOy;
  trax::normalize2(vx, vy);
  float pCAx = cOx + cR * vx;
  float pCAy = cOy + cR * vy;
  float tip_squared = pCAx * pCAx + pCAy * pCAy;
  valid = valid && (tip_squared <= (tipCut * tipCut));
  valid = valid && (cR >= c.minRcurv);
  return valid;
}

void filter_offsets(const Ctx& c, FilterOut& fo);

// TripletThetaPhiFilter::run (.cpp:10-206): count, popcount, scan, store,
// offset store and monotonize.
void filter(const Ctx& c, const PairOut& po, const PredOut& pr, FilterOut& fo) {
  uint nCand = (uint)(pr.cands.size() / 2);
  uint nWords = (nCand + 31) / 32;
  std::vector<uint> oracle(nWords, 0u);
  parallel_for(nWords, c.workers, 256, [&](uint64_t b, uint64_t e, uint) {  // words of 32 candidates
    for (uint64_t g = b; g < e; ++g)
      for (uint gid = (uint)g * 32; gid < std::min(nCand, (uint)g * 32 + 32); ++gid)
        if (filter_one(c, po, &pr.cands[2 * (size_t)gid])) oracle[gid / 32] |= (1u << (gid % 32));
  });
  std::vector<uint> prefix((size_t)nWords + 1, 0u);
  for (uint g = 0; g < nWords; ++g) {
    uint i = oracle[g];  // SWAR popcount (:173-176)
    i = i - ((i >> 1) & 0x55555555u);
    i = (i & 0x33333333u) + ((i >> 2) & 0x33333333u);
    prefix[g] = (((i + (i >> 4)) & 0x0F0F0F0Fu) * 0x01010101u) >> 24;
  }
  exclusive_scan(prefix, prefix.size());
  uint nFound = prefix[nWords];
  fo.h1.assign(nFound, 0u);
  fo.h2.assign(nFound, 0u);
  fo.h3.assign(nFound, 0u);
  parallel_for(nWords, c.workers, 4096, [&](uint64_t b, uint64_t e, uint) {
    for (uint g = (uint)b; g < (uint)e; ++g) {
      uint pos = prefix[g];
      uint lOracle = oracle[g];
      for (uint i = 0; i < 32; ++i) {
        bool valid = (lOracle >> i) & 1u;
        if (valid) {
          const uint* cand = &pr.cands[2 * ((size_t)g * 32 + i)];
          fo.h1[pos] = po.pairs[2 * (size_t)cand[0]];
          fo.h2[pos] = po.pairs[2 * (size_t)cand[0] + 1];
          fo.h3[pos] = cand[1];
        }
        pos += valid;
      }
    }
  });
  filter_offsets(c, fo);
}

// filterOffsetStore (TripletThetaPhiFilter.h:221-257) + monotonize (:267-280)
void filter_offsets(const Ctx& c, FilterOut& fo) {
  const uint nFound = (uint)fo.h1.size();
  fo.offsets.assign((size_t)c.E * c.nLT + 1, 0u);
  for (uint gid = 0; gid < nFound; ++gid) {
    uint hitId = fo.h1[gid];
    uint layerTriplet = c.h.layer[hitId];
    uint event = c.h.evt[hitId];
    if (gid > 0) {
      uint previousHitId = fo.h1[gid - 1];
      if (layerTriplet != c.h.layer[previousHitId] || event != c.h.evt[previousHitId])
        fo.offsets[(size_t)event * c.nLT + layerTriplet - 1] = gid;
      if ((gid + 1) == nFound) fo.offsets[(size_t)event * c.nLT + layerTriplet] = gid;
    } else {
      fo.offsets[(size_t)event * c.nLT + layerTriplet - 1] = gid;
    }
  }
  // filterOffsetMonotonizeStore (:267-280), serial
  for (size_t k = 1; k < fo.offsets.size(); ++k)
    if (fo.offsets[k] == 0) fo.offsets[k] = fo.offsets[k - 1];
}

// ---------------------------------------------------------- connectivity
struct ConnOut {
  std::vector<float> eta;
  std::vector<uint> basis, follower, linkEvent;
  std::vector<uint> connectable, nonConnectable;
  bool noLinks = true;
};

// TripletConnectivityTight.h:83-243 search range of one basis triplet;
// returns false when the kernel returns early.
bool conn_range(const Ctx& c, const FilterOut& fo, uint t, uint& begin, uint& end) {
  uint nOffsets = c.E * c.nLT + 1;
  if (t >= fo.offsets[nOffsets - 2]) return false;
  uint hitIndexInner = fo.h2[t];
  uint hitEventNumber = c.h.evt[hitIndexInner];
  uint hitLayerNumber = c.h.layer[hitIndexInner] - 1;
  size_t k = (size_t)hitEventNumber * c.nLT + hitLayerNumber;
  if (k + 1 >= nOffsets) return false;  // the reference reads past the offsets here
  begin = fo.offsets[k];
  end = fo.offsets[k + 1];
  // an empty range has no follower whose event the reference could compare
  // (it reads one past its triplets there); returning gives the same links
  // and counts as the empty loop
  if (begin >= end || hitEventNumber != c.h.evt[fo.h1[begin]]) return false;
  return true;
}

// The followers of every basis, as the count and store kernels visit them:
// the triplets i in the basis's search range [begin, end) whose (h1, h2) is
// the basis's (h2, h3), in ascending i.  The linear scan of
// TripletConnectivityTight.h:134-139 (links_mode 0), or a lookup in an index
// of all triplets by (h1, h2) (links_mode 1) -- the same indices in the same
// order, without the scan's quadratic cost on large segments.
struct FollowerIndex {
  std::unordered_map<uint64_t, std::vector<uint>> byPair;
  explicit FollowerIndex(const FilterOut& fo) {
    for (uint i = 0; i < (uint)fo.h1.size(); ++i)
      byPair[((uint64_t)fo.h1[i] << 32) | fo.h2[i]].push_back(i);  // ascending i
  }
  template <class F>
  void each(uint inner, uint outer, uint begin, uint end, F&& f) const {
    auto it = byPair.find(((uint64_t)inner << 32) | outer);
    if (it == byPair.end()) return;
    const std::vector<uint>& v = it->second;
    for (auto k = std::lower_bound(v.begin(), v.end(), begin); k != v.end() && *k < end; ++k) f(*k);
  }
};

// TripletConnectivityTight::run (.cpp:5-475)
void connectivity(const Ctx& c, const FilterOut& fo, ConnOut& co) {
  uint nT = (uint)fo.h1.size();
  co.eta.assign(nT, 0.0f);
  parallel_for(nT, c.workers, 4096, [&](uint64_t b, uint64_t e, uint) {
    for (uint t = (uint)b; t < (uint)e; ++t) {  // tripletEtaCalculatorStore (:47-79)
      uint hi = fo.h1[t], ho = fo.h3[t];
      float px = c.h.x[ho] - c.h.x[hi];
      float py = c.h.y[ho] - c.h.y[hi];
      float pz = c.h.z[ho] - c.h.z[hi];
      float tt = div_(pz, sqrt_(px * px + py * py));
      co.eta[t] = asinh_(tt);
    }
  });
  std::vector<uint> flags(nT, 0u);
  std::vector<uint> counts((size_t)nT + 1, 0u);
  float dEtaCut = c.in->d_eta_cut;
  const bool indexed = c.in->links_mode == 1;
  std::unique_ptr<FollowerIndex> index(indexed ? new FollowerIndex(fo) : nullptr);
  // a follower's flag is set by every basis that finds it: the same value,
  // stored with relaxed atomics when bases run on several threads
  auto set_flag = [&](uint i) { __atomic_store_n(&flags[i], 1u, __ATOMIC_RELAXED); };
  parallel_for(nT, c.workers, 1024, [&](uint64_t b, uint64_t e, uint) {
   for (uint t = (uint)b; t < (uint)e; ++t) {  // tripletConnectivityTightCount (:83-160)
    uint begin, end;
    if (!conn_range(c, fo, t, begin, end)) continue;
    uint inner = fo.h2[t], outer = fo.h3[t];
    float localEta = co.eta[t];
    uint cnt = 0;
    if (indexed) {
      index->each(inner, outer, begin, end, [&](uint i) {
        if (fabs_(localEta - co.eta[i]) < dEtaCut) {
          cnt++;
          set_flag(i);
        }
      });
    } else {
      for (uint i = begin; i < end; i++) {
        bool test = (inner == fo.h1[i]) && (outer == fo.h2[i]) && (fabs_(localEta - co.eta[i]) < dEtaCut);
        cnt += test;
        if (test) set_flag(i);
      }
    }
    counts[t] = cnt;
    if (cnt) set_flag(t);
   }
  });
  exclusive_scan(counts, counts.size());
  uint nLinks = counts[nT];
  if (!nLinks) {
    co.noLinks = true;
    return;
  }
  co.noLinks = false;
  co.basis.assign(nLinks, 0u);
  co.follower.assign(nLinks, 0u);
  co.linkEvent.assign(nLinks, 0u);
  parallel_for(nT, c.workers, 1024, [&](uint64_t b, uint64_t e, uint) {
   for (uint t = (uint)b; t < (uint)e; ++t) {  // tripletConnectivityTightStore (:169-236)
    uint begin, end;
    if (!conn_range(c, fo, t, begin, end)) continue;
    uint inner = fo.h2[t], outer = fo.h3[t];
    float localEta = co.eta[t];
    uint storeOffset = counts[t];
    uint next = counts[t + 1];
    uint ev = c.h.evt[inner];
    if (indexed) {
      // the scan's writes for non-matching i land on the slot the next match
      // overwrites: only the matches remain, in ascending i
      index->each(inner, outer, begin, end, [&](uint i) {
        if (storeOffset < next && fabs_(localEta - co.eta[i]) < dEtaCut) {
          co.basis[storeOffset] = t;
          co.follower[storeOffset] = i;
          co.linkEvent[storeOffset] = ev;
          storeOffset++;
        }
      });
      continue;
    }
    for (uint i = begin; (i < end) && (storeOffset < next); i++) {
      bool test = (inner == fo.h1[i]) && (outer == fo.h2[i]) && (fabs_(localEta - co.eta[i]) < dEtaCut);
      co.basis[storeOffset] = t;
      co.follower[storeOffset] = i;
      co.linkEvent[storeOffset] = ev;
      storeOffset += test;
    }
   }
  });
  // connectable / non-connectable index lists over the first nT-1 triplets (Q9)
  uint m = nT - 1;
  std::vector<uint> ps(flags), inv(nT, 0u);
  for (uint k = 0; k < m; ++k) inv[k] = !flags[k];
  exclusive_scan(ps, nT);
  exclusive_scan(inv, nT);
  uint nConn = ps[nT - 1];
  uint nNon = inv[nT - 1];
  co.connectable.assign(nConn, 0u);
  co.nonConnectable.assign(nNon, 0u);
  for (uint gid = 0; gid < m; ++gid) {
    if (ps[gid] != ps[gid + 1]) co.connectable[ps[gid]] = gid;
    if (nNon > 0 && inv[gid] != inv[gid + 1]) co.nonConnectable[inv[gid]] = gid;
  }
}

// ------------------------------------------------------------ circle fit
// TrackletCircleFitter.h:32-97: circle radius of each connectable triplet.
void circle_fit(const Ctx& c, const FilterOut& fo, const ConnOut& co, std::vector<float>& pt) {
  uint nT = (uint)fo.h1.size();
  pt.assign(nT, 0.0f);
  parallel_for(co.connectable.size(), c.workers, 4096, [&](uint64_t b, uint64_t e, uint) {
   for (uint64_t k = b; k < e; ++k) {
    uint tripletIndex = co.connectable[k];
    uint i0 = fo.h1[tripletIndex], i1 = fo.h2[tripletIndex], i2 = fo.h3[tripletIndex];
    trax::f3 pP0 = trax::make_f3(c.h.x[i0], c.h.y[i0], c.h.x[i0] * c.h.x[i0] + c.h.y[i0] * c.h.y[i0]);
    trax::f3 pP1 = trax::make_f3(c.h.x[i1], c.h.y[i1], c.h.x[i1] * c.h.x[i1] + c.h.y[i1] * c.h.y[i1]);
    trax::f3 pP2 = trax::make_f3(c.h.x[i2], c.h.y[i2], c.h.x[i2] * c.h.x[i2] + c.h.y[i2] * c.h.y[i2]);
    trax::f3 a = trax::sub3(pP1, pP0);
    trax::f3 b = trax::sub3(pP2, pP0);
    trax::f3 n = trax::cross3(a, b);
    trax::f3 un = trax::normalize3(n);
    float cc = -trax::dot3(un, pP0);
    float nz2 = un.z * un.z;
    pt[tripletIndex] = sqrt_(div_(1 - nz2 - 4 * cc * un.z, 4 * nz2));
   }
  });
}

// -------------------------------------------------------------------- CA
struct CAOut {
  std::vector<uint> states, best, isBest, tracks, trackOffsets;
  uint iterations = 0;
  bool capped = false;
};

// CellularAutomaton::run (.cpp:7-465) with the kernels of CellularAutomaton.h:52-327
void cellular_automaton(uint nT, const ConnOut& co, const std::vector<float>& pt, CAOut& ca) {
  uint nLinks = (uint)co.basis.size();
  std::vector<uint> S(nT, 1u), N(nT, 1u);
  uint alive;
  ca.iterations = 0;
  do {  // forward phase (:52-98)
    ca.iterations++;
    std::vector<uint> living(nT, 0u);
    for (uint p = 0; p < nLinks; ++p) {
      uint f = co.follower[p];
      uint fs = S[f];
      bool same = S[co.basis[p]] == fs;
      N[f] = std::max(N[f], fs + (uint)same);
      if (same) living[f] = 1;
    }
    alive = 0;
    for (uint v : living) alive += v;
    std::swap(S, N);
    if (ca.iterations > nT + 2) {
      ca.capped = true;
      break;
    }
  } while (alive > 0);
  // backward phase
  std::vector<uint> cnt((size_t)nT + 1, 0u);
  for (uint p = 0; p < nLinks; ++p) {  // followerBasisCount (:141-168)
    uint f = co.follower[p];
    if (S[co.basis[p]] + 1 != S[f]) continue;
    cnt[f]++;
  }
  exclusive_scan(cnt, cnt.size());
  uint total = cnt[nT];
  std::vector<uint> basisIdx(total, 0u);
  std::vector<float> ptDiff(total, 0.0f);
  std::vector<uint> ps(cnt);
  for (uint p = 0; p < nLinks; ++p) {  // followerBasisStore (:173-205), serial atomic order
    uint b = co.basis[p], f = co.follower[p];
    if (S[b] + 1 != S[f]) continue;
    uint slot = ps[f]++;
    basisIdx[slot] = b;
    ptDiff[slot] = fabs_(pt[b] - pt[f]);
  }
  ca.best.assign(nT, 0xffffffffu);
  ca.isBest.assign(nT, 0u);
  for (uint t = 0; t < nT; ++t) {  // followerBestBasisStore (:212-263)
    uint notThread0 = t > 0;
    uint off = (t - 1) * notThread0;
    uint begin = ps[off] * notThread0;
    uint end = ps[off + 1 * notThread0];
    if (begin == end) continue;
    float minPt = ptDiff[begin];
    uint minPtIndex = basisIdx[begin];
    for (uint i = begin + 1; i < end; i++) {
      float d = ptDiff[i];
      uint test = d < minPt;
      minPt = minPt * (float)(!test) + d * (float)test;
      minPtIndex = minPtIndex * (!test) + basisIdx[i] * test;
    }
    ca.best[t] = minPtIndex;
    ca.isBest[minPtIndex] = 1;
  }
  std::vector<uint> h((size_t)nT + 1, 0u);
  for (uint t = 0; t < nT; ++t) h[t] = (ca.isBest[t] == 0) * S[t];  // handlersStateStore (:270-288)
  exclusive_scan(h, h.size());
  uint len = h[nT];
  ca.tracks.assign(len, 0xffffffffu);
  for (uint t = 0; t < nT; ++t) {  // trackCollectionStore (:294-323)
    uint storageOffset = h[t];
    uint length = h[t + 1] - storageOffset;
    uint basisIndex = t;
    for (uint i = 0; i < length && basisIndex != 0xffffffffu; i++) {
      ca.tracks[storageOffset + i] = basisIndex;
      basisIndex = ca.best[basisIndex];
    }
  }
  ca.states = S;
  ca.trackOffsets = h;
}

enum Stat {
  ST_PAIRS = 0, ST_CANDS, ST_TRIPLETS, ST_LINKS, ST_CONNECTABLE, ST_NONCONN, ST_PAIR_DUP,
  ST_CAND_UNDEF, ST_CAND_TRUNC, ST_CA_ITER, ST_TRACK_ENTRIES, ST_PAIR_TESTS_LO, ST_PAIR_TESTS_HI,
  ST_PRED_TESTS_LO, ST_PRED_TESTS_HI, ST_NO_LINKS, ST_CA_CAPPED, ST_N
};

std::string run_group(const oracle_input* in, uint e0, uint e1, Group& G, uint workers) {
  Ctx c;
  c.in = in;
  c.workers = workers;
  c.E = e1 - e0;
  c.L = in->n_layers;
  c.nZ = in->n_z;
  c.nP = in->n_phi;
  c.C = (c.nZ + 1) * (c.nP + 1);
  c.nLT = in->n_lt;
  // Grid.h:9-15, 33-37: sizes computed in float on the host
  const float MIN_Z = -300.0f, MAX_Z = 300.0f;
  const float MIN_PHI = (float)-3.14159265358979323846, MAX_PHI = (float)3.14159265358979323846;
  c.minZ = MIN_Z;
  c.sZ = (MAX_Z - MIN_Z) / (float)c.nZ;
  c.minPhi = MIN_PHI;
  c.sP = (MAX_PHI - MIN_PHI) / (float)c.nP;
  c.minRcurv = min_radius_curvature(in->min_pt);
  uint hit0 = in->event_offsets[e0];
  uint hit1 = (e1 < in->n_events) ? in->event_offsets[e1] : in->n_hits;
  uint n = hit1 - hit0;
  c.eventOffsets.resize(c.E);
  c.layerHits.resize((size_t)c.E * c.L);
  c.layerOffsets.resize((size_t)c.E * c.L);
  for (uint e = 0; e < c.E; ++e) {
    c.eventOffsets[e] = in->event_offsets[e0 + e] - hit0;
    for (uint l = 0; l < c.L; ++l) {
      c.layerHits[e * c.L + l] = in->layer_hits[(size_t)(e0 + e) * c.L + l];
      c.layerOffsets[e * c.L + l] = in->layer_offsets[(size_t)(e0 + e) * c.L + l];
    }
  }
  Hits& h = c.h;
  h.x.assign(in->x + hit0, in->x + hit1);
  h.y.assign(in->y + hit0, in->y + hit1);
  h.z.assign(in->z + hit0, in->z + hit1);
  h.layer.assign(in->layer + hit0, in->layer + hit1);
  h.det.assign(in->det_id + hit0, in->det_id + hit1);
  h.hid.assign(in->hit_id + hit0, in->hit_id + hit1);
  h.evt.resize(n);
  h.orig.resize(n);
  for (uint k = 0; k < n; ++k) {
    h.evt[k] = in->event[hit0 + k] - e0;  // event number within the group
    h.orig[k] = hit0 + k;
  }
  std::vector<uint> grid;
  std::string err;
  if (!grid_build(c, grid, err)) return err;
  G.u("perm") = h.orig;
  G.u("grid") = grid;
  PairOut po;
  pair_gen(c, grid, po);
  PredOut pr;
  predict(c, grid, po, pr);
  FilterOut fo;
  filter(c, po, pr, fo);
  ConnOut co;
  if (in->links_mode != 2) connectivity(c, fo, co);
  std::vector<float> pt;
  CAOut ca;
  uint nT = (uint)fo.h1.size();
  if (in->links_mode != 2 && !co.noLinks) {
    circle_fit(c, fo, co, pt);
    cellular_automaton(nT, co, pt, ca);
  }
  G.u("pairs") = po.pairs;
  G.u("pair_offsets") = po.offsets;
  G.u("cands") = pr.cands;
  G.u("cand_offsets") = pr.offsets;
  G.u("trip_h1") = fo.h1;
  G.u("trip_h2") = fo.h2;
  G.u("trip_h3") = fo.h3;
  G.u("trip_offsets") = fo.offsets;
  G.put_f("eta", co.eta);
  G.u("link_basis") = co.basis;
  G.u("link_follower") = co.follower;
  G.u("connectable") = co.connectable;
  G.u("non_connectable") = co.nonConnectable;
  G.put_f("pt", pt);
  G.u("ca_states") = ca.states;
  G.u("ca_best") = ca.best;
  G.u("tracks") = ca.tracks;
  G.u("track_offsets") = ca.trackOffsets;
  std::vector<uint>& st = G.u("stats");
  st.assign(ST_N, 0u);
  auto sat = [](uint64_t v) { return (uint)std::min<uint64_t>(v, 0xffffffffu); };
  st[ST_PAIRS] = sat(po.pairs.size() / 2);
  st[ST_CANDS] = sat(pr.cands.size() / 2);
  st[ST_TRIPLETS] = nT;
  st[ST_LINKS] = sat(co.basis.size());
  st[ST_CONNECTABLE] = sat(co.connectable.size());
  st[ST_NONCONN] = sat(co.nonConnectable.size());
  st[ST_PAIR_DUP] = sat(po.dupSlots);
  st[ST_CAND_UNDEF] = sat(pr.undefinedSlots);
  st[ST_CAND_TRUNC] = sat(pr.truncated);
  st[ST_CA_ITER] = ca.iterations;
  st[ST_TRACK_ENTRIES] = sat(ca.tracks.size());
  st[ST_PAIR_TESTS_LO] = (uint)(po.windowTests & 0xffffffffu);
  st[ST_PAIR_TESTS_HI] = (uint)(po.windowTests >> 32);
  st[ST_PRED_TESTS_LO] = (uint)(pr.windowTests & 0xffffffffu);
  st[ST_PRED_TESTS_HI] = (uint)(pr.windowTests >> 32);
  st[ST_NO_LINKS] = co.noLinks ? 1u : 0u;
  st[ST_CA_CAPPED] = ca.capped ? 1u : 0u;
  return std::string();
}

// Connectivity, circle fit and CA on caller-provided triplets over a hit
// collection taken as is (TripletConnectivityTight::run takes any
// HitCollection and TrackletCollection, TripletConnectivityTight.h:42-44).
std::string run_link(const oracle_link_input* in, Group& G) {
  Ctx c;
  oracle_input dummy;
  memset(&dummy, 0, sizeof(dummy));
  dummy.d_eta_cut = in->d_eta_cut;
  c.in = &dummy;
  c.E = in->n_events;
  c.L = 0;
  c.nZ = c.nP = c.C = 0;
  c.nLT = in->n_lt;
  if (c.E == 0 || c.nLT == 0) return "need at least one event and one layer triplet";
  Hits& h = c.h;
  h.x.assign(in->x, in->x + in->n_hits);
  h.y.assign(in->y, in->y + in->n_hits);
  h.z.assign(in->z, in->z + in->n_hits);
  h.layer.assign(in->layer, in->layer + in->n_hits);
  h.evt.assign(in->event, in->event + in->n_hits);
  FilterOut fo;
  fo.h1.assign(in->h1, in->h1 + in->n_triplets);
  fo.h2.assign(in->h2, in->h2 + in->n_triplets);
  fo.h3.assign(in->h3, in->h3 + in->n_triplets);
  for (uint t = 0; t < in->n_triplets; ++t) {
    if (fo.h1[t] >= in->n_hits || fo.h2[t] >= in->n_hits || fo.h3[t] >= in->n_hits) return "triplet hit out of range";
    if (h.layer[fo.h1[t]] < 1 || h.layer[fo.h1[t]] > c.nLT || h.evt[fo.h1[t]] >= c.E)
      return "triplet first hit outside the layer-triplet/event range";
  }
  filter_offsets(c, fo);
  ConnOut co;
  connectivity(c, fo, co);
  std::vector<float> pt;
  CAOut ca;
  if (!co.noLinks) {
    circle_fit(c, fo, co, pt);
    cellular_automaton((uint)fo.h1.size(), co, pt, ca);
  }
  G.u("trip_offsets") = fo.offsets;
  G.put_f("eta", co.eta);
  G.u("link_basis") = co.basis;
  G.u("link_follower") = co.follower;
  G.u("connectable") = co.connectable;
  G.u("non_connectable") = co.nonConnectable;
  G.put_f("pt", pt);
  G.u("ca_states") = ca.states;
  G.u("ca_best") = ca.best;
  G.u("tracks") = ca.tracks;
  G.u("track_offsets") = ca.trackOffsets;
  std::vector<uint>& st = G.u("stats");
  st.assign(ST_N, 0u);
  st[ST_TRIPLETS] = (uint)fo.h1.size();
  st[ST_LINKS] = (uint)co.basis.size();
  st[ST_CONNECTABLE] = (uint)co.connectable.size();
  st[ST_NONCONN] = (uint)co.nonConnectable.size();
  st[ST_CA_ITER] = ca.iterations;
  st[ST_TRACK_ENTRIES] = (uint)ca.tracks.size();
  st[ST_NO_LINKS] = co.noLinks ? 1u : 0u;
  return std::string();
}

std::string validate(const oracle_input* in) {
  if (in->n_layers == 0 || in->n_z == 0 || in->n_phi == 0) return "n_layers, n_z and n_phi must be positive";
  uint64_t cells = (uint64_t)(in->n_z + 1) * (in->n_phi + 1);
  if (cells > 0xffffffffull / 4) return "grid too large";
  for (uint p = 0; p < in->n_lt; ++p) {
    if (in->lt_layer1[p] != p + 1) return "layer triplet p must start on layer p+1";
    if (in->lt_layer2[p] < 1 || in->lt_layer2[p] > in->n_layers || in->lt_layer3[p] < 1 ||
        in->lt_layer3[p] > in->n_layers || in->lt_layer1[p] > in->n_layers)
      return "layer triplet refers to a layer outside 1..n_layers";
  }
  uint64_t pos = 0;
  for (uint e = 0; e < in->n_events; ++e) {
    if (in->event_offsets[e] != pos) return "event offsets are not contiguous";
    uint64_t lpos = 0;
    for (uint l = 0; l < in->n_layers; ++l) {
      size_t k = (size_t)e * in->n_layers + l;
      if (in->layer_offsets[k] != lpos) return "layer offsets are not contiguous";
      for (uint i = 0; i < in->layer_hits[k]; ++i) {
        uint64_t hidx = pos + lpos + i;
        if (hidx >= in->n_hits) return "supplements describe more hits than given";
        if (in->layer[hidx] != l + 1 || in->event[hidx] != e) return "hit layer/event columns disagree with the supplements";
        if (trax::is_nan(in->x[hidx]) || trax::is_nan(in->y[hidx]) || trax::is_nan(in->z[hidx]) ||
            trax::is_inf(in->x[hidx]) || trax::is_inf(in->y[hidx]) || trax::is_inf(in->z[hidx]))
          return "hit coordinates must be finite";
      }
      lpos += in->layer_hits[k];
    }
    pos += lpos;
  }
  if (pos != in->n_hits) return "supplements describe fewer hits than given";
  return std::string();
}

}  // namespace

struct oracle_result {
  std::vector<Group> groups;
};

extern "C" {

const char* oracle_last_error(void) {
  std::lock_guard<std::mutex> lk(g_err_mu);
  return g_last_error.c_str();
}

int oracle_run(const oracle_input* in, oracle_result** out) {
  *out = nullptr;
  std::string err = validate(in);
  if (!err.empty()) {
    set_error(err);
    return -1;
  }
  uint G = in->event_grouping ? in->event_grouping : std::max(in->n_events, 1u);
  uint nGroups = (in->n_events + G - 1) / G;
  oracle_result* r = new oracle_result();
  r->groups.resize(nGroups);
  std::vector<std::string> errs(nGroups);
  uint nw = std::max(1u, std::min(in->n_workers, nGroups));
  if (nw <= 1) {
    // one group at a time: the host threads work inside each group
    for (uint g = 0; g < nGroups; ++g)
      errs[g] = run_group(in, g * G, std::min((g + 1) * G, in->n_events), r->groups[g],
                          std::max(1u, in->n_workers));
  } else {
    std::vector<std::thread> th;
    std::atomic<uint> next(0);
    for (uint w = 0; w < nw; ++w)
      th.emplace_back([&]() {
        for (;;) {
          uint g = next.fetch_add(1);
          if (g >= nGroups) break;
          errs[g] = run_group(in, g * G, std::min((g + 1) * G, in->n_events), r->groups[g], 1u);
        }
      });
    for (auto& t : th) t.join();
  }
  for (uint g = 0; g < nGroups; ++g)
    if (!errs[g].empty()) {
      set_error(errs[g]);
      delete r;
      return -2;
    }
  *out = r;
  return 0;
}

int oracle_link(const oracle_link_input* in, oracle_result** out) {
  *out = nullptr;
  oracle_result* r = new oracle_result();
  r->groups.resize(1);
  std::string err = run_link(in, r->groups[0]);
  if (!err.empty()) {
    set_error(err);
    delete r;
    return -1;
  }
  *out = r;
  return 0;
}

// CellularAutomaton::run (CellularAutomaton.h:43-49, .cpp:7-465) alone, on
// given links basis[i] -> follower[i] over n_triplets triplets and one pt per
// triplet (the caller-input form of the CA).
int oracle_ca(uint32_t n_triplets, const uint32_t* basis, const uint32_t* follower, uint32_t n_links,
              const float* pt, oracle_result** out) {
  *out = nullptr;
  for (uint32_t p = 0; p < n_links; ++p) {
    if (basis[p] >= n_triplets || follower[p] >= n_triplets) {
      set_error("link triplet index out of range");
      return -1;
    }
  }
  ConnOut co;
  co.basis.assign(basis, basis + n_links);
  co.follower.assign(follower, follower + n_links);
  co.noLinks = n_links == 0;
  std::vector<float> p(pt, pt + n_triplets);
  CAOut ca;
  cellular_automaton(n_triplets, co, p, ca);
  oracle_result* r = new oracle_result();
  r->groups.resize(1);
  Group& G = r->groups[0];
  G.u("ca_states") = ca.states;
  G.u("ca_best") = ca.best;
  G.u("tracks") = ca.tracks;
  G.u("track_offsets") = ca.trackOffsets;
  std::vector<uint>& st = G.u("stats");
  st.assign(ST_N, 0u);
  st[ST_TRIPLETS] = n_triplets;
  st[ST_LINKS] = n_links;
  st[ST_CA_ITER] = ca.iterations;
  st[ST_CA_CAPPED] = ca.capped ? 1u : 0u;
  st[ST_TRACK_ENTRIES] = (uint)ca.tracks.size();
  *out = r;
  return 0;
}

void oracle_free(oracle_result* r) { delete r; }

uint32_t oracle_n_groups(const oracle_result* r) { return (uint32_t)r->groups.size(); }

int64_t oracle_size(const oracle_result* r, uint32_t g, const char* name) {
  if (g >= r->groups.size()) return -1;
  auto it = r->groups[g].a.find(name);
  if (it == r->groups[g].a.end()) return -1;
  return (int64_t)it->second.size();
}

int oracle_copy(const oracle_result* r, uint32_t g, const char* name, void* dst) {
  if (g >= r->groups.size()) return -1;
  auto it = r->groups[g].a.find(name);
  if (it == r->groups[g].a.end()) return -1;
  if (!it->second.empty()) memcpy(dst, it->second.data(), it->second.size() * 4);
  return 0;
}

// ------------------------------------------------------------ prefix sum
static void blelloch_wg(uint* input, uint size, uint* partial, uint gid, uint ls, uint wg) {
  // one work-group of prefixSumWG / prefixSumPartial (PrefixSum.h:58-221)
  const uint padding = (wg << 1) / 16;
  std::vector<uint> data((size_t)(wg << 1) + padding + 1, 0u);
  auto BANK = [](uint i) { return i >> 4; };
  uint gOffset = gid * (ls << 1);
  for (uint lid = 0; lid < ls; ++lid) {
    data[lid + BANK(lid)] = (gOffset + lid) < size ? input[gOffset + lid] : 0;
    data[lid + ls + BANK(lid + ls)] = (gOffset + lid + ls) < size ? input[gOffset + lid + ls] : 0;
  }
  uint offset = 1;
  for (uint d = ls; d > 0; d >>= 1) {
    for (uint lid = 0; lid < d; ++lid) {
      uint ai = offset * ((lid << 1) + 1) - 1;
      uint bi = offset * ((lid << 1) + 2) - 1;
      ai += BANK(ai);
      bi += BANK(bi);
      data[bi] += data[ai];
    }
    offset <<= 1;
  }
  {
    uint idx = (ls << 1) - 1;
    idx += BANK(idx);
    if (partial) partial[gid] = data[idx];
    data[idx] = 0;
  }
  for (uint d = 1; d <= ls; d <<= 1) {
    offset >>= 1;
    for (uint lid = 0; lid < d; ++lid) {
      uint ai = offset * ((lid << 1) + 1) - 1;
      uint bi = offset * ((lid << 1) + 2) - 1;
      ai += BANK(ai);
      bi += BANK(bi);
      uint t = data[ai];
      data[ai] = data[bi];
      data[bi] += t;
    }
  }
  for (uint lid = 0; lid < ls; ++lid) {
    if (gOffset + lid < size) input[gOffset + lid] = data[lid + BANK(lid)];
    if (gOffset + lid + ls < size) input[gOffset + lid + ls] = data[lid + ls + BANK(lid + ls)];
  }
}

static uint next_pow2(uint n) {  // PrefixSum.cpp:61-71
  n--;
  n |= n >> 1;
  n |= n >> 2;
  n |= n >> 4;
  n |= n >> 8;
  n |= n >> 16;
  n++;
  return n;
}

static void recursive_scan(uint* input, uint size, uint wg) {  // PrefixSum.cpp:73-140
  uint nGroups = (uint)std::max(1.0f, std::ceil(((float)size) / (wg << 1)));
  if (nGroups == 1) {
    uint localSize = (uint)std::max(1.0f, std::ceil(((float)size) / 2));
    localSize = next_pow2(localSize);
    blelloch_wg(input, size, nullptr, 0, localSize, std::max(wg, localSize));
    return;
  }
  std::vector<uint> partial(nGroups, 0u);
  for (uint gid = 0; gid < nGroups; ++gid) blelloch_wg(input, size, partial.data(), gid, wg, wg);
  recursive_scan(partial.data(), nGroups, wg);
  for (uint gid = 0; gid < nGroups; ++gid) {  // prefixSumUniformAdd (:223-248)
    uint gOffset = gid * (wg << 1);
    uint add = partial[gid];
    for (uint lid = 0; lid < wg; ++lid) {
      if (gOffset + lid < size) input[gOffset + lid] += add;
      if (gOffset + lid + wg < size) input[gOffset + lid + wg] += add;
    }
  }
}

void oracle_prefix_sum_blelloch(uint32_t* data, uint32_t n, uint32_t wg) {
  if (n == 0 || wg == 0) return;
  recursive_scan(data, n, wg);
}

void oracle_math_eval(int fn, const float* a, const float* b, float* out, uint64_t n) {
  for (uint64_t i = 0; i < n; ++i) {
    switch (fn) {
      case 0: out[i] = trax::atan2_(a[i], b[i]); break;
      case 1: out[i] = trax::acos_(a[i]); break;
      case 2: out[i] = trax::atan_(a[i]); break;
      case 3: out[i] = trax::asinh_(a[i]); break;
      case 4: out[i] = trax::log_(a[i]); break;
      case 5: out[i] = trax::div_(a[i], b[i]); break;
      case 6: out[i] = trax::sqrt_(a[i]); break;
      case 7: out[i] = trax::floor_(a[i]); break;
      case 8: {  // the integer result's bits
        const uint32_t u = trax::f2u_sat(a[i]);
        memcpy(&out[i], &u, 4);
        break;
      }
      case 9: {
        const int32_t v = trax::f2i_sat(a[i]);
        memcpy(&out[i], &v, 4);
        break;
      }
      default: out[i] = 0.0f;
    }
  }
}

float oracle_min_radius_curvature(float min_pt) { return min_radius_curvature(min_pt); }

// The dphi cut of transverse segment pairs (u, v): filterCount's atan2
// evaluation (TripletThetaPhiFilter.h:118-128, as in filter_one) and the
// kernels' cross/dot decision trax::dphi_decide, for the tests that check
// the decision never disagrees with the evaluation.
void oracle_dphi_check(uint64_t n, const float* ux, const float* uy, const float* vx, const float* vy,
                       const float* cut, int32_t* exact, int32_t* decided) {
  for (uint64_t i = 0; i < n; ++i) {
    float delta = atan2_(vy[i], vx[i]) - atan2_(uy[i], ux[i]);
    delta += (delta > M_PI_F) ? -2 * M_PI_F : (delta < -M_PI_F) ? 2 * M_PI_F : 0;
    exact[i] = fabs_(delta) <= cut[i] ? 1 : 0;
    float lo, hi;
    trax::dphi_tan_bounds(cut[i], lo, hi);
    decided[i] = trax::dphi_decide(lo, hi, ux[i], uy[i], vx[i], vy[i]);
  }
}

}  // extern "C"
