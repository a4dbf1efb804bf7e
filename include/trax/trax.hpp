// trax.hpp -- C++ host classes of the triplet-seeding path over the C ABI.
//
// The reference's host side (JuantAldea/trax, C++ over OpenCL) is a set of
// containers -- TripletConfigurations, GridConfig / Grid, GeometrySupplement,
// HitCollection, EventSupplement, LayerSupplement, Pairing,
// TrackletCollection -- and algorithm classes with one run() each:
// GridBuilder, PairGeneratorBeamspot, TripletThetaPhiPredictor,
// TripletThetaPhiFilter, TripletConnectivityTight, TrackletCircleFitter,
// CellularAutomaton and PrefixSum.  This header keeps those names, the
// configuration each class carries and the argument meaning of every run(),
// and forwards to libtrax_gb300.so (include/trax/trax.h).  It is header-only
// and needs no CUDA headers.
//
// Differences from the reference, all of them in what the caller owns:
//   * clever::context becomes trax::Context (one CUDA stream and the device
//     buffers); intermediate results stay on the device inside it, so the
//     algorithm objects of one chain must share a Context, and each run()
//     consumes the previous stage's result held there;
//   * run() returns host containers (std::unique_ptr, as the reference's raw
//     owning pointers) filled from the device;
//   * the nThreads / printInfo arguments are accepted for call compatibility;
//     the work-group shape is the library's (trax_set_block_sizes,
//     trax_autotune);
//   * errors throw trax::Error carrying the C status code.
#ifndef TRAX_HPP_
#define TRAX_HPP_

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "trax.h"

namespace trax {

class Error : public std::runtime_error {
 public:
  Error(int code, const std::string& msg) : std::runtime_error(msg), code_(code) {}
  int code() const { return code_; }

 private:
  int code_;
};

// clever::context (TripletBuilder.cpp:66-129): owns the library context.
class Context {
 public:
  explicit Context(int device = 0) {
    const int rc = trax_create(&ctx_, device);
    if (rc != TRAX_OK) throw Error(rc, "trax_create failed (no usable CUDA device?)");
  }
  ~Context() { trax_destroy(ctx_); }
  Context(const Context&) = delete;
  Context& operator=(const Context&) = delete;
  trax_ctx* get() const { return ctx_; }
  void check(int rc) const {
    if (rc != TRAX_OK) throw Error(rc, trax_last_error(ctx_));
  }
  // generation of the device-side chain state, bumped by every stage run
  uint64_t generation() const { return gen_; }
  uint64_t bump() { return ++gen_; }
  // events of the uploaded batch (set by GridBuilder::run)
  uint32_t nEvents = 0;

 private:
  trax_ctx* ctx_ = nullptr;
  uint64_t gen_ = 0;
};

// ------------------------------------------------------------ configuration
// One row of TripletConfigurations (TripletConfiguration.h:74-140).
class TripletConfiguration {
 public:
  explicit TripletConfiguration(const trax_layer_triplet& r) : r_(r) {}
  uint32_t layer1() const { return r_.layer1; }
  uint32_t layer2() const { return r_.layer2; }
  uint32_t layer3() const { return r_.layer3; }
  float dThetaCut() const { return r_.dtheta_cut; }
  float sigmaZ() const { return r_.sigma_z; }
  float dPhiCut() const { return r_.dphi_cut; }
  float sigmaPhi() const { return r_.sigma_phi; }
  float tipCut() const { return r_.tip_cut; }
  uint32_t pairSpreadZ() const { return r_.pair_spread_z; }
  float z0() const { return r_.z0; }
  uint32_t pairSpreadPhi() const { return r_.pair_spread_phi; }
  uint32_t nCandidates() const { return r_.n_candidates; }

 private:
  trax_layer_triplet r_;
};

// TripletConfigurations (TripletConfiguration.h:37-72, .cpp:36-107).
class TripletConfigurations {
 public:
  explicit TripletConfigurations(float minPt) : minPt_(minPt) {}

  void addWithValue(uint32_t layer1, uint32_t layer2, uint32_t layer3, float dThetaCut, float sigmaZ, float dPhiCut,
                    float sigmaPhi, float tipCut, uint32_t pairSpreadZ, float z0, uint32_t pairSpreadPhi,
                    uint32_t nCandidates) {
    trax_layer_triplet r;
    r.layer1 = layer1;
    r.layer2 = layer2;
    r.layer3 = layer3;
    r.dtheta_cut = dThetaCut;
    r.sigma_z = sigmaZ;
    r.dphi_cut = dPhiCut;
    r.sigma_phi = sigmaPhi;
    r.tip_cut = tipCut;
    r.pair_spread_z = pairSpreadZ;
    r.z0 = z0;
    r.pair_spread_phi = pairSpreadPhi;
    r.n_candidates = nCandidates;
    rows_.push_back(r);
  }

  size_t size() const { return rows_.size(); }
  TripletConfiguration operator[](size_t i) const { return TripletConfiguration(rows_.at(i)); }
  const std::vector<trax_layer_triplet>& rows() const { return rows_; }
  float minPt() const { return minPt_; }

  // minRadiusCurvature (TripletConfiguration.cpp:36-43): R = pT / (B q) in cm
  // with the reference's ideal field and constants
  float minRadiusCurvature() const { return minRadiusCurvature(minPt_); }
  static float minRadiusCurvature(float minPt) {
    // the double IDEAL_BZ goes through the float Bz parameter of
    // minRadiusCurvature(minPt, Bz) (TripletConfiguration.h:56-70)
    const double IDEAL_BZ = 3.8112, Q = 1.602177E-19, GEV_C = 5.344286E-19;
    const float Bz = (float)IDEAL_BZ;
    return (float)(minPt * GEV_C / (Bz * Q) * 1E2);
  }

  // loadTripletConfigurationFromFile (TripletConfiguration.cpp:70-107): the
  // <layerTriplets><layerTriplet>...</layerTriplet></layerTriplets> file of
  // configs/layerTriplets.xml; z0 is read as an unsigned integer like the
  // reference's (Q11).  Returns the highest layer used.
  uint32_t loadTripletConfigurationFromFile(const std::string& filename, int n = -1) {
    std::ifstream f(filename);
    if (!f) throw Error(TRAX_ERR_ARG, "cannot open " + filename);
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string text = ss.str();
    uint32_t maxLayer = 0;
    int added = 0;
    size_t at = 0;
    while (true) {
      const size_t a = text.find("<layerTriplet>", at);
      if (a == std::string::npos) break;
      const size_t b = text.find("</layerTriplet>", a);
      if (b == std::string::npos) throw Error(TRAX_ERR_ARG, "unterminated <layerTriplet> in " + filename);
      const std::string blk = text.substr(a, b - a);
      at = b + 1;
      if (n != -1 && added >= n) continue;
      const uint32_t l1 = to_uint(tag(blk, "layer1")), l2 = to_uint(tag(blk, "layer2")),
                     l3 = to_uint(tag(blk, "layer3"));
      addWithValue(l1, l2, l3, to_float(tag(blk, "dThetaCut")), to_float(tag(blk, "sigmaZ")),
                   to_float(tag(blk, "dPhiCut")), to_float(tag(blk, "sigmaPhi")), to_float(tag(blk, "tipCut")),
                   to_uint(tag(blk, "pairSpreadZ")), (float)to_uint(tag(blk, "z0")),
                   to_uint(tag(blk, "pairSpreadPhi")), to_uint(tag(blk, "nCandidates")));
      ++added;
      if (l3 > maxLayer) maxLayer = l3;
    }
    return maxLayer;
  }

 private:
  static std::string tag(const std::string& blk, const char* name) {
    const std::string open = std::string("<") + name + ">", close = std::string("</") + name + ">";
    const size_t a = blk.find(open);
    const size_t b = a == std::string::npos ? a : blk.find(close, a);
    if (a == std::string::npos || b == std::string::npos)
      throw Error(TRAX_ERR_ARG, std::string("layer triplet without <") + name + ">");
    std::string v = blk.substr(a + open.size(), b - a - open.size());
    const size_t s = v.find_first_not_of(" \t\r\n"), e = v.find_last_not_of(" \t\r\n");
    return s == std::string::npos ? std::string() : v.substr(s, e - s + 1);
  }
  static uint32_t to_uint(const std::string& v) {
    if (v.empty() || v.find_first_not_of("0123456789") != std::string::npos)
      throw Error(TRAX_ERR_ARG, "expected an unsigned integer, got '" + v + "'");
    return (uint32_t)std::stoul(v);
  }
  static float to_float(const std::string& v) {
    size_t used = 0;
    const float f = std::stof(v, &used);
    if (used != v.size()) throw Error(TRAX_ERR_ARG, "expected a number, got '" + v + "'");
    return f;
  }

  float minPt_;
  std::vector<trax_layer_triplet> rows_;
};

// GridConfig (Grid.h:5-39): z in [-300, 300] cm, phi in [-pi, pi].
struct GridConfig {
  static constexpr float MIN_Z = -300.0f, MAX_Z = 300.0f;
  static constexpr float MIN_PHI = -3.14159265358979323846f, MAX_PHI = 3.14159265358979323846f;
  uint32_t nSectorsZ = 50, nSectorsPhi = 8;  // the reference's command-line defaults
  GridConfig() = default;
  GridConfig(uint32_t z, uint32_t phi) : nSectorsZ(z), nSectorsPhi(phi) {}
  float sectorSizeZ() const { return (MAX_Z - MIN_Z) / (float)nSectorsZ; }
  float sectorSizePhi() const { return (MAX_PHI - MIN_PHI) / (float)nSectorsPhi; }
};

// Grid (Grid.h:42-131): the configuration plus, after GridBuilder::run, the
// cell boundaries [events x layers x (nZ+1)(nPhi+1)].
struct Grid {
  GridConfig config;
  std::vector<uint32_t> boundaries;
  explicit Grid(const GridConfig& c) : config(c) {}
};

// GeometrySupplement (GeometrySupplement.h:21-81): min/max radius per layer.
class GeometrySupplement {
 public:
  void addEntry(uint32_t layer, float minRadius, float maxRadius) {
    if (layer == 0) throw Error(TRAX_ERR_ARG, "layers are 1-based");
    if (minR_.size() < layer) {
      minR_.resize(layer, 0.0f);
      maxR_.resize(layer, 0.0f);
    }
    minR_[layer - 1] = minRadius;
    maxR_[layer - 1] = maxRadius;
  }
  size_t size() const { return minR_.size(); }
  float minRadius(uint32_t layer) const { return minR_.at(layer - 1); }
  float maxRadius(uint32_t layer) const { return maxR_.at(layer - 1); }
  const std::vector<float>& minR() const { return minR_; }
  const std::vector<float>& maxR() const { return maxR_; }

 private:
  std::vector<float> minR_, maxR_;
};

// DetectorGeometry (DetectorGeometry.h:17-41) and Dictionary
// (Dictionary.h:16-38): the detector-id -> radius tables
// (configs/detectorRadius.dat, radiusDictionary.dat).  The reference passes
// both to its prediction kernels, which never read them
// (TripletThetaPhiPredictor.h:44-47, 54-55); they are kept for the call
// surface.
struct DetectorGeometry {
  std::vector<uint32_t> detectorId, detectorLayer;
  std::vector<uint8_t> radiusDict;  // index into Dictionary::radius
};
struct Dictionary {
  std::vector<float> radius;
};

// HitCollection (HitCollection.h:23-62): the seven hit columns, sorted by
// event then layer.  GridBuilder::run reorders it into grid order, like the
// reference's download of the permuted hits (GridBuilder.cpp:151).
class HitCollection {
 public:
  std::vector<float> x, y, z;
  std::vector<uint32_t> layer, detId, hitId, event;

  size_t size() const { return x.size(); }
  void addWithValue(float px, float py, float pz, uint32_t lay, uint32_t det, uint32_t hid, uint32_t evt) {
    x.push_back(px);
    y.push_back(py);
    z.push_back(pz);
    layer.push_back(lay);
    detId.push_back(det);
    hitId.push_back(hid);
    event.push_back(evt);
  }
  trax_hits_soa soa() const {
    return trax_hits_soa{x.data(), y.data(), z.data(), layer.data(), detId.data(), hitId.data(), event.data()};
  }
  // input index of every grid-ordered hit, after GridBuilder::run
  std::vector<uint32_t> inputIndex;
};

// EventSupplement (EventSupplement.h:8-32) and LayerSupplement
// (LayerSupplement.h:7-31): first hit of each event; hits and offset (from
// the event's first hit) of each (event, layer).
struct EventSupplement {
  std::vector<uint32_t> offset;
  uint32_t nEvents() const { return (uint32_t)offset.size(); }
};
struct LayerSupplement {
  uint32_t nLayers = 0;
  std::vector<uint32_t> nHits, offset;  // [nEvents * nLayers]
};

// The supplements of a collection sorted by event then layer.
inline void buildSupplements(const HitCollection& hits, uint32_t nEvents, uint32_t nLayers, EventSupplement& es,
                             LayerSupplement& ls) {
  es.offset.assign(nEvents, 0);
  ls.nLayers = nLayers;
  ls.nHits.assign((size_t)nEvents * nLayers, 0);
  ls.offset.assign((size_t)nEvents * nLayers, 0);
  for (size_t i = 0; i < hits.size(); ++i) {
    const uint32_t e = hits.event[i], l = hits.layer[i];
    if (e >= nEvents || l < 1 || l > nLayers) throw Error(TRAX_ERR_ARG, "hit outside the event/layer range");
    if (i > 0 && (e < hits.event[i - 1] || (e == hits.event[i - 1] && l < hits.layer[i - 1])))
      throw Error(TRAX_ERR_ARG, "hits must be sorted by event, then layer");
    ++ls.nHits[(size_t)e * nLayers + (l - 1)];
  }
  uint32_t run = 0;
  for (uint32_t e = 0; e < nEvents; ++e) {
    es.offset[e] = run;
    uint32_t inEvent = 0;
    for (uint32_t l = 0; l < nLayers; ++l) {
      ls.offset[(size_t)e * nLayers + l] = inEvent;
      inEvent += ls.nHits[(size_t)e * nLayers + l];
    }
    run += inEvent;
  }
}

// A PEventContainer file (the reference's Event.proto, PEventStore), read
// on the host.
class EventFile {
 public:
  explicit EventFile(const std::string& path) {
    const int rc = trax_events_read(path.c_str(), &set_, &n_);
    if (rc != TRAX_OK) throw Error(rc, "cannot read event file " + path);
  }
  ~EventFile() { trax_events_free(set_); }
  EventFile(const EventFile&) = delete;
  EventFile& operator=(const EventFile&) = delete;
  uint64_t size() const { return n_; }
  const trax_event_set* handle() const { return set_; }

 private:
  trax_event_set* set_ = nullptr;
  uint64_t n_ = 0;
};

// HitCollection::addEvent (HitCollection.cpp:21-180) for events [first,
// first + count) of a file, as the reference's loop over a PEventContainer
// calls it with evtInGroup = 0, 1, ...: the collection and the supplements
// are replaced by those events' hits; returns the findable (track id, event
// in the group) pairs, the reference's tTrackList per event.
inline std::vector<std::pair<uint32_t, uint32_t>> addEvents(const EventFile& file, uint64_t first, uint64_t count,
                                                            const TripletConfigurations& lts, int numTracks,
                                                            bool onlyTracks, HitCollection& hits,
                                                            EventSupplement& es, LayerSupplement& ls) {
  trax_loaded_sizes sz{};
  auto load = [&](float* x, float* y, float* z, uint32_t* layer, uint32_t* det, uint32_t* hid, uint32_t* evt,
                  uint32_t* eo, uint32_t* lh, uint32_t* lo, uint32_t* fid, uint32_t* fev) {
    const int rc = trax_events_load(file.handle(), first, count, lts.rows().data(), (int)lts.size(), lts.minPt(),
                                    numTracks, onlyTracks ? 1 : 0, &sz, x, y, z, layer, det, hid, evt, eo, lh, lo,
                                    fid, fev);
    if (rc != TRAX_OK) throw Error(rc, "trax_events_load failed");
  };
  load(nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
  hits.x.assign(sz.n_hits, 0.0f);
  hits.y.assign(sz.n_hits, 0.0f);
  hits.z.assign(sz.n_hits, 0.0f);
  hits.layer.assign(sz.n_hits, 0u);
  hits.detId.assign(sz.n_hits, 0u);
  hits.hitId.assign(sz.n_hits, 0u);
  hits.event.assign(sz.n_hits, 0u);
  es.offset.assign(sz.n_events, 0u);
  ls.nLayers = (uint32_t)sz.n_layers;
  ls.nHits.assign(sz.n_events * sz.n_layers, 0u);
  ls.offset.assign(sz.n_events * sz.n_layers, 0u);
  std::vector<uint32_t> fid(sz.n_findable), fev(sz.n_findable);
  load(hits.x.data(), hits.y.data(), hits.z.data(), hits.layer.data(), hits.detId.data(), hits.hitId.data(),
       hits.event.data(), es.offset.data(), ls.nHits.data(), ls.offset.data(), fid.data(), fev.data());
  std::vector<std::pair<uint32_t, uint32_t>> findable(sz.n_findable);
  for (size_t k = 0; k < findable.size(); ++k) findable[k] = {fid[k], fev[k]};
  return findable;
}

// Pairing (Pairings.h:9-59): (first, second) hit pairs and per-(event,
// layer triplet) offsets; also used for the predictor's (pair, third hit)
// candidates.
struct uint2_t {
  uint32_t x, y;
};
class Pairing {
 public:
  std::vector<uint2_t> pairing;
  std::vector<uint32_t> pairingOffsets;
  const std::vector<uint2_t>& getPairings() const { return pairing; }
  const std::vector<uint32_t>& getPairingOffsets() const { return pairingOffsets; }
  uint64_t generation = 0;  // chain state of the Context that produced it
};

// TrackletCollection (TrackletCollection.h:32-78).
class TrackletCollection {
 public:
  std::vector<uint32_t> hit1, hit2, hit3;
  std::vector<uint32_t> trackletOffsets;
  size_t size() const { return hit1.size(); }
  const std::vector<uint32_t>& getTrackletOffsets() const { return trackletOffsets; }
  // chain state of the Context that holds these triplets on the device (a
  // record of where the collection lives, updated by const run() methods too)
  mutable uint64_t generation = 0;
};

// ------------------------------------------------------------ algorithms
// KernelWrapper<T> (KernelWrapper.hpp:11-35): holds the context.
class KernelWrapper {
 public:
  explicit KernelWrapper(Context& c) : ctx(c) {}

 protected:
  Context& ctx;
};

// GridBuilder::run (GridBuilder.h:42, .cpp:6-161).  Uploads the hits, builds
// the grid and reorders `hits` into grid order.  Returns the number of hits.
class GridBuilder : public KernelWrapper {
 public:
  using KernelWrapper::KernelWrapper;
  uint64_t run(HitCollection& hits, uint32_t /*nThreads*/, const EventSupplement& es, const LayerSupplement& ls,
               Grid& grid, bool /*printInfo*/ = false) {
    const trax_hits_soa soa = hits.soa();
    ctx.check(trax_set_grid(ctx.get(), grid.config.nSectorsZ, grid.config.nSectorsPhi));
    ctx.check(trax_upload_hits(ctx.get(), &soa, (uint32_t)hits.size(), es.offset.data(), ls.nHits.data(),
                               ls.offset.data(), es.nEvents(), ls.nLayers));
    ctx.check(trax_grid_build(ctx.get()));
    ctx.nEvents = es.nEvents();
    ctx.bump();
    uint64_t cells = 0;
    ctx.check(trax_get_grid(ctx.get(), nullptr, &cells));
    grid.boundaries.resize(cells);
    ctx.check(trax_get_grid(ctx.get(), grid.boundaries.data(), &cells));
    std::vector<uint32_t> perm(hits.size());
    ctx.check(trax_get_hit_perm(ctx.get(), perm.data()));
    HitCollection sorted;
    for (uint32_t i : perm)
      sorted.addWithValue(hits.x[i], hits.y[i], hits.z[i], hits.layer[i], hits.detId[i], hits.hitId[i],
                          hits.event[i]);
    sorted.inputIndex = perm;
    hits = std::move(sorted);
    return hits.size();
  }
};

// PairGeneratorBeamspot::run (PairGeneratorBeamspot.h:40-41, .cpp:5-183).
class PairGeneratorBeamspot : public KernelWrapper {
 public:
  using KernelWrapper::KernelWrapper;
  std::unique_ptr<Pairing> run(HitCollection& /*hits*/, const GeometrySupplement& geom, uint32_t /*nThreads*/,
                               const TripletConfigurations& layerTriplets, const Grid& /*grid*/,
                               bool /*printInfo*/ = false) {
    ctx.check(trax_set_layer_triplets(ctx.get(), layerTriplets.rows().data(), (int)layerTriplets.size(),
                                      layerTriplets.minPt()));
    ctx.check(trax_set_geometry(ctx.get(), geom.minR().data(), geom.maxR().data(), (int)geom.size()));
    uint64_t n = 0;
    ctx.check(trax_pair_gen(ctx.get(), &n));
    std::unique_ptr<Pairing> p(new Pairing);
    p->pairing.resize(n);
    p->pairingOffsets.resize((size_t)ctx.nEvents * layerTriplets.size() + 1);
    ctx.check(trax_get_pairs(ctx.get(), reinterpret_cast<uint32_t*>(p->pairing.data()), p->pairingOffsets.data()));
    p->generation = ctx.bump();
    return p;
  }
};

namespace detail {
inline void expect_current(const Context& ctx, uint64_t gen, const char* what) {
  if (gen != ctx.generation())
    throw Error(TRAX_ERR_STATE, std::string(what) + " was not produced by the last run on this Context");
}
}  // namespace detail

// TripletThetaPhiPredictor::run (TripletThetaPhiPredictor.h:44-47, .cpp:10-168),
// with the reference's parameter list; the geometry tables are unused, as
// in the reference's kernels.
class TripletThetaPhiPredictor : public KernelWrapper {
 public:
  using KernelWrapper::KernelWrapper;
  std::unique_ptr<Pairing> run(HitCollection& /*hits*/, const DetectorGeometry& /*geom*/,
                               const GeometrySupplement& /*geomSupplement*/, const Dictionary& /*dict*/,
                               int /*nThreads*/, const TripletConfigurations& layerTriplets, const Grid& /*grid*/,
                               const Pairing& pairs, bool /*printInfo*/ = false) {
    detail::expect_current(ctx, pairs.generation, "the pairing");
    uint64_t n = 0;
    ctx.check(trax_triplet_predict(ctx.get(), &n));
    std::unique_ptr<Pairing> p(new Pairing);
    p->pairing.resize(n);
    p->pairingOffsets.resize(pairs.pairingOffsets.size());
    ctx.check(trax_get_candidates(ctx.get(), reinterpret_cast<uint32_t*>(p->pairing.data()),
                                  p->pairingOffsets.data()));
    (void)layerTriplets;
    p->generation = ctx.bump();
    return p;
  }
};

// TripletThetaPhiFilter::run (TripletThetaPhiFilter.h:46-48, .cpp:10-206).
class TripletThetaPhiFilter : public KernelWrapper {
 public:
  using KernelWrapper::KernelWrapper;
  std::unique_ptr<TrackletCollection> run(HitCollection& /*hits*/, const Grid& /*grid*/, const Pairing& pairs,
                                          const Pairing& candidates, int /*nThreads*/,
                                          const TripletConfigurations& /*layerTriplets*/,
                                          bool /*printInfo*/ = false) {
    detail::expect_current(ctx, candidates.generation, "the candidate pairing");
    uint64_t n = 0;
    ctx.check(trax_triplet_filter(ctx.get(), &n));
    std::unique_ptr<TrackletCollection> t(new TrackletCollection);
    t->hit1.resize(n);
    t->hit2.resize(n);
    t->hit3.resize(n);
    t->trackletOffsets.resize(pairs.pairingOffsets.size());
    ctx.check(trax_get_triplets(ctx.get(), t->hit1.data(), t->hit2.data(), t->hit3.data(),
                                t->trackletOffsets.data()));
    t->generation = ctx.bump();
    return t;
  }
};

// TripletConnectivityTight::run (TripletConnectivityTight.h:42-44, .cpp:5-475).
// Returns (basis, follower, connectable, non-connectable); all null when no
// link is found, like the reference (.cpp:127-129).  Tracklets that this
// Context did not produce (any TrackletCollection over `hits` in input
// order) are uploaded first.
struct ConnectivityResult {
  std::unique_ptr<std::vector<uint32_t>> basis, follower, connectable, nonConnectable;
};
class TripletConnectivityTight : public KernelWrapper {
 public:
  using KernelWrapper::KernelWrapper;
  ConnectivityResult run(const HitCollection& /*hits*/, TrackletCollection& tracklets,
                         const TripletConfigurations& /*layerTriplets*/, float dEtaCut, uint32_t /*nThreads*/,
                         bool /*printInfo*/ = false) {
    if (tracklets.generation != ctx.generation()) {
      ctx.check(trax_set_tracklets(ctx.get(), tracklets.hit1.data(), tracklets.hit2.data(), tracklets.hit3.data(),
                                   tracklets.size()));
    }
    uint64_t nLinks = 0;
    ctx.check(trax_connectivity(ctx.get(), dEtaCut, &nLinks));
    tracklets.generation = ctx.bump();
    ConnectivityResult r;
    if (nLinks == 0) return r;
    trax_batch_stats s;
    ctx.check(trax_get_stats(ctx.get(), &s));
    r.basis.reset(new std::vector<uint32_t>(s.n_links));
    r.follower.reset(new std::vector<uint32_t>(s.n_links));
    r.connectable.reset(new std::vector<uint32_t>(s.n_connectable));
    r.nonConnectable.reset(new std::vector<uint32_t>(s.n_non_connectable));
    ctx.check(trax_get_links(ctx.get(), r.basis->data(), r.follower->data(), r.connectable->data(),
                             r.nonConnectable->data()));
    return r;
  }
};

// TrackletCircleFitter::run (TrackletCircleFitter.h:25-29, .cpp:3-49): the
// circle radius of every triplet listed in validIdx, 0 for the others.
// Tracklets this Context did not produce (any TrackletCollection over `hits`
// in input order) are uploaded first; validIdx may be any list of their
// indices.
class TrackletCircleFitter : public KernelWrapper {
 public:
  using KernelWrapper::KernelWrapper;
  std::unique_ptr<std::vector<float>> run(const HitCollection& /*hits*/, const TrackletCollection& tracklets,
                                          const std::vector<uint32_t>& validIdx, uint32_t /*nThreads*/,
                                          bool /*printInfo*/ = false) {
    if (tracklets.generation != ctx.generation()) {
      ctx.check(trax_set_tracklets(ctx.get(), tracklets.hit1.data(), tracklets.hit2.data(), tracklets.hit3.data(),
                                   tracklets.size()));
      tracklets.generation = ctx.bump();
    }
    ctx.check(trax_circle_fit_on(ctx.get(), validIdx.data(), validIdx.size()));
    std::unique_ptr<std::vector<float>> pt(new std::vector<float>(tracklets.size()));
    ctx.check(trax_get_pt(ctx.get(), pt->data()));
    return pt;
  }
};

// CellularAutomaton::run (CellularAutomaton.h:43-49, .cpp:7-465) on the
// caller's links basis[i] -> followers[i] and one pt per triplet: the track
// collection and its per-triplet offsets.  Any acyclic link set is accepted.
// The connectable list is taken for the call surface; the reference's CA
// reads it only for its debug printout.  The CA's states are kept for
// states().
class CellularAutomaton : public KernelWrapper {
 public:
  using KernelWrapper::KernelWrapper;
  std::tuple<std::unique_ptr<std::vector<uint32_t>>, std::unique_ptr<std::vector<uint32_t>>> run(
      const std::vector<uint32_t>& basis, const std::vector<uint32_t>& followers, const std::vector<float>& pt,
      const std::vector<uint32_t>& /*connectable*/, uint32_t /*nThreads*/, bool /*printInfo*/ = false) {
    if (basis.size() != followers.size()) throw Error(TRAX_ERR_ARG, "basis and followers differ in length");
    uint64_t n = 0;
    ctx.check(trax_cellular_automaton_on(ctx.get(), basis.data(), followers.data(), basis.size(), pt.data(),
                                         pt.size(), &n));
    ctx.bump();
    std::unique_ptr<std::vector<uint32_t>> tracks(new std::vector<uint32_t>(n));
    std::unique_ptr<std::vector<uint32_t>> offsets(new std::vector<uint32_t>(pt.size() + 1));
    states_.assign(pt.size(), 0);
    ctx.check(trax_get_tracks(ctx.get(), states_.data(), tracks->data(), offsets->data()));
    return std::make_tuple(std::move(tracks), std::move(offsets));
  }
  const std::vector<uint32_t>& states() const { return states_; }

 private:
  std::vector<uint32_t> states_;
};

// PrefixSum::run (PrefixSum.h:43-44): exclusive uint32 scan in place, the
// total in the last element (the caller appends it).
class PrefixSum : public KernelWrapper {
 public:
  using KernelWrapper::KernelWrapper;
  void run(std::vector<uint32_t>& data, uint32_t /*nThreads*/ = 0) {
    ctx.check(trax_prefix_sum(ctx.get(), data.data(), data.size()));
  }
};

}  // namespace trax

#endif  // TRAX_HPP_
