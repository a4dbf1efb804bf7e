// host_events.cpp -- event files and physics bookkeeping on the host.
//
// Event files are PEventContainer messages (the reference's
// src/datastructures/serialize/Event.proto): read here with a small
// protocol-buffers wire-format decoder of our own (varints, 32-bit and
// length-delimited fields; no libprotobuf).  The loader restates
// HitCollection::addEvent (HitCollection.cpp:21-180): hits of simulated
// tracks above the minimum pT, "findable" tracks (hits on every layer used
// by the layer triplets) and the layer bucketing of the hit collection.
//
// The physics bookkeeping restates PhysicsRecord::fillData / merge / csvDump
// (PhysicsRecord.cpp:86-404: triplet efficiency, fake and clone rates per
// event and layer triplet, merged into means and deviations) and the track
// evaluation of TripletBuilder.cpp:840-1066 (track extraction from the CA
// output, clone removal, real/fake split, efficiency).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <list>
#include <map>
#include <memory>
#include <set>
#include <string>
#include <vector>

#include "trax/trax.h"
#include "trax_events.h"

struct trax_event_set;

namespace {

// ------------------------------------------------------------ wire format
struct PHit {
  float x = 0, y = 0, z = 0;
  int32_t detectorType = 0;
  uint64_t layer = 0, detectorId = 0, hitId = 0, simTrackID = 0;
  float simTrackPt = 0;
};

struct PEvent {
  uint64_t runNumber = 0, lumiSection = 0, eventNumber = 0;
  std::vector<PHit> hits;
};

class Reader {
 public:
  Reader(const uint8_t* p, size_t n) : p_(p), end_(p + n) {}
  bool done() const { return p_ >= end_; }
  bool varint(uint64_t& v) {
    v = 0;
    for (int shift = 0; shift < 64; shift += 7) {
      if (p_ >= end_) return false;
      const uint8_t b = *p_++;
      v |= (uint64_t)(b & 0x7f) << shift;
      if (!(b & 0x80)) return true;
    }
    return false;
  }
  bool fixed32(uint32_t& v) {
    if (end_ - p_ < 4) return false;
    v = (uint32_t)p_[0] | ((uint32_t)p_[1] << 8) | ((uint32_t)p_[2] << 16) | ((uint32_t)p_[3] << 24);
    p_ += 4;
    return true;
  }
  bool bytes(const uint8_t*& q, size_t& n) {
    uint64_t len;
    if (!varint(len) || (uint64_t)(end_ - p_) < len) return false;
    q = p_;
    n = (size_t)len;
    p_ += len;
    return true;
  }
  // skip a field of the given wire type
  bool skip(uint32_t wt) {
    uint64_t v;
    uint32_t f;
    const uint8_t* q;
    size_t n;
    switch (wt) {
      case 0: return varint(v);
      case 1:
        if (end_ - p_ < 8) return false;
        p_ += 8;
        return true;
      case 2: return bytes(q, n);
      case 5: return fixed32(f);
      default: return false;
    }
  }

 private:
  const uint8_t* p_;
  const uint8_t* end_;
};

float as_float(uint32_t b) {
  float f;
  std::memcpy(&f, &b, 4);
  return f;
}

bool parse_point(const uint8_t* p, size_t n, PHit& h) {
  Reader r(p, n);
  while (!r.done()) {
    uint64_t key;
    if (!r.varint(key)) return false;
    const uint32_t field = (uint32_t)(key >> 3), wt = (uint32_t)(key & 7);
    uint32_t v;
    if (wt == 5 && field >= 1 && field <= 3) {
      if (!r.fixed32(v)) return false;
      (field == 1 ? h.x : field == 2 ? h.y : h.z) = as_float(v);
    } else if (!r.skip(wt)) {
      return false;
    }
  }
  return true;
}

bool parse_hit(const uint8_t* p, size_t n, PHit& h) {
  Reader r(p, n);
  while (!r.done()) {
    uint64_t key;
    if (!r.varint(key)) return false;
    const uint32_t field = (uint32_t)(key >> 3), wt = (uint32_t)(key & 7);
    if (field == 1 && wt == 2) {
      const uint8_t* q;
      size_t m;
      if (!r.bytes(q, m) || !parse_point(q, m, h)) return false;
    } else if (wt == 0 && field >= 2 && field <= 6) {
      uint64_t v;
      if (!r.varint(v)) return false;
      switch (field) {
        case 2: h.detectorType = (int32_t)(int64_t)v; break;  // enum: negative values are 10-byte varints
        case 3: h.layer = v; break;
        case 4: h.detectorId = v; break;
        case 5: h.hitId = v; break;
        case 6: h.simTrackID = v; break;
      }
    } else if (field == 7 && wt == 5) {
      uint32_t v;
      if (!r.fixed32(v)) return false;
      h.simTrackPt = as_float(v);
    } else if (!r.skip(wt)) {
      return false;
    }
  }
  return true;
}

bool parse_event(const uint8_t* p, size_t n, PEvent& e) {
  Reader r(p, n);
  while (!r.done()) {
    uint64_t key;
    if (!r.varint(key)) return false;
    const uint32_t field = (uint32_t)(key >> 3), wt = (uint32_t)(key & 7);
    if (wt == 0 && field >= 1 && field <= 3) {
      uint64_t v;
      if (!r.varint(v)) return false;
      (field == 1 ? e.runNumber : field == 2 ? e.lumiSection : e.eventNumber) = v;
    } else if (field == 4 && wt == 2) {
      const uint8_t* q;
      size_t m;
      PHit h;
      if (!r.bytes(q, m) || !parse_hit(q, m, h)) return false;
      e.hits.push_back(h);
    } else if (!r.skip(wt)) {
      return false;
    }
  }
  return true;
}

// ------------------------------------------------------------ addEvent
struct Loaded {
  std::vector<float> x, y, z;
  std::vector<uint32_t> layer, det, hid, evt;
  std::vector<uint32_t> eventOffsets, layerHits, layerOffsets;  // layerOffsets relative to the event
  std::vector<uint32_t> findableId, findableEvent;
  uint32_t nLayers = 0;
};

// HitCollection::addEvent (HitCollection.cpp:21-180) for one event, as a
// walk: place(layer, hit) for every hit the reference pushes into its layer
// bucket, in push order (layers 1 .. maxLayer only: the others are never
// read out), and found(track id) for every findable track.  The hit
// collection is the buckets read out layer by layer, each in push order.
template <class Place, class Found>
void add_event_walk(const PEvent& ev, const std::set<uint32_t>& usedLayers, uint32_t maxLayer, float minPt,
                    int numTracks, bool onlyTracks, Place place, Found found) {
  // hits of each simulated track above the minimum pT (:45-57)
  std::map<uint64_t, std::vector<const PHit*>> allTracks;
  for (const PHit& h : ev.hits) {
    if (onlyTracks && h.simTrackID == 0) continue;
    if (h.simTrackPt < minPt) continue;
    allTracks[h.simTrackID].push_back(&h);
  }
  // layer order inside a track; equal layers keep their file order (:59-65)
  for (auto& t : allTracks)
    std::stable_sort(t.second.begin(), t.second.end(),
                     [](const PHit* a, const PHit* b) { return a->layer < b->layer; });
  std::vector<const std::vector<const PHit*>*> findable;
  std::vector<uint64_t> findableIds;
  int foundTracks = 0;
  for (auto it = allTracks.begin(); it != allTracks.end() && foundTracks != numTracks; ++it) {
    if (onlyTracks && it->first == 0) continue;
    // a track is findable when it has a hit on every used layer (:80-93);
    // layers above the highest used one are not counted
    std::vector<bool> cov(maxLayer, false);
    for (const PHit* h : it->second)
      if (h->layer >= 1 && h->layer <= maxLayer) cov[h->layer - 1] = true;
    bool missing = false;
    for (uint32_t l : usedLayers)
      if (!cov[l - 1]) missing = true;
    if (it->second[0]->simTrackPt < minPt) continue;
    if (!missing) {
      findable.push_back(&it->second);
      findableIds.push_back(it->first);
      ++foundTracks;
    } else if (!onlyTracks) {
      for (const PHit* h : it->second)
        if (h->layer >= 1 && h->layer <= maxLayer) place((uint32_t)h->layer, h);
    }
  }
  // findable tracks' hits after the others, layer by layer (:112-120)
  for (const auto* t : findable)
    for (const PHit* h : *t)
      if (h->layer >= 1 && h->layer <= maxLayer) place((uint32_t)h->layer, h);
  for (uint64_t id : findableIds) found(id);
}

// The loader's output for one event: the buckets read out layer by layer
// (:122-149).
void add_event(const PEvent& ev, uint32_t evtInGroup, const std::set<uint32_t>& usedLayers, uint32_t maxLayer,
               float minPt, int numTracks, bool onlyTracks, Loaded& out) {
  std::vector<std::vector<const PHit*>> layers(maxLayer + 1);
  add_event_walk(
      ev, usedLayers, maxLayer, minPt, numTracks, onlyTracks,
      [&](uint32_t l, const PHit* h) { layers[l].push_back(h); },
      [&](uint64_t id) {
        out.findableId.push_back((uint32_t)id);
        out.findableEvent.push_back(evtInGroup);
      });
  uint32_t inEvent = 0;
  for (uint32_t l = 1; l <= maxLayer; ++l) {
    const uint32_t n = (uint32_t)layers[l].size();
    out.layerHits.push_back(n);
    out.layerOffsets.push_back(inEvent);
    inEvent += n;
  }
  out.eventOffsets.push_back((uint32_t)out.x.size());
  for (uint32_t l = 1; l <= maxLayer; ++l)
    for (const PHit* h : layers[l]) {
      out.x.push_back(h->x);
      out.y.push_back(h->y);
      out.z.push_back(h->z);
      out.layer.push_back((uint32_t)h->layer);
      out.det.push_back((uint32_t)h->detectorId);
      out.hid.push_back((uint32_t)h->simTrackID);  // the HitId column carries the simulated track id
      out.evt.push_back(evtInGroup);
    }
}

template <class T>
void copy_out(const std::vector<T>& v, T* dst) {
  if (dst && !v.empty()) std::memcpy(dst, v.data(), v.size() * sizeof(T));
}

// ------------------------------------------------------------ physics
struct Stat {
  double mean = 0, m2 = 0;
};

// PhysicsRecord::merge (PhysicsRecord.cpp:338-358): n += c.n, then the
// running mean and the sum of squared deviations
void merge_stat(Stat& a, const Stat& c, double nNew, double cn) {
  const double delta = c.mean - a.mean;
  a.mean += cn * delta / std::max(nNew, 1.0);
  a.m2 += cn * delta * (c.mean - a.mean) + c.m2;
}

struct Record {
  uint32_t lt = 0;
  double n = 0;
  Stat eff, fake, clone;
  void merge(const Record& c) {
    n += c.n;
    merge_stat(eff, c.eff, n, c.n);
    merge_stat(fake, c.fake, n, c.n);
    merge_stat(clone, c.clone, n, c.n);
  }
  double dev(const Stat& s) const { return n > 1 ? std::sqrt(s.m2 / std::max(n - 1, 1.0)) : 0.0; }
};

}  // namespace

struct trax_event_set {
  std::vector<PEvent> events;
};

namespace {

// the layers the layer triplets use, and the highest of them
int used_layers(const trax_layer_triplet* lt, int n_lt, std::set<uint32_t>& used, uint32_t& maxLayer) {
  maxLayer = 0;
  for (int p = 0; p < n_lt; ++p) {
    for (uint32_t l : {lt[p].layer1, lt[p].layer2, lt[p].layer3}) {
      if (l == 0) return TRAX_ERR_ARG;
      used.insert(l);
    }
    maxLayer = std::max(maxLayer, lt[p].layer3);
  }
  return TRAX_OK;
}

}  // namespace

namespace trax {

int classify_events(const trax_event_set* s, uint64_t first, uint64_t count, const trax_layer_triplet* lt, int n_lt,
                    float min_pt, int num_tracks, int only_tracks, RawEvents& out) {
  if (!s || !lt || n_lt <= 0 || first > s->events.size()) return TRAX_ERR_ARG;
  const uint64_t last = std::min<uint64_t>(s->events.size(), first + count);
  std::set<uint32_t> used;
  uint32_t maxLayer = 0;
  if (used_layers(lt, n_lt, used, maxLayer) != TRAX_OK) return TRAX_ERR_ARG;
  out = RawEvents();
  out.nLayers = maxLayer;
  for (uint64_t e = first; e < last; ++e) {
    const PEvent& ev = s->events[e];
    if (ev.hits.size() >= EVENT_HITS_MAX) return TRAX_ERR_ARG;
    const size_t base = out.x.size();
    if (base + ev.hits.size() > 0xffffffffull) return TRAX_ERR_ARG;
    out.rawOffsets.push_back((uint32_t)base);
    for (const PHit& h : ev.hits) {
      out.x.push_back(h.x);
      out.y.push_back(h.y);
      out.z.push_back(h.z);
      out.layer.push_back((uint32_t)h.layer);
      out.det.push_back((uint32_t)h.detectorId);
      out.tid.push_back((uint32_t)h.simTrackID);
      out.key.push_back(EVENT_HIT_DROPPED);
    }
    const uint32_t evtInGroup = (uint32_t)(e - first);
    std::vector<uint32_t> perLayer(maxLayer + 1, 0);
    uint32_t pushed = 0;
    add_event_walk(
        ev, used, maxLayer, min_pt, num_tracks, only_tracks != 0,
        [&](uint32_t l, const PHit* h) {
          const uint32_t local = (uint32_t)(h - ev.hits.data());
          out.key[base + local] = event_hit_key(l, pushed++, local);
          ++perLayer[l];
        },
        [&](uint64_t id) {
          out.findableId.push_back((uint32_t)id);
          out.findableEvent.push_back(evtInGroup);
        });
    out.eventOffsets.push_back((uint32_t)out.nHits);
    uint32_t inEvent = 0;
    for (uint32_t l = 1; l <= maxLayer; ++l) {
      out.layerHits.push_back(perLayer[l]);
      out.layerOffsets.push_back(inEvent);
      inEvent += perLayer[l];
      out.maxLayerHits = std::max(out.maxLayerHits, perLayer[l]);
    }
    out.nHits += pushed;
  }
  out.rawOffsets.push_back((uint32_t)out.x.size());
  return out.nHits > 0xffffffffull ? TRAX_ERR_ARG : TRAX_OK;
}

void physics_records(uint32_t n_events, uint32_t n_lt, const uint32_t* offsets, const uint32_t* found,
                     const uint32_t* fakes, const uint32_t* clones, const uint32_t* truthSize,
                     trax_physics_record* out) {
  std::vector<Record> perLT(n_lt);
  std::vector<bool> seen(n_lt, false);
  for (uint32_t e = 0; e < n_events; ++e)
    for (uint32_t p = 0; p < n_lt; ++p) {
      const size_t seg = (size_t)e * n_lt + p;
      const uint32_t a = offsets[seg], b = offsets[seg + 1];
      const double nFound = b > a ? (double)(b - a) : 0.0;
      Record r;
      r.lt = p;
      r.n = 1;
      r.eff.mean = (double)found[seg] / std::max<double>((double)truthSize[e], 1.0);
      r.fake.mean = (double)fakes[seg] / std::max(nFound, 1.0);
      r.clone.mean = (double)clones[seg] / std::max(nFound, 1.0);
      // PhysicsRecords::addRecord (:360-371): merge by layer triplet
      if (!seen[p]) {
        perLT[p] = r;
        seen[p] = true;
      } else {
        perLT[p].merge(r);
      }
    }
  // csvDump (:380-404): every layer triplet, then the total over them
  for (uint32_t p = 0; p < n_lt; ++p) {
    const Record& r = perLT[p];
    out[p] = trax_physics_record{p, (uint64_t)r.n, r.eff.mean, r.dev(r.eff), r.fake.mean, r.dev(r.fake),
                                 r.clone.mean, r.dev(r.clone)};
  }
  Record total = perLT[0];
  for (uint32_t p = 1; p < n_lt; ++p) total.merge(perLT[p]);
  out[n_lt] = trax_physics_record{n_lt + 1, (uint64_t)total.n, total.eff.mean, total.dev(total.eff),
                                  total.fake.mean, total.dev(total.fake), total.clone.mean,
                                  total.dev(total.clone)};
}

}  // namespace trax

extern "C" {

int trax_events_read(const char* path, trax_event_set** out, uint64_t* n_events) {
  if (!path || !out) return TRAX_ERR_ARG;
  *out = nullptr;
  std::ifstream f(path, std::ios::binary);
  if (!f) return TRAX_ERR_ARG;
  std::vector<uint8_t> buf((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  std::unique_ptr<trax_event_set> s(new trax_event_set);
  Reader r(buf.data(), buf.size());
  while (!r.done()) {
    uint64_t key;
    if (!r.varint(key)) return TRAX_ERR_ARG;
    const uint32_t field = (uint32_t)(key >> 3), wt = (uint32_t)(key & 7);
    if (field == 1 && wt == 2) {
      const uint8_t* q;
      size_t m;
      PEvent e;
      if (!r.bytes(q, m) || !parse_event(q, m, e)) return TRAX_ERR_ARG;
      s->events.push_back(std::move(e));
    } else if (!r.skip(wt)) {
      return TRAX_ERR_ARG;
    }
  }
  if (n_events) *n_events = s->events.size();
  *out = s.release();
  return TRAX_OK;
}

void trax_events_free(trax_event_set* s) { delete s; }

int trax_events_raw(const trax_event_set* s, uint64_t e, uint64_t* n_hits, float* xyz, uint64_t* layer,
                    uint64_t* det_id, uint64_t* hit_id, uint64_t* sim_track_id, float* sim_pt, int32_t* det_type,
                    uint64_t* run_lumi_event) {
  if (!s || e >= s->events.size()) return TRAX_ERR_ARG;
  const PEvent& ev = s->events[e];
  if (n_hits) *n_hits = ev.hits.size();
  if (run_lumi_event) {
    run_lumi_event[0] = ev.runNumber;
    run_lumi_event[1] = ev.lumiSection;
    run_lumi_event[2] = ev.eventNumber;
  }
  for (size_t i = 0; i < ev.hits.size(); ++i) {
    const PHit& h = ev.hits[i];
    if (xyz) {
      xyz[3 * i] = h.x;
      xyz[3 * i + 1] = h.y;
      xyz[3 * i + 2] = h.z;
    }
    if (layer) layer[i] = h.layer;
    if (det_id) det_id[i] = h.detectorId;
    if (hit_id) hit_id[i] = h.hitId;
    if (sim_track_id) sim_track_id[i] = h.simTrackID;
    if (sim_pt) sim_pt[i] = h.simTrackPt;
    if (det_type) det_type[i] = h.detectorType;
  }
  return TRAX_OK;
}

int trax_events_load(const trax_event_set* s, uint64_t first, uint64_t count, const trax_layer_triplet* lt, int n_lt,
                     float min_pt, int num_tracks, int only_tracks, trax_loaded_sizes* sizes, float* x, float* y,
                     float* z, uint32_t* layer, uint32_t* det_id, uint32_t* hit_id, uint32_t* event,
                     uint32_t* event_offsets, uint32_t* layer_hits, uint32_t* layer_offsets, uint32_t* findable_id,
                     uint32_t* findable_event) {
  if (!s || !lt || n_lt <= 0 || !sizes) return TRAX_ERR_ARG;
  if (first > s->events.size()) return TRAX_ERR_ARG;
  const uint64_t last = std::min<uint64_t>(s->events.size(), first + count);
  std::set<uint32_t> used;
  uint32_t maxLayer = 0;
  if (used_layers(lt, n_lt, used, maxLayer) != TRAX_OK) return TRAX_ERR_ARG;
  Loaded out;
  out.nLayers = maxLayer;
  for (uint64_t e = first; e < last; ++e)
    add_event(s->events[e], (uint32_t)(e - first), used, maxLayer, min_pt, num_tracks, only_tracks != 0, out);
  sizes->n_hits = out.x.size();
  sizes->n_events = last - first;
  sizes->n_layers = maxLayer;
  sizes->n_findable = out.findableId.size();
  copy_out(out.x, x);
  copy_out(out.y, y);
  copy_out(out.z, z);
  copy_out(out.layer, layer);
  copy_out(out.det, det_id);
  copy_out(out.hid, hit_id);
  copy_out(out.evt, event);
  copy_out(out.eventOffsets, event_offsets);
  copy_out(out.layerHits, layer_hits);
  copy_out(out.layerOffsets, layer_offsets);
  copy_out(out.findableId, findable_id);
  copy_out(out.findableEvent, findable_event);
  return TRAX_OK;
}

int trax_geometry_from_files(const char* radius_dictionary, const char* detector_radius, uint32_t n_layers,
                             float* min_r, float* max_r) {
  if (!radius_dictionary || !detector_radius || !min_r || !max_r || n_layers == 0) return TRAX_ERR_ARG;
  // dictionary: "entry,radius" rows; detectors: "detId,entry,layer" rows
  std::ifstream fd(radius_dictionary), fg(detector_radius);
  if (!fd || !fg) return TRAX_ERR_ARG;
  std::map<uint32_t, float> dict;
  std::string line;
  while (std::getline(fd, line)) {
    unsigned entry;
    float radius;
    if (std::sscanf(line.c_str(), "%u,%f", &entry, &radius) == 2) dict[entry] = radius;
  }
  for (uint32_t l = 0; l < n_layers; ++l) {
    min_r[l] = 10000.0f;  // layers without modules keep (10000, 0), like TripletBuilder.cpp:157-160
    max_r[l] = 0.0f;
  }
  while (std::getline(fg, line)) {
    unsigned det, entry, layer;
    if (std::sscanf(line.c_str(), "%u,%u,%u", &det, &entry, &layer) != 3) continue;
    const auto it = dict.find(entry);
    if (it == dict.end() || layer < 1 || layer > n_layers) continue;
    min_r[layer - 1] = std::min(min_r[layer - 1], it->second);
    max_r[layer - 1] = std::max(max_r[layer - 1], it->second);
  }
  return TRAX_OK;
}

int trax_physics_triplets(const uint32_t* h1, const uint32_t* h2, const uint32_t* h3, const uint32_t* offsets,
                          uint32_t n_events, uint32_t n_lt, const uint32_t* hit_track_id, const uint32_t* findable_id,
                          const uint32_t* findable_event, uint64_t n_findable, trax_physics_record* out) {
  if (!offsets || !hit_track_id || !out || n_lt == 0) return TRAX_ERR_ARG;
  std::vector<std::set<uint32_t>> truth(n_events);
  for (uint64_t k = 0; k < n_findable; ++k)
    if (findable_event[k] < n_events) truth[findable_event[k]].insert(findable_id[k]);
  const size_t S = (size_t)n_events * n_lt;
  std::vector<uint32_t> found(S), fakes(S), clones(S), truthSize(n_events);
  for (uint32_t e = 0; e < n_events; ++e) {
    truthSize[e] = (uint32_t)truth[e].size();
    for (uint32_t p = 0; p < n_lt; ++p) {
      // PhysicsRecord::fillData (PhysicsRecord.cpp:86-313) for (e, p)
      const size_t seg = (size_t)e * n_lt + p;
      std::set<uint32_t> seen;
      for (uint32_t t = offsets[seg]; t < offsets[seg + 1]; ++t) {
        const uint32_t i1 = hit_track_id[h1[t]], i2 = hit_track_id[h2[t]], i3 = hit_track_id[h3[t]];
        if (i1 == i2 && i1 == i3) {
          if (truth[e].count(i1)) {
            if (!seen.insert(i1).second) ++clones[seg];
          }
        } else {
          ++fakes[seg];
        }
      }
      found[seg] = (uint32_t)seen.size();
    }
  }
  trax::physics_records(n_events, n_lt, offsets, found.data(), fakes.data(), clones.data(), truthSize.data(), out);
  return TRAX_OK;
}

int trax_physics_tracks(const uint32_t* tracks, const uint32_t* track_offsets, uint64_t n_triplets,
                        const uint32_t* h1, const uint32_t* h2, const uint32_t* h3, const uint32_t* hit_track_id,
                        uint64_t total_tracks, trax_track_metrics* out) {
  if (!track_offsets || !hit_track_id || !out) return TRAX_ERR_ARG;
  typedef std::pair<uint32_t, std::shared_ptr<std::vector<uint32_t>>> Track;
  // extractTracks (TripletBuilder.cpp:951-985): chains of three or more
  // triplets, hits from the outermost triplet inwards
  std::list<Track> raw;
  uint32_t id = 0;
  for (uint64_t i = 0; i < n_triplets; ++i) {
    const uint32_t off = track_offsets[i], len = track_offsets[i + 1] - off;
    if (len < 3) continue;
    std::shared_ptr<std::vector<uint32_t>> t(new std::vector<uint32_t>());
    for (uint32_t j = 0; j < len; ++j) {
      const uint32_t trip = tracks[off + (len - 1 - j)];
      if (t->empty()) {
        t->push_back(h1[trip]);
        t->push_back(h2[trip]);
      }
      t->push_back(h3[trip]);
    }
    raw.push_back(std::make_pair(id++, t));
  }
  // cloneRemoval (:882-907) with the shared-hit comparator (:846-866)
  auto same = [](const Track& base, const Track& other) {
    const Track& longer = base.second->size() < other.second->size() ? other : base;
    const Track& shorter = base.second->size() >= other.second->size() ? other : base;
    uint32_t shared = 0;
    for (uint32_t hit : *longer.second)
      if (std::find(shorter.second->begin(), shorter.second->end(), hit) != shorter.second->end()) ++shared;
    return shared / (float)shorter.second->size() >= 0.19f;
  };
  std::list<Track> filtered;
  for (const Track& t : raw) {
    auto found = std::find_if(filtered.begin(), filtered.end(), [&](const Track& o) { return same(t, o); });
    if (found == filtered.end()) {
      filtered.push_back(t);
    } else if (found->second->size() == t.second->size()) {
      filtered.push_back(t);
    } else if (found->second->size() < t.second->size()) {
      filtered.erase(found);
      filtered.push_back(t);
    }
  }
  // splitRealFakeTracks, findUniqueRealTracks (:868-880, :909-949, :987-996)
  uint64_t real = 0, fakes = 0;
  std::set<uint32_t> unique;
  for (const Track& t : filtered) {
    const uint32_t first = hit_track_id[t.second->front()];
    bool valid = true;
    for (uint32_t hit : *t.second)
      if (hit_track_id[hit] != first) valid = false;
    if (valid) {
      ++real;
      unique.insert(first);
    } else {
      ++fakes;
    }
  }
  out->total = raw.size();
  out->filtered = filtered.size();
  out->valid = real;
  out->valid_unique = unique.size();
  out->fakes = fakes;
  const double nf = (double)filtered.size();
  out->fake_rate = nf > 0 ? fakes / nf : 0.0;
  out->clone_rate = nf > 0 ? (double)(real - unique.size()) / nf : 0.0;
  out->efficiency = total_tracks ? (double)unique.size() / (double)total_tracks : 0.0;
  return TRAX_OK;
}

}  // extern "C"
