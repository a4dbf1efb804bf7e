// trax_events.h -- event-file hits classified on the host for the device
// bucketing step of trax_events_upload, and the physics records shared by
// the host and device counting.
//
// HitCollection::addEvent (HitCollection.cpp:21-180) decides per hit whether
// the loader keeps it (its track's pT, findability, the track limit) and in
// which layer bucket and position it lands; those decisions walk each
// event's tracks in id order through ordered maps and stay on the host.
// Each kept hit gets a key (layer, push position, index in its event) whose
// ascending order is the order the reference reads the buckets out in; the
// device sorts every event's keys and gathers the hit columns into that
// order (k_events.cu).
#pragma once

#include <cstdint>
#include <vector>

#include "trax/trax.h"

namespace trax {

// hits per event the keys can index (24 bits of push position and of index)
constexpr uint32_t EVENT_HITS_MAX = 1u << 24;
// the key of a hit the loader drops: sorts after every kept hit
constexpr uint64_t EVENT_HIT_DROPPED = ~0ull;

inline uint64_t event_hit_key(uint32_t layer, uint32_t pushed, uint32_t local) {
  return ((uint64_t)layer << 48) | ((uint64_t)pushed << 24) | local;
}

struct RawEvents {
  std::vector<float> x, y, z;             // every hit of the events, in file order
  std::vector<uint32_t> layer, det, tid;  // tid: the simulated track id (the hit_id column)
  std::vector<uint64_t> key;              // event_hit_key, or EVENT_HIT_DROPPED
  std::vector<uint32_t> rawOffsets;       // [E+1] first hit of each event in the arrays above
  // the loaded collection: [E] first kept hit of each event, [E*L] kept hits
  // per (event, layer) and their offsets inside the event
  std::vector<uint32_t> eventOffsets, layerHits, layerOffsets;
  std::vector<uint32_t> findableId, findableEvent;
  uint32_t nLayers = 0, maxLayerHits = 0;
  uint64_t nHits = 0;  // hits the loader keeps
};

// the classification of events [first, first + count): TRAX_OK or
// TRAX_ERR_ARG (bad arguments, an event of EVENT_HITS_MAX hits or more)
int classify_events(const trax_event_set* events, uint64_t first, uint64_t count, const trax_layer_triplet* lt,
                    int n_lt, float min_pt, int num_tracks, int only_tracks, RawEvents& out);

// PhysicsRecord's means and deviations (PhysicsRecord.cpp:86-404) from the
// counts of every (event, layer triplet) segment: distinct findable tracks
// found, fake triplets, clone triplets; truthSize: findable tracks per event.
// out [n_lt + 1]: every layer triplet, then the total.
void physics_records(uint32_t n_events, uint32_t n_lt, const uint32_t* offsets, const uint32_t* found,
                     const uint32_t* fakes, const uint32_t* clones, const uint32_t* truthSize,
                     trax_physics_record* out);

}  // namespace trax
