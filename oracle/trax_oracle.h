// trax_oracle.h -- C interface of the CPU oracle (test infrastructure only).
//
// The oracle is a literal single-threaded (per event group) restatement of the
// reference's OpenCL kernels for the triplet-seeding path.  It exists to check
// the CUDA path; nothing in the product links or calls it.
#pragma once

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_input {
  // hits, sorted by event then layer (HitCollection.cpp:120-163 order)
  uint32_t n_hits;
  const float* x;
  const float* y;
  const float* z;
  const uint32_t* layer;   // 1-based detector layer
  const uint32_t* det_id;
  const uint32_t* hit_id;  // simulated track id (the reference's HitId column)
  const uint32_t* event;   // event number, 0..n_events-1
  uint32_t n_events;
  uint32_t n_layers;                // layers 1..n_layers are present in the supplements
  const uint32_t* event_offsets;    // [n_events] first hit of each event
  const uint32_t* layer_hits;       // [n_events * n_layers]
  const uint32_t* layer_offsets;    // [n_events * n_layers] first hit of the layer within its event
  // grid
  uint32_t n_z;
  uint32_t n_phi;
  // layer triplets, the 12 columns of TripletConfiguration.h:33
  uint32_t n_lt;
  const uint32_t* lt_layer1;
  const uint32_t* lt_layer2;
  const uint32_t* lt_layer3;
  const float* lt_dtheta_cut;
  const float* lt_sigma_z;
  const float* lt_dphi_cut;
  const float* lt_sigma_phi;
  const float* lt_tip_cut;
  const uint32_t* lt_pair_spread_z;
  const float* lt_z0;
  const uint32_t* lt_pair_spread_phi;
  const uint32_t* lt_n_candidates;
  float min_pt;
  // geometry supplement, indexed by layer - 1
  const float* min_r;
  const float* max_r;
  float d_eta_cut;
  // execution
  uint32_t n_threads;       // work-items per (event, layer pair) in pair generation; 0 = one per outer hit
  uint32_t event_grouping;  // events per group; 0 = all events in one group
  uint32_t n_workers;       // host threads used over event groups (0 or 1 = serial); with one
                            // group at a time, the threads work inside each group
  // connectivity: 0 the reference's linear scan of the follower segment;
  // 1 the same result through an index of the triplets by (first, second)
  // hit (for events of hundreds of thousands of triplets); 2 no linking
  // (connectivity, circle fit and CA skipped)
  uint32_t links_mode;
} oracle_input;

typedef struct oracle_result oracle_result;

// Runs the whole chain.  Returns 0 on success, a negative code on invalid input.
int oracle_run(const oracle_input* in, oracle_result** out);

// Connectivity, circle fit and CA on given triplets over a hit collection
// used as is (one event group).  Triplets must be grouped by (event, layer
// triplet) in ascending order, layer triplet p starting on layer p+1.
typedef struct oracle_link_input {
  uint32_t n_hits;
  const float* x;
  const float* y;
  const float* z;
  const uint32_t* layer;
  const uint32_t* event;
  uint32_t n_events;
  uint32_t n_lt;
  uint32_t n_triplets;
  const uint32_t* h1;
  const uint32_t* h2;
  const uint32_t* h3;
  float d_eta_cut;
} oracle_link_input;
int oracle_link(const oracle_link_input* in, oracle_result** out);
// CellularAutomaton::run alone on given links and pt (n_triplets values).
int oracle_ca(uint32_t n_triplets, const uint32_t* basis, const uint32_t* follower, uint32_t n_links,
              const float* pt, oracle_result** out);
void oracle_free(oracle_result* r);
const char* oracle_last_error(void);

uint32_t oracle_n_groups(const oracle_result* r);
// Number of uint32/float elements of array `name` of group `g` (-1 if unknown).
int64_t oracle_size(const oracle_result* r, uint32_t g, const char* name);
// Copies array `name` of group `g` into dst (4-byte elements).  Returns 0 on success.
int oracle_copy(const oracle_result* r, uint32_t g, const char* name, void* dst);

// Literal restatement of PrefixSum.h:58-248 / PrefixSum.cpp:47-140 (recursive
// Blelloch scan with 16-bank padding) over `n` elements with work-group size `wg`.
void oracle_prefix_sum_blelloch(uint32_t* data, uint32_t n, uint32_t wg);

// Element-wise evaluation of the shared math (trax_math.h):
// fn 0 atan2(a, b), 1 acos(a), 2 atan(a), 3 asinh(a), 4 log(a).
void oracle_math_eval(int fn, const float* a, const float* b, float* out, uint64_t n);
void oracle_dphi_check(uint64_t n, const float* ux, const float* uy, const float* vx, const float* vy,
                       const float* cut, int32_t* exact, int32_t* decided);

// minRadiusCurvature(minPt) of TripletConfiguration.cpp:36-43 with IDEAL_BZ.
float oracle_min_radius_curvature(float min_pt);

#ifdef __cplusplus
}
#endif
