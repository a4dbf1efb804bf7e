/* trax.h -- C ABI of the sm_103a triplet-seeding library (libtrax_gb300.so).
 *
 * Plain C types only: the caller passes host pointers and sizes, the library
 * owns its device memory, stream and events.  Every call returns a status
 * code (TRAX_OK == 0); trax_last_error() describes the last failure.
 *
 * Each entry point replaces one operator of the reference's triplet-seeding
 * path (JuantAldea/trax, OpenCL).  The comment above each declaration names
 * the reference interface it stands in for (file:line inside that project).
 * In the reference those operators are C++ classes whose run() methods take
 * clever:: OpenCL containers; here the containers live inside the context
 * and run() becomes one call.
 *
 * Index conventions follow the reference: hit indices in results are
 * positions in the grid-ordered hit collection (what GridBuilder::run leaves
 * in the HitCollection, GridBuilder.cpp:151); trax_get_hit_perm maps them back
 * to the caller's input order.
 */
#ifndef TRAX_H_
#define TRAX_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define TRAX_OK 0
#define TRAX_ERR_CUDA 1          /* a CUDA runtime call failed */
#define TRAX_ERR_ARG 2           /* invalid argument or input */
#define TRAX_ERR_CAPACITY 3      /* a result does not fit the configured capacity */
#define TRAX_ERR_TIMEOUT 4       /* a bounded device-side wait ran out */
#define TRAX_ERR_DEVICE_ASSERT 5 /* a device-side bounds check fired */
#define TRAX_ERR_STATE 6         /* call out of order (e.g. a stage before its input exists) */

typedef struct trax_ctx trax_ctx;

/* One row of the layer-triplet table: the 12 columns of
 * TripletConfiguration.h:9-33 (configs/layerTriplets.xml). */
typedef struct trax_layer_triplet {
  uint32_t layer1, layer2, layer3;
  float dtheta_cut;
  float sigma_z;
  float dphi_cut;
  float sigma_phi;
  float tip_cut;
  uint32_t pair_spread_z;
  float z0;
  uint32_t pair_spread_phi;
  uint32_t n_candidates;
} trax_layer_triplet;

/* The 7 SoA columns of HitCollection (HitCollection.h:23). */
typedef struct trax_hits_soa {
  const float* x;
  const float* y;
  const float* z;
  const uint32_t* layer;  /* 1-based detector layer */
  const uint32_t* det_id;
  const uint32_t* hit_id; /* simulated track id */
  const uint32_t* event;  /* event number inside the batch */
} trax_hits_soa;

/* Options of the batched call. */
typedef struct trax_batch_opts {
  int use_graph;        /* capture the chain in a CUDA graph and replay it */
  int run_linking;      /* 1: connectivity, circle fit and CA; 0: stop after the filter */
  float d_eta_cut;      /* TripletConnectivityTight dEtaCut (TripletBuilder.cpp:793: 0.0256) */
} trax_batch_opts;

/* Sizes produced by the last chain run. */
typedef struct trax_batch_stats {
  uint64_t n_hits;
  uint64_t n_pairs;
  uint64_t n_candidates;
  uint64_t n_triplets;
  uint64_t n_links;
  uint64_t n_connectable;
  uint64_t n_non_connectable;
  uint64_t n_track_entries;
  uint64_t n_pair_sentinels;      /* pair slots the reference leaves unwritten */
  uint64_t n_candidate_sentinels; /* candidate slots the reference leaves unwritten */
  uint64_t kernel_launches;       /* kernels launched by the last run */
  double device_ms;               /* device time of the last run (CUDA events) */
  uint64_t graph_captures;        /* calibrate-and-capture passes of the last trax_seed_batch: 0 replayed the
                                     graph, 1 built it, 2 rebuilt it after a capacity overflow */
} trax_batch_stats;

/* ---------------------------------------------------------------- context
 * Replaces clever::context creation (TripletBuilder.cpp:66-129).
 * One context per host thread; it owns a CUDA stream and its buffers. */
int trax_create(trax_ctx** ctx, int device);
void trax_destroy(trax_ctx* ctx);
const char* trax_last_error(const trax_ctx* ctx);
const char* trax_version(void);

/* Page-locked host memory for the arrays passed to trax_upload_hits and the
 * trax_get_* calls: copies from and to it run at the link's DMA rate, copies
 * from ordinary (pageable) memory go through a staging copy.  No counterpart
 * in the reference (clever's buffers are OpenCL host-visible allocations).
 * NULL on failure. */
void* trax_host_alloc(size_t bytes);
void trax_host_free(void* ptr);

/* ---------------------------------------------------------- configuration
 * TripletConfigurations + minRadiusCurvature (TripletConfiguration.h:39-72,
 * TripletConfiguration.cpp:36-43).  Row p must have layer1 == p + 1 (the
 * reference derives the layer-triplet index from the first hit's layer,
 * TripletThetaPhiPredictor.h:88). */
int trax_set_layer_triplets(trax_ctx* ctx, const trax_layer_triplet* lt, int n, float min_pt);

/* GeometrySupplement (GeometrySupplement.h:21-43): min/max radius of layers 1..n. */
int trax_set_geometry(trax_ctx* ctx, const float* min_r, const float* max_r, int n_layers);

/* GridConfig (Grid.h:5-39): z range fixed to [-300, 300] cm, phi to [-pi, pi]. */
int trax_set_grid(trax_ctx* ctx, uint32_t n_z, uint32_t n_phi);

/* HitCollection + EventSupplement + LayerSupplement upload
 * (TripletBuilder.cpp:296-307; HitCollection.cpp:120-163 layout).
 * Hits are sorted by event, then layer; layer_hits/layer_offsets are
 * [n_events * n_layers], offsets relative to the event's first hit. */
int trax_upload_hits(trax_ctx* ctx, const trax_hits_soa* hits, uint32_t n_hits,
                     const uint32_t* event_offsets, const uint32_t* layer_hits,
                     const uint32_t* layer_offsets, uint32_t n_events, uint32_t n_layers);

/* ------------------------------------------------------ stage by stage
 * GridBuilder::run (GridBuilder.h:42, GridBuilder.cpp:6-161): per-(event,
 * layer) z/phi grid and the grid-ordered hit collection. */
int trax_grid_build(trax_ctx* ctx);

/* PairGeneratorBeamspot::run (PairGeneratorBeamspot.h:40-41, .cpp:5-183). */
int trax_pair_gen(trax_ctx* ctx, uint64_t* n_pairs);

/* TripletThetaPhiPredictor::run (TripletThetaPhiPredictor.h:44-47, .cpp:10-168). */
int trax_triplet_predict(trax_ctx* ctx, uint64_t* n_candidates);

/* TripletThetaPhiFilter::run (TripletThetaPhiFilter.h:46-48, .cpp:10-206). */
int trax_triplet_filter(trax_ctx* ctx, uint64_t* n_triplets);

/* TrackletCollection input for the linking stages: the reference's
 * TripletConnectivityTight::run takes any HitCollection and TrackletCollection
 * (TripletConnectivityTight.h:42-44).  The uploaded hits are used as the hit
 * collection in their input order (no grid build) and h1/h2/h3 index them;
 * triplets must be grouped by (event, layer triplet), ascending.  Afterwards
 * trax_connectivity, trax_circle_fit and trax_cellular_automaton can run. */
int trax_set_tracklets(trax_ctx* ctx, const uint32_t* h1, const uint32_t* h2, const uint32_t* h3, uint64_t n);

/* TripletConnectivityTight::run (TripletConnectivityTight.h:42-44, .cpp:5-475). */
int trax_connectivity(trax_ctx* ctx, float d_eta_cut, uint64_t* n_links);

/* TrackletCircleFitter::run (TrackletCircleFitter.h:25-29, .cpp:3-49) on the
 * connectable list of the last trax_connectivity. */
int trax_circle_fit(trax_ctx* ctx);

/* TrackletCircleFitter::run with the caller's validIdx list
 * (TrackletCircleFitter.h:25-29: `validTrackletsIndices`): the circle radius
 * of each listed triplet of the context's current triplet set (from the
 * filter or trax_set_tracklets), 0 for the others; read it with
 * trax_get_pt.  Indices must be below the number of triplets. */
int trax_circle_fit_on(trax_ctx* ctx, const uint32_t* valid_idx, uint64_t n_valid);
/* The pt of the current triplet set (n_triplets floats), after
 * trax_circle_fit, trax_circle_fit_on or trax_seed_batch with linking. */
int trax_get_pt(trax_ctx* ctx, float* pt);

/* CellularAutomaton::run (CellularAutomaton.h:43-49, .cpp:7-465) on the
 * links and pt of the last trax_connectivity / trax_circle_fit. */
int trax_cellular_automaton(trax_ctx* ctx, uint64_t* n_track_entries);

/* CellularAutomaton::run on the caller's inputs (CellularAutomaton.h:43-49:
 * tripletsBasis, tripletsFollowers, tripletsPt): n_links links
 * basis[i] -> follower[i] between triplets 0 .. n_triplets-1 and one pt per
 * triplet.  Any link set is accepted: the forward phase runs the reference's
 * iteration (CellularAutomaton.cpp:37-98) until no cell lives, so links need
 * not go from one layer triplet to the next; a set with a cycle never
 * settles in the reference and returns TRAX_ERR_ARG here.  Ties of the best
 * basis go to the lowest basis index.  When the context holds triplets,
 * n_triplets must equal their number; otherwise the context takes
 * n_triplets as its triplet count for this run.  Results: trax_get_tracks
 * (states, the track collection and its per-triplet offsets). */
int trax_cellular_automaton_on(trax_ctx* ctx, const uint32_t* basis, const uint32_t* follower, uint64_t n_links,
                               const float* pt, uint64_t n_triplets, uint64_t* n_track_entries);

/* PrefixSum::run (PrefixSum.h:43-44, PrefixSum.cpp:8-36): exclusive uint32
 * scan of `n` elements of the host array `data` in place (round trip through
 * the device; single-pass decoupled-lookback scan). */
int trax_prefix_sum(trax_ctx* ctx, uint32_t* data, uint64_t n);

/* Allocation-free exclusive uint32 scan of n elements from d_in to d_out
 * (device pointers owned by the caller; in place allowed), on the caller's
 * `stream` (a cudaStream_t, NULL for the legacy default stream) of the
 * current device.  No counterpart in the reference: it exists for callers
 * that must not allocate device memory -- code running inside another
 * framework's memory pool or under an allocator that forbids new device
 * allocations (a cudaMalloc there can fail, stall or break a budget), and
 * code that has to work when device memory is already exhausted.  It calls
 * no cudaMalloc, no cudaFree and no allocating library routine, and needs no
 * trax_ctx.
 *   - Its scratch (tile ticket, error word, one look-back status word per
 *     4096-element tile) is a fixed array inside the library, present on
 *     every GPU that loads it until the process exits; n is therefore limited
 *     to TRAX_NOALLOC_SCAN_MAX elements, larger n returns TRAX_ERR_ARG.
 *   - Every call looks up the array's device address in the current context
 *     (cudaGetSymbolAddress), so a device reset or another current context
 *     is picked up.  The first call in a context also loads the library's
 *     device code there.
 *   - No call can be captured into a CUDA graph: each one synchronises
 *     `stream` and reads the error word back (below), which a capturing
 *     stream refuses, invalidating the capture.
 *   - All calls share the array and each call clears what it uses; calls
 *     whose work overlaps on the GPU (other streams, other host threads) race.
 *   - Before returning, the call copies the scan's error word to the host and
 *     synchronises `stream`, so that a timed-out look-back wait is reported
 *     (TRAX_ERR_TIMEOUT).
 * A message is written to err_msg (err_len bytes, may be NULL) on failure. */
#define TRAX_NOALLOC_SCAN_MAX (16ull * 1024ull * 1024ull)
int trax_prefix_sum_noalloc(const uint32_t* d_in, uint32_t* d_out, uint64_t n, void* stream, char* err_msg,
                            size_t err_len);

/* Bounded device waits.  No counterpart in the reference, whose recursive
 * scan (PrefixSum.cpp:73-140) has no waits between work-groups.  Every
 * single-pass scan's look-back wait gives up after a number of polls
 * (default 2^22, each at least 64 ns), records the timeout and finishes; the
 * call then returns TRAX_ERR_TIMEOUT.
 * trax_set_wait_limit: polls per wait for the scans this context launches
 *   afterwards (0 restores the default).  A CUDA graph captured before keeps
 *   its old limit until trax_seed_batch recaptures, which it does when the
 *   setting changes.
 * trax_debug_skip_publish: a host-set fault for testing that path without a
 *   GPU fault: look-back tile `tile` (4096 elements each) of every later scan
 *   of this context publishes nothing, so the waits of the tiles after it run
 *   out and the call returns TRAX_ERR_TIMEOUT.  0xffffffff turns it off.
 * trax_noalloc_set_wait: the same two settings for trax_prefix_sum_noalloc,
 *   process-wide (it has no context). */
int trax_set_wait_limit(trax_ctx* ctx, uint32_t polls);
int trax_debug_skip_publish(trax_ctx* ctx, uint32_t tile);
int trax_noalloc_set_wait(uint32_t polls, uint32_t skip_tile);

/* The library's single-precision math evaluated on the device `device`:
 * out[i] = fn(a[i], b[i]) for n elements of host arrays, synchronously.  No
 * counterpart in the reference; the kernels evaluate OpenCL's atan2, acos,
 * atan and the float->integer conversions (e.g. PairGeneratorBeamspot.h:111-162,
 * TripletThetaPhiFilter.h:118-128) with these definitions, so that their
 * results are the same on every device.  fn: 0 atan2(a, b), 1 acos, 2 atan,
 * 3 asinh, 4 log, 5 a / b, 6 sqrt, 7 floor, 8 saturating float->uint32 and
 * 9 float->int32 (truncation, NaN -> 0; out holds the integer's bits);
 * 10-14 CUDA's own atan2f, acosf, atanf, asinhf, logf for comparison.
 * b may be null unless fn is 0, 5 or 10. */
int trax_math_eval(int device, int fn, const float* a, const float* b, float* out, uint64_t n);

/* Threads per block of the pair, prediction and filter kernels (multiples of
 * 32 in [32, 256]; defaults 128, 128, 256).  No counterpart in the reference,
 * whose work-group sizes are fixed per kernel in the run() methods (e.g.
 * PairGeneratorBeamspot.cpp:5-183, TripletThetaPhiPredictor.cpp:10-168). */
int trax_set_block_sizes(trax_ctx* ctx, uint32_t pair_threads, uint32_t predict_threads, uint32_t filter_threads);
/* out5 = n_z, n_phi, pair threads, prediction threads, filter threads. */
int trax_get_launch_config(trax_ctx* ctx, uint32_t* out5);
/* Pairs per thread of the prediction's count pass: 1, 2 or 4 (default 1).
 * With k > 1 a thread computes the windows of k pairs and walks their
 * candidate hits in one loop, which evens out the work of a warp's threads;
 * the results do not change.  No counterpart in the reference, where one
 * work-item takes one pair (TripletThetaPhiPredictor.cpp:22-41); trax_autotune
 * tunes it after the block sizes. */
int trax_set_pairs_per_thread(trax_ctx* ctx, uint32_t k);
int trax_get_pairs_per_thread(trax_ctx* ctx, uint32_t* k);
/* Candidates the prediction's count pass captures per pair for its store
 * pass: 4, 8, 16 or 32, or 0 for automatic (the default): after each
 * calibration of trax_seed_batch the library takes 4, 8, 16 or 32 from the
 * batch's mean candidates per pair (up to 1, 2.5, 6, above).  A pair with
 * more candidates than slots is walked again by the store pass; more slots
 * cost the pairs with few candidates more scattered writes and reads.  The
 * results do not change.  The reference's predictStore walks every pair
 * again (TripletThetaPhiPredictor.h:232-447).  get returns the number in
 * effect; trax_autotune tunes it after the pairs per thread. */
int trax_set_candidate_slots(trax_ctx* ctx, uint32_t k);
int trax_get_candidate_slots(trax_ctx* ctx, uint32_t* k);
/* Rows of the prediction count's fine z grid per row of the grid: 0 (none,
 * the default), 2, 4, 8 or 16.  With f > 0 the grid stage also sorts every
 * layer's grid-ordered hits by a z grid f times finer (f rows inside each
 * z row, the same phi columns), and the count pass walks only the fine rows
 * its window reaches; it finds the same hits and captures the same
 * candidates, so the results do not change.  It pays off where a grid row
 * is much longer than the windows (many hits walked per pair fail the z
 * test); it costs a second grid (4 bytes per fine cell per (event, layer))
 * and its build.  Pairs per thread do not apply to it.  No counterpart in
 * the reference, whose predictCount walks the grid's rows
 * (TripletThetaPhiPredictor.h:187-219); trax_autotune tunes it after the
 * candidate slots. */
int trax_set_fine_rows(trax_ctx* ctx, uint32_t f);
int trax_get_fine_rows(trax_ctx* ctx, uint32_t* f);

/* ------------------------------------------------------------- batched
 * The whole chain (buildTriplets, TripletBuilder.cpp:312-467) for all
 * uploaded events in one pass of batched launches, optionally replayed from a
 * CUDA graph. */
int trax_seed_batch(trax_ctx* ctx, const trax_batch_opts* opts, trax_batch_stats* stats);

/* Autotuner of the batched chain's launch shape.  No counterpart in the
 * reference, where the grid size is a command-line parameter
 * (grid.nSectorsZ / grid.nSectorsPhi, TripletBuilder.cpp:631-634) and work-group sizes
 * are fixed.  It times CUDA-graph replays of trax_seed_batch on the uploaded
 * hits for grid sizes n_z x n_phi (cells per layer within the shared-memory
 * grid build), then for the three kernels' block sizes, one coordinate at
 * a time, then for the prediction count's pairs per thread, candidate slots
 * and fine z grid, and leaves the fastest shape set on the context.  The result is
 * cached in the JSON file `cache_path` (may be NULL: no cache), keyed by a
 * hash of the workload (batch shape, layer triplets, geometry, minimum pT,
 * whether linking runs) and the GPU's SM count; a cached shape is applied
 * without timing.  The chosen grid changes the grid-ordered hit indices of
 * the results, not the triplets in input-hit terms. */
typedef struct trax_tune_opts {
  int search_grid; /* 1: search n_z x n_phi; 0: keep the context's grid */
  int run_linking; /* time the chain with linking (1) or up to the filter (0) */
  int replays;     /* timed graph replays per shape (best one counts); 0 -> 3 */
} trax_tune_opts;
typedef struct trax_tune_result {
  uint32_t n_z, n_phi;
  uint32_t pair_threads, predict_threads, filter_threads;
  uint32_t from_cache;       /* 1: taken from the cache file */
  uint32_t shapes_timed;     /* shapes timed by this call */
  uint32_t pairs_per_thread; /* of the prediction count (trax_set_pairs_per_thread) */
  uint32_t candidate_slots;  /* trax_set_candidate_slots: 0 = the library's choice */
  uint32_t fine_rows;        /* trax_set_fine_rows */
  uint32_t reserved;         /* 0 */
  double best_ms;            /* device time of one chain replay at the chosen shape */
  double default_ms;         /* the same for the shape the context had before */
} trax_tune_result;
int trax_autotune(trax_ctx* ctx, const char* cache_path, const trax_tune_opts* opts, trax_tune_result* result);

/* Device time of the last run, from CUDA events on the context's stream
 * (RuntimeRecord's per-stage count/scan/store classes, RuntimeRecord.cpp:123-192):
 * stage_ms[7] = grid, pairs, prediction, filter, connectivity, circle fit, CA;
 * kernel_ms[9] = grid build, pair count, pair store, prediction count,
 * prediction store, filter, filter store, connectivity count, connectivity
 * store.  Entries that did not run are -1. */
int trax_get_timings(trax_ctx* ctx, float* stage_ms, float* kernel_ms);

/* ------------------------------------------------------------- results
 * Sizes first (*_size), then copies into caller-allocated host buffers. */
int trax_get_stats(trax_ctx* ctx, trax_batch_stats* stats);
/* Pairing::pairing / pairingOffsets (Pairings.h:9-59): pairs as (inner, outer)
 * uint32 pairs, offsets [n_events * n_lt + 1]. */
int trax_get_pairs(trax_ctx* ctx, uint32_t* pairs2, uint32_t* offsets);
/* Candidates (pair index, third hit) and their offsets. */
int trax_get_candidates(trax_ctx* ctx, uint32_t* cands2, uint32_t* offsets);
/* TrackletCollection hit columns and trackletOffsets (TrackletCollection.h:32-78). */
int trax_get_triplets(trax_ctx* ctx, uint32_t* h1, uint32_t* h2, uint32_t* h3, uint32_t* offsets);
/* Per-triplet eta (TripletConnectivityTight.h:47-79) and circle radius (TrackletCircleFitter.h:97). */
int trax_get_triplet_eta_pt(trax_ctx* ctx, float* eta, float* pt);
/* Links (basis, follower) and connectable / non-connectable index lists. */
int trax_get_links(trax_ctx* ctx, uint32_t* basis, uint32_t* follower, uint32_t* connectable,
                   uint32_t* non_connectable);
/* CA states, track collection and its offsets [n_triplets + 1]. */
int trax_get_tracks(trax_ctx* ctx, uint32_t* states, uint32_t* tracks, uint32_t* track_offsets);
/* Grid boundaries [n_events * n_layers * (n_z+1)(n_phi+1)] and, for every
 * grid-ordered hit, its index in the uploaded input. */
int trax_get_grid(trax_ctx* ctx, uint32_t* grid, uint64_t* n_cells);
int trax_get_hit_perm(trax_ctx* ctx, uint32_t* perm);

/* ----------------------------------------------- differentiable alignment
 * No counterpart in the reference.  An FP32 circle/helix fit of every
 * selected triplet -- the circle through the three hits (curvature, signed
 * transverse impact parameter d0; TrackletCircleFitter.h:32-97,
 * FastCircle.h:41-118) and the least-squares line z = z0 + cot(theta) s in
 * arc length from the point of closest approach (FastLine.h:15-42) -- with
 *     chi2 = sum over triplets of d0^2 / sigma_tip^2 + sum_i e_i^2 / sigma_z^2,
 * e_i the line residuals.  Hits are corrected by per-layer shifts
 * align[3 l + (0, 1, 2)] = (dr [cm], dz [cm], dphi [rad]) of layer l + 1:
 * r -> r + dr, phi -> phi + dphi, z -> z + dz.  The per-triplet arithmetic is
 * FP32; only the sums over triplets are FP64, taken in a fixed order. */
typedef struct trax_fit_opts {
  float sigma_z;       /* z resolution of a hit [cm]; <= 0: 0.002 */
  float sigma_tip[16]; /* per layer triplet [cm]; <= 0: 1.4826 x median |d0| of its rows at zero alignment */
  int truth_only;      /* 1: only triplets whose three hits share a nonzero hit id */
} trax_fit_opts;

/* Freezes the fit rows for the current triplets (after trax_triplet_filter,
 * trax_seed_batch or trax_set_tracklets): triplets whose hits lie on their
 * layer triplet's layers, optionally truth-matched, with a finite fit at zero
 * alignment, ordered by layer triplet then event.  The cut decisions are not
 * revisited by the calls below. */
int trax_fit_prepare(trax_ctx* ctx, const trax_fit_opts* opts, uint64_t* n_fit);
/* chi2 at `align` [3 n_layers]; params [n_fit x 4] = (curvature 1/R [1/cm],
 * d0 [cm], z0 [cm], cot theta) per row when not NULL. */
int trax_fit_forward(trax_ctx* ctx, const double* align, double* chi2, float* params);
/* Adjoint kernel: chi2, d chi2 / d align [3 n_layers], an approximate
 * Gauss-Newton diagonal [3 n_layers] for preconditioning (sum over rows of
 * (d d0 / d align)^2 / sigma_tip^2 for dr and dphi, of the z residuals'
 * projector diagonal for dz, and cot(theta)^2 times it for dr) and, when
 * d_hits is not NULL, d chi2 / d(x, y, z) of every uploaded hit [3 n_hits],
 * input order.  Any output may be NULL. */
int trax_fit_backward(trax_ctx* ctx, const double* align, double* chi2, double* d_align, double* gn_diag,
                      float* d_hits);
/* Corrects the uploaded hits in place by the shifts `align` [3 n_layers]
 * (the same transformation as the fit), so that the seeding chain can run
 * again on the aligned geometry; results of earlier stages are dropped. */
int trax_apply_alignment(trax_ctx* ctx, const double* align);
/* Row -> triplet index (into trax_get_triplets' arrays) [n_fit], and the
 * sigma_tip used per layer triplet [n_lt]. */
int trax_fit_get_rows(trax_ctx* ctx, uint32_t* triplet_index, float* sigma_tip);

/* ------------------------------------------------------------ event files
 * PEventContainer files (the reference's src/datastructures/serialize/
 * Event.proto: PEvent { runNumber, lumiSection, eventNumber, repeated PHit
 * { position, detectorType, layer, detectorId, hitId, simTrackID,
 * simTrackPt } }) read with a wire-format decoder of our own.  Host-only: no
 * context and no GPU. */
typedef struct trax_event_set trax_event_set;
int trax_events_read(const char* path, trax_event_set** events, uint64_t* n_events);
void trax_events_free(trax_event_set* events);
/* The hits of event e as stored; every output may be NULL (first call for
 * n_hits).  xyz [3 n_hits]; run_lumi_event [3]. */
int trax_events_raw(const trax_event_set* events, uint64_t e, uint64_t* n_hits, float* xyz, uint64_t* layer,
                    uint64_t* det_id, uint64_t* hit_id, uint64_t* sim_track_id, float* sim_pt, int32_t* det_type,
                    uint64_t* run_lumi_event);

typedef struct trax_loaded_sizes {
  uint64_t n_hits, n_events, n_layers, n_findable;
} trax_loaded_sizes;
/* HitCollection::addEvent (HitCollection.cpp:21-180) for events
 * [first, first + count): hits of simulated tracks with pT >= min_pt; a track
 * is findable when it has a hit on every layer of the layer triplets
 * (num_tracks >= 0 stops after that many findable tracks; only_tracks drops
 * the hits of the other tracks); per event the hits are bucketed by layer 1
 * .. highest layer, findable tracks' hits after the others.  The hit_id
 * column carries the simulated track id, as in the reference.  Call with
 * NULL arrays first to get the sizes, then with arrays of those sizes:
 * x, y, z, layer, det_id, hit_id, event [n_hits]; event_offsets [n_events];
 * layer_hits, layer_offsets [n_events * n_layers] (offsets from the event's
 * first hit); findable_id, findable_event [n_findable]. */
int trax_events_load(const trax_event_set* events, uint64_t first, uint64_t count, const trax_layer_triplet* lt,
                     int n_lt, float min_pt, int num_tracks, int only_tracks, trax_loaded_sizes* sizes, float* x,
                     float* y, float* z, uint32_t* layer, uint32_t* det_id, uint32_t* hit_id, uint32_t* event,
                     uint32_t* event_offsets, uint32_t* layer_hits, uint32_t* layer_offsets, uint32_t* findable_id,
                     uint32_t* findable_event);

/* The same loader with its layer bucketing on the device, straight into the
 * context (in place of trax_events_load + trax_upload_hits): the host
 * classifies every hit of events [first, first + count) as addEvent does
 * (track pT, findability, the track limit) and gives each kept hit its
 * (layer, push position) key; one CTA per event then sorts the keys and
 * gathers the hit columns into the context's input arrays.  The context
 * ends up exactly as after trax_upload_hits with trax_events_load's output.
 * sizes as trax_events_load; the first min(n_findable, findable_cap)
 * findable track ids and events are copied out (either may be NULL). */
int trax_events_upload(trax_ctx* ctx, const trax_event_set* events, uint64_t first, uint64_t count,
                       const trax_layer_triplet* lt, int n_lt, float min_pt, int num_tracks, int only_tracks,
                       trax_loaded_sizes* sizes, uint32_t* findable_id, uint32_t* findable_event,
                       uint64_t findable_cap);

/* GeometrySupplement from the reference's detector tables
 * (TripletBuilder.cpp:140-184): radius_dictionary rows "entry,radius",
 * detector_radius rows "detId,entry,layer"; min/max radius of layers
 * 1..n_layers over their modules, (10000, 0) for a layer without any. */
int trax_geometry_from_files(const char* radius_dictionary, const char* detector_radius, uint32_t n_layers,
                             float* min_r, float* max_r);

/* ------------------------------------------------------------ physics
 * PhysicsRecord::fillData / merge / csvDump (PhysicsRecord.cpp:86-404):
 * per event and layer triplet, the fraction of findable tracks with a
 * triplet (efficiency), and the fractions of the segment's triplets that
 * are fakes (hits of different tracks) or clones (a track's second and
 * later triplets); merged over events into means and standard deviations
 * per layer triplet, out[p] for p < n_lt, and over all of them in
 * out[n_lt] (layer_triplet = n_lt + 1, as the reference's csv).  Host-only.
 * hit_track_id: the track id of every hit the triplets index. */
typedef struct trax_physics_record {
  uint32_t layer_triplet;
  uint64_t n;
  double efficiency, efficiency_dev, fake_rate, fake_rate_dev, clone_rate, clone_rate_dev;
} trax_physics_record;
int trax_physics_triplets(const uint32_t* h1, const uint32_t* h2, const uint32_t* h3, const uint32_t* offsets,
                          uint32_t n_events, uint32_t n_lt, const uint32_t* hit_track_id, const uint32_t* findable_id,
                          const uint32_t* findable_event, uint64_t n_findable, trax_physics_record* out);

/* The same records for the context's current triplets, counted on the
 * device: fake and real triplets and the distinct findable tracks found per
 * (event, layer triplet) are counted by kernels over the triplets and the
 * grid-ordered hit ids left on the device; only those counts come back for
 * the means and deviations.  Equal to trax_physics_triplets on the
 * downloaded triplets with the grid-ordered hit ids. */
int trax_physics_triplets_device(trax_ctx* ctx, const uint32_t* findable_id, const uint32_t* findable_event,
                                 uint64_t n_findable, trax_physics_record* out);

/* Track evaluation of TripletBuilder.cpp:840-1066: tracks of three or more
 * triplets from the CA output (trax_get_tracks), clone removal (tracks that
 * share at least 19 % of the shorter one's hits), real tracks (all hits of
 * one simulated track), fake and clone rates over the filtered tracks and
 * efficiency = distinct real tracks / total_tracks.  Host-only. */
typedef struct trax_track_metrics {
  uint64_t total, filtered, valid, valid_unique, fakes;
  double fake_rate, clone_rate, efficiency;
} trax_track_metrics;
int trax_physics_tracks(const uint32_t* tracks, const uint32_t* track_offsets, uint64_t n_triplets,
                        const uint32_t* h1, const uint32_t* h2, const uint32_t* h3, const uint32_t* hit_track_id,
                        uint64_t total_tracks, trax_track_metrics* out);
/* The same for the context's current CA output, on the device: the tracks
 * are extracted there, the clone removal runs as independent greedy passes
 * over the connected components of the "shares a hit" graph (two tracks
 * without a common hit never compare, so the components' passes give the
 * list's result), and only the counts come back. */
int trax_physics_tracks_device(trax_ctx* ctx, uint64_t total_tracks, trax_track_metrics* out);

#ifdef __cplusplus
}
#endif

#endif /* TRAX_H_ */
