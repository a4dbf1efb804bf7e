// trax_kernels.h -- host-side launchers of the sm_103a kernels.  Each
// launcher enqueues work on `st` and adds the number of kernels it launched
// to *launches.  Counts that are only known on the device are passed as
// device pointers together with a host-side capacity that sizes the grid.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "trax_device.cuh"

struct trax_ctx;

namespace trax {

// ---------------------------------------------------------------- scans
size_t scan_scratch_bytes(uint64_t maxN);
// Exclusive scan of n elements (or *nDev + nAdd when nDev != nullptr, with
// maxN bounding the launch), in place allowed.  Outputs wrap modulo 2^32;
// with flagOverflow a total of 2^32 or more sets TRAX_EBIT_OVERFLOW.  `ctl`
// bounds the look-back waits (and may name a tile that never publishes).
cudaError_t scan_exclusive(const uint32_t* in, uint32_t* out, uint64_t n, const uint32_t* nDev, uint32_t nAdd,
                           uint64_t maxN, void* scratch, uint32_t* err, cudaStream_t st, uint32_t* launches,
                           bool flagOverflow, WaitCtl ctl);
cudaError_t max_scan_inclusive(uint32_t* data, uint32_t n, cudaStream_t st, uint32_t* launches);

// ------------------------------------------------------ event bucketing
// The hits of a group of events as their file holds them, with the host's
// bucketing keys (trax_events.h); scratchOffsets[e]: the event's global
// sort scratch (events too large for shared memory).
struct RawEventHits {
  const float* x;
  const float* y;
  const float* z;
  const uint32_t* layer;
  const uint32_t* det;
  const uint32_t* tid;
  const unsigned long long* key;
  const uint32_t* rawOffsets;      // [E+1]
  const uint32_t* scratchOffsets;  // [E]
};
// the context's input hit columns and the first kept hit of each event
struct HitColumns {
  float* x;
  float* y;
  float* z;
  uint32_t* layer;
  uint32_t* det;
  uint32_t* hid;
  uint32_t* evt;
  const uint32_t* eventOffsets;  // [E]
};
// global scratch keys an event of this many hits needs (0: shared memory)
uint32_t bucket_scratch_keys(uint32_t hitsInEvent);
// every event's kept hits, sorted by key, into the columns at its offset
cudaError_t bucket_events(const RawEventHits& in, unsigned long long* scratch, uint32_t nEvents, uint32_t nKept,
                          HitColumns out, cudaStream_t st, uint32_t* launches);

// per (event, layer triplet) segment of the triplet offsets [S+1]: fake
// triplets, real
// triplets of findable tracks, distinct findable tracks found; findIds are
// each event's findable track ids, sorted, from findOff[e]; foundFlags
// [nLT * n_findable] zeroed by the caller, as are fakes and realFindable
cudaError_t physics_counts(const uint32_t* h1, const uint32_t* h2, const uint32_t* h3, const uint32_t* nTDev,
                           uint64_t maxT, const uint32_t* offsets, const uint32_t* hitTrack, uint32_t nEvents,
                           uint32_t nLT, const uint32_t* findOff,
                           const uint32_t* findIds, uint32_t* fakes, uint32_t* realFindable, uint32_t* foundFlags,
                           uint32_t* found, cudaStream_t st, uint32_t* launches);

// ------------------------------------------------------ track evaluation
// The tracks of the CA output (k_tracks.cu): [nTracks] hit-list start and
// size, real flag, first hit's simulated track id, union-find parent,
// component size / start / cursor (nTracks + 1 for the scan), members and
// the filtered list per component; [entries] hits and their track; [hits]
// the smallest track holding each hit.
struct TrackLists {
  uint32_t* start;
  uint32_t* size;
  uint32_t* real;
  uint32_t* firstId;
  uint32_t* parent;
  uint32_t* compSize;
  uint32_t* compStart;
  uint32_t* cursor;
  uint32_t* members;
  uint32_t* filtered;
  uint32_t* hits;
  uint32_t* entryTrack;
  uint32_t* owner;
};
// isTrack[i], hitsOf[i] for i <= nT (the +1 slots zero): chains of three or
// more triplets and their hit counts
cudaError_t track_sizes(const uint32_t* off, uint32_t nT, uint32_t* isTrack, uint32_t* hitsOf, cudaStream_t st);
// with isTrack / hitsOf scanned into trackOf / hitStart
cudaError_t track_extract(const uint32_t* off, const uint32_t* chain, uint32_t nT, const uint32_t* h1,
                          const uint32_t* h2, const uint32_t* h3, const uint32_t* hitTrack, const uint32_t* trackOf,
                          const uint32_t* hitStart, TrackLists t, cudaStream_t st);
// one union-find round (hook, compress); *changed set when a root moved
cudaError_t track_union_step(TrackLists t, uint32_t nTracks, uint32_t nEntries, uint32_t* changed, cudaStream_t st);
// place == false: component sizes; true: members at the scanned starts
cudaError_t track_members(TrackLists t, uint32_t nTracks, bool place, cudaStream_t st);
// per component the greedy clone removal; counts[0..2]: filtered, real,
// distinct real simulated track ids (table: 2^k zeroed slots, mask 2^k - 1)
cudaError_t track_greedy(TrackLists t, uint32_t nTracks, unsigned long long* table, uint32_t tableMask,
                         unsigned long long* counts, cudaStream_t st);

// ------------------------------------------------------------ grid build
struct GridInput {
  const float* x;
  const float* y;
  const float* z;
  const uint32_t* layer;
  const uint32_t* det;
  const uint32_t* hid;
  const uint32_t* evt;
  const uint32_t* eventOffsets;  // [E]
  const uint32_t* layerHits;     // [E*L]
  const uint32_t* layerOffsets;  // [E*L]
};

struct GridScratch {
  uint32_t* cell;    // [n]
  float* phi;        // [n]
  uint32_t* perm;    // [n]
  uint32_t* counts;  // [E*L*C] used when the cell counters do not fit in shared memory
};

cudaError_t grid_build(const DevConfig& cfg, const GridInput& in, uint32_t* grid, DevHits out,
                       GridScratch scratch, uint32_t maxLayerHits, uint32_t* err, cudaStream_t st,
                       uint32_t* launches);
cudaError_t grid_prepare(int device);  // one-time kernel attributes

// The fine z grid the prediction count walks when cfg.fineRows > 0: the
// grid-ordered hits of every (event, layer) sorted again by fine cell (fine
// row = fine_row of the hit's z inside its z row's block of fineRows rows,
// the same phi column), ties by grid order.  grid[E*L*fineC] holds the
// cell starts like the grid's, hits[n] each hit in fine order as (z, phi,
// its grid-order index as the bits of a float, 0): one 16-byte load gives
// a visit its test and its candidate.  Built from the grid and the
// grid-ordered packed hits (xyzp) after grid_build; `counters` (global
// scratch of fine_counter_cells(cfg) words) is used only when one z row's
// fine cells do not fit in shared memory.
struct FineGrid {
  uint32_t* grid;
  float4* hits;
};
// dynamic shared memory the grid builds give one CTA
#define TRAX_GRID_SMEM_BYTES (227u * 1024u - 256u)
inline uint32_t fine_row_cells(const DevConfig& cfg) { return cfg.fineRows * (cfg.nP + 1); }
inline uint64_t fine_counter_cells(const DevConfig& cfg) {
  return (uint64_t)fine_row_cells(cfg) * sizeof(uint32_t) > TRAX_GRID_SMEM_BYTES
             ? (uint64_t)cfg.E * cfg.L * cfg.nZ * fine_row_cells(cfg)
             : 0;
}
cudaError_t fine_grid_build(const DevConfig& cfg, const uint32_t* grid, const float4* xyzp, FineGrid fine,
                            uint32_t* counters, cudaStream_t st, uint32_t* launches);
// hit collection = uploaded hits in input order (plus the packed xyz-phi array)
cudaError_t identity_hits(const GridInput& in, uint32_t n, DevHits out, cudaStream_t st, uint32_t* launches);

// ----------------------------------------------------------------- pairs
// Per (event, layer triplet) segment: first outer hit and number of outer hits.
cudaError_t pair_segments(const DevConfig& cfg, const uint32_t* grid, uint32_t* segOuter, uint32_t* segCount,
                          cudaStream_t st, uint32_t* launches);
// What the count pass leaves for the store pass per outer-hit task k, so
// that the store pass neither searches the task's segment nor recomputes
// its window: bounds[k] = (zLow, zHigh, phiLow, phiHigh);
// secs[k] = (zLowSector | ordered << 31, zHighSector | wrap << 31, pL, pH),
// `ordered` when the task's visit ranges are disjoint and ascending
// (zLowSector <= INT32_MAX, zHighSector <= nZ < 2^22); ids[k] = (outer hit,
// segment).  pair_task_state_bytes(n) bytes hold the arrays of n tasks.
struct PairTaskState {
  float4* bounds;
  uint4* secs;
  uint2* ids;
};
inline size_t pair_task_state_bytes(uint64_t n) { return (size_t)n * 40u; }
inline PairTaskState pair_task_state(void* base, uint64_t n) {
  char* b = static_cast<char*>(base);
  return PairTaskState{reinterpret_cast<float4*>(b), reinterpret_cast<uint4*>(b + 16 * n),
                       reinterpret_cast<uint2*>(b + 32 * n)};
}

// Count (emit == false) or store (emit == true) pairs of every outer-hit task.
// taskBase[S+1] is the exclusive scan of segCount; nTasksDev = &taskBase[S].
// The count pass writes `state`, the store pass reads it.
cudaError_t pair_tasks(const DevConfig& cfg, bool emit, const uint32_t* grid, DevHits hits,
                       const uint32_t* segOuter, const uint32_t* taskBase, const uint32_t* nTasksDev,
                       uint64_t maxTasks, uint32_t* taskCount, PairTaskState state, uint2* pairs,
                       uint64_t capPairs, uint32_t* sentinelCount, uint32_t* err, cudaStream_t st,
                       uint32_t* launches);
// pairOffsets[s+1] = first pair of segment s+1 (Pairing::pairingOffsets)
cudaError_t pair_offsets(const DevConfig& cfg, const uint32_t* taskBase, const uint32_t* pairStart,
                         uint32_t* pairOffsets, cudaStream_t st, uint32_t* launches);

// ------------------------------------------------------------ prediction
// Count pass (emit == false): per pair the exclusive offset of its
// candidates within its warp of 32 pairs (candCount[nPairs]), the sum of
// each warp's counts in warpSums[ceil(nPairs/32) + 1] (+1 slot zeroed; the
// number of sums goes to *nWarpsOut) and up to cfg.predKeep captured
// candidates per pair in keep[nPairs * cfg.predKeep]; store pass
// (emit == true): with warpSums exclusively scanned, candidates at
// warpSums[gid / 32] + candCount[gid].  predKeep is 4 (TRAX_PRED_KEEP,
// the default) to TRAX_PRED_KEEP_MAX.
#define TRAX_PRED_KEEP 4
#define TRAX_PRED_KEEP_MAX 32
// words of the captured candidates of `pairs` pairs, whole warps of 32
// pairs; the slots of a warp's pairs are interleaved (keep_slots) with 16 or
// more slots per pair or with the fine z grid
inline uint64_t pred_keep_words(uint64_t pairs, uint32_t keep) { return (pairs + 31) / 32 * 32 * keep; }
inline bool keep_interleaved(const DevConfig& cfg) { return cfg.predKeep >= 16u || cfg.fineRows > 0u; }

// grids of up to this many cells per layer are built with shared-memory
// counters (4 bytes per cell)
#define TRAX_GRID_SMEM_CELLS 53248u
// With cfg.fineRows > 0 the count pass, and the store pass's re-walks of
// pairs with more candidates than slots, walk `fine` (same outputs).
cudaError_t predict_pairs(const DevConfig& cfg, bool emit, const uint32_t* grid, DevHits hits, const uint2* pairs,
                          const uint32_t* nPairsDev, uint64_t maxPairs, uint32_t* candCount, uint32_t* warpSums,
                          uint32_t* nWarpsOut, uint32_t* keep, uint2* cands, uint64_t capCands,
                          uint32_t* sentinelCount, uint32_t* err, cudaStream_t st, uint32_t* launches,
                          FineGrid fine = FineGrid{nullptr, nullptr});
cudaError_t predict_offsets(const DevConfig& cfg, const uint32_t* pairOffsets, const uint32_t* nPairsDev,
                            const uint32_t* candCount, const uint32_t* warpStart, uint32_t* candOffsets,
                            cudaStream_t st, uint32_t* launches);

// ---------------------------------------------------------------- filter
// the flags of 32 consecutive candidates as one word masks[g / 32] (bit
// g % 32), the number of flags set per word in warpSums[ceil(n/32) + 1]
// (+1 slot zeroed; the number of words goes to *nWordsOut)
cudaError_t filter_candidates(const DevConfig& cfg, DevHits hits, const uint2* pairs, const uint2* cands,
                              const uint32_t* nCandsDev, uint64_t maxCands, uint32_t* masks, uint32_t* warpSums,
                              uint32_t* nWordsOut, cudaStream_t st, uint32_t* launches);
// with warpSums exclusively scanned into wordStart: the triplets of the
// flagged candidates at wordStart[g / 32] + (flags below g in its word)
cudaError_t filter_store(const uint2* pairs, const uint2* cands, const uint32_t* nCandsDev, uint64_t maxCands,
                         const uint32_t* masks, const uint32_t* wordStart, uint32_t* h1, uint32_t* h2, uint32_t* h3,
                         uint64_t capT, cudaStream_t st, uint32_t* launches);
// trackletOffsets with the reference's filterOffsetStore + monotonize semantics
cudaError_t triplet_offsets(const DevConfig& cfg, DevHits hits, const uint32_t* h1, const uint32_t* nTDev,
                            uint64_t maxT, uint32_t* offsets, cudaStream_t st, uint32_t* launches);

// ---------------------------------------------------------- connectivity
struct TripletView {
  const uint32_t* h1;
  const uint32_t* h2;
  const uint32_t* h3;
  const uint32_t* nDev;
  uint64_t maxN;
};

cudaError_t triplet_eta(const DevConfig& cfg, DevHits hits, TripletView t, float* eta, uint32_t* seg,
                        cudaStream_t st, uint32_t* launches);
cudaError_t segment_bounds(const DevConfig& cfg, const uint32_t* seg, const uint32_t* nTDev, uint32_t* segStart,
                           cudaStream_t st, uint32_t* launches);
// runStart[t]: where the count pass found the (h2, h1) run of t's
// followers in sorted segments; the store pass starts there
cudaError_t connectivity_tasks(const DevConfig& cfg, bool emit, DevHits hits, TripletView t, const float* eta,
                               const uint32_t* offsets, const uint32_t* segStart, uint32_t* linkCount,
                               uint32_t* flags, uint32_t* runStart, uint32_t* basis, uint32_t* follower,
                               uint64_t capLinks, bool sortedSegments, cudaStream_t st, uint32_t* launches);
// flags[k] for k < n-1 -> words of 32 (flag) and (!flag) bits with the number
// set per word (+1 slots zeroed, the number of words to *nWordsOut)
cudaError_t connectable_words(const uint32_t* flags, const uint32_t* nTDev, uint64_t maxT, uint32_t* connWords,
                              uint32_t* connSums, uint32_t* nonWords, uint32_t* nonSums, uint32_t* nWordsOut,
                              cudaStream_t st, uint32_t* launches);
// with the sums scanned into wordStart: outIdx[wordStart[k / 32] + (bits
// below k in its word)] = k for every set bit k < *nTDev
cudaError_t compact_words(const uint32_t* words, const uint32_t* wordStart, const uint32_t* nTDev, uint64_t maxT,
                          uint32_t* outIdx, uint64_t capOut, cudaStream_t st, uint32_t* launches);
// *dst = data[n] (n = *nDev, or nHost when nDev is null): the total a scan of
// n+1 elements left in its last slot, clamped to cap (TRAX_EBIT_CAPACITY)
cudaError_t publish_total(const uint32_t* data, const uint32_t* nDev, uint64_t nHost, uint64_t cap, uint32_t* dst,
                          uint32_t* err, cudaStream_t st, uint32_t* launches);

// ---------------------------------------------------- circle fit and CA
cudaError_t circle_fit(DevHits hits, TripletView t, const uint32_t* connectable, const uint32_t* nConnDev,
                       uint64_t maxConn, float* pt, cudaStream_t st, uint32_t* launches);

struct CABuffers {
  uint32_t* states;    // [nT]
  uint32_t* inStart;   // [nT+1]
  uint32_t* inCursor;  // [nT]
  uint32_t* inList;    // [nLinks] bases of the incoming links, grouped by follower
  uint32_t* best;      // [nT]
  uint32_t* isBest;    // [nT]
  uint32_t* handlers;  // [nT+1]
  uint32_t* segOf;     // [nT] layer-triplet segment of each triplet
};

cudaError_t ca_in_degree(const uint32_t* follower, const uint32_t* nLinksDev, uint64_t maxLinks, CABuffers b,
                         const uint32_t* nTDev, uint64_t maxT, cudaStream_t st, uint32_t* launches);
cudaError_t ca_fill(const uint32_t* basis, const uint32_t* follower, const uint32_t* nLinksDev, uint64_t maxLinks,
                    CABuffers b, const uint32_t* nTDev, uint64_t maxT, cudaStream_t st, uint32_t* launches);
cudaError_t ca_forward(const DevConfig& cfg, CABuffers b, const uint32_t* nTDev, uint64_t maxT, cudaStream_t st,
                       uint32_t* launches);
// One forward iteration of the reference's CA over any link set
// (CellularAutomaton.h:52-100); *living is set when a cell lives.
cudaError_t ca_iteration(const uint32_t* basis, const uint32_t* follower, uint32_t nLinks, const uint32_t* cur,
                         uint32_t* next, uint32_t* living, cudaStream_t st, uint32_t* launches);
cudaError_t fill_u32(uint32_t* p, uint32_t v, uint32_t n, cudaStream_t st, uint32_t* launches);
cudaError_t ca_backward(const float* pt, CABuffers b, const uint32_t* nTDev, uint64_t maxT,
                        const uint32_t* nLinksDev, cudaStream_t st, uint32_t* launches);
cudaError_t ca_tracks(CABuffers b, const uint32_t* nTDev, uint64_t maxT, uint32_t* tracks, uint64_t maxTracks,
                      uint32_t* err, cudaStream_t st, uint32_t* launches);

// ------------------------------------------- differentiable triplet fit
// Fit rows are the selected triplets ordered by layer triplet; rows of layer
// triplet k are [ltBase[k], ltBase[k+1]) and are reduced by the blocks
// [blkStart[k], blkStart[k+1]), each taking FIT_CHUNK rows, so that every
// FP64 sum is taken in a fixed order.
#define TRAX_FIT_CHUNK 4096u
// per block: chi2, d chi2 / d(dr, dz, dphi) of the three hit layers, and an
// approximate Gauss-Newton diagonal for the same nine (a preconditioner)
#define TRAX_FIT_SLOTS 19

struct FitConfig {
  uint32_t L, nLT, nBlocks;
  uint32_t layer[3][TRAX_MAX_LT];  // 0-based layer of each hit slot of a layer triplet
  float wTip[TRAX_MAX_LT];         // 1 / sigma_tip^2 per layer triplet
  float wZ;                        // 1 / sigma_z^2
  // per-layer correction: r -> r + dr, z -> z + dz, rotation by dphi given
  // as sin(dphi) and cos(dphi) - 1 (both from double precision on the host)
  float dr[TRAX_MAX_LAYERS], dz[TRAX_MAX_LAYERS], sn[TRAX_MAX_LAYERS], cm1[TRAX_MAX_LAYERS];
  uint32_t ltBase[TRAX_MAX_LT + 1];
  uint32_t blkStart[TRAX_MAX_LT + 1];
};

// ok[t] = 1 for triplets whose hits lie on their layer triplet's layers, whose
// three hits share a nonzero hit id when truthOnly, and whose fit at the
// configured alignment is finite; segCount[s] counts them per segment
cudaError_t fit_select(const FitConfig& fc, const DevConfig& cfg, DevHits hits, TripletView t, uint64_t nT,
                       int truthOnly, uint32_t* ok, uint32_t* segCount, cudaStream_t st, uint32_t* launches);
// rows[okScan[t] + segDelta[seg(t)]] = t for the selected triplets
cudaError_t fit_scatter(const DevConfig& cfg, DevHits hits, TripletView t, uint64_t nT, const uint32_t* okScan,
                        const int32_t* segDelta, uint32_t* rows, cudaStream_t st, uint32_t* launches);
// chi2 (and with grad: alignment and hit gradients) of the fit rows.
// partials[b * TRAX_FIT_SLOTS + k]; params[row * 4] = (curvature, d0, z0,
// cot theta) when not null; dHits (double, grid order, 3 per hit) is added to
// when not null.
cudaError_t fit_eval(const FitConfig& fc, bool grad, DevHits hits, TripletView t, const uint32_t* rows,
                     double* partials, float* params, double* dHits, cudaStream_t st, uint32_t* launches);
// out[0] = chi2, out[1 + 3 l + p] = d chi2 / d(dr, dz, dphi)_l, and
// out[1 + 3 L + 3 l + p] = the approximate Gauss-Newton diagonal; fixed-order sums
cudaError_t fit_reduce(const FitConfig& fc, const double* partials, double* out, cudaStream_t st,
                       uint32_t* launches);
// uploaded (input-order) hits corrected in place by fc's per-layer shifts
cudaError_t fit_apply(const FitConfig& fc, float* x, float* y, float* z, const uint32_t* layer, uint64_t n,
                      cudaStream_t st, uint32_t* launches);
// float gradient per input hit from the double grid-order sums
cudaError_t fit_hits_out(const double* dHits, const uint32_t* orig, uint64_t nHits, float* out, cudaStream_t st,
                         uint32_t* launches);

// number of SMs of the current device (cached)
int sm_count();

// context hooks for the autotuner (capi.cu)
uint64_t workload_hash(const trax_ctx* c);
int ctx_device(const trax_ctx* c);
bool ctx_ready(const trax_ctx* c);
void ctx_set_error(trax_ctx* c, const char* msg);

}  // namespace trax
