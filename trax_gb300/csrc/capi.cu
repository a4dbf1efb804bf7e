// capi.cu -- the C ABI of include/trax/trax.h: context, configuration,
// uploads, the stage chain and result downloads.
//
// One chain implementation runs in two modes:
//   * SYNCED: after every compaction scan the host reads the total (one
//     4-byte device-to-host copy) and sizes the next buffers exactly -- the
//     launch structure of the reference's run() methods (count, scan,
//     downloadScalar, allocate, store).  The stage entry points use it.
//   * DEVICE: no host reads.  Every kernel takes its item count from a fixed
//     device slot (written by a one-thread publish kernel after each scan) and
//     every output has a capacity learnt from an earlier SYNCED run plus
//     headroom.  A total above its capacity is clamped and reported as
//     TRAX_ERR_CAPACITY, never silently truncated.  This mode is captured once
//     into a CUDA graph and replayed by trax_seed_batch.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "trax/trax.h"
#include "trax_events.h"
#include "trax_kernels.h"

using namespace trax;

namespace trax {

int sm_count() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
  }
  return n;
}

}  // namespace trax

namespace {

struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
};

template <typename T>
T* ptr(const DevBuf& b) {
  return static_cast<T*>(b.p);
}

// fixed device slots of the error word, counters and totals
enum Slot {
  S_ERR = 0,
  S_PAIR_SENT,
  S_CAND_SENT,
  S_TASKS,
  S_PAIRS,
  S_CANDS,
  S_TRIPLETS,
  S_LINKS,
  S_CONN,
  S_NONCONN,
  S_TRACKS,
  S_PRED_WARPS,
  S_FLAG_WORDS,
  S_CONN_WORDS,
  S_USER,    // length of a caller-provided list (trax_circle_fit_on)
  S_LIVING,  // living flag of the caller-link CA iteration
  S_N
};
static_assert(S_N <= 64, "the slot buffers hold 64 words");

enum Mode { SYNCED, DEVICE };

// kernels timed individually with CUDA events (order of trax_get_timings)
enum TimedKernel {
  TK_GRID = 0,
  TK_PAIR_COUNT,
  TK_PAIR_EMIT,
  TK_PRED_COUNT,
  TK_PRED_EMIT,
  TK_FILTER,
  TK_FILTER_STORE,
  TK_CONN_COUNT,
  TK_CONN_EMIT,
  TK_N
};
const int N_STAGES = 7;

const uint64_t NO_CAP = 0xffffffffull;

}  // namespace

struct trax_ctx {
  int device = 0;
  cudaStream_t st = nullptr;
  std::string err;
  // configuration
  std::vector<trax_layer_triplet> lts;
  float minPt = 0.0f;
  std::vector<float> minR, maxR;
  uint32_t nZ = 0, nP = 0;
  uint32_t pairThreads = 128, predThreads = 128, filterThreads = 256;  // launch shape
  uint32_t predK = 1;  // pairs per thread of the prediction count pass
  // candidates the prediction count captures per pair: keepSlots when the
  // caller set it, else keepAuto, chosen after each calibration
  uint32_t keepSlots = 0, keepAuto = TRAX_PRED_KEEP;
  uint32_t fineRows = 0;  // rows of the prediction count's fine z grid per grid row (0: none)
  uint32_t fineBuilt = 0;  // fineRows of the fine grid the last grid stage built
  bool haveLT = false, haveGeom = false, haveGrid = false, haveHits = false;
  bool cfgDirty = true;  // layer triplets or geometry changed since the device configuration was built
  // batch shape
  uint32_t E = 0, L = 0, nHits = 0;
  float dEtaCut = 0.0256f;
  DevConfig cfg;
  // inputs
  DevBuf in_x, in_y, in_z, in_layer, in_det, in_hid, in_evt, evOff, layHits, layOff;
  // event-file hits for the device bucketing (trax_events_upload)
  DevBuf raw_x, raw_y, raw_z, raw_layer, raw_det, raw_tid, raw_key, raw_off, raw_scratchOff, raw_scratch;
  // triplet physics counts (trax_physics_triplets_device)
  DevBuf phys_findOff, phys_findIds, phys_flags, phys_counts;
  // track evaluation (trax_physics_tracks_device)
  DevBuf trk_isTrack, trk_hitsOf, trk_start, trk_size, trk_real, trk_firstId, trk_parent, trk_compSize,
      trk_compStart, trk_cursor, trk_members, trk_filtered, trk_hits, trk_entryTrack, trk_owner, trk_table,
      trk_counts;
  // grid stage
  DevBuf grid, px, py, pz, player, pdet, phid, pevt, porig, pxyzp, sc_cell, sc_phi, sc_perm, sc_counts;
  DevBuf fineGrid, fineHits;  // the fine z grid (fineRows > 0)
  // pair stage
  DevBuf segOuter, taskBase, taskCount, taskState, pairs, pairOffsets;
  // prediction / filter
  DevBuf candLocal, predWarps, predKeep, cands, candOffsets, flagWords, flagSums, h1, h2, h3, tripOffsets;
  // connectivity / fit / CA
  DevBuf eta, segOf, segStart, linkCount, linkRun, cflags, basis, follower, connS, nonConnS, connW, nonConnW, connIdx, nonConnIdx, pt;
  DevBuf states, inStart, inCursor, inList, best, isBest, handlers, tracks;
  DevBuf userIdx, caNext;  // caller-provided fit list; second state buffer of the caller-link CA
  // bookkeeping
  DevBuf scanScratch, slots;
  uint32_t* hSlots = nullptr;  // pinned copy of the slots
  uint32_t maxLayerHits = 0;   // most hits of one (event, layer) in the uploaded batch
  // sizes of the last run
  uint64_t nTasks = 0, nPairs = 0, nCands = 0, nT = 0, nLinks = 0, nConn = 0, nNonConn = 0, nTracks = 0;
  uint64_t pairSent = 0, candSent = 0;
  int stage = 0;  // last completed stage: 1 grid .. 7 CA
  bool noLinks = true;
  // triplets of every segment ordered by (second hit, first hit): true for the
  // chain's own filter output; checked for caller-provided triplets
  bool sortedSegments = true;
  bool identityHits = false;  // hit collection taken as uploaded (trax_set_tracklets)
  uint32_t launches = 0;
  // DEVICE-mode capacities and the captured graph
  uint64_t capTasks = 0, capPairs = 0, capCands = 0, capT = 0, capLinks = 0, capTracks = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graphExec = nullptr;
  uint64_t graphKey = 0;
  uint64_t bufGeneration = 0;
  trax::WaitCtl wait;  // bounded-wait settings of every scan (trax_set_wait_limit, trax_debug_skip_publish)
  uint32_t graphLaunches = 0;
  uint64_t graphCaptures = 0;  // calibrate-and-capture passes of the last trax_seed_batch
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double lastMs = 0.0;
  // per-stage and per-kernel timing events of the last run
  // differentiable fit: rows frozen by trax_fit_prepare for one triplet set
  DevBuf fitOk, fitSegCnt, fitSegDelta, fitRows, fitPartials, fitOut, fitParams, fitDHits, fitDHitsF;
  FitConfig fitCfg;
  uint64_t nFit = 0;
  bool fitReady = false;
  uint64_t tripGen = 1, fitTripGen = 0;  // generation of the triplet set
  // pt and CA results valid for triplet set ptGen / caGen (set by the stages
  // and by the caller-input entry points)
  uint64_t ptGen = 0, caGen = 0;
  bool caOnly = false;  // triplet count taken from the CA's caller input, no triplet arrays
  float fitSigmaTip[TRAX_MAX_LT] = {};
  cudaEvent_t stageEv[N_STAGES + 1] = {};

  cudaEvent_t kEv[2 * TK_N] = {};
  bool stageUsed[N_STAGES] = {};
  bool kUsed[TK_N] = {};
};

namespace {

const char* kVersion = "trax_gb300 0.1 (sm_103a)";

int fail(trax_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

int cuda_fail(trax_ctx* c, cudaError_t e, const char* where) {
  std::string m = std::string(where) + ": " + cudaGetErrorString(e);
  return fail(c, TRAX_ERR_CUDA, m);
}

#define CK(call)                                           \
  do {                                                     \
    cudaError_t e_ = (call);                               \
    if (e_ != cudaSuccess) return cuda_fail(c, e_, #call); \
  } while (0)

#define RC(call)              \
  do {                        \
    int r_ = (call);          \
    if (r_ != TRAX_OK) return r_; \
  } while (0)

cudaError_t ensure(trax_ctx* c, DevBuf& b, size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (bytes <= b.cap) return cudaSuccess;
  if (b.p) {
    cudaError_t e = cudaFree(b.p);
    if (e != cudaSuccess) return e;
    b.p = nullptr;
    b.cap = 0;
  }
  size_t want = bytes + bytes / 8 + 256;
  cudaError_t e = cudaMalloc(&b.p, want);
  if (e != cudaSuccess) {
    b.p = nullptr;
    return e;
  }
  b.cap = want;
  c->bufGeneration++;
  return cudaSuccess;
}

void release(DevBuf& b) {
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.cap = 0;
}

DevHits dev_hits(trax_ctx* c) {
  DevHits h;
  h.x = ptr<float>(c->px);
  h.y = ptr<float>(c->py);
  h.z = ptr<float>(c->pz);
  h.layer = ptr<uint32_t>(c->player);
  h.det = ptr<uint32_t>(c->pdet);
  h.hid = ptr<uint32_t>(c->phid);
  h.evt = ptr<uint32_t>(c->pevt);
  h.orig = ptr<uint32_t>(c->porig);
  h.xyzp = ptr<float4>(c->pxyzp);
  return h;
}

uint32_t* slot(trax_ctx* c, int k) { return ptr<uint32_t>(c->slots) + k; }

// The fine grid's buffers (to build it), and the fine grid the prediction
// count may walk: only one the last grid stage built for the current
// configuration (stages run one by one may change it in between).
FineGrid fine_buffers(trax_ctx* c) {
  if (!c->cfg.fineRows) return FineGrid{nullptr, nullptr};
  return FineGrid{ptr<uint32_t>(c->fineGrid), ptr<float4>(c->fineHits)};
}
FineGrid fine_grid(trax_ctx* c) {
  if (c->fineBuilt != c->cfg.fineRows) return FineGrid{nullptr, nullptr};
  return fine_buffers(c);
}

// A named NVTX range for the host side of a stage or call (what the
// reference's per-run cl_event lists and RuntimeRecord classes show,
// KernelWrapper.hpp:29-33, RuntimeRecord.cpp:123-192); free when no tool
// is attached.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

// event marks around one kernel (recorded into the graph when capturing)
// While the stream is being captured the record becomes an event-record node
// of the graph (cudaEventRecordExternal); otherwise it is a plain record.
cudaError_t record(trax_ctx* c, cudaEvent_t ev) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(c->st, &cs);
  if (e != cudaSuccess) return e;
  if (cs == cudaStreamCaptureStatusActive) return cudaEventRecordWithFlags(ev, c->st, cudaEventRecordExternal);
  return cudaEventRecord(ev, c->st);
}

void kmark(trax_ctx* c, int k, bool end) {
  record(c, c->kEv[2 * k + (end ? 1 : 0)]);
  if (end) c->kUsed[k] = true;
}
#define KBEG(k) kmark(c, k, false)
#define KEND(k) kmark(c, k, true)
uint32_t* dev_err(trax_ctx* c) { return slot(c, S_ERR); }

float min_radius_curvature(float minPt) {
  // TripletConfiguration.cpp:36-43: minRadiusCurvature(minPt, Bz) takes Bz as
  // a float, so the double IDEAL_BZ = 3.8112 (TripletConfiguration.h:56-70) is
  // rounded to float before the double arithmetic.
  const double IDEAL_BZ = 3.8112;
  const float Bz = (float)IDEAL_BZ;
  const double Q = 1.602177E-19;
  const double GEV_C = 5.344286E-19;
  return (float)(minPt * GEV_C / (Bz * Q) * 1E2);
}

// Device configuration from the host-side settings.  The grid build needs
// only the grid and the hits; the seeding stages (`seeding`) also need the
// layer triplets and the geometry.
int build_config(trax_ctx* c, bool seeding = true) {
  if (!c->haveGrid || !c->haveHits) return fail(c, TRAX_ERR_STATE, "grid and hits must be set first");
  if (seeding && (!c->haveLT || !c->haveGeom))
    return fail(c, TRAX_ERR_STATE, "layer triplets, geometry, grid and hits must be set first");
  DevConfig& g = c->cfg;
  memset(&g, 0, sizeof(g));
  g.E = c->E;
  g.L = c->L;
  g.nZ = c->nZ;
  g.nP = c->nP;
  g.C = (c->nZ + 1) * (c->nP + 1);
  g.nLT = c->haveLT ? (uint32_t)c->lts.size() : 0u;
  // Grid.h:9-15, 33-37 (float arithmetic on the host)
  const float MIN_Z = -300.0f, MAX_Z = 300.0f;
  const float MIN_PHI = (float)-3.14159265358979323846, MAX_PHI = (float)3.14159265358979323846;
  g.minZ = MIN_Z;
  g.sZ = (MAX_Z - MIN_Z) / (float)c->nZ;
  g.minPhi = MIN_PHI;
  g.sP = (MAX_PHI - MIN_PHI) / (float)c->nP;
  g.minRcurv = min_radius_curvature(c->minPt);
  g.dEtaCut = c->dEtaCut;
  g.pairThreads = c->pairThreads;
  g.predThreads = c->predThreads;
  g.filterThreads = c->filterThreads;
  g.predPairsPerThread = c->predK;
  g.predKeep = c->keepSlots ? c->keepSlots : c->keepAuto;
  g.fineRows = c->fineRows;
  g.fineC = c->fineRows ? (c->fineRows * c->nZ + 1) * (c->nP + 1) : 0u;
  g.fineScale = c->fineRows ? (float)c->fineRows / g.sZ : 0.0f;
  g.nHits = (uint32_t)c->nHits;
  g.err = slot(c, S_ERR);
  for (uint32_t p = 0; p < g.nLT; ++p) {
    const trax_layer_triplet& t = c->lts[p];
    if (t.layer1 < 1 || t.layer2 < 1 || t.layer3 < 1 || t.layer1 > c->L || t.layer2 > c->L || t.layer3 > c->L)
      return fail(c, TRAX_ERR_ARG, "layer triplet refers to a layer outside the uploaded layers");
    g.layer1[p] = t.layer1;
    g.layer2[p] = t.layer2;
    g.layer3[p] = t.layer3;
    g.dThetaCut[p] = t.dtheta_cut;
    g.sigmaZ[p] = t.sigma_z;
    g.dPhiCut[p] = t.dphi_cut;
    dphi_tan_bounds(t.dphi_cut, g.dPhiTanLo[p], g.dPhiTanHi[p]);
    g.sigmaPhi[p] = t.sigma_phi;
    g.tipCut[p] = t.tip_cut;
    g.z0[p] = t.z0;
    float sp;  // Q1: pairSpreadPhi (uint) bound to the float* sigmaPhi parameter
    memcpy(&sp, &t.pair_spread_phi, 4);
    g.pairSigmaPhi[p] = sp;
  }
  c->cfgDirty = !(c->haveLT && c->haveGeom);
  if (!c->haveGeom) return TRAX_OK;
  if (c->minR.size() < c->L) return fail(c, TRAX_ERR_ARG, "geometry has fewer layers than the hits");
  const float twoR = 2 * g.minRcurv;
  for (uint32_t l = 0; l < c->L; ++l) {
    g.minR[l] = c->minR[l];
    g.maxR[l] = c->maxR[l];
    g.acosMinR[l] = trax::acos_(trax::div_(g.minR[l], twoR));
    g.acosMaxR[l] = trax::acos_(trax::div_(g.maxR[l], twoR));
  }
  return TRAX_OK;
}

// read all slots (error word, counters, totals) in one copy
int read_slots(trax_ctx* c) {
  CK(cudaMemcpyAsync(c->hSlots, c->slots.p, sizeof(uint32_t) * S_N, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return TRAX_OK;
}

int error_from_bits(trax_ctx* c, uint32_t bits);

// a stage total read by the host in SYNCED mode; the error word comes along so
// that an overflowed or timed-out scan stops the chain before its total is used
int read_slot(trax_ctx* c, int k, uint64_t* out) {
  CK(cudaMemcpyAsync(c->hSlots + k, slot(c, k), sizeof(uint32_t), cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(c->hSlots + S_ERR, slot(c, S_ERR), sizeof(uint32_t), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  *out = c->hSlots[k];
  return error_from_bits(c, c->hSlots[S_ERR] & (TRAX_EBIT_OVERFLOW | TRAX_EBIT_TIMEOUT));
}

int error_from_bits(trax_ctx* c, uint32_t bits) {
  if (bits & TRAX_EBIT_TIMEOUT) return fail(c, TRAX_ERR_TIMEOUT, "a bounded device wait ran out");
  if (bits & TRAX_EBIT_CAPACITY) return fail(c, TRAX_ERR_CAPACITY, "a stage produced more items than its capacity");
  if (bits & TRAX_EBIT_BOUNDS) return fail(c, TRAX_ERR_DEVICE_ASSERT, "a device-side bounds check fired");
  if (bits & TRAX_EBIT_OVERFLOW)
    return fail(c, TRAX_ERR_CAPACITY, "a stage's item count does not fit the 32-bit index space");
  return TRAX_OK;
}

int check_device_error(trax_ctx* c) {
  RC(read_slots(c));
  c->pairSent = c->hSlots[S_PAIR_SENT];
  c->candSent = c->hSlots[S_CAND_SENT];
  return error_from_bits(c, c->hSlots[S_ERR]);
}

// Buffer holding n elements of sz bytes: allocated in SYNCED mode, checked in DEVICE mode.
#define ENSURE(buf, n, sz)                                                      \
  do {                                                                          \
    if (mode == SYNCED) CK(ensure(c, c->buf, (size_t)(n) * (sz)));              \
    else if ((size_t)(n) * (sz) > c->buf.cap)                                   \
      return fail(c, TRAX_ERR_STATE, "device-mode buffer " #buf " too small");  \
  } while (0)

// exclusive scan of (count + 1) elements in place, count = nHost or *nDev;
// the total is published into slot `dst` (clamped to cap)
int scan_publish(trax_ctx* c, Mode mode, uint32_t* data, uint64_t nHost, const uint32_t* nDev, uint64_t maxCount,
                 int dst, uint64_t cap) {
  const uint64_t maxN = maxCount + 1;
  if (mode == SYNCED) CK(ensure(c, c->scanScratch, scan_scratch_bytes(maxN)));
  else if (scan_scratch_bytes(maxN) > c->scanScratch.cap)
    return fail(c, TRAX_ERR_STATE, "device-mode scan scratch too small");
  CK(scan_exclusive(data, data, nHost + 1, nDev, 1, maxN, c->scanScratch.p, dev_err(c), c->st, &c->launches,
                    true, c->wait));
  CK(publish_total(data, nDev, nHost, cap, slot(c, dst), dev_err(c), c->st, &c->launches));
  return TRAX_OK;
}

// ------------------------------------------------------------------ stages
int stage_grid(trax_ctx* c, Mode mode) {
  NvtxRange nvtx("trax.grid");
  const uint64_t n = c->nHits;
  const uint64_t cells = (uint64_t)c->E * c->L * c->cfg.C;
  ENSURE(grid, cells, 4);
  ENSURE(px, n, 4); ENSURE(py, n, 4); ENSURE(pz, n, 4);
  ENSURE(player, n, 4); ENSURE(pdet, n, 4); ENSURE(phid, n, 4); ENSURE(pevt, n, 4); ENSURE(porig, n, 4);
  ENSURE(pxyzp, n, 16);
  ENSURE(sc_cell, n, 4); ENSURE(sc_phi, n, 4); ENSURE(sc_perm, n, 4);
  uint64_t counters = c->cfg.C > TRAX_GRID_SMEM_CELLS ? cells : 0;
  if (fine_counter_cells(c->cfg) > counters) counters = fine_counter_cells(c->cfg);
  if (counters) ENSURE(sc_counts, counters, 4);
  if (c->cfg.fineRows) {
    ENSURE(fineGrid, (uint64_t)c->E * c->L * c->cfg.fineC, 4);
    ENSURE(fineHits, n, 16);
  } else if (mode == SYNCED && (c->fineGrid.p || c->fineHits.p)) {  // switched off: give its memory back
    release(c->fineGrid);
    release(c->fineHits);
    c->bufGeneration++;  // a captured graph that wrote them must not be replayed
  }
  GridInput in;
  in.x = ptr<float>(c->in_x);
  in.y = ptr<float>(c->in_y);
  in.z = ptr<float>(c->in_z);
  in.layer = ptr<uint32_t>(c->in_layer);
  in.det = ptr<uint32_t>(c->in_det);
  in.hid = ptr<uint32_t>(c->in_hid);
  in.evt = ptr<uint32_t>(c->in_evt);
  in.eventOffsets = ptr<uint32_t>(c->evOff);
  in.layerHits = ptr<uint32_t>(c->layHits);
  in.layerOffsets = ptr<uint32_t>(c->layOff);
  GridScratch sc;
  sc.cell = ptr<uint32_t>(c->sc_cell);
  sc.phi = ptr<float>(c->sc_phi);
  sc.perm = ptr<uint32_t>(c->sc_perm);
  sc.counts = ptr<uint32_t>(c->sc_counts);
  KBEG(TK_GRID);
  CK(grid_build(c->cfg, in, ptr<uint32_t>(c->grid), dev_hits(c), sc, c->maxLayerHits, dev_err(c), c->st,
                &c->launches));
  CK(fine_grid_build(c->cfg, ptr<uint32_t>(c->grid), ptr<float4>(c->pxyzp), fine_buffers(c), sc.counts, c->st,
                     &c->launches));
  c->fineBuilt = c->cfg.fineRows;
  KEND(TK_GRID);
  return TRAX_OK;
}

int stage_pairs(trax_ctx* c, Mode mode) {
  NvtxRange nvtx("trax.pairs");
  const uint32_t S = c->cfg.E * c->cfg.nLT;
  ENSURE(segOuter, S + 1, 4);
  ENSURE(taskBase, S + 1, 4);
  ENSURE(pairOffsets, S + 1, 4);
  uint32_t* taskBase = ptr<uint32_t>(c->taskBase);
  CK(pair_segments(c->cfg, ptr<uint32_t>(c->grid), ptr<uint32_t>(c->segOuter), taskBase, c->st, &c->launches));
  RC(scan_publish(c, mode, taskBase, S, nullptr, S, S_TASKS, mode == DEVICE ? c->capTasks : NO_CAP));
  const uint32_t* nTasksDev = slot(c, S_TASKS);
  uint64_t maxTasks = c->capTasks;
  if (mode == SYNCED) {
    RC(read_slot(c, S_TASKS, &c->nTasks));
    maxTasks = c->nTasks;
  }
  ENSURE(taskCount, maxTasks + 1, 4);
  ENSURE(taskState, pair_task_state_bytes(maxTasks) + 16, 1);
  uint32_t* taskCount = ptr<uint32_t>(c->taskCount);
  const PairTaskState taskState = pair_task_state(c->taskState.p, maxTasks);
  KBEG(TK_PAIR_COUNT);
  CK(pair_tasks(c->cfg, false, ptr<uint32_t>(c->grid), dev_hits(c), ptr<uint32_t>(c->segOuter), taskBase, nTasksDev,
                maxTasks, taskCount, taskState, nullptr, 0, slot(c, S_PAIR_SENT), dev_err(c), c->st,
                &c->launches));
  KEND(TK_PAIR_COUNT);
  RC(scan_publish(c, mode, taskCount, c->nTasks, mode == DEVICE ? nTasksDev : nullptr, maxTasks, S_PAIRS,
                  mode == DEVICE ? c->capPairs : NO_CAP));
  uint64_t maxPairs = c->capPairs;
  if (mode == SYNCED) {
    RC(read_slot(c, S_PAIRS, &c->nPairs));
    maxPairs = c->nPairs;
  }
  ENSURE(pairs, maxPairs, 8);
  KBEG(TK_PAIR_EMIT);
  CK(pair_tasks(c->cfg, true, ptr<uint32_t>(c->grid), dev_hits(c), ptr<uint32_t>(c->segOuter), taskBase, nTasksDev,
                maxTasks, taskCount, taskState, ptr<uint2>(c->pairs), maxPairs, slot(c, S_PAIR_SENT), dev_err(c),
                c->st, &c->launches));
  KEND(TK_PAIR_EMIT);
  CK(pair_offsets(c->cfg, taskBase, taskCount, ptr<uint32_t>(c->pairOffsets), c->st, &c->launches));
  return TRAX_OK;
}

int stage_predict(trax_ctx* c, Mode mode) {
  NvtxRange nvtx("trax.predict");
  const uint32_t S = c->cfg.E * c->cfg.nLT;
  const uint32_t* nPairsDev = slot(c, S_PAIRS);
  const uint64_t maxPairs = mode == SYNCED ? c->nPairs : c->capPairs;
  const uint64_t maxWarps = (maxPairs + 31) / 32;
  // per pair the offset of its candidates within its warp of 32 pairs, per
  // warp the candidates' sum (scanned into the warp's first position)
  ENSURE(candLocal, maxPairs + 1, 4);
  ENSURE(predWarps, maxWarps + 1, 4);
  ENSURE(predKeep, pred_keep_words(maxPairs, c->cfg.predKeep), 4);
  ENSURE(candOffsets, S + 1, 4);
  uint32_t* candLocal = ptr<uint32_t>(c->candLocal);
  uint32_t* warpSums = ptr<uint32_t>(c->predWarps);
  KBEG(TK_PRED_COUNT);
  CK(predict_pairs(c->cfg, false, ptr<uint32_t>(c->grid), dev_hits(c), ptr<uint2>(c->pairs), nPairsDev, maxPairs,
                   candLocal, warpSums, slot(c, S_PRED_WARPS), ptr<uint32_t>(c->predKeep), nullptr, 0,
                   slot(c, S_CAND_SENT), dev_err(c), c->st, &c->launches, fine_grid(c)));
  KEND(TK_PRED_COUNT);
  // the prefix sum runs over the per-warp sums of the counts
  RC(scan_publish(c, mode, warpSums, (c->nPairs + 31) / 32, mode == DEVICE ? slot(c, S_PRED_WARPS) : nullptr,
                  maxWarps, S_CANDS, mode == DEVICE ? c->capCands : NO_CAP));
  uint64_t maxCands = c->capCands;
  if (mode == SYNCED) {
    RC(read_slot(c, S_CANDS, &c->nCands));
    maxCands = c->nCands;
  }
  ENSURE(cands, maxCands, 8);
  KBEG(TK_PRED_EMIT);
  CK(predict_pairs(c->cfg, true, ptr<uint32_t>(c->grid), dev_hits(c), ptr<uint2>(c->pairs), nPairsDev, maxPairs,
                   candLocal, warpSums, nullptr, ptr<uint32_t>(c->predKeep), ptr<uint2>(c->cands), maxCands,
                   slot(c, S_CAND_SENT), dev_err(c), c->st, &c->launches, fine_grid(c)));
  KEND(TK_PRED_EMIT);
  CK(predict_offsets(c->cfg, ptr<uint32_t>(c->pairOffsets), nPairsDev, candLocal, warpSums,
                     ptr<uint32_t>(c->candOffsets), c->st, &c->launches));
  return TRAX_OK;
}

int stage_filter(trax_ctx* c, Mode mode) {
  NvtxRange nvtx("trax.filter");
  const uint32_t S = c->cfg.E * c->cfg.nLT;
  const uint32_t* nCandsDev = slot(c, S_CANDS);
  const uint64_t maxCands = mode == SYNCED ? c->nCands : c->capCands;
  const uint64_t maxWords = (maxCands + 31) / 32;
  ENSURE(flagWords, maxWords + 1, 4);
  ENSURE(flagSums, maxWords + 1, 4);
  ENSURE(tripOffsets, S + 1, 4);
  uint32_t* words = ptr<uint32_t>(c->flagWords);
  uint32_t* sums = ptr<uint32_t>(c->flagSums);
  KBEG(TK_FILTER);
  CK(filter_candidates(c->cfg, dev_hits(c), ptr<uint2>(c->pairs), ptr<uint2>(c->cands), nCandsDev, maxCands, words,
                       sums, slot(c, S_FLAG_WORDS), c->st, &c->launches));
  KEND(TK_FILTER);
  // the prefix sum runs over the numbers of flags per word of 32 candidates
  RC(scan_publish(c, mode, sums, (c->nCands + 31) / 32, mode == DEVICE ? slot(c, S_FLAG_WORDS) : nullptr, maxWords,
                  S_TRIPLETS, mode == DEVICE ? c->capT : NO_CAP));
  uint64_t maxT = c->capT;
  if (mode == SYNCED) {
    RC(read_slot(c, S_TRIPLETS, &c->nT));
    maxT = c->nT;
  }
  ENSURE(h1, maxT, 4);
  ENSURE(h2, maxT, 4);
  ENSURE(h3, maxT, 4);
  KBEG(TK_FILTER_STORE);
  CK(filter_store(ptr<uint2>(c->pairs), ptr<uint2>(c->cands), nCandsDev, maxCands, words, sums, ptr<uint32_t>(c->h1),
                  ptr<uint32_t>(c->h2), ptr<uint32_t>(c->h3), maxT, c->st, &c->launches));
  KEND(TK_FILTER_STORE);
  CK(triplet_offsets(c->cfg, dev_hits(c), ptr<uint32_t>(c->h1), slot(c, S_TRIPLETS), maxT,
                     ptr<uint32_t>(c->tripOffsets), c->st, &c->launches));
  return TRAX_OK;
}

TripletView triplets(trax_ctx* c, uint64_t maxT) {
  TripletView t;
  t.h1 = ptr<uint32_t>(c->h1);
  t.h2 = ptr<uint32_t>(c->h2);
  t.h3 = ptr<uint32_t>(c->h3);
  t.nDev = slot(c, S_TRIPLETS);
  t.maxN = maxT;
  return t;
}

int stage_connectivity(trax_ctx* c, Mode mode) {
  NvtxRange nvtx("trax.connectivity");
  const uint32_t S = c->cfg.E * c->cfg.nLT;
  const uint64_t maxT = mode == SYNCED ? c->nT : c->capT;
  const uint32_t* nTDev = slot(c, S_TRIPLETS);
  if (mode == SYNCED) {
    c->nLinks = c->nConn = c->nNonConn = c->nTracks = 0;
    c->noLinks = true;
  }
  ENSURE(eta, maxT, 4);
  ENSURE(segOf, maxT, 4);
  ENSURE(segStart, S + 1, 4);
  ENSURE(linkCount, maxT + 1, 4);
  ENSURE(linkRun, maxT + 1, 4);
  ENSURE(cflags, maxT + 1, 4);
  const uint64_t maxTW = (maxT + 31) / 32;
  ENSURE(connS, maxTW + 1, 4);
  ENSURE(nonConnS, maxTW + 1, 4);
  ENSURE(connW, maxTW + 1, 4);
  ENSURE(nonConnW, maxTW + 1, 4);
  ENSURE(connIdx, maxT, 4);
  ENSURE(nonConnIdx, maxT, 4);
  TripletView tv = triplets(c, maxT);
  CK(cudaMemsetAsync(c->cflags.p, 0, (size_t)(maxT + 1) * 4, c->st));
  CK(triplet_eta(c->cfg, dev_hits(c), tv, ptr<float>(c->eta), ptr<uint32_t>(c->segOf), c->st, &c->launches));
  CK(segment_bounds(c->cfg, ptr<uint32_t>(c->segOf), nTDev, ptr<uint32_t>(c->segStart), c->st, &c->launches));
  uint32_t* linkCount = ptr<uint32_t>(c->linkCount);
  KBEG(TK_CONN_COUNT);
  CK(connectivity_tasks(c->cfg, false, dev_hits(c), tv, ptr<float>(c->eta), ptr<uint32_t>(c->tripOffsets),
                        ptr<uint32_t>(c->segStart), linkCount, ptr<uint32_t>(c->cflags), ptr<uint32_t>(c->linkRun),
                        nullptr, nullptr, 0, c->sortedSegments, c->st, &c->launches));
  KEND(TK_CONN_COUNT);
  RC(scan_publish(c, mode, linkCount, c->nT, mode == DEVICE ? nTDev : nullptr, maxT, S_LINKS,
                  mode == DEVICE ? c->capLinks : NO_CAP));
  uint64_t maxLinks = c->capLinks;
  if (mode == SYNCED) {
    RC(read_slot(c, S_LINKS, &c->nLinks));
    maxLinks = c->nLinks;
    c->noLinks = c->nLinks == 0;
    if (c->noLinks) return TRAX_OK;  // TripletConnectivityTight.cpp:127-129
  }
  ENSURE(basis, maxLinks, 4);
  ENSURE(follower, maxLinks, 4);
  KBEG(TK_CONN_EMIT);
  CK(connectivity_tasks(c->cfg, true, dev_hits(c), tv, ptr<float>(c->eta), ptr<uint32_t>(c->tripOffsets),
                        ptr<uint32_t>(c->segStart), linkCount, ptr<uint32_t>(c->cflags), ptr<uint32_t>(c->linkRun),
                        ptr<uint32_t>(c->basis), ptr<uint32_t>(c->follower), maxLinks, c->sortedSegments, c->st,
                        &c->launches));
  KEND(TK_CONN_EMIT);
  // the two Q9 streams as words of 32 flags; the scans run over the words' counts
  CK(connectable_words(ptr<uint32_t>(c->cflags), nTDev, maxT, ptr<uint32_t>(c->connW), ptr<uint32_t>(c->connS),
                       ptr<uint32_t>(c->nonConnW), ptr<uint32_t>(c->nonConnS), slot(c, S_CONN_WORDS), c->st,
                       &c->launches));
  const uint64_t nTW = (c->nT + 31) / 32;
  const uint32_t* nTWDev = mode == DEVICE ? slot(c, S_CONN_WORDS) : nullptr;
  RC(scan_publish(c, mode, ptr<uint32_t>(c->connS), nTW, nTWDev, maxTW, S_CONN, NO_CAP));
  RC(scan_publish(c, mode, ptr<uint32_t>(c->nonConnS), nTW, nTWDev, maxTW, S_NONCONN, NO_CAP));
  CK(compact_words(ptr<uint32_t>(c->connW), ptr<uint32_t>(c->connS), nTDev, maxT, ptr<uint32_t>(c->connIdx), maxT,
                   c->st, &c->launches));
  CK(compact_words(ptr<uint32_t>(c->nonConnW), ptr<uint32_t>(c->nonConnS), nTDev, maxT, ptr<uint32_t>(c->nonConnIdx),
                   maxT, c->st, &c->launches));
  if (mode == SYNCED) {
    RC(read_slots(c));
    c->nConn = c->hSlots[S_CONN];
    c->nNonConn = c->hSlots[S_NONCONN];
  }
  return TRAX_OK;
}

int stage_fit(trax_ctx* c, Mode mode) {
  NvtxRange nvtx("trax.circle_fit");
  const uint64_t maxT = mode == SYNCED ? c->nT : c->capT;
  ENSURE(pt, maxT, 4);
  CK(cudaMemsetAsync(c->pt.p, 0, (size_t)std::max<uint64_t>(maxT, 1) * 4, c->st));
  if (mode == SYNCED && c->noLinks) return TRAX_OK;
  CK(circle_fit(dev_hits(c), triplets(c, maxT), ptr<uint32_t>(c->connIdx), slot(c, S_CONN), maxT, ptr<float>(c->pt),
                c->st, &c->launches));
  return TRAX_OK;
}

CABuffers ca_buffers(trax_ctx* c) {
  CABuffers b;
  b.states = ptr<uint32_t>(c->states);
  b.inStart = ptr<uint32_t>(c->inStart);
  b.inCursor = ptr<uint32_t>(c->inCursor);
  b.inList = ptr<uint32_t>(c->inList);
  b.best = ptr<uint32_t>(c->best);
  b.isBest = ptr<uint32_t>(c->isBest);
  b.handlers = ptr<uint32_t>(c->handlers);
  b.segOf = ptr<uint32_t>(c->segOf);
  return b;
}

int stage_ca(trax_ctx* c, Mode mode) {
  NvtxRange nvtx("trax.ca");
  if (mode == SYNCED && c->noLinks) {
    c->nTracks = 0;
    return TRAX_OK;
  }
  const uint64_t maxT = mode == SYNCED ? c->nT : c->capT;
  const uint64_t maxLinks = mode == SYNCED ? c->nLinks : c->capLinks;
  const uint32_t* nTDev = slot(c, S_TRIPLETS);
  const uint32_t* nLinksDev = slot(c, S_LINKS);
  ENSURE(states, maxT, 4);
  ENSURE(inStart, maxT + 1, 4);
  ENSURE(inCursor, maxT, 4);
  ENSURE(inList, maxLinks, 4);
  ENSURE(best, maxT, 4);
  ENSURE(isBest, maxT, 4);
  ENSURE(handlers, maxT + 1, 4);
  CABuffers b = ca_buffers(c);
  CK(ca_in_degree(ptr<uint32_t>(c->follower), nLinksDev, maxLinks, b, nTDev, maxT, c->st, &c->launches));
  // in-degree prefix (its total is the number of links; not published)
  if (mode == SYNCED) CK(ensure(c, c->scanScratch, scan_scratch_bytes(maxT + 1)));
  CK(scan_exclusive(b.inStart, b.inStart, c->nT + 1, mode == DEVICE ? nTDev : nullptr, 1, maxT + 1,
                    c->scanScratch.p, dev_err(c), c->st, &c->launches, true, c->wait));
  CK(ca_fill(ptr<uint32_t>(c->basis), ptr<uint32_t>(c->follower), nLinksDev, maxLinks, b, nTDev, maxT, c->st,
             &c->launches));
  CK(ca_forward(c->cfg, b, nTDev, maxT, c->st, &c->launches));
  CK(ca_backward(ptr<float>(c->pt), b, nTDev, maxT, nLinksDev, c->st, &c->launches));
  RC(scan_publish(c, mode, b.handlers, c->nT, mode == DEVICE ? nTDev : nullptr, maxT, S_TRACKS,
                  mode == DEVICE ? c->capTracks : NO_CAP));
  uint64_t maxTracks = c->capTracks;
  if (mode == SYNCED) {
    RC(read_slot(c, S_TRACKS, &c->nTracks));
    maxTracks = c->nTracks;
  }
  ENSURE(tracks, maxTracks, 4);
  CK(ca_tracks(b, nTDev, maxT, ptr<uint32_t>(c->tracks), maxTracks, dev_err(c), c->st, &c->launches));
  return TRAX_OK;
}

int begin_run(trax_ctx* c, bool seeding) {
  RC(build_config(c, seeding));
  c->sortedSegments = true;
  c->identityHits = false;
  CK(cudaSetDevice(c->device));
  CK(cudaMemsetAsync(c->slots.p, 0, sizeof(uint32_t) * S_N, c->st));
  return TRAX_OK;
}

int run_stage(trax_ctx* c, int stage) {
  if (stage > 1 && c->stage < stage - 1) return fail(c, TRAX_ERR_STATE, "the previous stage has not run");
  if (stage > 1 && c->cfgDirty) RC(build_config(c, true));  // layer triplets or geometry set after the grid
  int rc = TRAX_OK;
  if (stage == 1) {
    for (bool& u : c->stageUsed) u = false;
    for (bool& u : c->kUsed) u = false;
  }
  cudaEventRecord(c->stageEv[stage - 1], c->st);
  switch (stage) {
    case 1: rc = begin_run(c, false); if (!rc) rc = stage_grid(c, SYNCED); break;
    case 2: rc = stage_pairs(c, SYNCED); break;
    case 3: rc = stage_predict(c, SYNCED); break;
    case 4: rc = stage_filter(c, SYNCED); break;
    case 5: rc = stage_connectivity(c, SYNCED); break;
    case 6: rc = stage_fit(c, SYNCED); break;
    case 7: rc = stage_ca(c, SYNCED); break;
    default: return fail(c, TRAX_ERR_ARG, "unknown stage");
  }
  if (rc) return rc;
  cudaEventRecord(c->stageEv[stage], c->st);
  c->stageUsed[stage - 1] = true;
  RC(check_device_error(c));
  c->stage = stage;
  if (stage == 4) ++c->tripGen;
  if (stage == 6) c->ptGen = c->tripGen;
  if (stage == 7) c->caGen = c->tripGen;
  c->caOnly = false;
  return TRAX_OK;
}

int chain_device(trax_ctx* c, bool linking) {
  for (bool& u : c->stageUsed) u = false;
  for (bool& u : c->kUsed) u = false;
  int (*stages[N_STAGES])(trax_ctx*, Mode) = {stage_grid, stage_pairs, stage_predict, stage_filter,
                                              stage_connectivity, stage_fit, stage_ca};
  const int n = linking ? N_STAGES : 4;
  CK(record(c, c->stageEv[0]));
  for (int s = 0; s < n; ++s) {
    RC(stages[s](c, DEVICE));
    CK(record(c, c->stageEv[s + 1]));
    c->stageUsed[s] = true;
  }
  return TRAX_OK;
}

uint64_t with_headroom(uint64_t n) { return n + n / 4 + 4096; }

// Size every buffer for DEVICE mode from the sizes of the last SYNCED run.
int size_device_buffers(trax_ctx* c) {
  const Mode mode = SYNCED;
  c->capTasks = with_headroom(c->nTasks);
  c->capPairs = with_headroom(c->nPairs);
  c->capCands = with_headroom(c->nCands);
  c->capT = with_headroom(c->nT);
  c->capLinks = with_headroom(c->nLinks);
  c->capTracks = with_headroom(c->nTracks);
  const uint32_t S = c->cfg.E * c->cfg.nLT;
  ENSURE(taskCount, c->capTasks + 1, 4);
  ENSURE(taskState, pair_task_state_bytes(c->capTasks) + 16, 1);
  ENSURE(pairs, c->capPairs, 8);
  ENSURE(candLocal, c->capPairs + 1, 4);
  ENSURE(predWarps, (c->capPairs + 31) / 32 + 1, 4);
  ENSURE(predKeep, pred_keep_words(c->capPairs, c->cfg.predKeep), 4);
  ENSURE(cands, c->capCands, 8);
  ENSURE(flagWords, (c->capCands + 31) / 32 + 1, 4);
  ENSURE(flagSums, (c->capCands + 31) / 32 + 1, 4);
  ENSURE(h1, c->capT, 4); ENSURE(h2, c->capT, 4); ENSURE(h3, c->capT, 4);
  ENSURE(eta, c->capT, 4); ENSURE(segOf, c->capT, 4); ENSURE(segStart, S + 1, 4);
  ENSURE(linkCount, c->capT + 1, 4); ENSURE(linkRun, c->capT + 1, 4); ENSURE(cflags, c->capT + 1, 4);
  ENSURE(connS, (c->capT + 31) / 32 + 1, 4); ENSURE(nonConnS, (c->capT + 31) / 32 + 1, 4);
  ENSURE(connW, (c->capT + 31) / 32 + 1, 4); ENSURE(nonConnW, (c->capT + 31) / 32 + 1, 4);
  ENSURE(connIdx, c->capT, 4); ENSURE(nonConnIdx, c->capT, 4); ENSURE(pt, c->capT, 4);
  ENSURE(basis, c->capLinks, 4); ENSURE(follower, c->capLinks, 4);
  ENSURE(states, c->capT, 4); ENSURE(inStart, c->capT + 1, 4); ENSURE(inCursor, c->capT, 4);
  ENSURE(inList, c->capLinks, 4); ENSURE(best, c->capT, 4); ENSURE(isBest, c->capT, 4);
  ENSURE(handlers, c->capT + 1, 4); ENSURE(tracks, c->capTracks, 4);
  uint64_t maxScan = std::max({c->capTasks, c->capPairs, c->capCands, c->capT, (uint64_t)S}) + 1;
  CK(ensure(c, c->scanScratch, scan_scratch_bytes(maxScan)));
  return TRAX_OK;
}

void drop_graph(trax_ctx* c) {
  if (c->graphExec) cudaGraphExecDestroy(c->graphExec);
  if (c->graph) cudaGraphDestroy(c->graph);
  c->graphExec = nullptr;
  c->graph = nullptr;
  c->graphKey = 0;
}

// Candidates captured per pair when the caller leaves the choice to the
// library, from the mean candidates per pair m of the calibrated batch: 4
// up to m = 1, 8 up to 2.5, 16 up to 6, else 32.  More slots spare the
// store pass its re-walks of pairs with more candidates, and spread the
// captures of pairs with few over more sectors.  On GB300, at m = 0.5 (1000
// ttbar-like events) 4 slots are fastest (16: prediction store 0.47 ->
// 0.65 ms); at m = 4.2 (16 pileup events) 16 slots take the prediction
// store from 14.8 to 4.3 ms and the chain from 50.6 to 40.4 ms.
uint32_t auto_keep_slots(uint64_t nCands, uint64_t nPairs) {
  if (nPairs == 0 || nCands <= nPairs) return 4u;
  if (2 * nCands <= 5 * nPairs) return 8u;
  if (nCands <= 6 * nPairs) return 16u;
  return 32u;
}

uint64_t shape_key(trax_ctx* c, bool linking) {
  uint64_t k = 1469598103934665603ull;
  auto mix = [&k](uint64_t v) {
    k ^= v;
    k *= 1099511628211ull;
  };
  mix(c->E); mix(c->L); mix(c->nHits); mix(c->cfg.C); mix(c->cfg.nLT); mix(linking ? 1 : 0);
  mix(c->maxLayerHits > 0xffffu ? 1 : 0);  // the grid build's 16-bit counters hold layers below 65 536 hits
  mix(c->bufGeneration); mix(c->capTasks); mix(c->capPairs); mix(c->capCands); mix(c->capT); mix(c->capLinks);
  mix(c->capTracks);
  mix(c->wait.spinLimit); mix(c->wait.skipTile);  // captured into the scans' launch arguments
  const unsigned char* b = reinterpret_cast<const unsigned char*>(&c->cfg);
  for (size_t i = 0; i < sizeof(DevConfig); ++i) mix(b[i]);
  return k;
}

}  // namespace

namespace trax {

// Hash of what determines the best launch shape: batch shape, layer
// triplets, geometry and minimum pT (not the grid or block sizes).
uint64_t workload_hash(const trax_ctx* c) {
  uint64_t k = 1469598103934665603ull;
  auto mix = [&k](const void* p, size_t n) {
    const unsigned char* b = static_cast<const unsigned char*>(p);
    for (size_t i = 0; i < n; ++i) {
      k ^= b[i];
      k *= 1099511628211ull;
    }
  };
  mix(&c->E, sizeof(c->E));
  mix(&c->L, sizeof(c->L));
  mix(&c->nHits, sizeof(c->nHits));
  mix(&c->minPt, sizeof(c->minPt));
  if (!c->lts.empty()) mix(c->lts.data(), c->lts.size() * sizeof(trax_layer_triplet));
  if (!c->minR.empty()) mix(c->minR.data(), c->minR.size() * sizeof(float));
  if (!c->maxR.empty()) mix(c->maxR.data(), c->maxR.size() * sizeof(float));
  return k;
}

int ctx_device(const trax_ctx* c) { return c->device; }

bool ctx_ready(const trax_ctx* c) { return c->haveLT && c->haveGeom && c->haveGrid && c->haveHits; }

void ctx_set_error(trax_ctx* c, const char* msg) { c->err = msg; }

}  // namespace trax

namespace {

int run_synced_chain(trax_ctx* c, bool linking) {
  for (int s = 1; s <= (linking ? 7 : 4); ++s) RC(run_stage(c, s));
  return TRAX_OK;
}

void fill_stats(trax_ctx* c, trax_batch_stats* s) {
  if (!s) return;
  memset(s, 0, sizeof(*s));
  s->n_hits = c->nHits;
  s->n_pairs = c->nPairs;
  s->n_candidates = c->nCands;
  s->n_triplets = c->nT;
  s->n_links = c->nLinks;
  s->n_connectable = c->nConn;
  s->n_non_connectable = c->nNonConn;
  s->n_track_entries = c->nTracks;
  s->n_pair_sentinels = c->pairSent;
  s->n_candidate_sentinels = c->candSent;
  s->kernel_launches = c->launches;
  s->device_ms = c->lastMs;
  s->graph_captures = c->graphCaptures;
}

int copy_out(trax_ctx* c, void* dst, const DevBuf& src, size_t bytes) {
  if (!dst || bytes == 0) return TRAX_OK;
  CK(cudaMemcpyAsync(dst, src.p, bytes, cudaMemcpyDeviceToHost, c->st));
  return TRAX_OK;
}

// ------------------------------------------------------- differentiable fit
// per-layer corrections from double-precision shifts (dr, dz, dphi)
int fit_set_alignment(trax_ctx* c, const double* align) {
  FitConfig& f = c->fitCfg;
  for (uint32_t l = 0; l < TRAX_MAX_LAYERS; ++l) f.dr[l] = f.dz[l] = f.sn[l] = f.cm1[l] = 0.0f;
  if (!align) return TRAX_OK;
  for (uint32_t l = 0; l < c->L; ++l) {
    const double dr = align[3 * l], dz = align[3 * l + 1], dp = align[3 * l + 2];
    if (!std::isfinite(dr) || !std::isfinite(dz) || !std::isfinite(dp))
      return fail(c, TRAX_ERR_ARG, "alignment parameters must be finite");
    const double h = std::sin(0.5 * dp);
    f.dr[l] = (float)dr;
    f.dz[l] = (float)dz;
    f.sn[l] = (float)std::sin(dp);
    f.cm1[l] = (float)(-2.0 * h * h);  // cos(dphi) - 1 without cancellation
  }
  return TRAX_OK;
}

TripletView fit_triplets(trax_ctx* c) {
  TripletView t;
  t.h1 = ptr<uint32_t>(c->h1);
  t.h2 = ptr<uint32_t>(c->h2);
  t.h3 = ptr<uint32_t>(c->h3);
  t.nDev = nullptr;
  t.maxN = c->nT;
  return t;
}

int fit_check(trax_ctx* c) {
  if (!c->fitReady || c->fitTripGen != c->tripGen || c->stage < 4)
    return fail(c, TRAX_ERR_STATE, "trax_fit_prepare must run on the current triplets first");
  return TRAX_OK;
}

// chi2 and gradients at `align` into fitOut (1 + 3 L doubles); optional
// per-row parameters and grid-order hit gradients
int fit_run(trax_ctx* c, const double* align, bool grad, bool params, bool hitsGrad) {
  RC(fit_set_alignment(c, align));
  const FitConfig& f = c->fitCfg;
  CK(ensure(c, c->fitPartials, (size_t)std::max<uint32_t>(f.nBlocks, 1) * TRAX_FIT_SLOTS * sizeof(double)));
  CK(ensure(c, c->fitOut, (1 + 6 * (size_t)c->L) * sizeof(double)));
  if (params) CK(ensure(c, c->fitParams, std::max<uint64_t>(c->nFit, 1) * 16));
  double* dH = nullptr;
  if (hitsGrad) {
    CK(ensure(c, c->fitDHits, std::max<uint64_t>(c->nHits, 1) * 3 * sizeof(double)));
    CK(cudaMemsetAsync(c->fitDHits.p, 0, (size_t)c->nHits * 3 * sizeof(double), c->st));
    dH = ptr<double>(c->fitDHits);
  }
  CK(fit_eval(f, grad, dev_hits(c), fit_triplets(c), ptr<uint32_t>(c->fitRows), ptr<double>(c->fitPartials),
              params ? ptr<float>(c->fitParams) : nullptr, dH, c->st, &c->launches));
  CK(fit_reduce(f, ptr<double>(c->fitPartials), ptr<double>(c->fitOut), c->st, &c->launches));
  return TRAX_OK;
}

}  // namespace

// ======================================================================= C ABI
extern "C" {

const char* trax_version(void) { return kVersion; }

int trax_create(trax_ctx** out, int device) {
  if (!out) return TRAX_ERR_ARG;
  *out = nullptr;
  trax_ctx* c = new trax_ctx();
  c->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMallocHost(&c->hSlots, sizeof(uint32_t) * 64);
  if (e == cudaSuccess) e = ensure(c, c->slots, sizeof(uint32_t) * 64);
  if (e == cudaSuccess) e = cudaMemset(c->slots.p, 0, sizeof(uint32_t) * 64);
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
  for (int i = 0; i <= N_STAGES && e == cudaSuccess; ++i) e = cudaEventCreate(&c->stageEv[i]);
  for (int i = 0; i < 2 * TK_N && e == cudaSuccess; ++i) e = cudaEventCreate(&c->kEv[i]);
  if (e == cudaSuccess) e = grid_prepare(device);
  if (e != cudaSuccess) {
    trax_destroy(c);
    return TRAX_ERR_CUDA;
  }
  *out = c;
  return TRAX_OK;
}

void trax_destroy(trax_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->st) cudaStreamSynchronize(c->st);
  drop_graph(c);
  DevBuf* bufs[] = {&c->in_x, &c->in_y, &c->in_z, &c->in_layer, &c->in_det, &c->in_hid, &c->in_evt, &c->evOff,
                    &c->layHits, &c->layOff, &c->raw_x, &c->raw_y, &c->raw_z, &c->raw_layer, &c->raw_det,
                    &c->raw_tid, &c->raw_key, &c->raw_off, &c->raw_scratchOff, &c->raw_scratch, &c->phys_findOff,
                    &c->phys_findIds, &c->phys_flags, &c->phys_counts, &c->trk_isTrack, &c->trk_hitsOf,
                    &c->trk_start, &c->trk_size, &c->trk_real, &c->trk_firstId, &c->trk_parent, &c->trk_compSize,
                    &c->trk_compStart, &c->trk_cursor, &c->trk_members, &c->trk_filtered, &c->trk_hits,
                    &c->trk_entryTrack, &c->trk_owner, &c->trk_table, &c->trk_counts, &c->grid, &c->px, &c->py, &c->pz, &c->player, &c->pdet, &c->phid,
                    &c->pevt, &c->porig, &c->pxyzp, &c->sc_cell, &c->sc_phi, &c->sc_perm, &c->sc_counts,
                    &c->fineGrid, &c->fineHits, &c->segOuter, &c->taskBase, &c->taskCount, &c->taskState, &c->pairs, &c->pairOffsets, &c->candLocal, &c->predWarps, &c->predKeep, &c->cands,
                    &c->candOffsets, &c->flagWords, &c->flagSums, &c->h1, &c->h2, &c->h3, &c->tripOffsets, &c->eta, &c->segOf,
                    &c->segStart, &c->linkCount, &c->linkRun, &c->cflags, &c->basis, &c->follower, &c->connS, &c->nonConnS, &c->connW, &c->nonConnW,
                    &c->connIdx, &c->nonConnIdx, &c->pt, &c->states, &c->inStart, &c->inCursor, &c->inList, &c->best,
                    &c->isBest, &c->handlers, &c->tracks, &c->scanScratch, &c->slots, &c->fitOk, &c->fitSegCnt,
                    &c->fitSegDelta, &c->fitRows, &c->fitPartials, &c->fitOut, &c->fitParams, &c->fitDHits,
                    &c->fitDHitsF};
  for (DevBuf* b : bufs) release(*b);
  if (c->hSlots) cudaFreeHost(c->hSlots);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  for (cudaEvent_t& ev : c->stageEv)
    if (ev) cudaEventDestroy(ev);
  for (cudaEvent_t& ev : c->kEv)
    if (ev) cudaEventDestroy(ev);
  if (c->st) cudaStreamDestroy(c->st);
  delete c;
}

const char* trax_last_error(const trax_ctx* c) { return c ? c->err.c_str() : "null context"; }

int trax_set_layer_triplets(trax_ctx* c, const trax_layer_triplet* lt, int n, float min_pt) {
  if (!c || !lt || n <= 0) return fail(c, TRAX_ERR_ARG, "need at least one layer triplet");
  if (n > TRAX_MAX_LT) return fail(c, TRAX_ERR_ARG, "too many layer triplets");
  for (int p = 0; p < n; ++p) {
    if (lt[p].layer1 != (uint32_t)p + 1)
      return fail(c, TRAX_ERR_ARG, "layer triplet p must start on layer p+1 (the layer-triplet index is derived "
                                   "from the first hit's layer)");
    if (lt[p].layer2 <= lt[p].layer1 || lt[p].layer3 <= lt[p].layer2)
      return fail(c, TRAX_ERR_ARG, "layer triplets must run outwards (layer1 < layer2 < layer3)");
  }
  c->lts.assign(lt, lt + n);
  c->minPt = min_pt;
  c->haveLT = true;
  c->stage = c->identityHits ? 0 : std::min(c->stage, 1);  // a built grid stays valid
  c->cfgDirty = true;
  return TRAX_OK;
}

int trax_set_geometry(trax_ctx* c, const float* min_r, const float* max_r, int n_layers) {
  if (!c || !min_r || !max_r || n_layers <= 0 || n_layers > TRAX_MAX_LAYERS)
    return fail(c, TRAX_ERR_ARG, "invalid geometry");
  c->minR.assign(min_r, min_r + n_layers);
  c->maxR.assign(max_r, max_r + n_layers);
  c->haveGeom = true;
  c->stage = c->identityHits ? 0 : std::min(c->stage, 1);  // a built grid stays valid
  c->cfgDirty = true;
  return TRAX_OK;
}

int trax_set_grid(trax_ctx* c, uint32_t n_z, uint32_t n_phi) {
  if (!c || n_z == 0 || n_phi == 0) return fail(c, TRAX_ERR_ARG, "grid needs at least one z and one phi sector");
  if ((uint64_t)(n_z + 1) * (n_phi + 1) > (1u << 22)) return fail(c, TRAX_ERR_ARG, "grid too large");
  c->nZ = n_z;
  c->nP = n_phi;
  c->haveGrid = true;
  c->stage = 0;
  return TRAX_OK;
}

void* trax_host_alloc(size_t bytes) {
  void* p = nullptr;
  if (cudaHostAlloc(&p, bytes ? bytes : 1, cudaHostAllocDefault) != cudaSuccess) return nullptr;
  return p;
}

void trax_host_free(void* p) {
  if (p) cudaFreeHost(p);
}

int trax_set_block_sizes(trax_ctx* c, uint32_t pair_threads, uint32_t predict_threads, uint32_t filter_threads) {
  if (!c) return TRAX_ERR_ARG;
  for (uint32_t t : {pair_threads, predict_threads, filter_threads})
    if (t < 32 || t > TRAX_MAX_TUNED_THREADS || t % 32)
      return fail(c, TRAX_ERR_ARG, "block sizes must be multiples of 32 in [32, 256]");
  c->pairThreads = pair_threads;
  c->predThreads = predict_threads;
  c->filterThreads = filter_threads;
  return TRAX_OK;
}

int trax_set_pairs_per_thread(trax_ctx* c, uint32_t k) {
  if (!c) return TRAX_ERR_ARG;
  if (k != 1 && k != 2 && k != 4) return fail(c, TRAX_ERR_ARG, "pairs per thread must be 1, 2 or 4");
  c->predK = k;
  return TRAX_OK;
}

int trax_set_candidate_slots(trax_ctx* c, uint32_t k) {
  if (!c) return TRAX_ERR_ARG;
  if (k != 0 && k != 4 && k != 8 && k != 16 && k != 32)
    return fail(c, TRAX_ERR_ARG, "candidate slots must be 0 (automatic), 4, 8, 16 or 32");
  c->keepSlots = k;
  return TRAX_OK;
}

int trax_get_candidate_slots(trax_ctx* c, uint32_t* k) {
  if (!c || !k) return TRAX_ERR_ARG;
  *k = c->keepSlots ? c->keepSlots : c->keepAuto;
  return TRAX_OK;
}

int trax_set_fine_rows(trax_ctx* c, uint32_t f) {
  if (!c) return TRAX_ERR_ARG;
  if (f != 0 && f != 2 && f != 4 && f != 8 && f != 16)
    return fail(c, TRAX_ERR_ARG, "fine rows must be 0 (none), 2, 4, 8 or 16");
  c->fineRows = f;
  return TRAX_OK;
}

int trax_get_fine_rows(trax_ctx* c, uint32_t* f) {
  if (!c || !f) return TRAX_ERR_ARG;
  *f = c->fineRows;
  return TRAX_OK;
}

int trax_get_pairs_per_thread(trax_ctx* c, uint32_t* k) {
  if (!c || !k) return TRAX_ERR_ARG;
  *k = c->predK;
  return TRAX_OK;
}

int trax_get_launch_config(trax_ctx* c, uint32_t* out5) {
  if (!c || !out5) return TRAX_ERR_ARG;
  out5[0] = c->nZ;
  out5[1] = c->nP;
  out5[2] = c->pairThreads;
  out5[3] = c->predThreads;
  out5[4] = c->filterThreads;
  return TRAX_OK;
}

int trax_upload_hits(trax_ctx* c, const trax_hits_soa* h, uint32_t n_hits, const uint32_t* event_offsets,
                     const uint32_t* layer_hits, const uint32_t* layer_offsets, uint32_t n_events,
                     uint32_t n_layers) {
  if (!c || !h || !event_offsets || !layer_hits || !layer_offsets) return fail(c, TRAX_ERR_ARG, "null argument");
  if (n_layers == 0 || n_layers > TRAX_MAX_LAYERS) return fail(c, TRAX_ERR_ARG, "invalid number of layers");
  // the supplements must describe the hits contiguously (HitCollection.cpp:120-133)
  uint64_t pos = 0;
  uint32_t maxLayer = 0;
  for (uint32_t e = 0; e < n_events; ++e) {
    if (event_offsets[e] != pos) return fail(c, TRAX_ERR_ARG, "event offsets are not contiguous");
    uint64_t lpos = 0;
    for (uint32_t l = 0; l < n_layers; ++l) {
      const size_t k = (size_t)e * n_layers + l;
      if (layer_offsets[k] != lpos) return fail(c, TRAX_ERR_ARG, "layer offsets are not contiguous");
      lpos += layer_hits[k];
      maxLayer = std::max(maxLayer, layer_hits[k]);
    }
    pos += lpos;
  }
  if (pos != n_hits) return fail(c, TRAX_ERR_ARG, "supplements do not add up to n_hits");
  const Mode mode = SYNCED;
  const size_t n = n_hits;
  ENSURE(in_x, n, 4); ENSURE(in_y, n, 4); ENSURE(in_z, n, 4);
  ENSURE(in_layer, n, 4); ENSURE(in_det, n, 4); ENSURE(in_hid, n, 4); ENSURE(in_evt, n, 4);
  ENSURE(evOff, n_events, 4);
  ENSURE(layHits, (size_t)n_events * n_layers, 4);
  ENSURE(layOff, (size_t)n_events * n_layers, 4);
  CK(cudaMemcpyAsync(c->in_x.p, h->x, n * 4, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->in_y.p, h->y, n * 4, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->in_z.p, h->z, n * 4, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->in_layer.p, h->layer, n * 4, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->in_det.p, h->det_id, n * 4, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->in_hid.p, h->hit_id, n * 4, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->in_evt.p, h->event, n * 4, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->evOff.p, event_offsets, (size_t)n_events * 4, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->layHits.p, layer_hits, (size_t)n_events * n_layers * 4, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->layOff.p, layer_offsets, (size_t)n_events * n_layers * 4, cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  c->E = n_events;
  c->L = n_layers;
  c->nHits = n_hits;
  c->maxLayerHits = maxLayer;
  c->haveHits = true;
  c->stage = 0;
  return TRAX_OK;
}

int trax_events_upload(trax_ctx* c, const trax_event_set* events, uint64_t first, uint64_t count,
                       const trax_layer_triplet* lt, int n_lt, float min_pt, int num_tracks, int only_tracks,
                       trax_loaded_sizes* sizes, uint32_t* findable_id, uint32_t* findable_event,
                       uint64_t findable_cap) {
  if (!c || !events || !lt || !sizes) return fail(c, TRAX_ERR_ARG, "null argument");
  trax::RawEvents raw;
  if (trax::classify_events(events, first, count, lt, n_lt, min_pt, num_tracks, only_tracks, raw) != TRAX_OK)
    return fail(c, TRAX_ERR_ARG, "invalid event range, layer triplets or event size");
  const uint32_t E = (uint32_t)(raw.rawOffsets.size() - 1), L = raw.nLayers;
  if (L == 0 || L > TRAX_MAX_LAYERS) return fail(c, TRAX_ERR_ARG, "invalid number of layers");
  const Mode mode = SYNCED;
  const size_t nRaw = raw.x.size(), n = raw.nHits;
  // per event: the global sort scratch of events too large for shared memory
  std::vector<uint32_t> scratchOff(E + 1, 0);
  for (uint32_t e = 0; e < E; ++e)
    scratchOff[e + 1] = scratchOff[e] + bucket_scratch_keys(raw.rawOffsets[e + 1] - raw.rawOffsets[e]);
  ENSURE(raw_x, nRaw, 4); ENSURE(raw_y, nRaw, 4); ENSURE(raw_z, nRaw, 4);
  ENSURE(raw_layer, nRaw, 4); ENSURE(raw_det, nRaw, 4); ENSURE(raw_tid, nRaw, 4); ENSURE(raw_key, nRaw, 8);
  ENSURE(raw_off, E + 1, 4); ENSURE(raw_scratchOff, E + 1, 4); ENSURE(raw_scratch, scratchOff[E], 8);
  ENSURE(in_x, n, 4); ENSURE(in_y, n, 4); ENSURE(in_z, n, 4);
  ENSURE(in_layer, n, 4); ENSURE(in_det, n, 4); ENSURE(in_hid, n, 4); ENSURE(in_evt, n, 4);
  ENSURE(evOff, E, 4);
  ENSURE(layHits, (size_t)E * L, 4);
  ENSURE(layOff, (size_t)E * L, 4);
  auto up = [&](DevBuf& d, const void* h, size_t bytes) {
    return bytes ? cudaMemcpyAsync(d.p, h, bytes, cudaMemcpyHostToDevice, c->st) : cudaSuccess;
  };
  CK(up(c->raw_x, raw.x.data(), nRaw * 4));
  CK(up(c->raw_y, raw.y.data(), nRaw * 4));
  CK(up(c->raw_z, raw.z.data(), nRaw * 4));
  CK(up(c->raw_layer, raw.layer.data(), nRaw * 4));
  CK(up(c->raw_det, raw.det.data(), nRaw * 4));
  CK(up(c->raw_tid, raw.tid.data(), nRaw * 4));
  CK(up(c->raw_key, raw.key.data(), nRaw * 8));
  CK(up(c->raw_off, raw.rawOffsets.data(), (size_t)(E + 1) * 4));
  CK(up(c->raw_scratchOff, scratchOff.data(), (size_t)(E + 1) * 4));
  CK(up(c->evOff, raw.eventOffsets.data(), (size_t)E * 4));
  CK(up(c->layHits, raw.layerHits.data(), (size_t)E * L * 4));
  CK(up(c->layOff, raw.layerOffsets.data(), (size_t)E * L * 4));
  RawEventHits in{ptr<float>(c->raw_x), ptr<float>(c->raw_y), ptr<float>(c->raw_z), ptr<uint32_t>(c->raw_layer),
                  ptr<uint32_t>(c->raw_det), ptr<uint32_t>(c->raw_tid),
                  ptr<unsigned long long>(c->raw_key), ptr<uint32_t>(c->raw_off),
                  ptr<uint32_t>(c->raw_scratchOff)};
  HitColumns out{ptr<float>(c->in_x), ptr<float>(c->in_y), ptr<float>(c->in_z), ptr<uint32_t>(c->in_layer),
                 ptr<uint32_t>(c->in_det), ptr<uint32_t>(c->in_hid), ptr<uint32_t>(c->in_evt),
                 ptr<uint32_t>(c->evOff)};
  CK(bucket_events(in, ptr<unsigned long long>(c->raw_scratch), E, (uint32_t)n, out, c->st, nullptr));
  CK(cudaStreamSynchronize(c->st));
  c->E = E;
  c->L = L;
  c->nHits = n;
  c->maxLayerHits = raw.maxLayerHits;
  c->haveHits = true;
  c->stage = 0;
  sizes->n_hits = n;
  sizes->n_events = E;
  sizes->n_layers = L;
  sizes->n_findable = raw.findableId.size();
  const size_t nf = std::min<size_t>(raw.findableId.size(), findable_cap);
  if (findable_id && nf) std::memcpy(findable_id, raw.findableId.data(), nf * 4);
  if (findable_event && nf) std::memcpy(findable_event, raw.findableEvent.data(), nf * 4);
  return TRAX_OK;
}

int trax_grid_build(trax_ctx* c) { return c ? run_stage(c, 1) : TRAX_ERR_ARG; }

int trax_set_tracklets(trax_ctx* c, const uint32_t* h1, const uint32_t* h2, const uint32_t* h3, uint64_t n) {
  if (!c || (n && (!h1 || !h2 || !h3))) return fail(c, TRAX_ERR_ARG, "null triplet columns");
  RC(begin_run(c, true));
  const Mode mode = SYNCED;
  const uint64_t nh = c->nHits;
  if (n > 0xfffffff0ull) return fail(c, TRAX_ERR_ARG, "too many triplets");
  // host-side validation against the uploaded layer and event columns
  std::vector<uint32_t> layer(nh), evt(nh);
  if (nh) {
    CK(cudaMemcpyAsync(layer.data(), c->in_layer.p, nh * 4, cudaMemcpyDeviceToHost, c->st));
    CK(cudaMemcpyAsync(evt.data(), c->in_evt.p, nh * 4, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
  }
  uint64_t prevKey = 0;
  for (uint64_t t = 0; t < n; ++t) {
    if (h1[t] >= nh || h2[t] >= nh || h3[t] >= nh) return fail(c, TRAX_ERR_ARG, "triplet hit index out of range");
    const uint32_t l = layer[h1[t]], e = evt[h1[t]];
    if (l < 1 || l > c->cfg.nLT || e >= c->E)
      return fail(c, TRAX_ERR_ARG, "a triplet's first hit lies outside the layer-triplet/event range");
    const uint64_t key = (uint64_t)e * c->cfg.nLT + (l - 1);
    if (key < prevKey) return fail(c, TRAX_ERR_ARG, "triplets must be grouped by (event, layer triplet)");
    if (t > 0 && key == prevKey && (h2[t] < h2[t - 1] || (h2[t] == h2[t - 1] && h1[t] < h1[t - 1])))
      c->sortedSegments = false;  // connectivity then scans like the reference
    prevKey = key;
  }
  ENSURE(px, nh, 4); ENSURE(py, nh, 4); ENSURE(pz, nh, 4);
  ENSURE(player, nh, 4); ENSURE(pdet, nh, 4); ENSURE(phid, nh, 4); ENSURE(pevt, nh, 4); ENSURE(porig, nh, 4);
  ENSURE(pxyzp, nh, 16);
  ENSURE(h1, n, 4);
  ENSURE(h2, n, 4);
  ENSURE(h3, n, 4);
  ENSURE(tripOffsets, (size_t)c->cfg.E * c->cfg.nLT + 1, 4);
  GridInput in;
  memset(&in, 0, sizeof(in));
  in.x = ptr<float>(c->in_x);
  in.y = ptr<float>(c->in_y);
  in.z = ptr<float>(c->in_z);
  in.layer = ptr<uint32_t>(c->in_layer);
  in.det = ptr<uint32_t>(c->in_det);
  in.hid = ptr<uint32_t>(c->in_hid);
  in.evt = ptr<uint32_t>(c->in_evt);
  CK(identity_hits(in, (uint32_t)nh, dev_hits(c), c->st, &c->launches));
  c->fineBuilt = 0;  // the hit collection is no longer the grid's
  if (n) {
    CK(cudaMemcpyAsync(c->h1.p, h1, n * 4, cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(c->h2.p, h2, n * 4, cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(c->h3.p, h3, n * 4, cudaMemcpyHostToDevice, c->st));
  }
  c->hSlots[S_TRIPLETS] = (uint32_t)n;
  CK(cudaMemcpyAsync(slot(c, S_TRIPLETS), c->hSlots + S_TRIPLETS, 4, cudaMemcpyHostToDevice, c->st));
  CK(triplet_offsets(c->cfg, dev_hits(c), ptr<uint32_t>(c->h1), slot(c, S_TRIPLETS), n,
                     ptr<uint32_t>(c->tripOffsets), c->st, &c->launches));
  c->nPairs = c->nCands = 0;
  c->nT = n;
  c->identityHits = true;
  RC(check_device_error(c));
  c->stage = 4;
  ++c->tripGen;
  c->caOnly = false;
  return TRAX_OK;
}

int trax_pair_gen(trax_ctx* c, uint64_t* n_pairs) {
  if (!c) return TRAX_ERR_ARG;
  RC(run_stage(c, 2));
  if (n_pairs) *n_pairs = c->nPairs;
  return TRAX_OK;
}

int trax_triplet_predict(trax_ctx* c, uint64_t* n_candidates) {
  if (!c) return TRAX_ERR_ARG;
  RC(run_stage(c, 3));
  if (n_candidates) *n_candidates = c->nCands;
  return TRAX_OK;
}

int trax_triplet_filter(trax_ctx* c, uint64_t* n_triplets) {
  if (!c) return TRAX_ERR_ARG;
  RC(run_stage(c, 4));
  if (n_triplets) *n_triplets = c->nT;
  return TRAX_OK;
}

int trax_connectivity(trax_ctx* c, float d_eta_cut, uint64_t* n_links) {
  if (!c) return TRAX_ERR_ARG;
  c->dEtaCut = d_eta_cut;
  c->cfg.dEtaCut = d_eta_cut;
  RC(run_stage(c, 5));
  if (n_links) *n_links = c->nLinks;
  return TRAX_OK;
}

int trax_circle_fit(trax_ctx* c) { return c ? run_stage(c, 6) : TRAX_ERR_ARG; }

int trax_cellular_automaton(trax_ctx* c, uint64_t* n_track_entries) {
  if (!c) return TRAX_ERR_ARG;
  RC(run_stage(c, 7));
  if (n_track_entries) *n_track_entries = c->nTracks;
  return TRAX_OK;
}

int trax_circle_fit_on(trax_ctx* c, const uint32_t* valid_idx, uint64_t n_valid) {
  if (!c || (n_valid && !valid_idx)) return fail(c, TRAX_ERR_ARG, "null index list");
  if (c->stage < 4 || c->caOnly) return fail(c, TRAX_ERR_STATE, "no triplets: run the filter or trax_set_tracklets");
  const uint64_t nT = c->nT;
  for (uint64_t i = 0; i < n_valid; ++i)
    if (valid_idx[i] >= nT) return fail(c, TRAX_ERR_ARG, "triplet index out of range");
  CK(cudaSetDevice(c->device));
  const Mode mode = SYNCED;
  ENSURE(userIdx, n_valid, 4);
  ENSURE(pt, nT, 4);
  if (n_valid) CK(cudaMemcpyAsync(c->userIdx.p, valid_idx, n_valid * 4, cudaMemcpyHostToDevice, c->st));
  c->hSlots[S_USER] = (uint32_t)n_valid;
  CK(cudaMemcpyAsync(slot(c, S_USER), c->hSlots + S_USER, 4, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemsetAsync(c->pt.p, 0, (size_t)std::max<uint64_t>(nT, 1) * 4, c->st));
  CK(circle_fit(dev_hits(c), triplets(c, nT), ptr<uint32_t>(c->userIdx), slot(c, S_USER), n_valid,
                ptr<float>(c->pt), c->st, &c->launches));
  CK(cudaStreamSynchronize(c->st));
  RC(check_device_error(c));
  c->ptGen = c->tripGen;
  return TRAX_OK;
}

int trax_get_pt(trax_ctx* c, float* pt) {
  if (!c || (!pt && c->nT)) return TRAX_ERR_ARG;
  if (c->ptGen != c->tripGen) return fail(c, TRAX_ERR_STATE, "no circle fit of the current triplets");
  RC(copy_out(c, pt, c->pt, c->nT * 4));
  CK(cudaStreamSynchronize(c->st));
  return TRAX_OK;
}

int trax_cellular_automaton_on(trax_ctx* c, const uint32_t* basis, const uint32_t* follower, uint64_t n_links,
                               const float* pt, uint64_t n_triplets, uint64_t* n_track_entries) {
  if (!c || !basis || !follower || !pt) return fail(c, TRAX_ERR_ARG, "null input");
  if (n_links == 0 || n_triplets == 0) return fail(c, TRAX_ERR_ARG, "the CA needs links and triplets");
  if (n_links > 0xfffffff0ull || n_triplets > 0xfffffff0ull) return fail(c, TRAX_ERR_ARG, "input too large");
  const bool haveTriplets = c->stage >= 4 && !c->caOnly;
  if (haveTriplets && n_triplets != c->nT)
    return fail(c, TRAX_ERR_ARG, "pt must hold one value per triplet of the context's triplet set");
  for (uint64_t p = 0; p < n_links; ++p)
    if (basis[p] >= n_triplets || follower[p] >= n_triplets)
      return fail(c, TRAX_ERR_ARG, "link triplet index out of range");
  CK(cudaSetDevice(c->device));
  const Mode mode = SYNCED;
  const uint64_t nT = n_triplets, nL = n_links;
  if (!haveTriplets) {
    c->nT = nT;
    c->caOnly = true;
    ++c->tripGen;  // a triplet set of its own, without hits
  }
  ENSURE(basis, nL, 4);
  ENSURE(follower, nL, 4);
  ENSURE(pt, nT, 4);
  ENSURE(states, nT, 4);
  ENSURE(caNext, nT, 4);
  ENSURE(inStart, nT + 1, 4);
  ENSURE(inCursor, nT, 4);
  ENSURE(inList, nL, 4);
  ENSURE(best, nT, 4);
  ENSURE(isBest, nT, 4);
  ENSURE(handlers, nT + 1, 4);
  CK(ensure(c, c->scanScratch, scan_scratch_bytes(nT + 1)));
  CK(cudaMemcpyAsync(c->basis.p, basis, nL * 4, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->follower.p, follower, nL * 4, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemcpyAsync(c->pt.p, pt, nT * 4, cudaMemcpyHostToDevice, c->st));
  memset(c->hSlots, 0, sizeof(uint32_t) * S_N);
  c->hSlots[S_TRIPLETS] = (uint32_t)nT;
  c->hSlots[S_LINKS] = (uint32_t)nL;
  CK(cudaMemcpyAsync(c->slots.p, c->hSlots, sizeof(uint32_t) * S_N, cudaMemcpyHostToDevice, c->st));
  const uint32_t* nTDev = slot(c, S_TRIPLETS);
  const uint32_t* nLinksDev = slot(c, S_LINKS);
  CABuffers b = ca_buffers(c);
  // states 1, in-degrees, the incoming bases of every follower (ascending)
  CK(ca_in_degree(ptr<uint32_t>(c->follower), nLinksDev, nL, b, nTDev, nT, c->st, &c->launches));
  CK(scan_exclusive(b.inStart, b.inStart, nT + 1, nullptr, 0, nT + 1, c->scanScratch.p, dev_err(c), c->st,
                    &c->launches, true, c->wait));
  CK(ca_fill(ptr<uint32_t>(c->basis), ptr<uint32_t>(c->follower), nLinksDev, nL, b, nTDev, nT, c->st,
             &c->launches));
  // forward phase: the reference's iteration (CellularAutomaton.cpp:37-98),
  // both state buffers starting at 1, swapped without copying; a link set
  // with a cycle never settles and is rejected after nT + 2 iterations
  CK(fill_u32(ptr<uint32_t>(c->caNext), 1u, (uint32_t)nT, c->st, &c->launches));
  uint32_t* cur = ptr<uint32_t>(c->states);
  uint32_t* next = ptr<uint32_t>(c->caNext);
  uint32_t* living = slot(c, S_LIVING);
  uint64_t iterations = 0;
  uint32_t alive = 0;
  do {
    ++iterations;
    CK(cudaMemsetAsync(living, 0, 4, c->st));
    CK(ca_iteration(ptr<uint32_t>(c->basis), ptr<uint32_t>(c->follower), (uint32_t)nL, cur, next, living, c->st,
                    &c->launches));
    CK(cudaMemcpyAsync(&alive, living, 4, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    std::swap(cur, next);
  } while (alive && iterations <= nT + 2);
  if (alive) return fail(c, TRAX_ERR_ARG, "the links form a cycle: the CA's states never settle");
  if (cur != ptr<uint32_t>(c->states))
    CK(cudaMemcpyAsync(c->states.p, cur, nT * 4, cudaMemcpyDeviceToDevice, c->st));
  // backward phase, handlers and tracks as in the chain
  CK(ca_backward(ptr<float>(c->pt), b, nTDev, nT, nLinksDev, c->st, &c->launches));
  RC(scan_publish(c, SYNCED, b.handlers, nT, nullptr, nT, S_TRACKS, NO_CAP));
  RC(read_slot(c, S_TRACKS, &c->nTracks));
  ENSURE(tracks, c->nTracks, 4);
  CK(ca_tracks(b, nTDev, nT, ptr<uint32_t>(c->tracks), c->nTracks, dev_err(c), c->st, &c->launches));
  CK(cudaStreamSynchronize(c->st));
  RC(check_device_error(c));
  c->nLinks = nL;
  c->noLinks = false;
  c->nConn = c->nNonConn = 0;
  c->caGen = c->tripGen;
  if (n_track_entries) *n_track_entries = c->nTracks;
  return TRAX_OK;
}

int trax_prefix_sum(trax_ctx* c, uint32_t* data, uint64_t n) {
  if (!c || (!data && n)) return fail(c, TRAX_ERR_ARG, "null data");
  if (n == 0) return TRAX_OK;
  if (n > 0xffffffffull) return fail(c, TRAX_ERR_ARG, "scan length above 2^32 - 1");
  DevBuf tmp;
  CK(ensure(c, tmp, n * 4));
  int rc = TRAX_OK;
  cudaError_t e = cudaMemcpyAsync(tmp.p, data, n * 4, cudaMemcpyHostToDevice, c->st);
  if (e == cudaSuccess) e = ensure(c, c->scanScratch, scan_scratch_bytes(n));
  if (e == cudaSuccess) e = cudaMemsetAsync(c->slots.p, 0, 4, c->st);
  if (e == cudaSuccess)
    e = scan_exclusive(ptr<uint32_t>(tmp), ptr<uint32_t>(tmp), n, nullptr, 0, n, c->scanScratch.p, dev_err(c), c->st,
                       &c->launches, false, c->wait);  // wraps like PrefixSum's uint arithmetic
  if (e == cudaSuccess) e = cudaMemcpyAsync(data, tmp.p, n * 4, cudaMemcpyDeviceToHost, c->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
  if (e != cudaSuccess) rc = cuda_fail(c, e, "trax_prefix_sum");
  release(tmp);
  if (rc == TRAX_OK) rc = check_device_error(c);
  return rc;
}

int trax_set_wait_limit(trax_ctx* c, uint32_t polls) {
  if (!c) return TRAX_ERR_ARG;
  c->wait.spinLimit = polls;
  return TRAX_OK;
}

int trax_debug_skip_publish(trax_ctx* c, uint32_t tile) {
  if (!c) return TRAX_ERR_ARG;
  c->wait.skipTile = tile;
  return TRAX_OK;
}

int trax_seed_batch(trax_ctx* c, const trax_batch_opts* opts, trax_batch_stats* stats) {
  if (!c) return TRAX_ERR_ARG;
  NvtxRange nvtx("trax_seed_batch");
  const bool linking = opts ? opts->run_linking != 0 : true;
  const bool useGraph = opts ? opts->use_graph != 0 : false;
  if (opts && opts->d_eta_cut > 0.0f) c->dEtaCut = opts->d_eta_cut;
  c->launches = 0;
  c->graphCaptures = 0;
  c->identityHits = false;
  c->sortedSegments = true;
  if (!useGraph) {
    CK(cudaEventRecord(c->ev0, c->st));
    RC(run_synced_chain(c, linking));
    CK(cudaEventRecord(c->ev1, c->st));
    CK(cudaEventSynchronize(c->ev1));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    c->lastMs = ms;
    fill_stats(c, stats);
    return TRAX_OK;
  }
  for (int attempt = 0; attempt < 2; ++attempt) {
    RC(build_config(c));
    const uint64_t key = shape_key(c, linking);
    if (!c->graphExec || key != c->graphKey) {
      // calibrate the capacities with one host-synced run, then capture
      NvtxRange nvtxCal("trax.calibrate_and_capture");
      ++c->graphCaptures;
      drop_graph(c);
      RC(run_synced_chain(c, linking));
      if (!c->keepSlots) {  // the capture slots for what this batch's pairs hold
        c->keepAuto = auto_keep_slots(c->nCands, c->nPairs);
        c->cfg.predKeep = c->keepAuto;
      }
      RC(size_device_buffers(c));
      c->launches = 0;
      CK(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
      cudaMemsetAsync(c->slots.p, 0, sizeof(uint32_t) * S_N, c->st);
      int rc = chain_device(c, linking);
      cudaGraph_t g = nullptr;
      cudaError_t e = cudaStreamEndCapture(c->st, &g);
      if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
      }
      if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamEndCapture");
      c->graph = g;
      CK(cudaGraphInstantiate(&c->graphExec, g, 0));
      c->graphLaunches = c->launches;
      c->graphKey = shape_key(c, linking);
    }
    NvtxRange nvtxReplay("trax.replay");
    CK(cudaEventRecord(c->ev0, c->st));
    CK(cudaGraphLaunch(c->graphExec, c->st));
    CK(cudaEventRecord(c->ev1, c->st));
    RC(read_slots(c));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    c->lastMs = ms;
    c->launches = c->graphLaunches;
    const uint32_t bits = c->hSlots[S_ERR];
    c->nTasks = c->hSlots[S_TASKS];
    c->nPairs = c->hSlots[S_PAIRS];
    c->nCands = c->hSlots[S_CANDS];
    c->nT = c->hSlots[S_TRIPLETS];
    c->nLinks = linking ? c->hSlots[S_LINKS] : 0;
    c->nConn = linking ? c->hSlots[S_CONN] : 0;
    c->nNonConn = linking ? c->hSlots[S_NONCONN] : 0;
    c->nTracks = linking ? c->hSlots[S_TRACKS] : 0;
    c->noLinks = c->nLinks == 0;
    if (c->noLinks) c->nConn = c->nNonConn = c->nTracks = 0;  // the reference returns no lists then
    c->pairSent = c->hSlots[S_PAIR_SENT];
    c->candSent = c->hSlots[S_CAND_SENT];
    if (bits & TRAX_EBIT_CAPACITY) {
      // admission failed: recalibrate on these events and replay once more
      drop_graph(c);
      continue;
    }
    RC(error_from_bits(c, bits));
    c->stage = linking ? 7 : 4;
    ++c->tripGen;
    if (linking) c->ptGen = c->caGen = c->tripGen;
    c->caOnly = false;
    fill_stats(c, stats);
    return TRAX_OK;
  }
  return fail(c, TRAX_ERR_CAPACITY, "capacity exceeded after recalibration");
}

int trax_get_timings(trax_ctx* c, float* stage_ms, float* kernel_ms) {
  if (!c) return TRAX_ERR_ARG;
  CK(cudaStreamSynchronize(c->st));
  for (int s = 0; s < N_STAGES; ++s) {
    float ms = -1.0f;
    if (c->stageUsed[s] && cudaEventElapsedTime(&ms, c->stageEv[s], c->stageEv[s + 1]) != cudaSuccess) ms = -1.0f;
    if (stage_ms) stage_ms[s] = ms;
  }
  for (int k = 0; k < TK_N; ++k) {
    float ms = -1.0f;
    if (c->kUsed[k] && cudaEventElapsedTime(&ms, c->kEv[2 * k], c->kEv[2 * k + 1]) != cudaSuccess) ms = -1.0f;
    if (kernel_ms) kernel_ms[k] = ms;
  }
  cudaGetLastError();  // clear a "not ready"/"invalid handle" from unused events
  return TRAX_OK;
}

int trax_get_stats(trax_ctx* c, trax_batch_stats* s) {
  if (!c || !s) return TRAX_ERR_ARG;
  fill_stats(c, s);
  return TRAX_OK;
}

int trax_get_pairs(trax_ctx* c, uint32_t* pairs2, uint32_t* offsets) {
  if (!c) return TRAX_ERR_ARG;
  if (c->stage < 2) return fail(c, TRAX_ERR_STATE, "pairs not generated");
  RC(copy_out(c, pairs2, c->pairs, c->nPairs * 8));
  RC(copy_out(c, offsets, c->pairOffsets, ((size_t)c->cfg.E * c->cfg.nLT + 1) * 4));
  CK(cudaStreamSynchronize(c->st));
  return TRAX_OK;
}

int trax_get_candidates(trax_ctx* c, uint32_t* cands2, uint32_t* offsets) {
  if (!c) return TRAX_ERR_ARG;
  if (c->stage < 3) return fail(c, TRAX_ERR_STATE, "candidates not predicted");
  RC(copy_out(c, cands2, c->cands, c->nCands * 8));
  RC(copy_out(c, offsets, c->candOffsets, ((size_t)c->cfg.E * c->cfg.nLT + 1) * 4));
  CK(cudaStreamSynchronize(c->st));
  return TRAX_OK;
}

int trax_get_triplets(trax_ctx* c, uint32_t* h1, uint32_t* h2, uint32_t* h3, uint32_t* offsets) {
  if (!c) return TRAX_ERR_ARG;
  if (c->stage < 4) return fail(c, TRAX_ERR_STATE, "triplets not filtered");
  RC(copy_out(c, h1, c->h1, c->nT * 4));
  RC(copy_out(c, h2, c->h2, c->nT * 4));
  RC(copy_out(c, h3, c->h3, c->nT * 4));
  RC(copy_out(c, offsets, c->tripOffsets, ((size_t)c->cfg.E * c->cfg.nLT + 1) * 4));
  CK(cudaStreamSynchronize(c->st));
  return TRAX_OK;
}

int trax_physics_triplets_device(trax_ctx* c, const uint32_t* findable_id, const uint32_t* findable_event,
                                 uint64_t n_findable, trax_physics_record* out) {
  if (!c || !out || (n_findable && (!findable_id || !findable_event))) return fail(c, TRAX_ERR_ARG, "null argument");
  if (c->stage < 4) return fail(c, TRAX_ERR_STATE, "triplets not filtered");
  if (c->identityHits) return fail(c, TRAX_ERR_STATE, "the hits of caller triplets carry no grid order");
  const Mode mode = SYNCED;
  const uint32_t E = c->cfg.E, nLT = c->cfg.nLT;
  const size_t S = (size_t)E * nLT;
  // each event's findable track ids, sorted and distinct (the truth sets)
  std::vector<std::pair<uint32_t, uint32_t>> truth;
  for (uint64_t k = 0; k < n_findable; ++k)
    if (findable_event[k] < E) truth.emplace_back(findable_event[k], findable_id[k]);
  std::sort(truth.begin(), truth.end());
  truth.erase(std::unique(truth.begin(), truth.end()), truth.end());
  std::vector<uint32_t> findOff(E + 1, 0), findIds(truth.size()), truthSize(E, 0);
  for (size_t k = 0; k < truth.size(); ++k) {
    findIds[k] = truth[k].second;
    ++truthSize[truth[k].first];
  }
  for (uint32_t e = 0; e < E; ++e) findOff[e + 1] = findOff[e] + truthSize[e];
  ENSURE(phys_findOff, E + 1, 4);
  ENSURE(phys_findIds, std::max<size_t>(findIds.size(), 1), 4);
  ENSURE(phys_flags, std::max<size_t>(nLT * findIds.size(), 1), 4);
  ENSURE(phys_counts, 3 * S + 1, 4);
  CK(cudaMemcpyAsync(c->phys_findOff.p, findOff.data(), (size_t)(E + 1) * 4, cudaMemcpyHostToDevice, c->st));
  if (!findIds.empty())
    CK(cudaMemcpyAsync(c->phys_findIds.p, findIds.data(), findIds.size() * 4, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemsetAsync(c->phys_flags.p, 0, std::max<size_t>(nLT * findIds.size(), 1) * 4, c->st));
  CK(cudaMemsetAsync(c->phys_counts.p, 0, (3 * S + 1) * 4, c->st));
  uint32_t* counts = ptr<uint32_t>(c->phys_counts);
  CK(physics_counts(ptr<uint32_t>(c->h1), ptr<uint32_t>(c->h2), ptr<uint32_t>(c->h3), slot(c, S_TRIPLETS), c->nT,
                    ptr<uint32_t>(c->tripOffsets), ptr<uint32_t>(c->phid), E, nLT, ptr<uint32_t>(c->phys_findOff),
                    ptr<uint32_t>(c->phys_findIds), counts,
                    counts + S, ptr<uint32_t>(c->phys_flags), counts + 2 * S, c->st, nullptr));
  std::vector<uint32_t> h(3 * S), offsets(S + 1);
  if (S) CK(cudaMemcpyAsync(h.data(), counts, 3 * S * 4, cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(offsets.data(), c->tripOffsets.p, (S + 1) * 4, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  // clones: real triplets of findable tracks beyond the first per track
  std::vector<uint32_t> clones(S);
  for (size_t k = 0; k < S; ++k) clones[k] = h[S + k] - h[2 * S + k];
  trax::physics_records(E, nLT, offsets.data(), h.data() + 2 * S, h.data(), clones.data(), truthSize.data(), out);
  return TRAX_OK;
}

int trax_physics_tracks_device(trax_ctx* c, uint64_t total_tracks, trax_track_metrics* out) {
  if (!c || !out) return fail(c, TRAX_ERR_ARG, "null argument");
  if (c->identityHits) return fail(c, TRAX_ERR_STATE, "the hits of caller triplets carry no grid order");
  *out = trax_track_metrics{0, 0, 0, 0, 0, 0.0, 0.0, 0.0};
  if (c->stage >= 5 && c->noLinks) return TRAX_OK;  // no links: the reference runs no CA, no tracks
  if (c->stage < 7) return fail(c, TRAX_ERR_STATE, "cellular automaton not run");
  const Mode mode = SYNCED;
  const uint32_t nT = (uint32_t)c->nT;
  ENSURE(trk_isTrack, (size_t)nT + 1, 4);
  ENSURE(trk_hitsOf, (size_t)nT + 1, 4);
  CK(ensure(c, c->scanScratch, scan_scratch_bytes((uint64_t)nT + 1)));
  uint32_t* isTrack = ptr<uint32_t>(c->trk_isTrack);
  uint32_t* hitsOf = ptr<uint32_t>(c->trk_hitsOf);
  const uint32_t* off = ptr<uint32_t>(c->handlers);
  CK(track_sizes(off, nT, isTrack, hitsOf, c->st));
  CK(scan_exclusive(isTrack, isTrack, (uint64_t)nT + 1, nullptr, 0, (uint64_t)nT + 1, c->scanScratch.p, dev_err(c),
                    c->st, nullptr, true, c->wait));
  CK(scan_exclusive(hitsOf, hitsOf, (uint64_t)nT + 1, nullptr, 0, (uint64_t)nT + 1, c->scanScratch.p, dev_err(c),
                    c->st, nullptr, true, c->wait));
  uint32_t totals[2];
  CK(cudaMemcpyAsync(&totals[0], isTrack + nT, 4, cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(&totals[1], hitsOf + nT, 4, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  RC(check_device_error(c));
  const uint32_t nTracks = totals[0], nEntries = totals[1];
  const size_t nk = std::max<size_t>(nTracks, 1) + 1;
  ENSURE(trk_start, nk, 4); ENSURE(trk_size, nk, 4); ENSURE(trk_real, nk, 4); ENSURE(trk_firstId, nk, 4);
  ENSURE(trk_parent, nk, 4); ENSURE(trk_compSize, nk, 4); ENSURE(trk_compStart, nk, 4); ENSURE(trk_cursor, nk, 4);
  ENSURE(trk_members, nk, 4); ENSURE(trk_filtered, nk, 4);
  ENSURE(trk_hits, std::max<size_t>(nEntries, 1), 4); ENSURE(trk_entryTrack, std::max<size_t>(nEntries, 1), 4);
  ENSURE(trk_owner, std::max<size_t>(c->nHits, 1), 4);
  uint32_t tableSize = 1024;
  while (tableSize < 2ull * nTracks) tableSize <<= 1;
  ENSURE(trk_table, tableSize, 8);
  ENSURE(trk_counts, 4, 8);
  TrackLists t{ptr<uint32_t>(c->trk_start), ptr<uint32_t>(c->trk_size), ptr<uint32_t>(c->trk_real),
               ptr<uint32_t>(c->trk_firstId), ptr<uint32_t>(c->trk_parent), ptr<uint32_t>(c->trk_compSize),
               ptr<uint32_t>(c->trk_compStart), ptr<uint32_t>(c->trk_cursor), ptr<uint32_t>(c->trk_members),
               ptr<uint32_t>(c->trk_filtered), ptr<uint32_t>(c->trk_hits), ptr<uint32_t>(c->trk_entryTrack),
               ptr<uint32_t>(c->trk_owner)};
  CK(cudaMemsetAsync(t.owner, 0xFF, std::max<size_t>(c->nHits, 1) * 4, c->st));
  CK(cudaMemsetAsync(t.compSize, 0, nk * 4, c->st));
  CK(cudaMemsetAsync(t.cursor, 0, nk * 4, c->st));
  CK(cudaMemsetAsync(c->trk_table.p, 0, (size_t)tableSize * 8, c->st));
  CK(cudaMemsetAsync(c->trk_counts.p, 0, 4 * 8, c->st));
  CK(track_extract(off, ptr<uint32_t>(c->tracks), nT, ptr<uint32_t>(c->h1), ptr<uint32_t>(c->h2),
                   ptr<uint32_t>(c->h3), ptr<uint32_t>(c->phid), isTrack, hitsOf, t, c->st));
  // components of the "shares a hit" graph: union-find rounds until stable
  uint32_t* changed = ptr<uint32_t>(c->trk_counts) + 6;  // a spare word of the counts buffer
  bool stable = false;
  for (int round = 0; round < 64 && !stable; ++round) {
    CK(cudaMemsetAsync(changed, 0, 4, c->st));
    CK(track_union_step(t, nTracks, nEntries, changed, c->st));
    uint32_t h = 0;
    CK(cudaMemcpyAsync(&h, changed, 4, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    stable = h == 0;
  }
  if (!stable) return fail(c, TRAX_ERR_TIMEOUT, "track components did not settle in 64 rounds");
  CK(track_members(t, nTracks, false, c->st));
  CK(scan_exclusive(t.compSize, t.compStart, (uint64_t)nTracks + 1, nullptr, 0, (uint64_t)nTracks + 1,
                    c->scanScratch.p, dev_err(c), c->st, nullptr, true, c->wait));
  CK(track_members(t, nTracks, true, c->st));
  unsigned long long* counts = ptr<unsigned long long>(c->trk_counts);
  CK(track_greedy(t, nTracks, ptr<unsigned long long>(c->trk_table), tableSize - 1, counts, c->st));
  unsigned long long h[3];
  CK(cudaMemcpyAsync(h, counts, 3 * 8, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  RC(check_device_error(c));
  out->total = nTracks;
  out->filtered = h[0];
  out->valid = h[1];
  out->valid_unique = h[2];
  out->fakes = h[0] - h[1];
  const double nf = (double)h[0];
  out->fake_rate = nf > 0 ? (double)out->fakes / nf : 0.0;
  out->clone_rate = nf > 0 ? (double)(h[1] - h[2]) / nf : 0.0;
  out->efficiency = total_tracks ? (double)h[2] / (double)total_tracks : 0.0;
  return TRAX_OK;
}

int trax_get_triplet_eta_pt(trax_ctx* c, float* eta, float* pt) {
  if (!c) return TRAX_ERR_ARG;
  if (c->stage < 5) return fail(c, TRAX_ERR_STATE, "connectivity not run");
  RC(copy_out(c, eta, c->eta, c->nT * 4));
  if (c->stage >= 6) RC(copy_out(c, pt, c->pt, c->nT * 4));
  CK(cudaStreamSynchronize(c->st));
  return TRAX_OK;
}

int trax_get_links(trax_ctx* c, uint32_t* basis, uint32_t* follower, uint32_t* connectable, uint32_t* non_connectable) {
  if (!c) return TRAX_ERR_ARG;
  if (c->stage < 5) return fail(c, TRAX_ERR_STATE, "connectivity not run");
  if (c->noLinks) return TRAX_OK;
  RC(copy_out(c, basis, c->basis, c->nLinks * 4));
  RC(copy_out(c, follower, c->follower, c->nLinks * 4));
  RC(copy_out(c, connectable, c->connIdx, c->nConn * 4));
  RC(copy_out(c, non_connectable, c->nonConnIdx, c->nNonConn * 4));
  CK(cudaStreamSynchronize(c->st));
  return TRAX_OK;
}

int trax_get_tracks(trax_ctx* c, uint32_t* states, uint32_t* tracks, uint32_t* track_offsets) {
  if (!c) return TRAX_ERR_ARG;
  const bool caOn = c->caGen == c->tripGen;  // also set by trax_cellular_automaton_on
  if (!caOn && c->stage >= 5 && c->noLinks) return TRAX_OK;  // no links: the reference runs no CA
  if (!caOn && c->stage < 7) return fail(c, TRAX_ERR_STATE, "cellular automaton not run");
  RC(copy_out(c, states, c->states, c->nT * 4));
  RC(copy_out(c, tracks, c->tracks, c->nTracks * 4));
  RC(copy_out(c, track_offsets, c->handlers, (c->nT + 1) * 4));
  CK(cudaStreamSynchronize(c->st));
  return TRAX_OK;
}

int trax_get_grid(trax_ctx* c, uint32_t* grid, uint64_t* n_cells) {
  if (!c) return TRAX_ERR_ARG;
  if (c->stage < 1 || c->identityHits) return fail(c, TRAX_ERR_STATE, "grid not built");
  const uint64_t cells = (uint64_t)c->E * c->L * c->cfg.C;
  if (n_cells) *n_cells = cells;
  RC(copy_out(c, grid, c->grid, cells * 4));
  CK(cudaStreamSynchronize(c->st));
  return TRAX_OK;
}

int trax_get_hit_perm(trax_ctx* c, uint32_t* perm) {
  if (!c) return TRAX_ERR_ARG;
  if (c->stage < 1) return fail(c, TRAX_ERR_STATE, "grid not built");
  RC(copy_out(c, perm, c->porig, (size_t)c->nHits * 4));
  CK(cudaStreamSynchronize(c->st));
  return TRAX_OK;
}

// ------------------------------------------------------- differentiable fit
int trax_fit_prepare(trax_ctx* c, const trax_fit_opts* opts, uint64_t* n_fit) {
  if (!c) return TRAX_ERR_ARG;
  if (c->stage < 4) return fail(c, TRAX_ERR_STATE, "triplets not filtered");
  CK(cudaSetDevice(c->device));
  c->fitReady = false;
  const float sigmaZ = (opts && opts->sigma_z > 0.0f) ? opts->sigma_z : 0.002f;
  const int truthOnly = opts ? opts->truth_only : 0;
  FitConfig& f = c->fitCfg;
  memset(&f, 0, sizeof(f));
  f.L = c->L;
  f.nLT = (uint32_t)c->lts.size();
  for (uint32_t k = 0; k < f.nLT; ++k) {
    f.layer[0][k] = c->lts[k].layer1 - 1;
    f.layer[1][k] = c->lts[k].layer2 - 1;
    f.layer[2][k] = c->lts[k].layer3 - 1;
    f.wTip[k] = 1.0f;
  }
  f.wZ = 1.0f / (sigmaZ * sigmaZ);
  RC(fit_set_alignment(c, nullptr));
  const uint64_t nT = c->nT;
  const uint32_t S = c->E * f.nLT;
  // 1. selection flags and per-segment counts
  CK(ensure(c, c->fitOk, (nT + 1) * 4));
  CK(ensure(c, c->fitSegCnt, (size_t)S * 4));
  CK(ensure(c, c->fitSegDelta, (size_t)S * 4));
  CK(cudaMemsetAsync(c->fitSegCnt.p, 0, (size_t)S * 4, c->st));
  uint32_t* ok = ptr<uint32_t>(c->fitOk);
  CK(fit_select(f, c->cfg, dev_hits(c), fit_triplets(c), nT, truthOnly, ok, ptr<uint32_t>(c->fitSegCnt), c->st,
                &c->launches));
  CK(ensure(c, c->scanScratch, scan_scratch_bytes(nT + 1)));
  CK(scan_exclusive(ok, ok, nT + 1, nullptr, 0, nT + 1, c->scanScratch.p, dev_err(c), c->st, &c->launches, true,
                    c->wait));
  // 2. rows ordered by layer triplet, then by event (segment order inside a layer triplet)
  std::vector<uint32_t> cnt(S);
  if (S) CK(cudaMemcpyAsync(cnt.data(), c->fitSegCnt.p, (size_t)S * 4, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  RC(check_device_error(c));
  std::vector<uint64_t> cStart(S), ltCount(f.nLT, 0);
  uint64_t run = 0;
  for (uint32_t s = 0; s < S; ++s) {
    cStart[s] = run;
    run += cnt[s];
    ltCount[s % f.nLT] += cnt[s];
  }
  if (run > 0xffffffffull) return fail(c, TRAX_ERR_CAPACITY, "too many fit rows");
  c->nFit = run;
  uint64_t base = 0, blk = 0;
  for (uint32_t k = 0; k < f.nLT; ++k) {
    f.ltBase[k] = (uint32_t)base;
    f.blkStart[k] = (uint32_t)blk;
    base += ltCount[k];
    blk += (ltCount[k] + TRAX_FIT_CHUNK - 1) / TRAX_FIT_CHUNK;
  }
  f.ltBase[f.nLT] = (uint32_t)base;
  f.blkStart[f.nLT] = (uint32_t)blk;
  f.nBlocks = (uint32_t)blk;
  std::vector<int32_t> delta(S);
  std::vector<uint64_t> inLT(f.nLT, 0);
  for (uint32_t s = 0; s < S; ++s) {
    const uint32_t k = s % f.nLT;
    delta[s] = (int32_t)((int64_t)(f.ltBase[k] + inLT[k]) - (int64_t)cStart[s]);
    inLT[k] += cnt[s];
  }
  if (S) CK(cudaMemcpyAsync(c->fitSegDelta.p, delta.data(), (size_t)S * 4, cudaMemcpyHostToDevice, c->st));
  CK(ensure(c, c->fitRows, std::max<uint64_t>(c->nFit, 1) * 4));
  CK(fit_scatter(c->cfg, dev_hits(c), fit_triplets(c), nT, ok, ptr<int32_t>(c->fitSegDelta),
                 ptr<uint32_t>(c->fitRows), c->st, &c->launches));
  // 3. sigma_tip per layer triplet: given, or 1.4826 x median |d0| at zero alignment
  bool needD0 = false;
  for (uint32_t k = 0; k < f.nLT; ++k) {
    const float g = opts ? opts->sigma_tip[k] : 0.0f;
    c->fitSigmaTip[k] = g;
    needD0 = needD0 || !(g > 0.0f);
  }
  if (needD0 && c->nFit) {
    c->fitReady = true;
    c->fitTripGen = c->tripGen;
    RC(fit_run(c, nullptr, false, true, false));
    std::vector<float> prm(c->nFit * 4);
    CK(cudaMemcpyAsync(prm.data(), c->fitParams.p, c->nFit * 16, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    c->fitReady = false;
    for (uint32_t k = 0; k < f.nLT; ++k) {
      if (c->fitSigmaTip[k] > 0.0f) continue;
      std::vector<float> a;
      for (uint32_t r = f.ltBase[k]; r < f.ltBase[k + 1]; ++r) a.push_back(std::fabs(prm[4 * (size_t)r + 1]));
      float sig = 1.0f;
      if (!a.empty()) {
        std::nth_element(a.begin(), a.begin() + a.size() / 2, a.end());
        sig = 1.4826f * a[a.size() / 2];
        if (!(sig > 0.0f)) sig = 1e-4f;
      }
      c->fitSigmaTip[k] = sig;
    }
  }
  for (uint32_t k = 0; k < f.nLT; ++k) {
    const float sg = c->fitSigmaTip[k] > 0.0f ? c->fitSigmaTip[k] : 1.0f;
    c->fitSigmaTip[k] = sg;
    f.wTip[k] = 1.0f / (sg * sg);
  }
  c->fitReady = true;
  c->fitTripGen = c->tripGen;
  if (n_fit) *n_fit = c->nFit;
  return TRAX_OK;
}

int trax_fit_forward(trax_ctx* c, const double* align, double* chi2, float* params) {
  if (!c || !align) return TRAX_ERR_ARG;
  RC(fit_check(c));
  CK(cudaSetDevice(c->device));
  RC(fit_run(c, align, false, params != nullptr, false));
  double out = 0.0;
  CK(cudaMemcpyAsync(&out, c->fitOut.p, sizeof(double), cudaMemcpyDeviceToHost, c->st));
  if (params && c->nFit) CK(cudaMemcpyAsync(params, c->fitParams.p, c->nFit * 16, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  if (chi2) *chi2 = out;
  return TRAX_OK;
}

int trax_fit_backward(trax_ctx* c, const double* align, double* chi2, double* d_align, double* gn_diag,
                      float* d_hits) {
  if (!c || !align) return TRAX_ERR_ARG;
  RC(fit_check(c));
  CK(cudaSetDevice(c->device));
  RC(fit_run(c, align, true, false, d_hits != nullptr));
  std::vector<double> out(1 + 6 * (size_t)c->L);
  CK(cudaMemcpyAsync(out.data(), c->fitOut.p, out.size() * sizeof(double), cudaMemcpyDeviceToHost, c->st));
  if (d_hits && c->nHits) {
    CK(ensure(c, c->fitDHitsF, (size_t)c->nHits * 3 * sizeof(float)));
    CK(fit_hits_out(ptr<double>(c->fitDHits), ptr<uint32_t>(c->porig), c->nHits, ptr<float>(c->fitDHitsF), c->st,
                    &c->launches));
    CK(cudaMemcpyAsync(d_hits, c->fitDHitsF.p, (size_t)c->nHits * 3 * sizeof(float), cudaMemcpyDeviceToHost,
                       c->st));
  }
  CK(cudaStreamSynchronize(c->st));
  if (chi2) *chi2 = out[0];
  if (d_align)
    for (size_t k = 0; k < 3 * (size_t)c->L; ++k) d_align[k] = out[1 + k];
  if (gn_diag)
    for (size_t k = 0; k < 3 * (size_t)c->L; ++k) gn_diag[k] = out[1 + 3 * (size_t)c->L + k];
  return TRAX_OK;
}

int trax_apply_alignment(trax_ctx* c, const double* align) {
  if (!c || !align) return TRAX_ERR_ARG;
  if (!c->haveHits) return fail(c, TRAX_ERR_STATE, "no hits uploaded");
  CK(cudaSetDevice(c->device));
  c->fitCfg.L = c->L;
  RC(fit_set_alignment(c, align));
  CK(fit_apply(c->fitCfg, ptr<float>(c->in_x), ptr<float>(c->in_y), ptr<float>(c->in_z), ptr<uint32_t>(c->in_layer),
               c->nHits, c->st, &c->launches));
  CK(cudaStreamSynchronize(c->st));
  c->stage = 0;  // every stage output refers to the old positions
  c->fitReady = false;
  ++c->tripGen;
  drop_graph(c);
  return TRAX_OK;
}

int trax_fit_get_rows(trax_ctx* c, uint32_t* triplet_index, float* sigma_tip) {
  if (!c) return TRAX_ERR_ARG;
  RC(fit_check(c));
  if (triplet_index && c->nFit) RC(copy_out(c, triplet_index, c->fitRows, c->nFit * 4));
  if (sigma_tip)
    for (size_t k = 0; k < c->lts.size(); ++k) sigma_tip[k] = c->fitSigmaTip[k];
  CK(cudaStreamSynchronize(c->st));
  return TRAX_OK;
}

}  // extern "C"
