// trax_device.cuh -- device-side configuration, error reporting and the
// primitives shared by the sm_103a kernels of the triplet-seeding path.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "trax_math.h"

namespace trax {

#define TRAX_MAX_LT 16
#define TRAX_MAX_LAYERS 32
#define TRAX_SENTINEL 0xffffffffu

// error bits written by kernels into the context's device error word
#define TRAX_EBIT_TIMEOUT 1u
#define TRAX_EBIT_CAPACITY 2u
#define TRAX_EBIT_BOUNDS 4u
#define TRAX_EBIT_OVERFLOW 8u  // a count scan's total does not fit in 32 bits

// Everything a kernel needs to know about the workload, passed by value.
struct DevConfig {
  uint32_t E, L, nZ, nP, C, nLT;
  float minZ, sZ, minPhi, sP;
  float minRcurv;
  float dEtaCut;
  uint32_t layer1[TRAX_MAX_LT], layer2[TRAX_MAX_LT], layer3[TRAX_MAX_LT];
  float dThetaCut[TRAX_MAX_LT], sigmaZ[TRAX_MAX_LT], dPhiCut[TRAX_MAX_LT];
  float sigmaPhi[TRAX_MAX_LT], tipCut[TRAX_MAX_LT], z0[TRAX_MAX_LT];
  float pairSigmaPhi[TRAX_MAX_LT];  // pairSpreadPhi bit pattern read as float
  float dPhiTanLo[TRAX_MAX_LT], dPhiTanHi[TRAX_MAX_LT];  // dphi_tan_bounds of dPhiCut
  float minR[TRAX_MAX_LAYERS], maxR[TRAX_MAX_LAYERS];
  // acos(r / (2 minRadiusCurvature)) of each layer's min/max radius, computed on
  // the host with the same trax_math.h code as the kernels would
  float acosMinR[TRAX_MAX_LAYERS], acosMaxR[TRAX_MAX_LAYERS];
  // launch shape chosen by the autotuner (threads per block of the pair,
  // prediction and filter kernels; at most TRAX_MAX_TUNED_THREADS)
  uint32_t pairThreads, predThreads, filterThreads;
  uint32_t predPairsPerThread;  // 1, 2 or 4 pairs per thread in the prediction count pass
  uint32_t predKeep;            // candidates captured per pair by the count pass (4, 8, 16 or 32)
  // fine z grid of the prediction count: fineRows rows per z row of the grid
  // (0: none), fineC cells per (event, layer), fineScale = fineRows / sZ
  uint32_t fineRows, fineC;
  float fineScale;
  uint32_t nHits;               // hits of the batch (the length of every per-hit array)
  uint32_t* err;                // the context's device error word
};

#define TRAX_MAX_TUNED_THREADS 256

// Grid-ordered hit collection (the reference's HitCollection after GridBuilder).
struct DevHits {
  float* x;
  float* y;
  float* z;
  uint32_t* layer;
  uint32_t* det;
  uint32_t* hid;
  uint32_t* evt;
  uint32_t* orig;  // index of the hit in the uploaded input
  float4* xyzp;    // packed (x, y, z, phi) for the candidate loops
};

__device__ __forceinline__ void raise_error(uint32_t* err, uint32_t bit) {
  if (err) atomicOr(err, bit);
}

// A hit index that comes from data (grid offsets, pairs, candidates,
// triplets).  Bounds-checked builds (-DTRAX_BOUNDS_CHECK) record
// TRAX_EBIT_BOUNDS in the context's error word for an index outside the
// batch and read hit 0 instead, so that the call fails with
// TRAX_ERR_DEVICE_ASSERT and no access leaves the arrays; other builds use
// the index as it is.  A debugging aid where no memory checker runs.
__device__ __forceinline__ uint32_t trax_hit(uint32_t i, const DevConfig& cfg) {
#if defined(TRAX_BOUNDS_CHECK)
  if (i >= cfg.nHits) {
    raise_error(cfg.err, TRAX_EBIT_BOUNDS);
    return 0u;
  }
#endif
  return i;
}

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31u; }

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Layer-local grid read clamped to the last cell of the layer (the reference
// reads past the layer for NaN/inf windows; both sides clamp).
__device__ __forceinline__ uint32_t cell_at(const uint32_t* lGrid, uint32_t k, uint32_t C) {
  return lGrid[k < C ? k : C - 1];
}

// Maximum number of polls of a predecessor's scan status before a tile gives
// up, records TRAX_EBIT_TIMEOUT and carries on with what it has.
#define TRAX_SPIN_LIMIT (1u << 22)

// Settings of the scans' bounded waits, passed to every scan launch:
// spinLimit polls before a wait gives up (0: TRAX_SPIN_LIMIT), and a tile
// that publishes nothing (0xffffffff: none) -- a host-set fault that makes
// its successors' waits run out, for testing the timeout path.
struct WaitCtl {
  uint32_t spinLimit = 0;
  uint32_t skipTile = 0xffffffffu;
};

}  // namespace trax
