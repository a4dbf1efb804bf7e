// k_grid.cu -- per-(event, layer) z/phi grid and grid-ordered hit collection.
//
// Replaces gridCount / PrefixSum / gridStore (GridBuilder.h:48-427,
// GridBuilder.cpp:6-161).  One CTA owns one (event, layer): it histograms its
// hits into shared-memory cell counters, scans them in the CTA (the offset of
// the layer inside the event batch is known from the supplements, so the
// global scan of the reference reduces to base + local scan), places every
// hit at a STABLE slot (hits keep their input order inside a cell, one of
// the orders the reference's atomic_inc can produce) and finally gathers the
// seven hit columns into cell order with coalesced stores.  It also writes
// the packed (x, y, z, phi) array the candidate loops read with one 16-byte
// load, phi being the same atan2 the cell assignment used.
#include "trax_kernels.h"

namespace trax {

namespace {

constexpr int GRID_THREADS = 256;
constexpr int GRID_WARPS = GRID_THREADS / 32;
// cell counters live in shared memory up to TRAX_GRID_SMEM_CELLS cells (208 KB,
// one CTA per SM at the largest grids); larger grids count in global memory
constexpr uint32_t GRID_SMEM_CELLS = TRAX_GRID_SMEM_CELLS;

__global__ void __launch_bounds__(GRID_THREADS)
    grid_kernel(DevConfig cfg, GridInput in, uint32_t* __restrict__ grid, DevHits out, GridScratch sc,
                uint32_t* err, int useSmem) {
  extern __shared__ uint32_t smem[];
  __shared__ uint32_t s_warpSum[GRID_WARPS];
  const uint32_t task = blockIdx.x;  // event * L + layer
  const uint32_t e = task / cfg.L;
  const uint32_t C = cfg.C;
  const uint32_t n = in.layerHits[task];
  const uint32_t base = in.eventOffsets[e] + in.layerOffsets[task];
  uint32_t* cnt = useSmem ? smem : sc.counts + (size_t)task * C;
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;

  for (uint32_t c = tid; c < C; c += GRID_THREADS) cnt[c] = 0u;
  __syncthreads();

  // 1. cells (gridCount, GridBuilder.h:80-87)
  for (uint32_t i = tid; i < n; i += GRID_THREADS) {
    const uint32_t k = base + i;
    const float x = in.x[k], y = in.y[k], z = in.z[k];
    uint32_t zSector = f2u_sat(floor_(div_(z - cfg.minZ, cfg.sZ)));
    float phi = atan2_(y, x);
    uint32_t phiSector = f2u_sat(floor_(div_(phi - cfg.minPhi, cfg.sP)));
    if (zSector >= cfg.nZ || phiSector > cfg.nP) {
      raise_error(err, TRAX_EBIT_BOUNDS);
      zSector = min(zSector, cfg.nZ - 1);
      phiSector = min(phiSector, cfg.nP);
    }
    const uint32_t cell = zSector * (cfg.nP + 1) + phiSector;
    sc.cell[k] = cell;
    sc.phi[k] = phi;
    atomicAdd(&cnt[cell], 1u);
  }
  __syncthreads();

  // 2. CTA exclusive scan of the counters; write the grid boundaries
  const uint32_t chunk = (C + GRID_THREADS - 1) / GRID_THREADS;
  const uint32_t c0 = min(tid * chunk, C), c1 = min(c0 + chunk, C);
  uint32_t local = 0;
  for (uint32_t c = c0; c < c1; ++c) local += cnt[c];
  uint32_t incl = local;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    uint32_t t = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= (uint32_t)d) incl += t;
  }
  if (lane == 31) s_warpSum[warp] = incl;
  __syncthreads();
  uint32_t warpOff = 0;
  for (uint32_t w = 0; w < warp; ++w) warpOff += s_warpSum[w];
  uint32_t run = warpOff + incl - local;
  __syncthreads();
  for (uint32_t c = c0; c < c1; ++c) {
    uint32_t v = cnt[c];
    cnt[c] = run;  // becomes the next free slot of the cell
    run += v;
  }
  __syncthreads();
  // the boundaries, written with consecutive threads on consecutive cells
  uint32_t* gl = grid + (size_t)task * C;
  for (uint32_t c = tid; c < C; c += GRID_THREADS) gl[c] = base + cnt[c];
  __syncthreads();

  // 3. placement: a slot per hit from the cell cursors (shared-memory
  //    atomics, any order inside a cell), then every cell's slots sorted by
  //    input index -- the stable order, one of the orders the reference's
  //    atomic_inc can produce.  After the atomics cnt[c] is the end of cell c,
  //    and so the start of cell c + 1.
  for (uint32_t i = tid; i < n; i += GRID_THREADS) {
    const uint32_t cell = sc.cell[base + i];
    sc.perm[base + atomicAdd(&cnt[cell], 1u)] = i;
  }
  __syncthreads();
  for (uint32_t c = tid; c < C; c += GRID_THREADS) {
    const uint32_t lo = c ? cnt[c - 1] : 0u, hi = cnt[c];
    if (hi - lo < 2) continue;
    uint32_t* p = sc.perm + base;
    for (uint32_t a = lo + 1; a < hi; ++a) {  // insertion sort: cells hold a few hits
      const uint32_t v = p[a];
      uint32_t b = a;
      while (b > lo && p[b - 1] > v) {
        p[b] = p[b - 1];
        --b;
      }
      p[b] = v;
    }
  }
  __syncthreads();

  // 4. gather into cell order (gridStore, GridBuilder.h:243-253)
  for (uint32_t s = tid; s < n; s += GRID_THREADS) {
    const uint32_t dst = base + s;
    const uint32_t src = base + sc.perm[dst];
    const float x = in.x[src], y = in.y[src], z = in.z[src];
    out.x[dst] = x;
    out.y[dst] = y;
    out.z[dst] = z;
    out.layer[dst] = in.layer[src];
    out.det[dst] = in.det[src];
    out.hid[dst] = in.hid[src];
    out.evt[dst] = in.evt[src];
    out.orig[dst] = src;
    out.xyzp[dst] = make_float4(x, y, z, sc.phi[src]);
  }
}

// The uploaded hits taken as the hit collection as they are (identity
// order), for the linking stages run on caller-provided triplets.
__global__ void identity_hits_kernel(GridInput in, uint32_t n, DevHits out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float x = in.x[i], y = in.y[i], z = in.z[i];
    out.x[i] = x;
    out.y[i] = y;
    out.z[i] = z;
    out.layer[i] = in.layer[i];
    out.det[i] = in.det[i];
    out.hid[i] = in.hid[i];
    out.evt[i] = in.evt[i];
    out.orig[i] = i;
    out.xyzp[i] = make_float4(x, y, z, atan2_(y, x));
  }
}

}  // namespace

cudaError_t identity_hits(const GridInput& in, uint32_t n, DevHits out, cudaStream_t st, uint32_t* launches) {
  if (n == 0) return cudaSuccess;
  identity_hits_kernel<<<(n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096, 256, 0, st>>>(in, n, out);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

cudaError_t grid_prepare(int) {
  return cudaFuncSetAttribute(grid_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)(GRID_SMEM_CELLS * sizeof(uint32_t)));
}

cudaError_t grid_build(const DevConfig& cfg, const GridInput& in, uint32_t* grid, DevHits out, GridScratch sc,
                       uint32_t* err, cudaStream_t st, uint32_t* launches) {
  const uint32_t tasks = cfg.E * cfg.L;
  if (tasks == 0) return cudaSuccess;
  const int useSmem = cfg.C <= GRID_SMEM_CELLS ? 1 : 0;
  const size_t smemBytes = useSmem ? (size_t)cfg.C * sizeof(uint32_t) : 0;
  grid_kernel<<<tasks, GRID_THREADS, smemBytes, st>>>(cfg, in, grid, out, sc, err, useSmem);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

}  // namespace trax
