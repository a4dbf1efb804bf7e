// k_grid.cu -- per-(event, layer) z/phi grid and grid-ordered hit collection.
//
// Replaces gridCount / PrefixSum / gridStore (GridBuilder.h:48-427,
// GridBuilder.cpp:6-161).  One CTA owns one (event, layer): it histograms its
// hits into shared-memory cell counters, scans them in the CTA (the offset of
// the layer inside the event batch is known from the supplements, so the
// global scan of the reference reduces to base + local scan), places every
// hit at a STABLE slot (hits keep their input order inside a cell, one of
// the orders the reference's atomic_inc can produce) and finally gathers the
// seven hit columns into cell order with coalesced stores.  The cell, phi and
// slot of every hit stay in shared memory next to the counters when the
// largest layer fits, else in global scratch.  It also writes
// the packed (x, y, z, phi) array the candidate loops read with one 16-byte
// load, phi being the same atan2 the cell assignment used.  With
// cfg.fineRows > 0 a second kernel sorts each z row's hits again by a finer
// z grid for the prediction count (fine_grid_kernel).
#include <algorithm>

#include "trax_kernels.h"
#include "trax_stages.cuh"

namespace trax {

namespace {

constexpr int GRID_THREADS = 256;
constexpr int GRID_WARPS = GRID_THREADS / 32;
// cell counters live in shared memory up to TRAX_GRID_SMEM_CELLS cells (208 KB,
// one CTA per SM at the largest grids); larger grids count in global memory
constexpr uint32_t GRID_SMEM_CELLS = TRAX_GRID_SMEM_CELLS;
// dynamic shared memory a CTA may use: the counters plus, when they fit, the
// cell, phi and slot of each of the layer's hits (12 bytes per hit)
constexpr size_t GRID_SMEM_MAX = TRAX_GRID_SMEM_BYTES;

// The CTA's exclusive scan of C cell counters in place: cnt[c] becomes the
// first slot of cell c.  Each thread sums a chunk of consecutive cells,
// warps scan the sums with shuffles, and the chunks are rewritten.
__device__ __forceinline__ void cta_cell_scan(uint32_t* cnt, uint32_t C, uint32_t* s_warpSum) {
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
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
}

// Stable placement of n hits by cell: a slot per hit from the cell cursors
// cnt (atomics, any order inside a cell), then every cell's slots sorted by
// the hits' positions i.  After the atomics cnt[c] is the end of cell c,
// and so the start of cell c + 1.
__device__ __forceinline__ void cta_place_stable(uint32_t* cnt, uint32_t C, const uint32_t* cellOf, uint32_t* perm,
                                                 uint32_t n) {
  const uint32_t tid = threadIdx.x;
  for (uint32_t i = tid; i < n; i += GRID_THREADS) perm[atomicAdd(&cnt[cellOf[i]], 1u)] = i;
  __syncthreads();
  for (uint32_t c = tid; c < C; c += GRID_THREADS) {
    const uint32_t lo = c ? cnt[c - 1] : 0u, hi = cnt[c];
    if (hi - lo < 2) continue;
    for (uint32_t a = lo + 1; a < hi; ++a) {  // insertion sort: cells hold a few hits
      const uint32_t v = perm[a];
      uint32_t b = a;
      while (b > lo && perm[b - 1] > v) {
        perm[b] = perm[b - 1];
        --b;
      }
      perm[b] = v;
    }
  }
  __syncthreads();
}

// The per-hit cell, phi and slot arrays are in shared memory after the
// counters when the layer has at most maxHits hits (the room the launch
// gave them), otherwise in the global scratch arrays.
__global__ void __launch_bounds__(GRID_THREADS)
    grid_kernel(DevConfig cfg, GridInput in, uint32_t* __restrict__ grid, DevHits out, GridScratch sc,
                uint32_t* err, int useSmem, uint32_t maxHits) {
  extern __shared__ uint32_t smem[];
  __shared__ uint32_t s_warpSum[GRID_WARPS];
  const uint32_t task = blockIdx.x;  // event * L + layer
  const uint32_t e = task / cfg.L;
  const uint32_t C = cfg.C;
  const uint32_t n = in.layerHits[task];
  const uint32_t base = in.eventOffsets[e] + in.layerOffsets[task];
  uint32_t* cnt = useSmem ? smem : sc.counts + (size_t)task * C;
  // per-hit arrays, indexed by the hit's position i in the layer
  const bool inSmem = useSmem && n <= maxHits;
  uint32_t* cellOf = inSmem ? smem + C : sc.cell + base;
  float* phiOf = inSmem ? reinterpret_cast<float*>(smem + C + maxHits) : sc.phi + base;
  uint32_t* perm = inSmem ? smem + C + 2 * maxHits : sc.perm + base;
  const uint32_t tid = threadIdx.x;

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
    cellOf[i] = cell;
    phiOf[i] = phi;
    atomicAdd(&cnt[cell], 1u);
  }
  __syncthreads();

  // 2. CTA exclusive scan of the counters; write the grid boundaries
  cta_cell_scan(cnt, C, s_warpSum);
  // the boundaries, written with consecutive threads on consecutive cells
  uint32_t* gl = grid + (size_t)task * C;
  for (uint32_t c = tid; c < C; c += GRID_THREADS) gl[c] = base + cnt[c];
  __syncthreads();

  // 3. placement: a slot per hit from the cell cursors (shared-memory
  //    atomics, any order inside a cell), then every cell's slots sorted by
  //    input index -- the stable order, one of the orders the reference's
  //    atomic_inc can produce.
  cta_place_stable(cnt, C, cellOf, perm, n);

  // 4. gather into cell order (gridStore, GridBuilder.h:243-253)
  for (uint32_t s = tid; s < n; s += GRID_THREADS) {
    const uint32_t dst = base + s;
    const uint32_t i = perm[s];
    const uint32_t src = base + i;
    const float x = in.x[src], y = in.y[src], z = in.z[src];
    out.x[dst] = x;
    out.y[dst] = y;
    out.z[dst] = z;
    out.layer[dst] = in.layer[src];
    out.det[dst] = in.det[src];
    out.hid[dst] = in.hid[src];
    out.evt[dst] = in.evt[src];
    out.orig[dst] = src;
    out.xyzp[dst] = make_float4(x, y, z, phiOf[i]);
  }
}

// The same for layers of fewer than 65 536 hits and grids of fewer than
// 65 536 cells, in about half the shared memory, so that more CTAs share an
// SM: the cell counters are 16-bit halves of 32-bit words (two cells per
// word; a counter never passes the layer's hit count, so a half never
// carries into the other), and each hit's cell and slot are 16-bit.  The
// layout: phi [maxHits] f32, counters [(C + 1) / 2] u32, cell [maxHits] u16,
// slot [maxHits] u16.  A layer with more than maxHits hits keeps its per-hit
// arrays in global scratch.
__device__ __forceinline__ uint32_t half_of(uint32_t word, uint32_t c) { return (word >> ((c & 1u) * 16u)) & 0xffffu; }

__global__ void __launch_bounds__(GRID_THREADS)
    grid_kernel16(DevConfig cfg, GridInput in, uint32_t* __restrict__ grid, DevHits out, GridScratch sc,
                  uint32_t* err, uint32_t maxHits) {
  extern __shared__ uint32_t smem[];
  __shared__ uint32_t s_warpSum[GRID_WARPS];
  const uint32_t task = blockIdx.x;  // event * L + layer
  const uint32_t e = task / cfg.L;
  const uint32_t C = cfg.C, W = (C + 1) / 2;
  const uint32_t n = in.layerHits[task];
  const uint32_t base = in.eventOffsets[e] + in.layerOffsets[task];
  float* phiS = reinterpret_cast<float*>(smem);
  uint32_t* cnt = smem + maxHits;  // two 16-bit counters per word
  uint16_t* cellS = reinterpret_cast<uint16_t*>(cnt + W);
  uint16_t* permS = cellS + maxHits;
  const bool inSmem = n <= maxHits;
  const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
  if (n > 0xffffu) {
    // 16-bit counters cannot hold this layer (the launch is chosen for
    // layers below 65 536 hits): flag it and leave a consistent layer --
    // no cell holds a hit, the hits in input order
    if (tid == 0) raise_error(err, TRAX_EBIT_BOUNDS);
    uint32_t* gl = grid + (size_t)task * C;
    for (uint32_t c = tid; c < C; c += GRID_THREADS) gl[c] = base;
    for (uint32_t s = tid; s < n; s += GRID_THREADS) {
      const uint32_t k = base + s;
      const float x = in.x[k], y = in.y[k], z = in.z[k];
      out.x[k] = x;
      out.y[k] = y;
      out.z[k] = z;
      out.layer[k] = in.layer[k];
      out.det[k] = in.det[k];
      out.hid[k] = in.hid[k];
      out.evt[k] = in.evt[k];
      out.orig[k] = k;
      out.xyzp[k] = make_float4(x, y, z, 0.0f);
    }
    return;
  }

  for (uint32_t w = tid; w < W; w += GRID_THREADS) cnt[w] = 0u;
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
    if (inSmem) {
      cellS[i] = (uint16_t)cell;
      phiS[i] = phi;
    } else {
      sc.cell[k] = cell;
      sc.phi[k] = phi;
    }
    atomicAdd(&cnt[cell >> 1], 1u << ((cell & 1u) * 16u));
  }
  __syncthreads();

  // 2. CTA exclusive scan of the counters over whole words per thread;
  //    write the grid boundaries
  const uint32_t chunkW = (W + GRID_THREADS - 1) / GRID_THREADS;
  const uint32_t w0 = min(tid * chunkW, W), w1 = min(w0 + chunkW, W);
  uint32_t local = 0;
  for (uint32_t w = w0; w < w1; ++w) {
    const uint32_t v = cnt[w];
    local += (v & 0xffffu) + (v >> 16);
  }
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
  for (uint32_t w = w0; w < w1; ++w) {
    const uint32_t v = cnt[w];
    const uint32_t lo = run, hi = run + (v & 0xffffu);  // the next free slots of cells 2w and 2w + 1
    cnt[w] = lo | (hi << 16);
    run = hi + (v >> 16);
  }
  __syncthreads();
  // the boundaries, written with consecutive threads on consecutive cells
  uint32_t* gl = grid + (size_t)task * C;
  for (uint32_t c = tid; c < C; c += GRID_THREADS) gl[c] = base + half_of(cnt[c >> 1], c);
  __syncthreads();

  // 3. placement by the cell cursors, then the stable order inside each cell
  //    (as in grid_kernel); afterwards cursor c is the end of cell c
  if (inSmem) {
    for (uint32_t i = tid; i < n; i += GRID_THREADS) {
      const uint32_t cell = cellS[i];
      const uint32_t sh = (cell & 1u) * 16u;
      permS[(atomicAdd(&cnt[cell >> 1], 1u << sh) >> sh) & 0xffffu] = (uint16_t)i;
    }
  } else {
    for (uint32_t i = tid; i < n; i += GRID_THREADS) {
      const uint32_t cell = sc.cell[base + i];
      const uint32_t sh = (cell & 1u) * 16u;
      sc.perm[base + ((atomicAdd(&cnt[cell >> 1], 1u << sh) >> sh) & 0xffffu)] = i;
    }
  }
  __syncthreads();
  for (uint32_t c = tid; c < C; c += GRID_THREADS) {
    const uint32_t lo = c ? half_of(cnt[(c - 1) >> 1], c - 1) : 0u, hi = half_of(cnt[c >> 1], c);
    if (hi - lo < 2) continue;
    if (inSmem) {
      for (uint32_t a = lo + 1; a < hi; ++a) {  // insertion sort: cells hold a few hits
        const uint16_t v = permS[a];
        uint32_t b = a;
        while (b > lo && permS[b - 1] > v) {
          permS[b] = permS[b - 1];
          --b;
        }
        permS[b] = v;
      }
    } else {
      uint32_t* p = sc.perm + base;
      for (uint32_t a = lo + 1; a < hi; ++a) {
        const uint32_t v = p[a];
        uint32_t b = a;
        while (b > lo && p[b - 1] > v) {
          p[b] = p[b - 1];
          --b;
        }
        p[b] = v;
      }
    }
  }
  __syncthreads();

  // 4. gather into cell order (gridStore, GridBuilder.h:243-253)
  for (uint32_t s = tid; s < n; s += GRID_THREADS) {
    const uint32_t dst = base + s;
    const uint32_t i = inSmem ? (uint32_t)permS[s] : sc.perm[dst];
    const uint32_t src = base + i;
    const float x = in.x[src], y = in.y[src], z = in.z[src];
    out.x[dst] = x;
    out.y[dst] = y;
    out.z[dst] = z;
    out.layer[dst] = in.layer[src];
    out.det[dst] = in.det[src];
    out.hid[dst] = in.hid[src];
    out.evt[dst] = in.evt[src];
    out.orig[dst] = src;
    out.xyzp[dst] = make_float4(x, y, z, inSmem ? phiS[i] : sc.phi[src]);
  }
}

// The fine z grid (fine_grid_build).  A hit's fine row lies in the block of
// fineRows rows of its grid row, so the hits of one z row keep their range
// [s0, s1) of grid order in fine order: every (event, layer, z row) is
// sorted on its own, one warp each.  The warp counts the row's hits per
// fine cell (fineRows x (nP + 1) cells: the block's rows, the grid's phi
// columns), scans the counts into the fine grid's cell starts and places
// the hits 32 at a time in grid order, each after the hits of its cell
// before it (ranks among the lanes of equal cells), so ties keep grid
// order.  A hit's grid row is the row whose range holds it, and its phi
// column is recomputed with grid_kernel's operations on the same phi.
// Counters in shared memory (warpsPerBlock blocks of cells) or, when one
// block of cells does not fit, in global scratch.
__device__ __forceinline__ uint32_t fine_cell(const DevConfig& cfg, float4 h, uint32_t r) {
  const uint32_t s = fine_row(cfg, h.z, r) - r * cfg.fineRows;
  const uint32_t col = min(f2u_sat(floor_(div_(h.w - cfg.minPhi, cfg.sP))), cfg.nP);
  return s * (cfg.nP + 1) + col;
}

__global__ void __launch_bounds__(GRID_THREADS)
    fine_grid_kernel(DevConfig cfg, const uint32_t* __restrict__ grid, const float4* __restrict__ xyzp,
                     FineGrid fine, uint32_t* gcnt, uint32_t warpsPerBlock) {
  extern __shared__ uint32_t smem[];
  const uint32_t lane = threadIdx.x & 31u, wib = threadIdx.x >> 5;
  const uint32_t nZ = cfg.nZ, nP1 = cfg.nP + 1;
  const uint32_t BC = cfg.fineRows * nP1;  // fine cells of one z row
  const uint64_t task = (uint64_t)blockIdx.x * warpsPerBlock + wib;  // (event * L + layer) * nZ + row
  if (wib >= warpsPerBlock || task >= (uint64_t)cfg.E * cfg.L * nZ) return;  // no block barrier follows
  const uint32_t el = (uint32_t)(task / nZ), r = (uint32_t)(task % nZ);
  const uint32_t* lG = grid + (size_t)el * cfg.C;
  const uint32_t s0 = lG[r * nP1], s1 = lG[(r + 1) * nP1];
  uint32_t* cnt = gcnt ? gcnt + task * BC : smem + wib * BC;
  uint32_t* fG = fine.grid + (size_t)el * cfg.fineC + (size_t)r * BC;
  for (uint32_t c = lane; c < BC; c += 32) cnt[c] = 0u;
  __syncwarp();
  for (uint32_t k = s0 + lane; k < s1; k += 32) atomicAdd(&cnt[fine_cell(cfg, xyzp[k], r)], 1u);
  __syncwarp();
  // exclusive scan, 32 cells at a time: the cell starts (positions of the batch)
  uint32_t carry = s0;
  for (uint32_t c0 = 0; c0 < BC; c0 += 32) {
    const uint32_t c = c0 + lane;
    const uint32_t v = c < BC ? cnt[c] : 0u;
    uint32_t incl = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, incl, d);
      if (lane >= (uint32_t)d) incl += t;
    }
    if (c < BC) {
      cnt[c] = carry + incl - v;
      fG[c] = carry + incl - v;
    }
    carry += __shfl_sync(0xffffffffu, incl, 31);
  }
  if (r == nZ - 1)  // the row after the last holds no hit: its cells start at the layer's end
    for (uint32_t c = lane; c < nP1; c += 32) fG[BC + c] = s1;
  __syncwarp();
  const uint32_t below = (1u << lane) - 1u;
  for (uint32_t k0 = s0; k0 < s1; k0 += 32) {
    const uint32_t k = k0 + lane;
    const bool active = k < s1;
    const uint32_t mask = __ballot_sync(0xffffffffu, active);
    float4 h = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    uint32_t cell = 0, peers = 0, pos = 0;
    if (active) {
      h = xyzp[k];
      cell = fine_cell(cfg, h, r);
      peers = __match_any_sync(mask, cell);
      pos = cnt[cell] + __popc(peers & below);
    }
    __syncwarp();
    if (active) {
      if ((peers & below) == 0u) cnt[cell] += __popc(peers);  // the lowest lane of the cell moves its cursor
      fine.hits[pos] = make_float4(h.z, h.w, __uint_as_float(k), 0.0f);
    }
    __syncwarp();
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
  cudaError_t e = cudaFuncSetAttribute(grid_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)GRID_SMEM_MAX);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(grid_kernel16, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)GRID_SMEM_MAX);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(fine_grid_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)GRID_SMEM_MAX);
}

cudaError_t grid_build(const DevConfig& cfg, const GridInput& in, uint32_t* grid, DevHits out, GridScratch sc,
                       uint32_t maxLayerHits, uint32_t* err, cudaStream_t st, uint32_t* launches) {
  const uint32_t tasks = cfg.E * cfg.L;
  if (tasks == 0) return cudaSuccess;
  const int useSmem = cfg.C <= GRID_SMEM_CELLS ? 1 : 0;
  const size_t counterBytes = useSmem ? (size_t)cfg.C * sizeof(uint32_t) : 0;
  const size_t hitBytes = (size_t)maxLayerHits * 3 * sizeof(uint32_t);
  // 16-bit counters, cells and slots when every index fits
  const size_t bytes16 = (size_t)maxLayerHits * 8 + (size_t)(cfg.C + 1) / 2 * 4;
  if (useSmem && cfg.C < 65536u && maxLayerHits < 65536u && bytes16 <= GRID_SMEM_MAX) {
    grid_kernel16<<<tasks, GRID_THREADS, bytes16, st>>>(cfg, in, grid, out, sc, err, maxLayerHits);
    if (launches) *launches += 1;
    return cudaGetLastError();
  }
  const bool hitsFit = useSmem && counterBytes + hitBytes <= GRID_SMEM_MAX;
  grid_kernel<<<tasks, GRID_THREADS, counterBytes + (hitsFit ? hitBytes : 0), st>>>(
      cfg, in, grid, out, sc, err, useSmem, hitsFit ? maxLayerHits : 0u);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

cudaError_t fine_grid_build(const DevConfig& cfg, const uint32_t* grid, const float4* xyzp, FineGrid fine,
                            uint32_t* counters, cudaStream_t st, uint32_t* launches) {
  const uint64_t tasks = (uint64_t)cfg.E * cfg.L * cfg.nZ;
  if (tasks == 0 || cfg.fineRows == 0) return cudaSuccess;
  const size_t rowBytes = (size_t)fine_row_cells(cfg) * sizeof(uint32_t);
  uint32_t wpb = (uint32_t)std::min<size_t>(GRID_WARPS, GRID_SMEM_MAX / rowBytes);
  const bool inSmem = wpb > 0;
  if (!inSmem) wpb = GRID_WARPS;
  const uint64_t blocks = (tasks + wpb - 1) / wpb;
  fine_grid_kernel<<<(unsigned)blocks, wpb * 32, inSmem ? wpb * rowBytes : 0, st>>>(cfg, grid, xyzp, fine,
                                                                                     inSmem ? nullptr : counters, wpb);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

}  // namespace trax
