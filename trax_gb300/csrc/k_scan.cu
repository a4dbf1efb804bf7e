// k_scan.cu -- single-pass exclusive uint32 scan with decoupled look-back,
// the compaction primitive between the stages (the reference's PrefixSum:
// PrefixSum.h:58-248 recursive Blelloch scan, PrefixSum.cpp:73-140).
//
// One CTA scans one tile of SCAN_THREADS * SCAN_ITEMS elements.  Tiles are
// numbered by an atomic ticket in launch order, publish their aggregate, and
// look back over predecessors (a warp reads 32 status words at a time) until
// one with an inclusive prefix is found.  Every wait is bounded: after
// TRAX_SPIN_LIMIT polls the tile records TRAX_EBIT_TIMEOUT, treats the
// missing predecessor as zero and finishes, so a lost tile can never hang
// the GPU.
#include "trax_kernels.h"
#include "trax_lookback.cuh"

namespace trax {

namespace {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 16;
constexpr uint32_t SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__global__ void __launch_bounds__(SCAN_THREADS)
    scan_kernel(const uint32_t* __restrict__ in, uint32_t* out, uint64_t nHost, const uint32_t* nDev,
                uint32_t nAdd, unsigned long long* status, uint32_t* ticket, uint32_t* err, uint32_t overflowBit,
                WaitCtl ctl) {
  __shared__ uint32_t s_tile;
  __shared__ uint32_t s_warp[SCAN_THREADS / 32];
  __shared__ unsigned long long s_wide[SCAN_THREADS / 32];
  __shared__ uint32_t s_prefix;
  const uint64_t n = nDev ? (uint64_t)(*nDev) + nAdd : nHost;
  if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
  __syncthreads();
  const uint32_t tile = s_tile;
  const uint64_t base = (uint64_t)tile * SCAN_TILE;
  if (base >= n) return;  // successors of this tile do not exist either
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t v[SCAN_ITEMS];
  const uint64_t i0 = base + (uint64_t)threadIdx.x * SCAN_ITEMS;
  if (i0 + SCAN_ITEMS <= n && ((reinterpret_cast<uintptr_t>(in) & 15u) == 0)) {
    const uint4* p = reinterpret_cast<const uint4*>(in + i0);
#pragma unroll
    for (int q = 0; q < SCAN_ITEMS / 4; ++q) {
      const uint4 a = p[q];
      v[4 * q] = a.x;
      v[4 * q + 1] = a.y;
      v[4 * q + 2] = a.z;
      v[4 * q + 3] = a.w;
    }
  } else {
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) v[k] = (i0 + k < n) ? in[i0 + k] : 0u;
  }
  uint32_t sum = 0;
  unsigned long long wide = 0;  // exact thread sum, for the tile aggregate
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    uint32_t t = v[k];
    v[k] = sum;
    sum += t;
    wide += t;
  }
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) wide += __shfl_down_sync(0xffffffffu, wide, d);
  // block-wide exclusive scan of the per-thread sums
  uint32_t incl = sum;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    uint32_t t = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= (uint32_t)d) incl += t;
  }
  if (lane == 31) s_warp[warp] = incl;
  if (lane == 0) s_wide[warp] = wide;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = (lane < SCAN_THREADS / 32) ? s_warp[lane] : 0u;
    uint32_t wi = w;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      uint32_t t = __shfl_up_sync(0xffffffffu, wi, d);
      if (lane >= (uint32_t)d) wi += t;
    }
    if (lane < SCAN_THREADS / 32) s_warp[lane] = wi - w;  // exclusive warp offsets
    unsigned long long agg = (lane < SCAN_THREADS / 32) ? s_wide[lane] : 0ull;
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) agg += __shfl_down_sync(0xffffffffu, agg, d);
    agg = __shfl_sync(0xffffffffu, agg, 0);
    // publish and look back (bounded waits); the 32-bit outputs wrap like the
    // reference's uint scan, the exact total flags a count past 2^32
    const unsigned long long excl = lb_exclusive_prefix(status, tile, agg, err, ctl);
    if (lane == 0) {
      s_prefix = (uint32_t)excl;
      if (overflowBit && excl + agg > 0xffffffffull) raise_error(err, overflowBit);
    }
  }
  __syncthreads();
  const uint32_t off = s_prefix + s_warp[warp] + (incl - sum);
  if (i0 + SCAN_ITEMS <= n && ((reinterpret_cast<uintptr_t>(out) & 15u) == 0)) {
    uint4* p = reinterpret_cast<uint4*>(out + i0);
#pragma unroll
    for (int q = 0; q < SCAN_ITEMS / 4; ++q)
      p[q] = make_uint4(off + v[4 * q], off + v[4 * q + 1], off + v[4 * q + 2], off + v[4 * q + 3]);
  } else {
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k)
      if (i0 + k < n) out[i0 + k] = off + v[k];
  }
}

// Inclusive running maximum, one CTA (the serial semantics of the offset
// monotonize kernels, TripletThetaPhiFilter.h:267-280).
__global__ void __launch_bounds__(1024) max_scan_kernel(uint32_t* data, uint32_t n) {
  __shared__ uint32_t s_w[32];
  __shared__ uint32_t s_carry;
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  for (uint32_t b = 0; b < n; b += blockDim.x) {
    uint32_t i = b + threadIdx.x;
    uint32_t v = i < n ? data[i] : 0u;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      uint32_t t = __shfl_up_sync(0xffffffffu, v, d);
      if (lane >= (uint32_t)d) v = max(v, t);
    }
    if (lane == 31) s_w[warp] = v;
    __syncthreads();
    if (warp == 0) {
      uint32_t w = (lane < blockDim.x / 32) ? s_w[lane] : 0u;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, w, d);
        if (lane >= (uint32_t)d) w = max(w, t);
      }
      s_w[lane] = w;
    }
    __syncthreads();
    uint32_t pre = (warp > 0) ? s_w[warp - 1] : 0u;
    uint32_t r = max(max(v, pre), s_carry);
    if (i < n) data[i] = r;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) s_carry = r;
    __syncthreads();
  }
}

// dst = data[n] with n = *nDev (or nHost), clamped to cap
__global__ void publish_kernel(const uint32_t* data, const uint32_t* nDev, uint32_t nHost, uint32_t cap,
                               uint32_t* dst, uint32_t* err) {
  const uint32_t n = nDev ? *nDev : nHost;
  uint32_t v = data[n];
  if (v > cap) {
    v = cap;
    raise_error(err, TRAX_EBIT_CAPACITY);
  }
  *dst = v;
}

}  // namespace

cudaError_t publish_total(const uint32_t* data, const uint32_t* nDev, uint64_t nHost, uint64_t cap, uint32_t* dst,
                          uint32_t* err, cudaStream_t st, uint32_t* launches) {
  const uint32_t c = cap > 0xffffffffull ? 0xffffffffu : (uint32_t)cap;
  publish_kernel<<<1, 1, 0, st>>>(data, nDev, (uint32_t)nHost, c, dst, err);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

size_t scan_scratch_bytes(uint64_t maxN) {
  uint64_t tiles = (maxN + SCAN_TILE - 1) / SCAN_TILE + 1;
  return 256 + tiles * sizeof(unsigned long long);
}

cudaError_t scan_exclusive(const uint32_t* in, uint32_t* out, uint64_t n, const uint32_t* nDev, uint32_t nAdd,
                           uint64_t maxN, void* scratch, uint32_t* err, cudaStream_t st, uint32_t* launches,
                           bool flagOverflow, WaitCtl ctl) {
  uint64_t cap = nDev ? maxN : n;
  if (cap == 0) return cudaSuccess;
  uint64_t tiles = (cap + SCAN_TILE - 1) / SCAN_TILE;
  size_t bytes = 256 + tiles * sizeof(unsigned long long);
  cudaError_t e = cudaMemsetAsync(scratch, 0, bytes, st);
  if (e != cudaSuccess) return e;
  uint32_t* ticket = reinterpret_cast<uint32_t*>(scratch);
  unsigned long long* status = reinterpret_cast<unsigned long long*>(static_cast<char*>(scratch) + 256);
  scan_kernel<<<(unsigned)tiles, SCAN_THREADS, 0, st>>>(in, out, n, nDev, nAdd, status, ticket, err,
                                                        flagOverflow ? TRAX_EBIT_OVERFLOW : 0u, ctl);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

cudaError_t max_scan_inclusive(uint32_t* data, uint32_t n, cudaStream_t st, uint32_t* launches) {
  if (n == 0) return cudaSuccess;
  max_scan_kernel<<<1, 1024, 0, st>>>(data, n);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

}  // namespace trax

// ------------------------------------------------------------------------
// Allocation-free prefix sum for callers that cannot allocate device memory
// (see trax_prefix_sum_noalloc in include/trax/trax.h).
//
// The single-pass scan needs scratch besides its input and output: a tile
// ticket, an error word and one look-back status word per tile.  Here that
// scratch is a fixed file-scope device array, so the call itself never
// allocates.  It is sized for TRAX_NOALLOC_SCAN_MAX elements and, like any
// __device__ variable, lives on every GPU that loads this library until the
// process exits.  All calls share it: each call clears the part it uses
// before its kernel runs, and two calls whose work overlaps on the GPU (on
// different streams, or from different host threads) race on it.
#include <atomic>
#include <cstdio>

#include "trax/trax.h"

namespace {

constexpr uint64_t NOALLOC_TILES = (TRAX_NOALLOC_SCAN_MAX + trax::SCAN_TILE - 1) / trax::SCAN_TILE;
constexpr size_t NOALLOC_HEADER = 256;  // ticket at byte 0, error word at byte 4
constexpr size_t NOALLOC_BYTES = NOALLOC_HEADER + NOALLOC_TILES * sizeof(unsigned long long);

static __device__ __align__(256) unsigned char g_noalloc_scan_scratch[NOALLOC_BYTES];

// The no-alloc scan's wait settings (trax_noalloc_set_wait), process-wide.
std::atomic<uint32_t> g_noalloc_spin{0}, g_noalloc_skip{0xffffffffu};

trax::WaitCtl noalloc_wait() {
  trax::WaitCtl w;
  w.spinLimit = g_noalloc_spin.load();
  w.skipTile = g_noalloc_skip.load();
  return w;
}

void noalloc_msg(char* buf, size_t len, const char* msg) {
  if (buf && len) {
    snprintf(buf, len, "%s", msg);
  }
}

}  // namespace

extern "C" int trax_prefix_sum_noalloc(const uint32_t* d_in, uint32_t* d_out, uint64_t n, void* stream,
                                       char* err_msg, size_t err_len) {
  noalloc_msg(err_msg, err_len, "");
  if (n == 0) return TRAX_OK;
  if (!d_in || !d_out) {
    noalloc_msg(err_msg, err_len, "trax_prefix_sum_noalloc: null device pointer");
    return TRAX_ERR_ARG;
  }
  if (n > TRAX_NOALLOC_SCAN_MAX) {
    char b[160];
    snprintf(b, sizeof b, "trax_prefix_sum_noalloc: %llu elements exceed the fixed scratch limit of %llu",
             (unsigned long long)n, (unsigned long long)TRAX_NOALLOC_SCAN_MAX);
    noalloc_msg(err_msg, err_len, b);
    return TRAX_ERR_ARG;
  }
  // The array's device address, looked up on every call: an address belongs
  // to a CUDA context, not to a device, so a cached one would be wrong after
  // the caller resets the device or makes another context current.  Host code
  // may not use the symbol itself as a device pointer.  The lookup is cheap
  // next to the stream synchronisation below; the first one in a context also
  // loads this library's device code there.
  void* base = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&base, g_noalloc_scan_scratch);
  if (e != cudaSuccess || !base) {
    char b[200];
    snprintf(b, sizeof b, "trax_prefix_sum_noalloc: cudaGetSymbolAddress failed (%s)",
             e != cudaSuccess ? cudaGetErrorString(e) : "null address");
    noalloc_msg(err_msg, err_len, b);
    return TRAX_ERR_CUDA;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const uint64_t tiles = (n + trax::SCAN_TILE - 1) / trax::SCAN_TILE;
  uint32_t* ticket = static_cast<uint32_t*>(base);
  uint32_t* err = ticket + 1;
  unsigned long long* status = reinterpret_cast<unsigned long long*>(static_cast<char*>(base) + NOALLOC_HEADER);
  // the ticket, the error word and the status words of this call start at zero
  e = cudaMemsetAsync(base, 0, NOALLOC_HEADER + tiles * sizeof(unsigned long long), st);
  if (e == cudaSuccess) {
    trax::scan_kernel<<<(unsigned)tiles, trax::SCAN_THREADS, 0, st>>>(d_in, d_out, n, nullptr, 0, status, ticket,
                                                                      err, 0u, noalloc_wait());
    e = cudaGetLastError();
  }
  uint32_t hostErr = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&hostErr, err, sizeof(hostErr), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    noalloc_msg(err_msg, err_len, cudaGetErrorString(e));
    return TRAX_ERR_CUDA;
  }
  if (hostErr & TRAX_EBIT_TIMEOUT) {
    noalloc_msg(err_msg, err_len, "trax_prefix_sum_noalloc: a bounded look-back wait ran out");
    return TRAX_ERR_TIMEOUT;
  }
  return TRAX_OK;
}

extern "C" int trax_noalloc_set_wait(uint32_t polls, uint32_t skip_tile) {
  g_noalloc_spin.store(polls);
  g_noalloc_skip.store(skip_tile);
  return TRAX_OK;
}
