// k_events.cu -- the loader's layer bucketing on the device.
//
// HitCollection::addEvent (HitCollection.cpp:21-180) ends by reading its
// layer buckets out, layer by layer, each in push order, into the hit
// collection (:122-149).  The host gives every hit of an event a key
// (layer, push position, index in the event; trax_events.h) or marks it
// dropped; here one CTA per event sorts the event's keys (bitonic sort, in
// shared memory up to BUCKET_SMEM_KEYS keys, else in global scratch) and
// gathers the kept hits' columns into the context's input arrays at the
// event's offset.  Keys are distinct, so the sort needs no stability.
#include "trax_kernels.h"

namespace trax {

namespace {

constexpr int BUCKET_THREADS = 256;
constexpr uint32_t BUCKET_SMEM_KEYS = 4096;

__device__ __forceinline__ void bitonic_sort(unsigned long long* keys, uint32_t n) {
  for (uint32_t k = 2; k <= n; k <<= 1)
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const uint32_t l = i ^ j;
        if (l > i) {
          const unsigned long long a = keys[i], b = keys[l];
          if ((a > b) == ((i & k) == 0)) {
            keys[i] = b;
            keys[l] = a;
          }
        }
      }
      __syncthreads();
    }
}

__global__ void __launch_bounds__(BUCKET_THREADS)
    bucket_kernel(RawEventHits in, unsigned long long* scratch, uint32_t nKept, HitColumns out) {
  __shared__ unsigned long long s_keys[BUCKET_SMEM_KEYS];
  const uint32_t e = blockIdx.x;
  const uint32_t r0 = in.rawOffsets[e], n = in.rawOffsets[e + 1] - r0;
  const uint32_t dst0 = out.eventOffsets[e];
  const uint32_t kept = (e + 1 < gridDim.x ? out.eventOffsets[e + 1] : nKept) - dst0;
  uint32_t padded = 1;
  while (padded < n) padded <<= 1;
  unsigned long long* keys = padded <= BUCKET_SMEM_KEYS ? s_keys : scratch + in.scratchOffsets[e];
  for (uint32_t i = threadIdx.x; i < padded; i += blockDim.x) keys[i] = i < n ? in.key[r0 + i] : ~0ull;
  __syncthreads();
  bitonic_sort(keys, padded);
  for (uint32_t r = threadIdx.x; r < kept; r += blockDim.x) {
    const uint32_t src = r0 + (uint32_t)(keys[r] & 0xffffffull);
    const uint32_t dst = dst0 + r;
    out.x[dst] = in.x[src];
    out.y[dst] = in.y[src];
    out.z[dst] = in.z[src];
    out.layer[dst] = in.layer[src];
    out.det[dst] = in.det[src];
    out.hid[dst] = in.tid[src];
    out.evt[dst] = e;
  }
}

}  // namespace

uint32_t bucket_scratch_keys(uint32_t hitsInEvent) {
  uint32_t padded = 1;
  while (padded < hitsInEvent) padded <<= 1;
  return padded <= BUCKET_SMEM_KEYS ? 0u : padded;
}

cudaError_t bucket_events(const RawEventHits& in, unsigned long long* scratch, uint32_t nEvents, uint32_t nKept,
                          HitColumns out, cudaStream_t st, uint32_t* launches) {
  if (nEvents == 0) return cudaSuccess;
  bucket_kernel<<<nEvents, BUCKET_THREADS, 0, st>>>(in, scratch, nKept, out);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

}  // namespace trax
