// k_events.cu -- the loader's layer bucketing and the triplet physics counts
// on the device.
//
// HitCollection::addEvent (HitCollection.cpp:21-180) ends by reading its
// layer buckets out, layer by layer, each in push order, into the hit
// collection (:122-149).  The host gives every hit of an event a key
// (layer, push position, index in the event; trax_events.h) or marks it
// dropped; here one CTA per event sorts the event's keys (bitonic sort, in
// shared memory up to BUCKET_SMEM_KEYS keys, else in global scratch) and
// gathers the kept hits' columns into the context's input arrays at the
// event's offset.  Keys are distinct, so the sort needs no stability.
#include <algorithm>

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

// PhysicsRecord::fillData (PhysicsRecord.cpp:86-313) counted per triplet:
// a triplet whose three hits carry one simulated track id is real, else fake;
// a real triplet of a findable track (binary search in its event's sorted
// findable ids) marks that track found in its segment.  The segments are the
// triplet offsets' ranges, as fillData reads them: the reference's offsets
// leave the last triplet out of every range (filterOffsetStore), and so does
// this count.
__global__ void physics_triplet_kernel(const uint32_t* __restrict__ h1, const uint32_t* __restrict__ h2,
                                       const uint32_t* __restrict__ h3, const uint32_t* nTDev,
                                       const uint32_t* __restrict__ offsets, uint32_t S,
                                       const uint32_t* __restrict__ hitTrack, uint32_t nLT,
                                       const uint32_t* __restrict__ findOff, const uint32_t* __restrict__ findIds,
                                       uint32_t* fakes, uint32_t* realFindable, uint32_t* foundFlags) {
  const uint32_t nT = *nTDev;
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < nT; t += gridDim.x * blockDim.x) {
    // the segment whose range holds t: the last s with offsets[s] <= t
    uint32_t lo = 0, hi = S + 1;
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      if (offsets[mid] <= t) lo = mid + 1;
      else hi = mid;
    }
    if (lo == 0 || lo > S) continue;  // before the first range, or at or past offsets[S]
    const uint32_t seg = lo - 1;
    const uint32_t e = seg / nLT, p = seg % nLT;
    const uint32_t i1 = hitTrack[h1[t]], i2 = hitTrack[h2[t]], i3 = hitTrack[h3[t]];
    if (i1 != i2 || i1 != i3) {
      atomicAdd(&fakes[seg], 1u);
      continue;
    }
    lo = findOff[e];
    hi = findOff[e + 1];
    const uint32_t f0 = lo, nf = hi - lo;
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      if (findIds[mid] < i1) lo = mid + 1;
      else hi = mid;
    }
    if (lo < f0 + nf && findIds[lo] == i1) {
      atomicAdd(&realFindable[seg], 1u);
      foundFlags[(size_t)nLT * f0 + (size_t)p * nf + (lo - f0)] = 1u;
    }
  }
}

// distinct findable tracks found per segment
__global__ void physics_found_kernel(uint32_t S, uint32_t nLT, const uint32_t* __restrict__ findOff,
                                     const uint32_t* __restrict__ foundFlags, uint32_t* found) {
  for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < S; s += gridDim.x * blockDim.x) {
    const uint32_t e = s / nLT, p = s % nLT;
    const uint32_t f0 = findOff[e], nf = findOff[e + 1] - f0;
    const uint32_t* fl = foundFlags + (size_t)nLT * f0 + (size_t)p * nf;
    uint32_t n = 0;
    for (uint32_t q = 0; q < nf; ++q) n += fl[q];
    found[s] = n;
  }
}

}  // namespace

cudaError_t physics_counts(const uint32_t* h1, const uint32_t* h2, const uint32_t* h3, const uint32_t* nTDev,
                           uint64_t maxT, const uint32_t* offsets, const uint32_t* hitTrack, uint32_t nEvents,
                           uint32_t nLT, const uint32_t* findOff,
                           const uint32_t* findIds, uint32_t* fakes, uint32_t* realFindable, uint32_t* foundFlags,
                           uint32_t* found, cudaStream_t st, uint32_t* launches) {
  const uint32_t S = nEvents * nLT;
  if (maxT > 0) {
    const uint64_t b = std::min<uint64_t>((maxT + 255) / 256, 4096);
    physics_triplet_kernel<<<(unsigned)b, 256, 0, st>>>(h1, h2, h3, nTDev, offsets, S, hitTrack, nLT, findOff,
                                                        findIds, fakes, realFindable, foundFlags);
    if (launches) *launches += 1;
  }
  if (S > 0) {
    physics_found_kernel<<<(S + 255) / 256, 256, 0, st>>>(S, nLT, findOff, foundFlags, found);
    if (launches) *launches += 1;
  }
  return cudaGetLastError();
}

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
