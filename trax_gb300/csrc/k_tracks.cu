// k_tracks.cu -- the track evaluation of TripletBuilder.cpp:840-1066 on the
// device: track extraction from the CA output, clone removal, real / fake
// tracks and the distinct real tracks.
//
// extractTracks (:951-985) turns every CA chain of three or more triplets
// into a hit list, from the outermost triplet inwards.  cloneRemoval
// (:882-907) is a greedy pass over the tracks in order: a track is compared
// with the filtered list, in list order, and the first one that shares at
// least 19 % of the shorter's hits (:846-866) decides whether it is added,
// replaces that one or is dropped.  Two tracks without a common hit never
// compare equal, so the pass splits into independent passes over the
// connected components of the "shares a hit" graph, each over its tracks in
// order: the filtered set is the union of the components' filtered sets.
// Components come from a union-find over the tracks (hooking to the smaller
// root with atomicMin, then path compression, until nothing changes); one
// thread runs the greedy pass of one component.
#include "trax_kernels.h"

namespace trax {

namespace {

constexpr uint32_t NONE = 0xFFFFFFFFu;

// chains of three or more triplets are tracks of len + 2 hits
__global__ void track_sizes_kernel(const uint32_t* __restrict__ off, uint32_t nT, uint32_t* isTrack,
                                   uint32_t* hitsOf) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i <= nT; i += gridDim.x * blockDim.x) {
    const uint32_t len = i < nT ? off[i + 1] - off[i] : 0u;
    isTrack[i] = len >= 3 ? 1u : 0u;
    hitsOf[i] = len >= 3 ? len + 2 : 0u;
  }
}

// the hit list of each track: h1, h2 of its outermost triplet, then h3 of
// every triplet from the outermost inwards (:960-975); whether all its hits
// carry one simulated track id; the smallest track holding each hit
__global__ void track_extract_kernel(const uint32_t* __restrict__ off, const uint32_t* __restrict__ chain,
                                     uint32_t nT, const uint32_t* __restrict__ h1, const uint32_t* __restrict__ h2,
                                     const uint32_t* __restrict__ h3, const uint32_t* __restrict__ hitTrack,
                                     const uint32_t* __restrict__ trackOf, const uint32_t* __restrict__ hitStart,
                                     TrackLists t) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nT; i += gridDim.x * blockDim.x) {
    const uint32_t o = off[i], len = off[i + 1] - o;
    if (len < 3) continue;
    const uint32_t k = trackOf[i], s = hitStart[i];
    t.start[k] = s;
    t.size[k] = len + 2;
    uint32_t* hits = t.hits + s;
    const uint32_t outer = chain[o + len - 1];
    hits[0] = h1[outer];
    hits[1] = h2[outer];
    for (uint32_t j = 0; j < len; ++j) hits[2 + j] = h3[chain[o + (len - 1 - j)]];
    const uint32_t first = hitTrack[hits[0]];
    bool real = true;
    for (uint32_t q = 0; q < len + 2; ++q) {
      real = real && hitTrack[hits[q]] == first;
      t.entryTrack[s + q] = k;
      atomicMin(&t.owner[hits[q]], k);
    }
    t.real[k] = real ? 1u : 0u;
    t.firstId[k] = first;
    t.parent[k] = k;
  }
}

__device__ __forceinline__ uint32_t uf_root(const uint32_t* parent, uint32_t x) {
  uint32_t p = parent[x];
  while (p != x) {
    x = p;
    p = parent[x];
  }
  return x;
}

// every track with the smallest track of each of its hits
__global__ void track_hook_kernel(TrackLists t, uint32_t nEntries, uint32_t* changed) {
  for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < nEntries; e += gridDim.x * blockDim.x) {
    const uint32_t a = uf_root(t.parent, t.entryTrack[e]), b = uf_root(t.parent, t.owner[t.hits[e]]);
    if (a != b) {
      atomicMin(&t.parent[max(a, b)], min(a, b));
      *changed = 1u;
    }
  }
}

__global__ void track_compress_kernel(TrackLists t, uint32_t nTracks) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nTracks; k += gridDim.x * blockDim.x)
    t.parent[k] = uf_root(t.parent, k);
}

// tracks per component (root), then each component's members
__global__ void track_members_kernel(TrackLists t, uint32_t nTracks, bool place) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < nTracks; k += gridDim.x * blockDim.x) {
    const uint32_t r = t.parent[k];
    if (!place) atomicAdd(&t.compSize[r], 1u);
    else t.members[t.compStart[r] + atomicAdd(&t.cursor[r], 1u)] = k;
  }
}

// the clone test of :846-866 between a new track and a filtered one
__device__ bool same_track(const TrackLists& t, uint32_t base, uint32_t other) {
  const uint32_t sb = t.size[base], so = t.size[other];
  const uint32_t longer = sb < so ? other : base, shorter = sb >= so ? other : base;
  const uint32_t* L = t.hits + t.start[longer];
  const uint32_t* S = t.hits + t.start[shorter];
  const uint32_t nl = t.size[longer], ns = t.size[shorter];
  uint32_t shared = 0;
  for (uint32_t a = 0; a < nl; ++a)
    for (uint32_t b = 0; b < ns; ++b)
      if (S[b] == L[a]) {
        ++shared;
        break;
      }
  return (float)shared / (float)ns >= 0.19f;
}

// one thread per component: its members in track order, the greedy pass of
// :882-907 over them, and the counts of the filtered tracks
__global__ void track_greedy_kernel(TrackLists t, uint32_t nTracks, unsigned long long* table, uint32_t tableMask,
                                    unsigned long long* counts) {
  for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < nTracks; r += gridDim.x * blockDim.x) {
    if (t.parent[r] != r) continue;
    const uint32_t n = t.compSize[r];
    uint32_t* m = t.members + t.compStart[r];
    uint32_t* filt = t.filtered + t.compStart[r];
    for (uint32_t a = 1; a < n; ++a) {  // track order (insertion sort: components are small)
      const uint32_t v = m[a];
      uint32_t b = a;
      while (b > 0 && m[b - 1] > v) {
        m[b] = m[b - 1];
        --b;
      }
      m[b] = v;
    }
    uint32_t nf = 0;
    for (uint32_t a = 0; a < n; ++a) {
      const uint32_t k = m[a];
      uint32_t found = NONE;
      for (uint32_t q = 0; q < nf && found == NONE; ++q)
        if (filt[q] != NONE && same_track(t, k, filt[q])) found = q;
      if (found == NONE || t.size[filt[found]] == t.size[k]) {
        filt[nf++] = k;
      } else if (t.size[filt[found]] < t.size[k]) {
        filt[found] = NONE;
        filt[nf++] = k;
      }
    }
    unsigned long long nFiltered = 0, nReal = 0, nUnique = 0;
    for (uint32_t q = 0; q < nf; ++q) {
      const uint32_t k = filt[q];
      if (k == NONE) continue;
      ++nFiltered;
      if (!t.real[k]) continue;
      ++nReal;
      // distinct simulated track ids of the real tracks: open addressing
      const unsigned long long key = (1ull << 32) | t.firstId[k];
      uint32_t h = (t.firstId[k] * 2654435761u) & tableMask;
      for (uint32_t probe = 0; probe <= tableMask; ++probe) {
        const unsigned long long old = atomicCAS(&table[h], 0ull, key);
        if (old == 0ull) {
          ++nUnique;
          break;
        }
        if (old == key) break;
        h = (h + 1) & tableMask;
      }
    }
    if (nFiltered) atomicAdd(&counts[0], nFiltered);
    if (nReal) atomicAdd(&counts[1], nReal);
    if (nUnique) atomicAdd(&counts[2], nUnique);
  }
}

int blocks_for(uint64_t n) {
  const uint64_t b = (n + 255) / 256;
  return (int)(b < 1 ? 1 : (b > 4096 ? 4096 : b));
}

}  // namespace

cudaError_t track_sizes(const uint32_t* off, uint32_t nT, uint32_t* isTrack, uint32_t* hitsOf, cudaStream_t st) {
  track_sizes_kernel<<<blocks_for(nT + 1), 256, 0, st>>>(off, nT, isTrack, hitsOf);
  return cudaGetLastError();
}

cudaError_t track_extract(const uint32_t* off, const uint32_t* chain, uint32_t nT, const uint32_t* h1,
                          const uint32_t* h2, const uint32_t* h3, const uint32_t* hitTrack, const uint32_t* trackOf,
                          const uint32_t* hitStart, TrackLists t, cudaStream_t st) {
  if (nT == 0) return cudaSuccess;
  track_extract_kernel<<<blocks_for(nT), 256, 0, st>>>(off, chain, nT, h1, h2, h3, hitTrack, trackOf, hitStart, t);
  return cudaGetLastError();
}

cudaError_t track_union_step(TrackLists t, uint32_t nTracks, uint32_t nEntries, uint32_t* changed, cudaStream_t st) {
  if (nTracks == 0) return cudaSuccess;
  track_hook_kernel<<<blocks_for(nEntries), 256, 0, st>>>(t, nEntries, changed);
  track_compress_kernel<<<blocks_for(nTracks), 256, 0, st>>>(t, nTracks);
  return cudaGetLastError();
}

cudaError_t track_members(TrackLists t, uint32_t nTracks, bool place, cudaStream_t st) {
  if (nTracks == 0) return cudaSuccess;
  track_members_kernel<<<blocks_for(nTracks), 256, 0, st>>>(t, nTracks, place);
  return cudaGetLastError();
}

cudaError_t track_greedy(TrackLists t, uint32_t nTracks, unsigned long long* table, uint32_t tableMask,
                         unsigned long long* counts, cudaStream_t st) {
  if (nTracks == 0) return cudaSuccess;
  track_greedy_kernel<<<blocks_for(nTracks), 256, 0, st>>>(t, nTracks, table, tableMask, counts);
  return cudaGetLastError();
}

}  // namespace trax
