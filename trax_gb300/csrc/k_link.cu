// k_link.cu -- tight triplet connectivity, circle fit and the cellular automaton.
//
// Connectivity replaces tripletEtaCalculatorStore / tripletConnectivityTightCount /
// tripletConnectivityTightStore / predicateInversionStore /
// streamCompactionGetValidIndexesStore (TripletConnectivityTight.h:47-346,
// .cpp:5-475).  The reference scans, for every basis triplet, the whole next
// layer-triplet segment; here the followers sharing the basis' two outer hits
// are found by binary search, because inside one segment the triplets are
// ordered by (second hit, first hit) -- the pair order.  The search range is
// the reference's [offsets[k], offsets[k+1]) (with its quirks: the segment
// skip of :113-115, the event check of :130-132, the monotonized offsets)
// intersected with the true segment k, outside of which no follower can
// share the basis' hits.
//
// The circle fit is trackletCircleFitterStore (TrackletCircleFitter.h:32-97).
//
// The CA replaces the host-driven iteration loop and the backward kernels of
// CellularAutomaton.{h,cpp}.  Its forward phase converges to the length of
// the longest chain of links ending at each triplet (a link only ever raises
// a follower whose state equals its basis', so a basis can never overtake
// its follower, and at the fixed point every follower sits one above its
// highest basis); links always point to a higher layer triplet, so that fixed
// point is computed exactly in one sweep over the layer triplets, with no
// host round trip.  The backward phase keeps the reference's semantics:
// candidate bases with state + 1 == follower state, minimum |pT difference|
// with select-by-multiply, scanned in link order (ascending basis index, one
// of the orders the reference's atomic_inc allows).
#include "trax_kernels.h"

namespace trax {

namespace {

int grid_for(uint64_t items, int threads) {
  uint64_t blocks = (items + threads - 1) / threads;
  uint64_t cap = (uint64_t)sm_count() * 16;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  return (int)blocks;
}

#define GRID_STRIDE(i, n) for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += gridDim.x * blockDim.x)

__global__ void eta_kernel(DevConfig cfg, const float4* __restrict__ hits, const uint32_t* __restrict__ hitEvt,
                           const uint32_t* __restrict__ hitLayer, const uint32_t* __restrict__ h1,
                           const uint32_t* __restrict__ h3, const uint32_t* nTDev, float* eta, uint32_t* seg) {
  const uint32_t nT = *nTDev;
  GRID_STRIDE(t, nT) {
    const uint32_t hi = trax_hit(h1[t], cfg), ho = trax_hit(h3[t], cfg);
    const float4 a = hits[hi], b = hits[ho];
    const float px = b.x - a.x, py = b.y - a.y, pz = b.z - a.z;
    const float tt = div_(pz, sqrt_(px * px + py * py));
    eta[t] = asinh_(tt);
    seg[t] = hitEvt[hi] * cfg.nLT + (hitLayer[hi] - 1);
  }
}

// segStart[s] = first triplet of segment s (lower bound of s in seg[])
__global__ void seg_bounds_kernel(DevConfig cfg, const uint32_t* __restrict__ seg, const uint32_t* nTDev,
                                  uint32_t* segStart) {
  const uint32_t nT = *nTDev;
  const uint32_t S = cfg.E * cfg.nLT;
  GRID_STRIDE(s, S + 1) {
    uint32_t lo = 0, hi = nT;
    while (lo < hi) {
      uint32_t mid = (lo + hi) >> 1;
      if (seg[mid] < s) lo = mid + 1;
      else hi = mid;
    }
    segStart[s] = lo;
  }
}

// first index in [lo, hi) whose (h2, h1) key is >= (k2, k1)
__device__ __forceinline__ uint32_t key_lower_bound(const uint32_t* h1, const uint32_t* h2, uint32_t lo, uint32_t hi,
                                                    uint32_t k1, uint32_t k2) {
  while (lo < hi) {
    uint32_t mid = (lo + hi) >> 1;
    uint32_t a2 = h2[mid], a1 = h1[mid];
    if (a2 < k2 || (a2 == k2 && a1 < k1)) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

template <bool EMIT>
__global__ void __launch_bounds__(256)
    conn_kernel(DevConfig cfg, const uint32_t* __restrict__ hitEvt, const uint32_t* __restrict__ hitLayer,
                const uint32_t* __restrict__ h1, const uint32_t* __restrict__ h2, const uint32_t* __restrict__ h3,
                const uint32_t* nTDev, const float* __restrict__ eta, const uint32_t* __restrict__ offsets,
                const uint32_t* __restrict__ segStart, uint32_t* linkCount, uint32_t* flags, uint32_t* runStart,
                uint32_t* basis, uint32_t* follower, uint32_t capLinks, bool sortedSegments) {
  const uint32_t S = cfg.E * cfg.nLT;
  const uint32_t nT = S > 0 ? *nTDev : 0u;
  const float dEtaCut = cfg.dEtaCut;
  GRID_STRIDE(t, nT) {
    uint32_t cnt = 0;
    uint32_t pos = 0, limit = 0;
    if (EMIT) {
      pos = linkCount[t];
      limit = linkCount[t + 1] - pos;
      if (pos >= capLinks) limit = 0;
      else if (limit > capLinks - pos) limit = capLinks - pos;
      if (limit == 0) continue;  // no links of this basis to write
    }
    bool ok = !(t >= offsets[S - 1]);  // :113-115 (nOffsets - 2 == S - 1)
    uint32_t begin = 0, end = 0, k = 0;
    const uint32_t inner = h2[t], outer = h3[t];
    if (ok) {
      const uint32_t ev = hitEvt[trax_hit(inner, cfg)];
      k = ev * cfg.nLT + (hitLayer[trax_hit(inner, cfg)] - 1);
      ok = k < S;  // the reference would read past the offsets
      if (ok) {
        begin = offsets[k];
        end = offsets[k + 1];
        // :130-132; an empty range has no follower to compare (the reference
        // reads one past its triplets there) and gives no links either way
        ok = begin < end && ev == hitEvt[trax_hit(h1[begin], cfg)];
      }
    }
    if (ok) {
      const uint32_t lo = max(begin, segStart[k]);
      const uint32_t hi = min(end, segStart[k + 1]);
      const float localEta = eta[t];
      // sorted segments: binary search to the (h2, h1) run; otherwise scan
      // the whole range like the reference (caller-provided triplets)
      // the count pass leaves the run's start for the store pass
      uint32_t first = lo;
      if (sortedSegments) {
        if (EMIT) {
          first = runStart[t];
        } else {
          first = key_lower_bound(h1, h2, lo, hi, inner, outer);
          runStart[t] = first;
        }
      }
      for (uint32_t i = first; i < hi; ++i) {
        if (h2[i] != outer || h1[i] != inner) {
          if (sortedSegments) break;
          continue;
        }
        const bool test = fabs_(localEta - eta[i]) < dEtaCut;
        if (test) {
          if (EMIT) {
            if (cnt < limit) {
              basis[pos + cnt] = t;
              follower[pos + cnt] = i;
            }
          } else {
            flags[i] = 1u;
          }
          ++cnt;
        }
      }
    }
    if (!EMIT) {
      linkCount[t] = cnt;
      if (cnt) flags[t] = 1u;
    }
  }
  if (!EMIT && blockIdx.x == 0 && threadIdx.x == 0) linkCount[nT] = 0u;
}

// The Q9 predicate streams over the first nT-1 triplets as words of 32
// flags: connectable (flag set) and non-connectable (flag clear), with the
// number set in each word (+1 slots zeroed; the number of words to
// *nWordsOut), so that the two compactions scan one value per 32 triplets.
__global__ void conn_words_kernel(const uint32_t* __restrict__ flags, const uint32_t* nTDev, uint32_t* connWords,
                                  uint32_t* connSums, uint32_t* nonWords, uint32_t* nonSums, uint32_t* nWordsOut) {
  const uint32_t nT = *nTDev;
  const uint32_t lane = threadIdx.x & 31u;
  for (uint32_t base = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < nT; base += gridDim.x * blockDim.x) {
    const uint32_t k = base + lane;
    const bool inRange = k + 1 < nT;
    const bool f = inRange && flags[k] != 0u;
    const uint32_t cw = __ballot_sync(0xffffffffu, f), nw = __ballot_sync(0xffffffffu, inRange && !f);
    if (lane == 0) {
      connWords[base >> 5] = cw;
      connSums[base >> 5] = (uint32_t)__popc(cw);
      nonWords[base >> 5] = nw;
      nonSums[base >> 5] = (uint32_t)__popc(nw);
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const uint32_t nW = (nT + 31u) >> 5;
    connSums[nW] = 0u;
    nonSums[nW] = 0u;
    *nWordsOut = nW;
  }
}

// out[wordStart[k / 32] + (bits below k in its word)] = k for every set bit
__global__ void compact_words_kernel(const uint32_t* __restrict__ words, const uint32_t* __restrict__ wordStart,
                                     const uint32_t* nTDev, uint32_t* out, uint32_t capOut) {
  const uint32_t nT = *nTDev;
  GRID_STRIDE(k, nT) {
    const uint32_t w = words[k >> 5], bit = k & 31u;
    if ((w >> bit) & 1u) {
      const uint32_t p = wordStart[k >> 5] + (uint32_t)__popc(w & ((1u << bit) - 1u));
      if (p < capOut) out[p] = k;
    }
  }
}

__global__ void circle_fit_kernel(const float4* __restrict__ hits, const uint32_t* __restrict__ h1,
                                  const uint32_t* __restrict__ h2, const uint32_t* __restrict__ h3,
                                  const uint32_t* __restrict__ conn, const uint32_t* nConnDev, float* pt) {
  const uint32_t n = *nConnDev;
  GRID_STRIDE(j, n) {
    const uint32_t t = conn[j];
    const float4 a = hits[h1[t]], b = hits[h2[t]], c = hits[h3[t]];
    const f3 pP0 = make_f3(a.x, a.y, a.x * a.x + a.y * a.y);
    const f3 pP1 = make_f3(b.x, b.y, b.x * b.x + b.y * b.y);
    const f3 pP2 = make_f3(c.x, c.y, c.x * c.x + c.y * c.y);
    const f3 n3 = cross3(sub3(pP1, pP0), sub3(pP2, pP0));
    const f3 un = normalize3(n3);
    const float cc = -dot3(un, pP0);
    const float nz2 = un.z * un.z;
    pt[t] = sqrt_(div_(1 - nz2 - 4 * cc * un.z, 4 * nz2));
  }
}

__global__ void in_degree_kernel(const uint32_t* __restrict__ follower, const uint32_t* nLinksDev, uint32_t* inDeg) {
  const uint32_t n = *nLinksDev;
  GRID_STRIDE(p, n) atomicAdd(&inDeg[follower[p]], 1u);
}

// The bases of each follower's incoming links.  Links are stored in basis
// order, so the bases of one follower (all distinct) sort like the link
// indices do.
__global__ void in_fill_kernel(const uint32_t* __restrict__ basis, const uint32_t* __restrict__ follower,
                               const uint32_t* nLinksDev, const uint32_t* __restrict__ inStart, uint32_t* cursor,
                               uint32_t* inList) {
  const uint32_t n = *nLinksDev;
  GRID_STRIDE(p, n) {
    const uint32_t f = follower[p];
    inList[inStart[f] + atomicAdd(&cursor[f], 1u)] = basis[p];
  }
}

// the incoming bases of each follower in ascending order, which is the
// order of their links (insertion sort; lists are short)
__global__ void in_sort_kernel(const uint32_t* __restrict__ inStart, const uint32_t* nTDev, uint32_t* inList) {
  const uint32_t nT = *nTDev;
  GRID_STRIDE(t, nT) {
    const uint32_t a = inStart[t], b = inStart[t + 1];
    for (uint32_t i = a + 1; i < b; ++i) {
      const uint32_t v = inList[i];
      uint32_t j = i;
      while (j > a && inList[j - 1] > v) {
        inList[j] = inList[j - 1];
        --j;
      }
      inList[j] = v;
    }
  }
}

// the CA's per-triplet state before a run: in-degrees and cursors 0,
// states 1, no best basis
__global__ void ca_init_kernel(CABuffers b, const uint32_t* nTDev) {
  const uint32_t nT = *nTDev;
  GRID_STRIDE(i, nT + 1) {
    b.inStart[i] = 0u;
    if (i < nT) {
      b.inCursor[i] = 0u;
      b.states[i] = 1u;
      b.best[i] = TRAX_SENTINEL;
      b.isBest[i] = 0u;
    }
  }
}

// one layer-triplet level of the forward phase
__global__ void ca_level_kernel(DevConfig cfg, uint32_t level, const uint32_t* __restrict__ segOf,
                                const uint32_t* __restrict__ inStart, const uint32_t* __restrict__ inList,
                                const uint32_t* nTDev, uint32_t* states) {
  const uint32_t nT = *nTDev;
  GRID_STRIDE(t, nT) {
    if (segOf[t] % cfg.nLT != level) continue;
    const uint32_t a = inStart[t], b = inStart[t + 1];
    if (a == b) continue;
    uint32_t m = 0;
    for (uint32_t j = a; j < b; ++j) m = max(m, states[inList[j]]);
    states[t] = m + 1;
  }
}

// The reference's forward iteration over any link set (`iteration`,
// CellularAutomaton.h:52-100): next[f] = max(next[f], cur[f] + (cur[b] ==
// cur[f])) for every link b -> f, and a living flag when a follower's state
// equals its basis's.  The host repeats it, swapping the buffers without
// copying (CellularAutomaton.cpp:52-98), until no cell lives.  Used for
// caller-provided links, which need not go from one layer triplet to the
// next as the chain's own do.
__global__ void ca_iteration_kernel(const uint32_t* __restrict__ basis, const uint32_t* __restrict__ follower,
                                    uint32_t nLinks, const uint32_t* __restrict__ cur, uint32_t* next,
                                    uint32_t* living) {
  GRID_STRIDE(p, nLinks) {
    const uint32_t f = follower[p];
    const uint32_t fs = cur[f];
    const uint32_t same = cur[basis[p]] == fs ? 1u : 0u;
    atomicMax(&next[f], fs + same);
    if (same) *living = 1u;
  }
}

__global__ void fill_u32_kernel(uint32_t* p, uint32_t v, uint32_t n) {
  GRID_STRIDE(i, n) p[i] = v;
}

// followerBestBasisStore semantics (CellularAutomaton.h:212-263)
__global__ void ca_best_kernel(const float* __restrict__ pt,
                               const uint32_t* __restrict__ inStart, const uint32_t* __restrict__ inList,
                               const uint32_t* __restrict__ states, const uint32_t* nTDev, uint32_t* best,
                               uint32_t* isBest) {
  const uint32_t nT = *nTDev;
  GRID_STRIDE(t, nT) {
    const uint32_t a = inStart[t], b = inStart[t + 1];
    const uint32_t sf = states[t];
    bool have = false;
    float minPt = 0.0f;
    uint32_t minIdx = 0;
    for (uint32_t j = a; j < b; ++j) {
      const uint32_t bb = inList[j];
      if (states[bb] + 1 != sf) continue;
      const float d = fabs_(pt[bb] - pt[t]);
      if (!have) {
        minPt = d;
        minIdx = bb;
        have = true;
      } else {
        const uint32_t test = d < minPt;
        minPt = minPt * (float)(!test) + d * (float)test;
        minIdx = minIdx * (!test) + bb * test;
      }
    }
    if (have) {
      best[t] = minIdx;
      isBest[minIdx] = 1u;
    }
  }
}

// handlersStateStore (CellularAutomaton.h:270-288); no tracks at all when
// there are no links (the reference skips the CA, TripletBuilder.cpp:414-421)
__global__ void handlers_kernel(const uint32_t* __restrict__ states, const uint32_t* __restrict__ isBest,
                                const uint32_t* nTDev, const uint32_t* nLinksDev, uint32_t* handlers) {
  const uint32_t nT = *nTDev;
  const bool any = *nLinksDev != 0u;
  GRID_STRIDE(t, nT + 1) handlers[t] = (any && t < nT) ? (isBest[t] == 0u) * states[t] : 0u;
}

__global__ void tracks_kernel(const uint32_t* __restrict__ handlers, const uint32_t* __restrict__ best,
                              const uint32_t* nTDev, uint32_t* tracks, uint64_t maxTracks, uint32_t* err) {
  const uint32_t nT = *nTDev;
  GRID_STRIDE(t, nT) {
    const uint32_t off = handlers[t];
    const uint32_t len = handlers[t + 1] - off;
    uint32_t b = t;
    for (uint32_t i = 0; i < len && b != TRAX_SENTINEL; ++i) {
      if ((uint64_t)off + i >= maxTracks) {
        raise_error(err, TRAX_EBIT_CAPACITY);
        break;
      }
      tracks[off + i] = b;
      b = best[b];
    }
  }
}

}  // namespace

cudaError_t triplet_eta(const DevConfig& cfg, DevHits hits, TripletView t, float* eta, uint32_t* seg, cudaStream_t st,
                        uint32_t* launches) {
  if (t.maxN == 0) return cudaSuccess;
  eta_kernel<<<grid_for(t.maxN, 256), 256, 0, st>>>(cfg, hits.xyzp, hits.evt, hits.layer, t.h1, t.h3, t.nDev, eta,
                                                    seg);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

cudaError_t segment_bounds(const DevConfig& cfg, const uint32_t* seg, const uint32_t* nTDev, uint32_t* segStart,
                           cudaStream_t st, uint32_t* launches) {
  const uint32_t S = cfg.E * cfg.nLT;
  seg_bounds_kernel<<<grid_for(S + 1, 256), 256, 0, st>>>(cfg, seg, nTDev, segStart);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

cudaError_t connectivity_tasks(const DevConfig& cfg, bool emit, DevHits hits, TripletView t, const float* eta,
                               const uint32_t* offsets, const uint32_t* segStart, uint32_t* linkCount,
                               uint32_t* flags, uint32_t* runStart, uint32_t* basis, uint32_t* follower,
                               uint64_t capLinks, bool sortedSegments, cudaStream_t st, uint32_t* launches) {
  const int blocks = grid_for(t.maxN + 1, 256);
  const uint32_t cap = capLinks > 0xffffffffull ? 0xffffffffu : (uint32_t)capLinks;
  if (emit)
    conn_kernel<true><<<blocks, 256, 0, st>>>(cfg, hits.evt, hits.layer, t.h1, t.h2, t.h3, t.nDev, eta, offsets,
                                              segStart, linkCount, flags, runStart, basis, follower, cap,
                                              sortedSegments);
  else
    conn_kernel<false><<<blocks, 256, 0, st>>>(cfg, hits.evt, hits.layer, t.h1, t.h2, t.h3, t.nDev, eta, offsets,
                                               segStart, linkCount, flags, runStart, basis, follower, cap,
                                               sortedSegments);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

cudaError_t connectable_words(const uint32_t* flags, const uint32_t* nTDev, uint64_t maxT, uint32_t* connWords,
                              uint32_t* connSums, uint32_t* nonWords, uint32_t* nonSums, uint32_t* nWordsOut,
                              cudaStream_t st, uint32_t* launches) {
  conn_words_kernel<<<grid_for(maxT + 1, 256), 256, 0, st>>>(flags, nTDev, connWords, connSums, nonWords, nonSums,
                                                             nWordsOut);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

cudaError_t compact_words(const uint32_t* words, const uint32_t* wordStart, const uint32_t* nTDev, uint64_t maxT,
                          uint32_t* outIdx, uint64_t capOut, cudaStream_t st, uint32_t* launches) {
  if (maxT == 0) return cudaSuccess;
  const uint32_t cap = capOut > 0xffffffffull ? 0xffffffffu : (uint32_t)capOut;
  compact_words_kernel<<<grid_for(maxT, 256), 256, 0, st>>>(words, wordStart, nTDev, outIdx, cap);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

cudaError_t circle_fit(DevHits hits, TripletView t, const uint32_t* connectable, const uint32_t* nConnDev,
                       uint64_t maxConn, float* pt, cudaStream_t st, uint32_t* launches) {
  if (maxConn == 0) return cudaSuccess;
  circle_fit_kernel<<<grid_for(maxConn, 256), 256, 0, st>>>(hits.xyzp, t.h1, t.h2, t.h3, connectable, nConnDev, pt);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

cudaError_t ca_in_degree(const uint32_t* follower, const uint32_t* nLinksDev, uint64_t maxLinks, CABuffers b,
                         const uint32_t* nTDev, uint64_t maxT, cudaStream_t st, uint32_t* launches) {
  ca_init_kernel<<<grid_for(maxT + 1, 256), 256, 0, st>>>(b, nTDev);
  if (launches) *launches += 1;
  if (maxLinks > 0) {
    in_degree_kernel<<<grid_for(maxLinks, 256), 256, 0, st>>>(follower, nLinksDev, b.inStart);
    if (launches) *launches += 1;
  }
  return cudaGetLastError();
}

cudaError_t ca_fill(const uint32_t* basis, const uint32_t* follower, const uint32_t* nLinksDev, uint64_t maxLinks,
                    CABuffers b, const uint32_t* nTDev, uint64_t maxT, cudaStream_t st, uint32_t* launches) {
  if (maxLinks > 0) {
    in_fill_kernel<<<grid_for(maxLinks, 256), 256, 0, st>>>(basis, follower, nLinksDev, b.inStart, b.inCursor,
                                                            b.inList);
    if (launches) *launches += 1;
  }
  in_sort_kernel<<<grid_for(maxT, 256), 256, 0, st>>>(b.inStart, nTDev, b.inList);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

cudaError_t ca_forward(const DevConfig& cfg, CABuffers b, const uint32_t* nTDev, uint64_t maxT, cudaStream_t st,
                       uint32_t* launches) {
  for (uint32_t level = 1; level < cfg.nLT; ++level) {
    ca_level_kernel<<<grid_for(maxT, 256), 256, 0, st>>>(cfg, level, b.segOf, b.inStart, b.inList, nTDev, b.states);
    if (launches) *launches += 1;
  }
  return cudaGetLastError();
}

cudaError_t ca_iteration(const uint32_t* basis, const uint32_t* follower, uint32_t nLinks, const uint32_t* cur,
                         uint32_t* next, uint32_t* living, cudaStream_t st, uint32_t* launches) {
  if (nLinks == 0) return cudaSuccess;
  ca_iteration_kernel<<<grid_for(nLinks, 256), 256, 0, st>>>(basis, follower, nLinks, cur, next, living);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

cudaError_t fill_u32(uint32_t* p, uint32_t v, uint32_t n, cudaStream_t st, uint32_t* launches) {
  if (n == 0) return cudaSuccess;
  fill_u32_kernel<<<grid_for(n, 256), 256, 0, st>>>(p, v, n);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

cudaError_t ca_backward(const float* pt, CABuffers b, const uint32_t* nTDev, uint64_t maxT,
                        const uint32_t* nLinksDev, cudaStream_t st, uint32_t* launches) {
  ca_best_kernel<<<grid_for(maxT, 256), 256, 0, st>>>(pt, b.inStart, b.inList, b.states, nTDev, b.best, b.isBest);
  handlers_kernel<<<grid_for(maxT + 1, 256), 256, 0, st>>>(b.states, b.isBest, nTDev, nLinksDev, b.handlers);
  if (launches) *launches += 2;
  return cudaGetLastError();
}

cudaError_t ca_tracks(CABuffers b, const uint32_t* nTDev, uint64_t maxT, uint32_t* tracks, uint64_t maxTracks,
                      uint32_t* err, cudaStream_t st, uint32_t* launches) {
  if (maxT == 0) return cudaSuccess;
  tracks_kernel<<<grid_for(maxT, 256), 256, 0, st>>>(b.handlers, b.best, nTDev, tracks, maxTracks, err);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

}  // namespace trax
