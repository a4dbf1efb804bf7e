// The linking stages of the host classes on the caller's own inputs
// (include/trax/trax.hpp): CellularAutomaton::run (CellularAutomaton.h:43-49)
// is fed the links of the reference's four-layer connectivity fixture
// (src/algorithms/test/TripletConnectivityTest.h:66-94: triplets 0 -> 4 -> 8
// -> 12 link into one track) plus one competing link, with hand-made pt, on a
// Context that holds no triplets of its own.  Prints "OK ca inputs" and exits
// 0 when the track collection, offsets and states are the expected ones.
#include <cstdio>
#include <vector>

#include "trax/trax.hpp"

namespace {

int fails = 0;

void expect(const std::vector<uint32_t>& got, const std::vector<uint32_t>& want, const char* what) {
  if (got != want) {
    std::printf("MISMATCH %s:", what);
    for (uint32_t v : got) std::printf(" %u", v);
    std::printf("  want");
    for (uint32_t v : want) std::printf(" %u", v);
    std::printf("\n");
    ++fails;
  }
}

}  // namespace

int main() {
  trax::Context ctx(0);
  trax::CellularAutomaton ca(ctx);
  const uint32_t nT = 16;
  // the fixture's links, and triplet 1 as a second basis of triplet 4
  std::vector<uint32_t> basis = {0, 1, 4, 8};
  std::vector<uint32_t> followers = {4, 4, 8, 12};
  std::vector<uint32_t> connectable = {0, 1, 4, 8, 12};
  std::vector<float> pt(nT, 0.0f);
  pt[0] = 10.0f;
  pt[1] = 10.9f;  // closer to triplet 4's pt than triplet 0: the best basis of 4
  pt[4] = 11.0f;
  pt[8] = 12.0f;
  pt[12] = 13.0f;
  auto result = ca.run(basis, followers, pt, connectable, 256);
  const std::vector<uint32_t>& tracks = *std::get<0>(result);
  const std::vector<uint32_t>& offsets = *std::get<1>(result);
  // states: 1 everywhere but along the chain 1 -> 4 -> 8 -> 12
  std::vector<uint32_t> states(nT, 1);
  states[4] = 2;
  states[8] = 3;
  states[12] = 4;
  expect(ca.states(), states, "states");
  // handlers: triplets that are nobody's best basis, in index order, each
  // followed down its best bases; triplet 12 heads the four-triplet track
  std::vector<uint32_t> wantTracks, wantOffsets;
  for (uint32_t t = 0; t < nT; ++t) {
    wantOffsets.push_back((uint32_t)wantTracks.size());
    if (t == 1 || t == 4 || t == 8) continue;  // best bases
    if (t == 12) {
      wantTracks.insert(wantTracks.end(), {12, 8, 4, 1});
    } else {
      wantTracks.push_back(t);
    }
  }
  wantOffsets.push_back((uint32_t)wantTracks.size());
  expect(tracks, wantTracks, "tracks");
  expect(offsets, wantOffsets, "track offsets");
  // with triplet 0 closer in pt, the fixture's own chain 12 -> 8 -> 4 -> 0
  pt[0] = 10.95f;
  auto result2 = ca.run(basis, followers, pt, connectable, 256);
  const std::vector<uint32_t>& tracks2 = *std::get<0>(result2);
  const std::vector<uint32_t>& offsets2 = *std::get<1>(result2);
  const std::vector<uint32_t> chain(tracks2.begin() + offsets2[12], tracks2.begin() + offsets2[13]);
  expect(chain, std::vector<uint32_t>{12, 8, 4, 0}, "the fixture's chain");
  // a link set with a cycle is rejected with the C status code
  try {
    ca.run({0, 1, 2}, {1, 2, 0}, std::vector<float>(3, 1.0f), {}, 256);
    std::printf("MISMATCH no error for a cycle\n");
    ++fails;
  } catch (const trax::Error& e) {
    if (e.code() != TRAX_ERR_ARG) ++fails;
  }
  if (fails) return 1;
  std::printf("OK ca inputs: %zu track entries\n", tracks.size());
  return 0;
}
