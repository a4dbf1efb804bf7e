// Test of the C++ host classes (include/trax/trax.hpp): the reference's
// stage-by-stage chain -- GridBuilder, PairGeneratorBeamspot,
// TripletThetaPhiPredictor, TripletThetaPhiFilter, TripletConnectivityTight,
// TrackletCircleFitter, CellularAutomaton -- on a synthetic batch, compared
// element by element with one batched, graph-replayed trax_seed_batch of the
// same batch on a second context.  Usage: host_classes_test <layerTriplets.xml>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "trax/trax.hpp"

namespace {

struct Lcg {
  uint64_t s;
  double uniform() {
    s = s * 6364136223846793005ull + 1442695040888963407ull;
    return (double)(s >> 11) * (1.0 / 9007199254740992.0);
  }
};

int fails = 0;
template <class A, class B>
void expect_equal(const A& a, const B& b, size_t n, const char* what) {
  for (size_t i = 0; i < n; ++i)
    if (!(a[i] == b[i])) {
      std::printf("MISMATCH %s at %zu\n", what, i);
      ++fails;
      return;
    }
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) {
    std::printf("usage: %s layerTriplets.xml\n", argv[0]);
    return 2;
  }
  const uint32_t nEvents = 6, nLayers = 4;
  const double radii[4] = {4.4, 7.3, 10.2, 25.5};
  trax::TripletConfigurations lts(1.0f);
  const uint32_t maxLayer = lts.loadTripletConfigurationFromFile(argv[1]);
  if (lts.size() != 2 || maxLayer != 4 || lts[1].layer1() != 2 || lts[0].z0() != 10.0f) {
    std::printf("layer-triplet file not read as expected\n");
    return 1;
  }
  trax::GeometrySupplement geom;
  for (uint32_t l = 0; l < nLayers; ++l) geom.addEntry(l + 1, (float)(radii[l] - 0.05), (float)(radii[l] + 0.05));

  // synthetic events: helices from the beam line plus uniform noise hits
  Lcg rng{12345};
  trax::HitCollection hits;
  for (uint32_t e = 0; e < nEvents; ++e) {
    std::vector<std::vector<double>> perLayer[4];
    const int nTracks = 40 + 10 * (int)e;
    for (int t = 0; t < nTracks; ++t) {
      const double pt = 1.0 + 4.0 * rng.uniform();
      const double R = pt / (0.299792458 * 3.8) * 100.0;
      const double phi0 = -M_PI + 2.0 * M_PI * rng.uniform();
      const double eta = -1.0 + 2.0 * rng.uniform();
      const double q = rng.uniform() < 0.5 ? -1.0 : 1.0;
      const double z0 = 5.0 * (rng.uniform() - 0.5);
      for (uint32_t l = 0; l < nLayers; ++l) {
        const double r = radii[l] + 0.04 * (rng.uniform() - 0.5);
        const double a = std::asin(r / (2.0 * R));
        const double phi = phi0 - q * a;
        const double z = z0 + std::sinh(eta) * 2.0 * R * a;
        if (std::fabs(z) > 26.0 + 40.0 * (l == 3)) continue;
        perLayer[l].push_back({r * std::cos(phi), r * std::sin(phi), z, (double)(t + 1)});
      }
    }
    for (uint32_t l = 0; l < nLayers; ++l) {
      const int noise = 8;
      for (int k = 0; k < noise; ++k) {
        const double ph = -M_PI + 2.0 * M_PI * rng.uniform();
        perLayer[l].push_back({radii[l] * std::cos(ph), radii[l] * std::sin(ph), 50.0 * (rng.uniform() - 0.5), 0.0});
      }
      for (const auto& h : perLayer[l])
        hits.addWithValue((float)h[0], (float)h[1], (float)h[2], l + 1, 1000 * (l + 1), (uint32_t)h[3], e);
    }
  }
  trax::EventSupplement es;
  trax::LayerSupplement ls;
  trax::buildSupplements(hits, nEvents, nLayers, es, ls);
  const trax::HitCollection input = hits;

  // the reference's stage-by-stage chain through the host classes
  trax::Context ctx(0);
  trax::Grid grid(trax::GridConfig(40, 100));
  trax::GridBuilder gridBuilder(ctx);
  trax::PairGeneratorBeamspot pairGen(ctx);
  trax::TripletThetaPhiPredictor predictor(ctx);
  trax::TripletThetaPhiFilter filter(ctx);
  trax::TripletConnectivityTight connectivity(ctx);
  trax::TrackletCircleFitter fitter(ctx);
  trax::CellularAutomaton ca(ctx);
  gridBuilder.run(hits, 256, es, ls, grid);
  auto pairs = pairGen.run(hits, geom, 256, lts, grid);
  trax::DetectorGeometry detGeom;
  trax::Dictionary dict;
  auto cands = predictor.run(hits, detGeom, geom, dict, 256, lts, grid, *pairs);
  auto tracklets = filter.run(hits, grid, *pairs, *cands, 256, lts);
  auto links = connectivity.run(hits, *tracklets, lts, 0.0256f, 256);
  std::unique_ptr<std::vector<float>> pt;
  std::unique_ptr<std::vector<uint32_t>> tracks, trackOffsets;
  if (links.basis) {
    pt = fitter.run(hits, *tracklets, *links.connectable, 256);
    std::tie(tracks, trackOffsets) = ca.run(*links.basis, *links.follower, *pt, *links.connectable, 256);
  }

  // the same batch in one batched call on a second context
  trax::Context ctx2(0);
  trax_ctx* c2 = ctx2.get();
  const trax_hits_soa soa = input.soa();
  ctx2.check(trax_set_layer_triplets(c2, lts.rows().data(), (int)lts.size(), lts.minPt()));
  ctx2.check(trax_set_geometry(c2, geom.minR().data(), geom.maxR().data(), (int)geom.size()));
  ctx2.check(trax_set_grid(c2, 40, 100));
  ctx2.check(trax_upload_hits(c2, &soa, (uint32_t)input.size(), es.offset.data(), ls.nHits.data(), ls.offset.data(),
                              nEvents, nLayers));
  trax_batch_opts opts{1, 1, 0.0256f};
  trax_batch_stats st;
  ctx2.check(trax_seed_batch(c2, &opts, &st));
  const size_t nOff = (size_t)nEvents * lts.size() + 1;
  std::vector<uint32_t> p2(2 * st.n_pairs), po2(nOff), cd2(2 * st.n_candidates), co2(nOff);
  std::vector<uint32_t> t1(st.n_triplets), t2(st.n_triplets), t3(st.n_triplets), to2(nOff);
  ctx2.check(trax_get_pairs(c2, p2.data(), po2.data()));
  ctx2.check(trax_get_candidates(c2, cd2.data(), co2.data()));
  ctx2.check(trax_get_triplets(c2, t1.data(), t2.data(), t3.data(), to2.data()));

  if (pairs->pairing.size() != st.n_pairs || cands->pairing.size() != st.n_candidates ||
      tracklets->size() != st.n_triplets) {
    std::printf("MISMATCH sizes: pairs %zu/%llu candidates %zu/%llu triplets %zu/%llu\n", pairs->pairing.size(),
                (unsigned long long)st.n_pairs, cands->pairing.size(), (unsigned long long)st.n_candidates,
                tracklets->size(), (unsigned long long)st.n_triplets);
    return 1;
  }
  std::vector<uint32_t> p1(2 * st.n_pairs), c1(2 * st.n_candidates);
  std::memcpy(p1.data(), pairs->pairing.data(), p1.size() * 4);
  std::memcpy(c1.data(), cands->pairing.data(), c1.size() * 4);
  expect_equal(p1, p2, p1.size(), "pairs");
  expect_equal(pairs->pairingOffsets, po2, nOff, "pair offsets");
  expect_equal(c1, cd2, c1.size(), "candidates");
  expect_equal(tracklets->hit1, t1, t1.size(), "triplet hit1");
  expect_equal(tracklets->hit2, t2, t2.size(), "triplet hit2");
  expect_equal(tracklets->hit3, t3, t3.size(), "triplet hit3");
  expect_equal(tracklets->trackletOffsets, to2, nOff, "triplet offsets");
  if ((st.n_links == 0) != !links.basis) {
    std::printf("MISMATCH link presence\n");
    return 1;
  }
  if (links.basis) {
    std::vector<uint32_t> b2(st.n_links), f2(st.n_links), cn2(st.n_connectable), nc2(st.n_non_connectable);
    ctx2.check(trax_get_links(c2, b2.data(), f2.data(), cn2.data(), nc2.data()));
    expect_equal(*links.basis, b2, b2.size(), "links basis");
    expect_equal(*links.follower, f2, f2.size(), "links follower");
    expect_equal(*links.connectable, cn2, cn2.size(), "connectable");
    std::vector<uint32_t> states(st.n_triplets), tr2(st.n_track_entries), tro2(st.n_triplets + 1);
    ctx2.check(trax_get_tracks(c2, states.data(), tr2.data(), tro2.data()));
    expect_equal(*tracks, tr2, tr2.size(), "tracks");
    expect_equal(*trackOffsets, tro2, tro2.size(), "track offsets");
  }
  // grid order: the host collection was reordered like the reference's download
  for (size_t i = 0; i < hits.size(); ++i)
    if (hits.x[i] != input.x[hits.inputIndex[i]] || hits.layer[i] != input.layer[hits.inputIndex[i]]) {
      std::printf("MISMATCH grid-ordered hit %zu\n", i);
      ++fails;
      break;
    }
  // PrefixSum
  trax::PrefixSum scan(ctx);
  std::vector<uint32_t> v(5000);
  for (size_t i = 0; i < v.size(); ++i) v[i] = (uint32_t)(i % 7);
  std::vector<uint32_t> want(v.size());
  uint32_t run = 0;
  for (size_t i = 0; i < v.size(); ++i) {
    want[i] = run;
    run += v[i];
  }
  scan.run(v);
  expect_equal(v, want, v.size(), "prefix sum");
  // an out-of-order call throws with the C status code
  try {
    trax::Context ctx3(0);
    trax::TripletThetaPhiFilter f3(ctx3);
    trax::Pairing none;
    f3.run(hits, grid, none, none, 256, lts);
    std::printf("MISMATCH no error for a filter without candidates\n");
    ++fails;
  } catch (const trax::Error& e) {
    if (e.code() != TRAX_ERR_STATE) ++fails;
  }
  if (fails) return 1;
  std::printf("OK host classes: %zu hits, %llu pairs, %llu candidates, %llu triplets, %llu links, %llu track entries\n",
              hits.size(), (unsigned long long)st.n_pairs, (unsigned long long)st.n_candidates,
              (unsigned long long)st.n_triplets, (unsigned long long)st.n_links,
              (unsigned long long)st.n_track_entries);
  return 0;
}
