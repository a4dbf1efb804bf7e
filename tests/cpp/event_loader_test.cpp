// Test of the C++ loader classes (include/trax/trax.hpp): trax::EventFile and
// trax::addEvents on a PEventContainer file, with the layer triplets given by
// a layerTriplets.xml.  Prints the loaded sizes and the columns, one value
// per line, for the Python side to compare with the C ABI's loader.  Usage:
// event_loader_test <events.pb> <layerTriplets.xml> <minPt> <numTracks> <onlyTracks>
#include <cstdio>
#include <cstdlib>

#include "trax/trax.hpp"

int main(int argc, char** argv) {
  if (argc < 6) {
    std::printf("usage: %s events.pb layerTriplets.xml minPt numTracks onlyTracks\n", argv[0]);
    return 2;
  }
  try {
    trax::EventFile file(argv[1]);
    trax::TripletConfigurations lts((float)std::atof(argv[3]));
    lts.loadTripletConfigurationFromFile(argv[2]);
    trax::HitCollection hits;
    trax::EventSupplement es;
    trax::LayerSupplement ls;
    const auto findable =
        trax::addEvents(file, 0, file.size(), lts, std::atoi(argv[4]), std::atoi(argv[5]) != 0, hits, es, ls);
    std::printf("SIZES %zu %u %u %zu\n", hits.size(), es.nEvents(), ls.nLayers, findable.size());
    for (size_t i = 0; i < hits.size(); ++i)
      std::printf("HIT %.9g %.9g %.9g %u %u %u %u\n", hits.x[i], hits.y[i], hits.z[i], hits.layer[i], hits.detId[i],
                  hits.hitId[i], hits.event[i]);
    for (size_t k = 0; k < ls.nHits.size(); ++k) std::printf("LAYER %u %u\n", ls.nHits[k], ls.offset[k]);
    for (uint32_t e = 0; e < es.nEvents(); ++e) std::printf("EVENT %u\n", es.offset[e]);
    for (const auto& f : findable) std::printf("FINDABLE %u %u\n", f.first, f.second);
  } catch (const trax::Error& e) {
    std::printf("ERROR %d %s\n", e.code(), e.what());
    return 1;
  }
  return 0;
}
