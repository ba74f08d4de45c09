// Compile check of include/opensubdiv_gb300/far/gb300StencilTableFactory.h: the mask recorder
// driven the way Far::PrimvarRefiner drives a StencilBuilder::Index, and (with OpenSubdiv's
// headers) the Far-facing GB300StencilTableFactory::Create.
#ifdef FACTORY_CLIENT_WITH_FAR
#include <opensubdiv/far/topologyRefiner.h>
#endif
#include <opensubdiv_gb300/far/gb300StencilTableFactory.h>

#include <cstdio>
#include <vector>

#ifdef OSD_GB300_HAVE_OPENSUBDIV
using namespace OpenSubdiv::OPENSUBDIV_VERSION;
#else
using namespace OpenSubdiv;
#endif

// One "level": child 0 = face point of control vertices 0..3, child 1 = its own face point
// plus two control vertices (a same-level reference, as Catmark edge points make).
int record_example(std::vector<int64_t> &off, std::vector<int> &src, std::vector<float> &w) {
    Osd::GB300MaskRecorder rec;
    Osd::GB300MaskRecorder::Index control(&rec, 0), level(&rec, 4);
    level[0].Clear();
    for (int i = 0; i < 4; ++i) level[0].AddWithWeight(control[i], 0.25f);
    level[1].Clear();
    level[1].AddWithWeight(control[0], 0.25f);
    level[1].AddWithWeight(control[1], 0.25f);
    level[1].AddWithWeight(level[0], 0.5f);
    level[1].AddWithWeight(control[2], 0.0f);  // dropped, like StencilBuilder
    return rec.GetMasks(4, 2, off, src, w) ? (int)src.size() : -1;
}

#ifdef OSD_GB300_HAVE_FAR
Osd::GB300StencilTable *build(Far::TopologyRefiner const &refiner) {
    Osd::GB300StencilTableFactory::Options o;
    o.generateIntermediateLevels = false;
    return Osd::GB300StencilTableFactory::Create(refiner, o, nullptr, true);
}
#endif

int main() {
    std::vector<int64_t> off;
    std::vector<int> src;
    std::vector<float> w;
    std::printf("%d\n", record_example(off, src, w));
    return 0;
}
