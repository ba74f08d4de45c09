// A client written against OpenSubdiv's own headers -- Far::StencilTable, Far::LimitStencilTable
// (with second-derivative weights) and Far::PatchTable, through the Osd evaluator template
// forms -- with CudaEvaluator's type names switched to the GB300 ones.  Compiled (not run) by a
// CPU test with the reference's source tree on the include path; the refine path repeats the
// calls Osd::Mesh::Refine makes (osd/mesh.h:501-547): the stencil table converted with
// convertToCompatibleStencilTable, the evaluator looked up in an EvaluatorCacheT (GB300Evaluator,
// like CudaEvaluator, is not instantiatable, so the lookup yields NULL and the static forms
// run).
#include <opensubdiv/far/patchTable.h>
#include <opensubdiv/far/stencilTable.h>
#include <opensubdiv/osd/mesh.h>
#include <opensubdiv/bfr/refinerSurfaceFactory.h>
#include <opensubdiv/bfr/tessellation.h>
#include <opensubdiv_gb300/osd/gb300Evaluator.h>
#include <opensubdiv_gb300/bfr/gb300Tessellation.h>

using namespace OpenSubdiv;

// Device patch coords with the BindCudaBuffer() the template forms call.
struct PatchCoordBuffer {
    Osd::PatchCoord *d;
    Osd::PatchCoord *BindCudaBuffer() { return d; }
};

bool Refine(Far::StencilTable const *farStencils, Osd::GB300VertexBuffer *vertexBuffer,
            int numControlVertices, Osd::EvaluatorCacheT<Osd::GB300Evaluator> *cache,
            void *deviceContext) {
    Osd::GB300StencilTable const *table =
        Osd::convertToCompatibleStencilTable<Osd::GB300StencilTable>(farStencils,
                                                                      deviceContext);
    Osd::BufferDescriptor srcDesc(0, 3, 3), dstDesc(numControlVertices * 3, 3, 3);
    Osd::GB300Evaluator const *instance =
        Osd::GetEvaluator<Osd::GB300Evaluator>(cache, srcDesc, dstDesc, deviceContext);
    bool ok = Osd::GB300Evaluator::EvalStencils(vertexBuffer, srcDesc, vertexBuffer, dstDesc,
                                                table, instance, deviceContext);
    Osd::GB300Evaluator::Synchronize(deviceContext);
    delete table;
    return ok;
}

bool LimitWithSecondDerivatives(Far::LimitStencilTable const *farStencils,
                                Osd::GB300VertexBuffer *cvs, Osd::GB300VertexBuffer *out[6]) {
    Osd::GB300StencilTable *table = Osd::GB300StencilTable::Create(farStencils);
    Osd::BufferDescriptor d(0, 3, 3);
    bool ok = table && Osd::GB300Evaluator::EvalStencils(cvs, d, out[0], d, out[1], d, out[2], d,
                                                         out[3], d, out[4], d, out[5], d, table);
    ok = ok && Osd::GB300Evaluator::EvalStencils(cvs, d, out[0], d, out[1], d, out[2], d, table);
    delete table;
    return ok;
}

bool LimitSurface(Far::PatchTable const *farPatches, Osd::GB300VertexBuffer *src,
                  Osd::GB300VertexBuffer *fvarSrc, PatchCoordBuffer *coords, int numCoords,
                  Osd::GB300VertexBuffer *out[6], Osd::GB300VertexBuffer *fvarOut[6]) {
    Osd::GB300PatchTable *table = Osd::GB300PatchTable::Create(farPatches);
    Osd::BufferDescriptor d(0, 3, 3), uv(0, 2, 2);
    bool ok = table &&
              Osd::GB300Evaluator::EvalPatches(src, d, out[0], d, out[1], d, out[2], d, out[3],
                                               d, out[4], d, out[5], d, numCoords, coords,
                                               table) &&
              Osd::GB300Evaluator::EvalPatches(src, d, out[0], d, out[1], d, out[2], d,
                                               numCoords, coords, table) &&
              Osd::GB300Evaluator::EvalPatches(src, d, out[0], d, numCoords, coords, table) &&
              Osd::GB300Evaluator::EvalPatchesVarying(src, d, out[0], d, out[1], d, out[2], d,
                                                      out[3], d, out[4], d, out[5], d, numCoords,
                                                      coords, table) &&
              Osd::GB300Evaluator::EvalPatchesFaceVarying(
                  fvarSrc, uv, fvarOut[0], uv, fvarOut[1], uv, fvarOut[2], uv, fvarOut[3], uv,
                  fvarOut[4], uv, fvarOut[5], uv, numCoords, coords, table, 0);
    delete table;
    return ok;
}

// The Bfr tutorials' loop (tutorials/bfr/tutorial_1_2/bfr_tutorial_1_2.cpp:155-238) with the
// per-face Bfr::Tessellation replaced by one device tessellation of the mesh: the client's own
// Bfr::Tessellation::Options carry over, the face sizes come from its refiner, and the Far table
// pairs with Bfr::SurfaceFactory's approximation (as the reference's Bfr regression builds it).
bool tessellateLikeTheTutorial(Far::TopologyRefiner &mesh, int const *deviceFaceSizes,
                               int tessUniformRate, bool tessQuadsFlag, float *coords,
                               int *facets, PatchCoordBuffer *coordsOut) {
    Far::PatchTable const *farTable = Bfr::GB300CreateSurfacePatchTable(mesh);
    Bfr::Tessellation::Options tessOptions;
    tessOptions.SetFacetSize(3 + tessQuadsFlag);
    tessOptions.PreserveQuads(tessQuadsFlag);
    const int regularFaceSize = Sdc::SchemeTypeTraits::GetRegularFaceSize(mesh.GetSchemeType());
    Osd::GB300PatchTable *table = Osd::GB300PatchTable::Create(farTable);
    Bfr::GB300MeshTessellation *tess = Bfr::GB300MeshTessellation::Create(
        regularFaceSize, mesh.GetLevel(0).GetNumFaces(), deviceFaceSizes, tessUniformRate,
        Bfr::GB300MeshTessellation::Options(tessOptions));
    const bool ok = table && tess && tess->Generate(coords, facets, true, table, coordsOut->d);
    delete tess;
    delete table;
    delete farTable;
    return ok;
}

// The reference's tutorial 2.2 (tutorials/bfr/tutorial_2_2/bfr_tutorial_2_2.cpp:160-430):
// the same tessellation with the points of mesh vertices and edges shared between faces --
// the base level's face vertices and edges go to the device, Share rewrites the facets to
// shared point indices and each point is evaluated once.
long long tessellateWatertight(Far::TopologyRefiner &mesh, int const *deviceFaceSizes,
                               int tessUniformRate, float *coords, int *facets,
                               PatchCoordBuffer *coordsOut, Osd::PatchCoord *points,
                               int64_t *pointOffsets) {
    Far::PatchTable const *farTable = Bfr::GB300CreateSurfacePatchTable(mesh);
    const int regularFaceSize = Sdc::SchemeTypeTraits::GetRegularFaceSize(mesh.GetSchemeType());
    Osd::GB300PatchTable *table = Osd::GB300PatchTable::Create(farTable);
    Bfr::GB300MeshTessellation *tess = Bfr::GB300MeshTessellation::Create(
        regularFaceSize, mesh.GetLevel(0).GetNumFaces(), deviceFaceSizes, tessUniformRate);
    std::vector<int> faceVerts, faceEdges;
    Bfr::GB300GetFaceVerticesAndEdges(mesh, faceVerts, faceEdges);
    int *dv = nullptr, *de = nullptr;
    cudaMalloc(&dv, sizeof(int) * faceVerts.size());
    cudaMalloc(&de, sizeof(int) * faceEdges.size());
    cudaMemcpy(dv, faceVerts.data(), sizeof(int) * faceVerts.size(), cudaMemcpyHostToDevice);
    cudaMemcpy(de, faceEdges.data(), sizeof(int) * faceEdges.size(), cudaMemcpyHostToDevice);
    long long n = -1;
    if (table && tess && tess->Generate(coords, facets, true, table, coordsOut->d))
        n = tess->Share(dv, de, (int64_t)faceVerts.size(), mesh.GetLevel(0).GetNumVertices(),
                        mesh.GetLevel(0).GetNumEdges(), facets, coordsOut->d, pointOffsets,
                        points);
    cudaFree(dv);
    cudaFree(de);
    delete tess;
    delete table;
    delete farTable;
    return n;
}

// The reference's tutorial 2.1 (tutorials/bfr/tutorial_2_1/bfr_tutorial_2_1.cpp:160-360):
// per-edge rates from the control hull's edge lengths, then the non-uniform tessellation --
// the rates computed on the device from the mesh's face vertices and positions.
bool tessellateByEdgeLength(Far::TopologyRefiner &mesh, int const *deviceFaceSizes,
                            float const *devicePositions, float tessInterval, int tessRateMax,
                            float *coords, int *facets, PatchCoordBuffer *coordsOut) {
    Far::TopologyLevel const &base = mesh.GetLevel(0);
    std::vector<int> faceVerts, faceEdges;
    Bfr::GB300GetFaceVerticesAndEdges(mesh, faceVerts, faceEdges);
    int *dv = nullptr, *rateOffsets = nullptr, *rates = nullptr;
    cudaMalloc(&dv, sizeof(int) * faceVerts.size());
    cudaMalloc(&rateOffsets, sizeof(int) * (base.GetNumFaces() + 1));
    cudaMalloc(&rates, sizeof(int) * faceVerts.size());
    cudaMemcpy(dv, faceVerts.data(), sizeof(int) * faceVerts.size(), cudaMemcpyHostToDevice);
    bool ok = Bfr::GB300MeshTessellation::ComputeEdgeRates(
        base.GetNumFaces(), deviceFaceSizes, dv, (int64_t)faceVerts.size(), devicePositions,
        base.GetNumVertices(), 3, false, tessInterval, tessRateMax, rateOffsets, rates);
    Far::PatchTable const *farTable = Bfr::GB300CreateSurfacePatchTable(mesh);
    Osd::GB300PatchTable *table = Osd::GB300PatchTable::Create(farTable);
    Bfr::GB300MeshTessellation *tess =
        ok ? Bfr::GB300MeshTessellation::Create(
                 Sdc::SchemeTypeTraits::GetRegularFaceSize(mesh.GetSchemeType()),
                 base.GetNumFaces(), deviceFaceSizes, rateOffsets, rates)
           : nullptr;
    ok = table && tess && tess->Generate(coords, facets, true, table, coordsOut->d);
    delete tess;
    delete table;
    delete farTable;
    cudaFree(dv);
    cudaFree(rateOffsets);
    cudaFree(rates);
    return ok;
}

int main() { return 0; }
