// A C++ client of the Bfr-shaped header: the tessellate-and-evaluate loop of the reference's
// Bfr tutorials (tutorials/bfr/tutorial_1_2/bfr_tutorial_1_2.cpp:170-238) for every face of a
// mesh at once -- GB300MeshTessellation (per-face rates, mesh-wide facet indices, PatchCoords on
// a device patch table), its Evaluate (Surface::Evaluate: P and all five derivatives), and the
// same coords through GB300Evaluator::EvalPatches (P, Du, Dv); then the shared (watertight)
// points of the reference's tutorial 2.2 (GB300MeshTessellation::Share + EvaluatePoints).
//
// usage: bfr_client <dir>  (reads *.bin written by the test; writes coords.bin, facets.bin,
//                           patch_coords.bin, p{k}.bin for k = 0..5, g{k}.bin for k = 0..2,
//                           shared_facets.bin, point_offsets.bin, point_p.bin)
#include <opensubdiv_gb300/bfr/gb300Tessellation.h>

#include <cuda_runtime.h>

#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

template <class T>
static std::vector<T> read(const std::string &path) {
    std::ifstream f(path, std::ios::binary | std::ios::ate);
    std::vector<T> v((size_t)f.tellg() / sizeof(T));
    f.seekg(0);
    f.read(reinterpret_cast<char *>(v.data()), (std::streamsize)(v.size() * sizeof(T)));
    return v;
}

template <class T>
static void write(const std::string &path, const T *d, size_t n) {
    std::vector<T> v(n);
    cudaMemcpy(v.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost);
    std::ofstream(path, std::ios::binary)
        .write(reinterpret_cast<const char *>(v.data()), (std::streamsize)(n * sizeof(T)));
}

template <class T>
static T *upload(std::vector<T> const &v) {
    T *d = nullptr;
    cudaMalloc(&d, v.size() * sizeof(T) + 16);
    cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
    return d;
}

struct CoordBuffer {
    OpenSubdiv::Osd::PatchCoord *d = nullptr;
    OpenSubdiv::Osd::PatchCoord *BindCudaBuffer() { return d; }
};

int main(int argc, char **argv) {
    using namespace OpenSubdiv;
    if (argc < 2) return 2;
    const std::string dir = argv[1];
    auto sizes = read<int>(dir + "/verts_per_face.bin");
    auto rateOffsets = read<int>(dir + "/rate_offsets.bin");
    auto rates = read<int>(dir + "/rates.bin");
    auto arrays = read<Osd::PatchArray>(dir + "/arrays.bin");
    auto indices = read<int>(dir + "/patch_indices.bin");
    auto params = read<Osd::PatchParam>(dir + "/params.bin");
    auto src = read<float>(dir + "/src.bin");
    auto opts = read<int>(dir + "/options.bin");  // regular face size, facet size, quads, tri
    const int numFaces = (int)sizes.size();

    Osd::GB300PatchTable *table = Osd::GB300PatchTable::Create(
        (int)arrays.size(), arrays.data(), (int64_t)indices.size(), indices.data(),
        (int)params.size(), params.data(), opts[3] != 0);
    Bfr::GB300MeshTessellation::Options o;
    o.SetFacetSize(opts[1]).PreserveQuads(opts[2] != 0);
    int *dSizes = upload(sizes), *dOffsets = upload(rateOffsets), *dRates = upload(rates);
    Bfr::GB300MeshTessellation *tess = table ? Bfr::GB300MeshTessellation::Create(
                                                   opts[0], numFaces, dSizes, dOffsets, dRates, o)
                                             : nullptr;
    if (!tess) {
        std::fprintf(stderr, "setup failed: %s\n", GB300GetLastErrorString());
        return 1;
    }
    const int n = tess->GetNumCoords(), nf = tess->GetNumFacets();
    float *coords;
    int *facets;
    CoordBuffer pc;
    cudaMalloc(&coords, sizeof(float) * 2 * (size_t)n);
    cudaMalloc(&facets, sizeof(int) * (size_t)tess->GetFacetStride() * nf);
    cudaMalloc(&pc.d, sizeof(Osd::PatchCoord) * (size_t)n);
    if (!tess->Generate(coords, facets, true, table, pc.d)) {
        std::fprintf(stderr, "Generate failed: %s\n", GB300GetLastErrorString());
        return 1;
    }
    const int nsrc = (int)src.size() / 3;
    Osd::GB300VertexBuffer *vsrc = Osd::GB300VertexBuffer::Create(3, nsrc);
    vsrc->UpdateData(src.data(), 0, nsrc);
    Osd::GB300VertexBuffer *p[6];
    for (int k = 0; k < 6; ++k) p[k] = Osd::GB300VertexBuffer::Create(3, n);
    // Surface::Evaluate at every coord (P and all five derivatives), and P, Du, Dv of the same
    // coords through the evaluator header's EvalPatches into a second set of buffers
    if (!tess->Evaluate(table, pc.d, vsrc->BindCudaBuffer(), 3, 3, p[0]->BindCudaBuffer(),
                        p[1]->BindCudaBuffer(), p[2]->BindCudaBuffer(), p[3]->BindCudaBuffer(),
                        p[4]->BindCudaBuffer(), p[5]->BindCudaBuffer())) {
        std::fprintf(stderr, "Evaluate failed: %s\n", GB300GetLastErrorString());
        return 1;
    }
    Osd::GB300VertexBuffer *g[3];
    for (int k = 0; k < 3; ++k) g[k] = Osd::GB300VertexBuffer::Create(3, n);
    Osd::BufferDescriptor d3(0, 3, 3);
    if (!Osd::GB300Evaluator::EvalPatches(vsrc, d3, g[0], d3, g[1], d3, g[2], d3, n, &pc,
                                          table)) {
        std::fprintf(stderr, "EvalPatches failed: %s\n", GB300GetLastErrorString());
        return 1;
    }
    // shared (watertight) points: the reference's tutorial 2.2 bookkeeping on a copy of the
    // facets, each point evaluated once
    auto faceVerts = read<int>(dir + "/face_verts.bin");
    auto faceEdges = read<int>(dir + "/face_edges.bin");
    auto topo = read<int>(dir + "/topology.bin");  // vertices, edges
    int *dVerts = upload(faceVerts), *dEdges = upload(faceEdges), *shared = nullptr;
    int64_t *pointOffsets = nullptr;
    Osd::PatchCoord *pointCoords = nullptr;
    const size_t facetInts = (size_t)tess->GetFacetStride() * nf;
    cudaMalloc(&shared, sizeof(int) * facetInts);
    cudaMemcpy(shared, facets, sizeof(int) * facetInts, cudaMemcpyDeviceToDevice);
    cudaMalloc(&pointOffsets, sizeof(int64_t) * (size_t)(numFaces + 1));
    cudaMalloc(&pointCoords, sizeof(Osd::PatchCoord) * (size_t)n);
    const int64_t numPoints = tess->Share(dVerts, dEdges, (int64_t)faceVerts.size(), topo[0],
                                          topo[1], shared, pc.d, pointOffsets, pointCoords);
    if (numPoints < 0) {
        std::fprintf(stderr, "Share failed: %s\n", GB300GetLastErrorString());
        return 1;
    }
    Osd::GB300VertexBuffer *sp = Osd::GB300VertexBuffer::Create(3, (int)numPoints);
    if (!tess->EvaluatePoints(table, pointCoords, (int)numPoints, vsrc->BindCudaBuffer(), 3, 3,
                              sp->BindCudaBuffer())) {
        std::fprintf(stderr, "EvaluatePoints failed: %s\n", GB300GetLastErrorString());
        return 1;
    }
    cudaDeviceSynchronize();
    write(dir + "/shared_facets.bin", shared, facetInts);
    write(dir + "/point_offsets.bin", pointOffsets, (size_t)numFaces + 1);
    write(dir + "/point_p.bin", sp->BindCudaBuffer(), 3 * (size_t)numPoints);
    delete sp;
    cudaFree(shared);
    cudaFree(pointOffsets);
    cudaFree(pointCoords);
    write(dir + "/coords.bin", coords, 2 * (size_t)n);
    write(dir + "/facets.bin", facets, (size_t)tess->GetFacetStride() * nf);
    write(dir + "/patch_coords.bin", reinterpret_cast<int *>(pc.d), 5 * (size_t)n);
    for (int k = 0; k < 6; ++k)
        write(dir + "/p" + std::to_string(k) + ".bin", p[k]->BindCudaBuffer(), 3 * (size_t)n);
    for (int k = 0; k < 3; ++k) {
        write(dir + "/g" + std::to_string(k) + ".bin", g[k]->BindCudaBuffer(), 3 * (size_t)n);
        delete g[k];
    }
    delete tess;
    delete table;
    for (auto *b : p) delete b;
    delete vsrc;
    return 0;
}
