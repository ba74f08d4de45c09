// A C++ client of the drop-in header: builds a GB300StencilTable from a Far::StencilTable
// stand-in (the same member functions Far::StencilTable exposes), uploads the control points
// through GB300VertexBuffer, evaluates with the GB300Evaluator template form (the call shape of
// CudaEvaluator::EvalStencils, osd/cudaEvaluator.h:125-142) and writes the refined points.
//
// usage: dropin_client <dir>  (reads sizes/offsets/indices/weights/src .bin, writes out.bin)
#include <opensubdiv_gb300/osd/gb300Evaluator.h>

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

// Member-for-member stand-in of Far::StencilTable (far/stencilTable.h:141-269).
struct StencilTableLike {
    std::vector<int> sizes, offsets, indices;
    std::vector<float> weights;
    int GetNumStencils() const { return (int)sizes.size(); }
    std::vector<int> const &GetSizes() const { return sizes; }
    std::vector<int> const &GetOffsets() const { return offsets; }
    std::vector<int> const &GetControlIndices() const { return indices; }
    std::vector<float> const &GetWeights() const { return weights; }
};

int main(int argc, char **argv) {
    using namespace OpenSubdiv;
    if (argc < 2) return 2;
    const std::string dir = argv[1];
    StencilTableLike far;
    far.sizes = read<int>(dir + "/sizes.bin");
    far.offsets = read<int>(dir + "/offsets.bin");
    far.indices = read<int>(dir + "/indices.bin");
    far.weights = read<float>(dir + "/weights.bin");
    std::vector<float> src = read<float>(dir + "/src.bin");
    const int nCV = (int)src.size() / 3, n = far.GetNumStencils();

    Osd::GB300StencilTable *table = Osd::GB300StencilTable::Create(&far);
    // one buffer holding control points then refined points, as Osd::Mesh::Refine uses it
    Osd::GB300VertexBuffer *buf = Osd::GB300VertexBuffer::Create(3, nCV + n);
    if (!table || !buf) {
        std::fprintf(stderr, "create failed: %s\n", GB300GetLastErrorString());
        return 1;
    }
    buf->UpdateData(src.data(), 0, nCV);
    Osd::BufferDescriptor srcDesc(0, 3, 3), dstDesc(nCV * 3, 3, 3);
    if (!Osd::GB300Evaluator::EvalStencils(buf, srcDesc, buf, dstDesc, table)) {
        std::fprintf(stderr, "eval failed: %s\n", GB300GetLastErrorString());
        return 1;
    }
    Osd::GB300Evaluator::Synchronize();
    std::vector<float> out((size_t)n * 3);
    cudaMemcpy(out.data(), buf->BindCudaBuffer() + nCV * 3, out.size() * sizeof(float),
               cudaMemcpyDeviceToHost);
    std::ofstream(dir + "/out.bin", std::ios::binary)
        .write(reinterpret_cast<const char *>(out.data()), (std::streamsize)(out.size() * 4));
    delete table;
    delete buf;
    std::printf("ok %d stencils\n", n);
    return 0;
}
