// A C++ client evaluating limit stencils with first and second derivatives through the drop-in
// header's template forms (the call shapes of CudaEvaluator::EvalStencils,
// osd/cudaEvaluator.h:219-249 and 352-375):
//   1. a GB300StencilTable created from a Far::LimitStencilTable stand-in (the members
//      Far::LimitStencilTable exposes), evaluated through its own device layout;
//   2. a client-owned device table exposing CudaStencilTable's accessors (Get*Buffer,
//      GetNumStencils), the STENCIL_TABLE type parameter, evaluated through the raw entry points.
//
// usage: dropin_derivatives <dir>  (reads limit_*.bin and src.bin, writes a{k}.bin, b{k}.bin
//                                   for the six outputs P, du, dv, duu, duv, dvv)
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

// Member-for-member stand-in of Far::LimitStencilTable (far/stencilTable.h:409-579).
struct LimitStencilTableLike {
    std::vector<int> sizes, offsets, indices;
    std::vector<float> w[6];
    int GetNumStencils() const { return (int)sizes.size(); }
    std::vector<int> const &GetSizes() const { return sizes; }
    std::vector<int> const &GetOffsets() const { return offsets; }
    std::vector<int> const &GetControlIndices() const { return indices; }
    std::vector<float> const &GetWeights() const { return w[0]; }
    std::vector<float> const &GetDuWeights() const { return w[1]; }
    std::vector<float> const &GetDvWeights() const { return w[2]; }
    std::vector<float> const &GetDuuWeights() const { return w[3]; }
    std::vector<float> const &GetDuvWeights() const { return w[4]; }
    std::vector<float> const &GetDvvWeights() const { return w[5]; }
};

template <class T>
static T *upload(std::vector<T> const &v) {
    T *d = nullptr;
    cudaMalloc(&d, v.size() * sizeof(T));
    cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
    return d;
}

// A device stencil table of the client's own, with CudaStencilTable's accessors
// (osd/cudaEvaluator.h:52-92).
struct ClientDeviceStencilTable {
    int n = 0;
    int *sizes = nullptr, *offsets = nullptr, *indices = nullptr;
    float *w[6] = {};
    void *GetSizesBuffer() const { return sizes; }
    void *GetOffsetsBuffer() const { return offsets; }
    void *GetIndicesBuffer() const { return indices; }
    void *GetWeightsBuffer() const { return w[0]; }
    void *GetDuWeightsBuffer() const { return w[1]; }
    void *GetDvWeightsBuffer() const { return w[2]; }
    void *GetDuuWeightsBuffer() const { return w[3]; }
    void *GetDuvWeightsBuffer() const { return w[4]; }
    void *GetDvvWeightsBuffer() const { return w[5]; }
    int GetNumStencils() const { return n; }
};

int main(int argc, char **argv) {
    using namespace OpenSubdiv;
    if (argc < 2) return 2;
    const std::string dir = argv[1];
    LimitStencilTableLike far;
    far.sizes = read<int>(dir + "/limit_sizes.bin");
    far.offsets = read<int>(dir + "/limit_offsets.bin");
    far.indices = read<int>(dir + "/limit_indices.bin");
    const char *names[6] = {"weights", "du_weights", "dv_weights", "duu_weights", "duv_weights",
                            "dvv_weights"};
    for (int k = 0; k < 6; ++k) far.w[k] = read<float>(dir + "/limit_" + names[k] + ".bin");
    std::vector<float> src = read<float>(dir + "/src.bin");
    const int nCV = (int)src.size() / 3, n = far.GetNumStencils();

    Osd::GB300VertexBuffer *in = Osd::GB300VertexBuffer::Create(3, nCV);
    in->UpdateData(src.data(), 0, nCV);
    Osd::GB300VertexBuffer *a[6], *b[6];
    for (int k = 0; k < 6; ++k) {
        a[k] = Osd::GB300VertexBuffer::Create(3, n);
        b[k] = Osd::GB300VertexBuffer::Create(3, n);
    }
    Osd::BufferDescriptor d(0, 3, 3);

    // 1. the library's table object
    Osd::GB300StencilTable *table = Osd::GB300StencilTable::Create(&far);
    if (!table || !Osd::GB300Evaluator::EvalStencils(in, d, a[0], d, a[1], d, a[2], d, a[3], d,
                                                     a[4], d, a[5], d, table)) {
        std::fprintf(stderr, "table eval failed: %s\n", GB300GetLastErrorString());
        return 1;
    }
    // 2. a device table of the client's own type
    ClientDeviceStencilTable own;
    own.n = n;
    own.sizes = upload(far.sizes);
    own.offsets = upload(far.offsets);
    own.indices = upload(far.indices);
    for (int k = 0; k < 6; ++k) own.w[k] = upload(far.w[k]);
    if (!Osd::GB300Evaluator::EvalStencils(in, d, b[0], d, b[1], d, b[2], d, b[3], d, b[4], d,
                                           b[5], d, &own)) {
        std::fprintf(stderr, "raw-table eval failed: %s\n", GB300GetLastErrorString());
        return 1;
    }
    // P, du, dv only (the 3-output form) must leave the second-derivative weights unread
    Osd::GB300VertexBuffer *c0 = Osd::GB300VertexBuffer::Create(3, n);
    if (!Osd::GB300Evaluator::EvalStencils(in, d, c0, d, b[1], d, b[2], d, &own)) return 1;
    // a mismatched descriptor length is rejected (osd/cpuEvaluator.cpp:46-47)
    Osd::BufferDescriptor bad(0, 2, 3);
    if (Osd::GB300Evaluator::EvalStencils(in, d, a[0], d, a[1], bad, a[2], d, table)) return 1;
    Osd::GB300Evaluator::Synchronize();
    std::vector<float> out((size_t)n * 3);
    for (int k = 0; k < 6; ++k) {
        for (int which = 0; which < 2; ++which) {
            Osd::GB300VertexBuffer *v = which ? b[k] : a[k];
            cudaMemcpy(out.data(), v->BindCudaBuffer(), out.size() * 4, cudaMemcpyDeviceToHost);
            std::ofstream(dir + "/" + (which ? "b" : "a") + std::to_string(k) + ".bin",
                          std::ios::binary)
                .write(reinterpret_cast<const char *>(out.data()),
                       (std::streamsize)(out.size() * 4));
        }
    }
    cudaMemcpy(out.data(), c0->BindCudaBuffer(), out.size() * 4, cudaMemcpyDeviceToHost);
    std::ofstream(dir + "/c0.bin", std::ios::binary)
        .write(reinterpret_cast<const char *>(out.data()), (std::streamsize)(out.size() * 4));
    std::printf("ok %d stencils\n", n);
    return 0;
}
