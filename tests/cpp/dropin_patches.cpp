// A C++ client of the drop-in header on the patch path: GB300PatchTable from flattened
// (Osd::CpuPatchTable layout) arrays plus its varying and face-varying tables, the device
// PatchMap, and the GB300Evaluator template forms EvalPatches (P and all five derivatives),
// EvalPatchesVarying and EvalPatchesFaceVarying (all five derivatives) with vertex buffers and
// a patch-coord buffer (the call shapes of CudaEvaluator, osd/cudaEvaluator.h:502-680 and
// 857-1255); then the same six-output EvalPatches over a device patch table of the client's own
// type with CudaPatchTable's accessors (the PATCH_TABLE type parameter).
//
// usage: dropin_patches <dir>  (reads *.bin written by the test, writes handles.bin,
//                               p{k}.bin, g{k}.bin, fvar{k}.bin (k = 0..5), var{k}.bin (0..2))
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

template <class T>
static void write(const std::string &path, const std::vector<T> &v) {
    std::ofstream(path, std::ios::binary)
        .write(reinterpret_cast<const char *>(v.data()), (std::streamsize)(v.size() * sizeof(T)));
}

// Device array of patch coords with the BindCudaBuffer() the template forms call.
struct CoordBuffer {
    OpenSubdiv::Osd::PatchCoord *d = nullptr;
    OpenSubdiv::Osd::PatchCoord *BindCudaBuffer() { return d; }
};

template <class T>
static T *upload(std::vector<T> const &v) {
    T *d = nullptr;
    cudaMalloc(&d, v.size() * sizeof(T));
    cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
    return d;
}

// A device patch table of the client's own, with CudaPatchTable's vertex accessors
// (osd/cudaPatchTable.h:51-110).
struct ClientDevicePatchTable {
    void *arrays = nullptr, *indices = nullptr, *params = nullptr;
    void *GetPatchArrayBuffer() const { return arrays; }
    void *GetPatchIndexBuffer() const { return indices; }
    void *GetPatchParamBuffer() const { return params; }
    void *GetVaryingPatchArrayBuffer() const { return nullptr; }
    void *GetVaryingPatchIndexBuffer() const { return nullptr; }
    void *GetFVarPatchArrayBuffer(int) const { return nullptr; }
    void *GetFVarPatchIndexBuffer(int) const { return nullptr; }
    void *GetFVarPatchParamBuffer(int) const { return nullptr; }
};

static void save(const std::string &path, OpenSubdiv::Osd::GB300VertexBuffer *b,
                 size_t count) {
    std::vector<float> out(count);
    cudaMemcpy(out.data(), b->BindCudaBuffer(), count * sizeof(float), cudaMemcpyDeviceToHost);
    write(path, out);
}

int main(int argc, char **argv) {
    using namespace OpenSubdiv;
    if (argc < 2) return 2;
    const std::string dir = argv[1];
    auto arrays = read<Osd::PatchArray>(dir + "/arrays.bin");
    auto indices = read<int>(dir + "/patch_indices.bin");
    auto params = read<Osd::PatchParam>(dir + "/params.bin");
    auto varrays = read<Osd::PatchArray>(dir + "/varying_arrays.bin");
    auto vindices = read<int>(dir + "/varying_indices.bin");
    auto farrays = read<Osd::PatchArray>(dir + "/fvar_arrays.bin");
    auto findices = read<int>(dir + "/fvar_indices.bin");
    auto fparams = read<Osd::PatchParam>(dir + "/fvar_params.bin");
    auto src = read<float>(dir + "/src.bin");
    auto fsrc = read<float>(dir + "/fvar_src.bin");
    auto qface = read<int>(dir + "/q_face.bin");
    auto qu = read<float>(dir + "/q_u.bin");
    auto qv = read<float>(dir + "/q_v.bin");
    auto tri = read<int>(dir + "/triangular.bin");
    const int nq = (int)qface.size();

    Osd::GB300PatchTable *table = Osd::GB300PatchTable::Create(
        (int)arrays.size(), arrays.data(), (int64_t)indices.size(), indices.data(),
        (int)params.size(), params.data(), tri[0] != 0);
    if (!table || !table->SetVarying((int)varrays.size(), varrays.data(),
                                     (int64_t)vindices.size(), vindices.data()) ||
        table->AddFVarChannel((int)farrays.size(), farrays.data(), (int64_t)findices.size(),
                              findices.data(), (int)fparams.size(), fparams.data()) != 0) {
        std::fprintf(stderr, "table failed: %s\n", GB300GetLastErrorString());
        return 1;
    }
    // queries on the device, device PatchMap
    int *dFace;
    float *dU, *dV;
    CoordBuffer coords;
    cudaMalloc(&dFace, nq * sizeof(int));
    cudaMalloc(&dU, nq * sizeof(float));
    cudaMalloc(&dV, nq * sizeof(float));
    cudaMalloc(&coords.d, nq * sizeof(Osd::PatchCoord));
    cudaMemcpy(dFace, qface.data(), nq * sizeof(int), cudaMemcpyHostToDevice);
    cudaMemcpy(dU, qu.data(), nq * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(dV, qv.data(), nq * sizeof(float), cudaMemcpyHostToDevice);
    if (!table->FindPatches(nq, dFace, dU, dV, coords.d)) {
        std::fprintf(stderr, "FindPatches failed: %s\n", GB300GetLastErrorString());
        return 1;
    }
    // P and all five derivatives of xyz; varying (4 primvars) with du, dv; face-varying uv
    // with all five derivatives
    const int nsrc = (int)src.size() / 3, nf = (int)fsrc.size() / 2;
    auto vsrcv = read<float>(dir + "/varying_src.bin");
    const int nv = (int)vsrcv.size() / 4;
    Osd::GB300VertexBuffer *vsrc = Osd::GB300VertexBuffer::Create(3, nsrc);
    Osd::GB300VertexBuffer *vf = Osd::GB300VertexBuffer::Create(2, nf);
    Osd::GB300VertexBuffer *vv = Osd::GB300VertexBuffer::Create(4, nv);
    vsrc->UpdateData(src.data(), 0, nsrc);
    vf->UpdateData(fsrc.data(), 0, nf);
    vv->UpdateData(vsrcv.data(), 0, nv);
    Osd::GB300VertexBuffer *p[6], *g[6], *fo[6], *vo[3];
    for (int k = 0; k < 6; ++k) {
        p[k] = Osd::GB300VertexBuffer::Create(3, nq);
        g[k] = Osd::GB300VertexBuffer::Create(3, nq);
        fo[k] = Osd::GB300VertexBuffer::Create(2, nq);
    }
    for (int k = 0; k < 3; ++k) vo[k] = Osd::GB300VertexBuffer::Create(4, nq);
    Osd::BufferDescriptor d3(0, 3, 3), d2(0, 2, 2), d4(0, 4, 4);
    if (!Osd::GB300Evaluator::EvalPatches(vsrc, d3, p[0], d3, p[1], d3, p[2], d3, p[3], d3,
                                          p[4], d3, p[5], d3, nq, &coords, table) ||
        !Osd::GB300Evaluator::EvalPatchesVarying(vv, d4, vo[0], d4, vo[1], d4, vo[2], d4, nq,
                                                 &coords, table) ||
        !Osd::GB300Evaluator::EvalPatchesFaceVarying(vf, d2, fo[0], d2, fo[1], d2, fo[2], d2,
                                                     fo[3], d2, fo[4], d2, fo[5], d2, nq,
                                                     &coords, table, 0)) {
        std::fprintf(stderr, "eval failed: %s\n", GB300GetLastErrorString());
        return 1;
    }
    // the same points through a device table of the client's own type
    ClientDevicePatchTable own;
    own.arrays = upload(arrays);
    own.indices = upload(indices);
    own.params = upload(params);
    if (!Osd::GB300Evaluator::EvalPatches(vsrc, d3, g[0], d3, g[1], d3, g[2], d3, g[3], d3,
                                          g[4], d3, g[5], d3, nq, &coords, &own)) {
        std::fprintf(stderr, "raw-table eval failed: %s\n", GB300GetLastErrorString());
        return 1;
    }
    Osd::GB300Evaluator::Synchronize();
    std::vector<Osd::PatchCoord> hc(nq);
    cudaMemcpy(hc.data(), coords.d, nq * sizeof(Osd::PatchCoord), cudaMemcpyDeviceToHost);
    std::vector<int> handles((size_t)nq * 3);
    for (int i = 0; i < nq; ++i) {
        handles[3 * i] = hc[i].handle.arrayIndex;
        handles[3 * i + 1] = hc[i].handle.patchIndex;
        handles[3 * i + 2] = hc[i].handle.vertIndex;
    }
    write(dir + "/handles.bin", handles);
    for (int k = 0; k < 6; ++k) {
        save(dir + "/p" + std::to_string(k) + ".bin", p[k], (size_t)nq * 3);
        save(dir + "/g" + std::to_string(k) + ".bin", g[k], (size_t)nq * 3);
        save(dir + "/fvar" + std::to_string(k) + ".bin", fo[k], (size_t)nq * 2);
    }
    for (int k = 0; k < 3; ++k) save(dir + "/var" + std::to_string(k) + ".bin", vo[k], (size_t)nq * 4);
    delete table;
    std::printf("ok %d queries\n", nq);
    return 0;
}
