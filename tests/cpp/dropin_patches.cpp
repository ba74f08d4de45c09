// A C++ client of the drop-in header on the patch path: GB300PatchTable from flattened
// (Osd::CpuPatchTable layout) arrays plus its varying and face-varying tables, the device
// PatchMap, and the GB300Evaluator template forms EvalPatches / EvalPatchesFaceVarying with
// vertex buffers and a patch-coord buffer (the call shapes of CudaEvaluator,
// osd/cudaEvaluator.h:502-525 and 1070-1255).
//
// usage: dropin_patches <dir>  (reads *.bin written by the test, writes handles.bin,
//                               p.bin, du.bin, dv.bin, fvar.bin)
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
    // P, dPdu, dPdv of xyz, and face-varying uv with derivatives
    const int nsrc = (int)src.size() / 3, nf = (int)fsrc.size() / 2;
    Osd::GB300VertexBuffer *vsrc = Osd::GB300VertexBuffer::Create(3, nsrc);
    Osd::GB300VertexBuffer *vf = Osd::GB300VertexBuffer::Create(2, nf);
    Osd::GB300VertexBuffer *p = Osd::GB300VertexBuffer::Create(3, nq);
    Osd::GB300VertexBuffer *du = Osd::GB300VertexBuffer::Create(3, nq);
    Osd::GB300VertexBuffer *dv = Osd::GB300VertexBuffer::Create(3, nq);
    Osd::GB300VertexBuffer *fo = Osd::GB300VertexBuffer::Create(2, nq);
    vsrc->UpdateData(src.data(), 0, nsrc);
    vf->UpdateData(fsrc.data(), 0, nf);
    Osd::BufferDescriptor d3(0, 3, 3), d2(0, 2, 2);
    if (!Osd::GB300Evaluator::EvalPatches(vsrc, d3, p, d3, du, d3, dv, d3, nq, &coords, table) ||
        !Osd::GB300Evaluator::EvalPatchesFaceVarying(vf, d2, fo, d2, nq, &coords, table, 0)) {
        std::fprintf(stderr, "eval failed: %s\n", GB300GetLastErrorString());
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
    std::vector<float> out((size_t)nq * 3);
    const char *names[3] = {"p", "du", "dv"};
    Osd::GB300VertexBuffer *outs[3] = {p, du, dv};
    for (int k = 0; k < 3; ++k) {
        cudaMemcpy(out.data(), outs[k]->BindCudaBuffer(), out.size() * sizeof(float),
                   cudaMemcpyDeviceToHost);
        write(dir + "/" + names[k] + ".bin", out);
    }
    std::vector<float> fout((size_t)nq * 2);
    cudaMemcpy(fout.data(), fo->BindCudaBuffer(), fout.size() * sizeof(float),
               cudaMemcpyDeviceToHost);
    write(dir + "/fvar.bin", fout);
    delete table;
    std::printf("ok %d queries\n", nq);
    return 0;
}
