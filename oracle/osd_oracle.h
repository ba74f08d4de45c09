/*
 * osd_oracle.h -- CPU restatement of the Osd evaluation path, used ONLY as the checker.
 *
 * TEST INFRASTRUCTURE.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg may load liboracle.so.  The GB300 product never calls into it.
 *
 * Pinning: every function here is checked against fixtures produced by the reference itself
 * (tests/golden/make_golden.py drives oracle/_ref/libosdref.so, the reference's own Far/Osd
 * CPU code compiled from source).  Float results are required to be bitwise identical to
 * Osd::CpuEvaluator; integer results (PatchMap handles, PatchParam decode) identical.
 *
 * Conventions shared with the C-ABI in include/osd_gb300.h:
 *   - a buffer descriptor is int[3] = {offset, length, stride} (osd/bufferDescriptor.h:61-103)
 *     and raw pointers exclude the offset (osd/cudaEvaluator.h:147-155);
 *   - a stencil range [start, end) writes dst element i (absolute), as the reference CUDA
 *     kernels do (osd/cudaKernel.cu:85-98);
 *   - a patch coord is 5 x 32-bit {arrayIndex, patchIndex, vertIndex, float s, float t}
 *     (osd/patchBasisTypes.h:249-255), a patch array 6 ints (:272-279), a patch param
 *     3 x 32-bit {field0, field1, float sharpness} (:301-305).
 */
#ifndef OSD_ORACLE_H
#define OSD_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* EvalStencils: nout = 1 (P), 3 (P, du, dv) or 6 (P, du, dv, duu, duv, dvv).
 * Sequential float accumulation in stencil order (osd/cpuKernel.cpp:71-240).
 * Returns 1 on success, 0 when a descriptor length differs from the source length. */
int orc_eval_stencils_f(const float *src, const int *srcDesc, int nout, float *const *dst,
                        const int *dstDesc, const int *sizes, const int *offsets,
                        const int *indices, const float *const *weights, int start, int end,
                        int nthreads);

/* FP64 oracle: the same float tables applied in double; dst are double buffers laid out with
 * the same descriptors. */
int orc_eval_stencils_d(const float *src, const int *srcDesc, int nout, double *const *dst,
                        const int *dstDesc, const int *sizes, const int *offsets,
                        const int *indices, const float *const *weights, int start, int end,
                        int nthreads);

/* Patch basis for one point (osd/patchBasis.h:1558-1610): w is [6][20] (P, Ds, Dt, Dss, Dst,
 * Dtt); returns the number of control points (0 for an unknown type). */
int orc_patch_basis_f(int patchType, int field0, int field1, float s, float t, float *w);
int orc_patch_basis_d(int patchType, int field0, int field1, double s, double t, double *w);

/* EvalPatches (osd/cpuEvaluator.cpp:157-381).  dst[k] may be NULL to skip an output. */
int orc_eval_patches_f(const float *src, const int *srcDesc, int nout, float *const *dst,
                       const int *dstDesc, int ncoords, const void *coords, const int *arrays,
                       const int *patchIndices, const void *params, int nthreads);
int orc_eval_patches_d(const float *src, const int *srcDesc, int nout, double *const *dst,
                       const int *dstDesc, int ncoords, const void *coords, const int *arrays,
                       const int *patchIndices, const void *params, int nthreads);

/* sum_j |w_j x_j| per output and element (double): the scale of float rounding error. */
int orc_eval_patches_abs(const float *src, const int *srcDesc, int nout, double *const *dst,
                         const int *dstDesc, int ncoords, const void *coords, const int *arrays,
                         const int *patchIndices, const void *params, int nthreads);

/* PatchMap (far/patchMap.h, far/patchMap.cpp).  params: 3 x 32-bit per patch (only
 * field0/field1 are read); arrays: 6 ints per patch array; triangular: 1 when the table's
 * varying patches have 3 CVs (tri patch layout). */
void *orc_patchmap_build(int numArrays, const int *arrays, const void *params, int triangular);
void orc_patchmap_free(void *map);
/* handles: 3 ints per query (arrayIndex, patchIndex, vertIndex), -1s when not found.
 * Returns the number of queries found. */
int orc_find_patches(const void *map, int n, const int *faces, const double *u,
                     const double *v, int *handles);

/* ---- stencil-table factory (far/stencilTableFactory.cpp, far/stencilBuilder.cpp) ---------- */

/* A stencil table produced by the factory restatements below (malloc'ed; free with
 * orc_table_free).  w[c] for c < numChannels. */
typedef struct orc_table {
    int numStencils, numChannels;
    long long nnz;
    int *sizes, *offsets, *indices;
    float *w[6];
} orc_table;

void orc_table_free(orc_table *t);

/* Far::StencilTableFactory::Create with factorizeIntermediateLevels from recorded per-level
 * masks (levels[l]: numRows[l], offsets[l][numRows + 1], sources[l], weights[l]; sources are
 * global vertex indices).  Rows are merged as far/stencilBuilder.cpp:164-198 (AddWithWeight)
 * and :310-385 (merge / add) do: first-touch entry order, float products and sums; rows of a
 * level are processed after the same-level rows their masks refer to (the order PrimvarRefiner
 * interpolates in).  Returns NULL on malformed masks. */
orc_table *orc_factory_create(int numControl, int numLevels, const int *numRows,
                              const long long *const *offsets, const int *const *sources,
                              const float *const *weights, int generateIntermediateLevels,
                              int generateControlVerts);

/* Rows composed from a base table with StencilBuilder::Index::AddWithWeight(StencilReal, ...)
 * (far/stencilBuilder.cpp:520-598): row i merges weights[c][k] * w over the entries (index, w)
 * of base stencil sources[k], zero w skipped.  appendBase puts the base stencils first
 * (AppendLocalPointStencilTable, far/stencilTableFactory.cpp:255-407). */
orc_table *orc_compose_rows(int baseNumStencils, const int *baseSizes, const int *baseOffsets,
                            const int *baseIndices, const float *baseWeights, int numRows,
                            const long long *offsets, const int *sources, int numChannels,
                            const float *const *weights, int appendBase);

/* ---- Bfr (bfr_oracle.c) ---- */

/* Bfr::Parameterization::ConvertCoordToNormalizedSubFace (bfr/parameterization.cpp:135-162)
 * for n (u,v) pairs of a face of size N; sub-face 0 and the coords unchanged where the face
 * has no sub-faces.  Returns 0 for an invalid parameterization. */
int orc_param_to_subface(int regFaceSize, int N, int n, const float *uv, int *sub, float *st);

/* Bfr::Tessellation inventory (bfr/tessellation.cpp:2023-2272): counts = {coords, facets,
 * boundary coords, uniform}.  Returns 0 (and zero counts) for invalid arguments. */
int orc_tess_inventory(int regFaceSize, int N, int numRates, const int *rates, int facetSize,
                       int preserveQuads, int *counts);

/* Tessellation::GetCoords<float> + GetFacets (bfr/tessellation.cpp:2300-2426) for one face.
 * Strides 0 select the defaults (2 and the facet size).  Returns 1, 0 when invalid, -1 when
 * the produced counts disagree with the inventory. */
int orc_tess_generate(int regFaceSize, int N, int numRates, const int *rates, int facetSize,
                      int preserveQuads, float *coords, int coordStride, int *facets,
                      int facetStride);

/* Every face of a mesh at the offsets of the inventory's exclusive scans, facet indices
 * offset to the mesh-wide coord numbering. */
int orc_tess_mesh(int regFaceSize, int numFaces, const int *faceSizes, const int *rateOffsets,
                  const int *rates, int facetSize, int preserveQuads, const long *coordOffsets,
                  const long *facetOffsets, float *coords, int *facets, int threads);

/* Ptex face and normalized (s, t) of every coord of a mesh tessellation. */
int orc_tess_locate_mesh(int regFaceSize, int numFaces, const int *faceSizes,
                         const long *coordOffsets, const long *ptexOffsets, const float *coords,
                         int *ptexFaces, float *st, int threads);

/* Shared (watertight) points of a mesh tessellation (tutorials/bfr/tutorial_2_2/
 * bfr_tutorial_2_2.cpp:244-430): facets (written by orc_tess_mesh when meshIndices, else
 * face-local) rewritten in place to point indices; pointOffsets (numFaces + 1) and
 * pointSources (one mesh coord per point, capacity = the number of coords).  Returns the
 * number of points, or a negative code (bfr_oracle.c). */
long orc_tess_share(int regFaceSize, int numFaces, const int *faceSizes, const int *faceVerts,
                    const int *faceEdges, int numVertices, int numEdges, const int *rateOffsets,
                    const int *rates, int facetSize, int preserveQuads, const long *coordOffsets,
                    const long *facetOffsets, int facetStride, int meshIndices, int *facets,
                    long *pointOffsets, long *pointSources);

/* ---- draw-time tessellation factors (tess_factors_oracle.c) ---- */

/* Per-patch tess levels of the patch shaders (osd/glslPatchCommonTess.glsl:92-550): outer[4],
 * inner[2], and the Lo / Hi outer halves (4 each) per patch in param order; arrays are the
 * flattened PatchArray (6 ints), params 3 ints per patch, matrices column-major. */
int orc_tess_factors(const int *arrays, int numArrays, const int *indices, const int *params,
                     int numPatches, const float *src, int srcStride, float tessLevel,
                     float maxTessLevel, int screenSpace, int spacing, const float *mv,
                     const float *proj, float *outer, float *inner, float *outLo, float *outHi);

/* OsdGetTessParameterization[Triangle] (osd/glslPatchCommonTess.glsl:692-730) */
int orc_tess_parameterization(int n, const float *domain, const int *patchIndex,
                              const float *outerLo, const float *outerHi, int spacing,
                              int triangular, float *uv);

#ifdef __cplusplus
}
#endif
#endif
