/*
 * osd_gb300.h -- C ABI of the GB300 (sm_103a) Osd evaluator: libosd_gb300.so.
 *
 * This is the boundary the reference's own FFI for the evaluation path binds: the extern "C"
 * block of opensubdiv/osd/cudaKernel.cu:349-426 (CudaEvalStencils, CudaEvalPatches,
 * CudaEvalPatchesWithDerivatives) plus the device-table and vertex-buffer objects of
 * osd/cudaEvaluator.h:52-92, osd/cudaPatchTable.h:51-110 and osd/cudaVertexBuffer.h:42-79.
 * No C++ or CUDA types cross it: plain pointers, ints and an opaque stream handle
 * (a cudaStream_t passed as void*; NULL means the legacy default stream).
 *
 * Pointer conventions follow the reference exactly:
 *   - EvalStencils / EvalPatches take raw DEVICE pointers that already include the
 *     BufferDescriptor offset (cudaEvaluator.cpp:159-162 adds srcDesc.offset before calling
 *     CudaEvalStencils); `length` floats are read/written per element, `*Stride` floats apart;
 *   - a stencil range [start, end) writes destination elements start..end-1 at their absolute
 *     positions, as cudaKernel.cu:85-98 does;
 *   - patch coords / arrays / params are the POD layouts OsdPatchCoord (5 x 32 bit),
 *     OsdPatchArray (6 ints) and OsdPatchParam (3 x 32 bit) of osd/patchBasisTypes.h:249-313.
 *
 * Differences from the reference, all additive:
 *   - every call returns a status (GB300_OK = 0) instead of void, and validates its
 *     arguments on the host before any launch; GB300GetLastErrorString() explains a failure;
 *   - every call takes a stream;
 *   - derivative stencils are ONE fused launch (the reference makes 3 or 6 launches,
 *     cudaEvaluator.cpp:171-292).
 * Launches are asynchronous: results are ready after GB300Synchronize(stream) (the
 * reference's CudaEvaluator::Synchronize, cudaEvaluator.cpp:377-380) or any later
 * synchronising call on that stream.
 */
#ifndef OSD_GB300_H
#define OSD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    GB300_OK = 0,
    GB300_ERR_INVALID_ARGUMENT = 1, /* null pointer, bad length/stride, inconsistent sizes */
    GB300_ERR_CUDA = 2,             /* a CUDA runtime call or launch failed */
    GB300_ERR_OUT_OF_MEMORY = 3,    /* device allocation failed; nothing was left allocated */
    GB300_ERR_UNSUPPORTED = 4,      /* e.g. an unknown patch type in a patch array */
    GB300_ERR_DEVICE_TIMEOUT = 5    /* a bounded device-side wait (4 s) gave up; the kernel
                                       recorded it and returned instead of waiting longer */
};

/* Patch types (Far::PatchDescriptor::Type, far/patchDescriptor.h:48-63). */
enum {
    GB300_PATCH_QUADS = 3,
    GB300_PATCH_TRIANGLES = 4,
    GB300_PATCH_LOOP = 5,
    GB300_PATCH_REGULAR = 6,
    GB300_PATCH_GREGORY_BASIS = 9,
    GB300_PATCH_GREGORY_TRIANGLE = 10
};

/* ---- status ---------------------------------------------------------------------------- */

/* Message for the last failing call on this thread ("" after success). */
const char *GB300GetLastErrorString(void);

/* Library version as MAJOR*10000 + MINOR*100 + PATCH. */
int GB300GetVersion(void);

/* Blocks until all work queued on `stream` has finished; replaces
 * CudaEvaluator::Synchronize (osd/cudaEvaluator.cpp:377-380). */
int GB300Synchronize(void *stream);

/* ---- EvalStencils -------------------------------------------------------------------------- */

/* dst[i] = sum_j weights[offsets[i]+j] * src[indices[offsets[i]+j]] for i in [start, end).
 * Replaces CudaEvalStencils (osd/cudaKernel.cu:351-383).  `sizes`, `offsets`, `indices`,
 * `weights` are device arrays of the Far::StencilTable (far/stencilTable.h:263-268).
 * Source and destination may be the same buffer (Osd::Mesh::Refine, osd/mesh.h:501-540) as
 * long as no destination element is also read as a source by another stencil.  Source rows
 * whose start and stride allow it are read with 128-/256-bit loads that may touch the row's
 * elements up to its stride: the source buffer must span every row's full stride (as Osd
 * vertex buffers of numVertices x stride floats do). */
int GB300EvalStencils(const float *src, float *dst, int length, int srcStride, int dstStride,
                      const int *sizes, const int *offsets, const int *indices,
                      const float *weights, int start, int end, void *stream);

/* Fused value + first (+ second) derivative stencils in one pass over the table.
 * Replaces the 3- and 6-launch paths of CudaEvaluator::EvalStencils
 * (osd/cudaEvaluator.cpp:171-292) over a Far::LimitStencilTable (stencilTable.h:409-579).
 * Any output pointer may be NULL to skip it (its weights are then not read); duu/duv/dvv
 * with their weights may all be NULL for first derivatives only. */
int GB300EvalStencilsWithDerivatives(
    const float *src, float *dst, float *du, float *dv, float *duu, float *duv, float *dvv,
    int length, int srcStride, int dstStride, int duStride, int dvStride, int duuStride,
    int duvStride, int dvvStride, const int *sizes, const int *offsets, const int *indices,
    const float *weights, const float *duWeights, const float *dvWeights,
    const float *duuWeights, const float *duvWeights, const float *dvvWeights, int start,
    int end, void *stream);

/* ---- EvalPatches --------------------------------------------------------------------------- */

/* Limit-surface positions at `numPatchCoords` patch coordinates.  Replaces CudaEvalPatches
 * (osd/cudaKernel.cu:387-402).  Coords whose arrayIndex is negative (a PatchMap miss) produce
 * zeros. */
int GB300EvalPatches(const float *src, float *dst, int length, int srcStride, int dstStride,
                     int numPatchCoords, const void *patchCoords, const void *patchArrays,
                     const int *patchIndices, const void *patchParams, void *stream);

/* Positions and derivatives; any output may be NULL.  Replaces
 * CudaEvalPatchesWithDerivatives (osd/cudaKernel.cu:404-424). */
int GB300EvalPatchesWithDerivatives(
    const float *src, float *dst, float *du, float *dv, float *duu, float *duv, float *dvv,
    int length, int srcStride, int dstStride, int duStride, int dvStride, int duuStride,
    int duvStride, int dvvStride, int numPatchCoords, const void *patchCoords,
    const void *patchArrays, const int *patchIndices, const void *patchParams, void *stream);

/* ---- device stencil table (CudaStencilTable, osd/cudaEvaluator.h:52-92) ------------------ */

typedef struct GB300StencilTable GB300StencilTable;

/* Copies a stencil table from HOST arrays (Far::StencilTable::GetSizes/GetOffsets/
 * GetControlIndices/GetWeights and, for limit tables, GetDu..DvvWeights; pass NULL for absent
 * derivative arrays) into device memory.  nnz = number of control indices.  Every stencil's
 * entries [offsets[i], offsets[i] + sizes[i]) must lie inside [0, nnz)
 * (GB300_ERR_INVALID_ARGUMENT otherwise).  On failure returns NULL and frees anything
 * partially allocated.
 * Device layout: when the stencils' entry ranges are disjoint (as Far builds them), the
 * entries of each stencil are stored in ascending control-index order with their weights
 * permuted alongside -- the same stencils, reordered so that neighbouring stencils gather the
 * same source rows together.  The Get*Buffer arrays hold that layout.  The table also keeps a
 * second, evaluation-only copy built on the device (32-stencil slices stored entry-major, in
 * locality order), which GB300StencilTableEval reads; it takes about as much device memory
 * as the Get*Buffer arrays. */
GB300StencilTable *GB300StencilTableCreate(int numStencils, int64_t nnz, const int *sizes,
                                           const int *offsets, const int *indices,
                                           const float *weights, const float *duWeights,
                                           const float *dvWeights, const float *duuWeights,
                                           const float *duvWeights, const float *dvvWeights,
                                           void *stream);
void GB300StencilTableDestroy(GB300StencilTable *table);
int GB300StencilTableGetNumStencils(const GB300StencilTable *table);
int64_t GB300StencilTableGetNumIndices(const GB300StencilTable *table);
/* which: 0 sizes, 1 offsets, 2 indices, 3 weights, 4 du, 5 dv, 6 duu, 7 duv, 8 dvv. */
void *GB300StencilTableGetBuffer(const GB300StencilTable *table, int which);

/* EvalStencils over a device table (CudaEvaluator::EvalStencils template form,
 * osd/cudaEvaluator.h:125-142): all stencils [0, numStencils), outputs as in
 * GB300EvalStencilsWithDerivatives (NULL outputs skipped). */
int GB300StencilTableEval(const GB300StencilTable *table, const float *src, float *dst,
                          float *du, float *dv, float *duu, float *duv, float *dvv, int length,
                          int srcStride, int dstStride, int duStride, int dvStride,
                          int duuStride, int duvStride, int dvvStride, void *stream);

/* Copies device buffer `which` (as GB300StencilTableGetBuffer) of a table to HOST memory:
 * numStencils ints for sizes / offsets, numIndices elements otherwise.  Synchronous. */
int GB300StencilTableCopyBuffer(const GB300StencilTable *table, int which, void *hostDst,
                                void *stream);

/* ---- GPU stencil-table factory (Far::StencilTableFactory, far/stencilTableFactory.cpp) ---- */

/* The subdivision masks of one refinement level, in HOST memory: for each vertex of the level
 * (row order), the (source, weight) pairs that Far::PrimvarRefiner::Interpolate /
 * InterpolateVarying / InterpolateFaceVarying passes to StencilBuilder::Index::AddWithWeight
 * (far/primvarRefiner.h:475-650, far/stencilBuilder.cpp:509-518), in call order, zero weights
 * left out.  Sources are global vertex indices: control vertices [0, numControl), then the
 * vertices of level 1, 2, ... concatenated.  A level's masks refer to the previous level and
 * to vertices of their own level (Catmark face points feed edge and vertex points). */
typedef struct GB300StencilMasks {
    int numRows;
    int64_t nnz;
    const int64_t *offsets; /* numRows + 1 */
    const int *sources;     /* nnz */
    const float *weights;   /* nnz */
} GB300StencilMasks;

/* Far::StencilTableFactory::Create (far/stencilTableFactory.cpp:78-151) with
 * factorizeIntermediateLevels, merging on the device: each row is the merge, in first-touch
 * order with float products and sums, of its mask weights times the factorized rows of its
 * sources (control vertices are rows of one entry of weight 1), exactly as WeightTable::merge
 * (far/stencilBuilder.cpp:164-198,310-385).  The table holds the rows of every level
 * (generateIntermediateLevels) or of the last level only, preceded by one identity stencil per
 * control vertex when generateControlVerts is set.  sortEntries = 0 keeps each stencil's
 * entries in Far's order (the table then equals Far's bit for bit); 1 sorts them by control
 * index (the GB300StencilTableCreate layout).  Returns NULL on failure (status recorded). */
GB300StencilTable *GB300StencilTableFactoryCreate(int numControl, int numLevels,
                                                  const GB300StencilMasks *levels,
                                                  int generateIntermediateLevels,
                                                  int generateControlVerts, int sortEntries,
                                                  void *stream);

/* Stencils composed from the stencils of a DEVICE table given by its arrays in Far's layout
 * (baseSizes / baseOffsets per stencil, baseIndices, baseWeights): row i merges, over its mask
 * entries k (HOST arrays offsets[numRows + 1], sources, weights[c] for c < numChannels), the
 * products weights[c][k] * w of the entries (index, w) of base stencil sources[k], zero w
 * skipped, first-touch order, float arithmetic -- StencilBuilder::Index::AddWithWeight with a
 * StencilReal source (far/stencilBuilder.cpp:520-598).  numChannels 1, 3 (P, du, dv) or
 * 6 (+ duu, duv, dvv).  appendBase = 1 puts the base stencils first (AppendLocalPointStencilTable,
 * far/stencilTableFactory.cpp:255-407, with local-point stencils as the masks); 0 returns the
 * composed rows alone (LimitStencilTableFactory's per-location stencils,
 * far/stencilTableFactory.cpp:560-640, with patch CVs and basis weights as the masks). */
GB300StencilTable *GB300StencilTableComposeRows(
    int baseNumStencils, int64_t baseNumIndices, const int *baseSizes, const int *baseOffsets,
    const int *baseIndices, const float *baseWeights, int numRows, int64_t nnz,
    const int64_t *offsets, const int *sources, int numChannels, const float *const *weights,
    int appendBase, int sortEntries, void *stream);

/* ---- device patch table (CudaPatchTable, osd/cudaPatchTable.h:51-110) -------------------- */

typedef struct GB300PatchTable GB300PatchTable;

/* Copies a flattened patch table (Osd::CpuPatchTable layout: PatchArray[numArrays],
 * patch index buffer, PatchParam[numPatches]) from HOST memory into device memory, and
 * builds the device PatchMap (far/patchMap.cpp) from the params.  `triangular` selects the
 * triangle quadtree (Loop-scheme tables). */
GB300PatchTable *GB300PatchTableCreate(int numArrays, const void *patchArrays,
                                       int64_t numIndices, const int *patchIndices,
                                       int numPatches, const void *patchParams, int triangular,
                                       void *stream);
void GB300PatchTableDestroy(GB300PatchTable *table);
/* which: 0 patch arrays, 1 patch indices, 2 patch params. */
void *GB300PatchTableGetBuffer(const GB300PatchTable *table, int which);
int GB300PatchTableGetNumArrays(const GB300PatchTable *table);
int GB300PatchTableGetNumPatches(const GB300PatchTable *table);

/* Device Far::PatchMap::FindPatch (far/patchMap.h:192-231) for n queries (face, u, v) held in
 * DEVICE memory; writes one OsdPatchCoord per query (s, t = u, v) to `coordsOut` (device).
 * Misses (faces outside the table or holes) get handle {-1, -1, -1}.  Handles are bit-exact
 * with the reference's double-precision walk for float inputs. */
int GB300PatchTableFindPatches(const GB300PatchTable *table, int n, const int *faces,
                               const float *u, const float *v, void *coordsOut, void *stream);

/* EvalPatches against a device table (CudaEvaluator::EvalPatches template form). */
int GB300PatchTableEval(const GB300PatchTable *table, const float *src, float *dst, float *du,
                        float *dv, float *duu, float *duv, float *dvv, int length,
                        int srcStride, int dstStride, int duStride, int dvStride,
                        int duuStride, int duvStride, int dvvStride, int numPatchCoords,
                        const void *patchCoords, void *stream);

/* Varying and face-varying patch tables (CudaPatchTable's varying / fvar buffers,
 * osd/cudaPatchTable.h:51-110, flattened as osd/cpuPatchTable.cpp:75-114).  Both describe the
 * vertex table's patches -- the same arrays with the same patch counts and first patches -- so
 * the vertex PatchMap's coords index them.  Varying patches use the vertex patch params; each
 * face-varying channel has its own params (numParams = the vertex table's numPatches).
 * HOST arrays in, as for GB300PatchTableCreate.  AddFVarChannel writes the channel index. */
int GB300PatchTableSetVarying(GB300PatchTable *table, int numArrays, const void *patchArrays,
                              int64_t numIndices, const int *patchIndices, void *stream);
int GB300PatchTableAddFVarChannel(GB300PatchTable *table, int numArrays, const void *patchArrays,
                                  int64_t numIndices, const int *patchIndices, int numParams,
                                  const void *patchParams, int *channel, void *stream);
int GB300PatchTableGetNumFVarChannels(const GB300PatchTable *table);
/* which: 0 patch arrays, 1 patch indices (NULL when no varying table was set). */
void *GB300PatchTableGetVaryingBuffer(const GB300PatchTable *table, int which);
/* which: 0 patch arrays, 1 patch indices, 2 patch params of face-varying `channel`. */
void *GB300PatchTableGetFVarBuffer(const GB300PatchTable *table, int channel, int which);

/* CudaEvaluator::EvalPatchesVarying (osd/cudaEvaluator.h:859-1060): EvalPatches over the
 * varying arrays / indices with the vertex patch params. */
int GB300PatchTableEvalVarying(const GB300PatchTable *table, const float *src, float *dst,
                               float *du, float *dv, float *duu, float *duv, float *dvv,
                               int length, int srcStride, int dstStride, int duStride,
                               int dvStride, int duuStride, int duvStride, int dvvStride,
                               int numPatchCoords, const void *patchCoords, void *stream);
/* CudaEvaluator::EvalPatchesFaceVarying (osd/cudaEvaluator.h:1070-1255): EvalPatches over
 * face-varying channel `channel` (its arrays, indices and params). */
int GB300PatchTableEvalFaceVarying(const GB300PatchTable *table, int channel, const float *src,
                                   float *dst, float *du, float *dv, float *duu, float *duv,
                                   float *dvv, int length, int srcStride, int dstStride,
                                   int duStride, int dvStride, int duuStride, int duvStride,
                                   int dvvStride, int numPatchCoords, const void *patchCoords,
                                   void *stream);

/* ---- Bfr tessellation of a mesh (Bfr::Tessellation, bfr/tessellation.h:142-262) ----------- */

/* Bfr::Tessellation::Options (bfr/tessellation.h:60-100).  facetSize: 4 selects quads-capable
 * 4-tuples (a triangle's 4th index is -1), anything else triangles (SetFacetSize);
 * preserveQuads keeps quads of quad-based faces when facetSize is 4; coordStride / facetStride
 * are floats between (u,v) pairs and ints between facets, 0 for the defaults (2, facetSize). */
typedef struct GB300TessellationOptions {
    int facetSize;
    int preserveQuads;
    int coordStride;
    int facetStride;
} GB300TessellationOptions;

/* One Bfr::Tessellation(Parameterization(scheme, faceSizes[f]), rates, options) per face of a
 * mesh, all faces at once.  regularFaceSize is the scheme's regular face size (4: Catmark or
 * Bilinear, 3: Loop) that Bfr::Parameterization derives from the scheme
 * (bfr/parameterization.cpp:40-66).  Rates, all DEVICE arrays:
 *   rates == NULL      every face uses the single rate uniformRate (Tessellation(p, rate));
 *   rateOffsets == NULL  face f uses the single rate rates[f];
 *   otherwise          face f uses rates[rateOffsets[f] .. rateOffsets[f+1]), interpreted as
 *                      Tessellation(p, numRates, rates) interprets them (1 inner rate, N edge
 *                      rates, N+1, or for quads 2 or N+2; bfr/tessellation.h:125-150).
 * A face whose tessellation is invalid (a rate < 1, a face size the scheme rejects) gets no
 * coords and no facets, as an invalid Bfr::Tessellation has none; callers skip faces without
 * a limit surface (holes) the same way, with a rate of 0.
 *
 * Count writes, into DEVICE arrays of numFaces + 1 entries, the exclusive scans of each face's
 * coord count (GetNumCoords), facet count (GetNumFacets) and ptex-face count (Far::PtexIndices,
 * far/ptexIndices.cpp:37-55: 1 for a regular face, N for an N-gon), and the three totals into
 * the HOST array totals[3].  It synchronizes `stream` to read the totals.  Totals above
 * INT_MAX coords are rejected (facet indices are ints). */
int GB300TessellationCount(int regularFaceSize, int numFaces, const int *faceSizes,
                           const int *rateOffsets, const int *rates, int uniformRate,
                           const GB300TessellationOptions *options, int64_t *coordOffsets,
                           int64_t *facetOffsets, int64_t *ptexOffsets, int64_t *totals,
                           void *stream);

/* Writes every face's coords (Tessellation::GetCoords: boundary coords first, then interior,
 * bit-identical to the reference's float coords) at coordOffsets[f] and its facets
 * (GetFacets) at facetOffsets[f], into DEVICE buffers sized from Count's totals.  With
 * offsetFacetIndices the facet indices are offset by coordOffsets[f] to number the mesh's
 * coords (Tessellation::TransformFacetCoordIndices(facets, commonOffset),
 * tessellation.cpp:2429-2447); otherwise they are face-local, as GetFacets returns them.
 *
 * With a patch table (built with the approximation the surfaces should have, e.g. the Far
 * options the reference's Bfr regression pairs with Bfr::SurfaceFactory's defaults: isolation
 * 6 for sharp and 2 for smooth features, Gregory-basis end caps, infinitely sharp patches,
 * regression/bfr_evaluate/farPatchEvaluator.cpp:52-78) and ptexOffsets from Count, each coord
 * is also located: Parameterization::ConvertCoordToNormalizedSubFace picks an N-gon's ptex
 * sub-face and the table's PatchMap finds the patch, giving one OsdPatchCoord per coord in
 * `patchCoords` (DEVICE, 5 x 32 bits each) for GB300PatchTableEval -- the Bfr::Surface::
 * Evaluate of every tessellation coord of the mesh. */
int GB300TessellationGenerate(int regularFaceSize, int numFaces, const int *faceSizes,
                              const int *rateOffsets, const int *rates, int uniformRate,
                              const GB300TessellationOptions *options,
                              const int64_t *coordOffsets, const int64_t *facetOffsets,
                              const int64_t *ptexOffsets, float *coords, int *facets,
                              int offsetFacetIndices, const GB300PatchTable *table,
                              void *patchCoords, void *stream);

/* Bfr::Surface::Evaluate (bfr/surface.h:227-242) at every coord of a mesh tessellation: P and
 * any of Du, Dv, Duu, Duv, Dvv (NULL to skip) of `length`-wide points at the PatchCoords that
 * GB300TessellationGenerate located on `table`.  The same arithmetic as GB300PatchTableEval,
 * with the kernel chosen for coords grouped by patch, as a tessellation's are (one point per
 * thread: the warp shares each patch's row loads and every point's basis is computed once).
 * DEVICE pointers; strides in floats. */
int GB300TessellationEvaluate(const GB300PatchTable *table, const float *src, float *P,
                              float *Du, float *Dv, float *Duu, float *Duv, float *Dvv,
                              int length, int srcStride, int pStride, int duStride, int dvStride,
                              int duuStride, int duvStride, int dvvStride, int numCoords,
                              const void *patchCoords, void *stream);

/* Per-edge tessellation rates from edge lengths, the non-uniform rates of the reference's Bfr
 * tutorial 2.1 (tutorials/bfr/tutorial_2_1/bfr_tutorial_2_1.cpp:121-166, 240-308): for every
 * face corner, the length of the edge to the next corner of its face (float, from the absolute
 * coordinate differences of the two points) and the rate 1 + (int)(length / interval), capped
 * at maxRate.  Points (DEVICE, xyz at `pointStride` floats): with pointsPerCorner 0, one per
 * mesh vertex, named by faceVerts (the tutorial's control-hull option); with pointsPerCorner 1,
 * one per face corner in corner order (the tutorial's limit option: the limit positions at the
 * face's corners, e.g. GB300TessellationEvaluate at the rate-1 tessellation's vertex coords).
 * Writes rates (DEVICE, numCorners ints) and, if not NULL, rateOffsets (DEVICE, numFaces + 1:
 * the exclusive scan of the face sizes), the per-face runs GB300TessellationCount takes.  With
 * hull points a shared edge gets one rate from both faces.  Synchronizes `stream`. */
int GB300TessellationEdgeRates(int numFaces, const int *faceSizes, const int *faceVerts,
                               int64_t numCorners, const float *points, int numPoints,
                               int pointStride, int pointsPerCorner, float interval,
                               int maxRate, int *rateOffsets, int *rates, void *stream);

/* Shared (watertight) points of a mesh tessellation: the bookkeeping of the reference's Bfr
 * tutorial with shared vertex and edge points (tutorials/bfr/tutorial_2_2/
 * bfr_tutorial_2_2.cpp:244-430), for every face at once, after Count and Generate with the
 * same faces, rates and options.  faceVerts / faceEdges (DEVICE, numCorners entries each, one
 * per face corner, faces in order: Far::TopologyLevel::GetFaceVertices / GetFaceEdges of the
 * base level, edge i running from corner i to corner i + 1; the face sizes must add up to
 * numCorners) name numVertices vertices and numEdges edges.
 *
 * The point of a mesh vertex, and the rate - 1 points inside a mesh edge, are made by the
 * first face (in face order) that reaches them, from its own coords; later faces reuse them,
 * edge points reversed where a face runs the edge from the other end.  A face's interior coords
 * are all new points.  Points are numbered face by face, in each face its new boundary points
 * in boundary order and then its interior coords, as the tutorial numbers them.  Faces without
 * coords take no part.  An edge needs one rate in all its faces (rates from edge lengths have
 * that); an edge with two rates is rejected.
 *
 * facets (DEVICE, in place): Generate's facets, mesh-wide (meshFacetIndices != 0) or face-local
 * coord indices in, point indices out (Tessellation::TransformFacetCoordIndices(facets,
 * boundaryIndices, interiorOffset), tessellation.cpp:2449-2464); -1 entries stay -1.
 * pointOffsets (DEVICE, numFaces + 1): the first point each face makes; *numPoints (HOST) the
 * total.  Optional DEVICE outputs, one entry per point (capacity: Count's coord total):
 * pointPatchCoords (5 x 32 bits, copied from the coord's PatchCoord in coordPatchCoords, so
 * GB300TessellationEvaluate evaluates each point once), pointCoords (the coord's (u, v)) and
 * pointFaces (the face that made it); vertexPoints (numVertices) and edgePoints (numEdges: the
 * first point inside the edge in its maker's direction), -1 where none.  Synchronizes
 * `stream`.  Overlapping calls with the same outputs race. */
int GB300TessellationShare(int regularFaceSize, int numFaces, const int *faceSizes,
                           const int *rateOffsets, const int *rates, int uniformRate,
                           const GB300TessellationOptions *options,
                           const int64_t *coordOffsets, const int64_t *facetOffsets,
                           const int *faceVerts, const int *faceEdges, int64_t numCorners,
                           int numVertices, int numEdges, int *facets, int meshFacetIndices,
                           const void *coordPatchCoords, const float *coords,
                           int64_t *pointOffsets, void *pointPatchCoords, float *pointCoords,
                           int *pointFaces, int *vertexPoints, int *edgePoints,
                           int64_t *numPoints, void *stream);

/* Bfr::Surface::EvaluateStencil (bfr/surface.h:244-265) at every point: one limit stencil per
 * PatchCoord (DEVICE, 5 x 32 bits each, e.g. located by GB300TessellationGenerate or shared by
 * GB300TessellationShare) over the mesh's control vertices, so that GB300EvalStencils /
 * GB300StencilTableEval evaluate the points straight from the control vertices, frame after
 * frame, without refining.  The base table (DEVICE arrays in Far's layout: sizes / offsets per
 * stencil, indices, weights) holds one stencil per point the patch indices name, in their
 * numbering: the control vertices first (identity rows), then the refined and local points --
 * Far::StencilTableFactory with generateControlVerts plus AppendLocalPointStencilTable, as
 * Far::LimitStencilTableFactory builds it (far/stencilTableFactory.cpp:411-662).  Each point's
 * stencil merges the basis weights of its patch's control points (P; with numChannels 3 also
 * Du, Dv; with 6 the second derivatives) times their base stencils, in first-touch order, as
 * LimitStencilTableFactory merges its per-location masks.  sortEntries as in
 * GB300StencilTableComposeRows.  Returns NULL on failure (status recorded). */
GB300StencilTable *GB300TessellationStencils(const GB300PatchTable *table, int numPoints,
                                             const void *patchCoords, int baseNumStencils,
                                             int64_t baseNumIndices, const int *baseSizes,
                                             const int *baseOffsets, const int *baseIndices,
                                             const float *baseWeights, int numChannels,
                                             int sortEntries, void *stream);

/* ---- draw-time tessellation factors (osd/glslPatchCommonTess.glsl:92-760) ------------------ */

/* The tess-control settings of OpenSubdiv's patch shaders.  tessLevel: OsdTessLevel();
 * maxTessLevel: the device maximum the shaders read as gl_MaxTessGenLevel (64 on current
 * hardware); screenSpace: OSD_ENABLE_SCREENSPACE_TESSELLATION; spacing: 0 equal,
 * 1 fractional even, 2 fractional odd (OSD_FRACTIONAL_EVEN/ODD_SPACING); modelView,
 * projection: OsdModelViewMatrix() / OsdProjectionMatrix(), column-major like a GLSL mat4. */
typedef struct GB300PatchTessOptions {
    float tessLevel;
    float maxTessLevel;
    int screenSpace;
    int spacing;
    float modelView[16];
    float projection[16];
} GB300PatchTessOptions;

/* Per-patch tessellation factors for every patch of a device table, as the tess-control stage
 * of the patch shaders computes them: uniform (OsdGetTessLevelsUniform[Triangle], from the
 * refinement level and transition mask) or screen-space (OsdComputeTessLevel of each boundary
 * edge, and of each half of a transition edge, between limit positions at the patch's corners
 * and edge midpoints), then outer and inner levels for the spacing (OsdComputeTessLevels
 * [Triangle]).  src: the patch points (xyz at srcStride floats; only read for screen-space
 * factors).  DEVICE outputs per patch, in patch-param order: outer[4] (16-byte aligned),
 * inner[2], and optionally the Lo / Hi halves of the outer levels (tessOuterLo / tessOuterHi,
 * 16-byte aligned) that GB300PatchTessParameterization needs. */
int GB300PatchTableTessFactors(const GB300PatchTable *table, const float *src, int srcStride,
                               const GB300PatchTessOptions *options, float *outer, float *inner,
                               float *outerLo, float *outerHi, void *stream);

/* OsdGetTessParameterization[Triangle] (glslPatchCommonTess.glsl:692-730): maps n tessellator
 * domain points (u, v, w; w unused for quads) of patches patchIndex[i] to patch coordinates,
 * placing the points of split transition edges on their two halves.  DEVICE arrays; uv gets 2
 * floats per point. */
int GB300PatchTessParameterization(int n, const float *domain, const int *patchIndex,
                                   const float *outerLo, const float *outerHi, int spacing,
                                   int triangular, float *uv, void *stream);

/* ---- vertex buffer (CudaVertexBuffer, osd/cudaVertexBuffer.h:42-79) ---------------------- */

typedef struct GB300VertexBuffer GB300VertexBuffer;

/* numElements floats per vertex; sizes are computed in 64 bits (the reference computes them
 * in int, cudaVertexBuffer.cpp:85). */
GB300VertexBuffer *GB300VertexBufferCreate(int numElements, int numVertices);
void GB300VertexBufferDestroy(GB300VertexBuffer *buffer);
/* Host -> device copy of numVertices vertices starting at startVertex
 * (CudaVertexBuffer::UpdateData, cudaVertexBuffer.cpp:55-63).  Asynchronous on `stream`
 * (pageable host memory makes it effectively synchronous). */
int GB300VertexBufferUpdateData(GB300VertexBuffer *buffer, const float *src, int startVertex,
                                int numVertices, void *stream);
float *GB300VertexBufferBindCudaBuffer(GB300VertexBuffer *buffer);
int GB300VertexBufferGetNumElements(const GB300VertexBuffer *buffer);
int GB300VertexBufferGetNumVertices(const GB300VertexBuffer *buffer);

/* ---- batched EvalStencils (no counterpart in the reference) ------------------------------ */

/* A batch evaluates many meshes' device stencil tables in ONE persistent launch, instead of one
 * GB300StencilTableEval (CudaEvaluator::EvalStencils, osd/cudaEvaluator.h:125-142) per mesh:
 * job i computes dst[i][k*dstStride[i] + e] = sum_j w_j * src[i][idx_j*srcStride[i] + e] for
 * every stencil k of tables[i] and element e < length[i] (pointers already include the
 * BufferDescriptor offset, as in the raw EvalStencils forms).  Results are those of the
 * per-mesh call (bit-identical for stencils evaluated one per thread, within float rounding
 * for warp-evaluated large stencils).  The batch keeps the pointers: tables and buffers must
 * outlive it, and the source / destination contents may change between evaluations. */
typedef struct GB300StencilBatch GB300StencilBatch;

/* Builds the job table and the tile prefix on the device (synchronous on `stream`).  When
 * every table has its sliced evaluation layout (tables from GB300StencilTableCreate and the
 * factories), the batch reads those: tiles of 8 slices, one warp per 32-stencil slice;
 * otherwise the Far-layout arrays.  Jobs whose source rows are unaligned (no 16-byte vector
 * loads) and at most 8 floats wide get a device buffer for a padded copy of their source
 * (rows of 8 floats), refreshed by every evaluation.  Uses the tuned configuration cached for batches with the same work histogram,
 * if any.  Returns NULL on failure (error string set). */
GB300StencilBatch *GB300StencilBatchCreate(int numJobs, GB300StencilTable *const *tables,
                                           const float *const *src, float *const *dst,
                                           const int *length, const int *srcStride,
                                           const int *dstStride, void *stream);
void GB300StencilBatchDestroy(GB300StencilBatch *batch);
/* One evaluation of every job: a counter reset and one kernel on `stream`. */
int GB300StencilBatchEval(GB300StencilBatch *batch, void *stream);
/* The same, replayed from a CUDA graph captured on the first call (on a private stream) and
 * launched on `stream`.  The graph is dropped and recaptured after GB300StencilBatchTune. */
int GB300StencilBatchEvalGraph(GB300StencilBatch *batch, void *stream);
/* Autotuner: times each candidate (stencils per tile, CTAs per SM (1-3, capped by what the
 * kernel keeps resident), mean stencil size above which a job switches to one warp per
 * stencil, tiles claimed from a work counter or assigned round-robin; sliced batches only try
 * the CTA counts and the claim order) over `iterations` evaluations on the batch itself, keeps the fastest, and
 * caches it for later batches with the same histogram of work over (stencil size, job size,
 * primvar width) classes.  Writes the outputs as Eval does. */
int GB300StencilBatchTune(GB300StencilBatch *batch, int iterations, void *stream);
int GB300StencilBatchGetConfig(const GB300StencilBatch *batch, int *tileStencils,
                               int *ctasPerSm, int *warpThreshold, int *numTiles,
                               int *dynamicClaims);
/* Reads and clears the batch kernel's status word (GB300_OK or GB300_ERR_DEVICE_TIMEOUT);
 * synchronous. */
int GB300StencilBatchGetDeviceStatus(GB300StencilBatch *batch, int *status);

/* ---- serving loop (no counterpart in the reference) --------------------------------------- */

/* A request server for many topologies: keeps their stencil and patch tables resident in a
 * fixed device-memory budget (least-recently-used topologies are evicted and re-uploaded on
 * demand), batches the refine and limit-evaluation requests that are pending when a stream
 * frees up into one round (one batched stencil launch + PatchMap/EvalPatches per limit
 * request), and overlaps rounds on several streams.  Requests carry HOST control values and
 * receive HOST results; pinned host memory keeps the copies asynchronous.  All device memory
 * (table pool + request arena) is allocated by GB300ServerCreate. */
typedef struct GB300Server GB300Server;

enum { GB300_REQUEST_REFINE = 0, GB300_REQUEST_LIMIT = 1 };

typedef struct {
    size_t tableBudgetBytes;  /* device bytes for resident topologies (LRU-evicted) */
    size_t arenaBytes;        /* device bytes for the inputs/outputs of requests in flight */
    int streams;              /* rounds in flight, one stream each */
    int maxRequestsPerRound;
    int plain;                /* 1: one request at a time through the plain entry points */
    int pinHostTables;        /* 1: page-lock each topology's host arrays when it is added
                                 (cudaHostRegister), so uploads after an eviction are
                                 asynchronous; arrays shared by several topologies are
                                 registered once */
} GB300ServerConfig;

/* A topology's tables, as HOST arrays that must stay valid while the server exists (they are
 * re-uploaded after an eviction).  Refine: a Far-layout stencil table over the numControl
 * control vertices (each `length` floats).  Limit (optional, numPatchArrays = 0 disables it):
 * the patch points -- every point the patch table indexes -- as stencils over the control
 * vertices' first 3 floats (patch point k = stencil k), and the flattened patch table
 * (Osd::CpuPatchTable layout, as GB300PatchTableCreate takes it). */
typedef struct {
    int numControl;
    int length;
    int numStencils;
    int64_t nnz;
    const int *sizes, *offsets, *indices;
    const float *weights;
    int numPatchPoints;
    int64_t patchPointNnz;
    const int *ppSizes, *ppOffsets, *ppIndices;
    const float *ppWeights;
    int numPatchArrays;
    const void *patchArrays;
    int64_t numPatchIndices;
    const int *patchIndices;
    int numPatches;
    const void *patchParams;
    int triangular;
} GB300TopologyDesc;

/* One request.  REFINE: out = numStencils x length floats (the refined points).  LIMIT:
 * numPoints (ptex face, u, v) queries; out = P, dPdu, dPdv, each numPoints x 3 floats, one
 * after the other (a query that misses the patch map gives zeros). */
typedef struct {
    int topology;
    int kind;
    const float *controlValues;
    float *out;
    int numPoints;
    const int *faces;
    const float *u, *v;
} GB300Request;

typedef struct {
    uint64_t submitted, completed, failed, rounds, uploads, evictions;
    uint64_t bytesUploaded, residentBytes, peakResidentBytes;
    /* where the time goes (nanoseconds): the scheduler thread queueing rounds (host API
     * calls), waiting with requests pending while every stream is busy, waiting with
     * requests pending for arena or table-pool space; and the rounds' device time (first
     * copy to completion, CUDA events, summed over rounds) */
    uint64_t launchNanos, streamsBusyNanos, memoryWaitNanos, roundDeviceNanos;
    /* request bytes copied host -> device (control values, queries) and back (results) */
    uint64_t h2dBytes, d2hBytes;
    /* host table bytes page-locked by the server (pinHostTables), and table ranges that could
     * not be (their uploads are staged through pageable copies) */
    uint64_t hostPinnedBytes, hostPinFailures;
} GB300ServerStats;

/* ---- table cache (no counterpart in the reference) --------------------------------------- */

/* Writes a topology's tables (the arrays a GB300TopologyDesc points at) to one file: a 256-byte
 * header with counts, array offsets and an FNV-1a checksum, then the arrays, 64-byte aligned.
 * Written to `<path>.tmp` and renamed, so readers never see a partial file. */
int GB300TableCacheWrite(const char *path, const GB300TopologyDesc *desc);
/* Maps a table cache read-only and fills `desc` with pointers into the mapping (valid until
 * GB300TableCacheClose(*handle)).  verify = 1 checks the payload checksum (reads the file). */
int GB300TableCacheOpen(const char *path, int verify, GB300TopologyDesc *desc, void **handle);
void GB300TableCacheClose(void *handle);

GB300Server *GB300ServerCreate(const GB300ServerConfig *config);
/* Finishes every submitted request, then frees the server. */
void GB300ServerDestroy(GB300Server *server);
int GB300ServerAddTopology(GB300Server *server, int id, const GB300TopologyDesc *desc);
/* The same from a table cache file: the server keeps the file mapped and uploads from the
 * mapping, so a topology evicted from device memory is re-read from the file (through the page
 * cache) instead of being held in host memory. */
int GB300ServerAddTopologyFromCache(GB300Server *server, int id, const char *path);
/* Queues a request (thread-safe); its buffers must stay valid until it completes. */
int GB300ServerSubmit(GB300Server *server, const GB300Request *request, uint64_t *ticket);
/* Blocks until the request completed; latency = submit -> results in host memory. */
int GB300ServerWait(GB300Server *server, uint64_t ticket, double *latencySeconds);
/* Open-loop load: submits request i at arrivalSeconds[i] after the call starts, waits for
 * all, and writes each request's latency. */
int GB300ServerReplay(GB300Server *server, int n, const GB300Request *requests,
                      const double *arrivalSeconds, double *latencySeconds);
int GB300ServerGetStats(GB300Server *server, GB300ServerStats *stats);

/* ---- batched EvalStencils that allocates nothing (no counterpart in the reference) -------- */

/* For callers that cannot allocate: a renderer running under a fixed device-memory budget or
 * a pool it does not own, or code that must not call cudaMalloc / cudaFree (they synchronise
 * the device) inside its frame loop.  Evaluates numJobs raw-pointer EvalStencils jobs (the
 * arguments of GB300EvalStencils per job, over stencils [0, numStencils[k]); every array
 * argument is a HOST array indexed by job, holding device pointers or ints) in one batched
 * launch, like GB300StencilBatchEval with one stencil per thread.  It allocates no device or
 * host memory: its scratch (work counter, job table, tile prefix) is a fixed 36,352-byte device
 * array inside the library (256 + 256 job descriptors of 136 bytes + 1,280), so at most 256
 * jobs per call (more are rejected with GB300_ERR_INVALID_ARGUMENT and a message).  The job
 * table is copied into that array from the host stack with cudaMemcpyAsync on `stream`, and
 * the counter is cleared on `stream` before the kernel.  Table arrays must be 16-byte aligned.
 * A bounded wait that expires inside the kernel leaves outputs incomplete and is reported by
 * the next GB300GetDeviceStatus(), like every other staged kernel of the library.
 * The first call on each device looks up the array's device address (cudaGetSymbolAddress,
 * with that device current): make that first call before any stream capture.  There is one
 * array per device, so calls that can overlap on a device (different streams, or different
 * host threads without ordering) race: serialise them on one stream. */
int GB300EvalStencilsBatchedNoAlloc(int numJobs, const float *const *src, float *const *dst,
                                    const int *length, const int *srcStride,
                                    const int *dstStride, const int *numStencils,
                                    const int *const *sizes, const int *const *offsets,
                                    const int *const *indices, const float *const *weights,
                                    void *stream);

/* Reads and clears the device-side status word of the current device: GB300_OK, or
 * GB300_ERR_DEVICE_TIMEOUT if a bounded wait inside a staged kernel gave up (the kernel then
 * left its outputs incomplete).  Synchronises the device. */
int GB300GetDeviceStatus(void);

/* ---- measurement (no counterpart in the reference) ---------------------------------------- */

/* Times a compute-only FP32 fused multiply-add kernel on `stream` (one full-occupancy wave,
 * 5 timed launches after a warm-up, CUDA events) and writes the rate in TFLOP/s (an FMA counts
 * as 2).  The compute denominator of the EvalPatches roofline. */
int GB300MeasureFp32Rate(double *tflops, void *stream);

/* ---- kernel accounting -------------------------------------------------------------------- */

/* Number of this library's kernels launched since load (for launch-count reporting). */
uint64_t GB300GetLaunchCount(void);

#ifdef __cplusplus
}
#endif
#endif /* OSD_GB300_H */
