/*
 * osd_oracle.c -- CPU restatement of the Osd evaluation path (the checker).
 *
 * TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline; never by the product.  Built by oracle/Makefile with floating-point contraction
 * disabled so its float results round exactly like the reference's Osd::CpuEvaluator.
 *
 * Reference citations are relative to the OpenSubdiv 3.6.0 source tree.
 */
#include "osd_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- patch basis, float and double instantiations ------------------------------------ */
#define R float
#define SFX _f
#define ORC_K6 (1.0f / 6.0f)
#define ORC_K12 (1.0f / 12.0f)
#include "oracle_basis.inc"
#undef R
#undef SFX
#undef ORC_K6
#undef ORC_K12

#define R double
#define SFX _d
#define ORC_K6 (1.0 / 6.0)
#define ORC_K12 (1.0 / 12.0)
#include "oracle_basis.inc"
#undef R
#undef SFX
#undef ORC_K6
#undef ORC_K12

/* ---- EvalStencils (osd/cpuKernel.cpp:71-240, osd/cpuEvaluator.cpp:37-125) ------------ */

static int descs_ok(const int *srcDesc, int nout, const int *dstDesc) {
    for (int k = 0; k < nout; ++k)
        if (dstDesc[3 * k + 1] != srcDesc[1]) return 0;
    return 1;
}

#define MAX_LEN 256

int orc_eval_stencils_f(const float *src, const int *srcDesc, int nout, float *const *dst,
                        const int *dstDesc, const int *sizes, const int *offsets,
                        const int *indices, const float *const *weights, int start, int end,
                        int nthreads) {
    if (end <= start) return 1;
    if (!descs_ok(srcDesc, nout, dstDesc)) return 0;
    const int len = srcDesc[1], sstride = srcDesc[2];
    if (len > MAX_LEN) return 0;
    const float *s0 = src + srcDesc[0];
#pragma omp parallel for schedule(static, 4096) num_threads(nthreads > 0 ? nthreads : 1)
    for (int i = start; i < end; ++i) {
        float acc[6][MAX_LEN];
        for (int k = 0; k < nout; ++k)
            for (int e = 0; e < len; ++e) acc[k][e] = 0.0f;
        const int n = sizes[i], o = offsets[i];
        for (int j = 0; j < n; ++j) {
            const float *row = s0 + (size_t)indices[o + j] * sstride;
            for (int k = 0; k < nout; ++k) {
                const float wk = weights[k][o + j];
                for (int e = 0; e < len; ++e) acc[k][e] += row[e] * wk;
            }
        }
        for (int k = 0; k < nout; ++k) {
            if (!dst[k]) continue;
            float *d = dst[k] + dstDesc[3 * k] + (size_t)i * dstDesc[3 * k + 2];
            memcpy(d, acc[k], sizeof(float) * len);
        }
    }
    return 1;
}

int orc_eval_stencils_d(const float *src, const int *srcDesc, int nout, double *const *dst,
                        const int *dstDesc, const int *sizes, const int *offsets,
                        const int *indices, const float *const *weights, int start, int end,
                        int nthreads) {
    if (end <= start) return 1;
    if (!descs_ok(srcDesc, nout, dstDesc)) return 0;
    const int len = srcDesc[1], sstride = srcDesc[2];
    if (len > MAX_LEN) return 0;
    const float *s0 = src + srcDesc[0];
#pragma omp parallel for schedule(static, 4096) num_threads(nthreads > 0 ? nthreads : 1)
    for (int i = start; i < end; ++i) {
        double acc[6][MAX_LEN];
        for (int k = 0; k < nout; ++k)
            for (int e = 0; e < len; ++e) acc[k][e] = 0.0;
        const int n = sizes[i], o = offsets[i];
        for (int j = 0; j < n; ++j) {
            const float *row = s0 + (size_t)indices[o + j] * sstride;
            for (int k = 0; k < nout; ++k) {
                const double wk = (double)weights[k][o + j];
                for (int e = 0; e < len; ++e) acc[k][e] += (double)row[e] * wk;
            }
        }
        for (int k = 0; k < nout; ++k) {
            if (!dst[k]) continue;
            double *d = dst[k] + dstDesc[3 * k] + (size_t)i * dstDesc[3 * k + 2];
            memcpy(d, acc[k], sizeof(double) * len);
        }
    }
    return 1;
}

/* ---- EvalPatches (osd/cpuEvaluator.cpp:157-381) -------------------------------------- */

typedef struct { int arrayIndex, patchIndex, vertIndex; float s, t; } orc_coord;
typedef struct { int field0, field1; float sharpness; } orc_param;

/* Type of the patch a coord lands in: regular or irregular descriptor of its array
 * (cpuEvaluator.cpp:191-193). */
static int coord_patch_type(const int *arrays, const orc_param *pp, const orc_coord *c) {
    const int *a = arrays + 6 * c->arrayIndex;
    return orc_pp_regular(pp[c->patchIndex].field1) ? a[0] : a[1];
}

/* cvs = index[indexBase + stride * (patchIndex - primitiveIdBase)] (cpuEvaluator.cpp:198-201) */
static const int *coord_cvs(const int *arrays, const int *idx, const orc_coord *c) {
    const int *a = arrays + 6 * c->arrayIndex;
    return idx + a[3] + a[4] * (c->patchIndex - a[5]);
}

int orc_eval_patches_f(const float *src, const int *srcDesc, int nout, float *const *dst,
                       const int *dstDesc, int ncoords, const void *coords, const int *arrays,
                       const int *patchIndices, const void *params, int nthreads) {
    if (!src) return 0;
    for (int k = 0; k < nout; ++k)
        if (dst[k] && dstDesc[3 * k + 1] != srcDesc[1]) return 0;
    const int len = srcDesc[1], sstride = srcDesc[2];
    if (len > MAX_LEN) return 0;
    const float *s0 = src + srcDesc[0];
    const orc_coord *pc = (const orc_coord *)coords;
    const orc_param *pp = (const orc_param *)params;
#pragma omp parallel for schedule(static, 1024) num_threads(nthreads > 0 ? nthreads : 1)
    for (int i = 0; i < ncoords; ++i) {
        float w[6 * 20];
        float acc[MAX_LEN];
        const orc_coord *c = pc + i;
        const orc_param *p = pp + c->patchIndex;
        int type = coord_patch_type(arrays, pp, c);
        int n = orc_patch_basis_f(type, p->field0, p->field1, c->s, c->t, w);
        const int *cvs = coord_cvs(arrays, patchIndices, c);
        for (int k = 0; k < nout; ++k) {
            if (!dst[k]) continue;
            for (int e = 0; e < len; ++e) acc[e] = 0.0f;
            for (int j = 0; j < n; ++j) {
                const float *row = s0 + (size_t)cvs[j] * sstride;
                const float wk = w[20 * k + j];
                for (int e = 0; e < len; ++e) acc[e] += row[e] * wk;
            }
            float *d = dst[k] + dstDesc[3 * k] + (size_t)i * dstDesc[3 * k + 2];
            memcpy(d, acc, sizeof(float) * len);
        }
    }
    return 1;
}

int orc_eval_patches_d(const float *src, const int *srcDesc, int nout, double *const *dst,
                       const int *dstDesc, int ncoords, const void *coords, const int *arrays,
                       const int *patchIndices, const void *params, int nthreads) {
    if (!src) return 0;
    for (int k = 0; k < nout; ++k)
        if (dst[k] && dstDesc[3 * k + 1] != srcDesc[1]) return 0;
    const int len = srcDesc[1], sstride = srcDesc[2];
    if (len > MAX_LEN) return 0;
    const float *s0 = src + srcDesc[0];
    const orc_coord *pc = (const orc_coord *)coords;
    const orc_param *pp = (const orc_param *)params;
#pragma omp parallel for schedule(static, 1024) num_threads(nthreads > 0 ? nthreads : 1)
    for (int i = 0; i < ncoords; ++i) {
        double w[6 * 20];
        double acc[MAX_LEN];
        const orc_coord *c = pc + i;
        const orc_param *p = pp + c->patchIndex;
        int type = coord_patch_type(arrays, pp, c);
        int n = orc_patch_basis_d(type, p->field0, p->field1, (double)c->s, (double)c->t, w);
        const int *cvs = coord_cvs(arrays, patchIndices, c);
        for (int k = 0; k < nout; ++k) {
            if (!dst[k]) continue;
            for (int e = 0; e < len; ++e) acc[e] = 0.0;
            for (int j = 0; j < n; ++j) {
                const float *row = s0 + (size_t)cvs[j] * sstride;
                for (int e = 0; e < len; ++e) acc[e] += (double)row[e] * w[20 * k + j];
            }
            double *d = dst[k] + dstDesc[3 * k] + (size_t)i * dstDesc[3 * k + 2];
            memcpy(d, acc, sizeof(double) * len);
        }
    }
    return 1;
}

/* Magnitude of the summands, sum_j |w_j| |x_j|, per output: the natural scale of the float
 * rounding error of a (possibly cancelling) weighted sum.  Used by tests to state tolerances
 * for derivative outputs. */
int orc_eval_patches_abs(const float *src, const int *srcDesc, int nout, double *const *dst,
                         const int *dstDesc, int ncoords, const void *coords, const int *arrays,
                         const int *patchIndices, const void *params, int nthreads) {
    if (!src) return 0;
    const int len = srcDesc[1], sstride = srcDesc[2];
    if (len > MAX_LEN) return 0;
    const float *s0 = src + srcDesc[0];
    const orc_coord *pc = (const orc_coord *)coords;
    const orc_param *pp = (const orc_param *)params;
#pragma omp parallel for schedule(static, 1024) num_threads(nthreads > 0 ? nthreads : 1)
    for (int i = 0; i < ncoords; ++i) {
        double w[6 * 20];
        double acc[MAX_LEN];
        const orc_coord *c = pc + i;
        const orc_param *p = pp + c->patchIndex;
        int type = coord_patch_type(arrays, pp, c);
        int n = orc_patch_basis_d(type, p->field0, p->field1, (double)c->s, (double)c->t, w);
        const int *cvs = coord_cvs(arrays, patchIndices, c);
        for (int k = 0; k < nout; ++k) {
            if (!dst[k]) continue;
            for (int e = 0; e < len; ++e) acc[e] = 0.0;
            for (int j = 0; j < n; ++j) {
                const float *row = s0 + (size_t)cvs[j] * sstride;
                for (int e = 0; e < len; ++e) acc[e] += fabs((double)row[e] * w[20 * k + j]);
            }
            double *d = dst[k] + dstDesc[3 * k] + (size_t)i * dstDesc[3 * k + 2];
            memcpy(d, acc, sizeof(double) * len);
        }
    }
    return 1;
}

/* ---- PatchMap (far/patchMap.h:49-231, far/patchMap.cpp:89-202) ------------------------ */

/* A quadtree child: set / leaf flags and an index into the node or handle list. */
typedef struct { uint8_t set, leaf; int32_t index; } orc_child;
typedef struct { orc_child c[4]; } orc_node;

typedef struct {
    int triangular, minFace, maxFace, maxDepth;
    int numHandles;
    int *handles;      /* 3 ints per patch */
    orc_node *nodes;
    int numNodes, capNodes;
} orc_map;

static int map_new_node(orc_map *m) {
    if (m->numNodes == m->capNodes) {
        m->capNodes = m->capNodes ? 2 * m->capNodes : 1024;
        m->nodes = (orc_node *)realloc(m->nodes, sizeof(orc_node) * (size_t)m->capNodes);
    }
    memset(&m->nodes[m->numNodes], 0, sizeof(orc_node));
    return m->numNodes++;
}

/* Quadrant of (u,v) within a node of half-width `median` for triangular layouts, updating
 * (u,v) and the rotation flag (far/patchMap.h:159-189). */
static int tri_quadrant(double median, double *u, double *v, int *rot) {
    if (!*rot) {
        if (*u >= median) { *u -= median; return 1; }
        if (*v >= median) { *v -= median; return 2; }
        if ((*u + *v) >= median) { *rot = 1; return 3; }
        return 0;
    }
    if (*u < median) { *v -= median; return 1; }
    if (*v < median) { *u -= median; return 2; }
    *u -= median;
    *v -= median;
    if ((*u + *v) < median) { *rot = 0; return 3; }
    return 0;
}

/* Quadrant for quad layouts (far/patchMap.h:145-156). */
static int quad_quadrant(double median, double *u, double *v) {
    int uh = (*u >= median);
    if (uh) *u -= median;
    int vh = (*v >= median);
    if (vh) *v -= median;
    return (vh << 1) | uh;
}

/* Descend into (or create) the child of `node` in `quadrant`; with leaf set, record the
 * patch instead (far/patchMap.cpp:66-83). */
static int map_descend(orc_map *m, int node, int leaf, int quadrant, int handle) {
    orc_child *ch = &m->nodes[node].c[quadrant];
    if (leaf) {
        ch->set = 1; ch->leaf = 1; ch->index = handle;
        return node;
    }
    if (ch->set) return ch->index;
    int nn = map_new_node(m);
    ch = &m->nodes[node].c[quadrant];
    ch->set = 1; ch->leaf = 0; ch->index = nn;
    return nn;
}

void *orc_patchmap_build(int numArrays, const int *arrays, const void *params, int triangular) {
    const orc_param *pp = (const orc_param *)params;
    orc_map *m = (orc_map *)calloc(1, sizeof(orc_map));
    m->triangular = triangular;
    int total = 0;
    for (int a = 0; a < numArrays; ++a) total += arrays[6 * a + 2];
    m->numHandles = total;
    m->minFace = m->maxFace = -1;
    if (total <= 0) return m;
    m->handles = (int *)malloc(sizeof(int) * 3 * (size_t)total);
    m->minFace = m->maxFace = pp[0].field0 & 0xfffffff;
    /* handles (far/patchMap.cpp:100-132): array, global patch index, j * patch size.  The
     * patch size is the array's descriptor size, which is its stride in the flattened
     * Osd layout. */
    int h = 0;
    for (int a = 0; a < numArrays; ++a) {
        int np = arrays[6 * a + 2], stride = arrays[6 * a + 4];
        for (int j = 0; j < np; ++j, ++h) {
            m->handles[3 * h + 0] = a;
            m->handles[3 * h + 1] = h;
            m->handles[3 * h + 2] = j * stride;
            int f = pp[h].field0 & 0xfffffff;
            if (f < m->minFace) m->minFace = f;
            if (f > m->maxFace) m->maxFace = f;
        }
    }
    int nroots = m->maxFace - m->minFace + 1;
    for (int i = 0; i < nroots; ++i) map_new_node(m);
    /* quadtree (far/patchMap.cpp:134-194) */
    for (h = 0; h < total; ++h) {
        int f1 = pp[h].field1;
        int depth = orc_pp_depth(f1), root = orc_pp_nonquad(f1);
        if (depth > m->maxDepth) m->maxDepth = depth;
        int node = (pp[h].field0 & 0xfffffff) - m->minFace;
        if (depth == root) {
            for (int q = 0; q < 4; ++q) {
                m->nodes[node].c[q].set = 1;
                m->nodes[node].c[q].leaf = 1;
                m->nodes[node].c[q].index = h;
            }
            continue;
        }
        if (!triangular) {
            int u = orc_pp_u(f1), v = orc_pp_v(f1);
            for (int j = root + 1; j <= depth; ++j) {
                int q = (((v >> (depth - j)) & 1) << 1) | ((u >> (depth - j)) & 1);
                node = map_descend(m, node, j == depth, q, h);
            }
        } else {
            /* interior point (0.25, 0.25) of the patch, unnormalised (patchParam.h:311-323) */
            double u = 0.25, v = 0.25;
            float frac = 1.0f / (float)(1 << (depth - root));
            if ((orc_pp_u(f1) + orc_pp_v(f1)) >= (1 << depth)) {
                int df = 1 << depth;
                u = ((double)(df - orc_pp_u(f1)) - u) * frac;
                v = ((double)(df - orc_pp_v(f1)) - v) * frac;
            } else {
                u = (u + (double)orc_pp_u(f1)) * (double)frac;
                v = (v + (double)orc_pp_v(f1)) * (double)frac;
            }
            double median = 0.5;
            int rot = 0;
            for (int j = root + 1; j <= depth; ++j, median *= 0.5) {
                int q = tri_quadrant(median, &u, &v, &rot);
                node = map_descend(m, node, j == depth, q, h);
            }
        }
    }
    return m;
}

void orc_patchmap_free(void *p) {
    orc_map *m = (orc_map *)p;
    if (!m) return;
    free(m->handles);
    free(m->nodes);
    free(m);
}

int orc_find_patches(const void *p, int n, const int *faces, const double *uu,
                     const double *vv, int *out) {
    const orc_map *m = (const orc_map *)p;
    int found = 0;
    for (int i = 0; i < n; ++i) {
        int *o = out + 3 * i;
        o[0] = o[1] = o[2] = -1;
        int f = faces[i];
        if (m->numHandles == 0 || f < m->minFace || f > m->maxFace) continue;
        int node = f - m->minFace;
        if (!m->nodes[node].c[0].set) continue;
        double u = uu[i], v = vv[i], median = 0.5;
        int rot = 0;
        for (int depth = 0; depth <= m->maxDepth; ++depth, median *= 0.5) {
            int q = m->triangular ? tri_quadrant(median, &u, &v, &rot)
                                  : quad_quadrant(median, &u, &v);
            const orc_child *ch = &m->nodes[node].c[q];
            if (!ch->set) break;
            if (ch->leaf) {
                memcpy(o, m->handles + 3 * ch->index, sizeof(int) * 3);
                ++found;
                break;
            }
            node = ch->index;
        }
    }
    return found;
}

/* ---- stencil-table factory ----------------------------------------------------------------
 * A restatement of Far's StencilBuilder (far/stencilBuilder.cpp): a row is built by merging
 * (index, weight) terms; a term whose index is already in the row is added to that entry
 * (WeightTable::merge, :310-346), otherwise appended (WeightTable::add, :348-385).  A mask
 * entry (source s, weight m) contributes m itself for a control vertex and w * m for every
 * entry (i, w) of s's factorized row otherwise (WeightTable::AddWithWeight, :164-198). */

typedef struct {
    int *idx;
    float *w[6];
    long long n, cap;
    int nc;
} orc_arena;

static int arena_grow(orc_arena *a, long long need) {
    if (need <= a->cap) return 1;
    long long cap = a->cap ? a->cap : 1024;
    while (cap < need) cap *= 2;
    int *ni = (int *)realloc(a->idx, (size_t)cap * sizeof(int));
    if (!ni) return 0;
    a->idx = ni;
    for (int c = 0; c < a->nc; ++c) {
        float *nw = (float *)realloc(a->w[c], (size_t)cap * sizeof(float));
        if (!nw) return 0;
        a->w[c] = nw;
    }
    a->cap = cap;
    return 1;
}

static void arena_free(orc_arena *a) {
    free(a->idx);
    for (int c = 0; c < 6; ++c) free(a->w[c]);
}

/* merges term (q, x[0..nc)) into the row that starts at `start` (the arena's last row) */
static int row_merge(orc_arena *a, long long start, int q, const float *x) {
    for (long long i = start; i < a->n; ++i)
        if (a->idx[i] == q) {
            for (int c = 0; c < a->nc; ++c) a->w[c][i] += x[c];
            return 1;
        }
    if (!arena_grow(a, a->n + 1)) return 0;
    a->idx[a->n] = q;
    for (int c = 0; c < a->nc; ++c) a->w[c][a->n] = x[c];
    ++a->n;
    return 1;
}

void orc_table_free(orc_table *t) {
    if (!t) return;
    free(t->sizes);
    free(t->offsets);
    free(t->indices);
    for (int c = 0; c < 6; ++c) free(t->w[c]);
    free(t);
}

static orc_table *table_alloc(int n, long long nnz, int nc) {
    orc_table *t = (orc_table *)calloc(1, sizeof(orc_table));
    if (!t) return NULL;
    t->numStencils = n;
    t->numChannels = nc;
    t->nnz = nnz;
    t->sizes = (int *)malloc((size_t)(n ? n : 1) * sizeof(int));
    t->offsets = (int *)malloc((size_t)(n ? n : 1) * sizeof(int));
    t->indices = (int *)malloc((size_t)(nnz ? nnz : 1) * sizeof(int));
    int good = t->sizes && t->offsets && t->indices;
    for (int c = 0; c < nc; ++c) {
        t->w[c] = (float *)malloc((size_t)(nnz ? nnz : 1) * sizeof(float));
        good = good && t->w[c];
    }
    if (!good) {
        orc_table_free(t);
        return NULL;
    }
    return t;
}

orc_table *orc_factory_create(int numControl, int numLevels, const int *numRows,
                              const long long *const *offsets, const int *const *sources,
                              const float *const *weights, int generateIntermediateLevels,
                              int generateControlVerts) {
    if (numControl < 0 || numLevels < 0) return NULL;
    long long total = 0;
    for (int l = 0; l < numLevels; ++l) total += numRows[l];
    long long *rowOff = (long long *)malloc((size_t)(total ? total : 1) * sizeof(long long));
    int *rowSize = (int *)malloc((size_t)(total ? total : 1) * sizeof(int));
    char *done = (char *)calloc((size_t)(total ? total : 1), 1);
    orc_arena a;
    memset(&a, 0, sizeof(a));
    a.nc = 1;
    orc_table *t = NULL;
    int good = rowOff && rowSize && done;
    long long first = numControl; /* global index of the current level's row 0 */
    for (int l = 0; l < numLevels && good; ++l) {
        const long long prevFirst = l ? first - numRows[l - 1] : 0;
        const long long *mo = offsets[l];
        const int *ms = sources[l];
        const float *mw = weights[l];
        long long left = numRows[l];
        while (left > 0 && good) {
            long long progress = 0;
            for (int r = 0; r < numRows[l] && good; ++r) {
                const long long g = first + r - numControl;
                if (done[g]) continue;
                int ready = 1;
                for (long long k = mo[r]; k < mo[r + 1]; ++k) {
                    const long long s = ms[k];
                    if (s < 0 || s >= first + numRows[l] ||
                        (s >= numControl && s < (l ? prevFirst : numControl))) {
                        good = 0; /* a source outside the previous level and this one */
                        break;
                    }
                    if (s >= first && !done[s - numControl]) ready = 0;
                }
                if (!good || !ready) continue;
                const long long start = a.n;
                for (long long k = mo[r]; k < mo[r + 1] && good; ++k) {
                    const int s = ms[k];
                    const float m = mw[k];
                    if (m == 0.0f) continue;
                    if (s < numControl) {
                        const float x = m * 1.0f;
                        good = row_merge(&a, start, s, &x);
                        continue;
                    }
                    const long long o = rowOff[s - numControl];
                    const int n = rowSize[s - numControl];
                    for (int j = 0; j < n && good; ++j) {
                        const float x = a.w[0][o + j] * m;
                        good = row_merge(&a, start, a.idx[o + j], &x);
                    }
                }
                rowOff[g] = start;
                rowSize[g] = (int)(a.n - start);
                done[g] = 1;
                ++progress;
                --left;
            }
            if (!progress) good = 0; /* rows that wait on each other */
        }
        first += numRows[l];
    }
    if (good) {
        const int firstLevel = generateIntermediateLevels ? 0 : (numLevels ? numLevels - 1 : 0);
        long long firstRow = 0;
        for (int l = 0; l < firstLevel; ++l) firstRow += numRows[l];
        const int nc = generateControlVerts ? numControl : 0;
        const long long nr = numLevels ? total - firstRow : 0;
        long long nnz = nc;
        for (long long g = firstRow; g < firstRow + nr; ++g) nnz += rowSize[g];
        t = table_alloc((int)(nc + nr), nnz, 1);
        if (t) {
            long long e = 0;
            int i = 0;
            for (int v = 0; v < nc; ++v, ++i) {
                t->sizes[i] = 1;
                t->offsets[i] = (int)e;
                t->indices[e] = v;
                t->w[0][e++] = 1.0f;
            }
            for (long long g = firstRow; g < firstRow + nr; ++g, ++i) {
                t->sizes[i] = rowSize[g];
                t->offsets[i] = (int)e;
                memcpy(t->indices + e, a.idx + rowOff[g], (size_t)rowSize[g] * sizeof(int));
                memcpy(t->w[0] + e, a.w[0] + rowOff[g], (size_t)rowSize[g] * sizeof(float));
                e += rowSize[g];
            }
        }
    }
    free(rowOff);
    free(rowSize);
    free(done);
    arena_free(&a);
    return t;
}

orc_table *orc_compose_rows(int baseNumStencils, const int *baseSizes, const int *baseOffsets,
                            const int *baseIndices, const float *baseWeights, int numRows,
                            const long long *offsets, const int *sources, int numChannels,
                            const float *const *weights, int appendBase) {
    if (numChannels != 1 && numChannels != 3 && numChannels != 6) return NULL;
    orc_arena a;
    memset(&a, 0, sizeof(a));
    a.nc = numChannels;
    long long *rowOff = (long long *)malloc((size_t)(numRows ? numRows : 1) * sizeof(long long));
    int good = rowOff != NULL;
    for (int r = 0; r < numRows && good; ++r) {
        const long long start = a.n;
        for (long long k = offsets[r]; k < offsets[r + 1] && good; ++k) {
            const int s = sources[k];
            if (s < 0 || s >= baseNumStencils) {
                good = 0;
                break;
            }
            float m[6];
            int any = 0;
            for (int c = 0; c < numChannels; ++c) {
                m[c] = weights[c][k];
                any |= m[c] != 0.0f;
            }
            if (!any) continue;
            for (int j = 0; j < baseSizes[s] && good; ++j) {
                const float w = baseWeights[baseOffsets[s] + j];
                if (w == 0.0f) continue;
                float x[6];
                for (int c = 0; c < numChannels; ++c) x[c] = m[c] * w;
                good = row_merge(&a, start, baseIndices[baseOffsets[s] + j], x);
            }
        }
        rowOff[r] = start;
    }
    orc_table *t = NULL;
    if (good) {
        long long baseNnz = 0;
        const int nb = appendBase ? baseNumStencils : 0;
        for (int i = 0; i < nb; ++i) baseNnz += baseSizes[i];
        t = table_alloc(nb + numRows, baseNnz + a.n, numChannels);
        if (t) {
            long long e = 0;
            int i = 0;
            for (int b = 0; b < nb; ++b, ++i) {
                t->sizes[i] = baseSizes[b];
                t->offsets[i] = (int)e;
                for (int j = 0; j < baseSizes[b]; ++j, ++e) {
                    t->indices[e] = baseIndices[baseOffsets[b] + j];
                    t->w[0][e] = baseWeights[baseOffsets[b] + j];
                    for (int c = 1; c < numChannels; ++c) t->w[c][e] = 0.0f;
                }
            }
            for (int r = 0; r < numRows; ++r, ++i) {
                const long long end = r + 1 < numRows ? rowOff[r + 1] : a.n;
                t->sizes[i] = (int)(end - rowOff[r]);
                t->offsets[i] = (int)e;
                for (long long j = rowOff[r]; j < end; ++j, ++e) {
                    t->indices[e] = a.idx[j];
                    for (int c = 0; c < numChannels; ++c) t->w[c][e] = a.w[c][j];
                }
            }
        }
    }
    free(rowOff);
    arena_free(&a);
    return t;
}
