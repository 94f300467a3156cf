/*
 * adeco_oracle.c -- CPU oracle for the phase-space tetrahedron mass deposit.
 *
 * TEST INFRASTRUCTURE ONLY.  Used by tests/ (as the checker), by
 * __graft_entry__.smoke() (as the checker) and by bench.py's cpu_baseline /
 * --impl reference legs (as the timed CPU baseline).  Nothing in the
 * adeco_gb300 product path links or loads it.
 *
 * It restates ADECO's CPU algorithm for the deposit hot path:
 *   - tet construction: sample_cell_vertices + tet_conn + the CPU orientation
 *     rule (swap v0<->v3 when the signed volume is negative)
 *       src/AdDepositTets2Grid.h:207-231, 554-567, 917-1053
 *   - candidate cell range, classification, exact clipping volume, scatter
 *       src/AdDepositTets2Grid.h:509-665, 286-363; src/AdTetIntersection.h:66-514
 *   - the DepositWrapper::deposit_tets CPU boundary  src/AdDeposit2Grid.cpp:67-125
 *   - MetaMesh meta-cells and the octree refinement estimate
 *       src/AdTypeDefinitions.h:715-1022 (estimate at :812-825)
 *   - generate_tree / distribute_tets_to_children / refineNode / getLeafNodes
 *       src/AdOctreeGeneration.h:76-258, src/AdOctree.h:187-305
 * with the floating-point operation order kept, so that the FP32 build (with
 * -ffp-contract=off) reproduces the reference bit-for-bit; the FP64
 * instantiation is the FP64 oracle every GPU error is stated against.
 *
 * The lookup tables below (split table, per-case sub-tet counts, tet edges,
 * the 6-tet cube table and the corner sampling order) are the reference's
 * data: they define which sub-tets and tets exist, so they must be the same.
 */
#include "adeco_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

static _Thread_local uint64_t ora_flop_counter;
#define FLOPS(n) (ora_flop_counter += (uint64_t)(n))

void ora_flops_reset(void) { ora_flop_counter = 0; }
uint64_t ora_flops_get(void) { return ora_flop_counter; }

/* Sub-tets of the part of a tet on the positive side of a plane, indexed by
 * the 4-bit vertex-side mask (bit p = vertex p on the positive side).  Entries
 * 0..3 are the tet's vertices, 4..9 the cut points on edges 0..5.
 * (src/AdTetIntersection.h:66-93)                                          */
static const unsigned char ora_split_table[16][3][4] = {
    {{255, 255, 255, 255}, {255, 255, 255, 255}, {255, 255, 255, 255}},
    {{0, 5, 6, 4}, {255, 255, 255, 255}, {255, 255, 255, 255}},
    {{7, 1, 8, 4}, {255, 255, 255, 255}, {255, 255, 255, 255}},
    {{0, 6, 8, 7}, {6, 0, 5, 7}, {1, 0, 8, 7}},
    {{2, 7, 9, 5}, {255, 255, 255, 255}, {255, 255, 255, 255}},
    {{6, 0, 9, 7}, {0, 6, 4, 7}, {0, 2, 9, 7}},
    {{5, 1, 9, 8}, {9, 1, 5, 2}, {1, 5, 4, 8}},
    {{6, 0, 9, 8}, {0, 2, 9, 8}, {0, 1, 2, 8}},
    {{8, 3, 9, 6}, {255, 255, 255, 255}, {255, 255, 255, 255}},
    {{0, 5, 9, 8}, {5, 0, 4, 8}, {3, 0, 9, 8}},
    {{1, 6, 9, 7}, {1, 9, 6, 3}, {6, 1, 4, 7}},
    {{0, 5, 9, 7}, {3, 0, 9, 7}, {1, 0, 3, 7}},
    {{6, 2, 8, 7}, {6, 8, 2, 3}, {2, 6, 5, 7}},
    {{4, 0, 8, 7}, {0, 3, 8, 7}, {0, 2, 3, 7}},
    {{1, 4, 6, 5}, {3, 1, 6, 5}, {2, 1, 3, 5}},
    {{0, 2, 3, 1}, {255, 255, 255, 255}, {255, 255, 255, 255}},
};
static const int ora_split_count[16] = {0, 1, 1, 3, 1, 3, 3, 3, 1, 3, 3, 3, 3, 3, 3, 1};
static const int ora_tet_edges[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
/* 6 tets of a lattice cube, as slots of the 8 sampled corners
 * (src/AdDepositTets2Grid.h:207-219)                                       */
static const int ora_tet_conn[6][4] = {{1, 0, 2, 4}, {4, 2, 1, 3}, {3, 5, 1, 4},
                                       {4, 5, 6, 3}, {3, 2, 6, 4}, {3, 7, 5, 6}};
/* corner offsets of the 8 slots in sample_cell_vertices order
 * (src/AdDepositTets2Grid.h:947-973)                                       */
static const int ora_ref_corner[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {1, 1, 0},
                                         {0, 1, 1}, {1, 1, 1}, {0, 0, 1}, {1, 0, 1}};

#define REAL float
#define SFX(name) name##_f
#include "oracle_core.inc"
#undef REAL
#undef SFX

#define REAL double
#define SFX(name) name##_d
#include "oracle_core.inc"
#undef REAL
#undef SFX

/* ------------------------------------------------------------------------- */
/* multi-threaded driver (worker pool with private grids, then a sum)        */

typedef struct {
    const float *positions;
    int m, dims, order, is_double;
    const float *bbox;
    double mass;
    size_t cube_begin, cube_end, chunk;
    size_t *next;                 /* shared cursor */
    pthread_mutex_t *lock;
    void *grid;                   /* private grid */
} ora_job;

static void *ora_worker(void *arg)
{
    ora_job *j = (ora_job *)arg;
    for (;;) {
        pthread_mutex_lock(j->lock);
        const size_t b = *j->next;
        *j->next = (b + j->chunk < j->cube_end) ? b + j->chunk : j->cube_end;
        pthread_mutex_unlock(j->lock);
        if (b >= j->cube_end) break;
        const size_t e = (b + j->chunk < j->cube_end) ? b + j->chunk : j->cube_end;
        if (j->is_double)
            ora_deposit_cubes_d(b, e, j->positions, j->m, j->bbox, j->dims, j->order, j->mass,
                                (double *)j->grid, NULL, NULL);
        else
            ora_deposit_cubes_f(b, e, j->positions, j->m, j->bbox, j->dims, j->order, (float)j->mass,
                                (float *)j->grid, NULL, NULL);
    }
    return NULL;
}

static int ora_mt(size_t patch_offset, size_t num_patches, const float *positions, size_t positions_size,
                  int m, const float bbox[6], int dims, int order, double mass, void *grid, int threads,
                  int is_double)
{
    if (positions_size == 0) return 0;
    const size_t fpp = 3 * (size_t)(m + 1) * (m + 1) * (m + 1);
    const size_t cpp = (size_t)m * m * m;
    if (cpp * num_patches >= 2147483647u) return -1;
    if (positions_size % fpp != 0) return -2;
    if (patch_offset + num_patches > positions_size / fpp) return -3;
    if (threads < 1) threads = 1;
    const size_t ncell = (size_t)dims * dims * dims;
    const size_t esz = is_double ? sizeof(double) : sizeof(float);
    pthread_t *tid = (pthread_t *)calloc((size_t)threads, sizeof(pthread_t));
    ora_job *jobs = (ora_job *)calloc((size_t)threads, sizeof(ora_job));
    pthread_mutex_t lock;
    pthread_mutex_init(&lock, NULL);
    size_t next = patch_offset * cpp;
    const size_t end = (patch_offset + num_patches) * cpp;
    size_t chunk = (end - next) / (10 * (size_t)threads);
    if (chunk < 64) chunk = 64;
    for (int t = 0; t < threads; ++t) {
        jobs[t].positions = positions; jobs[t].m = m; jobs[t].dims = dims; jobs[t].order = order;
        jobs[t].is_double = is_double; jobs[t].bbox = bbox; jobs[t].mass = mass;
        jobs[t].cube_begin = next; jobs[t].cube_end = end; jobs[t].chunk = chunk;
        jobs[t].next = &next; jobs[t].lock = &lock;
        jobs[t].grid = calloc(ncell, esz);
        pthread_create(&tid[t], NULL, ora_worker, &jobs[t]);
    }
    for (int t = 0; t < threads; ++t) {
        pthread_join(tid[t], NULL);
        if (is_double) {
            double *g = (double *)grid, *p = (double *)jobs[t].grid;
            for (size_t c = 0; c < ncell; ++c) g[c] += p[c];
        } else {
            float *g = (float *)grid, *p = (float *)jobs[t].grid;
            for (size_t c = 0; c < ncell; ++c) g[c] += p[c];
        }
        free(jobs[t].grid);
    }
    pthread_mutex_destroy(&lock);
    free(jobs);
    free(tid);
    return 0;
}

int ora_deposit_patches_mt_f(size_t patch_offset, size_t num_patches, const float *positions,
                             size_t positions_size, int m, const float bbox[6], int dims, int order,
                             float mass, float *grid, int threads)
{
    return ora_mt(patch_offset, num_patches, positions, positions_size, m, bbox, dims, order, mass, grid,
                  threads, 0);
}

int ora_deposit_patches_mt_d(size_t patch_offset, size_t num_patches, const float *positions,
                             size_t positions_size, int m, const float bbox[6], int dims, int order,
                             double mass, double *grid, int threads)
{
    return ora_mt(patch_offset, num_patches, positions, positions_size, m, bbox, dims, order, mass, grid,
                  threads, 1);
}

/* ------------------------------------------------------------------------- */
/* MetaMesh + octree (src/AdTypeDefinitions.h:715-1022, src/AdOctreeGeneration.h,
 * src/AdOctree.h)                                                            */

#define ORA_MC 7

static int ora_ceil_div(int x, int y) { return x / y + (x % y > 0); }

static void ora_meta_dims(int nx, int ny, int nz, int cd[3])
{
    cd[0] = ora_ceil_div(nx - 1, ORA_MC);
    cd[1] = ora_ceil_div(ny - 1, ORA_MC);
    cd[2] = ora_ceil_div(nz - 1, ORA_MC);
}

size_t ora_meta_count(int nx, int ny, int nz)
{
    if (nx < 2 || ny < 2 || nz < 2) return 0;
    int cd[3];
    ora_meta_dims(nx, ny, nz, cd);
    return (size_t)cd[0] * cd[1] * cd[2];
}

/* vertex index range of meta-cell (cx,cy,cz): min corner and vertex counts */
static void ora_meta_range(int nx, int ny, int nz, const int cd[3], int cx, int cy, int cz, int mn[3], int d[3])
{
    const int pd[3] = {nx, ny, nz};
    const int c[3] = {cx, cy, cz};
    for (int a = 0; a < 3; ++a) {
        mn[a] = c[a] * ORA_MC;
        d[a] = (c[a] + 1 == cd[a]) ? (pd[a] - mn[a]) : ORA_MC + 1;
    }
}

static void ora_meta_range_id(int nx, int ny, int nz, uint64_t mc, int mn[3], int d[3])
{
    int cd[3];
    ora_meta_dims(nx, ny, nz, cd);
    const uint64_t nb = (uint64_t)cd[0], nb2 = (uint64_t)cd[0] * (uint64_t)cd[1];
    const int cz = (int)(mc / nb2), rem = (int)(mc % nb2), cy = (int)(rem / nb), cx = (int)(rem % nb);
    ora_meta_range(nx, ny, nz, cd, cx, cy, cz, mn, d);
}

void ora_meta_bboxes(const float *pos, int nx, int ny, int nz, float *bbox6)
{
    int cd[3];
    ora_meta_dims(nx, ny, nz, cd);
    size_t mc = 0;
    for (int cz = 0; cz < cd[2]; ++cz)
        for (int cy = 0; cy < cd[1]; ++cy)
            for (int cx = 0; cx < cd[0]; ++cx, ++mc) {
                int mn[3], d[3];
                ora_meta_range(nx, ny, nz, cd, cx, cy, cz, mn, d);
                float *b = bbox6 + 6 * mc;
                const size_t id0 = (size_t)mn[0] + (size_t)nx * ((size_t)mn[1] + (size_t)ny * (size_t)mn[2]);
                for (int a = 0; a < 3; ++a) { b[a] = pos[3 * id0 + a]; b[3 + a] = pos[3 * id0 + a]; }
                for (int k = 0; k < d[2]; ++k)
                    for (int j = 0; j < d[1]; ++j)
                        for (int i = 0; i < d[0]; ++i) {
                            const size_t id = (size_t)(mn[0] + i) +
                                              (size_t)nx * ((size_t)(mn[1] + j) + (size_t)ny * (size_t)(mn[2] + k));
                            for (int a = 0; a < 3; ++a) {
                                const float p = pos[3 * id + a];
                                if (p < b[a]) b[a] = p;          /* std::min(min, p) */
                                if (b[3 + a] < p) b[3 + a] = p;  /* std::max(max, p) */
                            }
                        }
            }
}

static int ora_aabb_meet(const float *a6, const float *b6)
{
    return a6[0] < b6[3] && b6[0] < a6[3] && a6[1] < b6[4] && b6[1] < a6[4] && a6[2] < b6[5] && b6[2] < a6[5];
}

static float ora_aabb_volume(const float *b6)
{
    return (b6[3] - b6[0]) * (b6[4] - b6[1]) * (b6[5] - b6[2]);
}

uint64_t ora_meta_estimate(int nx, int ny, int nz, const float *mc_bbox6, uint64_t mc, const float box6[6])
{
    int mn[3], d[3];
    ora_meta_range_id(nx, ny, nz, mc, mn, d);
    const size_t cells = (size_t)(d[0] - 1) * (size_t)(d[1] - 1) * (size_t)(d[2] - 1);
    const float *m6 = mc_bbox6 + 6 * mc;
    float ib[6];
    /* the callers only pass strictly-overlapping boxes (see header notes) */
    for (int a = 0; a < 3; ++a) {
        ib[a] = (box6[a] < m6[a]) ? m6[a] : box6[a];
        ib[3 + a] = (box6[3 + a] < m6[3 + a]) ? box6[3 + a] : m6[3 + a];
    }
    const float num = (float)(6 * cells) * ora_aabb_volume(ib);
    const float est = num / ora_aabb_volume(m6);
    return (uint64_t)est;
}

static void ora_node_box(const ora_node *n, float b6[6])
{
    for (int a = 0; a < 3; ++a) { b6[a] = n->min[a]; b6[3 + a] = n->min[a] + n->ext; }
}

int ora_generate_tree(const float *pos, int nx, int ny, int nz, const float box6[6], const float roi6[6],
                      uint64_t max_tets_per_node, int max_level, ora_node *nodes, int max_nodes,
                      int64_t *meta_off, uint64_t *meta_ids, int64_t max_ids)
{
    const size_t nmc = ora_meta_count(nx, ny, nz);
    float *mcb = (float *)malloc(6 * (nmc ? nmc : 1) * sizeof(float));
    ora_meta_bboxes(pos, nx, ny, nz, mcb);

    float roi[6];
    if (roi6[0] > roi6[3] || roi6[1] > roi6[4] || roi6[2] > roi6[5]) memcpy(roi, box6, sizeof roi);
    else memcpy(roi, roi6, sizeof roi);

    /* per-node meta lists: simple growable arrays, compacted to CSR at the end */
    uint64_t **lists = (uint64_t **)calloc((size_t)max_nodes, sizeof(uint64_t *));
    size_t *lsz = (size_t *)calloc((size_t)max_nodes, sizeof(size_t));
    size_t *lcap = (size_t *)calloc((size_t)max_nodes, sizeof(size_t));

    int n_nodes = 1;
    const float e0 = box6[3] - box6[0], e1 = box6[4] - box6[1], e2 = box6[5] - box6[2];
    const float e01 = (e0 < e1) ? e1 : e0;
    nodes[0].min[0] = box6[0]; nodes[0].min[1] = box6[1]; nodes[0].min[2] = box6[2];
    nodes[0].ext = (e01 < e2) ? e2 : e01;
    nodes[0].level = 0; nodes[0].parent = -1; nodes[0].first_child = -1; nodes[0].pad = 0; nodes[0].estimate = 0;
    lists[0] = (uint64_t *)malloc((nmc ? nmc : 1) * sizeof(uint64_t));
    for (size_t i = 0; i < nmc; ++i) lists[0][i] = i;
    lsz[0] = lcap[0] = nmc;

    int *stack = (int *)malloc((size_t)max_nodes * sizeof(int));
    int top = 0;
    stack[top++] = 0;
    int overflow = 0;
    while (top > 0) {
        const int cur = stack[--top];
        float cb[6];
        ora_node_box(&nodes[cur], cb);
        uint64_t est = 0;
        for (size_t m = 0; m < lsz[cur]; ++m) est += ora_meta_estimate(nx, ny, nz, mcb, lists[cur][m], cb);
        nodes[cur].estimate = est;
        if (!ora_aabb_meet(roi, cb)) continue;
        if (!(est > 0 && est > max_tets_per_node && nodes[cur].level < max_level)) continue;
        if (n_nodes + 8 > max_nodes) { overflow = 1; break; }
        /* refineNode: 8 children appended, x fastest */
        const int first = n_nodes;
        nodes[cur].first_child = first;
        const float cext = (float)((double)nodes[cur].ext / 2.);
        int c = 0;
        for (int k = 0; k < 2; ++k)
            for (int j = 0; j < 2; ++j)
                for (int i = 0; i < 2; ++i, ++c) {
                    ora_node *ch = &nodes[first + c];
                    ch->min[0] = nodes[cur].min[0] + (float)i * cext;
                    ch->min[1] = nodes[cur].min[1] + (float)j * cext;
                    ch->min[2] = nodes[cur].min[2] + (float)k * cext;
                    ch->ext = cext;
                    ch->level = nodes[cur].level + 1;
                    ch->parent = cur;
                    ch->first_child = -1;
                    ch->pad = 0;
                    ch->estimate = 0;
                }
        n_nodes += 8;
        /* distribute_tets_to_children */
        float chb[8][6];
        for (int q = 0; q < 8; ++q) ora_node_box(&nodes[first + q], chb[q]);
        for (size_t m = 0; m < lsz[cur]; ++m) {
            const uint64_t id = lists[cur][m];
            for (int q = 0; q < 8; ++q) {
                if (!ora_aabb_meet(mcb + 6 * id, chb[q])) continue;
                const int ci = first + q;
                if (lsz[ci] == lcap[ci]) {
                    lcap[ci] = lcap[ci] ? 2 * lcap[ci] : 64;
                    lists[ci] = (uint64_t *)realloc(lists[ci], lcap[ci] * sizeof(uint64_t));
                }
                lists[ci][lsz[ci]++] = id;
            }
        }
        free(lists[cur]);
        lists[cur] = NULL;
        lsz[cur] = lcap[cur] = 0;
        for (int q = 0; q < 8; ++q) stack[top++] = first + q;
    }
    int64_t off = 0;
    for (int i = 0; i < n_nodes && !overflow; ++i) {
        meta_off[i] = off;
        if (off + (int64_t)lsz[i] > max_ids) { overflow = 1; break; }
        for (size_t m = 0; m < lsz[i]; ++m) meta_ids[off + (int64_t)m] = lists[i][m];
        off += (int64_t)lsz[i];
    }
    if (!overflow) meta_off[n_nodes] = off;
    for (int i = 0; i < max_nodes; ++i) free(lists[i]);
    free(lists); free(lsz); free(lcap); free(stack); free(mcb);
    return overflow ? -1 : n_nodes;
}

int ora_leaf_order(const ora_node *nodes, int n_nodes, int *leaf_ids)
{
    int *stack = (int *)malloc((size_t)(n_nodes + 8) * sizeof(int));
    int top = 0, nl = 0;
    stack[top++] = 0;
    while (top > 0) {
        const int cur = stack[--top];
        if (nodes[cur].first_child > 0) {
            for (int q = 0; q < 8; ++q) stack[top++] = nodes[cur].first_child + q;
        } else {
            leaf_ids[nl++] = cur;
        }
    }
    free(stack);
    return nl;
}

/* Leaf deposit over meta-cell blocks: the same cubes, tets and accumulation
 * order as gather_local_tets + deposit_tets on a single worker
 * (src/AdDynamicLoadBalancing.h:894-950, src/AdTypeDefinitions.h:762-810).  */
#define ORA_META_DEPOSIT(SUF, RT)                                                                    \
    void ora_deposit_meta_##SUF(const float *pos, int nx, int ny, int nz, const uint64_t *ids, size_t n, \
                                const float bbox[6], int dims, int order, RT mass, RT *grid, ora_stats *st) \
    {                                                                                                \
        float block[3 * 8 * 8 * 8];                                                                  \
        for (size_t q = 0; q < n; ++q) {                                                             \
            int mn[3], d[3];                                                                         \
            ora_meta_range_id(nx, ny, nz, ids[q], mn, d);                                            \
            for (int t = 0; t < 3 * 512; ++t) block[t] = 666.f;                                     \
            for (int k = 0; k < d[2]; ++k)                                                           \
                for (int j = 0; j < d[1]; ++j)                                                       \
                    for (int i = 0; i < d[0]; ++i) {                                                 \
                        const size_t src = (size_t)(mn[0] + i) +                                     \
                            (size_t)nx * ((size_t)(mn[1] + j) + (size_t)ny * (size_t)(mn[2] + k));   \
                        const size_t dst = (size_t)i + 8 * ((size_t)j + 8 * (size_t)k);              \
                        block[3 * dst + 0] = pos[3 * src + 0];                                       \
                        block[3 * dst + 1] = pos[3 * src + 1];                                       \
                        block[3 * dst + 2] = pos[3 * src + 2];                                       \
                    }                                                                                \
            ora_deposit_cubes_##SUF(0, 343, block, 7, bbox, dims, order, mass, grid, NULL, st);     \
        }                                                                                            \
    }
ORA_META_DEPOSIT(f, float)
ORA_META_DEPOSIT(d, double)
