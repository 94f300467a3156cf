/*
 * adeco_oracle.h -- CPU oracle for the phase-space tetrahedron mass deposit.
 *
 * TEST INFRASTRUCTURE ONLY.  This library restates, in plain C, ADECO's CPU
 * deposit (src/AdDeposit2Grid.cpp, src/AdDepositTets2Grid.h,
 * src/AdTetIntersection.h) and its octree construction
 * (src/AdOctreeGeneration.h, src/AdOctree.h, src/AdTypeDefinitions.h
 * MetaMesh).  It is the checker the GPU path is compared against and the
 * CPU baseline that bench.py times; the product path (adeco_gb300) never
 * links, loads or calls it.
 *
 * Parity pin: the FP32 instantiation is compared bit-for-bit with the
 * reference's own code compiled from its sources (oracle/build_ref.sh ->
 * oracle/_ref/), and the committed fixtures under tests/golden/ were made by
 * that reference build (tests/golden/make_golden.py).
 */
#ifndef ADECO_ORACLE_H
#define ADECO_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORA_NO_INTERSECTION = 0, ORA_TET_INSIDE_CELL = 1, ORA_CELL_INSIDE_TET = 2, ORA_PARTIAL = 3 };
enum { ORA_ORDER_REF = 0, ORA_ORDER_CONFORMING = 1 };

typedef struct {
    uint64_t cubes;             /* cubes processed (not padded)              */
    uint64_t padded_cubes;      /* cubes skipped for a 666 padding vertex    */
    uint64_t tets_in_grid;      /* tets whose AABB strictly meets the grid   */
    uint64_t zero_volume;       /* of those, skipped with zero volume        */
    uint64_t candidate_pairs;   /* (tet, cell) pairs in the candidate ranges */
    uint64_t bbox_pairs;        /* pairs passing the strict cell-AABB test   */
    uint64_t no_pairs;          /* classified NO_INTERSECTION                */
    uint64_t tet_inside_pairs;
    uint64_t cell_inside_pairs;
    uint64_t partial_pairs;     /* clipped                                   */
} ora_stats;

/* FLOP counter of the calling thread (instrumented restatement). */
void ora_flops_reset(void);
uint64_t ora_flops_get(void);

/* --- geometry primitives (f = FP32, d = FP64) --- */
float  ora_vol6_f(const float *a, const float *b, const float *c, const float *d);
double ora_vol6_d(const double *a, const double *b, const double *c, const double *d);
float  ora_clip_volume_f(const float tet[4][3]);
double ora_clip_volume_d(const double tet[4][3]);
int    ora_classify_f(const float s[4][3]);
int    ora_classify_d(const double s[4][3]);
void   ora_grid_delta_f(const float bbox[6], int dims, float delta[3]);
void   ora_grid_delta_d(const float bbox[6], int dims, double delta[3]);

/* --- one tet into a grid (bbox = xmin,xmax,ymin,ymax,zmin,zmax) --- */
void ora_deposit_tet_f(const float v[4][3], float mass, int dims, const float bbox[6], float *grid,
                       unsigned int *cand, ora_stats *st);
void ora_deposit_tet_d(const double v[4][3], double mass, int dims, const float bbox[6], double *grid,
                       unsigned int *cand, ora_stats *st);

/* --- the reference boundary: patches of (m+1)^3 x 3 floats --- */
int ora_deposit_patches_f(size_t patch_offset, size_t num_patches, const float *positions,
                          size_t positions_size, int m, const float bbox[6], int dims, int order,
                          float mass, float *grid, unsigned int *cand, ora_stats *st);
int ora_deposit_patches_d(size_t patch_offset, size_t num_patches, const float *positions,
                          size_t positions_size, int m, const float bbox[6], int dims, int order,
                          double mass, double *grid, unsigned int *cand, ora_stats *st);
void ora_deposit_cubes_f(size_t cube_begin, size_t cube_end, const float *positions, int m,
                         const float bbox[6], int dims, int order, float mass, float *grid,
                         unsigned int *cand, ora_stats *st);
void ora_deposit_cubes_d(size_t cube_begin, size_t cube_end, const float *positions, int m,
                         const float bbox[6], int dims, int order, double mass, double *grid,
                         unsigned int *cand, ora_stats *st);

/* Multi-threaded patch deposit: cubes split over `threads` pthreads, each
 * with a private grid, then summed (the reference's worker-pool pattern).  */
int ora_deposit_patches_mt_f(size_t patch_offset, size_t num_patches, const float *positions,
                             size_t positions_size, int m, const float bbox[6], int dims, int order,
                             float mass, float *grid, int threads);
int ora_deposit_patches_mt_d(size_t patch_offset, size_t num_patches, const float *positions,
                             size_t positions_size, int m, const float bbox[6], int dims, int order,
                             double mass, double *grid, int threads);

/* 13 ints per tet: 4 vertex slots after the orientation rule, volume sign,
 * in-grid flag, candidate range (x0,x1,y0,y1,z0,z1), 0.                  */
void ora_tet_records_f(size_t cube_begin, size_t cube_end, const float *positions, int m,
                       const float bbox[6], int dims, int order, int *rec);

/* --- octree (FP32, as the reference) --- */
typedef struct {
    float    min[3];
    float    ext;
    int32_t  level;
    int32_t  parent;
    int32_t  first_child;   /* -1 for a leaf */
    int32_t  pad;
    uint64_t estimate;      /* num_tets_covering_node_estimate */
} ora_node;

/* Meta-cell AABBs of an nx*ny*nz vertex lattice (x fastest, 3 floats per
 * vertex): 7^3-cube meta-cells; out bbox: 6 floats each (min xyz, max xyz). */
size_t ora_meta_count(int nx, int ny, int nz);
void   ora_meta_bboxes(const float *pos, int nx, int ny, int nz, float *bbox6);
/* est = floor(6 * cells * vol(box ∩ mc) / vol(mc)), box = min xyz, max xyz */
uint64_t ora_meta_estimate(int nx, int ny, int nz, const float *mc_bbox6, uint64_t mc, const float box6[6]);

/* generate_tree; returns the node count (or -1 if max_nodes is too small).
 * leaf_meta_off/leaf_meta_ids: CSR of the meta-cell lists of every node
 * (only leaves keep theirs), sized max_nodes+1 / max_ids.                 */
int ora_generate_tree(const float *pos, int nx, int ny, int nz, const float box6[6], const float roi6[6],
                      uint64_t max_tets_per_node, int max_level, ora_node *nodes, int max_nodes,
                      int64_t *meta_off, uint64_t *meta_ids, int64_t max_ids);
/* DFS leaf order of Octree::getLeafNodes. Returns the leaf count. */
int ora_leaf_order(const ora_node *nodes, int n_nodes, int *leaf_ids);

/* Deposit all cubes of meta-cells `ids[0..n)` (lattice pos, x fastest) into a
 * leaf grid over bbox (xmin,xmax,...) exactly like the reference leaf loop
 * with one thread (meta-cell blocks in list order, cubes x fastest).      */
void ora_deposit_meta_f(const float *pos, int nx, int ny, int nz, const uint64_t *ids, size_t n,
                        const float bbox[6], int dims, int order, float mass, float *grid, ora_stats *st);
void ora_deposit_meta_d(const float *pos, int nx, int ny, int nz, const uint64_t *ids, size_t n,
                        const float bbox[6], int dims, int order, double mass, double *grid, ora_stats *st);

#ifdef __cplusplus
}
#endif
#endif
