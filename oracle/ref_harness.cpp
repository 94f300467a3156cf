// ref_harness.cpp -- C entry points over the reference's own deposit and
// octree code, compiled from the reference sources by oracle/build_ref.sh into
// oracle/_ref/libadeco_ref.so.  TEST INFRASTRUCTURE ONLY: it pins the C oracle
// (oracle/adeco_oracle.c) and generates the golden fixtures; nothing in the
// product loads it.  It contains no reference code, only calls into it.
//
// Calls made:
//   AdaptiveMassDeposit::DepositWrapper::deposit_tets (CPU)  src/AdDeposit2Grid.cpp:67
//   deposit_tet_2_grid<double,double>                      src/AdDepositTets2Grid.h:509
//   compute_unit_cube_tet_intersection_volume<T>           src/AdTetIntersection.h:383
//   intersection_test<T>                                   src/AdDepositTets2Grid.h:286
//   MetaMesh / AdOctreeGeneration::generate_tree / Octree::getLeafNodes
//                                                          src/AdTypeDefinitions.h:715,
//                                                          src/AdOctreeGeneration.h:76,
//                                                          src/AdOctree.h:265
#include <cstring>
#include <cstdint>
#include <vector>

// Single-rank stand-ins for the three MPI names generate_tree uses; with one
// rank MPI_Allgather is a copy.
#define MPI_CHAR 0
#define MPI_COMM_WORLD 0
static inline int MPI_Allgather(const void *s, int sc, int, void *r, int, int, int)
{
    std::memcpy(r, s, (size_t)sc);
    return 0;
}
#define CHECK_MPI_ERROR(x) (void)(x)

// The reference's headers define non-inline functions, so its CPU deposit
// translation unit is compiled as part of this one (included by path from the
// reference tree, not copied).
#include "AdDeposit2Grid.cpp"
#include "AdTypeDefinitions.h"
#include "AdOctree.h"
#include "AdOctreeGeneration.h"

using namespace AdaptiveMassDeposit;

extern "C" {

int ref_deposit_patches_f32(size_t patch_offset, size_t num_patches, const float *positions,
                            size_t positions_size, int m, const float bbox[6], int dims, float *grid)
{
    try {
        DepositWrapper::deposit_tets(false, 0, patch_offset, num_patches, positions, positions_size, m, bbox,
                                     dims, grid);
    } catch (...) {
        return -1;
    }
    return 0;
}

// FP64: the reference's deposit_tet_2_grid<double,double> fed with the corners
// of each cube, either in sample_cell_vertices order (order 0) or in the binary
// vert[] order (order 1, slot = 4x+2y+z).
int ref_deposit_patches_f64(size_t patch_offset, size_t num_patches, const float *positions, int m,
                            const float bbox[6], int dims, int order, double *grid)
{
    const int fpp = 3 * (m + 1) * (m + 1) * (m + 1);
    const int cpp = m * m * m;
    const int grid_dims[3] = {dims, dims, dims};
    const dbox<double> gb(dvec3<double>(bbox[0], bbox[2], bbox[4]), dvec3<double>(bbox[1], bbox[3], bbox[5]));
    for (size_t p = patch_offset; p < patch_offset + num_patches; ++p) {
        const float *patch = positions + p * (size_t)fpp;
        for (int c = 0; c < cpp; ++c) {
            float cp[24];
            if (order == 0) {
                sample_cell_vertices<float>(c, patch, m, cp);
            } else {
                const int k = c / (m * m), rem = c % (m * m), j = rem / m, i = rem % m;
                for (int s = 0; s < 8; ++s) {
                    const int dx = (s >> 2) & 1, dy = (s >> 1) & 1, dz = s & 1;
                    const int id = (i + dx) + (m + 1) * ((j + dy) + (m + 1) * (k + dz));
                    cp[3 * s] = patch[3 * id]; cp[3 * s + 1] = patch[3 * id + 1]; cp[3 * s + 2] = patch[3 * id + 2];
                }
            }
            bool pad = false;
            for (int q = 0; q < 24; q += 3)
                if (fabsf(cp[q] - 666.f) + fabsf(cp[q + 1] - 666.f) + fabsf(cp[q + 2] - 666.f) < 1.E-03) pad = true;
            if (pad) continue;
            for (int t = 0; t < 6; ++t) {
                dvec3<double> tv[4];
                for (int v = 0; v < 4; ++v) {
                    const int idx = 3 * tet_conn[t][v];
                    tv[v] = dvec3<double>(cp[idx], cp[idx + 1], cp[idx + 2]);
                }
                deposit_tet_2_grid<double, double>(tv, 1.0, grid_dims, gb, grid);
            }
        }
    }
    return 0;
}

float ref_clip_volume_f32(const float tet[12])
{
    dvec3<float> t[4];
    for (int v = 0; v < 4; ++v) t[v] = dvec3<float>(tet[3 * v], tet[3 * v + 1], tet[3 * v + 2]);
    return compute_unit_cube_tet_intersection_volume<float>(t);
}

double ref_clip_volume_f64(const double tet[12])
{
    dvec3<double> t[4];
    for (int v = 0; v < 4; ++v) t[v] = dvec3<double>(tet[3 * v], tet[3 * v + 1], tet[3 * v + 2]);
    return compute_unit_cube_tet_intersection_volume<double>(t);
}

int ref_classify_f32(const float tet[12])
{
    dvec3<float> t[4];
    for (int v = 0; v < 4; ++v) t[v] = dvec3<float>(tet[3 * v], tet[3 * v + 1], tet[3 * v + 2]);
    dvec3<float> cell[8];
    get_cell(dvec3<float>(0.f, 0.f, 0.f), dvec3<float>(1.f, 1.f, 1.f), cell);
    dbox<float> ub(dvec3<float>(0.f, 0.f, 0.f), dvec3<float>(1.f, 1.f, 1.f));
    return (int)intersection_test(ub, cell, t);
}

// generate_tree over an nx*ny*nz lattice (x fastest, 3 floats per vertex).
// Fills node records (min xyz, ext, level, parent, first_child, estimate) and
// the leaf order of getLeafNodes plus each leaf's meta-cell list (CSR in leaf
// order).  Returns the node count, or -1 when the outputs are too small.
int ref_generate_tree(const float *pos, int nx, int ny, int nz, const float box6[6], const float roi6[6],
                      uint64_t max_tets, int max_level, float *node_f /*4 per node*/,
                      int32_t *node_i /*3 per node*/, uint64_t *node_est, int max_nodes, int32_t *leaf_ids,
                      int32_t *n_leaves, int64_t *leaf_meta_off, uint64_t *leaf_meta_ids, int64_t max_ids)
{
    Tetrahedra<ColumnMajorOrder> tets;
    const size_t n = (size_t)nx * ny * nz;
    tets.particles.set_num_positions(n);
    for (size_t i = 0; i < n; ++i) tets.particles.set_position(i, pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    tets.set_patch_dims(nx, ny, nz);
    MetaMesh<ColumnMajorOrder> mesh(tets);
    AABBox box(PosVec(box6[0], box6[1], box6[2]), PosVec(box6[3], box6[4], box6[5]));
    AABBox roi(PosVec(roi6[0], roi6[1], roi6[2]), PosVec(roi6[3], roi6[4], roi6[5]));
    TetOctree octree;
    AdOctreeGeneration<ColumnMajorOrder>::generate_tree(1, 0, box, roi, max_tets, max_level, mesh, octree);
    const int nn = (int)octree.getNodes().size();
    if (nn > max_nodes) return -1;
    for (int i = 0; i < nn; ++i) {
        const TetOctree::Node &nd = octree.getNode(i);
        node_f[4 * i + 0] = nd.getLowerLeft()[0];
        node_f[4 * i + 1] = nd.getLowerLeft()[1];
        node_f[4 * i + 2] = nd.getLowerLeft()[2];
        node_f[4 * i + 3] = nd.getExtension();
        node_i[3 * i + 0] = nd.getLevel();
        node_i[3 * i + 1] = nd.getParentId();
        node_i[3 * i + 2] = nd.isRefined() ? nd.getChildId(0) : -1;
        node_est[i] = nd.getNodeData().num_tets_covering_node_estimate;
    }
    std::vector<node_id_t> leaves;
    octree.getLeafNodes(leaves);
    *n_leaves = (int32_t)leaves.size();
    int64_t off = 0;
    for (size_t l = 0; l < leaves.size(); ++l) {
        leaf_ids[l] = leaves[l];
        leaf_meta_off[l] = off;
        const std::vector<uint64_t> &ids = octree.getNode(leaves[l]).getNodeData().local_meta_cell_ids;
        if (off + (int64_t)ids.size() > max_ids) return -1;
        for (size_t q = 0; q < ids.size(); ++q) leaf_meta_ids[off + (int64_t)q] = ids[q];
        off += (int64_t)ids.size();
    }
    leaf_meta_off[leaves.size()] = off;
    return nn;
}

// The reference leaf loop on one worker: positions of the leaf's meta-cells
// gathered with MetaMesh::get_tets (666-padded 8^3 blocks), then deposit_tets.
int ref_deposit_leaf_f32(const float *pos, int nx, int ny, int nz, const uint64_t *ids, size_t n_ids,
                         const float bbox[6], int dims, float *grid)
{
    Tetrahedra<ColumnMajorOrder> tets;
    const size_t n = (size_t)nx * ny * nz;
    tets.particles.set_num_positions(n);
    for (size_t i = 0; i < n; ++i) tets.particles.set_position(i, pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    tets.set_patch_dims(nx, ny, nz);
    MetaMesh<ColumnMajorOrder> mesh(tets);
    std::vector<float> all, one;
    AABBox dummy;
    for (size_t q = 0; q < n_ids; ++q) {
        mesh.get_tets(dummy, ids[q], one);
        all.insert(all.end(), one.begin(), one.end());
    }
    if (all.empty()) return 0;
    const int m = MetaMesh<ColumnMajorOrder>::get_number_of_cells_per_dimension();
    const size_t fpp = 3 * (size_t)(m + 1) * (m + 1) * (m + 1);
    try {
        DepositWrapper::deposit_tets(false, 0, 0, all.size() / fpp, all.data(), all.size(), m, bbox, dims, grid);
    } catch (...) {
        return -1;
    }
    return 0;
}

}  // extern "C"
