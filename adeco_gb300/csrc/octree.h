// octree.h -- host-side octree refinement for the resident lattice.
//
// Reproduces the topology of ADECO's generate_tree bit-for-bit:
//   * meta-cells of 7^3 lattice cubes, ids x fastest       src/AdTypeDefinitions.h:715-1022
//   * estimate = (uint64)((float)(6*cells) * vol(box ∩ mcAABB) / vol(mcAABB))
//                                                           src/AdTypeDefinitions.h:812-825
//   * refine when estimate > max_tets, level < max_level and the node meets
//     the region of interest (strict AABB test); children x fastest; a child
//     inherits every parent meta-cell whose AABB strictly meets it
//                                                           src/AdOctreeGeneration.h:76-258,
//                                                           src/AdOctree.h:201-237
//   * leaves in the stack-DFS order of getLeafNodes        src/AdOctree.h:265-305
// The FP32 expressions keep the reference's operation order.
#pragma once

#include <cstdint>
#include <vector>

namespace adeco {

constexpr int kMetaCubes = 7;  // lattice cubes per meta-cell edge

// float -> uint64 of an estimate, truncating.  The reference converts
// implicitly, which is undefined for negative, NaN and huge values (a
// degenerate meta-cell AABB, or a root box that misses a meta-cell); here
// those saturate: NaN and values <= 0 give 0, values >= 2^64 give 2^64 - 1,
// as the device conversion (round toward zero, saturating) does.
inline uint64_t estimate_to_u64(float est)
{
    if (!(est > 0.f)) return 0;
    if (est >= 18446744073709551616.f) return ~0ull;
    return (uint64_t)est;
}

struct MetaGrid {
    int nx = 0, ny = 0, nz = 0;   // lattice vertices
    int cd[3] = {0, 0, 0};        // meta-cells per axis
    std::vector<float> bbox;      // 6 per meta-cell: min xyz, max xyz

    static int ceil_div(int x, int y) { return x / y + (x % y > 0); }
    void init(int nx_, int ny_, int nz_)
    {
        nx = nx_; ny = ny_; nz = nz_;
        cd[0] = ceil_div(nx - 1, kMetaCubes);
        cd[1] = ceil_div(ny - 1, kMetaCubes);
        cd[2] = ceil_div(nz - 1, kMetaCubes);
    }
    uint64_t count() const { return (uint64_t)cd[0] * cd[1] * cd[2]; }
    // vertex origin and vertex counts of meta-cell id
    void range(uint64_t id, int org[3], int nv[3]) const
    {
        const uint64_t nb = (uint64_t)cd[0], nb2 = nb * (uint64_t)cd[1];
        int c[3];
        if (id < (1ull << 32) && nb2 < (1ull << 32)) {  // every lattice that fits a GPU: 32-bit divisions
            const uint32_t i = (uint32_t)id, b = (uint32_t)nb, b2 = (uint32_t)nb2;
            const uint32_t z = i / b2, r = i - z * b2, y = r / b;
            c[0] = (int)(r - y * b);
            c[1] = (int)y;
            c[2] = (int)z;
        } else {
            c[0] = (int)(id % nb);
            c[1] = (int)((id % nb2) / nb);
            c[2] = (int)(id / nb2);
        }
        const int n[3] = {nx, ny, nz};
        for (int a = 0; a < 3; ++a) {
            org[a] = c[a] * kMetaCubes;
            nv[a] = (c[a] + 1 == cd[a]) ? (n[a] - org[a]) : kMetaCubes + 1;
        }
    }
    uint64_t estimate(uint64_t id, const float box[6]) const;
};

struct OctNode {
    float min[3];
    float ext;
    int32_t level;
    int32_t parent;
    int32_t first_child;
    uint64_t estimate;
};

// Spatial index over the meta-cells' AABBs: a uniform grid of buckets, each
// listing the meta-cells whose AABB meets it, so that a zoom box visits only
// the meta-cells near it instead of all of them.
struct MetaIndex {
    float lo[3] = {0, 0, 0}, inv[3] = {0, 0, 0};
    int nb[3] = {0, 0, 0};
    std::vector<uint32_t> start;  // CSR over the buckets, x fastest
    std::vector<uint32_t> ids;
    bool built = false;

    void build(const MetaGrid &mg);
    // meta-cells whose AABB strictly meets box6 (min xyz, max xyz), ascending
    void query(const MetaGrid &mg, const float box6[6], std::vector<uint32_t> &out) const;
};

struct Octree {
    std::vector<OctNode> nodes;
    std::vector<int32_t> leaves;              // getLeafNodes order
    std::vector<int64_t> leaf_meta_off;       // CSR over `leaves`
    std::vector<uint64_t> leaf_meta_ids;
    int levels = 0;

    // box6 / roi6: min xyz, max xyz.  Returns false on an internal overflow.
    bool build(const MetaGrid &mg, const float box6[6], const float roi6[6], uint64_t max_tets, int max_level);
};

}  // namespace adeco
