// Host harness for the CPU test of the host octree builder (octree.cpp): reads
// a lattice and the generate_tree parameters, forms the meta-cells' AABBs as
// meta_bbox_kernel does (FP32 min / max over each 8^3 vertex block), builds
// the tree and writes nodes, leaf order and leaf meta-cell lists.
//   in : int32 n, int32 max_level, int64 max_tets, float box[6], float roi[6],
//        float positions[n^3 * 3] (x fastest)
//   out: int32 n_nodes, nodes {float min[3], ext; int32 level, parent,
//        first_child; uint64 estimate}, int32 n_leaves, int32 leaves[],
//        int64 leaf_meta_off[n_leaves + 1], uint64 leaf_meta_ids[]
#include "../adeco_gb300/csrc/octree.h"

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <vector>

using namespace adeco;

template <typename T>
static bool get(FILE *f, T *p, size_t n)
{
    return std::fread(p, sizeof(T), n, f) == n;
}

template <typename T>
static void put(FILE *f, const T *p, size_t n)
{
    std::fwrite(p, sizeof(T), n, f);
}

int main(int argc, char **argv)
{
    if (argc != 3) return 2;
    FILE *in = std::fopen(argv[1], "rb");
    if (!in) return 2;
    int32_t n = 0, max_level = 0;
    int64_t max_tets = 0;
    float box[6], roi[6];
    if (!get(in, &n, 1) || !get(in, &max_level, 1) || !get(in, &max_tets, 1) || !get(in, box, 6) || !get(in, roi, 6))
        return 2;
    std::vector<float> pos((size_t)n * n * n * 3);
    if (!get(in, pos.data(), pos.size())) return 2;
    std::fclose(in);

    MetaGrid mg;
    mg.init(n, n, n);
    mg.bbox.resize(mg.count() * 6);
    for (uint64_t id = 0; id < mg.count(); ++id) {
        int org[3], nv[3];
        mg.range(id, org, nv);
        float mn[3] = {3.4e38f, 3.4e38f, 3.4e38f}, mx[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
        for (int k = 0; k < nv[2]; ++k)
            for (int j = 0; j < nv[1]; ++j)
                for (int i = 0; i < nv[0]; ++i) {
                    const size_t v = (size_t)(org[0] + i) + (size_t)n * ((size_t)(org[1] + j) + (size_t)n * (org[2] + k));
                    for (int a = 0; a < 3; ++a) {
                        mn[a] = std::min(mn[a], pos[3 * v + a]);
                        mx[a] = std::max(mx[a], pos[3 * v + a]);
                    }
                }
        for (int a = 0; a < 3; ++a) {
            mg.bbox[6 * id + a] = mn[a];
            mg.bbox[6 * id + 3 + a] = mx[a];
        }
    }
    const uint64_t total = 6ull * (uint64_t)(n - 1) * (uint64_t)(n - 1) * (uint64_t)(n - 1);
    Octree t;
    if (!t.build(mg, box, roi, std::min<uint64_t>(total, (uint64_t)max_tets), max_level)) return 3;

    FILE *out = std::fopen(argv[2], "wb");
    if (!out) return 2;
    const int32_t nn = (int32_t)t.nodes.size();
    put(out, &nn, 1);
    for (const OctNode &o : t.nodes) {
        put(out, o.min, 3);
        put(out, &o.ext, 1);
        put(out, &o.level, 1);
        put(out, &o.parent, 1);
        put(out, &o.first_child, 1);
        put(out, &o.estimate, 1);
    }
    const int32_t nl = (int32_t)t.leaves.size();
    put(out, &nl, 1);
    put(out, t.leaves.data(), t.leaves.size());
    put(out, t.leaf_meta_off.data(), t.leaf_meta_off.size());
    put(out, t.leaf_meta_ids.data(), t.leaf_meta_ids.size());
    std::fclose(out);
    return 0;
}
