// octree.cpp -- see octree.h.  Built with -ffp-contract=off so every FP32
// expression is evaluated as written on x86-64 and on Arm hosts alike.
#include "octree.h"

#include <algorithm>

namespace adeco {

namespace {

inline bool meets(const float *a, const float *b)  // strict AABB overlap, min xyz max xyz
{
    return a[0] < b[3] && b[0] < a[3] && a[1] < b[4] && b[1] < a[4] && a[2] < b[5] && b[2] < a[5];
}

inline float box_volume(const float *b)
{
    const float ex = b[3] - b[0];
    const float ey = b[4] - b[1];
    const float ez = b[5] - b[2];
    const float exy = ex * ey;
    return exy * ez;
}

inline void node_box(const OctNode &n, float b[6])
{
    for (int a = 0; a < 3; ++a) {
        b[a] = n.min[a];
        b[3 + a] = n.min[a] + n.ext;
    }
}

}  // namespace

uint64_t MetaGrid::estimate(uint64_t id, const float box[6]) const
{
    int org[3], nv[3];
    range(id, org, nv);
    const uint64_t cells = (uint64_t)(nv[0] - 1) * (uint64_t)(nv[1] - 1) * (uint64_t)(nv[2] - 1);
    const float *m = &bbox[6 * id];
    float ib[6];
    for (int a = 0; a < 3; ++a) {
        ib[a] = (box[a] < m[a]) ? m[a] : box[a];
        ib[3 + a] = (box[3 + a] < m[3 + a]) ? box[3 + a] : m[3 + a];
    }
    const float scaled = (float)(6 * cells) * box_volume(ib);
    const float est = scaled / box_volume(m);
    return (uint64_t)est;
}

bool Octree::build(const MetaGrid &mg, const float box6[6], const float roi6[6], uint64_t max_tets, int max_level)
{
    nodes.clear();
    leaves.clear();
    leaf_meta_off.clear();
    leaf_meta_ids.clear();
    float roi[6];
    const bool invalid_roi = roi6 == nullptr || roi6[0] > roi6[3] || roi6[1] > roi6[4] || roi6[2] > roi6[5];
    for (int a = 0; a < 6; ++a) roi[a] = invalid_roi ? box6[a] : roi6[a];

    const float e0 = box6[3] - box6[0], e1 = box6[4] - box6[1], e2 = box6[5] - box6[2];
    OctNode root;
    root.min[0] = box6[0];
    root.min[1] = box6[1];
    root.min[2] = box6[2];
    root.ext = std::max(std::max(e0, e1), e2);
    root.level = 0;
    root.parent = -1;
    root.first_child = -1;
    root.estimate = 0;
    nodes.push_back(root);
    levels = 1;

    std::vector<std::vector<uint64_t>> lists(1);
    lists[0].resize(mg.count());
    for (uint64_t i = 0; i < mg.count(); ++i) lists[0][i] = i;

    std::vector<int32_t> stack;
    stack.push_back(0);
    size_t guard = 0;
    while (!stack.empty()) {
        if (++guard > 100000000u) return false;
        const int32_t cur = stack.back();
        stack.pop_back();
        float cb[6];
        node_box(nodes[cur], cb);
        uint64_t est = 0;
        for (uint64_t id : lists[cur]) est += mg.estimate(id, cb);
        nodes[cur].estimate = est;
        if (!meets(roi, cb)) continue;
        if (!(est > 0 && est > max_tets && nodes[cur].level < max_level)) continue;
        const int32_t first = (int32_t)nodes.size();
        nodes[cur].first_child = first;
        const float cext = (float)((double)nodes[cur].ext / 2.);
        const OctNode parent = nodes[cur];
        for (int k = 0; k < 2; ++k)
            for (int j = 0; j < 2; ++j)
                for (int i = 0; i < 2; ++i) {
                    OctNode ch;
                    ch.min[0] = parent.min[0] + (float)i * cext;
                    ch.min[1] = parent.min[1] + (float)j * cext;
                    ch.min[2] = parent.min[2] + (float)k * cext;
                    ch.ext = cext;
                    ch.level = parent.level + 1;
                    ch.parent = cur;
                    ch.first_child = -1;
                    ch.estimate = 0;
                    nodes.push_back(ch);
                }
        levels = std::max(levels, parent.level + 2);
        lists.resize(nodes.size());
        float chb[8][6];
        for (int q = 0; q < 8; ++q) node_box(nodes[first + q], chb[q]);
        for (uint64_t id : lists[cur]) {
            const float *mb = &mg.bbox[6 * id];
            for (int q = 0; q < 8; ++q)
                if (meets(mb, chb[q])) lists[first + q].push_back(id);
        }
        std::vector<uint64_t>().swap(lists[cur]);
        for (int q = 0; q < 8; ++q) stack.push_back(first + q);
    }
    // getLeafNodes order
    stack.clear();
    stack.push_back(0);
    while (!stack.empty()) {
        const int32_t cur = stack.back();
        stack.pop_back();
        if (nodes[cur].first_child > 0) {
            for (int q = 0; q < 8; ++q) stack.push_back(nodes[cur].first_child + q);
        } else {
            leaves.push_back(cur);
        }
    }
    leaf_meta_off.reserve(leaves.size() + 1);
    int64_t off = 0;
    for (int32_t l : leaves) {
        leaf_meta_off.push_back(off);
        leaf_meta_ids.insert(leaf_meta_ids.end(), lists[l].begin(), lists[l].end());
        off += (int64_t)lists[l].size();
    }
    leaf_meta_off.push_back(off);
    return true;
}

}  // namespace adeco
