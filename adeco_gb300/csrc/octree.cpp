// octree.cpp -- see octree.h.  Built with -ffp-contract=off so every FP32
// expression is evaluated as written on x86-64 and on Arm hosts alike.
#include "octree.h"

#include <algorithm>
#include <cmath>

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
    return estimate_to_u64(est);
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

void MetaIndex::build(const MetaGrid &mg)
{
    const uint64_t n = mg.count();
    float hi[3] = {0, 0, 0};
    double ext[3] = {0, 0, 0};
    for (int a = 0; a < 3; ++a) {
        lo[a] = n ? mg.bbox[a] : 0.f;
        hi[a] = n ? mg.bbox[3 + a] : 0.f;
    }
    for (uint64_t id = 0; id < n; ++id) {
        const float *b = &mg.bbox[6 * id];
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], b[a]);
            hi[a] = std::max(hi[a], b[3 + a]);
            ext[a] += (double)b[3 + a] - (double)b[a];
        }
    }
    // buckets about twice a meta-cell's mean extent, at most 64 per axis
    for (int a = 0; a < 3; ++a) {
        const double span = std::max((double)hi[a] - (double)lo[a], 1e-30);
        const double want = n ? 2.0 * ext[a] / (double)n : span;
        nb[a] = (int)std::min(64.0, std::max(1.0, std::floor(span / std::max(want, 1e-30))));
        inv[a] = (float)(nb[a] / span);
    }
    const size_t nbk = (size_t)nb[0] * nb[1] * nb[2];
    start.assign(nbk + 1, 0);
    std::vector<uint32_t> fill;
    for (int pass = 0; pass < 2; ++pass) {
        if (pass == 1) {
            for (size_t k = 0; k < nbk; ++k) start[k + 1] += start[k];
            ids.assign(start[nbk], 0);
            fill.assign(start.begin(), start.end() - 1);
        }
        for (uint64_t id = 0; id < n; ++id) {
            const float *b = &mg.bbox[6 * id];
            int r[6];
            for (int a = 0; a < 3; ++a) {
                r[a] = std::max(0, std::min(nb[a] - 1, (int)((b[a] - lo[a]) * inv[a])));
                r[3 + a] = std::max(0, std::min(nb[a] - 1, (int)((b[3 + a] - lo[a]) * inv[a])));
            }
            for (int z = r[2]; z <= r[5]; ++z)
                for (int y = r[1]; y <= r[4]; ++y)
                    for (int x = r[0]; x <= r[3]; ++x) {
                        const size_t k = (size_t)x + (size_t)nb[0] * ((size_t)y + (size_t)nb[1] * z);
                        if (pass == 0)
                            ++start[k + 1];
                        else
                            ids[fill[k]++] = (uint32_t)id;
                    }
        }
    }
    built = true;
}

void MetaIndex::query(const MetaGrid &mg, const float box6[6], std::vector<uint32_t> &out) const
{
    out.clear();
    int r[6];
    for (int a = 0; a < 3; ++a) {
        r[a] = std::max(0, std::min(nb[a] - 1, (int)((box6[a] - lo[a]) * inv[a])));
        r[3 + a] = std::max(0, std::min(nb[a] - 1, (int)((box6[3 + a] - lo[a]) * inv[a])));
    }
    for (int z = r[2]; z <= r[5]; ++z)
        for (int y = r[1]; y <= r[4]; ++y)
            for (int x = r[0]; x <= r[3]; ++x) {
                const size_t k = (size_t)x + (size_t)nb[0] * ((size_t)y + (size_t)nb[1] * z);
                for (uint32_t q = start[k]; q < start[k + 1]; ++q)
                    if (meets(&mg.bbox[6 * (size_t)ids[q]], box6)) out.push_back(ids[q]);
            }
    std::sort(out.begin(), out.end());
    out.erase(std::unique(out.begin(), out.end()), out.end());
}

}  // namespace adeco
