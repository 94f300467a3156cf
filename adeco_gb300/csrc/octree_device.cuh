// octree_device.cuh -- octree refinement with the per-(node, meta-cell) work on
// the device.  Included by runtime.cu after DevBuf, fail() and CUDA_TRY.
//
// The tree is the one Octree::build (octree.cpp) makes, field for field and
// in the same node numbering, for the reference's generate_tree
// (src/AdOctreeGeneration.h:76-258, estimate src/AdTypeDefinitions.h:812-825,
// getLeafNodes src/AdOctree.h:265-305).  The work is split by size:
//
//   device, O(pairs): every (node, meta-cell) pair of a level -- the estimate
//     Σ_meta trunc(6·cells·vol(node ∩ AABB)/vol(AABB)) and the strict AABB test
//     that hands a meta-cell to each of the 8 children, with an ordered
//     compaction so each child's list keeps its parent's (ascending) order;
//   host, O(nodes): the refinement decision, the child boxes (the same FP32
//     expressions as octree.cpp, so the boxes are the same bits), and at the
//     end the depth-first numbering and leaf order of the stack walk.
//
// Levels are built breadth first: one launch sequence and one small
// device-to-host read (child list offsets and estimates) per level.  The
// estimates are integer sums, so their order does not matter; the FP32 terms
// use explicitly rounded intrinsics (no contraction), so each term has the
// bits of the host's.

namespace adeco {

constexpr int kTreeChunk = 2048;   // pairs of one parent per block
constexpr int kTreeThreads = 256;  // 8 warps
constexpr size_t kTreeMaxNodes = (size_t)1 << 24;

struct TreeMeta {  // MetaGrid's shape, by value for the kernels
    int nx, ny, nz;
    int cd[3];
};

struct TreeBox {
    float v[6];  // min xyz, max xyz
};

struct TreeChunk {
    int parent;  // rank of the refined parent within the level
    int start;   // first pair in the level's id list
    int len;
    int pad;
};

__device__ __forceinline__ bool tree_meets(const float *a, const float *b)
{
    return a[0] < b[3] && b[0] < a[3] && a[1] < b[4] && b[1] < a[4] && a[2] < b[5] && b[2] < a[5];
}

__device__ __forceinline__ float tree_box_volume(const float *b)
{
    const float ex = __fsub_rn(b[3], b[0]);
    const float ey = __fsub_rn(b[4], b[1]);
    const float ez = __fsub_rn(b[5], b[2]);
    return __fmul_rn(__fmul_rn(ex, ey), ez);
}

// MetaGrid::estimate for meta-cell `id` with AABB `m` against `box`
__device__ __forceinline__ unsigned long long tree_estimate(const TreeMeta &md, unsigned id, const float *m,
                                                            const float *box)
{
    const unsigned nb = (unsigned)md.cd[0], nb2 = nb * (unsigned)md.cd[1];
    const int c[3] = {(int)(id % nb), (int)((id % nb2) / nb), (int)(id / nb2)};
    const int n[3] = {md.nx, md.ny, md.nz};
    unsigned long long cells = 1;
    float ib[6];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int org = c[a] * kMetaCubes;
        const int nv = (c[a] + 1 == md.cd[a]) ? (n[a] - org) : kMetaCubes + 1;
        cells *= (unsigned long long)(nv - 1);
        ib[a] = (box[a] < m[a]) ? m[a] : box[a];
        ib[3 + a] = (box[3 + a] < m[3 + a]) ? box[3 + a] : m[3 + a];
    }
    const float scaled = __fmul_rn(__ull2float_rn(6ull * cells), tree_box_volume(ib));
    return __float2ull_rz(__fdiv_rn(scaled, tree_box_volume(m)));
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// root: the list is every meta-cell, in id order; estimate against the root box
__global__ void tree_root_kernel(TreeMeta md, const float *__restrict__ mbb, unsigned nmc, TreeBox box,
                                 unsigned *__restrict__ ids, unsigned long long *__restrict__ est)
{
    unsigned long long sum = 0;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < nmc; i += gridDim.x * blockDim.x) {
        ids[i] = i;
        float m[6];
#pragma unroll
        for (int a = 0; a < 6; ++a) m[a] = mbb[6 * (size_t)i + a];
        sum += tree_estimate(md, i, m, box.v);
    }
    sum = warp_sum_u64(sum);
    if ((threadIdx.x & 31) == 0 && sum) atomicAdd(est, sum);
}

// pass 1: per chunk, how many of its meta-cells each child receives
__global__ void __launch_bounds__(kTreeThreads) tree_count_kernel(const float *__restrict__ mbb,
                                                                  const unsigned *__restrict__ ids,
                                                                  const TreeChunk *__restrict__ chunks,
                                                                  const float *__restrict__ child_box,
                                                                  int *__restrict__ chunk_cnt)
{
    __shared__ float cb[8][6];
    __shared__ int cnt[8];
    const TreeChunk ch = chunks[blockIdx.x];
    if (threadIdx.x < 48) cb[threadIdx.x / 6][threadIdx.x % 6] = child_box[(size_t)ch.parent * 48 + threadIdx.x];
    if (threadIdx.x < 8) cnt[threadIdx.x] = 0;
    __syncthreads();
    int mine[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = threadIdx.x; i < ch.len; i += blockDim.x) {
        const unsigned id = ids[ch.start + i];
        float m[6];
#pragma unroll
        for (int a = 0; a < 6; ++a) m[a] = mbb[6 * (size_t)id + a];
#pragma unroll
        for (int q = 0; q < 8; ++q) mine[q] += tree_meets(m, cb[q]) ? 1 : 0;
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        int v = mine[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0 && v) atomicAdd(&cnt[q], v);
    }
    __syncthreads();
    if (threadIdx.x < 8) chunk_cnt[(size_t)blockIdx.x * 8 + threadIdx.x] = cnt[threadIdx.x];
}

// pass 2 (one block): each chunk's first slot in each child list, and the
// child lists' offsets in the next level's id list (child_off[nc] = total)
__global__ void __launch_bounds__(1024) tree_scan_kernel(const TreeChunk *__restrict__ chunks, int nchunks,
                                                         const int *__restrict__ parent_first_chunk, int n_ref,
                                                         const int *__restrict__ chunk_cnt,
                                                         int *__restrict__ chunk_base, int *__restrict__ child_off)
{
    __shared__ int part[1024];
    __shared__ int carry;
    const int nc = 8 * n_ref;
    // child list lengths, and each chunk's place within its parent's child lists
    for (int c = threadIdx.x; c < nc; c += blockDim.x) {
        const int k = c >> 3, q = c & 7;
        int run = 0;
        for (int t = parent_first_chunk[k]; t < parent_first_chunk[k + 1]; ++t) {
            chunk_base[(size_t)t * 8 + q] = run;
            run += chunk_cnt[(size_t)t * 8 + q];
        }
        child_off[c] = run;
    }
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    // exclusive scan of the lengths, 1024 at a time
    for (int base = 0; base < nc; base += blockDim.x) {
        const int c = base + threadIdx.x;
        const int v = c < nc ? child_off[c] : 0;
        part[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < (int)blockDim.x; o <<= 1) {
            const int add = threadIdx.x >= (unsigned)o ? part[threadIdx.x - o] : 0;
            __syncthreads();
            part[threadIdx.x] += add;
            __syncthreads();
        }
        if (c < nc) child_off[c] = carry + part[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry += part[threadIdx.x];
        __syncthreads();
    }
    if (threadIdx.x == 0) child_off[nc] = carry;
    __syncthreads();
    for (int e = threadIdx.x; e < nchunks * 8; e += blockDim.x) {
        const int t = e >> 3, q = e & 7;
        chunk_base[e] += child_off[chunks[t].parent * 8 + q];
    }
}

// pass 3: ordered compaction of each chunk into the child lists, with the
// children's estimates
__global__ void __launch_bounds__(kTreeThreads) tree_fill_kernel(TreeMeta md, const float *__restrict__ mbb,
                                                                 const unsigned *__restrict__ ids,
                                                                 const TreeChunk *__restrict__ chunks,
                                                                 const float *__restrict__ child_box,
                                                                 const int *__restrict__ chunk_base,
                                                                 unsigned *__restrict__ next_ids,
                                                                 unsigned long long *__restrict__ child_est)
{
    __shared__ float cb[8][6];
    __shared__ int wtot[8][kTreeThreads / 32];
    __shared__ int run[8];
    __shared__ unsigned long long est[8];
    const TreeChunk ch = chunks[blockIdx.x];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x < 48) cb[threadIdx.x / 6][threadIdx.x % 6] = child_box[(size_t)ch.parent * 48 + threadIdx.x];
    if (threadIdx.x < 8) {
        run[threadIdx.x] = chunk_base[(size_t)blockIdx.x * 8 + threadIdx.x];
        est[threadIdx.x] = 0;
    }
    __syncthreads();
    unsigned long long mine[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const unsigned lt = (1u << lane) - 1u;
    for (int r0 = 0; r0 < ch.len; r0 += blockDim.x) {
        const int i = r0 + threadIdx.x;
        unsigned id = 0;
        float m[6] = {0, 0, 0, 0, 0, 0};
        if (i < ch.len) {
            id = ids[ch.start + i];
#pragma unroll
            for (int a = 0; a < 6; ++a) m[a] = mbb[6 * (size_t)id + a];
        }
        unsigned bits[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const bool in = i < ch.len && tree_meets(m, cb[q]);
            bits[q] = __ballot_sync(0xffffffffu, in);
            if (lane == 0) wtot[q][warp] = __popc(bits[q]);
            if (in) mine[q] += tree_estimate(md, id, m, cb[q]);
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            if ((bits[q] >> lane) & 1u) {
                int pos = run[q] + __popc(bits[q] & lt);
                for (int w = 0; w < warp; ++w) pos += wtot[q][w];
                next_ids[pos] = id;
            }
        }
        __syncthreads();
        if (threadIdx.x < 8) {
            int s = 0;
            for (int w = 0; w < kTreeThreads / 32; ++w) s += wtot[threadIdx.x][w];
            run[threadIdx.x] += s;
        }
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const unsigned long long v = warp_sum_u64(mine[q]);
        if (lane == 0 && v) atomicAdd(&est[q], v);
    }
    __syncthreads();
    if (threadIdx.x < 8 && est[threadIdx.x]) atomicAdd(&child_est[(size_t)ch.parent * 8 + threadIdx.x], est[threadIdx.x]);
}

namespace tree_host {

inline bool meets(const float *a, const float *b)
{
    return a[0] < b[3] && b[0] < a[3] && a[1] < b[4] && b[1] < a[4] && a[2] < b[5] && b[2] < a[5];
}

inline void node_box(const OctNode &n, float b[6])
{
    for (int a = 0; a < 3; ++a) {
        b[a] = n.min[a];
        b[3 + a] = n.min[a] + n.ext;
    }
}

struct BfsNode {
    OctNode n;       // parent / first_child are breadth-first indices here
    int lv = 0;      // level buffer holding its list
    int off = 0, len = 0;
};

}  // namespace tree_host

// Builds `tree` as Octree::build(mg, box6, roi6, max_tets, max_level) does.
// d_mbb: the meta-cells' AABBs on the device (6 floats each, min xyz, max xyz).
static int build_octree_device(const MetaGrid &mg, const float *d_mbb, const float box6[6], const float *roi6,
                               uint64_t max_tets, int max_level, cudaStream_t st, Octree &tree)
{
    using namespace tree_host;
    tree.nodes.clear();
    tree.leaves.clear();
    tree.leaf_meta_off.clear();
    tree.leaf_meta_ids.clear();
    const uint64_t nmc64 = mg.count();
    if (nmc64 == 0 || nmc64 >= (1ull << 31)) return fail(ADECO_ERR_LIMIT, "meta-cell count %llu out of range",
                                                         (unsigned long long)nmc64);
    const unsigned nmc = (unsigned)nmc64;
    float roi[6];
    const bool invalid_roi = roi6 == nullptr || roi6[0] > roi6[3] || roi6[1] > roi6[4] || roi6[2] > roi6[5];
    for (int a = 0; a < 6; ++a) roi[a] = invalid_roi ? box6[a] : roi6[a];
    TreeMeta md;
    md.nx = mg.nx; md.ny = mg.ny; md.nz = mg.nz;
    for (int a = 0; a < 3; ++a) md.cd[a] = mg.cd[a];

    std::vector<std::unique_ptr<DevBuf<unsigned>>> lv_ids;
    // A level's small arrays share one device block and one host block, so
    // a level costs one copy each way and the block is reallocated only when
    // it grows (by 2x at least): est | off (brought back), chunks | pfc | cbox
    // (sent), cnt | base (device only).
    DevBuf<unsigned char> d_lvl;
    std::vector<unsigned char> h_lvl;
    int rc;

    std::vector<BfsNode> bfs(1);
    {
        const float e0 = box6[3] - box6[0], e1 = box6[4] - box6[1], e2 = box6[5] - box6[2];
        OctNode &root = bfs[0].n;
        root.min[0] = box6[0];
        root.min[1] = box6[1];
        root.min[2] = box6[2];
        root.ext = std::max(std::max(e0, e1), e2);
        root.level = 0;
        root.parent = -1;
        root.first_child = -1;
        root.estimate = 0;
        bfs[0].lv = 0;
        bfs[0].off = 0;
        bfs[0].len = (int)nmc;
    }
    int levels = 1;
    lv_ids.emplace_back(new DevBuf<unsigned>());
    if ((rc = lv_ids[0]->reserve(nmc)) || (rc = d_lvl.reserve(4096))) return rc;
    {
        unsigned long long *d_est = reinterpret_cast<unsigned long long *>(d_lvl.p);
        CUDA_TRY(cudaMemsetAsync(d_est, 0, sizeof(unsigned long long), st));
        TreeBox rb;
        node_box(bfs[0].n, rb.v);
        const unsigned blocks = std::min<unsigned>((nmc + 255) / 256, 4096u);
        tree_root_kernel<<<blocks, 256, 0, st>>>(md, d_mbb, nmc, rb, lv_ids[0]->p, d_est);
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(cudaMemcpyAsync(&bfs[0].n.estimate, d_est, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
    }

    size_t lv_begin = 0, lv_end = 1;  // this level's nodes in `bfs`
    std::vector<int> refined, pfc;
    std::vector<TreeChunk> chunks;
    std::vector<float> cbox;
    for (int lv = 0; lv_begin < lv_end; ++lv) {
        refined.clear();
        for (size_t i = lv_begin; i < lv_end; ++i) {
            const OctNode &n = bfs[i].n;
            float cb[6];
            node_box(n, cb);
            if (!meets(roi, cb)) continue;
            if (!(n.estimate > 0 && n.estimate > max_tets && n.level < max_level)) continue;
            refined.push_back((int)i);
        }
        if (refined.empty()) break;
        if (bfs.size() + 8 * refined.size() > kTreeMaxNodes) return fail(ADECO_ERR_LIMIT, "octree exceeds %zu nodes",
                                                                          kTreeMaxNodes);
        // children (x fastest), their boxes, and the chunks of the parents' lists
        chunks.clear();
        pfc.assign(1, 0);
        cbox.resize(refined.size() * 48);
        size_t pairs = 0;
        const size_t first_child = bfs.size();
        for (size_t k = 0; k < refined.size(); ++k) {
            const int pi = refined[k];
            const OctNode parent = bfs[pi].n;
            bfs[pi].n.first_child = (int32_t)(first_child + 8 * k);
            const float cext = (float)((double)parent.ext / 2.);
            for (int z = 0; z < 2; ++z)
                for (int y = 0; y < 2; ++y)
                    for (int x = 0; x < 2; ++x) {
                        BfsNode c;
                        c.n.min[0] = parent.min[0] + (float)x * cext;
                        c.n.min[1] = parent.min[1] + (float)y * cext;
                        c.n.min[2] = parent.min[2] + (float)z * cext;
                        c.n.ext = cext;
                        c.n.level = parent.level + 1;
                        c.n.parent = pi;
                        c.n.first_child = -1;
                        c.n.estimate = 0;
                        c.lv = lv + 1;
                        node_box(c.n, &cbox[k * 48 + 6 * (x + 2 * y + 4 * z)]);
                        bfs.push_back(c);
                    }
            levels = std::max(levels, parent.level + 2);
            const int len = bfs[pi].len;
            for (int s0 = 0; s0 < len; s0 += kTreeChunk) {
                TreeChunk t;
                t.parent = (int)k;
                t.start = bfs[pi].off + s0;
                t.len = std::min(kTreeChunk, len - s0);
                t.pad = 0;
                chunks.push_back(t);
            }
            pfc.push_back((int)chunks.size());
            pairs += (size_t)len;
        }
        const size_t nc = 8 * refined.size();
        const size_t cap = 8 * pairs;
        if (cap >= (1ull << 31)) return fail(ADECO_ERR_LIMIT, "octree level lists exceed 2^31 entries");
        lv_ids.emplace_back(new DevBuf<unsigned>());
        const int nch = (int)chunks.size();
        // byte offsets in the level block, each 16-byte aligned
        const auto up = [](size_t b) { return (b + 15) & ~(size_t)15; };
        const size_t o_est = 0, o_off = up(nc * sizeof(unsigned long long));
        const size_t o_chunks = up(o_off + (nc + 1) * sizeof(int));
        const size_t o_pfc = up(o_chunks + (size_t)nch * sizeof(TreeChunk));
        const size_t o_cbox = up(o_pfc + pfc.size() * sizeof(int));
        const size_t o_cnt = up(o_cbox + cbox.size() * sizeof(float));
        const size_t o_base = up(o_cnt + (size_t)nch * 8 * sizeof(int));
        const size_t bytes = up(o_base + (size_t)nch * 8 * sizeof(int));
        if ((rc = lv_ids[lv + 1]->reserve(cap))) return rc;
        if (bytes > d_lvl.n && (rc = d_lvl.reserve(std::max(bytes, 2 * d_lvl.n)))) return rc;
        h_lvl.resize(std::max(h_lvl.size(), bytes));
        std::memcpy(h_lvl.data() + o_chunks, chunks.data(), (size_t)nch * sizeof(TreeChunk));
        std::memcpy(h_lvl.data() + o_pfc, pfc.data(), pfc.size() * sizeof(int));
        std::memcpy(h_lvl.data() + o_cbox, cbox.data(), cbox.size() * sizeof(float));
        unsigned char *blk = d_lvl.p;
        unsigned long long *d_est = reinterpret_cast<unsigned long long *>(blk + o_est);
        int *d_off = reinterpret_cast<int *>(blk + o_off);
        const TreeChunk *d_chunks = reinterpret_cast<const TreeChunk *>(blk + o_chunks);
        const int *d_pfc = reinterpret_cast<const int *>(blk + o_pfc);
        const float *d_cbox = reinterpret_cast<const float *>(blk + o_cbox);
        int *d_cnt = reinterpret_cast<int *>(blk + o_cnt);
        int *d_base = reinterpret_cast<int *>(blk + o_base);
        CUDA_TRY(cudaMemcpyAsync(blk + o_chunks, h_lvl.data() + o_chunks, o_cnt - o_chunks, cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemsetAsync(d_est, 0, nc * sizeof(unsigned long long), st));
        tree_count_kernel<<<nch, kTreeThreads, 0, st>>>(d_mbb, lv_ids[lv]->p, d_chunks, d_cbox, d_cnt);
        CUDA_TRY(cudaGetLastError());
        tree_scan_kernel<<<1, 1024, 0, st>>>(d_chunks, nch, d_pfc, (int)refined.size(), d_cnt, d_base, d_off);
        CUDA_TRY(cudaGetLastError());
        tree_fill_kernel<<<nch, kTreeThreads, 0, st>>>(md, d_mbb, lv_ids[lv]->p, d_chunks, d_cbox, d_base,
                                                        lv_ids[lv + 1]->p, d_est);
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(cudaMemcpyAsync(h_lvl.data(), blk, o_chunks, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        for (size_t c = 0; c < nc; ++c) {
            BfsNode &b = bfs[first_child + c];
            unsigned long long e;
            int o0, o1;
            std::memcpy(&e, h_lvl.data() + o_est + c * sizeof e, sizeof e);
            std::memcpy(&o0, h_lvl.data() + o_off + c * sizeof(int), sizeof(int));
            std::memcpy(&o1, h_lvl.data() + o_off + (c + 1) * sizeof(int), sizeof(int));
            b.n.estimate = e;
            b.off = o0;
            b.len = o1 - o0;
        }
        lv_begin = first_child;
        lv_end = bfs.size();
    }

    // depth-first numbering of the stack walk (children pushed x fastest,
    // popped last first); a node's children get ids when it is popped
    std::vector<int> bfs_of(1, 0);
    tree.nodes.reserve(bfs.size());
    tree.nodes.push_back(bfs[0].n);
    tree.nodes[0].first_child = -1;
    std::vector<int32_t> stack(1, 0);
    while (!stack.empty()) {
        const int32_t cur = stack.back();
        stack.pop_back();
        const BfsNode &b = bfs[bfs_of[cur]];
        if (b.n.first_child < 0) continue;
        const int32_t first = (int32_t)tree.nodes.size();
        tree.nodes[cur].first_child = first;
        for (int q = 0; q < 8; ++q) {
            OctNode c = bfs[b.n.first_child + q].n;
            c.parent = cur;
            c.first_child = -1;
            tree.nodes.push_back(c);
            bfs_of.push_back(b.n.first_child + q);
        }
        for (int q = 0; q < 8; ++q) stack.push_back(first + q);
    }
    tree.levels = levels;
    // getLeafNodes order
    stack.assign(1, 0);
    while (!stack.empty()) {
        const int32_t cur = stack.back();
        stack.pop_back();
        if (tree.nodes[cur].first_child > 0) {
            for (int q = 0; q < 8; ++q) stack.push_back(tree.nodes[cur].first_child + q);
        } else {
            tree.leaves.push_back(cur);
        }
    }
    // leaf lists: bring the levels' id lists back once, then copy per leaf
    std::vector<std::vector<unsigned>> h_ids(lv_ids.size());
    std::vector<size_t> lv_len(lv_ids.size(), 0);
    for (const BfsNode &b : bfs) lv_len[b.lv] = std::max(lv_len[b.lv], (size_t)b.off + (size_t)b.len);
    for (size_t l = 0; l < lv_ids.size(); ++l) {
        h_ids[l].resize(lv_len[l]);
        if (lv_len[l])
            CUDA_TRY(cudaMemcpyAsync(h_ids[l].data(), lv_ids[l]->p, lv_len[l] * sizeof(unsigned), cudaMemcpyDeviceToHost,
                                     st));
    }
    CUDA_TRY(cudaStreamSynchronize(st));
    tree.leaf_meta_off.reserve(tree.leaves.size() + 1);
    size_t total = 0;
    for (int32_t l : tree.leaves) total += (size_t)bfs[bfs_of[l]].len;
    tree.leaf_meta_ids.reserve(total);
    int64_t off = 0;
    for (int32_t l : tree.leaves) {
        const BfsNode &b = bfs[bfs_of[l]];
        tree.leaf_meta_off.push_back(off);
        const unsigned *src = h_ids[b.lv].data() + b.off;
        tree.leaf_meta_ids.insert(tree.leaf_meta_ids.end(), src, src + b.len);
        off += b.len;
    }
    tree.leaf_meta_off.push_back(off);
    return ADECO_OK;
}

}  // namespace adeco
