// kernels.cuh -- the deposit kernels.
//
// Work decomposition: a deposit is a list of work items; an item pairs one
// output grid (a GridDesc: an octree leaf block, a zoom box, or the grid of a
// reference-boundary call) with one vertex block of at most 8^3 vertices
// (7^3 lattice cubes: a meta-cell of a resident lattice, or a sub-block of a
// reference-format patch).  A CTA stages the block's vertices in shared
// memory, culls its cubes against the grid box, and deposits the surviving
// tets with one warp per 32 tets: the tets' candidate (tet, cell) pairs are
// flattened across the warp, classified with per-tet plane bounds, easy
// cells are scattered at once and partial cells go through a per-warp
// shared-memory queue so that 32 lanes always clip together.
//
// Mass is accumulated as 64-bit fixed point (2^shift units per mass unit)
// with integer atomics: the sum is exact and independent of the order in
// which tets land, so results are bit-reproducible run to run and the same
// whether a request runs alone or inside a batch.
#pragma once

#include "clip_engine.cuh"
#include "geometry.cuh"

namespace adeco {

// 8 warps per CTA and 2 CTAs per SM (16 warps, <= 128 registers, 2 x ~115 KB
// of shared memory): the staged vertex block (20 KB) is shared by 8 warps
// instead of 4, which leaves room for a fourth warp per scheduler.  Against 3
// CTAs of 4 warps (12 warps per SM) this is 5.6% faster on a 208^3 lattice;
// 8 warps per SM is 11% slower.
constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kMaxVerts = 512;   // 8^3
constexpr int kMaxCubes = 343;   // 7^3
constexpr int kQueue = kPairs;  // partial pairs listed per warp before clipping

struct Item {
    long long base;  // vertex index of the block origin (lattice) or of the patch origin + offset
    int grid;        // GridDesc index
    int nv;          // vertex counts vx | vy<<8 | vz<<16 (each <= 8)
};

enum SrcKind : int { SRC_LATTICE_F4 = 0, SRC_PATCH_F3 = 1 };

struct DepositParams {
    const Item *items;
    int n_items;
    int src_kind;
    const GridDesc *grids;
    const void *src;
    long long stride_y, stride_z;     // vertex strides of the source
    int order;                        // ORDER_REF or ORDER_CONFORMING
    int pad_check;                    // skip cubes with a 666 vertex (patch inputs)
    unsigned long long *out;          // fixed-point accumulators (mixed path)
    double *out_d;                    // FP64 grids (plain path)
    int *counter;                     // persistent work counter
    unsigned long long *stats;        // kNumStats counters or nullptr
    int *error;                       // device error flag (bit 0: tet too large, bit 2: route list full,
                                      // bit 3: a work-sharing wait timed out)
    // ill-conditioned tets, deposited by a second launch (route_fp64_kernel):
    // entries item << 16 | (cube slot * 6 + tet), count in *route_count
    unsigned long long *route;
    unsigned long long *route_count;
    unsigned long long route_cap;
    // launch-shape and batching parameters (set by the host, tunable)
    int per_cta_items;   // items a CTA takes before it exits (0: persistent, until the queue is empty)
    int share_chunk;     // work sharing: candidate pairs per chunk (zoom grids)
    int clip_batch;      // partial pairs a warp lists before its engine clips them (64..kQueue)
    unsigned help_spins; // work sharing: sleeps a helper looks for open slots before leaving
    unsigned close_spins;  // work sharing: sleeps an owner waits for its helpers (then error bit 3)
};

enum Stat : int {
    ST_TETS = 0,         // tets with nonzero volume that meet the grid
    ST_CAND = 1,         // candidate pairs
    ST_BBOX = 2,         // pairs passing the AABB test
    ST_INSIDE = 3,       // TET_INSIDE_CELL pairs
    ST_CELLIN = 4,       // CELL_INSIDE_TET pairs
    ST_PARTIAL = 5,      // clipped pairs
    ST_FP64 = 6,         // pairs decided by the FP64 plane test
    ST_FALLBACK = 7,     // pieces clipped serially because the warp pool was full
    kNumStats = 8
};

// Per-warp table of up to 32 tets (structure of arrays in shared memory).
// Two CTAs of 8 warps fill an SM's shared memory to within a few hundred
// bytes, so the fields are as narrow as their ranges allow.
struct WarpTets {
    float q[12][32];     // vertices in the tet's anchor-cell frame (cell units), rounded
    float qlo[12][32];   // rounding remainders: q + qlo carries the vertex to ~44 bits
    float n[4][3][32];   // inward face normals
    float d[4][32];      // plane offsets n . (face centroid): inside <=> n.x - d > 0
    float dlo[4][32];    //   and their remainders (d + dlo: ~44 bits)
    float tol[32];       // FP32 error bound of the plane tests (largest face)
    float bmin[3][32];   // tet AABB in the anchor frame
    float bmax[3][32];
    float f6[32];        // mass per unit of 6x clipped volume (tet mass / |6V| in cell units)
    uint16_t lo[3][32];  // anchor cell (first candidate cell) in grid indices (dims <= 4096)
    uint16_t ex[3][32];  // candidate extents (cells per axis)
    int scan[33];        // exclusive prefix of candidate counts
};

// Tets whose conditioning kappa = (longest edge)^3 / |6V| exceeds this take
// the FP64 route: FP32 vertices in the cell frame carry ~2^-24 * kappa
// relative error into every cell fraction, so a flat tet (kappa >> 1) would
// miss the 1e-5 per-cell bar.  Lattice tets sit near kappa = 5.2.
constexpr float kKappaFp64 = 32.f;

// Work sharing inside an item: default pairs per chunk, and the default
// bounds of its waits (a helper looking for work gives up; an owner waiting
// for its helpers sets error bit 3 -- the value 8 -- and goes on).
constexpr int kChunk = 512;
constexpr unsigned kHelpSpins = 1u << 14;
constexpr unsigned kCloseSpins = 1u << 26;

// Waits, sleeping `ns` between looks, until *count is 0, at most `limit`
// looks; false if the limit ran out first.  Every spin-wait of the deposit
// kernels goes through here, so that none can wait forever.
__device__ __forceinline__ bool wait_zero_bounded(const int *count, unsigned limit, unsigned ns)
{
    for (unsigned spin = 0; *(volatile const int *)count != 0; ++spin) {
        if (spin >= limit) return false;
        __nanosleep(ns);
    }
    return true;
}

struct SharedMixed {
    float4 vert[kMaxVerts];
    float gh[3][kMaxVerts];   // grid-frame coordinates of the staged vertices, hi
    float gl[3][kMaxVerts];   //   and lo parts
    uint16_t cubes[kMaxCubes + 1];
    int n_cubes;
    int item;
    int next_group;
    GridDesc g;
    WarpTets wt[kWarps];
    uint32_t queue[kWarps][kQueue];
    WarpPool pool[kWarps];
    // work sharing inside an item: slot w = warp w's current group
    int slot_total[kWarps];  // its candidate pairs
    int slot_next[kWarps];   // first pair not yet taken
    int slot_busy[kWarps];   // helpers inside the slot
    int slot_open[kWarps];   // 1 while helpers may join
    int groups_set;  // groups of the item set up (published or kept private)
};

__device__ __forceinline__ void stat_add(unsigned long long *stats, int which, unsigned long long v)
{
    if (stats && v) atomicAdd(stats + which, v);
}

// warp-wide sum of a per-lane count, added once per warp
__device__ __forceinline__ void warp_stat(unsigned long long *stats, int which, unsigned v)
{
    if (!stats) return;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) stat_add(stats, which, v);
}

// ---------------------------------------------------------------- staging
__device__ __forceinline__ void stage_block(const DepositParams &P, const Item &it, float4 *vert, int vx, int vy,
                                            int vz, float (*gh)[kMaxVerts] = nullptr,
                                            float (*gl)[kMaxVerts] = nullptr)
{
    const GridDesc *gd = P.grids + it.grid;
    const int nvt = vx * vy * vz;
    for (int v = threadIdx.x; v < nvt; v += blockDim.x) {
        const int i = v % vx, r = v / vx, j = r % vy, k = r / vy;
        const long long gi = it.base + i + P.stride_y * j + P.stride_z * k;
        float4 p;
        if (P.src_kind == SRC_LATTICE_F4) {
            p = __ldg(reinterpret_cast<const float4 *>(P.src) + gi);
            p.w = 0.f;
        } else {
            const float *s = reinterpret_cast<const float *>(P.src) + 3 * gi;
            p = make_float4(__ldg(s), __ldg(s + 1), __ldg(s + 2), 0.f);
            if (P.pad_check) {
                // the reference's padding test on the float inputs
                const float sum = __fadd_rn(__fadd_rn(fabsf(__fsub_rn(p.x, 666.f)), fabsf(__fsub_rn(p.y, 666.f))),
                                            fabsf(__fsub_rn(p.z, 666.f)));
                if ((double)sum < 1.E-03) p.w = 1.f;
            }
        }
        vert[v] = p;
        if (gh) {
            grid_frame(p.x, __ldg(&gd->gmin[0]), __ldg(&gd->scale_hi[0]), __ldg(&gd->scale_lo[0]), gh[0][v], gl[0][v]);
            grid_frame(p.y, __ldg(&gd->gmin[1]), __ldg(&gd->scale_hi[1]), __ldg(&gd->scale_lo[1]), gh[1][v], gl[1][v]);
            grid_frame(p.z, __ldg(&gd->gmin[2]), __ldg(&gd->scale_hi[2]), __ldg(&gd->scale_lo[2]), gh[2][v], gl[2][v]);
        }
    }
}

// cube (ci,cj,ck) of the staged block: alive if no padding vertex and its AABB
// strictly overlaps the grid box
__device__ __forceinline__ bool cube_alive(const float4 *vert, int vx, int vy, int ci, int cj, int ck,
                                           const GridDesc &g)
{
    float mn[3] = {3.4e38f, 3.4e38f, 3.4e38f}, mx[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
    bool pad = false;
#pragma unroll
    for (int s = 0; s < 8; ++s) {
        const float4 p = vert[(ci + (s & 1)) + vx * ((cj + ((s >> 1) & 1)) + vy * (ck + (s >> 2)))];
        pad |= (p.w != 0.f);
        mn[0] = fminf(mn[0], p.x); mx[0] = fmaxf(mx[0], p.x);
        mn[1] = fminf(mn[1], p.y); mx[1] = fmaxf(mx[1], p.y);
        mn[2] = fminf(mn[2], p.z); mx[2] = fmaxf(mx[2], p.z);
    }
    if (pad) return false;
#pragma unroll
    for (int a = 0; a < 3; ++a)
        if (!(mn[a] < g.cull_max[a] && g.cull_min[a] < mx[a])) return false;
    return true;
}

__device__ __forceinline__ void load_tet(const float4 *vert, int vx, int vy, int cube_local_idx, int t, int order,
                                         int cvx, int cvy, float3 v[4], int *vid = nullptr)
{
    const int ci = cube_local_idx % cvx, r = cube_local_idx / cvx, cj = r % cvy, ck = r / cvy;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int3 o = corner_offset(order, tet_conn(t, q));
        const int id = (ci + o.x) + vx * ((cj + o.y) + vy * (ck + o.z));
        const float4 p = vert[id];
        v[q] = make_float3(p.x, p.y, p.z);
        if (vid) vid[q] = id;
    }
}

// ------------------------------------------------------ per-tet set-up
// Build one tet (bit-exact orientation rule and candidate range), then its
// FP64 anchor-frame geometry, rounded once to FP32.  Returns the candidate
// pair count (0 if the tet is skipped).
// Candidate pairs of one tet are limited to kMaxPairsPerTet so that the
// per-warp flattened pair index fits 32 bits and a queue entry (5-bit slot,
// 27-bit local index); a larger tet sets the error flag and is skipped.
constexpr long long kMaxPairsPerTet = 1LL << 25;

// Offset of a tet face's plane n . x = d through the face's centroid, from
// its vertices as FP32 pairs (hi + lo) and the FP32 normal n: 3 d = n . (va
// + vb + vc) in double-float, divided by 3 as a product with 1/3 whose
// remainder (exact, fma) is carried into the low part, so that d_hi + d_lo
// keeps ~44 bits.
ADECO_HD inline F2 plane_offset(const float qa[3], const float la[3], const float qb[3], const float lb[3],
                                const float qc[3], const float lc[3], const float n[3])
{
    F2 dd = {0.f, 0.f};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const F2 sum = f2_add(f2_add(F2{qa[a], la[a]}, F2{qb[a], lb[a]}), F2{qc[a], lc[a]});
        dd = f2_add(dd, f2_mul_f(sum, n[a]));
    }
    constexpr float kThird = 1.f / 3.f;
    const float d_hi = dd.hi * kThird;
    return {d_hi, (fmaf(-d_hi, 3.f, dd.hi) + dd.lo) * kThird};
}

// kExactD: store each face's exact plane offset (d, dlo: the one-face closed
// form reads them).  Otherwise only an FP32 d for the classification, whose
// error band covers its rounding; the closed form then forms the exact
// offset itself (plane_offset from the stored vertices) for the few pairs
// that take it.  Octree leaves at the benchmark's cell sizes send almost no
// pair to the closed form, and the double-float offsets had been ~40% of the
// set-up; zoom grids, fine against the tets, send many.
template <bool kExactD = true>
ADECO_HD inline int setup_tet(const float3 vin[4], const float ghin[4][3], const float glin[4][3], const GridDesc &g,
                              WarpTets &W, int lane, int *error, bool *fp64_route)
{
    *fp64_route = false;
    float3 v[4] = {vin[0], vin[1], vin[2], vin[3]};
    const float v6 = vol6_exact(v[0], v[1], v[2], v[3]);
    const int sgn = vol6_sign_ref(v6);
    int lo[3], hi[3];
    if (!candidate_range(v, g, lo, hi)) return 0;
    if (sgn == 0) return 0;
    if (!tile_clamp(g, lo, hi)) return 0;
    {
        const long long cnt0 = (long long)(hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1);
        if (cnt0 > kMaxPairsPerTet) {
#ifdef __CUDA_ARCH__
            if (error) atomicOr(error, 1);
#else
            if (error) *error |= 1;
#endif
            return 0;
        }
    }
    // orientation rule on the vertex order: swap 0 <-> 3 when negative
    const bool swap03 = sgn < 0;  // selects, not an index: an indexed vertex array would live in local memory
    // Tight range: of the candidate cells [lo, hi], only those whose box
    // [c r, c r + 1] (grid frame) meets the tet's AABB can receive mass (the
    // rest fail the AABB test).  Bounds widened by the FP32 rounding of the
    // grid-frame coordinates; the frame is then anchored at the first cell.
    float qf[4][3], ql[4][3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float g0 = ghin[0][a], g1 = ghin[1][a], g2 = ghin[2][a], g3 = ghin[3][a];
        const float bmn = fminf(fminf(g0, g1), fminf(g2, g3)), bmx = fmaxf(fmaxf(g0, g1), fmaxf(g2, g3));
        const float ir = g.inv_rcell_f[a];
        const float m0 = 4e-7f * (fabsf(bmn) + 2.f), m1 = 4e-7f * (fabsf(bmx) + 2.f);
        const int c0 = max(lo[a], (int)floorf((bmn - 1.f) * ir - m0) + 1);
        const int c1 = min(hi[a], (int)ceilf(bmx * ir + m1) - 1);
        if (c1 < c0) return 0;
        lo[a] = c0;
        hi[a] = c1;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int src = (q == 0) ? 0 : ((q == 3) ? 3 : q);  // the vertex before the orientation swap
            const float h = (q == 0 || q == 3) ? (swap03 ? ghin[3 - src][a] : ghin[src][a]) : ghin[q][a];
            const float l = (q == 0 || q == 3) ? (swap03 ? glin[3 - src][a] : glin[src][a]) : glin[q][a];
            shift_frame(h, l, c0, g.drcell[a], qf[q][a], ql[q][a]);
        }
    }
    // |6 V| in the anchor frame from the FP32 pairs, in double-float (the
    // tet's volume normaliser): edge vectors from vertex 3, then the triple
    // product with TwoProd / TwoSum
    F2 e[3][3];
#pragma unroll
    for (int q = 0; q < 3; ++q)
#pragma unroll
        for (int a = 0; a < 3; ++a) e[q][a] = f2_add(F2{qf[q][a], ql[q][a]}, F2{-qf[3][a], -ql[3][a]});
    const F2 cx = f2_add(f2_mul(e[1][1], e[2][2]), f2_neg(f2_mul(e[1][2], e[2][1])));
    const F2 cy = f2_add(f2_mul(e[1][2], e[2][0]), f2_neg(f2_mul(e[1][0], e[2][2])));
    const F2 cz = f2_add(f2_mul(e[1][0], e[2][1]), f2_neg(f2_mul(e[1][1], e[2][0])));
    F2 w6 = f2_add(f2_add(f2_mul(e[0][0], cx), f2_mul(e[0][1], cy)), f2_mul(e[0][2], cz));
    if (w6.hi < 0.f) w6 = f2_neg(w6);
    const float vq6 = w6.hi;
    const float f6 = f2_div_to_f(F2{g.mf_hi, g.mf_lo}, w6);  // mass per unit of 6x volume
    // planes from the FP32 vertices: inward normals (outward ones negated:
    // faces (0,1,2) (0,2,3) (0,3,1) (1,3,2)); each plane's offset is taken
    // through the face's centroid, so that the FP32 rounding of the normal
    // only turns the plane about the centroid (the one-face closed form
    // relies on it)
    const int fa[4] = {0, 0, 0, 1}, fb[4] = {2, 3, 1, 2}, fc[4] = {1, 2, 3, 3};
    float R = 0.f;
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int a = 0; a < 3; ++a) R = fmaxf(R, fabsf(qf[q][a]));
    R = fmaxf(R, (float)max(max(hi[0] - lo[0], hi[1] - lo[1]), hi[2] - lo[2]) + 1.f);
    float tolmax = 0.f;
#pragma unroll
    for (int f = 0; f < 4; ++f) {
        // n_in = (vb - va) x (vc - va) with the outward order reversed
        const float e1x = qf[fb[f]][0] - qf[fa[f]][0], e1y = qf[fb[f]][1] - qf[fa[f]][1],
                    e1z = qf[fb[f]][2] - qf[fa[f]][2];
        const float e2x = qf[fc[f]][0] - qf[fa[f]][0], e2y = qf[fc[f]][1] - qf[fa[f]][1],
                    e2z = qf[fc[f]][2] - qf[fa[f]][2];
        const float nx = e1y * e2z - e1z * e2y, ny = e1z * e2x - e1x * e2z, nz = e1x * e2y - e1y * e2x;
        const float nn[3] = {nx, ny, nz};
        W.n[f][0][lane] = nx;
        W.n[f][1][lane] = ny;
        W.n[f][2][lane] = nz;
        if (kExactD) {
            const F2 d = plane_offset(qf[fa[f]], ql[fa[f]], qf[fb[f]], ql[fb[f]], qf[fc[f]], ql[fc[f]], nn);
            W.d[f][lane] = d.hi;
            W.dlo[f][lane] = d.lo;
        } else {
            constexpr float kThird = 1.f / 3.f;
            W.d[f][lane] = (nx * (qf[fa[f]][0] + qf[fb[f]][0] + qf[fc[f]][0]) +
                            ny * (qf[fa[f]][1] + qf[fb[f]][1] + qf[fc[f]][1]) +
                            nz * (qf[fa[f]][2] + qf[fb[f]][2] + qf[fc[f]][2])) * kThird;
        }
        const float L1 = fmaxf(fmaxf(fabsf(e1x), fabsf(e1y)), fabsf(e1z));
        const float L2 = fmaxf(fmaxf(fabsf(e2x), fabsf(e2y)), fabsf(e2z));
        // generous bound on the FP32 rounding of n.x - d (|x| <= R + 1)
        tolmax = fmaxf(tolmax, 1.0e-5f * L1 * L2 * (R + 1.f));
    }
    W.tol[lane] = tolmax;
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            W.q[3 * q + a][lane] = qf[q][a];
            W.qlo[3 * q + a][lane] = ql[q][a];
        }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        W.bmin[a][lane] = fminf(fminf(qf[0][a], qf[1][a]), fminf(qf[2][a], qf[3][a]));
        W.bmax[a][lane] = fmaxf(fmaxf(qf[0][a], qf[1][a]), fmaxf(qf[2][a], qf[3][a]));
        W.lo[a][lane] = (uint16_t)lo[a];
        W.ex[a][lane] = (uint16_t)(hi[a] - lo[a] + 1);
    }
    W.f6[lane] = f6;
    // conditioning: longest edge cubed over |6V|, both in cell units
    float L2 = 0.f;
#pragma unroll
    for (int a0 = 0; a0 < 4; ++a0)
#pragma unroll
        for (int b0 = a0 + 1; b0 < 4; ++b0) {
            const float dx = qf[a0][0] - qf[b0][0], dy = qf[a0][1] - qf[b0][1], dz = qf[a0][2] - qf[b0][2];
            L2 = fmaxf(L2, dx * dx + dy * dy + dz * dz);
        }
    // L^3 <= kappa |6V| squared (both sides non-negative): no square root;
    // NaN or an overflow routes the tet
    *fp64_route = !(L2 * L2 * L2 <= (kKappaFp64 * kKappaFp64) * (vq6 * vq6));
    return (hi[0] - lo[0] + 1) * (hi[1] - lo[1] + 1) * (hi[2] - lo[2] + 1);
}

enum PairClass : int { P_NO = 0, P_TET_INSIDE = 1, P_CELL_INSIDE = 2, P_PARTIAL = 3 };

#ifdef __CUDACC__
// One positively oriented tet, candidate range [lo, hi], deposited by the
// whole warp in FP64 (the plain baseline): lanes stride over the candidate
// cells, each classified with FP64 face planes and, when partial, clipped in
// FP64; FP64 atomics.  Counts the (candidate, partial) pairs seen by this lane.
__device__ __noinline__ void deposit_tet_fp64_warp(const float3 v[4], const int lo[3], const int hi[3], const GridDesc &g,
                                                   double *out_d, unsigned &n_cand, unsigned &n_part)
{
    const int lane = threadIdx.x & 31;
    double qd[4][3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double anchor = fma((double)lo[a], g.delta_d[a], g.gmin_d[a]);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const double x = (a == 0) ? (double)v[q].x : ((a == 1) ? (double)v[q].y : (double)v[q].z);
            qd[q][a] = (x - anchor) * g.scale_d[a];
        }
    }
    const double vq6 = fabs(vol6_fast<double>(qd[0], qd[1], qd[2], qd[3]));
    const double f6 = g.mass_factor / vq6;
    double bmin[3], bmax[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        bmin[a] = fmin(fmin(qd[0][a], qd[1][a]), fmin(qd[2][a], qd[3][a]));
        bmax[a] = fmax(fmax(qd[0][a], qd[1][a]), fmax(qd[2][a], qd[3][a]));
    }
    // inward face planes: faces (0,2,1) (0,3,2) (0,1,3) (1,2,3)
    double pn[4][3], pd[4], pp[4], pm[4];
    {
        const int fa[4] = {0, 0, 0, 1}, fb[4] = {2, 3, 1, 2}, fc[4] = {1, 2, 3, 3};
#pragma unroll
        for (int f = 0; f < 4; ++f) {
            const double e1x = qd[fb[f]][0] - qd[fa[f]][0], e1y = qd[fb[f]][1] - qd[fa[f]][1],
                         e1z = qd[fb[f]][2] - qd[fa[f]][2];
            const double e2x = qd[fc[f]][0] - qd[fa[f]][0], e2y = qd[fc[f]][1] - qd[fa[f]][1],
                         e2z = qd[fc[f]][2] - qd[fa[f]][2];
            pn[f][0] = e1y * e2z - e1z * e2y;
            pn[f][1] = e1z * e2x - e1x * e2z;
            pn[f][2] = e1x * e2y - e1y * e2x;
            pd[f] = pn[f][0] * qd[fa[f]][0] + pn[f][1] * qd[fa[f]][1] + pn[f][2] * qd[fa[f]][2];
            pp[f] = fmax(pn[f][0], 0.0) + fmax(pn[f][1], 0.0) + fmax(pn[f][2], 0.0);
            pm[f] = fmin(pn[f][0], 0.0) + fmin(pn[f][1], 0.0) + fmin(pn[f][2], 0.0);
        }
    }
    const int ex0 = hi[0] - lo[0] + 1, ex1 = hi[1] - lo[1] + 1, ex2 = hi[2] - lo[2] + 1;
    auto put = [&](long long idx, double dm) { atomicAdd(out_d + idx, dm); };
    // one cell, decided exactly in FP64 (bbox, plane bounds, clipping)
    auto cell = [&](int a, int b, int k) {
        ++n_cand;
        // cell origin in the anchor frame (the cell extends 1 along each axis)
        const double oa = a * g.rcell[0], ob = b * g.rcell[1], ok = k * g.rcell[2];
        if (!(bmin[0] < oa + 1.0 && oa < bmax[0] && bmin[1] < ob + 1.0 && ob < bmax[1] && bmin[2] < ok + 1.0 &&
              ok < bmax[2]))
            return;
        bool outside = false, all_in = true;
#pragma unroll
        for (int f = 0; f < 4; ++f) {
            const double base = pn[f][0] * oa + pn[f][1] * ob + pn[f][2] * ok - pd[f];
            if (base + pp[f] <= 0.0) outside = true;
            if (!(base + pm[f] > 0.0)) all_in = false;
        }
        if (outside) return;
        double dm;
        if (bmin[0] >= oa && bmax[0] <= oa + 1.0 && bmin[1] >= ob && bmax[1] <= ob + 1.0 && bmin[2] >= ok &&
            bmax[2] <= ok + 1.0) {
            dm = (double)g.tet_mass;
        } else if (all_in) {
            dm = 6.0 * f6;
        } else {
            double p[4][3];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                p[q][0] = qd[q][0] - oa;
                p[q][1] = qd[q][1] - ob;
                p[q][2] = qd[q][2] - ok;
            }
            ++n_part;
            dm = clip_volume6<double, double>(p) * f6;
        }
        if (!(dm > 0.0)) return;
        put(g.out_offset + (lo[0] + a) + (long long)g.dims * ((lo[1] + b) + (long long)g.dims * (lo[2] + k)), dm);
    };
    if (ex0 < 8) {  // short rows: one lane per cell
        const long long ncell = (long long)ex0 * ex1 * ex2;
        for (long long cc = lane; cc < ncell; cc += 32) {
            const long long rr = cc / ex0;
            cell((int)(cc % ex0), (int)(rr % ex1), (int)(rr / ex1));
        }
        return;
    }
    // Long rows along x, one per lane.  The plane bounds are linear in the
    // cell index a, so each plane bounds a; widened / narrowed by a cell
    // against rounding, cells outside [c0, c1] cannot meet the tet and cells
    // inside [i0, i1] lie inside it (CELL_INSIDE_TET: the mass the per-cell
    // test gives them); only the cells in between are tested one by one.
    const long long nrows = (long long)ex1 * ex2;
    for (long long rr = lane; rr < nrows; rr += 32) {
        const int b = (int)(rr % ex1), k = (int)(rr / ex1);
        const double ob = b * g.rcell[1], ok = k * g.rcell[2];
        double c0 = 0.0, c1 = ex0 - 1, i0 = 0.0, i1 = ex0 - 1;
        bool none = false, no_in = false;
#pragma unroll
        for (int f = 0; f < 4; ++f) {
            const double nx = pn[f][0] * g.rcell[0];
            const double K = pn[f][1] * ob + pn[f][2] * ok - pd[f];
            if (nx > 0.0) {
                c0 = fmax(c0, floor(-(K + pp[f]) / nx) - 1.0);
                i0 = fmax(i0, floor(-(K + pm[f]) / nx) + 2.0);
            } else if (nx < 0.0) {
                c1 = fmin(c1, ceil(-(K + pp[f]) / nx) + 1.0);
                i1 = fmin(i1, ceil(-(K + pm[f]) / nx) - 2.0);
            } else {
                none = none || !(K + pp[f] > 0.0);
                no_in = no_in || !(K + pm[f] > 0.0);
            }
        }
        if (none) continue;
        const int lc = (int)fmax(c0, 0.0), hc = (int)fmin(c1, (double)(ex0 - 1));
        int li = (int)fmax(i0, (double)lc), hi_ = (int)fmin(i1, (double)hc);
        if (no_in || li > hi_) {
            li = hc + 1;
            hi_ = hc;
        }
        for (int a = lc; a < li; ++a) cell(a, b, k);
        if (li <= hi_) {
            n_cand += hi_ - li + 1;
            const long long row =
                g.out_offset + lo[0] + (long long)g.dims * ((lo[1] + b) + (long long)g.dims * (lo[2] + k));
            for (int a = li; a <= hi_; ++a) put(row + a, 6.0 * f6);
        }
        for (int a = hi_ + 1; a <= hc; ++a) cell(a, b, k);
    }
}
#endif

// FP64 evaluation of the four plane bounds for a cell whose FP32 test was
// inside the error band: exact decision for the FP32-rounded tet.
ADECO_HD
#ifdef __CUDA_ARCH__
__noinline__
#endif
int classify_fp64(const WarpTets &W, const GridDesc &g, int s, int a, int b, int c)
{
    const double ca = a * g.rcell[0], cb = b * g.rcell[1], cc = c * g.rcell[2];
    double q[4][3];
#pragma unroll
    for (int v = 0; v < 4; ++v)
#pragma unroll
        for (int x = 0; x < 3; ++x) q[v][x] = (double)W.q[3 * v + x][s] + (double)W.qlo[3 * v + x][s];
    const int fa[4] = {0, 0, 0, 1}, fb[4] = {2, 3, 1, 2}, fc[4] = {1, 2, 3, 3};
    bool all_in = true;
    for (int f = 0; f < 4; ++f) {
        const double e1x = q[fb[f]][0] - q[fa[f]][0], e1y = q[fb[f]][1] - q[fa[f]][1], e1z = q[fb[f]][2] - q[fa[f]][2];
        const double e2x = q[fc[f]][0] - q[fa[f]][0], e2y = q[fc[f]][1] - q[fa[f]][1], e2z = q[fc[f]][2] - q[fa[f]][2];
        const double nx = e1y * e2z - e1z * e2y, ny = e1z * e2x - e1x * e2z, nz = e1x * e2y - e1y * e2x;
        const double base = nx * (ca - q[fa[f]][0]) + ny * (cb - q[fa[f]][1]) + nz * (cc - q[fa[f]][2]);
        const double mx = base + fmax(nx, 0.0) + fmax(ny, 0.0) + fmax(nz, 0.0);
        const double mn = base + fmin(nx, 0.0) + fmin(ny, 0.0) + fmin(nz, 0.0);
        if (mx <= 0.0) return P_NO;
        all_in = all_in && (mn > 0.0);
    }
    return all_in ? P_CELL_INSIDE : P_PARTIAL;
}

// cross: the one tet face plane the cell straddles when the cell is certainly
// inside the other three (then cell ∩ tet = cell ∩ that face's half-space),
// else -1.
ADECO_HD inline int classify_pair(const WarpTets &W, const GridDesc &g, int s, int a, int b, int c, bool &used_fp64,
                                  int &cross)
{
    cross = -1;
    const float fa = (float)a, fb = (float)b, fc = (float)c;
    // strict AABB overlap with the cell [a,a+1] x [b,b+1] x [c,c+1]
    if (!(W.bmin[0][s] < fa + 1.f && fa < W.bmax[0][s] && W.bmin[1][s] < fb + 1.f && fb < W.bmax[1][s] &&
          W.bmin[2][s] < fc + 1.f && fc < W.bmax[2][s]))
        return P_NO;
    if (W.bmin[0][s] >= fa && W.bmax[0][s] <= fa + 1.f && W.bmin[1][s] >= fb && W.bmax[1][s] <= fb + 1.f &&
        W.bmin[2][s] >= fc && W.bmax[2][s] <= fc + 1.f)
        return P_TET_INSIDE;
    bool all_in = true, unsure = false;
    int ncross = 0, fcross = 0;
    const float t = W.tol[s];
#pragma unroll
    for (int f = 0; f < 4; ++f) {
        const float nx = W.n[f][0][s], ny = W.n[f][1][s], nz = W.n[f][2][s];
        const float base = fmaf(nx, fa, fmaf(ny, fb, fmaf(nz, fc, -W.d[f][s])));
        const float pos = fmaxf(nx, 0.f) + fmaxf(ny, 0.f) + fmaxf(nz, 0.f);
        const float mx = base + pos;
        const float mn = base + ((nx + ny + nz) - pos);
        if (mx < -t) return P_NO;
        if (mx <= t) unsure = true;
        if (mn > t) continue;
        all_in = false;
        ++ncross;
        fcross = f;
        if (mn > -t) unsure = true;
    }
    if (unsure) {
        used_fp64 = true;
        return classify_fp64(W, g, s, a, b, c);
    }
    if (ncross == 1) cross = fcross;
    return all_in ? P_CELL_INSIDE : P_PARTIAL;
}

// Value at the origin of cell (a, b, c) of face f's linear function G(u) =
// n . (cell origin + u - centroid), taken about the face's centroid so that
// the FP32 rounding of its normal only turns the plane about the centroid:
// the volume a slightly turned plane adds on one side of the centroid it
// removes on the other, and the tet's mass stays conserved over its cells.
// n . origin - (d + dlo) cancels terms as large as the tet is wide in cells:
// it is formed exactly in double-float (TwoProd of n with the integer cell
// offsets) and kept as a pair for the corner values.
template <bool kExactD = true>
ADECO_HD inline F2 face_value_at_cell(const WarpTets &W, const GridDesc &g, int s, int a, int b, int c, int f)
{
    const int cc[3] = {a, b, c};
    F2 G;
    if (kExactD) {
        G = {-W.d[f][s], -W.dlo[f][s]};
    } else {  // the exact offset setup_tet<true> would have stored
        const int fa = f == 3 ? 1 : 0, fb = f == 0 ? 2 : (f == 1 ? 3 : (f == 2 ? 1 : 2)),
                  fc = f == 0 ? 1 : (f == 1 ? 2 : 3);
        float q[3][3], l[3][3];
#pragma unroll
        for (int x = 0; x < 3; ++x) {
            q[0][x] = W.q[3 * fa + x][s];
            l[0][x] = W.qlo[3 * fa + x][s];
            q[1][x] = W.q[3 * fb + x][s];
            l[1][x] = W.qlo[3 * fb + x][s];
            q[2][x] = W.q[3 * fc + x][s];
            l[2][x] = W.qlo[3 * fc + x][s];
        }
        const float n[3] = {W.n[f][0][s], W.n[f][1][s], W.n[f][2][s]};
        const F2 d = plane_offset(q[0], l[0], q[1], l[1], q[2], l[2], n);
        G = {-d.hi, -d.lo};
    }
    float small = 0.f;  // the cells' deviation from unit size: n_x c_x dr_x, tiny
#pragma unroll
    for (int x = 0; x < 3; ++x) {
        const float nx = W.n[f][x][s], fc = (float)cc[x];
        G = f2_add(G, f2_two_prod(nx, fc));
        small = fmaf(nx * fc, g.drcell[x], small);
    }
    return f2_norm(G.hi, G.lo + small);
}

// 6x volume of cell (a, b, c) ∩ slot s's tet when the cell straddles only
// face f: the cube's part on its inside.
template <bool kExactD = true>
#ifdef __CUDA_ARCH__
__device__ __noinline__
#else
inline
#endif
float halfspace_pair_vol6(const WarpTets &W, const GridDesc &g, int s, int a, int b, int c, int f)
{
    return halfspace_cube_vol6(face_value_at_cell<kExactD>(W, g, s, a, b, c, f), W.n[f][0][s], W.n[f][1][s],
                               W.n[f][2][s]);
}

// Non-negative mass of a pair (FP32, about 1e-7 relative) -> the cell's
// 64-bit fixed-point accumulator, with integer operations only.  Inlined: as
// a call it made the pair loop save and restore its live registers in local
// memory around every scatter (C2: 16% of the kernel time).
__device__ __forceinline__ void scatter(const DepositParams &P, const GridDesc &g, const WarpTets &W, int s, int a,
                                        int b, int c, float m)
{
    const unsigned long long fx = to_fixed(m, g.shift);
    if (fx == 0ull) return;
    const long long i = W.lo[0][s] + a, j = W.lo[1][s] + b, k = W.lo[2][s] + c;
    const long long idx = g.out_offset + i + (long long)g.dims * (j + (long long)g.dims * k);
    atomicAdd(P.out + idx, fx);
}

// A pair's 6x volume, summed in fixed point 2^kVolShift (0 <= vacc < 2^59),
// times the tet's mass per unit of 6x volume.  The sum is converted to FP32
// with one rounding from two exact 24-bit parts (bits 35..58 and 11..34): the
// fma rounds their exact sum to nearest.  Rounding the upper part alone would
// drop the lower bits first -- a truncation, a bias of -6e-9 relative that
// showed in the total mass.  Bits 0..10 (below 3e-14 of a tet's 6x volume)
// are left out.
ADECO_HD inline float pair_mass(long long vacc, float f6)
{
    const float hi = (float)(int)(vacc >> 35), mid = (float)(int)((vacc >> 11) & 0xffffff);
    const float v = fmaf(hi, 0x1p35f, mid * 0x1p11f);
    return v * (f6 * 0x1p-56f);
}

// Tet of slot s in the frame of its candidate cell (a, b, c), as the clip
// engine takes it.  Along an axis whose lower face the tet does not reach,
// the cell's mirrored frame is used, so that the face it crosses lies at 0:
// a thin slice under the upper face otherwise lost ~6e-8 cell units per
// vertex (up to 5e-5 of such a cell's mass on a 256^3 lattice; 5e-7
// mirrored).  An odd number of reflections is undone by swapping vertices 0
// and 1 (the engine wants a positively oriented tet).
ADECO_HD inline void piece_coords(const WarpTets &W, const GridDesc &g, int s, int a, int b, int c, float p[12])
{
    const int cc[3] = {a, b, c};
    int nflip = 0;
#pragma unroll
    for (int x = 0; x < 3; ++x) {
        const bool flip = W.bmin[x][s] > (float)cc[x];
        nflip += flip;
#pragma unroll
        for (int v = 0; v < 4; ++v)
            p[3 * v + x] = cell_coord_fast(W.q[3 * v + x][s], W.qlo[3 * v + x][s], cc[x], g.drcell[x], flip);
    }
    if (nflip & 1) {
#pragma unroll
        for (int x = 0; x < 3; ++x) {
            const float t = p[x];
            p[x] = p[3 + x];
            p[3 + x] = t;
        }
    }
}

#ifdef __CUDACC__
// piece of pair `entry` (slot << 27 | local pair index) in its cell's frame
__device__ __forceinline__ void pair_piece(const GridDesc &g, const WarpTets &W, uint32_t entry, float p[12], int &s,
                                           int &a, int &b, int &c)
{
    s = entry >> 27;
    const int local = entry & ((1u << 27) - 1);
    const int ex0 = W.ex[0][s], ex1 = W.ex[1][s];
    a = local % ex0;
    const int r = local / ex0;
    b = r % ex1;
    c = r / ex1;
    piece_coords(W, g, s, a, b, c, p);
}
#endif

// clip the warp's listed partial pairs Q[0..np), then scatter them
__device__ __forceinline__ void clip_list(const DepositParams &P, const GridDesc &g, const WarpTets &W,
                                          WarpPool &pool, const uint32_t *Q, int np, unsigned &fallbacks)
{
    clip_pairs(
        pool, np,
        [&](int j, float *p) {
            int s, a, b, c;
            pair_piece(g, W, Q[j], p, s, a, b, c);
        },
        fallbacks);
    for (int j = threadIdx.x & 31; j < np; j += 32) {
        const uint32_t e = Q[j];
        const int s = e >> 27;
        const int local = e & ((1u << 27) - 1);
        const int ex0 = W.ex[0][s], ex1 = W.ex[1][s];
        const int a = local % ex0, r = local / ex0, b = r % ex1, c = r / ex1;
        const long long v = pool.vacc[j];
        if (v > 0) scatter(P, g, W, s, a, b, c, pair_mass(v, W.f6[s]));
    }
    __syncwarp();
}

// -------------------------------------------------- mixed batched kernel
// per-thread pair counters
struct PairStats {
    unsigned tets = 0, cand = 0, bbox = 0, in = 0, cin = 0, part = 0, fp64 = 0, fb = 0;
};

// Sets up group grp (tets 32 grp .. 32 grp + 31 of the item's live cubes) in
// the warp's table W and returns its candidate pairs.  route64: this lane's
// tet is ill-conditioned (listed by group_route, no pairs here).
template <bool kShare>
__device__ __forceinline__ int group_setup(const DepositParams &P, const SharedMixed &S, WarpTets &W,
                                           const GridDesc &g, int grp, int ntet, int vx, int vy, int cvx, int cvy,
                                           int lane, PairStats &st, bool &route64, int &tid)
{
    tid = grp * 32 + lane;
    int cnt = 0;
    route64 = false;
    if (tid < ntet) {
        float3 v[4];
        int vid[4];
        load_tet(S.vert, vx, vy, S.cubes[tid / 6], tid % 6, P.order, cvx, cvy, v, vid);
        float gh[4][3], gl[4][3];
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                gh[q][a] = S.gh[a][vid[q]];
                gl[q][a] = S.gl[a][vid[q]];
            }
        cnt = setup_tet<kShare>(v, gh, gl, g, W, lane, P.error, &route64);
    }
    st.tets += (cnt > 0);
    route64 = route64 && cnt > 0;
    if (route64) cnt = 0;  // deposited by route_fp64_kernel
    // exclusive scan of the pair counts across the warp
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    W.scan[lane] = incl - cnt;
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    if (lane == 31) W.scan[32] = total;
    __syncwarp();
    return total;
}

// Ill-conditioned tets are listed for route_fp64_kernel: calling their
// (large) routine from the pair loop made the whole loop spill.
__device__ __forceinline__ void group_route(const DepositParams &P, const SharedMixed &S, int item, bool route64,
                                            int tid)
{
    if (route64) {
        const unsigned long long k = atomicAdd(P.route_count, 1ull);
        if (k < P.route_cap)
            P.route[k] = ((unsigned long long)item << 16) | (unsigned long long)(S.cubes[tid / 6] * 6 + tid % 6);
        else
            atomicOr(P.error, 4);
    }
}

// Candidate pairs [c0, c1) of the group in table Wc, flattened across the
// warp: classified, inside cells and one-face cells deposited at once,
// partial cells listed in Q and clipped by the engine (one call site keeps a
// single copy of it).
template <bool kShare>
__device__ __forceinline__ void pair_range(const DepositParams &P, const GridDesc &g, const WarpTets &Wc,
                                           WarpPool &pool, uint32_t *Q, int c0, int c1, int lane, PairStats &st)
{
    int np = 0;  // partial pairs listed in Q
    // clip once more than `flush` pairs are listed (then np + 32 <= kQueue)
    const int flush = min(max(P.clip_batch, 64), kQueue) - 32;
    for (int pb = c0;; pb += 32) {
        if (np > flush || (pb >= c1 && np)) {
            clip_list(P, g, Wc, pool, Q, np, st.fb);
            np = 0;
        }
        if (pb >= c1) break;
        const int pidx = pb + lane;
        bool part = false;
        uint32_t entry = 0;
        if (pidx < c1) {
            int s = 0;
#pragma unroll
            for (int step = 16; step > 0; step >>= 1)
                if (Wc.scan[s + step] <= pidx) s += step;
            const int local = pidx - Wc.scan[s];
            const int ex0 = Wc.ex[0][s], ex1 = Wc.ex[1][s];
            const int a = local % ex0, r = local / ex0, b = r % ex1, c = r / ex1;
            ++st.cand;
            bool f64 = false;
            int cross = -1;
            const int cls = classify_pair(Wc, g, s, a, b, c, f64, cross);
            st.fp64 += f64;
            if (cls == P_TET_INSIDE) {
                ++st.in;
                ++st.bbox;
                scatter(P, g, Wc, s, a, b, c, g.tet_mass);
            } else if (cls == P_CELL_INSIDE) {
                ++st.cin;
                ++st.bbox;
                scatter(P, g, Wc, s, a, b, c, 6.f * Wc.f6[s]);
            } else if (cls == P_PARTIAL) {
                ++st.part;
                ++st.bbox;
                if (cross >= 0) {  // one face cuts the cell: closed form, no clipping
                    const float dm = halfspace_pair_vol6<kShare>(Wc, g, s, a, b, c, cross) * Wc.f6[s];
                    if (dm > 0.f) scatter(P, g, Wc, s, a, b, c, dm);
                } else {
                    part = true;
                    entry = ((uint32_t)s << 27) | (uint32_t)local;
                }
            }
        }
        const unsigned bal = __ballot_sync(0xffffffffu, part);
        if (part) Q[np + __popc(bal & ((1u << lane) - 1))] = entry;
        np += __popc(bal);
        __syncwarp();
    }
}

// Persistent: CTAs take work items (grid x vertex block) from a global
// counter; inside an item the warps take groups of 32 tets from a shared
// counter, so no warp waits for another until the item is done.
// kShare (zoom batches): a group with more than one chunk of pairs is
// published in its warp's slot, and warps whose groups are done take chunks
// of P.share_chunk pairs from open slots instead of waiting for the slowest warp at
// the end of the item.  On fine grids an item holds few tets with thousands
// of cells each, and one warp carried most of it (zoom batch 8.19 s without,
// 6.2 s with).  On coarse grids every group is a single chunk: kShare false
// keeps the plain loop there, whose registers the slot state would crowd
// (octree leaves 12% slower with it).
template <bool kShare>
__global__ void __launch_bounds__(kThreads, 2) deposit_mixed_kernel(DepositParams P)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SharedMixed &S = *reinterpret_cast<SharedMixed *>(smem_raw);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    WarpTets &W = S.wt[warp];
    uint32_t *Q = S.queue[warp];
    WarpPool &pool = S.pool[warp];
    PairStats st;
    const int chunk = P.share_chunk > 0 ? P.share_chunk : kChunk;  // pairs per shared chunk (> 0)
    if (kShare && threadIdx.x < kWarps) {
        S.slot_busy[threadIdx.x] = 0;
        S.slot_open[threadIdx.x] = 0;
    }

    for (int taken = 0;; ++taken) {
        // one-item CTAs (serving): a CTA exits after its items, so that the
        // CTAs of other requests' launches get SMs as these finish
        if (P.per_cta_items > 0 && taken >= P.per_cta_items) break;
        if (threadIdx.x == 0) {
            S.item = atomicAdd(P.counter, 1);
            S.n_cubes = 0;
            S.next_group = 0;
            S.groups_set = 0;
        }
        __syncthreads();
        const int item = S.item;
        if (item >= P.n_items) break;
        const Item it = P.items[item];
        if (threadIdx.x == 0) S.g = P.grids[it.grid];
        const int vx = it.nv & 0xff, vy = (it.nv >> 8) & 0xff, vz = (it.nv >> 16) & 0xff;
        stage_block(P, it, S.vert, vx, vy, vz, S.gh, S.gl);
        __syncthreads();
        const GridDesc &g = S.g;
        const int cvx = vx - 1, cvy = vy - 1, cvz = vz - 1;
        const int ncube = (cvx > 0 && cvy > 0 && cvz > 0) ? cvx * cvy * cvz : 0;
        for (int c = threadIdx.x; c < ncube; c += blockDim.x) {
            const int ci = c % cvx, r = c / cvx, cj = r % cvy, ck = r / cvy;
            if (cube_alive(S.vert, vx, vy, ci, cj, ck, g)) S.cubes[atomicAdd(&S.n_cubes, 1)] = (uint16_t)c;
        }
        __syncthreads();
        const int ntet = 6 * S.n_cubes;
        const int ngroups = (ntet + 31) / 32;
        if (!kShare) {
            for (;;) {
                int grp = 0;
                if (lane == 0) grp = atomicAdd(&S.next_group, 1);
                grp = __shfl_sync(0xffffffffu, grp, 0);
                if (grp >= ngroups) break;
                bool route64;
                int tid;
                const int total = group_setup<kShare>(P, S, W, g, grp, ntet, vx, vy, cvx, cvy, lane, st, route64, tid);
                pair_range<kShare>(P, g, W, pool, Q, 0, total, lane, st);
                group_route(P, S, item, route64, tid);
                __syncwarp();
            }
        } else {
            int cur = -1;      // slot whose pairs this warp takes (its own: cur == warp)
            int total = 0;     // pairs of slot cur
            int own_next = 0;  // own group: next pair if kept private, -1 if published
            for (;;) {
                if (cur < 0) {
                    int grp = 0;
                    if (lane == 0) grp = atomicAdd(&S.next_group, 1);
                    grp = __shfl_sync(0xffffffffu, grp, 0);
                    if (grp < ngroups) {
                        bool route64;
                        int tid;
                        total = group_setup<kShare>(P, S, W, g, grp, ntet, vx, vy, cvx, cvy, lane, st, route64, tid);
                        group_route(P, S, item, route64, tid);
                        // a group of one chunk or less is kept private
                        const bool pub = total > chunk;
                        if (lane == 0) {
                            if (pub) {
                                S.slot_total[warp] = total;
                                S.slot_next[warp] = 0;
                                __threadfence_block();
                                *(volatile int *)&S.slot_open[warp] = 1;
                            }
                            atomicAdd(&S.groups_set, 1);
                        }
                        __syncwarp();
                        cur = warp;
                        own_next = pub ? -1 : 0;
                    } else {
                        // help: join an open slot with pairs left; leave once every
                        // group is set up and none has pairs left (bounded wait)
                        int h = -1, ht = 0;
                        for (unsigned spin = 0;; ++spin) {
                            int set = 0;
                            if (lane == 0) {
                                // read before the scan: if every group was set up by
                                // then, the scan sees every slot that still has pairs
                                set = *(volatile int *)&S.groups_set;
                                __threadfence_block();
                                for (int d = 1; d < kWarps && h < 0; ++d) {
                                    const int w = (warp + d) % kWarps;
                                    if (*(volatile int *)&S.slot_open[w] &&
                                        *(volatile int *)&S.slot_next[w] < *(volatile int *)&S.slot_total[w]) {
                                        atomicAdd(&S.slot_busy[w], 1);
                                        __threadfence_block();
                                        if (*(volatile int *)&S.slot_open[w]) {
                                            __threadfence_block();  // then the owner's table is visible
                                            h = w;
                                            ht = *(volatile int *)&S.slot_total[w];
                                        } else {
                                            atomicSub(&S.slot_busy[w], 1);
                                        }
                                    }
                                }
                            }
                            h = __shfl_sync(0xffffffffu, h, 0);
                            set = __shfl_sync(0xffffffffu, set, 0);
                            if (h >= 0 || set >= ngroups || spin > P.help_spins) break;
                            __nanosleep(256);
                        }
                        if (h < 0) break;
                        cur = h;
                        total = __shfl_sync(0xffffffffu, ht, 0);
                        own_next = -1;
                    }
                }
                // next chunk of slot cur
                int c0 = own_next;
                if (own_next >= 0) {
                    own_next = total;
                } else {
                    if (lane == 0) c0 = atomicAdd(&S.slot_next[cur], chunk);
                    c0 = __shfl_sync(0xffffffffu, c0, 0);
                }
                if (c0 >= total) {
                    if (lane == 0) {
                        if (cur != warp) {
                            atomicSub(&S.slot_busy[cur], 1);
                        } else if (*(volatile int *)&S.slot_open[warp]) {
                            // close the slot, then wait for the helpers still reading W
                            *(volatile int *)&S.slot_open[warp] = 0;
                            __threadfence_block();
                            if (!wait_zero_bounded(&S.slot_busy[warp], P.close_spins, 32)) atomicOr(P.error, 8);
                        }
                    }
                    __syncwarp();
                    cur = -1;
                    continue;
                }
                pair_range<kShare>(P, g, S.wt[cur], pool, Q, c0, min(total, c0 + chunk), lane, st);
            }
        }
        __syncthreads();
    }
    if (P.stats) {
        warp_stat(P.stats, ST_TETS, st.tets);
        warp_stat(P.stats, ST_CAND, st.cand);
        warp_stat(P.stats, ST_BBOX, st.bbox);
        warp_stat(P.stats, ST_INSIDE, st.in);
        warp_stat(P.stats, ST_CELLIN, st.cin);
        warp_stat(P.stats, ST_PARTIAL, st.part);
        warp_stat(P.stats, ST_FP64, st.fp64);
        warp_stat(P.stats, ST_FALLBACK, st.fb);
    }
}

// ------------------------------------------------------ plain FP64 kernel
// The baseline the batched kernel is measured against: one warp per cube,
// every tet classified and clipped in FP64 lane-per-cell, FP64 atomics into
// the output grid; one launch per request.
__global__ void __launch_bounds__(kThreads) deposit_plain_fp64_kernel(DepositParams P, long long cube_begin,
                                                                      long long cube_end,
                                                                      const long long *item_cube_offset)
{
    const int lane = threadIdx.x & 31;
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long cube = cube_begin + gw; cube < cube_end; cube += nw) {
        // item owning this cube (binary search over the cube offsets)
        int lo_i = 0, hi_i = P.n_items - 1;
        while (lo_i < hi_i) {
            const int mid = (lo_i + hi_i + 1) >> 1;
            if (item_cube_offset[mid] <= cube) lo_i = mid; else hi_i = mid - 1;
        }
        const Item it = P.items[lo_i];
        const GridDesc g = P.grids[it.grid];
        const int vx = it.nv & 0xff, vy = (it.nv >> 8) & 0xff;
        const int cvx = vx - 1, cvy = vy - 1;
        const int c = (int)(cube - item_cube_offset[lo_i]);
        const int ci = c % cvx, r = c / cvx, cj = r % cvy, ck = r / cvy;
        float3 corner[8];
        bool pad = false;
#pragma unroll
        for (int s = 0; s < 8; ++s) {
            const int3 o = corner_offset(P.order, s);
            const long long gi = it.base + (ci + o.x) + P.stride_y * (cj + o.y) + P.stride_z * (ck + o.z);
            if (P.src_kind == SRC_LATTICE_F4) {
                const float4 p = __ldg(reinterpret_cast<const float4 *>(P.src) + gi);
                corner[s] = make_float3(p.x, p.y, p.z);
            } else {
                const float *q = reinterpret_cast<const float *>(P.src) + 3 * gi;
                corner[s] = make_float3(__ldg(q), __ldg(q + 1), __ldg(q + 2));
                if (P.pad_check) {
                    const float sum = __fadd_rn(__fadd_rn(fabsf(__fsub_rn(corner[s].x, 666.f)),
                                                          fabsf(__fsub_rn(corner[s].y, 666.f))),
                                                fabsf(__fsub_rn(corner[s].z, 666.f)));
                    pad |= ((double)sum < 1.E-03);
                }
            }
        }
        if (pad) continue;
        for (int t = 0; t < 6; ++t) {
            float3 v[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) v[q] = corner[tet_conn(t, q)];
            const float v6 = vol6_exact(v[0], v[1], v[2], v[3]);
            const int sgn = vol6_sign_ref(v6);
            int lo[3], hi[3];
            if (!candidate_range(v, g, lo, hi) || sgn == 0 || !tile_clamp(g, lo, hi)) continue;
            if (sgn < 0) { const float3 tt = v[0]; v[0] = v[3]; v[3] = tt; }
            unsigned nc = 0, np = 0;
            deposit_tet_fp64_warp(v, lo, hi, g, P.out_d, nc, np);
        }
    }
}

// -------------------------------------------------- ill-conditioned tets
// Per-warp state of the tet being routed (shared memory, written by lane 0):
// FP64 planes for the error-band fallback and the row bounds, the FP32
// vertex pairs hi + lo in the anchor frame, their planes and error band.
struct RouteTet {
    double pn[4][3], pd[4], pp[4], pm[4], rnx[4];
    double f6;
    float qf[4][3], ql[4][3], fn[4][3], fd[4], bmin[3], bmax[3], tol;
    int ex[3];
};

struct RouteWarp {
    BaryPool pool;
    RouteTet t;
};

constexpr size_t kRouteSmem = sizeof(RouteWarp) * kWarps;

__device__ __forceinline__ void route_setup(const float3 v[4], const int lo[3], const int hi[3], const GridDesc &g,
                                            RouteTet &T)
{
    double qd[4][3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double anchor = fma((double)lo[a], g.delta_d[a], g.gmin_d[a]);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const double x = (a == 0) ? (double)v[q].x : ((a == 1) ? (double)v[q].y : (double)v[q].z);
            qd[q][a] = (x - anchor) * g.scale_d[a];
        }
    }
    T.f6 = g.mass_factor / fabs(vol6_fast<double>(qd[0], qd[1], qd[2], qd[3]));
    const int fa[4] = {0, 0, 0, 1}, fb[4] = {2, 3, 1, 2}, fc[4] = {1, 2, 3, 3};
#pragma unroll
    for (int f = 0; f < 4; ++f) {
        const double e1x = qd[fb[f]][0] - qd[fa[f]][0], e1y = qd[fb[f]][1] - qd[fa[f]][1],
                     e1z = qd[fb[f]][2] - qd[fa[f]][2];
        const double e2x = qd[fc[f]][0] - qd[fa[f]][0], e2y = qd[fc[f]][1] - qd[fa[f]][1],
                     e2z = qd[fc[f]][2] - qd[fa[f]][2];
        const double nx = e1y * e2z - e1z * e2y, ny = e1z * e2x - e1x * e2z, nz = e1x * e2y - e1y * e2x;
        T.pn[f][0] = nx;
        T.pn[f][1] = ny;
        T.pn[f][2] = nz;
        T.pd[f] = nx * qd[fa[f]][0] + ny * qd[fa[f]][1] + nz * qd[fa[f]][2];
        T.pp[f] = fmax(nx, 0.0) + fmax(ny, 0.0) + fmax(nz, 0.0);
        T.pm[f] = fmin(nx, 0.0) + fmin(ny, 0.0) + fmin(nz, 0.0);
        const double nxr = nx * g.rcell[0];
        T.rnx[f] = nxr != 0.0 ? 1.0 / nxr : 0.0;
    }
    float R = 0.f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        T.ex[a] = hi[a] - lo[a] + 1;
        R = fmaxf(R, (float)T.ex[a]);
    }
    float qf[4][3];
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            qf[q][a] = __double2float_rn(qd[q][a]);
            T.qf[q][a] = qf[q][a];
            T.ql[q][a] = __double2float_rn(qd[q][a] - (double)qf[q][a]);
            R = fmaxf(R, fabsf(qf[q][a]));
        }
    float tol = 0.f;
#pragma unroll
    for (int f = 0; f < 4; ++f) {
        const float e1x = qf[fb[f]][0] - qf[fa[f]][0], e1y = qf[fb[f]][1] - qf[fa[f]][1],
                    e1z = qf[fb[f]][2] - qf[fa[f]][2];
        const float e2x = qf[fc[f]][0] - qf[fa[f]][0], e2y = qf[fc[f]][1] - qf[fa[f]][1],
                    e2z = qf[fc[f]][2] - qf[fa[f]][2];
        const float nx = e1y * e2z - e1z * e2y, ny = e1z * e2x - e1x * e2z, nz = e1x * e2y - e1y * e2x;
        T.fn[f][0] = nx;
        T.fn[f][1] = ny;
        T.fn[f][2] = nz;
        T.fd[f] = nx * qf[fa[f]][0] + ny * qf[fa[f]][1] + nz * qf[fa[f]][2];
        const float L1 = fmaxf(fmaxf(fabsf(e1x), fabsf(e1y)), fabsf(e1z));
        const float L2 = fmaxf(fmaxf(fabsf(e2x), fabsf(e2y)), fabsf(e2z));
        tol = fmaxf(tol, 1.0e-5f * L1 * L2 * (R + 1.f));
    }
    T.tol = tol;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        T.bmin[a] = fminf(fminf(qf[0][a], qf[1][a]), fminf(qf[2][a], qf[3][a]));
        T.bmax[a] = fmaxf(fmaxf(qf[0][a], qf[1][a]), fmaxf(qf[2][a], qf[3][a]));
    }
}

// Cell (a, b, k) of the routed tet: 0 outside, 1 holding the whole tet, 2
// inside the tet, 3 partial -- classify_pair's tests (FP32 planes with an
// error band, FP64 planes inside it).
__device__ __forceinline__ int route_classify(const RouteTet &T, const GridDesc &g, int a, int b, int k, unsigned &n64)
{
    const float xa = (float)a, xb = (float)b, xk = (float)k;
    if (!(T.bmin[0] < xa + 1.f && xa < T.bmax[0] && T.bmin[1] < xb + 1.f && xb < T.bmax[1] && T.bmin[2] < xk + 1.f &&
          xk < T.bmax[2]))
        return 0;
    if (T.bmin[0] >= xa && T.bmax[0] <= xa + 1.f && T.bmin[1] >= xb && T.bmax[1] <= xb + 1.f && T.bmin[2] >= xk &&
        T.bmax[2] <= xk + 1.f)
        return 1;
    bool all_in = true, unsure = false;
#pragma unroll
    for (int f = 0; f < 4; ++f) {
        const float nx = T.fn[f][0], ny = T.fn[f][1], nz = T.fn[f][2];
        const float base = fmaf(nx, xa, fmaf(ny, xb, fmaf(nz, xk, -T.fd[f])));
        const float pos = fmaxf(nx, 0.f) + fmaxf(ny, 0.f) + fmaxf(nz, 0.f);
        const float mx = base + pos;
        const float mn = base + ((nx + ny + nz) - pos);
        if (mx < -T.tol) return 0;
        if (mx <= T.tol) unsure = true;
        if (mn > T.tol) continue;
        all_in = false;
        if (mn > -T.tol) unsure = true;
    }
    if (!unsure) return all_in ? 2 : 3;
    ++n64;
    const double oa = a * g.rcell[0], ob = b * g.rcell[1], ok = k * g.rcell[2];
    all_in = true;
    for (int f = 0; f < 4; ++f) {
        const double base = T.pn[f][0] * oa + T.pn[f][1] * ob + T.pn[f][2] * ok - T.pd[f];
        if (base + T.pp[f] <= 0.0) return 0;
        if (!(base + T.pm[f] > 0.0)) all_in = false;
    }
    return all_in ? 2 : 3;
}

// Clip the np partial cells listed in RW.pool (local indices a + ex0 (b +
// ex1 k)) with the barycentric warp engine and deposit their masses; returns
// the pieces clipped serially.  One copy of the engine, called from every
// place a list fills.  Arguments by value: a reference to a caller's local
// variable would put it in local memory.
__device__ __noinline__ unsigned route_flush(RouteWarp &RW, const GridDesc &g, int lo0, int lo1, int lo2, int np,
                                             unsigned long long *out)
{
    unsigned fallbacks = 0;
    const int lane = threadIdx.x & 31;
    const RouteTet &T = RW.t;
    BaryPool &pool = RW.pool;
    const int ex0 = T.ex[0], ex1 = T.ex[1];
    clip_bary_pairs(
        pool, np,
        [&](int j, float *r) {
            const uint32_t c = pool.cell[j];
            const int a = (int)(c % (uint32_t)ex0), rr = (int)(c / (uint32_t)ex0);
            const int b = rr % ex1, k = rr / ex1;
#pragma unroll
            bary_identity(r);
            // coordinates in the cell's mirrored frame along axes whose lower
            // face the tet does not reach (as pair_piece); the shares come
            // from the weights, so no reordering is needed
            const int cc[3] = {a, b, k};
#pragma unroll
            for (int x = 0; x < 3; ++x) {
                const bool flip = T.bmin[x] > (float)cc[x];
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    r[12 + 3 * q + x] = cell_coord_sel(T.qf[q][x], T.ql[q][x], cc[x], g.drcell[x], flip);
            }
        },
        fallbacks);
    for (int j = lane; j < np; j += 32) {
        const uint32_t c = pool.cell[j];
        const int a = (int)(c % (uint32_t)ex0), rr = (int)(c / (uint32_t)ex0);
        const int b = rr % ex1, k = rr / ex1;
        const double dm = ldexp((double)pool.acc[j], -kVolShift) * g.mass_factor;
        const unsigned long long fx = (unsigned long long)llrint(ldexp(dm, g.shift));
        if (dm > 0.0 && fx)
            atomicAdd(out + g.out_offset + (lo0 + a) + (long long)g.dims * ((lo1 + b) + (long long)g.dims * (lo2 + k)),
                      fx);
    }
    __syncwarp();
    return fallbacks;
}

// One ill-conditioned tet, candidate range [lo, hi], deposited by a warp.
// Cells are offered in warp-wide rounds, at most one per lane: short rows
// (fewer than 8 cells along x) a cell per lane; long rows a row per lane,
// where the FP64 plane bounds, linear in the cell index and widened by a cell
// against rounding, skip the cells certainly outside and fill those certainly
// inside, and only the cells in between are offered.  Cells holding the tet
// or inside it are deposited at once; partial cells are listed and, 32 or
// more at a time, clipped by the barycentric warp engine from the FP32 hi +
// lo cell coordinates: the share of the tet times its exact mass.
__device__ __forceinline__ void route_tet_warp(const float3 v[4], const int lo[3], const int hi[3], const GridDesc &g,
                                               unsigned long long *out, RouteWarp &RW, unsigned &n_cand,
                                               unsigned &n_part, unsigned &n64, unsigned &fallbacks)
{
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1;
    RouteTet &T = RW.t;
    BaryPool &pool = RW.pool;
    __syncwarp();  // no lane still reads the previous tet's state
    if (lane == 0) route_setup(v, lo, hi, g, T);
    __syncwarp();
    const int ex0 = T.ex[0], ex1 = T.ex[1], ex2 = T.ex[2];
    const double inside6 = 6.0 * T.f6;
    auto put = [&](int a, int b, int k, double dm) {
        const unsigned long long fx = (unsigned long long)llrint(ldexp(dm, g.shift));
        if (fx)
            atomicAdd(out + g.out_offset + (lo[0] + a) +
                          (long long)g.dims * ((lo[1] + b) + (long long)g.dims * (lo[2] + k)),
                      fx);
    };
    int np = 0;  // listed partial cells (the same in every lane)
    auto flush = [&]() {
        fallbacks += route_flush(RW, g, lo[0], lo[1], lo[2], np, out);
        np = 0;
    };
    auto offer = [&](bool has, int a, int b, int k) {
        int cls = 0;
        if (has) {
            ++n_cand;
            cls = route_classify(T, g, a, b, k, n64);
            if (cls == 1) put(a, b, k, (double)g.tet_mass);
            if (cls == 2) put(a, b, k, inside6);
        }
        const unsigned part = __ballot_sync(0xffffffffu, cls == 3);
        if (cls == 3) {
            pool.cell[np + __popc(part & lt)] = (uint32_t)a + (uint32_t)ex0 * ((uint32_t)b + (uint32_t)ex1 * (uint32_t)k);
            ++n_part;
        }
        np += __popc(part);
        __syncwarp();
        if (np > kBaryList - 32) flush();
    };
    // one loop, one offer site (so the classification and the list code are
    // compiled once): short rows offer a cell per lane, long rows a row per
    // lane with the cells between the row bounds (the mode is the warp's)
    const bool by_rows = ex0 >= 8;
    const long long ncell = (long long)ex0 * ex1 * ex2, nrows = (long long)ex1 * ex2;
    long long c0 = 0;     // cells: first flattened cell of this round
    long long rr = lane;  // rows: this lane's row
    int b = 0, k = 0, a = 0, a1 = 0, a2 = 0, a3 = -1;  // the row's cells to offer: [a, a1), then [a2, a3]
    bool active = false;
    for (;;) {
        bool has = false;
        int ca = 0, cb = 0, ck = 0;
        if (!by_rows) {
            if (c0 >= ncell) break;
            const long long cc = c0 + lane;
            c0 += 32;
            has = cc < ncell;
            if (has) {
                const long long q = cc / ex0;
                ca = (int)(cc % ex0);
                cb = (int)(q % ex1);
                ck = (int)(q / ex1);
            }
        } else {
            while (!active && rr < nrows) {
                b = (int)(rr % ex1);
                k = (int)(rr / ex1);
                const double ob = b * g.rcell[1], ok = k * g.rcell[2];
                double lo_c = 0.0, hi_c = ex0 - 1, lo_i = 0.0, hi_i = ex0 - 1;
                bool none = false, no_in = false;
#pragma unroll
                for (int f = 0; f < 4; ++f) {
                    const double nx = T.pn[f][0];
                    const double K = T.pn[f][1] * ob + T.pn[f][2] * ok - T.pd[f];
                    if (nx > 0.0) {
                        lo_c = fmax(lo_c, floor(-(K + T.pp[f]) * T.rnx[f]) - 1.0);
                        lo_i = fmax(lo_i, floor(-(K + T.pm[f]) * T.rnx[f]) + 2.0);
                    } else if (nx < 0.0) {
                        hi_c = fmin(hi_c, ceil(-(K + T.pp[f]) * T.rnx[f]) + 1.0);
                        hi_i = fmin(hi_i, ceil(-(K + T.pm[f]) * T.rnx[f]) - 2.0);
                    } else {
                        none = none || !(K + T.pp[f] > 0.0);
                        no_in = no_in || !(K + T.pm[f] > 0.0);
                    }
                }
                if (none) {
                    rr += 32;
                    continue;
                }
                const int lc = (int)fmax(lo_c, 0.0), hc = (int)fmin(hi_c, (double)(ex0 - 1));
                int li = (int)fmax(lo_i, (double)lc), hi_ = (int)fmin(hi_i, (double)hc);
                if (no_in || li > hi_) {
                    li = hc + 1;
                    hi_ = hc;
                }
                for (int x = li; x <= hi_; ++x) put(x, b, k, inside6);
                if (li <= hi_) n_cand += hi_ - li + 1;
                a = lc;
                a1 = li;
                a2 = hi_ + 1;
                a3 = hc;
                active = a < a1 || a2 <= a3;
                if (!active) rr += 32;
            }
            if (!__any_sync(0xffffffffu, active)) break;
            if (active) {
                has = true;
                ca = a < a1 ? a++ : a2++;
                cb = b;
                ck = k;
                if (a >= a1 && a2 > a3) {
                    active = false;
                    rr += 32;
                }
            }
        }
        offer(has, ca, cb, ck);
    }
    if (np) flush();
}

// The tets deposit_mixed_kernel listed (kappa > kKappaFp64), one warp each:
// vertices re-read from the source, then route_tet_warp.
// Two CTAs of 8 warps per SM (128 registers a thread): with 28-float pieces
// the engine spilled in its inner loop, and one CTA per SM without spills
// (~220 registers) was slower still (a 256^3 clustered lattice: 696 against
// 636 ms); its 24-float pieces now spill almost nothing.
__global__ void __launch_bounds__(kThreads, 2) route_fp64_kernel(DepositParams P)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    RouteWarp &RW = reinterpret_cast<RouteWarp *>(smem_raw)[threadIdx.x >> 5];
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    const unsigned long long count = *P.route_count;
    const unsigned long long n = count < P.route_cap ? count : P.route_cap;
    unsigned cand = 0, part = 0, n64 = 0, fb = 0;
    for (unsigned long long e = warp; e < n; e += nwarps) {
        const unsigned long long entry = P.route[e];
        const Item it = P.items[entry >> 16];
        const int local = (int)(entry & 0xffff), c = local / 6, t = local % 6;
        const int vx = it.nv & 0xff, vy = (it.nv >> 8) & 0xff;
        const int cvx = vx - 1, cvy = vy - 1;
        const int ci = c % cvx, r = c / cvx, cj = r % cvy, ck = r / cvy;
        float3 v[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int3 o = corner_offset(P.order, tet_conn(t, q));
            const long long gi = it.base + (ci + o.x) + P.stride_y * (cj + o.y) + P.stride_z * (ck + o.z);
            if (P.src_kind == SRC_LATTICE_F4) {
                const float4 p = __ldg(reinterpret_cast<const float4 *>(P.src) + gi);
                v[q] = make_float3(p.x, p.y, p.z);
            } else {
                const float *s = reinterpret_cast<const float *>(P.src) + 3 * gi;
                v[q] = make_float3(__ldg(s), __ldg(s + 1), __ldg(s + 2));
            }
        }
        if (vol6_sign_ref(vol6_exact(v[0], v[1], v[2], v[3])) < 0) {
            const float3 tmp = v[0];
            v[0] = v[3];
            v[3] = tmp;
        }
        const GridDesc &g = P.grids[it.grid];
        int lo[3], hi[3];
        if (!candidate_range(v, g, lo, hi) || !tile_clamp(g, lo, hi)) continue;
        route_tet_warp(v, lo, hi, g, P.out, RW, cand, part, n64, fb);
    }
    if (P.stats) {
        warp_stat(P.stats, ST_CAND, cand);
        warp_stat(P.stats, ST_PARTIAL, part);
        warp_stat(P.stats, ST_FP64, n64);
        warp_stat(P.stats, ST_FALLBACK, fb);
    }
}

// ------------------------------------------- parity / diagnostics kernels
// Per tet of a patch sequence: vertex slots after the orientation rule, the
// volume sign, in-grid flag and candidate range (13 ints, as the oracle's
// records); and per cell the number of tets whose candidate range covers it.
__global__ void tet_records_kernel(const float *patches, int m, long long cube_begin, long long cube_end,
                                   GridDesc g, int order, int *rec, unsigned int *cand)
{
    const long long cube = cube_begin + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (cube >= cube_end) return;
    const long long cpp = (long long)m * m * m;
    const long long fpp = 3LL * (m + 1) * (m + 1) * (m + 1);
    const float *patch = patches + (cube / cpp) * fpp;
    const int local = (int)(cube % cpp);
    const int k = local / (m * m), r = local % (m * m), j = r / m, i = r % m;
    float3 corner[8];
    for (int s = 0; s < 8; ++s) {
        const int3 o = corner_offset(order, s);
        const long long id = (i + o.x) + (long long)(m + 1) * ((j + o.y) + (long long)(m + 1) * (k + o.z));
        corner[s] = make_float3(patch[3 * id], patch[3 * id + 1], patch[3 * id + 2]);
    }
    for (int t = 0; t < 6; ++t) {
        int *R = rec ? rec + 13 * ((cube - cube_begin) * 6 + t) : nullptr;
        float3 v[4];
        int slot[4];
        for (int q = 0; q < 4; ++q) {
            slot[q] = tet_conn(t, q);
            v[q] = corner[slot[q]];
        }
        const int sgn = vol6_sign_ref(vol6_exact(v[0], v[1], v[2], v[3]));
        if (sgn < 0) { const int tmp = slot[0]; slot[0] = slot[3]; slot[3] = tmp; }
        int lo[3], hi[3];
        const bool in = candidate_range(v, g, lo, hi);
        if (R) {
            for (int q = 0; q < 4; ++q) R[q] = slot[q];
            R[4] = sgn;
            R[5] = in ? 1 : 0;
            for (int a = 0; a < 3; ++a) {
                R[6 + 2 * a] = in ? lo[a] : -1;
                R[7 + 2 * a] = in ? hi[a] : -1;
            }
            R[12] = 0;
        }
        if (cand && in && sgn != 0)
            for (int z = lo[2]; z <= hi[2]; ++z)
                for (int y = lo[1]; y <= hi[1]; ++y)
                    for (int x = lo[0]; x <= hi[0]; ++x)
                        atomicAdd(cand + x + (long long)g.dims * (y + (long long)g.dims * z), 1u);
    }
}

// Bounding box of the vertices of a patch slice (3 floats each), padding
// vertices (all three coordinates 666) left out: per block min xyz, max xyz
// and a NaN flag (7 floats) into part[blockIdx.x * 7 ...].  A cell a tet
// deposits into lies in the tet's candidate range, inside the box of its
// vertices, so the cells outside this box's range receive nothing.
constexpr int kBoxThreads = 256;
__global__ void __launch_bounds__(kBoxThreads) patch_bbox_kernel(const float *pos, long long nvert, float *part)
{
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
    float nan = 0.f;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nvert; i += (long long)gridDim.x * blockDim.x) {
        const float x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
        if (x == 666.f && y == 666.f && z == 666.f) continue;
        if (x != x || y != y || z != z) nan = 1.f;
        mn[0] = fminf(mn[0], x); mn[1] = fminf(mn[1], y); mn[2] = fminf(mn[2], z);
        mx[0] = fmaxf(mx[0], x); mx[1] = fmaxf(mx[1], y); mx[2] = fmaxf(mx[2], z);
    }
    __shared__ float red[kBoxThreads / 32][7];
    float v[7] = {mn[0], mn[1], mn[2], mx[0], mx[1], mx[2], nan};
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int q = 0; q < 7; ++q) {
            const float w = __shfl_down_sync(0xffffffffu, v[q], o);
            v[q] = (q < 3) ? fminf(v[q], w) : fmaxf(v[q], w);
        }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0)
        for (int q = 0; q < 7; ++q) red[warp][q] = v[q];
    __syncthreads();
    if (threadIdx.x < 7) {
        const int q = threadIdx.x;
        float r = red[0][q];
        for (int w = 1; w < kBoxThreads / 32; ++w) r = (q < 3) ? fminf(r, red[w][q]) : fmaxf(r, red[w][q]);
        part[blockIdx.x * 7 + q] = r;
    }
}

// Cells [lo, lo + ext) of a dims^3 grid, packed x fastest: from the fixed
// point grid (times scale) when `fixed` is set, else copied from `f64`.
__global__ void grid_box_kernel(const unsigned long long *fixed, const double *f64, double *out, int dims, int lo0,
                                int lo1, int lo2, int e0, int e1, int e2, double scale)
{
    const long long n = (long long)e0 * e1 * e2;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long r = i / e0;
        const int x = (int)(i - r * e0), y = (int)(r % e1), z = (int)(r / e1);
        const long long c = (lo0 + x) + (long long)dims * ((lo1 + y) + (long long)dims * (lo2 + z));
        out[i] = fixed ? (double)fixed[c] * scale : f64[c];
    }
}

// fixed-point sums -> FP64 masses, added into an FP64 grid
__global__ void fixed_accumulate_f64_kernel(const unsigned long long *in, double *out, long long n, double scale)
{
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] += (double)in[i] * scale;
}

// per-leaf fixed-point grids -> FP64 with each grid's own scale
__global__ void fixed_to_f64_grids_kernel(const unsigned long long *in, double *out, const GridDesc *grids,
                                          int n_grids, long long cells_per_grid)
{
    const long long n = (long long)n_grids * cells_per_grid;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int gi = (int)(i / cells_per_grid);
        out[i] = ldexp((double)in[i], -grids[gi].shift);
    }
}

// Meta-cell AABBs of a resident float4 lattice (7^3-cube meta-cells): one
// warp per meta-cell, min/max over its <= 8^3 vertices.
__global__ void meta_bbox_kernel(const float4 *pos, int nx, int ny, int nz, int cdx, int cdy, int cdz, float *bbox6)
{
    const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const long long nmc = (long long)cdx * cdy * cdz;
    if (w >= nmc) return;
    const int cx = (int)(w % cdx), r = (int)(w / cdx), cy = r % cdy, cz = r / cdy;
    const int ox = cx * 7, oy = cy * 7, oz = cz * 7;
    const int dx = (cx + 1 == cdx) ? nx - ox : 8, dy = (cy + 1 == cdy) ? ny - oy : 8, dz = (cz + 1 == cdz) ? nz - oz : 8;
    float mn[3] = {3.4e38f, 3.4e38f, 3.4e38f}, mx[3] = {-3.4e38f, -3.4e38f, -3.4e38f};
    const int nv = dx * dy * dz;
    for (int v = lane; v < nv; v += 32) {
        const int i = v % dx, rr = v / dx, j = rr % dy, k = rr / dy;
        const float4 p = pos[(ox + i) + (long long)nx * ((oy + j) + (long long)ny * (oz + k))];
        mn[0] = fminf(mn[0], p.x); mx[0] = fmaxf(mx[0], p.x);
        mn[1] = fminf(mn[1], p.y); mx[1] = fmaxf(mx[1], p.y);
        mn[2] = fminf(mn[2], p.z); mx[2] = fmaxf(mx[2], p.z);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            mn[a] = fminf(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], o));
            mx[a] = fmaxf(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], o));
        }
    if (lane == 0)
        for (int a = 0; a < 3; ++a) {
            bbox6[6 * w + a] = mn[a];
            bbox6[6 * w + 3 + a] = mx[a];
        }
}

}  // namespace adeco
