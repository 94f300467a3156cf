// clip_engine.cuh -- warp-cooperative exact clipping of tets against unit cells.
//
// A batch of up to 32 (tet, cell) pairs is clipped by the whole warp at once.
// Every lane holds one piece (a tet, 12 FP32 coordinates in the cell frame)
// in registers.  Each step a lane either
//   * drops its piece (entirely outside a cell face it has not yet passed),
//   * finishes it (inside all six faces): its 6x volume is added, as exact
//     64-bit fixed point, to the accumulator of the pair it came from, or
//   * splits it by the next cell face it crosses into 1 or 3 inside pieces,
//     keeps one and pushes the others onto a per-warp shared-memory pool;
// then idle lanes pop pieces from the pool (last in, first out).  All lanes
// run the same split code every step, so a pair whose tet crosses several
// faces (up to 3^6 pieces) spreads over the warp instead of serialising one
// lane.  No per-thread stack: nothing spills to local memory.
//
// The split keeps every piece positively oriented: the vertices are permuted
// (an even permutation) so that the k inside vertices come first, then the
// inside part is written as 1 tet (k = 1) or as a 3-tet prism decomposition
// (k = 2, 3) over the cut points on the crossing edges.
#pragma once

#include "geometry.cuh"

namespace adeco {

// inside-first even permutation (4 x 2 bits) and inside count per side mask
#define ADECO_SPLIT_PERM {228, 228, 177, 228, 210, 210, 201, 228, 99, 156, 135, 177, 78, 120, 54, 228}
#define ADECO_SPLIT_KIN {0, 1, 1, 2, 1, 2, 2, 3, 1, 2, 2, 3, 2, 3, 3, 4}
#ifdef __CUDACC__
__constant__ uint8_t c_split_perm[16] = ADECO_SPLIT_PERM;
__constant__ int8_t c_split_kin[16] = ADECO_SPLIT_KIN;
#endif
static const uint8_t h_split_perm[16] = ADECO_SPLIT_PERM;
static const int8_t h_split_kin[16] = ADECO_SPLIT_KIN;

ADECO_HD inline int split_perm(int m)
{
#ifdef __CUDA_ARCH__
    return c_split_perm[m];
#else
    return h_split_perm[m];
#endif
}
ADECO_HD inline int split_kin(int m)
{
#ifdef __CUDA_ARCH__
    return c_split_kin[m];
#else
    return h_split_kin[m];
#endif
}

ADECO_HD inline float sel4(int i, float a, float b, float c, float d)
{
    return (i & 2) ? ((i & 1) ? d : c) : ((i & 1) ? b : a);
}
ADECO_HD inline float sel3(int i, float x, float y, float z) { return i == 0 ? x : (i == 1 ? y : z); }

// 6 inside bits of a point: bit 2a = (x_a > 0), bit 2a+1 = (x_a < 1)
ADECO_HD inline int face_bits(float x, float y, float z)
{
    return (int)(x > 0.f) | ((int)(x < 1.f) << 1) | ((int)(y > 0.f) << 2) | ((int)(y < 1.f) << 3) |
           ((int)(z > 0.f) << 4) | ((int)(z < 1.f) << 5);
}

// point where edge in->out crosses the plane x_axis = plane (snapped onto it)
ADECO_HD inline void cut_point(const float *pin, const float *pout, int axis, float plane, float *x)
{
    const float din = sel3(axis, pin[0], pin[1], pin[2]);
    const float dout = sel3(axis, pout[0], pout[1], pout[2]);
#ifdef __CUDA_ARCH__
    float t = __fdividef(plane - din, dout - din);  // |dout - din| > 0 for a crossing edge
#else
    float t = (plane - din) / (dout - din);
#endif
    t = fminf(fmaxf(t, 0.f), 1.f);
    x[0] = (axis == 0) ? plane : fmaf(t, pout[0] - pin[0], pin[0]);
    x[1] = (axis == 1) ? plane : fmaf(t, pout[1] - pin[1], pin[1]);
    x[2] = (axis == 2) ? plane : fmaf(t, pout[2] - pin[2], pin[2]);
}

// Inside part of piece p w.r.t. face f (mask = 4-bit inside flags, 0 < mask <
// 15) as n = 1 or 3 positively oriented pieces c0..c2.  With the vertices
// permuted to A B C D (inside first, even permutation) and k inside:
//   k = 1: (A, Xab, Xac, Xad)
//   k = 2: (A, B, Xbc, Xbd) (A, Xbc, Xac, Xbd) (A, Xac, Xad, Xbd)
//   k = 3: (A, B, C, Xcd)  (A, B, Xcd, Xbd) (A, Xbd, Xcd, Xad)
// written as one code path: four cut points E0..E3 chosen by k, then the
// children's vertices picked by k.
ADECO_HD inline int split_piece(const float p[12], int mask, int f, float c0[12], float c1[12], float c2[12])
{
    const int axis = f >> 1;
    const float plane = (f & 1) ? 1.f : 0.f;
    const int pm = split_perm(mask), k = split_kin(mask);
    const int ia = pm & 3, ib = (pm >> 2) & 3, ic = (pm >> 4) & 3, id = (pm >> 6) & 3;
    float A[3], B[3], C[3], D[3];
#pragma unroll
    for (int x = 0; x < 3; ++x) {
        A[x] = sel4(ia, p[x], p[3 + x], p[6 + x], p[9 + x]);
        B[x] = sel4(ib, p[x], p[3 + x], p[6 + x], p[9 + x]);
        C[x] = sel4(ic, p[x], p[3 + x], p[6 + x], p[9 + x]);
        D[x] = sel4(id, p[x], p[3 + x], p[6 + x], p[9 + x]);
    }
    // edge end points: k=1: AB AC AD AD; k=2: AC AD BC BD; k=3: AD BD CD CD
    float i0[3], o0[3], i1[3], o1[3], i2[3], o2[3], i3[3], o3[3];
#pragma unroll
    for (int x = 0; x < 3; ++x) {
        i0[x] = A[x];
        o0[x] = (k == 1) ? B[x] : ((k == 2) ? C[x] : D[x]);
        i1[x] = (k == 3) ? B[x] : A[x];
        o1[x] = (k == 1) ? C[x] : D[x];
        i2[x] = (k == 1) ? A[x] : ((k == 2) ? B[x] : C[x]);
        o2[x] = (k == 2) ? C[x] : D[x];
        i3[x] = (k == 2) ? B[x] : ((k == 3) ? C[x] : A[x]);
        o3[x] = D[x];
    }
    float E0[3], E1[3], E2[3], E3[3];
    cut_point(i0, o0, axis, plane, E0);
    cut_point(i1, o1, axis, plane, E1);
    cut_point(i2, o2, axis, plane, E2);
    cut_point(i3, o3, axis, plane, E3);
    // k=1: E0=Xab E1=Xac E2=Xad | k=2: E0=Xac E1=Xad E2=Xbc E3=Xbd | k=3: E0=Xad E1=Xbd E2=Xcd
    const bool k1 = (k == 1), k2 = (k == 2);
#pragma unroll
    for (int x = 0; x < 3; ++x) {
        c0[x] = A[x];
        c0[3 + x] = k1 ? E0[x] : B[x];
        c0[6 + x] = k1 ? E1[x] : (k2 ? E2[x] : C[x]);
        c0[9 + x] = k1 ? E2[x] : (k2 ? E3[x] : E2[x]);
        c1[x] = A[x];
        c1[3 + x] = k2 ? E2[x] : B[x];
        c1[6 + x] = k2 ? E0[x] : E2[x];
        c1[9 + x] = k2 ? E3[x] : E1[x];
        c2[x] = A[x];
        c2[3 + x] = k2 ? E0[x] : E1[x];
        c2[6 + x] = k2 ? E1[x] : E2[x];
        c2[9 + x] = k2 ? E3[x] : E0[x];
    }
    return k1 ? 1 : 3;
}

constexpr int kVolShift = 56;  // fixed point of 6x piece volumes (each <= 6)

ADECO_HD inline long long vol_fixed(float v6)
{
    const unsigned long long m = to_fixed(fabsf(v6), kVolShift);
    return v6 < 0.f ? -(long long)m : (long long)m;
}

ADECO_HD inline float piece_vol6(const float p[12])
{
    return vol6_fast<float>(p, p + 3, p + 6, p + 9);
}

// state of one piece: next face to examine -> (code, face); code 0 = dropped,
// 1 = finished, 2 = split at `face` with inside mask `mask`
ADECO_HD inline int piece_step(const float p[12], int face0, int &face, int &mask)
{
    const int b0 = face_bits(p[0], p[1], p[2]), b1 = face_bits(p[3], p[4], p[5]);
    const int b2 = face_bits(p[6], p[7], p[8]), b3 = face_bits(p[9], p[10], p[11]);
    const int all_in = b0 & b1 & b2 & b3, any_in = b0 | b1 | b2 | b3;
    const int relevant = (63 >> face0) << face0;
    if ((~any_in) & relevant) return 0;  // entirely outside a remaining face
    const int next = (~all_in) & relevant;
    if (!next) return 1;
#ifdef __CUDA_ARCH__
    face = __ffs(next) - 1;
#else
    face = __builtin_ctz(next);
#endif
    mask = ((b0 >> face) & 1) | (((b1 >> face) & 1) << 1) | (((b2 >> face) & 1) << 2) | (((b3 >> face) & 1) << 3);
    return 2;
}

// Serial clipping of one piece from face `face0` on (used when the warp pool
// is full, and by the host model): depth-first over the same splits, so the
// fixed-point sum is identical to the warp engine's.
#ifdef __CUDA_ARCH__
__device__ __noinline__
#else
inline
#endif
long long clip_piece_serial(const float p0[12], int face0)
{
    constexpr int kDepth = 16;  // 2 pending siblings per face level + 3
    float stk[kDepth][12];
    int sface[kDepth];
#pragma unroll
    for (int x = 0; x < 12; ++x) stk[0][x] = p0[x];
    sface[0] = face0;
    int sp = 1;
    long long acc = 0;
    while (sp > 0) {
        --sp;
        float p[12];
#pragma unroll
        for (int x = 0; x < 12; ++x) p[x] = stk[sp][x];
        int face = 0, mask = 0;
        const int code = piece_step(p, sface[sp], face, mask);
        if (code == 0) continue;
        if (code == 1) {
            acc += vol_fixed(piece_vol6(p));
            continue;
        }
        float c0[12], c1[12], c2[12];
        const int n = split_piece(p, mask, face, c0, c1, c2);
        if (sp + n > kDepth) continue;  // cannot happen (depth <= 2*5 + 3)
#pragma unroll
        for (int x = 0; x < 12; ++x) stk[sp][x] = c0[x];
        sface[sp++] = face + 1;
        if (n == 3) {
#pragma unroll
            for (int x = 0; x < 12; ++x) stk[sp][x] = c1[x];
            sface[sp++] = face + 1;
#pragma unroll
            for (int x = 0; x < 12; ++x) stk[sp][x] = c2[x];
            sface[sp++] = face + 1;
        }
    }
    return acc;
}

#ifdef __CUDACC__
constexpr int kPool = 64;  // pieces per warp pool

struct WarpPool {
    float v[12][kPool];
    uint32_t meta[kPool];   // owner lane | next face << 8
    long long vacc[32];     // 6x volume of each pair of the batch, fixed point 2^kVolShift
};

// Clip the warp's batch: lane l < nb holds piece p (pair l) on entry.  On
// return pool.vacc[l] is the exact-sum 6x volume of pair l.  `fallbacks`
// counts pieces clipped serially because the pool was full.
__device__ __forceinline__ void clip_batch(WarpPool &pool, float p[12], int nb, unsigned &fallbacks)
{
    const int lane = threadIdx.x & 31;
    bool valid = lane < nb;
    int owner = lane, face = 0;
    pool.vacc[lane] = 0;
    __syncwarp();
    int top = 0;
    for (;;) {
        int npush = 0;
        float c1[12], c2[12];
        if (valid) {
            int f = 0, mask = 0;
            const int code = piece_step(p, face, f, mask);
            if (code == 0) {
                valid = false;
            } else if (code == 1) {
                atomicAdd(reinterpret_cast<unsigned long long *>(&pool.vacc[owner]),
                          (unsigned long long)vol_fixed(piece_vol6(p)));
                valid = false;
            } else {
                float c0[12];
                const int n = split_piece(p, mask, f, c0, c1, c2);
#pragma unroll
                for (int x = 0; x < 12; ++x) p[x] = c0[x];
                face = f + 1;
                npush = n - 1;
            }
        }
        // push the extra pieces (warp-wide exclusive scan of npush)
        int incl = npush;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        if (total) {
            if (top + total <= kPool) {
                const int base = top + incl - npush;
                if (npush >= 1) {
#pragma unroll
                    for (int x = 0; x < 12; ++x) pool.v[x][base] = c1[x];
                    pool.meta[base] = (uint32_t)owner | ((uint32_t)face << 8);
                }
                if (npush == 2) {
#pragma unroll
                    for (int x = 0; x < 12; ++x) pool.v[x][base + 1] = c2[x];
                    pool.meta[base + 1] = (uint32_t)owner | ((uint32_t)face << 8);
                }
                top += total;
            } else if (npush) {  // pool full: finish this lane's extra pieces serially
                long long acc = clip_piece_serial(c1, face);
                if (npush == 2) acc += clip_piece_serial(c2, face);
                atomicAdd(reinterpret_cast<unsigned long long *>(&pool.vacc[owner]), (unsigned long long)acc);
                ++fallbacks;
            }
        }
        __syncwarp();
        // idle lanes take pieces from the pool, last in first out
        const unsigned need = __ballot_sync(0xffffffffu, !valid);
        const int rank = __popc(need & ((1u << lane) - 1));
        const int nneed = __popc(need);
        if (!valid && rank < top) {
            const int idx = top - 1 - rank;
#pragma unroll
            for (int x = 0; x < 12; ++x) p[x] = pool.v[x][idx];
            const uint32_t m = pool.meta[idx];
            owner = (int)(m & 0xff);
            face = (int)(m >> 8);
            valid = true;
        }
        top -= (nneed < top) ? nneed : top;
        __syncwarp();
        if (!__any_sync(0xffffffffu, valid)) break;
    }
    __syncwarp();
}
#endif

}  // namespace adeco
