// clip_engine.cuh -- warp-cooperative exact clipping of tets against unit cells.
//
// A batch of up to 32 (tet, cell) pairs is clipped by the whole warp at once.
// Every lane holds one piece (a tet, 12 FP32 coordinates in the cell frame)
// in registers.  Each step a lane either
//   * drops its piece (entirely outside a cell face it has not yet passed),
//   * finishes it (inside all six faces): its 6x volume is added, as exact
//     64-bit fixed point, to the accumulator of the pair it came from, or
//   * at the last cell face it crosses, adds the inside fraction of its
//     volume (from the edge parameters alone, no cut points), or
//   * splits it by a cell face it crosses (of those, one with the fewest of
//     its vertices inside: next_face) into 1 or 3 inside pieces, keeps one
//     and pushes the others onto a per-warp shared-memory pool;
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
static const uint8_t h_split_perm[16] = ADECO_SPLIT_PERM;
static const int8_t h_split_kin[16] = ADECO_SPLIT_KIN;

// The tables are read with lane-dependent masks, which a constant-memory load
// serialises per distinct address; the entries are therefore taken from two
// 64-bit immediates (the permutation, a byte per mask) and from the popcount
// (the inside count) -- the same values as ADECO_SPLIT_PERM / ADECO_SPLIT_KIN.
ADECO_HD inline int split_perm(int m)
{
    const unsigned long long w = (m & 8) ? 0xe436784eb1879c63ull : 0xe4c9d2d2e4b1e4e4ull;
    return (int)((w >> ((m & 7) * 8)) & 0xffu);
}
ADECO_HD inline int split_kin(int m)
{
#ifdef __CUDA_ARCH__
    return __popc((unsigned)m);
#else
    return __builtin_popcount((unsigned)m);
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

// The cut of piece p by face f (mask: its vertices inside, 0 < mask < 15;
// k of them), shared by a split and a last-face fraction: the vertices
// permuted to A B C D, inside first by an even permutation (the orientation
// is kept), the four cut edges' end points -- k=1: AB AC AD AD; k=2: AC AD
// BC BD; k=3: AD BD CD CD -- and on each edge the reciprocal r of its extent
// along the face's axis and the face's parameter t from the inside end.
struct Cut {
    float A[3], B[3], C[3], D[3];
    float i[4][3], o[4][3];
    float t[4], r[4];
    int k;
};

ADECO_HD inline void cut_piece(const float p[12], int mask, int f, Cut &c)
{
    const int axis = f >> 1;
    const float plane = (f & 1) ? 1.f : 0.f;
    const int pm = split_perm(mask), k = split_kin(mask);
    c.k = k;
    const int ia = pm & 3, ib = (pm >> 2) & 3, ic = (pm >> 4) & 3, id = (pm >> 6) & 3;
#pragma unroll
    for (int x = 0; x < 3; ++x) {
        c.A[x] = sel4(ia, p[x], p[3 + x], p[6 + x], p[9 + x]);
        c.B[x] = sel4(ib, p[x], p[3 + x], p[6 + x], p[9 + x]);
        c.C[x] = sel4(ic, p[x], p[3 + x], p[6 + x], p[9 + x]);
        c.D[x] = sel4(id, p[x], p[3 + x], p[6 + x], p[9 + x]);
        c.i[0][x] = c.A[x];
        c.o[0][x] = (k == 1) ? c.B[x] : ((k == 2) ? c.C[x] : c.D[x]);
        c.i[1][x] = (k == 3) ? c.B[x] : c.A[x];
        c.o[1][x] = (k == 1) ? c.C[x] : c.D[x];
        c.i[2][x] = (k == 1) ? c.A[x] : ((k == 2) ? c.B[x] : c.C[x]);
        c.o[2][x] = (k == 2) ? c.C[x] : c.D[x];
        c.i[3][x] = (k == 2) ? c.B[x] : ((k == 3) ? c.C[x] : c.A[x]);
        c.o[3][x] = c.D[x];
    }
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const float din = sel3(axis, c.i[e][0], c.i[e][1], c.i[e][2]);
        const float dout = sel3(axis, c.o[e][0], c.o[e][1], c.o[e][2]);
        c.r[e] = rcp_nr(dout - din);  // |dout - din| > 0 on a crossing edge
        c.t[e] = fminf(fmaxf((plane - din) * c.r[e], 0.f), 1.f);
    }
}

// Inside part of a cut piece as n = 1 or 3 positively oriented pieces
// c0..c2, from the cut points E0..E3 of the cut's edges (snapped onto the
// face):
//   k = 1: (A, Xab, Xac, Xad)
//   k = 2: (A, B, Xbc, Xbd) (A, Xbc, Xac, Xbd) (A, Xac, Xad, Xbd)
//   k = 3: (A, B, C, Xcd)  (A, B, Xcd, Xbd) (A, Xbd, Xcd, Xad)
// written as one code path: the children's vertices picked by k.
ADECO_HD inline int split_cut(const Cut &c, int f, float c0[12], float c1[12], float c2[12])
{
    const int axis = f >> 1;
    const float plane = (f & 1) ? 1.f : 0.f;
    float E[4][3];
#pragma unroll
    for (int e = 0; e < 4; ++e)
#pragma unroll
        for (int x = 0; x < 3; ++x)
            E[e][x] = (x == axis) ? plane : fmaf(c.t[e], c.o[e][x] - c.i[e][x], c.i[e][x]);
    // k=1: E0=Xab E1=Xac E2=Xad | k=2: E0=Xac E1=Xad E2=Xbc E3=Xbd | k=3: E0=Xad E1=Xbd E2=Xcd
    const bool k1 = (c.k == 1), k2 = (c.k == 2);
#pragma unroll
    for (int x = 0; x < 3; ++x) {
        c0[x] = c.A[x];
        c0[3 + x] = k1 ? E[0][x] : c.B[x];
        c0[6 + x] = k1 ? E[1][x] : (k2 ? E[2][x] : c.C[x]);
        c0[9 + x] = k1 ? E[2][x] : (k2 ? E[3][x] : E[2][x]);
        c1[x] = c.A[x];
        c1[3 + x] = k2 ? E[2][x] : c.B[x];
        c1[6 + x] = k2 ? E[0][x] : E[2][x];
        c1[9 + x] = k2 ? E[3][x] : E[1][x];
        c2[x] = c.A[x];
        c2[3 + x] = k2 ? E[0][x] : E[1][x];
        c2[6 + x] = k2 ? E[1][x] : E[2][x];
        c2[9 + x] = k2 ? E[3][x] : E[0][x];
    }
    return k1 ? 1 : 3;
}

// The fraction of a cut piece inside the face (its last crossed face), from
// the edge parameters alone: t from the cut, u = 1 - t taken as (x_o -
// plane) r so both keep their relative precision (side_fraction's formulas,
// on the same edges).
ADECO_HD inline float cut_fraction(const Cut &c, int f)
{
    const int axis = f >> 1;
    const float plane = (f & 1) ? 1.f : 0.f;
    float u[4];
#pragma unroll
    for (int e = 0; e < 4; ++e)
        u[e] = fminf(fmaxf((sel3(axis, c.o[e][0], c.o[e][1], c.o[e][2]) - plane) * c.r[e], 0.f), 1.f);
    const float *t = c.t;
    if (c.k == 1) return t[0] * t[1] * t[2];
    if (c.k == 2) return fmaf(t[2], t[3], t[0] * (t[3] * u[2] + t[1] * u[3]));
    return fmaf(u[0], fmaf(u[1], t[2], t[1]), t[0]);
}

// Fraction of piece p inside face f (mask = 4-bit inside flags, 0 < mask <
// 15), from the edge parameters alone.  On an edge from inside vertex i to
// outside vertex o the plane sits at t = (plane - x_i) / (x_o - x_i); with u =
// 1 - t taken as (x_o - plane) / (x_o - x_i) so both keep their relative
// precision, and with the vertices ordered A B C D (inside first):
//   k = 1: t_AB t_AC t_AD                          (the corner tet at A)
//   k = 2: t_BC t_BD + t_AC t_BD u_BC + t_AC t_AD u_BD   (the 3-tet prism)
//   k = 3: 1 - u_AD u_BD u_CD = t_AD + u_AD (t_BD + u_BD t_CD)
// Every term is non-negative, so the fraction carries a few ulps of relative
// error and the inside volume needs no cut points and no child volumes.
// The same fraction for any linear function over the tet: x0..x3 its values
// at the vertices, inside = the side of `plane` given by mask.
ADECO_HD inline float side_fraction(float x0, float x1, float x2, float x3, int mask, float plane)
{
    const int pm = split_perm(mask), k = split_kin(mask);
    const float a = sel4(pm & 3, x0, x1, x2, x3), b = sel4((pm >> 2) & 3, x0, x1, x2, x3);
    const float c = sel4((pm >> 4) & 3, x0, x1, x2, x3), d = sel4((pm >> 6) & 3, x0, x1, x2, x3);
    // edges as in cut_piece: k=1: AB AC AD; k=2: AC AD BC BD; k=3: AD BD CD
    const float i0 = a, o0 = (k == 1) ? b : ((k == 2) ? c : d);
    const float i1 = (k == 3) ? b : a, o1 = (k == 1) ? c : d;
    const float i2 = (k == 1) ? a : ((k == 2) ? b : c), o2 = (k == 2) ? c : d;
    const float i3 = b, o3 = d;
    float t[4], u[4];
    const float in[4] = {i0, i1, i2, i3}, out[4] = {o0, o1, o2, o3};
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        // an unbiased reciprocal (rcp_nr): an approximate one biases the
        // fractions of all pairs the same way and shows in the total mass
        const float r = rcp_nr(out[e] - in[e]);
        t[e] = fminf(fmaxf((plane - in[e]) * r, 0.f), 1.f);
        u[e] = fminf(fmaxf((out[e] - plane) * r, 0.f), 1.f);
    }
    if (k == 1) return t[0] * t[1] * t[2];
    if (k == 2) return fmaf(t[2], t[3], t[0] * (t[3] * u[2] + t[1] * u[3]));
    return fmaf(u[0], fmaf(u[1], t[2], t[1]), t[0]);
}

// 6x volume of the unit cube's part where G(u) = G0 + n.u > 0 (G0 a
// double-float pair).  The cube is first reflected along every axis where
// n_i < 0 (the volume does not change), so that n >= 0 and G grows along
// every edge path from corner 0 to corner 7.  The corner values are then
// formed exactly (TwoSum) and rounded once, which keeps that order, and the
// cube is split into the 6 tets around the diagonal 0-7, each of 6x volume 1:
// tet (0, a, b, 7) for the paths a -> b in {1,2,4} -> {3,5,6}, with values
// g0 <= ga <= gb <= g7.  The part of a tet where G > 0 is then a suffix of its
// path, and its fraction comes from the parameters t = g_in / (g_in - g_out)
// and u = 1 - t = -g_out / (g_in - g_out) of its crossing edges:
//   only 7 inside (gb <= 0 < g7):  t_70 t_7a t_7b        (the corner tet)
//   7, b inside (ga <= 0 < gb):    t_b0 t_ba + t_70 t_ba u_b0 + t_70 t_7a u_ba   (the prism)
//   0 outside (g0 <= 0 < ga):      t_a0 + u_a0 (t_b0 + u_b0 t_70)
// -- non-negative terms only, the same instructions on every lane, and the 19
// edge reciprocals shared by the 6 tets.  A face function turns a value a
// few ulps off its exact one, so a plane passing close to a corner keeps its
// relative precision.
ADECO_HD inline float halfspace_cube_vol6(F2 G0, float nx, float ny, float nz)
{
    G0 = f2_add(G0, F2{fminf(nx, 0.f), 0.f});
    G0 = f2_add(G0, F2{fminf(ny, 0.f), 0.f});
    G0 = f2_add(G0, F2{fminf(nz, 0.f), 0.f});
    nx = fabsf(nx);
    ny = fabsf(ny);
    nz = fabsf(nz);
    const F2 e1 = f2_add(G0, F2{nx, 0.f}), e2 = f2_add(G0, F2{ny, 0.f}), e4 = f2_add(G0, F2{nz, 0.f});
    const F2 e3 = f2_add(e1, F2{ny, 0.f}), e5 = f2_add(e1, F2{nz, 0.f}), e6 = f2_add(e2, F2{nz, 0.f});
    const F2 e7 = f2_add(e3, F2{nz, 0.f});
    const float g0 = G0.hi + G0.lo, g7 = e7.hi;
    const float ga[3] = {e1.hi, e2.hi, e4.hi};  // a = 1, 2, 4
    const float gb[3] = {e3.hi, e5.hi, e6.hi};  // b = 3, 5, 6
    if (!(g7 > 0.f)) return 0.f;
    if (g0 > 0.f) return 6.f;
    const float r70 = rcp_nr(g7 - g0);
    const float t70 = g7 * r70;
    float ta0[3], ua0[3], t7a[3], tb0[3], ub0[3], t7b[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float ra0 = rcp_nr(ga[i] - g0), rb0 = rcp_nr(gb[i] - g0);
        ta0[i] = ga[i] * ra0;
        ua0[i] = -g0 * ra0;
        tb0[i] = gb[i] * rb0;
        ub0[i] = -g0 * rb0;
        t7a[i] = g7 * rcp_nr(g7 - ga[i]);
        t7b[i] = g7 * rcp_nr(g7 - gb[i]);
    }
    // tets (a, b) by index into ga / gb: (1,3) (1,5) (2,3) (2,6) (4,5) (4,6)
    const int ia[6] = {0, 0, 1, 1, 2, 2}, ib[6] = {0, 1, 0, 2, 1, 2};
    float v = 0.f;
#pragma unroll
    for (int q = 0; q < 6; ++q) {
        const int i = ia[q], j = ib[q];
        const float rba = rcp_nr(gb[j] - ga[i]);
        const float tba = gb[j] * rba, uba = -ga[i] * rba;
        const float k1 = t70 * t7a[i] * t7b[j];
        const float k2 = fmaf(tb0[j], tba, t70 * fmaf(tba, ub0[j], t7a[i] * uba));
        const float k3 = fmaf(ua0[i], fmaf(ub0[j], t70, tb0[j]), ta0[i]);
        v += (gb[j] <= 0.f) ? k1 : ((ga[i] <= 0.f) ? k2 : k3);
    }
    return v;
}

// 2x2 minor a d - b c
ADECO_HD inline F2 f2_minor(F2 a, F2 d, F2 b, F2 c)
{
    const F2 bc = f2_mul(b, c);
    return f2_add(f2_mul(a, d), {-bc.hi, -bc.lo});
}

// The cell face a piece is clipped by next, from its vertices' 6-bit inside
// flags b0..b3 and the faces already done (`done`, one bit per face):
// returns 0 if the piece lies beyond a remaining face (dropped), 1 if it lies
// inside all of them (finished), else 2 with `face` the crossed face that has
// the fewest of the piece's vertices inside, `mask` those vertices and `last`
// set when no other face is crossed.  Fewest inside first: a single inside
// vertex gives a single child, the corner tet at that vertex, which often
// clears the other faces; two or three give three children.  Serial model on
// lattice-like tets, steps per clipped pair with the lowest crossed face
// first / this order: 19.1 / 8.7 at cells half a tet wide, 8.5 / 5.2 at
// tet-sized cells, 4.2 / 3.1 at cells two tets wide.
ADECO_HD inline int next_face(int b0, int b1, int b2, int b3, int done, int &face, int &mask, bool &last)
{
    const int all_in = b0 & b1 & b2 & b3, any_in = b0 | b1 | b2 | b3;
    const int relevant = 63 & ~done;
    if ((~any_in) & relevant) return 0;  // entirely outside a remaining face
    const int next = (~all_in) & relevant;
    if (!next) return 1;
    // per crossed face 1..3 vertices inside: odd -> 1 or 3, `two` -> at least 2
    const int odd = b0 ^ b1 ^ b2 ^ b3;
    const int two = (b0 & b1) | (b2 & b3) | ((b0 | b1) & (b2 | b3));
    int pick = next & odd & ~two;   // one vertex inside
    if (!pick) pick = next & ~odd;  // two inside
    if (!pick) pick = next;         // three inside
#ifdef __CUDA_ARCH__
    face = __ffs(pick) - 1;
#else
    face = __builtin_ctz(pick);
#endif
    mask = ((b0 >> face) & 1) | (((b1 >> face) & 1) << 1) | (((b2 >> face) & 1) << 2) | (((b3 >> face) & 1) << 3);
    last = (next & (next - 1)) == 0;
    return 2;
}

// ---------------------------------------------------- barycentric clipping
// Fraction of a tet's volume inside the unit cube, for tets too flat for the
// FP32 engine.  A flat tet's volume L^2 h, computed from FP32 coordinates as
// a determinant, carries an error ~ 2^-24 L^3 -- relative 2^-24 kappa.  Here
// every piece also carries its barycentric coordinates in the tet (4 weights
// per vertex): clipping is affine, so a cut point's weights follow from the
// same edge parameter t as its coordinates, and a piece's share of the tet is
// the determinant of its weights -- well conditioned whatever the tet's
// shape; the mass is that share times the tet's exact mass.  Face tests, cut
// points (snapped onto the face), splits, last-face fractions and the face
// order are the engine's, on the piece's own coordinates.

// A piece's signed share of the tet: the determinant of its weight
// differences (the weights of vertices 1..3 minus those of vertex 0), from
// exact differences in double-float.  A record carries a vertex's weights
// of tet vertices 1..3 only: the weight of vertex 0 (one minus their sum)
// does not enter the determinant.  Signed: every piece keeps the tet's
// orientation, and |det| would round near-degenerate pieces up and bias the
// sum.
ADECO_HD inline F2 bary_share(const float *w)
{
    F2 d[3][3];
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int i = 0; i < 3; ++i) d[j][i] = f2_two_sum(w[3 * (j + 1) + i], -w[i]);
    const F2 m0 = f2_minor(d[1][1], d[2][2], d[1][2], d[2][1]);
    const F2 m1 = f2_minor(d[1][0], d[2][2], d[1][2], d[2][0]);
    const F2 m2 = f2_minor(d[1][0], d[2][1], d[1][1], d[2][0]);
    const F2 t1 = f2_mul(d[0][1], m1);
    return f2_add(f2_add(f2_mul(d[0][0], m0), {-t1.hi, -t1.lo}), f2_mul(d[0][2], m2));
}

constexpr int kBaryRec = 24;  // a barycentric piece: 12 weights (3 per vertex), then 12 coordinates

// the tet itself: vertex v (1..3) has weight 1 for tet vertex v, vertex 0 none
ADECO_HD inline void bary_identity(float *r)
{
#pragma unroll
    for (int i = 0; i < 12; ++i) r[i] = (i & 3) == 3 ? 1.f : 0.f;  // entries 3, 7, 11
}

// record entry of vertex v's value i (0..2 weights, 3..5 coordinates)
ADECO_HD inline int bary_idx(int v, int i) { return i < 3 ? 3 * v + i : 12 + 3 * v + (i - 3); }

// Split of barycentric piece r by face f (mask: its vertices inside, k of
// them), with split_cut's patterns over the 6 values of a vertex: the
// vertices permuted to A B C D (inside first, even permutation), the cut
// points E0..E3 of the edges k=1: AB AC AD AD; k=2: AC AD BC BD; k=3: AD BD CD
// CD (weights interpolated with the coordinate's edge parameter, the
// coordinate snapped onto the face), and the children
//   c0 = (A, k1 ? E0 : B, k1 ? E1 : (k2 ? E2 : C), k1 ? E2 : (k2 ? E3 : E2))
//   c1 = (A, k2 ? E2 : B, k2 ? E0 : E2, k2 ? E3 : E1)
//   c2 = (A, k2 ? E0 : E1, k2 ? E1 : E2, k2 ? E3 : E0)
// written entry by entry as put(child, record index, value): each child
// vertex is a select between at most three candidates, no lookup.  Returns
// the number of children (1 or 3).
template <typename Put>
ADECO_HD inline int bary_split(const float *r, int f, int mask, Put put)
{
    const int axis = f >> 1;
    const float plane = (f & 1) ? 1.f : 0.f;
    const int pm = split_perm(mask), k = split_kin(mask);
    const bool k1 = k == 1, k2 = k == 2, k3 = k == 3;
    const int ia = pm & 3, ib = (pm >> 2) & 3, ic = (pm >> 4) & 3, id = (pm >> 6) & 3;
    float A[6], B[6], C[6], D[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        const float a0 = r[bary_idx(0, i)], a1 = r[bary_idx(1, i)], a2 = r[bary_idx(2, i)], a3 = r[bary_idx(3, i)];
        A[i] = sel4(ia, a0, a1, a2, a3);
        B[i] = sel4(ib, a0, a1, a2, a3);
        C[i] = sel4(ic, a0, a1, a2, a3);
        D[i] = sel4(id, a0, a1, a2, a3);
    }
    float E[4][6];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        float in[6], out[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            in[i] = e == 0 ? A[i] : (e == 1 ? (k3 ? B[i] : A[i]) : (e == 2 ? (k1 ? A[i] : (k2 ? B[i] : C[i]))
                                                                             : (k2 ? B[i] : (k3 ? C[i] : A[i]))));
            out[i] = e == 0 ? (k1 ? B[i] : (k2 ? C[i] : D[i])) : (e == 1 ? (k1 ? C[i] : D[i])
                                                                          : (e == 2 ? (k2 ? C[i] : D[i]) : D[i]));
        }
        const float xin = sel3(axis, in[3], in[4], in[5]), xout = sel3(axis, out[3], out[4], out[5]);
        const float t = fminf(fmaxf((plane - xin) * rcp_nr(xout - xin), 0.f), 1.f);
#pragma unroll
        for (int i = 0; i < 6; ++i) E[e][i] = (i == 3 + axis) ? plane : fmaf(t, out[i] - in[i], in[i]);
    }
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        put(0, bary_idx(0, i), A[i]);
        put(0, bary_idx(1, i), k1 ? E[0][i] : B[i]);
        put(0, bary_idx(2, i), k1 ? E[1][i] : (k2 ? E[2][i] : C[i]));
        put(0, bary_idx(3, i), k1 ? E[2][i] : (k2 ? E[3][i] : E[2][i]));
        put(1, bary_idx(0, i), A[i]);
        put(1, bary_idx(1, i), k2 ? E[2][i] : B[i]);
        put(1, bary_idx(2, i), k2 ? E[0][i] : E[2][i]);
        put(1, bary_idx(3, i), k2 ? E[3][i] : E[1][i]);
        put(2, bary_idx(0, i), A[i]);
        put(2, bary_idx(1, i), k2 ? E[0][i] : E[1][i]);
        put(2, bary_idx(2, i), k2 ? E[1][i] : E[2][i]);
        put(2, bary_idx(3, i), k2 ? E[3][i] : E[0][i]);
    }
    return k1 ? 1 : 3;
}


// The share inside the unit cube of one barycentric piece rec0 whose faces
// in done0 are already done, clipped serially with a stack.
ADECO_HD
#ifdef __CUDA_ARCH__
__noinline__
#else
inline
#endif
F2 clip_bary_serial(const float *rec0, int done0)
{
    constexpr int kDepth = 16;
    constexpr int kRec = kBaryRec;
    float stk[kDepth][kRec];
    int sdone[kDepth];
    for (int i = 0; i < kRec; ++i) stk[0][i] = rec0[i];
    sdone[0] = done0;
    int sp = 1;
    F2 acc = {0.f, 0.f};
    while (sp > 0) {
        --sp;
        float r[kRec];
#pragma unroll
        for (int i = 0; i < kRec; ++i) r[i] = stk[sp][i];
        const float *w = r, *x = r + 12;
        const int done = sdone[sp];
        int f = 0, mask = 0;
        bool last = false;
        const int code = next_face(face_bits(x[0], x[1], x[2]), face_bits(x[3], x[4], x[5]),
                                   face_bits(x[6], x[7], x[8]), face_bits(x[9], x[10], x[11]), done, f, mask, last);
        if (code == 0) continue;  // beyond a face
        if (code == 1) {
            acc = f2_add(acc, bary_share(w));
            continue;
        }
        const int axis = f >> 1;
        const float plane = (f & 1) ? 1.f : 0.f;
        const float xa[4] = {x[axis], x[3 + axis], x[6 + axis], x[9 + axis]};
        if (last) {  // last crossed face: the inside fraction of the piece
            acc = f2_add(acc, f2_mul_f(bary_share(w), side_fraction(xa[0], xa[1], xa[2], xa[3], mask, plane)));
            continue;
        }
        // split by face f into 1 or 3 pieces (bary_split, as the warp engine)
        const int n = split_kin(mask) == 1 ? 1 : 3;
        if (sp + n > kDepth) continue;  // cannot happen: at most 2 pending pieces per face level
        bary_split(r, f, mask, [&](int ch, int e, float val) {
            if (ch < n) stk[sp + ch][e] = val;
        });
        for (int c = 0; c < n; ++c) {
            sdone[sp] = done | (1 << f);
            ++sp;
        }
    }
    return acc;
}


constexpr int kVolShift = 56;  // fixed point of 6x piece volumes (each <= 6)
static_assert(kVolShift == 56, "vol_fixed scales by 0x1p56f");

ADECO_HD inline long long vol_fixed(float v6)
{
#ifdef __CUDA_ARCH__
    return __float2ll_rn(v6 * 0x1p56f);  // the signed form of to_fixed(|v6|, kVolShift)
#else
    const unsigned long long m = to_fixed(fabsf(v6), kVolShift);
    return v6 < 0.f ? -(long long)m : (long long)m;
#endif
}

ADECO_HD inline float piece_vol6(const float p[12])
{
    return vol6_fast<float>(p, p + 3, p + 6, p + 9);
}

// state of one piece whose faces in `done` are done (next_face): code 0 =
// dropped, 1 = finished, 2 = crossing `face` with inside mask `mask`
ADECO_HD inline int piece_step(const float p[12], int done, int &face, int &mask, bool &last)
{
    return next_face(face_bits(p[0], p[1], p[2]), face_bits(p[3], p[4], p[5]), face_bits(p[6], p[7], p[8]),
                     face_bits(p[9], p[10], p[11]), done, face, mask, last);
}

// Serial clipping of one piece whose faces in `done0` are done (used when the
// warp pool is full): depth-first over the same splits and last-face fractions, so the
// fixed-point sum is the warp engine's.
#ifdef __CUDA_ARCH__
__device__ __noinline__
#else
inline
#endif
long long clip_piece_serial(const float p0[12], int done0)
{
    constexpr int kDepth = 16;  // 2 pending pieces per face level + 3
    float stk[kDepth][12];
    int sdone[kDepth];
#pragma unroll
    for (int x = 0; x < 12; ++x) stk[0][x] = p0[x];
    sdone[0] = done0;
    int sp = 1;
    long long acc = 0;
    while (sp > 0) {
        --sp;
        float p[12];
#pragma unroll
        for (int x = 0; x < 12; ++x) p[x] = stk[sp][x];
        int face = 0, mask = 0;
        bool last = false;
        const int code = piece_step(p, sdone[sp], face, mask, last);
        if (code == 0) continue;
        if (code == 1) {
            acc += vol_fixed(piece_vol6(p));
            continue;
        }
        Cut cut;
        cut_piece(p, mask, face, cut);
        if (last) {
            acc += vol_fixed(piece_vol6(p) * cut_fraction(cut, face));
            continue;
        }
        float c0[12], c1[12], c2[12];
        const int n = split_cut(cut, face, c0, c1, c2);
        if (sp + 3 > kDepth) continue;  // cannot happen (depth <= 2*5 + 3)
        const int d = sdone[sp] | (1 << face);
#pragma unroll
        for (int x = 0; x < 12; ++x) stk[sp][x] = c0[x];
        sdone[sp] = d;
        ++sp;
        if (n == 3) {
#pragma unroll
            for (int x = 0; x < 12; ++x) stk[sp][x] = c1[x];
            sdone[sp] = d;
            ++sp;
#pragma unroll
            for (int x = 0; x < 12; ++x) stk[sp][x] = c2[x];
            sdone[sp] = d;
            ++sp;
        }
    }
    return acc;
}

#ifdef __CUDACC__
constexpr int kPool = 56;    // pieces per warp pool (2 CTAs of 8 warps fit in an SM's shared memory)
constexpr int kPairs = 128;  // partial pairs per warp list

struct WarpPool {
    float4 v[kPool][3];       // a piece's 12 coordinates per slot: 48 bytes, moved as three 16-byte words
    uint32_t meta[kPool];     // owner | faces done << 8
    long long vacc[kPairs];   // 6x volume of each listed pair, fixed point 2^kVolShift
};

// Clip the warp's list of np partial pairs: an idle lane takes a piece from
// the pool (last in, first out) or, when the pool is empty, the next pair of
// the list (build(j, p) writes its tet in cell coordinates).  Each step a
// lane makes at most one split: at the piece's last crossed face the
// children are summed in place, otherwise one child is kept and the others
// pushed.  On return pool.vacc[0..np) hold the pairs' 6x volumes.
template <typename Build>
__device__ __forceinline__ void clip_pairs(WarpPool &pool, int np, Build build, unsigned &fallbacks)
{
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1;
    for (int j = lane; j < np; j += 32) pool.vacc[j] = 0;
    __syncwarp();
    bool valid = false;
    float p[12];
    int owner = 0, done = 0;  // the piece's pair and its faces done (one bit per face)
    int top = 0, next = 0;
    for (;;) {
        // refill idle lanes
        const unsigned need = __ballot_sync(0xffffffffu, !valid);
        const int rank = __popc(need & lt), nneed = __popc(need);
        if (!valid) {
            if (rank < top) {
                const int idx = top - 1 - rank;
#pragma unroll
                for (int w = 0; w < 3; ++w) {
                    const float4 q = pool.v[idx][w];
                    p[4 * w] = q.x;
                    p[4 * w + 1] = q.y;
                    p[4 * w + 2] = q.z;
                    p[4 * w + 3] = q.w;
                }
                const uint32_t m = pool.meta[idx];
                owner = (int)(m & 0xff);
                done = (int)(m >> 8);
                valid = true;
            } else {
                const int j = next + rank - top;
                if (j < np) {
                    build(j, p);
                    owner = j;
                    done = 0;
                    valid = true;
                }
            }
        }
        const int from_pool = nneed < top ? nneed : top;
        top -= from_pool;
        next = min(np, next + (nneed - from_pool));
        const unsigned held = __ballot_sync(0xffffffffu, valid);
        if (!held) break;
        __syncwarp();  // the pool slots just read may be written by this step's pushes
        // one step.  A lane about to split into three reserves room in the
        // pool for its two extra children first: in lane order, as many as
        // fit.  A lane whose children do not fit keeps its piece and steps
        // again next round, while the other lanes finish pieces and idle lanes
        // drain the pool.  Only when every lane holds a piece and none can
        // move does one lane clip its piece alone (serially, with a local
        // stack): letting every pushing lane of a full pool do that had put
        // most of the fine-grid time into one-lane serial clipping.
        int f = 0, mask = 0, code = 0;
        bool last = false;
        if (valid) code = piece_step(p, done, f, mask, last);
        const bool split = valid && code == 2 && !last;
        const bool push = split && split_kin(mask) != 1;  // two children to push
        const unsigned pushing = __ballot_sync(0xffffffffu, push);
        const int fit = (kPool - top) >> 1;  // pushing lanes whose children fit
        const int prank = __popc(pushing & lt);
        const bool defer = push && prank >= fit;
        const int nfit = min(__popc(pushing), fit);
        const bool stuck = held == 0xffffffffu && pushing == 0xffffffffu && fit == 0;
        if (valid && !defer) {
            long long v = 0;
            // the cut is shared by the lanes that split and the lanes at
            // their last crossed face, so the warp runs it once per step
            float frac = 1.f;
            Cut cut;
            if (code == 2) cut_piece(p, mask, f, cut);
            if (split) {
                float c0[12], c1[12], c2[12];
                split_cut(cut, f, c0, c1, c2);
#pragma unroll
                for (int x = 0; x < 12; ++x) p[x] = c0[x];
                done |= 1 << f;
                if (push) {
                    // second children in one block, third children in the
                    // next: consecutive pushing lanes write slots 48 bytes
                    // apart, which spreads a quarter-warp's 16-byte words
                    // over all banks
                    const int s1 = top + prank, s2 = top + nfit + prank;
                    const uint32_t m = (uint32_t)owner | ((uint32_t)done << 8);
#pragma unroll
                    for (int w = 0; w < 3; ++w) {
                        pool.v[s1][w] = make_float4(c1[4 * w], c1[4 * w + 1], c1[4 * w + 2], c1[4 * w + 3]);
                        pool.v[s2][w] = make_float4(c2[4 * w], c2[4 * w + 1], c2[4 * w + 2], c2[4 * w + 3]);
                    }
                    pool.meta[s1] = m;
                    pool.meta[s2] = m;
                }
            } else {
                // finished, or at its last crossed face: the inside part
                // needs no more clipping, so its volume is added here
                if (code == 2) frac = cut_fraction(cut, f);
                if (code != 0) v = vol_fixed(piece_vol6(p) * frac);
                valid = false;
            }
            if (v) atomicAdd(reinterpret_cast<unsigned long long *>(&pool.vacc[owner]), (unsigned long long)v);
        } else if (stuck && lane == 0) {
            // a copy made here: handing p itself to the out-of-line routine
            // takes its address, and p then lives in local memory, stored
            // there on every step although this branch almost never runs
            float q[12];
#pragma unroll
            for (int x = 0; x < 12; ++x) q[x] = p[x];
            const long long acc = clip_piece_serial(q, done);
            atomicAdd(reinterpret_cast<unsigned long long *>(&pool.vacc[owner]), (unsigned long long)acc);
            valid = false;
            ++fallbacks;
        }
        top += 2 * nfit;
        __syncwarp();
    }
    __syncwarp();
}

// ------------------------------------------- barycentric warp engine
// clip_pairs for barycentric pieces (kBaryRec floats each): the partial cells
// of the ill-conditioned tets are listed per warp and clipped with every lane
// busy, a lane per piece, instead of a lane per cell.  Steps, faces, cut
// points, children and last-face fractions are clip_bary_serial's; a lane's
// piece stays in registers (the vertex permutation and the child patterns
// are selects, not indexed loads).
constexpr int kBaryPool = 128;  // pieces per warp pool
constexpr int kBaryList = 64;  // partial cells per warp list

struct BaryPool {
    float v[kBaryRec][kBaryPool];
    uint32_t meta[kBaryPool];  // owner | faces done << 8
    long long acc[kBaryList];  // share of each listed cell, fixed point 2^kVolShift
    uint32_t cell[kBaryList];  // the listed cells (the caller's encoding)
};


// next_face of a barycentric piece whose faces in `done` are done
__device__ __forceinline__ int bary_step(const float *r, int done, int &face, int &mask, bool &last)
{
    return next_face(face_bits(r[12], r[13], r[14]), face_bits(r[15], r[16], r[17]), face_bits(r[18], r[19], r[20]),
                     face_bits(r[21], r[22], r[23]), done, face, mask, last);
}

__device__ __forceinline__ float bary_last_fraction(const float *r, int f, int mask)
{
    const int axis = f >> 1;
    const float plane = (f & 1) ? 1.f : 0.f;
    return side_fraction(sel3(axis, r[12], r[13], r[14]), sel3(axis, r[15], r[16], r[17]),
                         sel3(axis, r[18], r[19], r[20]), sel3(axis, r[21], r[22], r[23]), mask, plane);
}

__device__ __forceinline__ long long share_fixed(F2 c)
{
    return vol_fixed(c.hi) + vol_fixed(c.lo);
}

// Clip the warp's np listed cells: build(j, r) writes cell j's piece (the
// tet in the cell's frame with identity weights).  On return pool.acc[0..np)
// hold the cells' shares of the tet in fixed point 2^kVolShift.
template <typename Build>
__device__ __forceinline__ void clip_bary_pairs(BaryPool &pool, int np, Build build, unsigned &fallbacks)
{
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1;
    for (int j = lane; j < np; j += 32) pool.acc[j] = 0;
    __syncwarp();
    bool valid = false;
    float r[kBaryRec];
    int owner = 0, done = 0;  // the piece's cell and its faces done (one bit per face)
    int top = 0, next = 0;
    for (;;) {
        // refill idle lanes: pool first (last in, first out), then the list
        const unsigned need = __ballot_sync(0xffffffffu, !valid);
        const int rank = __popc(need & lt), nneed = __popc(need);
        if (!valid) {
            if (rank < top) {
                const int idx = top - 1 - rank;
#pragma unroll
                for (int x = 0; x < kBaryRec; ++x) r[x] = pool.v[x][idx];
                const uint32_t m = pool.meta[idx];
                owner = (int)(m & 0xff);
                done = (int)(m >> 8);
                valid = true;
            } else {
                const int j = next + rank - top;
                if (j < np) {
                    build(j, r);
                    owner = j;
                    done = 0;
                    valid = true;
                }
            }
        }
        const int from_pool = nneed < top ? nneed : top;
        top -= from_pool;
        next = min(np, next + (nneed - from_pool));
        const unsigned held = __ballot_sync(0xffffffffu, valid);
        if (!held) break;
        __syncwarp();  // the pool slots just read may be written by this step's pushes
        // one step, with the main engine's pool reservation: a lane whose two
        // extra children do not fit keeps its piece for the next round; one
        // lane clips serially only when every lane holds a piece and none can
        // move
        int f = 0, mask = 0, code = 0;
        bool last = false;
        if (valid) code = bary_step(r, done, f, mask, last);
        const bool want_split = valid && code == 2 && !last;
        const bool push = want_split && split_kin(mask) != 1;
        const unsigned pushing = __ballot_sync(0xffffffffu, push);
        const int fit = (kBaryPool - top) >> 1;
        const int prank = __popc(pushing & lt);
        const bool defer = push && prank >= fit;
        const int nfit = min(__popc(pushing), fit);
        const bool stuck = held == 0xffffffffu && pushing == 0xffffffffu && fit == 0;
        if (valid && !defer) {
            F2 c = {0.f, 0.f};
            if (want_split) {
                // the children of r: the first replaces r, the others go to
                // the pool (written after every entry of r has been read)
                const int base = top + 2 * prank;
                bary_split(r, f, mask, [&](int ch, int x, float val) {
                    if (ch == 0) r[x] = val;  // after bary_split's last read of r
                    else if (push) pool.v[x][base + ch - 1] = val;
                });
                done |= 1 << f;
                if (push) {
                    const uint32_t m = (uint32_t)owner | ((uint32_t)done << 8);
                    pool.meta[base] = m;
                    pool.meta[base + 1] = m;
                }
            } else {
                if (code == 1) c = bary_share(r);
                if (code == 2) c = f2_mul_f(bary_share(r), bary_last_fraction(r, f, mask));
                valid = false;
            }
            const long long v = share_fixed(c);
            if (v) atomicAdd(reinterpret_cast<unsigned long long *>(&pool.acc[owner]), (unsigned long long)v);
        } else if (stuck && lane == 0) {
            float q[kBaryRec];  // a copy, so that r itself never needs an address (see clip_pairs)
#pragma unroll
            for (int x = 0; x < kBaryRec; ++x) q[x] = r[x];
            atomicAdd(reinterpret_cast<unsigned long long *>(&pool.acc[owner]),
                      (unsigned long long)share_fixed(clip_bary_serial(q, done)));
            valid = false;
            ++fallbacks;
        }
        top += 2 * nfit;
        __syncwarp();
    }
    __syncwarp();
}
#endif

}  // namespace adeco
