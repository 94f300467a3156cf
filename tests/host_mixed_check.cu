// Host check of the mixed path's per-pair arithmetic against FP64 clipping
// (built for the host only; no GPU).  Seeded random lattice-like tets (unit
// lattice cubes with displaced corners) over grids whose cells are 1/4 to 2
// lattice spacings, origins shifted so that tets land anywhere relative to
// cell faces.  Each tet goes through setup_tet; each candidate pair through
// classify_pair and then the closed form (one face) or the clip engine's
// steps (clip_piece_serial on piece_coords, the frame the GPU engine uses).
// The FP64 reference clips the FP64 tet against the same cell.
// Prints the worst errors and exits non-zero if a bound is broken.
#include "../adeco_gb300/csrc/kernels.cuh"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>

using namespace adeco;

static GridDesc grid(const float bbox[6], int dims)
{
    GridDesc g;
    std::memset(&g, 0, sizeof g);
    for (int a = 0; a < 3; ++a) {
        g.gmin[a] = bbox[2 * a];
        g.gmax[a] = bbox[2 * a + 1];
        g.delta[a] = (g.gmax[a] - g.gmin[a]) / (float)dims;
        g.gmin_d[a] = (double)g.gmin[a];
        g.delta_d[a] = ((double)g.gmax[a] - (double)g.gmin[a]) / (double)dims;
    }
    const double s = 1.0 / g.delta_d[0];
    for (int a = 0; a < 3; ++a) g.scale_d[a] = s;
    g.mass_factor = g.delta_d[0] * g.delta_d[1] * g.delta_d[2] * s * s * s;
    for (int a = 0; a < 3; ++a) {
        g.rcell[a] = g.delta_d[a] * g.scale_d[a];
        g.inv_rcell[a] = 1.0 / g.rcell[a];
        g.drcell[a] = (float)(g.rcell[a] - 1.0);
        g.inv_rcell_f[a] = (float)g.inv_rcell[a];
        g.tile_lo[a] = 0;
        g.tile_hi[a] = dims - 1;
        g.cull_min[a] = g.gmin[a];
        g.cull_max[a] = g.gmax[a];
    }
    g.tet_mass = 1.f;
    for (int a = 0; a < 3; ++a) {
        g.scale_hi[a] = (float)g.scale_d[a];
        g.scale_lo[a] = (float)(g.scale_d[a] - (double)g.scale_hi[a]);
    }
    g.mf_hi = (float)g.mass_factor;
    g.mf_lo = (float)(g.mass_factor - (double)g.mf_hi);
    g.dims = dims;
    return g;
}

int main()
{
    std::mt19937_64 rng(2024);
    std::normal_distribution<double> N(0.0, 0.2);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    static WarpTets W, W2;
    const double cell_sizes[4] = {0.25, 0.5, 1.0, 2.0};
    double worst_rel = 0.0, worst_abs = 0.0, sum_err = 0.0, sum_mass = 0.0;
    double wr[3] = {0, 0, 0}, wa[3] = {0, 0, 0};  // by path: 0 exact classes, 1 one-face closed form, 2 clipped
    long npath[3] = {0, 0, 0};
    long pairs = 0, partial = 0, tets = 0, lazy_diff = 0;
    for (int trial = 0; trial < 4000; ++trial) {
        const double dx = cell_sizes[trial % 4];
        const int dims = 16;
        const float x0 = (float)(-4.0 - U(rng) * dx), y0 = (float)(-4.0 - U(rng) * dx), z0 = (float)(-4.0 - U(rng) * dx);
        const float bbox[6] = {x0, (float)(x0 + dims * dx), y0, (float)(y0 + dims * dx), z0, (float)(z0 + dims * dx)};
        const GridDesc g = grid(bbox, dims);
        // one displaced lattice cube near the origin
        float3 corner[8];
        for (int s = 0; s < 8; ++s) {
            const int3 o = corner_offset(ORDER_REF, s);
            corner[s] = make_float3((float)(o.x + N(rng)), (float)(o.y + N(rng)), (float)(o.z + N(rng)));
        }
        for (int t = 0; t < 6; ++t) {
            float3 v[4];
            for (int q = 0; q < 4; ++q) v[q] = corner[tet_conn(t, q)];
            float gh[4][3], gl[4][3];
            for (int q = 0; q < 4; ++q) {
                grid_frame(v[q].x, g.gmin[0], g.scale_hi[0], g.scale_lo[0], gh[q][0], gl[q][0]);
                grid_frame(v[q].y, g.gmin[1], g.scale_hi[1], g.scale_lo[1], gh[q][1], gl[q][1]);
                grid_frame(v[q].z, g.gmin[2], g.scale_hi[2], g.scale_lo[2], gh[q][2], gl[q][2]);
            }
            bool r64 = false;
            int err = 0;
            const int cnt = setup_tet(v, gh, gl, g, W, 0, &err, &r64);
            if (cnt <= 0 || r64) continue;
            // the octree-leaf form: FP32 plane offsets, exact ones formed by the closed form itself
            bool r64b = false;
            setup_tet<false>(v, gh, gl, g, W2, 0, &err, &r64b);
            ++tets;
            // the FP64 tet, positively oriented, in scaled grid units
            double T[4][3];
            for (int q = 0; q < 4; ++q) {
                const double x[3] = {(double)v[q].x, (double)v[q].y, (double)v[q].z};
                for (int a = 0; a < 3; ++a) T[q][a] = (x[a] - g.gmin_d[a]) * g.scale_d[a];
            }
            const double v6 = vol6_fast<double>(T[0], T[1], T[2], T[3]);
            if (v6 < 0)
                for (int a = 0; a < 3; ++a) std::swap(T[0][a], T[3][a]);
            const double f6 = g.mass_factor / std::fabs(v6);
            for (int c = 0; c < W.ex[2][0]; ++c)
                for (int b = 0; b < W.ex[1][0]; ++b)
                    for (int a = 0; a < W.ex[0][0]; ++a) {
                        bool f64 = false;
                        int cross = -1;
                        const int cls = classify_pair(W, g, 0, a, b, c, f64, cross);
                        double dm = 0.0;
                        int path = 0;
                        if (cls == P_TET_INSIDE) {
                            dm = 1.0;
                        } else if (cls == P_CELL_INSIDE) {
                            dm = (double)(6.f * W.f6[0]);
                        } else if (cls == P_PARTIAL) {
                            // the GPU's FP32 pair masses (then converted to fixed point exactly)
                            if (cross >= 0) {
                                dm = (double)(halfspace_pair_vol6(W, g, 0, a, b, c, cross) * W.f6[0]);
                                path = 1;
                                lazy_diff += halfspace_pair_vol6<false>(W2, g, 0, a, b, c, cross) !=
                                             halfspace_pair_vol6<true>(W, g, 0, a, b, c, cross);
                            } else {
                                path = 2;
                                float p[12];
                                piece_coords(W, g, 0, a, b, c, p);
                                const long long v = clip_piece_serial(p, 0);
                                dm = v > 0 ? (double)pair_mass(v, W.f6[0]) : 0.0;
                                ++partial;
                            }
                        }
                        const int cell[3] = {W.lo[0][0] + a, W.lo[1][0] + b, W.lo[2][0] + c};
                        double P[4][3];
                        for (int q = 0; q < 4; ++q)
                            for (int x = 0; x < 3; ++x) P[q][x] = T[q][x] - (double)cell[x] * g.rcell[x];
                        const double ref = clip_volume6<double, double>(P) * f6;
                        const double e = std::fabs(dm - ref);
                        ++pairs;
                        sum_err += dm - ref;
                        sum_mass += ref;
                        worst_abs = std::fmax(worst_abs, e);
                        if (ref > 1e-3) worst_rel = std::fmax(worst_rel, e / ref);
                        if (cls != P_NO) ++npath[path];
                        wa[path] = std::fmax(wa[path], e);
                        if (ref > 1e-3) wr[path] = std::fmax(wr[path], e / ref);
                    }
        }
    }
    std::printf("tets %ld, pairs %ld (%ld clipped): worst relative error %.3e (pairs above 1e-3 tet masses), "
                "worst absolute %.3e tet masses, summed error %.3e of %.1f\n",
                tets, pairs, partial, worst_rel, worst_abs, sum_err, sum_mass);
    const char *names[3] = {"inside / holding", "one-face closed form", "clipped"};
    for (int k = 0; k < 3; ++k)
        std::printf("  %s (%ld pairs): worst relative %.3e, worst absolute %.3e\n", names[k], npath[k], wr[k], wa[k]);
    // Bounds, per pair: the clip engine's FP32 steps (worst 1.4e-5 relative on pairs above 1e-3 tet
    // masses, 1e-6 absolute: slices under an upper face of tets that also cross the lower face);
    // the closed form (3.7e-6, 3.7e-8).  The summed error is the noise of the per-pair errors: over
    // 16 seeds of this sample it is -1.2e-10 +- 5.7e-10 (s.d.) of the mass, for either face order of
    // next_face, with no bias to detect at this size; the bound, 2e-9, is 3.5 s.d.
    std::printf("  closed form with the plane offsets formed per pair: %ld of %ld pairs differ\n", lazy_diff, npath[1]);
    const bool ok = wr[2] < 5e-5 && wa[2] < 2e-6 && wr[1] < 2e-5 && wa[1] < 2e-7 && wr[0] < 1e-6 && wa[0] < 1e-6 &&
                    std::fabs(sum_err) < 2e-9 * sum_mass && lazy_diff == 0;
    std::printf("%s\n", ok ? "ok" : "FAIL");
    return ok ? 0 : 1;
}
