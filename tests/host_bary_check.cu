// Host check of the barycentric clipping used for ill-conditioned (flat)
// tets, against FP64 clipping (built for the host only; no GPU).  Seeded
// random flat tets -- a triangle of extent ~3 cells lifted by h = 1e-2 ..
// 1e-4 of that extent to a fourth vertex -- over the cells of their range.
// The piece is formed as the route does (FP64 anchor frame split into FP32
// hi + lo, cell coordinates mirrored along axes whose lower face the tet does
// not reach, identity weights) and clipped by clip_bary_serial, whose steps,
// cut points and double-float shares are the warp engine's.  The share times
// the tet's mass is compared with the FP64 clip of the FP64 tet.
#include "../adeco_gb300/csrc/clip_engine.cuh"

#include <cmath>
#include <cstdio>
#include <random>

using namespace adeco;

int main()
{
    std::mt19937_64 rng(99);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    const double heights[3] = {1e-2, 1e-3, 1e-4};
    double worst_rel[3] = {0, 0, 0}, worst_abs[3] = {0, 0, 0}, sum_err[3] = {0, 0, 0}, sum_mass[3] = {0, 0, 0};
    double worst_coord_rel[3] = {0, 0, 0};  // the FP32 coordinate determinant, for comparison
    long cells = 0;
    for (int trial = 0; trial < 3000; ++trial) {
        const int hk = trial % 3;
        // flat tet in cell units, anchored near the origin of a 6^3 block
        double T[4][3];
        for (int q = 0; q < 3; ++q)
            for (int a = 0; a < 3; ++a) T[q][a] = 1.0 + 3.0 * U(rng);
        double n[3];
        {
            const double e1[3] = {T[1][0] - T[0][0], T[1][1] - T[0][1], T[1][2] - T[0][2]};
            const double e2[3] = {T[2][0] - T[0][0], T[2][1] - T[0][1], T[2][2] - T[0][2]};
            n[0] = e1[1] * e2[2] - e1[2] * e2[1];
            n[1] = e1[2] * e2[0] - e1[0] * e2[2];
            n[2] = e1[0] * e2[1] - e1[1] * e2[0];
            const double ln = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
            if (ln < 1e-3) continue;
            for (int a = 0; a < 3; ++a) n[a] /= ln;
        }
        const double h = heights[hk] * 3.0;
        const double w0 = U(rng), w1 = U(rng) * (1.0 - w0), w2 = 1.0 - w0 - w1;
        for (int a = 0; a < 3; ++a) T[3][a] = w0 * T[0][a] + w1 * T[1][a] + w2 * T[2][a] + h * n[a];
        // FP32 vertices (the data), then everything from them
        float F[4][3];
        double D[4][3];
        for (int q = 0; q < 4; ++q)
            for (int a = 0; a < 3; ++a) {
                F[q][a] = (float)T[q][a];
                D[q][a] = (double)F[q][a];
            }
        double v6 = vol6_fast<double>(D[0], D[1], D[2], D[3]);
        if (v6 < 0) {
            for (int a = 0; a < 3; ++a) {
                std::swap(D[0][a], D[3][a]);
                std::swap(F[0][a], F[3][a]);
            }
            v6 = -v6;
        }
        if (!(v6 > 0)) continue;
        float qf[4][3], ql[4][3], bmin[3] = {1e30f, 1e30f, 1e30f};
        for (int q = 0; q < 4; ++q)
            for (int a = 0; a < 3; ++a) {
                qf[q][a] = (float)D[q][a];
                ql[q][a] = (float)(D[q][a] - (double)qf[q][a]);
                bmin[a] = std::fmin(bmin[a], qf[q][a]);
            }
        for (int k = 0; k < 6; ++k)
            for (int j = 0; j < 6; ++j)
                for (int i = 0; i < 6; ++i) {
                    const int cc[3] = {i, j, k};
                    double P[4][3];
                    for (int q = 0; q < 4; ++q)
                        for (int a = 0; a < 3; ++a) P[q][a] = D[q][a] - cc[a];
                    const double ref = clip_volume6<double, double>(P) / v6;
                    if (ref <= 0.0) continue;
                    float rec[kBaryRec], X[4][3];
                    bary_identity(rec);
                    for (int a = 0; a < 3; ++a) {
                        const bool flip = bmin[a] > (float)cc[a];
                        for (int q = 0; q < 4; ++q) {
                            rec[12 + 3 * q + a] = cell_coord_sel(qf[q][a], ql[q][a], cc[a], 0.f, flip);
                            X[q][a] = cell_coord(qf[q][a], ql[q][a], cc[a], 0.f);
                        }
                    }
                    const F2 sh = clip_bary_serial(rec, 0);
                    const double got = (double)sh.hi + (double)sh.lo;
                    // the same cell by the FP32 coordinate engine, for comparison
                    float p[12];
                    for (int q = 0; q < 4; ++q)
                        for (int a = 0; a < 3; ++a) p[3 * q + a] = X[q][a];
                    const float fv6 = vol6_fast<float>(p, p + 3, p + 6, p + 9);
                    const double coord = std::ldexp((double)clip_piece_serial(p, 0), -kVolShift) / (double)fv6;
                    const double e = std::fabs(got - ref);
                    ++cells;
                    sum_err[hk] += got - ref;
                    sum_mass[hk] += ref;
                    worst_abs[hk] = std::fmax(worst_abs[hk], e);
                    if (ref > 1e-3) {
                        worst_rel[hk] = std::fmax(worst_rel[hk], e / ref);
                        worst_coord_rel[hk] = std::fmax(worst_coord_rel[hk], std::fabs(coord - ref) / ref);
                    }
                }
    }
    bool ok = cells > 10000;
    std::printf("cells %ld\n", cells);
    for (int hk = 0; hk < 3; ++hk) {
        std::printf("thickness %.0e: barycentric worst relative %.3e (fractions above 1e-3), worst absolute %.3e, "
                    "summed %.3e of %.1f; FP32 coordinate determinant worst relative %.3e\n",
                    heights[hk], worst_rel[hk], worst_abs[hk], sum_err[hk], sum_mass[hk], worst_coord_rel[hk]);
        // measured: 3.6e-6 / 6.3e-6 / 1.2e-5 worst relative, sums within 1.2e-9 of the mass; the FP32
        // coordinate determinant is 16-570x worse, which is why such tets take this route
        ok = ok && worst_rel[hk] < 5e-5 && std::fabs(sum_err[hk]) < 1e-8 * sum_mass[hk] &&
             worst_coord_rel[hk] > 4.0 * worst_rel[hk];
    }
    std::printf("%s\n", ok ? "ok" : "FAIL");
    return ok ? 0 : 1;
}
