// Host-side checks of the FP32 helpers the mixed path relies on (built for
// the host only; no GPU needed).  Prints one line per check, "ok" or the
// first failure, and exits non-zero on any failure.
//   1. cell_coord_sel == cell_coord / cell_coord_mirrored, bit for bit;
//   2. the mirrored coordinate is 1 - x to within its own final rounding;
//   3. double-float: TwoSum and TwoProd are exact, a share of identity
//      weights is exactly 1.
#include "../adeco_gb300/csrc/kernels.cuh"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>

using namespace adeco;

static bool same_bits(float a, float b) { return std::memcmp(&a, &b, sizeof a) == 0; }

int main()
{
    int failures = 0;
    std::mt19937_64 rng(7);
    std::uniform_real_distribution<double> U(-300.0, 300.0), D(-3e-7, 3e-7), F(-4.0, 4.0);

    long bad_sel = 0, bad_mirror = 0;
    for (long i = 0; i < 2000000; ++i) {
        const double q = U(rng);
        const float hi = (float)q, lo = (float)(q - (double)hi);
        const int c = (int)(rng() % 400) - 50;
        const float dr = (float)D(rng);
        const float x = cell_coord(hi, lo, c, dr), y = cell_coord_mirrored(hi, lo, c, dr);
        if (!same_bits(x, cell_coord_sel(hi, lo, c, dr, false)) || !same_bits(y, cell_coord_sel(hi, lo, c, dr, true)))
            ++bad_sel;
        // exact 1 - x with the low part rounded as the helpers round it
        const double low = (double)sub_rn(mul_rn((float)c, dr), lo);
        const double want = (double)(c + 1) - (double)hi + low;
        if (std::fabs((double)y - want) > 0.5 * std::ldexp(1.0, std::ilogb((double)y) - 23) + 1e-30) ++bad_mirror;
    }
    std::printf("cell_coord_sel bit-exact: %s (%ld mismatches)\n", bad_sel ? "FAIL" : "ok", bad_sel);
    std::printf("mirrored coordinate = 1 - x within its rounding: %s (%ld)\n", bad_mirror ? "FAIL" : "ok", bad_mirror);
    failures += (bad_sel != 0) + (bad_mirror != 0);

    long bad_sum = 0, bad_prod = 0;
    for (long i = 0; i < 2000000; ++i) {
        const float a = (float)F(rng), b = (float)std::ldexp(F(rng), (int)(rng() % 40) - 20);
        const F2 s = f2_two_sum(a, b);
        if ((double)s.hi + (double)s.lo != (double)a + (double)b) ++bad_sum;
        const F2 p = f2_mul({a, 0.f}, {b, 0.f});
        if ((double)p.hi + (double)p.lo != (double)a * (double)b) ++bad_prod;
    }
    std::printf("double-float TwoSum exact: %s (%ld)\n", bad_sum ? "FAIL" : "ok", bad_sum);
    std::printf("double-float TwoProd exact: %s (%ld)\n", bad_prod ? "FAIL" : "ok", bad_prod);
    failures += (bad_sum != 0) + (bad_prod != 0);

    float w[12];
    bary_identity(w);
    const F2 one = bary_share(w);
    const bool ok_share = one.hi == 1.f && one.lo == 0.f;
    std::printf("share of identity weights == 1: %s\n", ok_share ? "ok" : "FAIL");
    failures += !ok_share;

    // the packed-immediate lookups equal the tables they stand for
    int bad_tab = 0;
    for (int m = 0; m < 16; ++m) bad_tab += (split_perm(m) != h_split_perm[m]) + (split_kin(m) != h_split_kin[m]);
    for (int t = 0; t < 6; ++t)
        for (int q = 0; q < 4; ++q) bad_tab += tet_conn(t, q) != h_tet_conn[t][q];
    for (int c = 0; c < 8; ++c)
        for (int a = 0; a < 3; ++a) bad_tab += ref_corner(c, a) != h_ref_corner[c][a];
    std::printf("packed table lookups equal the tables: %s (%d)\n", bad_tab ? "FAIL" : "ok", bad_tab);
    failures += bad_tab != 0;

    // pair_mass: one rounding of the fixed-point sum, no drift from truncation
    double pm_bias = 0.0, pm_total = 0.0;
    std::uniform_real_distribution<double> U01(0.0, 1.0);
    for (long i = 0; i < 1000000; ++i) {
        const long long v = vol_fixed((float)(U01(rng) * 6.0)) + vol_fixed((float)(U01(rng) * 0.5));
        const float f6 = (float)(0.1 + U01(rng));
        const double x = std::ldexp((double)v, -kVolShift) * (double)f6;
        pm_bias += (double)pair_mass(v, f6) - x;
        pm_total += x;
    }
    const bool ok_pm = std::fabs(pm_bias) < 1e-10 * pm_total;
    std::printf("pair_mass unbiased: %s (%.2e relative)\n", ok_pm ? "ok" : "FAIL", pm_bias / pm_total);
    failures += !ok_pm;
    return failures ? 1 : 0;
}
