// Host check of the FP32 fast path's decisions against the exact f64 trace.
//
// Compiles the product's model header for the host and, for every (wavelength,
// sorted ray) of the given points, compares fast_ray -- run on the host, with IEEE
// single-precision sqrt and division where the device uses its approximate MUFU
// instructions -- with the exact trace: a ray the fast path reports HIT or LOST must
// have the exact outcome and bin. Rays it flags are re-traced on the device and are
// only counted. The float-float re-trace (trace_df) is checked on every ray: same
// outcome and bin as the exact trace, transmittance within 2e-6 relative.
//
// usage: fastpath_check design.bin W R lam_u.bin ray_u.bin
// prints: rays <n> mismatches <m> flagged <f> outside_band_hits <h> df_mismatches <d>
//         fast_t_relerr_e9 <e> (largest relative t error of a fast-path hit, x 1e9, rounded up)
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "cpd_df.h"
#include "cpd_host.h"
#include "cpd_model.h"

using namespace cpd;

int main(int argc, char **argv)
{
    if (argc < 6) return 2;
    cpd_design d;
    FILE *f = std::fopen(argv[1], "rb");
    if (!f || std::fread(&d, sizeof d, 1, f) != 1) return 3;
    std::fclose(f);
    const int W = std::atoi(argv[2]), R = std::atoi(argv[3]);
    std::vector<double> lu(W), ru(R);
    f = std::fopen(argv[4], "rb");
    if (!f || std::fread(lu.data(), 8, W, f) != (size_t)W) return 3;
    std::fclose(f);
    f = std::fopen(argv[5], "rb");
    if (!f || std::fread(ru.data(), 8, R, f) != (size_t)R) return 3;
    std::fclose(f);
    DevDesign D;
    design_to_dev(d, D);
    std::vector<double> z64;
    std::vector<float> z32;
    ray_table(ru.data(), R, z64, z32);
    long n = 0, mism = 0, flag = 0, outside = 0, dfmism = 0;
    double terr = 0.0;  // largest |t_fast - t| / t over fast-path hits
    for (int k = 0; k < W; k++) {
        const double lam = x::wavelength(D, lu[k]);
        LamParams P;
        LamDF E;
        lambda_setup_df(D, lu[k], z32.data(), (uint32_t)z64.size(), P, kYGuardRel, &E);
        for (uint32_t j = 0; j < z64.size(); j++) {
            n++;
            uint32_t b = 0;
            double t = 0;
            const int e = x::trace(D, lam, x::beam_y(D, z64[j]), b, t);
            // the float-float re-trace must decide every ray like the exact trace
            uint32_t bd = 0;
            float td = 0.f;
            const bool hd = trace_df(D, E, z32[2 * j], z32[2 * j + 1], bd, td);
            if (hd != (e == 0) || (hd && (bd != b || std::fabs(td - t) > 2e-6 * t))) dfmism++;
            const bool in_band = j >= P.band_lo && j < P.band_hi;
            if (!in_band) {
                outside += e == 0;
                continue;
            }
            if (j < P.core_lo || j >= P.core_hi || P.all_exact) continue;
            uint32_t bf = 0;
            float tf = 0;
            const int r = fast_ray(D.fc, P, default_guards(), z32[2 * j], z32[2 * j + 1], bf, tf);
            if (r == RAY_FLAG) {
                flag++;
                continue;
            }
            if ((r == RAY_HIT) != (e == 0) || (r == RAY_HIT && bf != b)) mism++;
            if (r == RAY_HIT && e == 0) terr = std::fmax(terr, std::fabs((double)tf - t) / t);
        }
    }
    std::printf("rays %ld mismatches %ld flagged %ld outside_band_hits %ld df_mismatches %ld fast_t_relerr_e9 %ld\n", n,
                mism, flag, outside, dfmism, (long)std::ceil(terr * 1e9));
    return 0;
}
