// cpd_host.h -- host-side helpers shared by the C ABI translation units.
#pragma once

#include <cstdint>
#include <memory>
#include <vector>

#include "../../include/cpd.h"

namespace cpd {
struct DevDesign;

int build_prism(const cpd_spectrometer_params &p, cpd_design &d);
void design_to_dev(const cpd_design &d, DevDesign &D);
double norminv(double u);
// Sorted ray table: z = norminv(u) ascending, non-finite values dropped; z32 holds
// the f32 (hi, lo) split of each z, interleaved.
// rank (optional): for each ray index j, its position in the sorted table (~0u if its
// start height is not finite).
void ray_table(const double *ray_u, uint32_t R, std::vector<double> &z64, std::vector<float> &z32,
               std::vector<uint32_t> *rank = nullptr);
// u_i = fract(fma(first + i, 1/phi, seed)), i < n.
void seed_points(double seed, uint32_t first, uint32_t n, double *out);

// A sorted ray table with its f32 split and rank (see ray_table).
struct RayTable {
    std::vector<double> z64;
    std::vector<float> z32;
    std::vector<uint32_t> rank;  // ray index -> sorted position (adaptive sampling)
};
using RayTablePtr = std::shared_ptr<const RayTable>;
using LamPtr = std::shared_ptr<const std::vector<double>>;

// What other translation units need of a context (cpd_runtime.cu): its device, SM count
// and float-float log2 table on the device, and its caches of the GPU seed policy's tables
// (ray tables per (seed, R); wavelength points per seed, max(1024, W rounded up to a power
// of two) of them).
int context_device(const cpd_context *ctx);
int context_sms(const cpd_context *ctx);
const float *context_logtab(const cpd_context *ctx);
RayTablePtr context_ray_table(cpd_context *ctx, double seed, uint32_t R);
LamPtr context_lam_points(cpd_context *ctx, double seed, uint32_t W);
}  // namespace cpd
