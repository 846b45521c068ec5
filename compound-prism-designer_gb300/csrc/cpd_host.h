// cpd_host.h -- host-side helpers shared by the C ABI translation units.
#pragma once

#include <cstdint>
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
}  // namespace cpd
