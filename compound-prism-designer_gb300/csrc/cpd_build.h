// cpd_build.h -- design construction, shared by the host and the device.
//
// create_joined_trapezoids and CurvedPlane::from_hyperplane (geometry.rs:283-314,
// 430-489), LinearDetectorArray::new (spectrometer.rs:183-219), detector_array_positioning
// with fit_ray_difference_surface (spectrometer.rs:322-364, geometry.rs:495-542),
// size_and_deviation (spectrometer.rs:429-437), and the conversion of the f64 tables to
// the device record. The host compiles it with the C library's sin/cos/sqrt and gives the
// same tables as before this code was shared; on the device (designs built by the GPU from
// parameter records, csrc/cpd_kernels.cu build kernels) sin/cos are CUDA's f64 functions,
// which may differ from the C library's in the last bit.
#pragma once

#include <cmath>
#include <cstring>

#include "../../include/cpd.h"
#include "cpd_ff.h"
#include "cpd_model.h"

namespace cpd {
namespace build {

struct V2 {
    double x, y;
};
CPD_HD double cos_(double v) { return cos(v); }
CPD_HD double sin_(double v) { return sin(v); }
CPD_HD bool sign_bit(double v)
{
#if defined(__CUDA_ARCH__)
    return signbit(v);
#else
    return std::signbit(v);
#endif
}
CPD_HD bool finite(double v)
{
#if defined(__CUDA_ARCH__)
    return isfinite(v);
#else
    return std::isfinite(v);
#endif
}
CPD_HD V2 angled(double th) { return V2{cos_(th), sin_(th)}; }  // Vector::angled_xy (vector.rs:336-343)
CPD_HD V2 rot180(V2 a) { return V2{-a.x, -a.y}; }
CPD_HD V2 rot90(V2 a) { return V2{-a.y, a.x}; }
CPD_HD V2 rot90ccw(V2 a) { return V2{a.y, -a.x}; }
CPD_HD V2 vfma(V2 a, double b, V2 c) { return V2{x::fma_(a.x, b, c.x), x::fma_(a.y, b, c.y)}; }
// Every product, sum and quotient below goes through cpd::x (explicitly rounded on the
// device, no contraction; plain on the host, which compiles without contraction), so a
// device build differs from the host's only through sin/cos.

// create_joined_trapezoids (geometry.rs:430-489) and CurvedPlane::from_hyperplane
// (geometry.rs:283-314), into the cpd_design tables.
CPD_HDN inline int prism(const cpd_spectrometer_params &p, cpd_design &d)
{
    const int G = p.nglass;
    if (G < 1 || G > CPD_MAX_GLASS) return CPD_INVALID_ARGUMENT;
    if (!(p.height > 0.0) || !(fabs(p.curvature) > 0.0) || !(fabs(p.curvature) <= 1.0)) return CPD_INVALID_ARGUMENT;
    d.nglass = G;
    d.ar_coated = p.ar_coated ? 1 : 0;
    memcpy(d.glass, p.glass, sizeof(d.glass));
    d.height = p.height;
    const double h2 = x::mul(p.height, 0.5);
    V2 n0 = rot180(angled(p.angles[0]));
    V2 pt0{x::mul(fabs(x::div(n0.y, n0.x)), h2), h2};
    d.face_point[0][0] = pt0.x;
    d.face_point[0][1] = pt0.y;
    d.face_normal[0][0] = n0.x;
    d.face_normal[0][1] = n0.y;
    bool prev_sign = !sign_bit(n0.y);
    double d1 = pt0.x, mx = pt0.x;
    V2 last_pt{0, 0}, last_n{0, 0};
    // array_prepend (utils.rs:5-12): face k (1..G-1) uses lengths[k-1], the exit face lengths[G-1]
    for (int k = 1; k <= G; k++) {
        V2 n = rot180(angled(p.angles[k]));
        bool sign = !sign_bit(n.y);
        double d2 = x::mul(fabs(x::div(n.y, n.x)), h2);
        double sep = x::add(p.lengths[k - 1], prev_sign != sign ? x::add(d1, d2) : fabs(x::sub(d1, d2)));
        prev_sign = sign;
        d1 = d2;
        mx = x::add(mx, sep);
        if (k < G) {
            d.face_point[k][0] = mx;
            d.face_point[k][1] = h2;
            d.face_normal[k][0] = n.x;
            d.face_normal[k][1] = n.y;
        } else {
            last_pt = V2{mx, h2};
            last_n = n;
        }
    }
    const double kc = p.curvature;
    const double chord = fabs(x::div(p.height, last_n.x));
    const double radius = x::div(x::mul(chord, 0.5), fabs(kc));
    const double apothem = x::sqrt_(x::sub(x::mul(radius, radius), x::mul(x::mul(chord, chord), 0.25)));
    const double sagitta = x::sub(radius, apothem);
    V2 c = vfma(last_n, copysign(apothem, kc), last_pt);
    V2 m = vfma(last_n, -copysign(sagitta, kc), last_pt);
    d.exit_center[0] = c.x;
    d.exit_center[1] = c.y;
    d.exit_radius = radius;
    d.exit_bound_center[0] = m.x;
    d.exit_bound_center[1] = m.y;
    d.exit_bound_r2 = x::add(x::mul(sagitta, sagitta), x::mul(x::mul(chord, chord), 0.25));
    for (int k = 0; k < G; k++)
        if (!finite(d.face_point[k][0]) || !finite(d.face_normal[k][0])) return CPD_INVALID_ARGUMENT;
    if (!finite(radius) || !finite(apothem)) return CPD_INVALID_ARGUMENT;
    return CPD_OK;
}

CPD_HD void source(const cpd_spectrometer_params &p, cpd_design &d)
{
    d.wavelength_bounds[0] = p.wavelength_bounds[0];
    d.wavelength_bounds[1] = p.wavelength_bounds[1];
    d.beam_width = p.beam_width;
    d.beam_y_mean = p.beam_y_mean;
}

// f64 tables -> device record (exact part copied, FP32 fast-path constants derived in f64).
CPD_HDN inline void to_dev(const cpd_design &d, DevDesign &D)
{
    memset(&D, 0, sizeof(D));
    D.G = d.nglass;
    D.B = d.bin_count;
    D.ar = d.ar_coated;
    memcpy(D.glass, d.glass, sizeof(D.glass));
    for (int k = 0; k < CPD_MAX_GLASS; k++) {
        D.ppx[k] = d.face_point[k][0];
        D.ppy[k] = d.face_point[k][1];
        D.pnx[k] = d.face_normal[k][0];
        D.pny[k] = d.face_normal[k][1];
    }
    D.height = d.height;
    D.ccx = d.exit_center[0];
    D.ccy = d.exit_center[1];
    D.crad = d.exit_radius;
    D.cbx = d.exit_bound_center[0];
    D.cby = d.exit_bound_center[1];
    D.cbr2 = d.exit_bound_r2;
    D.bin_size = d.bin_size;
    D.slope = d.linear_slope;
    D.intercept = d.linear_intercept;
    D.min_ci = d.min_ci;
    D.L = d.det_length;
    D.dnx = d.det_normal[0];
    D.dny = d.det_normal[1];
    D.dpx = d.det_position[0];
    D.dpy = d.det_position[1];
    D.dux = d.det_direction[0];
    D.duy = d.det_direction[1];
    D.wmin = d.wavelength_bounds[0];
    D.wmax = d.wavelength_bounds[1];
    D.bw = d.beam_width;
    D.bym = d.beam_y_mean;
    D.size = d.size;
    D.deviation = d.deviation;
    FastConst &f = D.fc;
    f.inv_rc = (float)x::div(1.0, D.crad);
    f.rho = (float)x::sqrt_(D.cbr2);
    f.rho2 = (float)D.cbr2;
    f.dnfx = (float)D.dnx;
    f.dnfy = (float)D.dny;
    f.dufx = (float)D.dux;
    f.dufy = (float)D.duy;
    f.min_ci = (float)D.min_ci;
    f.L = (float)D.L;
    f.c0 = (float)D.intercept;
    f.slope = (float)D.slope;
    f.inv_slope = (float)x::div(1.0, D.slope);
    f.bin_size = (float)D.bin_size;
    f.bw = (float)D.bw;
    f.hL = (float)x::mul(0.5, D.L);
    f.ar = D.ar;
    f.B = D.B;
    DFConst &c = D.dc;
    auto sp = [](double v) {
        ff::F2 r;
        ff::split(v, r.hi, r.lo);
        return r;
    };
    for (int k = 0; k < CPD_MAX_GLASS; k++) {
        for (int i = 0; i < 6; i++) c.glass[k][i] = sp(D.glass[k][i]);
        c.ppx[k] = sp(D.ppx[k]);
        c.ppy[k] = sp(D.ppy[k]);
        c.pnx[k] = sp(D.pnx[k]);
        c.pny[k] = sp(D.pny[k]);
    }
    c.height = sp(D.height);
    c.ccx = sp(D.ccx);
    c.ccy = sp(D.ccy);
    c.rc2 = sp(x::mul(D.crad, D.crad));
    c.irc = sp(x::div(1.0, D.crad));
    c.cbx = sp(D.cbx);
    c.cby = sp(D.cby);
    c.cbr2 = sp(D.cbr2);
    c.vx = sp(x::sub(D.cbx, D.ccx));
    c.vy = sp(x::sub(D.cby, D.ccy));
    c.bin_size = sp(D.bin_size);
    c.slope = sp(D.slope);
    c.islope = sp(x::div(1.0, D.slope));
    c.intercept = sp(D.intercept);
    c.min_ci = sp(D.min_ci);
    c.L = sp(D.L);
    c.dnx = sp(D.dnx);
    c.dny = sp(D.dny);
    c.dpx = sp(D.dpx);
    c.dpy = sp(D.dpy);
    c.dux = sp(D.dux);
    c.duy = sp(D.duy);
    c.qx = sp(x::sub(D.dpx, D.cbx));
    c.qy = sp(x::sub(D.dpy, D.cby));
    c.wmin = sp(D.wmin);
    c.wspan = sp(x::sub(D.wmax, D.wmin));
    c.bw = sp(D.bw);
    c.bym = sp(D.bym);
}

// detector_array_positioning (spectrometer.rs:322-364) with fit_ray_difference_surface
// (geometry.rs:495-542): the detector position (and flip) that catches the acceptance
// band of wavelengths. Reads the prism, source, det_length and det_angle fields.
CPD_HDN inline int position(const cpd_spectrometer_params &p, double acceptance, double pos[2], int32_t &flipped)
{
    if (!(acceptance > 0.0) || !(acceptance <= 1.0)) return CPD_INVALID_ARGUMENT;
    cpd_design d;
    memset(&d, 0, sizeof(d));
    int e = prism(p, d);
    if (e) return e;
    source(p, d);
    DevDesign D;
    to_dev(d, D);
    const double uh = x::mul(fmax(x::sub(1.0, acceptance), 0.0), 0.5);
    const double wmin = x::wavelength(D, uh);
    const double wmax = x::wavelength(D, x::sub(1.0, uh));
    x::Ray lo{0.0, D.bym, 1.0, 0.0, 1.0, 1.0}, up = lo;
    e = x::prism(D, wmin, lo);
    if (e) return e;
    e = x::prism(D, wmax, up);
    if (e) return e;
    if (x::mul(x::add(lo.ts, lo.tp), 0.5) <= 1e-3 || x::mul(x::add(up.ts, up.tp), 0.5) <= 1e-3)
        return CPD_RAYTRACE_ANGULAR_RESPONSE_TOO_WEAK;
    V2 spec_dir = rot90(angled(p.det_angle));
    V2 spec{x::mul(spec_dir.x, p.det_length), x::mul(spec_dir.y, p.det_length)};
    const double a = up.dx, b = -lo.dx, c = up.dy, dd = -lo.dy;
    const double det = x::sub(x::mul(a, dd), x::mul(b, c));
    if (det == 0.0) return CPD_RAYTRACE_NO_SURFACE_INTERSECTION;
    const double i10 = x::div(-c, det), i11 = x::div(a, det);
    double tx = x::add(x::sub(spec.x, up.ox), lo.ox), ty = x::add(x::sub(spec.y, up.oy), lo.oy);
    double d2 = x::add(x::mul(i10, tx), x::mul(i11, ty));
    int32_t fl = 0;
    if (!(d2 > 0.0)) {
        tx = x::add(x::sub(-spec.x, up.ox), lo.ox);
        ty = x::add(x::sub(-spec.y, up.oy), lo.oy);
        d2 = x::add(x::mul(i10, tx), x::mul(i11, ty));
        if (d2 < 0.0) return CPD_RAYTRACE_NO_SURFACE_INTERSECTION;
        fl = 1;
    }
    pos[0] = x::fma_(lo.dx, d2, lo.ox);
    pos[1] = x::fma_(lo.dy, d2, lo.oy);
    flipped = fl;
    return CPD_OK;
}

// The whole design (cpd_design_build): argument checks of SizedCompoundPrism::new
// (src/pylib.rs:514-561), the prism, the detector array (min_ci = cos, src/pylib.rs:886)
// and size_and_deviation with mid_pt (spectrometer.rs:429-437, 305-308).
CPD_HDN inline int design(const cpd_spectrometer_params &p, cpd_design &out)
{
    if (p.bin_count == 0 || p.bin_count > CPD_MAX_BINS) return CPD_INVALID_ARGUMENT;
    if (!(p.linear_slope > 0.0) || !(p.bin_size > 0.0) || !(p.det_length > 0.0)) return CPD_INVALID_ARGUMENT;
    if (!(p.wavelength_bounds[1] >= p.wavelength_bounds[0])) return CPD_INVALID_ARGUMENT;
    cpd_design &d = out;
    memset(&d, 0, sizeof(d));
    int e = prism(p, d);
    if (e) return e;
    source(p, d);
    d.bin_count = p.bin_count;
    d.bin_size = p.bin_size;
    d.linear_slope = p.linear_slope;
    d.linear_intercept = p.linear_intercept;
    d.min_ci = cos_(p.max_incident_angle);
    d.det_length = p.det_length;
    V2 n = rot180(angled(p.det_angle));
    V2 u = p.det_flipped ? rot90(n) : rot90ccw(n);
    d.det_normal[0] = n.x;
    d.det_normal[1] = n.y;
    d.det_direction[0] = u.x;
    d.det_direction[1] = u.y;
    d.det_position[0] = p.det_position[0];
    d.det_position[1] = p.det_position[1];
    V2 mid = vfma(u, x::mul(p.det_length, 0.5), V2{d.det_position[0], d.det_position[1]});
    const double dx = mid.x, dy = x::sub(mid.y, p.beam_y_mean);
    const double size = x::sqrt_(x::add(x::mul(dx, dx), x::mul(dy, dy)));
    d.size = size;
    d.deviation = fabs(x::div(dy, size));
    return CPD_OK;
}

// cpd_design_build_batch's per-design step: positioning first when acceptance > 0.
CPD_HDN inline int design_positioned(cpd_spectrometer_params q, double acceptance, cpd_design &out)
{
    int e = CPD_OK;
    if (acceptance > 0.0) e = position(q, acceptance, q.det_position, q.det_flipped);
    if (!e) e = design(q, out);
    if (e) memset(&out, 0, sizeof(cpd_design));
    return e;
}

}  // namespace build
}  // namespace cpd
