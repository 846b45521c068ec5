// ops_count.cpp -- TEST INFRASTRUCTURE ONLY: the op-counting build of the oracle.
//
// Compiles the oracle's per-ray model (cpd_oracle_model.h, the reference's f64 trace)
// with a scalar that counts every operation it performs, and traces W x R rays of a
// design with it. The counts are the algorithmic work per ray of the reference's per-ray
// formulation (src/spectrometer/ray.rs:485-499, spectrometer.rs:265-303,421-427): the
// denominators-free numerator of the FP32 roofline. Categories: add/sub, mul, fma,
// div, sqrt, compare, log, trig (cos/sin), other (neg, abs, copysign, sign bit,
// trunc). FLOP = add + mul + 2 fma + compare; div and sqrt are counted apart (special
// function or multi-instruction sequences on every GPU). Glass::calc_n, which the
// reference repeats per ray and surface but which depends on the wavelength alone, is
// booked in a bank of its own; so is the beam's inverse CDF (Shaw's norminv), which the
// GPU path tabulates once per ray index.
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>

#include "cpd_oracle.h"

namespace orc_ops {
enum { ADD, MUL, FMA, DIV, SQRT, CMP, LOG, TRIG, OTHER, NKIND };
enum { BANK_RAY, BANK_LAMBDA, NBANK };
static uint64_t count[NBANK][NKIND];
static int bank = BANK_RAY;
inline void tick(int k) { count[bank][k]++; }

struct Cnt {
    double v;
    Cnt() = default;
    Cnt(double x) : v(x) {}
};
inline Cnt operator+(Cnt a, Cnt b) { tick(ADD); return Cnt(a.v + b.v); }
inline Cnt operator-(Cnt a, Cnt b) { tick(ADD); return Cnt(a.v - b.v); }
inline Cnt operator*(Cnt a, Cnt b) { tick(MUL); return Cnt(a.v * b.v); }
inline Cnt operator/(Cnt a, Cnt b) { tick(DIV); return Cnt(a.v / b.v); }
inline Cnt operator-(Cnt a) { tick(OTHER); return Cnt(-a.v); }
inline Cnt &operator+=(Cnt &a, Cnt b) { a = a + b; return a; }
inline Cnt &operator-=(Cnt &a, Cnt b) { a = a - b; return a; }
inline Cnt &operator*=(Cnt &a, Cnt b) { a = a * b; return a; }
inline bool operator<(Cnt a, Cnt b) { tick(CMP); return a.v < b.v; }
inline bool operator<=(Cnt a, Cnt b) { tick(CMP); return a.v <= b.v; }
inline bool operator>(Cnt a, Cnt b) { tick(CMP); return a.v > b.v; }
inline bool operator>=(Cnt a, Cnt b) { tick(CMP); return a.v >= b.v; }
inline bool operator==(Cnt a, Cnt b) { tick(CMP); return a.v == b.v; }
inline bool operator!=(Cnt a, Cnt b) { tick(CMP); return a.v != b.v; }
inline Cnt fma(Cnt a, Cnt b, Cnt c) { tick(FMA); return Cnt(std::fma(a.v, b.v, c.v)); }
inline Cnt sqrt(Cnt a) { tick(SQRT); return Cnt(std::sqrt(a.v)); }
inline Cnt log(Cnt a) { tick(LOG); return Cnt(std::log(a.v)); }
inline Cnt log2(Cnt a) { tick(LOG); return Cnt(std::log2(a.v)); }
inline Cnt cos(Cnt a) { tick(TRIG); return Cnt(std::cos(a.v)); }
inline Cnt sin(Cnt a) { tick(TRIG); return Cnt(std::sin(a.v)); }
inline Cnt fabs(Cnt a) { tick(OTHER); return Cnt(std::fabs(a.v)); }
inline Cnt trunc(Cnt a) { tick(OTHER); return Cnt(std::trunc(a.v)); }
inline Cnt copysign(Cnt a, Cnt b) { tick(OTHER); return Cnt(std::copysign(a.v, b.v)); }
inline bool signbit(Cnt a) { tick(OTHER); return std::signbit(a.v); }
}  // namespace orc_ops

using orc_ops::cos;
using orc_ops::copysign;
using orc_ops::fabs;
using orc_ops::fma;
using orc_ops::log;
using orc_ops::log2;
using orc_ops::signbit;
using orc_ops::sin;
using orc_ops::sqrt;
using orc_ops::trunc;
typedef orc_ops::Cnt real;
#define ORC_D(x) ((x).v)
#define ORC_PER_LAMBDA_BEGIN const int orc_saved_bank = orc_ops::bank; orc_ops::bank = orc_ops::BANK_LAMBDA
#define ORC_PER_LAMBDA_END orc_ops::bank = orc_saved_bank
#include "cpd_oracle_model.h"

extern "C" {

// Traces rays (lam_u[k], ray_u[r]) for every k < W, r < R with the counting scalar.
// ray_ops / lambda_ops (NKIND each): totals over the W R rays of the per-ray work and of the
// per-wavelength work the reference repeats per ray (calc_n); hit_ray_ops: totals over the
// rays that reached a bin; beam_ops: the inverse CDF of the R start heights. Returns
// ORC_OK or a build error; *hits = rays that reached a bin.
int orc_ops_trace(const orc_spec *s, const double *lam_u, size_t W, const double *ray_u, size_t R, uint64_t *ray_ops,
                  uint64_t *lambda_ops, uint64_t *hit_ray_ops, uint64_t *beam_ops, uint64_t *hits)
{
    using namespace orc_ops;
    spectrometer sp;
    int e = build_spectrometer(s, &sp);
    if (e) return e;
    real *ys = (real *)std::malloc(sizeof(real) * R);
    if (!ys) return ORC_INVALID;
    std::memset(count, 0, sizeof(count));
    bank = BANK_RAY;
    for (size_t r = 0; r < R; r++) ys[r] = beam_y(&sp, ray_u[r]);
    for (int k = 0; k < NKIND; k++) beam_ops[k] = count[BANK_RAY][k];
    uint64_t tot[NBANK][NKIND] = {}, hit_tot[NKIND] = {}, nh = 0;
    for (size_t k = 0; k < W; k++) {
        const real w = sample_wavelength(&sp, lam_u[k]);
        for (size_t r = 0; r < R; r++) {
            std::memset(count, 0, sizeof(count));
            uint32_t bin = 0;
            real t = 0.0;
            const bool hit = spec_propagate(&sp, ys[r], w, &bin, &t) == ORC_OK;
            for (int b = 0; b < NBANK; b++)
                for (int q = 0; q < NKIND; q++) tot[b][q] += count[b][q];
            if (hit) {
                nh++;
                for (int q = 0; q < NKIND; q++) hit_tot[q] += count[BANK_RAY][q];
            }
        }
    }
    for (int q = 0; q < NKIND; q++) {
        ray_ops[q] = tot[BANK_RAY][q];
        lambda_ops[q] = tot[BANK_LAMBDA][q];
        hit_ray_ops[q] = hit_tot[q];
    }
    *hits = nh;
    std::free(ys);
    return ORC_OK;
}

int orc_ops_kinds(void) { return orc_ops::NKIND; }

}  // extern "C"
