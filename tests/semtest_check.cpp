// Host check of the adaptive stop test's FP32 screen (cpd_model.h, sem_quick) against the
// exact 128-bit test (sem_test): whenever the screen decides, it must decide like the
// exact test, for delta 0 (float-float transmittances) and kTqDelta (FP32 ones).
//
// Cases: Welford states of simulated bins (rounds of 32 samples, hit transmittances from
// several distributions), and states built to sit at the test's boundary (q2 solved for
// lhs = rhs, and for lhs = rhs +- err, then moved by a few units or a small relative step).
//
// usage: semtest_check <cases>
// prints: cases <n> decided <d> disagreements <m> boundary_cases <b>
#include <cstdint>
#include <cstdio>
#include <cstdlib>

#include "cpd_model.h"

using namespace cpd;
typedef unsigned __int128 u128;

static uint64_t rng_state = 0x9e3779b97f4a7c15ull;
static uint64_t next_u64()
{
    // splitmix64
    uint64_t z = (rng_state += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
static uint64_t below(uint64_t n) { return n ? next_u64() % n : 0u; }

static long cases = 0, decided = 0, bad = 0, boundary = 0;

static void check(uint32_t N, uint32_t h, uint64_t q1, uint64_t q2)
{
    // only consistent states: q1 <= h 2^20, q2 <= h 2^40, N q2 >= q1^2, h <= N
    if (h > N || q1 > ((uint64_t)h << 20) || q2 > ((uint64_t)h << 40)) return;
    if ((u128)N * q2 < (u128)q1 * q1) return;
    const uint32_t deltas[2] = {0u, kTqDelta};
    for (uint32_t delta : deltas) {
        cases++;
        const int q = sem_quick(N, h, q1, q2, delta);
        if (q < 0) continue;
        decided++;
        if (q != sem_test(N, h, q1, q2, delta)) {
            if (bad < 10)
                std::printf("# N %u h %u q1 %llu q2 %llu delta %u: quick %d exact %d\n", N, h,
                            (unsigned long long)q1, (unsigned long long)q2, delta, q,
                            sem_test(N, h, q1, q2, delta));
            bad++;
        }
    }
}

// A bin hit in `rounds` of 32 samples, k hits per round on average.
static void simulated_bin()
{
    const uint32_t rounds = 1u + (uint32_t)below(1u << (1 + below(17)));  // up to 2^17 rounds
    const uint32_t N = rounds * 32u;
    const int dist = (int)below(4);
    const uint32_t base = (uint32_t)below((1u << 20) + 1u);
    const uint32_t spread = (uint32_t)below(1u << below(21));
    uint32_t h = 0;
    uint64_t q1 = 0, q2 = 0;
    const uint32_t per = 1u + (uint32_t)below(32);
    // sample at most 2^16 hits explicitly; longer bins repeat the sampled block exactly
    const uint32_t hits = (uint32_t)(N < (uint64_t)rounds * per ? N : rounds * per);
    const uint32_t draw = hits < 65536u ? hits : 65536u;
    for (uint32_t i = 0; i < draw; i++) {
        uint32_t t;
        if (dist == 0) t = base;  // equal transmittances: zero variance among the hits
        else if (dist == 1) t = (uint32_t)below((1u << 20) + 1u);
        else if (dist == 2) {
            const uint64_t v = (uint64_t)base + below((uint64_t)spread + 1u);  // a narrow spread
            t = v > (1u << 20) ? (1u << 20) : (uint32_t)v;
        }
        else t = below(2) ? (1u << 20) : (uint32_t)below(1024u);
        h++;
        q1 += t;
        q2 += (uint64_t)t * t;
    }
    if (draw < hits) {
        const uint64_t rep = hits / draw;
        h *= (uint32_t)rep;
        q1 *= rep;
        q2 *= rep;
    }
    check(N, h, q1, q2);
}

// States at the boundary of the exact test.
static void boundary_bin()
{
    const uint32_t N = 32u * (1u + (uint32_t)below(1u << (1 + below(17))));
    const uint32_t h = 1u + (uint32_t)below(N);
    const uint64_t q1 = below(((uint64_t)h << 20) + 1u);
    // lhs = rhs  <=>  N q2 = q1^2 + N^2 (N - 1) 2^40 / 40000
    const u128 rhs = ((u128)N * N * (N - 1u)) << 40;
    u128 target = (rhs / 40000u + (u128)q1 * q1) / N;
    const int which = (int)below(3);
    if (which) {
        const u128 hd = (u128)h * kTqDelta;
        const u128 err =
            (u128)40000u * ((u128)N * h * ((u128)kTqDelta * ((1u << 21) + kTqDelta)) + hd * (2u * (u128)q1 + hd));
        const u128 shift = err / 40000u / N;
        target = which == 1 ? target + shift : (target > shift ? target - shift : 0u);
    }
    if (target > ((u128)h << 40)) return;
    boundary++;
    const uint64_t t = (uint64_t)target;
    for (int64_t k = -3; k <= 3; k++)
        if ((int64_t)t + k >= 0) check(N, h, q1, (uint64_t)((int64_t)t + k));
    for (int e = 6; e <= 24; e += 3) {
        const uint64_t step = t >> e;
        check(N, h, q1, t + step);
        if (t >= step) check(N, h, q1, t - step);
    }
}

int main(int argc, char **argv)
{
    const long n = argc > 1 ? std::atol(argv[1]) : 100000;
    for (long i = 0; i < n; i++) {
        simulated_bin();
        boundary_bin();
    }
    std::printf("cases %ld decided %ld disagreements %ld boundary_cases %ld\n", cases, decided, bad, boundary);
    return 0;
}
