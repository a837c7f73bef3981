// Host build of the device's correctly rounded sin / cos / asin / atan2
// (ornis_gb300/csrc/avbd_crmath.cuh) against long-double references rounded
// to float, over argument sweeps.  Prints one line per function: arguments
// tried and mismatches (the first few with their values).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <cstdlib>

#include "../../ornis_gb300/csrc/avbd_crmath.cuh"

static float u2f(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
static uint32_t f2u_h(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
static bool same(float a, float b) { return f2u_h(a) == f2u_h(b) || (a != a && b != b); }

static uint64_t rng_state = 0x9e3779b97f4a7c15ull;
static uint64_t next_u64() {  // splitmix64
    uint64_t z = (rng_state += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

struct Tally {
    const char* name;
    long n = 0, bad = 0;
    void check(float a, float b, float got, float want) {
        n++;
        if (same(got, want)) return;
        if (bad < 5) printf("  %s(%a, %a) = %a, reference %a\n", name, a, b, got, want);
        bad++;
    }
};

int main(int argc, char** argv) {
    long stride = argc > 1 ? atol(argv[1]) : 4099;  // every stride-th float bit pattern
    long randoms = argc > 2 ? atol(argv[2]) : 200000;
    Tally ts{"sin"}, tc{"cos"}, tsc{"sincos"}, ta{"asin"}, t2{"atan2"};
    auto one = [&](float x) {
        float s = avbd::crm::sinf(x), c = avbd::crm::cosf(x), s2, c2;
        avbd::crm::sincosf(x, &s2, &c2);
        float rs = (float)sinl((long double)x), rc = (float)cosl((long double)x);
        ts.check(x, 0, s, rs);
        tc.check(x, 0, c, rc);
        tsc.check(x, 0, s2, rs);
        tsc.check(x, 0, c2, rc);
        ta.check(x, 0, avbd::crm::asinf(x), (float)asinl((long double)x));
    };
    // every stride-th bit pattern over all floats (both signs, NaN and infinities included)
    for (uint64_t u = 0; u < (1ull << 32); u += (uint64_t)stride) one(u2f((uint32_t)u));
    // dense: every float in [2^-14, 4) near the physics' arguments, thinned
    for (uint32_t u = f2u_h(0x1p-14f); u < f2u_h(4.0f); u += 7) one(u2f(u));
    // every float in [0.5, 1] for asin (its two-branch boundary and the top)
    for (uint32_t u = f2u_h(0.5f); u <= f2u_h(1.0f); u += 3) ta.check(u2f(u), 0, avbd::crm::asinf(u2f(u)),
                                                                      (float)asinl((long double)u2f(u)));
    // atan2: random pairs of floats across exponents, quadrants, and special values
    const float sp[] = {0.0f, -0.0f, INFINITY, -INFINITY, 1.0f, -1.0f, 1e-30f, -1e-30f, 3e38f, -3e38f, NAN};
    for (float a : sp)
        for (float b : sp) t2.check(a, b, avbd::crm::atan2f(a, b), (float)atan2l((long double)a, (long double)b));
    for (long i = 0; i < randoms; i++) {
        uint64_t r = next_u64();
        float a = u2f((uint32_t)r), b = u2f((uint32_t)(r >> 32));
        if (i % 4 == 1) b = a * u2f(0x3f800000u + (uint32_t)(next_u64() & 0x7fffffu));  // |y| ~ |x|
        if (i % 4 == 2) {  // unit-quaternion style arguments: both in [-1, 1]
            a = (float)((int32_t)(r & 0xffffff) - 0x800000) * 0x1p-23f;
            b = (float)((int32_t)((r >> 32) & 0xffffff) - 0x800000) * 0x1p-23f;
        }
        t2.check(a, b, avbd::crm::atan2f(a, b), (float)atan2l((long double)a, (long double)b));
    }
    // the float stage of atan2: x near 1 (unit quaternions' w), |y| up to x/16
    for (long i = 0; i < randoms * 10; i++) {
        uint64_t r = next_u64();
        float x = u2f(0x3f700000u + (uint32_t)(r & 0xfffffu));  // [0.9375, 1)
        if (i % 3 == 0) x = u2f(0x3f800000u + (uint32_t)(r & 0x7fffffu));  // [1, 2)
        int ex = (int)((r >> 24) & 31);  // |y| in [2^-(4+ex+1), 2^-(4+ex)) x
        float y = x * u2f(0x3f800000u + (uint32_t)((r >> 32) & 0x7fffffu)) * ldexpf(1.0f, -5 - ex);
        if ((r >> 63) & 1) y = -y;
        t2.check(y, x, avbd::crm::atan2f(y, x), (float)atan2l((long double)y, (long double)x));
    }
    for (Tally* t : {&ts, &tc, &tsc, &ta, &t2}) printf("%s %ld %ld\n", t->name, t->n, t->bad);
    return 0;
}
