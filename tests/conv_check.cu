// f32_rn and f64_of (dem_device.cuh) against the C conversions on the
// host.  f32_rn: random doubles over the whole normal float range, values
// next to rounding ties, powers of two, the range limits, zeros,
// infinities and NaNs (below 2^-126 the expected result is signed zero).
// f64_of: every float bit pattern (subnormals expected as signed zero).
// Prints ALL OK when every result matches.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>

#include "../dem_mbd_cuda_gb300/csrc/dem_device.cuh"

using demgb::f32_rn;
using demgb::f64_of;

static unsigned bits(float f) { unsigned u; std::memcpy(&u, &f, 4); return u; }

static long bad = 0, total = 0;

static void check(double x)
{
    ++total;
    const float got = f32_rn(x);
    float want = (float)x;
    if (std::fabs(x) < 0x1p-126) want = std::signbit(x) ? -0.0f : 0.0f;
    const bool ok = std::isnan(want) ? std::isnan(got) : bits(got) == bits(want);
    if (!ok && bad++ < 10) std::printf("mismatch x=%.17g got=%.9g want=%.9g\n", x, got, want);
}

int main()
{
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> ex(-126.0, 128.0), unit(1.0, 2.0);
    for (int i = 0; i < 4000000; ++i) {
        double x = std::ldexp(unit(rng), (int)std::floor(ex(rng)) - 1);
        if (i & 1) x = -x;
        check(x);
    }
    for (int i = 0; i < 2000000; ++i) {
        // exact halfway points between two floats and their neighbours
        const float f = std::ldexp((float)unit(rng), (int)std::floor(ex(rng)) - 1);
        const double h = ((double)f + (double)std::nextafter(f, 1e38f)) * 0.5;
        check(h);
        check(std::nextafter(h, 0.0));
        check(std::nextafter(h, 1e300));
        check(-h);
    }
    for (int e = -1074; e <= 1023; ++e) { check(std::ldexp(1.0, e)); check(-std::ldexp(1.0, e)); }
    const double special[] = {0.0, -0.0, 1.0, -1.0, 0x1p-126, 0x1.fffffffffffffp-127, 0x1p-149, (double)3.4028234663852886e38,
                              3.4028235677973366e38, 3.4028235677973362e38, 0x1p128, 1e300, -1e300, INFINITY, -INFINITY,
                              NAN, 0.1, 0.2, 0.3, 1e-5, 6.25e-3, 0.4, 1.0 / 3.0};
    for (double x : special) check(x);
    for (uint64_t u = 0; u <= 0xffffffffull; u += 1) {
        const unsigned v = (unsigned)u;
        float f;
        std::memcpy(&f, &v, 4);
        double want = (double)f;
        if (std::fabs(f) < 0x1p-126f) want = std::signbit(f) ? -0.0 : 0.0;
        const double got = f64_of(f);
        ++total;
        uint64_t a, b;
        std::memcpy(&a, &got, 8);
        std::memcpy(&b, &want, 8);
        const bool ok = std::isnan(want) ? std::isnan(got) : a == b;
        if (!ok && bad++ < 20) std::printf("f64_of mismatch bits=%08x got=%.17g want=%.17g\n", v, got, want);
    }
    std::printf("%ld of %ld mismatched\n", bad, total);
    if (bad == 0) std::printf("ALL OK\n");
    return bad == 0 ? 0 : 1;
}
